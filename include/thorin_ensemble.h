/* thorin_ensemble.h -- ensembles of independent disks on one GPU.
 *
 * The reference advances one disk per process.  An ensemble here is a set
 * of thorin_disk objects of any grid sizes on the current CUDA device.
 * Every disk has its own streams, and one call advances each disk by one DT
 * (thorin_gpu_algogas).  A pool of host worker threads takes the disks from
 * a queue.  A disk's kernels fill the GPU between the host round trips of
 * the others (CFL count, SOR convergence checks, planet kicks), so small
 * disks that alone leave most multiprocessors idle run side by side.  A
 * disk's results do not depend on the worker count or the order: each
 * disk's kernels and reductions run in a fixed order on its own streams.
 * No counterpart in the reference.
 */
#ifndef THORIN_ENSEMBLE_H
#define THORIN_ENSEMBLE_H

#include "thorin_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define THORIN_ORDER_GIVEN    0   /* disks in the order given               */
#define THORIN_ORDER_LARGEST  1   /* largest grid first (longest job first)  */

/* Advance every disk by one DT on `workers` host threads (1 = one after the
 * other on the calling thread).  status[k] (may be NULL) receives disk k's
 * return code; the call returns the first non-zero one, or THORIN_OK. */
int thorin_ensemble_algogas(thorin_disk *const *disks, thorin_planets *const *systems, int n, int workers,
                            int order, int *status);

/* Autotuner: advances the ensemble by `ndt` DTs for every candidate
 * schedule (worker counts 1, 2, 4, ... up to max_workers and n, each in
 * both orders), timing each on the wall clock after a device
 * synchronisation.  It writes the fastest schedule and its milliseconds
 * per DT, and the one-worker, given-order time for reference.  The DTs are
 * real steps of the run, each candidate on the next ones, so call it once
 * the disks are past their initial transient: while the cost per DT still
 * falls, the first candidates (the one-worker time among them) see the
 * costlier DTs. */
int thorin_ensemble_tune(thorin_disk *const *disks, thorin_planets *const *systems, int n, int max_workers, int ndt,
                         int *best_workers, int *best_order, double *best_ms_per_dt, double *sequential_ms_per_dt);

/* One DT of every disk as device-resident DT graphs (thorin_gpu_algogas_graph),
 * all launched on the disks' own streams from the calling thread before any
 * is waited for, so that the disks run side by side with no host round trip
 * inside the DT.  A disk's first DT runs on the host path (omega
 * calibration).  status[k] as for thorin_ensemble_algogas. */
int thorin_ensemble_algogas_graph(thorin_disk **disks, thorin_planets **systems, int n, int *status);

#ifdef __cplusplus
}
#endif
#endif

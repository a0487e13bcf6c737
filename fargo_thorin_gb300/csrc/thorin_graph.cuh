// thorin_graph.cuh -- device-side control of a whole DT (the substep loop,
// the planet side and the SOR omega schedule), so that one DT of a disk is
// one CUDA graph launch with no host round trip.  The control kernels live in
// thorin_graph.cu, compiled without FMA contraction like the host code whose
// arithmetic they repeat (thorin_planet.cuh).
#pragma once
#include "thorin_planet.cuh"

#define GRAPH_MAX_SUBSTEPS 100000   // bound of the substep loop (an error, not a hang, beyond it)

// Counters of the device-resident DT, read back once per DT.
struct GraphStats {
  int nsub;            // substeps of this DT
  int crashed;         // DetectCrash of the last substep
  int sor_calls;       // SOR solves in this DT
  int sor_last_niter;
  long long sor_sweeps;
  int niterlast;       // Niterlast of the omega schedule
  int capped;          // a solve hit the iteration cap
  int error;           // 1 SOR loop without an exit decision, 2 substep bound, 3 dt not positive
  double omega_used;   // omega of the last solve
};

// Everything the control kernels of one disk touch (device pointers, and the
// per-disk constants by value).
struct StepDev {
  DevGrid g;
  PlConst c;
  thorin_planets *sys;        // the planetary system, resident on the device during the DT
  double *scal;
  int *iscal;
  AccArgs *acc;               // pointer fields set by the host once; the scalars per planet and substep
  int *ring_info;             // [0,1]: accretion ring and ring count; [2 + k]: ring of planet k (-1 outside)
  DevPlanet *pl;
  int *heat_idx;
  double *heat_val;
  GraphStats *st;
  SorCtl sor;
  double DT, evaporation_rate;
  int npl, pebbles, accret_heating, indirect_term;
  cudaGraphConditionalHandle h_sub, h_sor;
};

// launchers (thorin_graph.cu); each is a one-block kernel on stream s
void graph_dt_begin(const StepDev &S, cudaStream_t s);
void graph_sub_begin(const StepDev &S, cudaStream_t s);
void graph_acc_init(const StepDev &S, cudaStream_t s);
void graph_acc_prep(const StepDev &S, int k, cudaStream_t s);
void graph_acc_finish(const StepDev &S, int k, cudaStream_t s);
void graph_force_prep(const StepDev &S, cudaStream_t s);
void graph_planet_step(const StepDev &S, cudaStream_t s);
void graph_sor_begin(const StepDev &S, cudaStream_t s);
void graph_sor_end(const StepDev &S, cudaStream_t s);
void graph_sub_end(const StepDev &S, cudaStream_t s);
// Ring mean of f at ring ring_info[slot] (count ring_info[slot + 1] when
// two_slots, else 1 if the ring is >= 0), with the summation of
// aux_ring_means; out[0..n).
void graph_ring_means_at(const DevGrid &g, const double *f, double *out, const int *ring_info, int slot, int two_slots,
                         cudaStream_t s);

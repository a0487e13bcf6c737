/* thorin_warmnet.h -- learned warm start of the radiative-diffusion SOR solve.
 *
 * The reference solves the implicit energy equation of
 * ImplicitRadiativeDiffusion (src_main/EnergySources.c:201-335) with
 * SuccessiveOverrelaxation (EnergySources.c:406-511), starting every solve
 * from the previous temperature.  This interface adds, beside that plain
 * method, a small polar-periodic convolutional encoder-decoder that predicts
 * the temperature update of a solve from the local fields; SOR then iterates
 * from the prediction to the same residual threshold as the plain solve
 * (eps times the L1 residual of the previous-temperature start), so the
 * converged temperature is the method's own.  It has no counterpart in the
 * reference.
 *
 * Network (fixed): 4 levels, 3x3 convolutions periodic in azimuth and
 * zero-padded in radius, 32 channels, ReLU, 2x2 average pooling down and
 * nearest-neighbour upsampling with additive skips up, one output channel;
 * 57,825 FP32 master parameters, BF16 weights and activations, FP32
 * accumulation on the tensor cores.  Inputs per cell (7 of 16 channels):
 * the Jacobi-scaled SOR residual of the start temperature (divided by its
 * grid mean and clipped to +-16), the four neighbour weights -M/Ml of the
 * SOR matrix, the local stiffness -log(1 - sum of the weights) / 4, and the
 * previous solve's update T_conv - T_start in the output's units (clipped;
 * zero before the disk's first solve with the network attached).  These
 * carry Sigma, T_old, the heating, the opacity and the dt-scaled diffusion
 * coefficients through the matrix and right-hand side that they build.
 * Output: the update beyond one Jacobi step, in units of 32 times the
 * residual scale.
 */
#ifndef THORIN_WARMNET_H
#define THORIN_WARMNET_H

#include <stdint.h>
#include "thorin_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define THORIN_WN_INPUTS   16    /* input channels per cell (7 used, rest zero) */
#define THORIN_WN_NPARAMS  57825 /* FP32 parameters */

#define THORIN_WS_OFF      0     /* plain SOR (the reference's method)          */
#define THORIN_WS_PREDICT  1     /* warm-start every SOR solve from the network */
#define THORIN_WS_TRAIN    2     /* plain SOR; each solve then trains the net   */
#define THORIN_WS_EXTRAPOLATE 3  /* start from T_old + the extrapolated update  */
#define THORIN_WS_MAX_ORDER 4    /* longest extrapolation (recorded solves)      */

typedef struct thorin_warmnet thorin_warmnet;

/* A network with activations for batch images of nrad x nsec cells
 * (nrad and nsec multiples of 8) on the current CUDA device.  Parameters
 * start at zero: set them with thorin_warmnet_set_params. */
int thorin_warmnet_create(int nrad, int nsec, int max_batch, thorin_warmnet **out);
int thorin_warmnet_destroy(thorin_warmnet *n);

/* FP32 parameters, per layer (e0, e1, e2, e3, d2, d1, d0, out) the weights
 * W[cout][3x3 tap (dr, dphi) row-major][cin] followed by the bias[cout]. */
int thorin_warmnet_set_params(thorin_warmnet *n, const float *host, int count);
int thorin_warmnet_get_params(thorin_warmnet *n, float *host, int count);

/* Raw network I/O (host buffers).  x: bf16 bit patterns
 * [batch][nrad][nsec][THORIN_WN_INPUTS]; y, target: [batch][nrad][nsec].
 * thorin_warmnet_gradient evaluates the loss
 *   mean over rings 1..nrad-2 of (y - target)^2
 * and its gradient with respect to the parameters (grad may be NULL; the
 * gradient also stays on the device for thorin_warmnet_adam). */
int thorin_warmnet_forward(thorin_warmnet *n, int batch, const uint16_t *x, float *y);
int thorin_warmnet_gradient(thorin_warmnet *n, int batch, const uint16_t *x, const float *target, float *loss,
                            float *grad);

/* One Adam step with the last gradient, clipped to global norm max_norm. */
int thorin_warmnet_adam(thorin_warmnet *n, float lr, float beta1, float beta2, float eps, float max_norm);

/* A network holds one set of activation buffers: attach it to one disk at
 * a time (in an ensemble advanced by several threads, give each disk its
 * own network).
 *
 * Attach a network to a disk or detach it (mode
 * THORIN_WS_OFF, n may be NULL).  The network's grid is the disk's nrad x
 * nsec, or half of it in both directions: then each network cell takes the
 * mean of its 2 x 2 disk cells' inputs and its prediction applies to all
 * four, while the Jacobi step stays per disk cell.  PREDICT: every SOR solve of the disk
 * starts from T_old + Jacobi step + network prediction (a cell whose
 * predicted temperature is not positive keeps T_old).  TRAIN: the solve is
 * plain; afterwards one Adam step (learning rate lr, moments 0.9/0.999,
 * norm clip 1) fits the network to that solve.  The loss of a step from
 * start temperature T_k is
 *   mean((A T_pred - rhs)^2) / mean|A T_k - rhs|^2 + 0.1 mean((y - target)^2)
 * over the unknowns, T_pred = T_k + Jacobi step + the prediction and target
 * the converged update beyond the Jacobi step in the network's units.
 * EXTRAPOLATE (no network, n ignored): every SOR solve starts from
 *   T_s - R(T_s) / Ml,   T_s = T_old + s u,   u = dt * r,
 * i.e. one Jacobi step from T_s, with r the update rate
 * (T_conv - T_start) / dt of the last m solves extrapolated to this one as
 * an evenly spaced sequence (m = the order, 2 unless set: r = 2 r_1 - r_2;
 * order 1 takes r = r_1, order 3 r = 3 r_1 - 3 r_2 + r_3), and s in [0, 2]
 * the step that minimises the L2 norm of the residual R along u (s = 1 is
 * the plain extrapolation; s near 0 where u does not help, as in fast
 * transients).  While fewer than m solves are recorded since attaching the
 * order is what they allow, and the first solve starts from T_old.  A cell
 * whose start is not positive keeps T_old.  The recorded updates belong to
 * the disk, not to its fields: after restoring other fields, attach the mode
 * again (every attach starts without recorded updates) so that the next
 * solves do not extrapolate from updates of another state.  In every mode the exit tests and the
 * threshold (eps times the L1 residual of T_old) are the plain solve's. */
int thorin_gpu_warmstart(thorin_disk *d, thorin_warmnet *n, int mode, float lr);

/* Order of the EXTRAPOLATE start, 1 .. THORIN_WS_MAX_ORDER (default 2). */
int thorin_gpu_warmstart_order(thorin_disk *d, int order);

/* The weights c[0..order) of the last `order` update rates in the
 * extrapolated rate r = sum_k c[k] r_(k+1): backward differences to the next
 * point of an evenly spaced sequence, c[k] = (-1)^k binom(order, k+1)
 * (2, -1 for order 2).  Host only; no GPU needed. */
int thorin_warmstart_coefficients(int order, double *c);

/* Layout check of the tensor-core path: D[128][32] = A[128][64] * B[32][64]^T
 * with bf16 bit patterns a, b (row-major) and FP32 d, on one CTA. */
int thorin_selftest_umma(const uint16_t *a, const uint16_t *b, float *d);

/* Self-test of the bounded mbarrier wait behind every tensor-core
 * completion: a wait for a barrier that nothing arrives at gives up after
 * `polls` polls (*timed_out = 1) and the kernel returns normally; after an
 * arrival the same wait completes (*completed_after_arrival = 1).  The
 * network kernels turn such a give-up into THORIN_ERR_TIMEOUT. */
int thorin_selftest_bounded_wait(long long polls, int *timed_out, int *completed_after_arrival);

/* Counters of the attached network's use on this disk. */
typedef struct thorin_ws_stats {
  long long predictions;   /* network applications inside SOR solves   */
  long long train_steps;   /* training steps taken                     */
  double last_loss;        /* loss of the last training step           */
  double last_res_loss;    /* its residual term                        */
  double last_sup_loss;    /* its supervised term                      */
  double step_sum;         /* EXTRAPOLATE: sum of the step lengths s    */
} thorin_ws_stats;
int thorin_gpu_warmstart_stats(thorin_disk *d, thorin_ws_stats *out);

#ifdef __cplusplus
}
#endif
#endif

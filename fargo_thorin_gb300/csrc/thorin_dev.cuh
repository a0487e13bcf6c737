// thorin_dev.cuh -- device-side layout and helpers shared by the kernels.
//
// One disk lives on one GPU.  Every 2D field uses the reference's PolarGrid
// layout (src_main/LowTasks.c:73-103): (nrad+1) rows of nsec FP64 values,
// azimuth contiguous, l = j + i*nsec; row nrad is the outer v_rad face.
// Ring (1D) arrays hold nrad+2 values; entries the reference never sets stay
// zero, like its zero-initialised MAX1D globals.
//
// Floating point.  The kernels are compiled with FMA contraction (the FP64
// pipe is the bound on GB300, and a fused multiply-add is one instruction
// instead of two), so per-cell results differ from the reference's
// separately rounded C arithmetic in the last bits; integer decisions
// (FARGO shifts, SOR iteration counts, substep counts) stay exact.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/thorin_gpu.h"

#define TH_PI 3.14159265358979323844
#define TH_MPI 3.14159265358979323846
#define TH_CFLSECURITY 0.5
#define TH_CVNR 1.41
#define TH_SORMIN 1.0e-15
#define TH_SORPRECISION 1.0e-15
#define TH_OMEGAUPPER 1.9
#define TH_KAPPAFLOOR 1.0e-12
#define TH_FULL 0xffffffffu

// Unit constants of src_main/fondam.h, evaluated once on the host with the
// host libm (so they are the reference's bits) and passed in DevConst.
struct DevConst {
  double opa2cu, t2si, rho2cgs, sigma_sb, sqrt2pi_inv, pebbulkdens, cv, sqrt_adiabind_inv;
  double evaptemp;           // EVAPORATIONTEMPERATURE / T2SI
  double sqrt3;              // sqrt(3.0)
  double dpns;               // 2 pi / nsec, the azimuthal cell width in radians
  // OpacityTable SM03: the Malygin gas table (device copies)
  const double *sm_pgrid, *sm_tgrid, *sm_ross;
  int sm_rows, sm_cols;
};

// Ring arrays (device pointers, nrad+2 entries each).
struct DevRings {
  const double *Rinf, *Rsup, *Rmed, *Surf, *InvRmed, *InvSurf, *InvDiffRmed, *InvDiffRsup, *InvRinf;
  const double *OmegaInv, *Rmed2, *WaveKiller;
  const double *Omega;                  // 1 / OmegaInv
  const double *InvDxtheta;             // 1 / (2 pi / nsec * Rmed)
  const double *Rmed15, *Rinf15;        // pow(Rmed,1.5), pow(Rinf,1.5) (FViscosity)
  const double *costab, *sintab;         // cos/sin(2 pi j / nsec), nsec entries
  const double *SigmaMed, *EnergyMed, *VthetaMed;
  const double *PebDensInit, *PebVradInit, *PebVthetaInit;
  double *csmean;                        // globcsvec   (ring mean of c_s)
  double *tempmean;                      // globtempervec
  double *nu_med, *nu_inf;               // FViscosity(Rmed[i]), FViscosity(Rinf[i])
};

// The disk's control block: scalars that change from one substep to the
// next.  Kernels read them from device memory instead of taking them as
// arguments, so that the launches of a substep do not depend on host values
// and a whole DT can be captured and replayed as one CUDA graph.  The host
// path writes them (k_set_ctl) before the kernels that read them; the graph
// path computes them on the device.
enum {
  CTL_DT = 0,            // substep length dt
  CTL_OMEGA_FRAME,       // OmegaFrame
  CTL_MASS_TAPER,        // MassTaper (SourceEuler.c:230-231)
  CTL_SOR_OMEGA,         // relaxation parameter of the current SOR solve
  CTL_FACC_EVAP,         // EvaporatePebbles' fraction min(EVAPORATIONRATE dt, 1)
  CTL_INDX_PL,           // indirect acceleration of the planets (x, y)
  CTL_INDY_PL,
  CTL_DELTAT,            // the DT's remaining interval DT - dtemp (ConditionCFL)
  CTL_INVDTREB,          // MinStepForRebound's rate invdtreb_sq
  CTL_TIME,              // PhysicalTime
  CTL_DTEMP,             // time advanced so far in this DT
  CTL_SOR_DOMEGA,        // omega schedule step (EnergySources.c:298-317)
  CTL_COUNT = 32
};

struct DevGrid {
  int nr, ns;
  int nsm;                               // multiprocessors of the disk's GPU
  DevRings r;
  DevConst k;
  double *ctl;                           // control block (CTL_*), CTL_COUNT doubles
  int sor_tpsm;                          // SOR pass: resident threads per multiprocessor (0: 1536)
};

__device__ __forceinline__ int jp_of(int j, int ns) { return (j == ns - 1) ? 0 : j + 1; }
__device__ __forceinline__ int jm_of(int j, int ns) { return (j == 0) ? ns - 1 : j - 1; }

// Sum of row[0..n) in strictly left-to-right order (the reference's
// sequential ring sums, e.g. mpi_make1Dprofile, mpiTasks.c:26-32), computed by
// one warp: lanes load coalesced chunks, the running sum walks the chunk in
// order through shuffles.  All lanes return the sum.
__device__ __forceinline__ double warp_seq_sum(const double *row, int n)
{
  const int lane = threadIdx.x & 31;
  double acc = 0.0;
  for (int base = 0; base < n; base += 32) {
    double v = (base + lane < n) ? row[base + lane] : 0.0;
    int cnt = n - base < 32 ? n - base : 32;
    for (int k = 0; k < cnt; k++) acc += __shfl_sync(TH_FULL, v, k);
  }
  return acc;
}

// Block-wide reductions (fixed order: warp shuffles then warp partials) -----
template <typename T, typename Op>
__device__ __forceinline__ T warp_reduce(T v, Op op)
{
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_down_sync(TH_FULL, v, o));
  return v;
}

struct OpAdd { __device__ double operator()(double a, double b) const { return a + b; } };
struct OpMin { __device__ double operator()(double a, double b) const { return b < a ? b : a; } };
struct OpMax { __device__ double operator()(double a, double b) const { return b > a ? b : a; } };
struct OpAddI { __device__ int operator()(int a, int b) const { return a + b; } };

// Result valid in thread 0.  blockDim.x must be a multiple of 32 (<= 1024).
template <typename T, typename Op>
__device__ T block_reduce(T v, Op op, T identity)
{
  __shared__ T sh[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_reduce(v, op);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : identity;
  if (wid == 0) v = warp_reduce(v, op);
  return v;
}

// Quotient for the van Leer slopes only.  The harmonic-mean slope
// 2 dq- dq+ / (dq- + dq+) enters a face value as a correction of at most
// half a cell width times the slope, beside the cell value itself, so a
// relative error e of the slope moves the face value by at most
// e |dq| dx / |q|.  The reciprocal estimate with one Newton-Raphson step,
// y = y + y(1 - d y), times x is two FP64 instructions shorter than
// div_fast; thorin_selftest_slope_division measures its distance from IEEE
// division on the GPU.  Same exponent guard as div_fast.
__device__ __forceinline__ double div_slope(double x, double d)
{
  const unsigned ex = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
  const unsigned ed = ((unsigned)__double2hiint(d) >> 20) & 0x7ffu;
  if (((ex - 523u) < 1001u || ex == 0u) && (ed - 523u) < 1001u) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
    y = __fma_rn(y, __fma_rn(-d, y, 1.0), y);
    return x * y;
  }
  return x / d;
}

// |x| by clearing the sign bit on the integer pipe (same bits as fabs).
__device__ __forceinline__ double abs_i(double x)
{
  return __hiloint2double(__double2hiint(x) & 0x7fffffff, __double2loint(x));
}

// The SOR coefficients (Ml, Mlip, Mlim, Mljp, Mljm, RHS) are stored packed
// by colour: for ring i, the cells of pass 1 (j = i-1 mod 2) then those of
// pass 2, each as k = j/2, so that a colour pass reads them contiguously.
// Every reader of those arrays indexes them through sor_pidx.
__device__ __forceinline__ size_t sor_pidx(int i, int j, int half)
{
  const int c = (j ^ (i - 1)) & 1;
  return (size_t)((i << 1) + c) * half + (j >> 1);
}

// Block reduction for blocks of exactly NT threads through shared memory:
// warp 0 folds the NT / 32 values of its lane's column, then one shuffle
// tree finishes.  On the FP64 pipe that is NT/32 + 4 warp instructions
// instead of the 5 (NT/32 + 1) of block_reduce.  Result valid in thread 0;
// fixed order.  Safe to call repeatedly (the first barrier waits for the
// previous call's readers).
template <int NT, typename T, typename Op>
__device__ __forceinline__ T block_reduce_smem(T v, Op op)
{
  static_assert(NT % 32 == 0 && NT <= 1024, "block of whole warps");
  __shared__ T sh[NT];
  __syncthreads();
  sh[threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    T s = sh[threadIdx.x];
#pragma unroll
    for (int k = 1; k < NT / 32; k++) s = op(s, sh[threadIdx.x + 32 * k]);
    v = warp_reduce(s, op);
  }
  return v;
}

// x^3 correctly rounded (Dekker two-product with fma): the reference uses
// pow(T, 3.0) (EnergySources.c:95,590), which glibc returns correctly
// rounded in all but vanishingly rare cases.
__device__ __forceinline__ double cube_rn(double x)
{
  double h = x * x;
  double l = __fma_rn(x, x, -h);          // x*x = h + l exactly
  double p = h * x;
  double e = __fma_rn(h, x, -p);          // h*x = p + e exactly
  double t = __fma_rn(l, x, e);           // remaining terms
  return __dadd_rn(p, t);
}

// Division without the IEEE divide sequence, for the hot stencils.  The
// hardware reciprocal estimate (rcp.approx.ftz.f64) gets one Newton-Raphson
// step, y = y + y(1 - d y); the quotient q = x y then gets Markstein's
// correction q + (x - d q) y with the residual formed exactly by an FMA
// (P. W. Markstein, IBM J. Res. Dev. 34(1):111-119, 1990).  Operands whose
// exponents lie in [2^-500, 2^500] (x may also be zero or subnormal) take this
// path, anything else the IEEE division.  thorin_selftest_division measures
// it against IEEE division on the GPU (no difference in 1e9 random quotients).
__device__ __forceinline__ double div_fast(double x, double d)
{
  const unsigned ex = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
  const unsigned ed = ((unsigned)__double2hiint(d) >> 20) & 0x7ffu;
  if (((ex - 523u) < 1001u || ex == 0u) && (ed - 523u) < 1001u) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
    const double e = __fma_rn(-d, y, 1.0);
    y = __fma_rn(y, e, y);
    const double q = x * y;
    const double r = __fma_rn(-d, q, x);
    return __fma_rn(r, y, q);
  }
  return x / d;
}


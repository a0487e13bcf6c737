// thorin_planet.cuh -- the planet side of one substep, shared by the host
// path (thorin_api.cu) and the device-resident DT (thorin_graph.cu).
//
// Each function is __host__ __device__: the host path runs it on the host
// between kernel launches, the whole-DT graph runs the same source in
// one-thread device kernels.  Device code that includes this file is
// compiled without FMA contraction (like the host code), so additions,
// products, quotients and square roots round identically on both sides;
// only the transcendental functions (pow, atan2, sin, cos) come from
// different libraries and may differ in the last bit.
#pragma once
#include <math.h>
#include "thorin_kernels.cuh"
#include "../../include/thorin_gpu.h"

#define PL_HD __host__ __device__ inline
#define PL_PI 3.14159265358979323844          // src_main/fondam.h:14
#define PL_MPI 3.14159265358979323846         // glibc M_PI

// Per-disk constants of the planet side, computed once on the host (some
// involve the host libm, e.g. the unit conversion of the planetary density).
struct PlConst {
  int nr, ns;
  double rin, rout;               // Rinf[0], Rsup[nr-1]: the disk's radial extent
  double plrho;                   // PLANETARYDENSITY / RHO2CGS
  double tdelay;                  // 4 DT HEATINGDELAY (Heating1's taper time)
  double thickness_smoothing, sqrt_adiabind_inv, adiabind;
  double pebble_alpha, vertical_damping;
  double mass_taper_param;        // MASSTAPER
  int indirect_term, accret_heating, feel_disk_any;
};

// The reference finds rings by linear scans ("while (Rsup[i] < r) i++").  On
// the increasing ring radii a bisection finds the same index; in a
// one-thread device kernel it takes log2(nr) dependent loads instead of up
// to nr.

// First i in [lo, hi) with a[i] >= r (hi if none); a increasing.
PL_HD int pl_first_ge(const double *a, int lo, int hi, double r)
{
  while (lo < hi) {
    const int mid = lo + (hi - lo) / 2;
    if (a[mid] < r) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// First i in [lo, hi) with a[i] > r (hi if none); a increasing.
PL_HD int pl_first_gt(const double *a, int lo, int hi, double r)
{
  while (lo < hi) {
    const int mid = lo + (hi - lo) / 2;
    if (a[mid] <= r) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// "while (Rsup[i] < r) i++", bounded at the last ring (ThicknessSmoothing's
// and DampingTW04's ring search).
PL_HD int pl_ring_of(const double *Rsup, int nr, double r)
{
  return pl_first_ge(Rsup, 0, nr - 1, r);
}

// GetGlobalIFrac (LowTasks.c:21-31) on the cell-centre radii.
PL_HD double pl_global_ifrac(const double *Rmed, int nr, double r)
{
  if (r < Rmed[0]) return 0.0;
  if (r > Rmed[nr - 1]) return (double)nr - 1.0;
  const int i = pl_first_gt(Rmed, 0, nr, r);            // "while (Rmed[i] <= r) i++"
  return (double)i + (r - Rmed[i - 1]) / (Rmed[i] - Rmed[i - 1]) - 1.0;
}

// MassTaper of AlgoGas (SourceEuler.c:230-231).
PL_HD double pl_mass_taper(double time, double mass_taper_param)
{
  double mt = time / (mass_taper_param * 2.0 * PL_MPI);
  return (mt > 1.0 ? 1.0 : pow(sin(mt * PL_MPI / 2.0), 2.0));
}

// MinStepForRebound (ReboundInterface.c:360-385): returns invdtreb_sq.
PL_HD double pl_min_step_for_rebound(const thorin_planets *sys)
{
  double dt = 1.e30;
  for (int i = 0; i < sys->nb; i++)
    for (int j = i + 1; j < sys->nb; j++) {
      double dx = sys->x[i] - sys->x[j], dy = sys->y[i] - sys->y[j], dz = sys->z[i] - sys->z[j];
      double dvx = sys->vx[i] - sys->vx[j], dvy = sys->vy[i] - sys->vy[j], dvz = sys->vz[i] - sys->vz[j];
      double r2 = dx * dx + dy * dy + dz * dz, rv = dx * dvx + dy * dvy + dz * dvz;
      double dtnew = fabs(r2 / rv);
      if (dtnew < dt) dt = dtnew;
    }
  dt *= 0.25;
  dt *= dt;
  return 1.0 / dt;
}

// The N-body step standing in for REBOUND's IAS15 (ReboundInterface.c:
// 262-325): heliocentric -> barycentric, star + planets with mutual gravity
// over dt (classical RK4 with 256 substeps), back to heliocentric.
#define PL_NMAX (MAXPL_DEV + 1)

// Bodies 0..N-1 (0 the star) with compile-time N: the loops unroll fully, so
// that on the device the state stays in registers (a one-thread kernel with
// its arrays in local memory spends most of its time waiting on loads).  The
// host path runs the same template, so the arithmetic and its order agree.
template <int N>
PL_HD void pl_nbody_accel_n(const double *m, const double *x, double *a)
{
#pragma unroll
  for (int i = 0; i < 3 * N; i++) a[i] = 0.0;
#pragma unroll
  for (int i = 0; i < N; i++)
#pragma unroll
    for (int j = i + 1; j < N; j++) {
      double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1], dz = x[3 * j + 2] - x[3 * i + 2];
      double r2 = dx * dx + dy * dy + dz * dz, r = sqrt(r2), ir3 = 1.0 / (r2 * r);
      a[3 * i] += 1.0 * m[j] * dx * ir3; a[3 * i + 1] += 1.0 * m[j] * dy * ir3; a[3 * i + 2] += 1.0 * m[j] * dz * ir3;
      a[3 * j] -= 1.0 * m[i] * dx * ir3; a[3 * j + 1] -= 1.0 * m[i] * dy * ir3; a[3 * j + 2] -= 1.0 * m[i] * dz * ir3;
    }
}

template <int N>
PL_HD void pl_nbody_step_n(thorin_planets *sys, double dt)
{
  double m[N], x[3 * N], v[3 * N], k1x[3 * N], k1v[3 * N], xt[3 * N], ax[3 * N], sx[3 * N], sv[3 * N];
  m[0] = 1.0;
#pragma unroll
  for (int c = 0; c < 3; c++) { x[c] = 0.0; v[c] = 0.0; }
#pragma unroll
  for (int k = 0; k < N - 1; k++) {
    m[k + 1] = sys->mass[k];
    x[3 * k + 3] = sys->x[k]; x[3 * k + 4] = sys->y[k]; x[3 * k + 5] = sys->z[k];
    v[3 * k + 3] = sys->vx[k]; v[3 * k + 4] = sys->vy[k]; v[3 * k + 5] = sys->vz[k];
  }
  double M = 0, cx[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < N; i++) {
    M += m[i];
#pragma unroll
    for (int c = 0; c < 3; c++) { cx[c] += m[i] * x[3 * i + c]; cv[c] += m[i] * v[3 * i + c]; }
  }
#pragma unroll
  for (int i = 0; i < N; i++)
#pragma unroll
    for (int c = 0; c < 3; c++) { x[3 * i + c] -= cx[c] / M; v[3 * i + c] -= cv[c] / M; }
  const int nsteps = 256;
  const double h = dt / nsteps;
  const double wts[4] = {1.0, 2.0, 2.0, 1.0}, cs[4] = {0.0, 0.5, 0.5, 1.0};
  for (int s = 0; s < nsteps; s++) {
#pragma unroll
    for (int q = 0; q < 3 * N; q++) { sx[q] = 0; sv[q] = 0; k1x[q] = 0; k1v[q] = 0; }
#pragma unroll
    for (int stage = 0; stage < 4; stage++) {
#pragma unroll
      for (int q = 0; q < 3 * N; q++) xt[q] = x[q] + cs[stage] * h * k1x[q];
      pl_nbody_accel_n<N>(m, xt, ax);
#pragma unroll
      for (int q = 0; q < 3 * N; q++) {
        double vx = v[q] + cs[stage] * h * k1v[q];
        k1x[q] = vx; k1v[q] = ax[q];
        sx[q] += wts[stage] * k1x[q]; sv[q] += wts[stage] * k1v[q];
      }
    }
#pragma unroll
    for (int q = 0; q < 3 * N; q++) { x[q] += h / 6.0 * sx[q]; v[q] += h / 6.0 * sv[q]; }
  }
#pragma unroll
  for (int k = 0; k < N - 1; k++) {
    sys->x[k] = x[3 * k + 3] - x[0]; sys->y[k] = x[3 * k + 4] - x[1]; sys->z[k] = x[3 * k + 5] - x[2];
    sys->vx[k] = v[3 * k + 3] - v[0]; sys->vy[k] = v[3 * k + 4] - v[1]; sys->vz[k] = v[3 * k + 5] - v[2];
  }
}

// The N-body step for the star and sys->nb (at most MAXPL_DEV) planets.
PL_HD void pl_nbody_step(thorin_planets *sys, double dt)
{
  switch (sys->nb) {
  case 0: break;
  case 1: pl_nbody_step_n<2>(sys, dt); break;
  case 2: pl_nbody_step_n<3>(sys, dt); break;
  case 3: pl_nbody_step_n<4>(sys, dt); break;
  case 4: pl_nbody_step_n<5>(sys, dt); break;
  case 5: pl_nbody_step_n<6>(sys, dt); break;
  case 6: pl_nbody_step_n<7>(sys, dt); break;
  case 7: pl_nbody_step_n<8>(sys, dt); break;
  default: pl_nbody_step_n<9>(sys, dt); break;
  }
}

// RotatePsys (Psys.c:336-355).
PL_HD void pl_rotate(thorin_planets *sys, double angle)
{
  double sint = sin(angle), cost = cos(angle);
  for (int k = 0; k < sys->nb; k++) {
    double xt = sys->x[k], yt = sys->y[k];
    sys->x[k] = xt * cost + yt * sint; sys->y[k] = -xt * sint + yt * cost;
    xt = sys->vx[k]; yt = sys->vy[k];
    sys->vx[k] = xt * cost + yt * sint; sys->vy[k] = -xt * sint + yt * cost;
  }
}

// AdvanceSystemFromDisk (Pframeforce.c:514-566) with DampingTW04 (:571-603):
// rrho/rcs are the ring means of Sigma and c_s at each planet (0 outside).
PL_HD void pl_advance_from_disk(const PlConst &c, thorin_planets *sys, double dt, const double ind[2],
                                const double *rrho, const double *rcs)
{
  for (int k = 0; k < sys->nb; k++) {
    if (!sys->feel_disk[k]) continue;
    const double x = sys->x[k], y = sys->y[k], z = sys->z[k], vz = sys->vz[k], m = sys->mass[k];
    double damp = 0.0;
    const double r = sqrt(x * x + y * y);
    if ((c.vertical_damping > 0.0) && (r >= c.rin && r <= c.rout)) {
      const double cs4inv = pow(rcs[k], -4.0), Omega = pow(r, -1.5);
      damp = c.vertical_damping * m * rrho[k] * Omega * cs4inv * (-2.176 * vz - 0.871 * z * Omega);
    }
    sys->vx[k] += dt * sys->ax[k];
    sys->vy[k] += dt * sys->ay[k];
    sys->vz[k] += dt * (sys->az[k] + damp);
    sys->vx[k] += dt * ind[0];
    sys->vy[k] += dt * ind[1];
  }
}

// Heating1 (Planet.c:222-247): the accretion luminosity of a planet goes
// into its cell.  Returns 0 (and touches nothing) outside the disk, else
// sets the cell index and the heating rate to add.
PL_HD int pl_heating1(const PlConst &c, const double *Rsup, const double *Surf, double time, double Mp, double dMp,
                      double Xp, double Yp, double dt, int *idx, double *add)
{
  const int ns = c.ns;
  const double Rperp = sqrt(Xp * Xp + Yp * Yp);
  if (Rperp < c.rin || Rperp > c.rout) return 0;
  double taper = time / c.tdelay;
  if (taper > 1.0) taper = 1.0;
  const double plradius = pow(3.0 * Mp / (4.0 * PL_PI * c.plrho), 1.0 / 3.0);
  const double L = Mp * dMp / dt / plradius;
  double ang = atan2(Yp, Xp);
  if (ang < 0.0) ang += 2.0 * PL_PI;
  const int i = pl_first_ge(Rsup, 0, c.nr, Rperp);        // "while (Rsup[i] < Rperp) i++"
  int j = (int)floor((double)ns / 2.0 / PL_PI * ang + 0.5);
  if (j == ns) j = 0;
  *idx = j + i * ns;
  *add = L * taper / Surf[i];
  return 1;
}

// AccretePebblesOntoPlanets' set-up for planet k (Pebbles.c:353-420): the
// scalar fields of AccArgs (the pointers are the caller's), and the block
// count of the annulus [imin, imax] that holds the Hill sphere (0 if none).
PL_HD void pl_pebble_acc_prep(const PlConst &c, const double *Rinf, const double *Rsup, const double *Rmed,
                              const thorin_planets *sys, int k, double omega_frame, double dt, int acc_bx, AccArgs *a)
{
  a->Xp = sys->x[k]; a->Yp = sys->y[k]; a->Zp = sys->z[k];
  a->VXp = sys->vx[k]; a->VYp = sys->vy[k]; a->VZp = sys->vz[k];
  a->Mp = sys->mass[k];
  double Rp = a->Xp * a->Xp + a->Yp * a->Yp;
  const double Rp3D = sqrt(Rp + a->Zp * a->Zp);
  Rp = sqrt(Rp);
  a->Rp = Rp;
  a->Rhill = Rp3D * pow(1.0 / 3.0 * a->Mp, 1.0 / 3.0);
  a->Omegap = pow(Rp, -1.5);
  a->Rp15 = pow(Rp, 1.5);
  const double ifrac = pl_global_ifrac(Rmed, c.nr, Rp);
  a->frac = ifrac - floor(ifrac);
  a->iflow = (int)ifrac;
  a->omega_frame = omega_frame;
  a->dt = dt;
  a->pebble_alpha = c.pebble_alpha;
  // Pebbles.c:408-409: "while (Rinf[imax] > Rp + Rhill) imax--" from the
  // last ring, then "while (Rsup[imin] < Rp - Rhill) imin++" from the first,
  // not past imax (for a planet inside the inner edge the reference's scan
  // reads Rinf[-1]; the bisection stops at imax = -1)
  const int imax = pl_first_gt(Rinf, 0, c.nr, Rp + a->Rhill) - 1;
  const int imin = pl_first_ge(Rsup, 0, imax + 1, Rp - a->Rhill);
  a->imin = imin; a->imax = imax;
  a->nb = (imin <= imax) ? ((imax - imin + 1) * c.ns + acc_bx - 1) / acc_bx : 0;
}

// The planet's new mass and velocity after accreting dMp with momentum
// (dPx, dPy) (Pebbles.c:520-539).
PL_HD void pl_pebble_acc_finish(thorin_planets *sys, int k, const AccArgs &a, double dMp, double dPx, double dPy)
{
  double PX = a.VXp * a.Mp + dPx, PY = a.VYp * a.Mp + dPy, M = a.Mp + dMp;
  sys->mass[k] = M;
  sys->solid[k] = sys->solid[k] + dMp;
  sys->vx[k] = PX / M;
  sys->vy[k] = PY / M;
}

// FillForcesArrays' per-planet constants (Pframeforce.c:60-110) with
// ThicknessSmoothing (Force.c:75-102) from the ring mean of c_s at the
// planet's ring; adds the planet's indirect pull to (axs, ays).
PL_HD void pl_force_planet(const PlConst &c, const double *Rsup, const double *csmean, const double *OmegaInv,
                           const thorin_planets *sys, int k, double mass_taper, DevPlanet *P, double *axs,
                           double *ays)
{
  const double xpl = sys->x[k], ypl = sys->y[k], zpl = sys->z[k];
  double mpl = sys->mass[k];
  const double dpl = sqrt(xpl * xpl + ypl * ypl + zpl * zpl);
  P->x = xpl; P->y = ypl; P->z = zpl; P->m = mpl;
  P->rhill = dpl * pow((1.0 / 3.0 * mpl), 1.0 / 3.0);
  double smoothing = 0.0;
  const double r = sqrt(xpl * xpl + ypl * ypl);
  if (r >= c.rin && r <= c.rout) {
    const int i = pl_ring_of(Rsup, c.nr, r);
    smoothing = c.thickness_smoothing * (csmean[i] * OmegaInv[i] * c.sqrt_adiabind_inv);
  }
  P->Hpl = smoothing / c.thickness_smoothing;
  P->smoothing2 = smoothing * smoothing;
  const double rst = 0.5 * P->rhill;
  P->rst2 = rst * rst; P->rst3 = P->rst2 * rst; P->rst4 = P->rst3 * rst;
  const double rsm = 0.05 * P->rhill;
  P->rsm2 = rsm * rsm;
  P->rmorevert2 = 2.0 * P->rhill;
  P->rmorevert2 *= P->rmorevert2;
  P->near_h2 = 10.0 * P->Hpl;
  P->near_h2 *= P->near_h2;
  P->near_hill2 = 5.0 * P->rhill;
  P->near_hill2 *= P->near_hill2;
  if (c.indirect_term) {
    const double invdpl3 = 1.0 / (dpl * dpl * dpl);
    mpl *= mass_taper;
    *axs += mpl * invdpl3 * xpl;
    *ays += mpl * invdpl3 * ypl;
  }
}

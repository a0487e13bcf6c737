// thorin_graph.cu -- the control kernels of a device-resident DT.
//
// One DT of AlgoGas (SourceEuler.c:210-317) runs as one CUDA graph: a WHILE
// node whose body is one substep, with the SOR sweep loop a WHILE node inside
// it.  Everything the host path decides between launches is decided here on
// the device, by one-thread kernels that run the host path's own source
// (thorin_planet.cuh): the substep interval and MinStepForRebound before the
// CFL, the pebble accretion set-up and Heating1 for each planet, the
// per-planet force constants and the indirect term, the planet kick, the
// N-body step and the frame rotation, the SOR omega schedule around each
// solve, and the loop condition.  This file is compiled without FMA
// contraction, so these kernels round like the host code.
//
// Bounded loops: the substep loop stops after GRAPH_MAX_SUBSTEPS substeps or
// on a non-positive dt (with an error flag the host reads); the SOR loop
// stops at the iteration cap (its completion step, k_sor_pass).
#include "thorin_graph.cuh"

__global__ void k_g_dt_begin(StepDev S)
{
  if (threadIdx.x != 0) return;
  S.g.ctl[CTL_DTEMP] = 0.0;
  GraphStats *st = S.st;
  st->nsub = 0;
  st->crashed = 0;
  st->sor_calls = 0;
  st->sor_sweeps = 0;
  st->capped = 0;
  st->error = 0;
}

// SourceEuler.c:230-244 up to ConditionCFL: MassTaper, MinStepForRebound and
// the remaining interval of the DT.
__global__ void k_g_sub_begin(StepDev S)
{
  if (threadIdx.x != 0) return;
  double *ctl = S.g.ctl;
  ctl[CTL_MASS_TAPER] = pl_mass_taper(ctl[CTL_TIME], S.c.mass_taper_param);
  ctl[CTL_INVDTREB] = pl_min_step_for_rebound(S.sys);
  ctl[CTL_DELTAT] = S.DT - ctl[CTL_DTEMP];
}

// InitHeating (Planet.c:251) and EvaporatePebbles' fraction of this dt.
__global__ void k_g_acc_init(StepDev S)
{
  if (threadIdx.x != 0) return;
  for (int k = 0; k < S.npl; k++) { S.heat_val[k] = 0.0; S.heat_idx[k] = -1; }
  double facc = S.evaporation_rate * S.g.ctl[CTL_DT];
  if (facc > 1.0) facc = 1.0;
  S.g.ctl[CTL_FACC_EVAP] = facc;
}

// AccretePebblesOntoPlanets' set-up for planet k; the ring means of v_theta
// at the planet's ring follow from ring_info[0..1].
__global__ void k_g_acc_prep(StepDev S, int k)
{
  if (threadIdx.x != 0) return;
  AccArgs a = *S.acc;
  pl_pebble_acc_prep(S.c, S.g.r.Rinf, S.g.r.Rsup, S.g.r.Rmed, S.sys, k, S.g.ctl[CTL_OMEGA_FRAME], S.g.ctl[CTL_DT],
                     ACC_BX, &a);
  *S.acc = a;
  S.ring_info[0] = a.nb > 0 ? a.iflow : -1;
  S.ring_info[1] = (a.iflow + 1 < S.g.nr) ? 2 : 1;
}

// Heating1 and the planet's new mass and velocity after the accretion.
__global__ void k_g_acc_finish(StepDev S, int k)
{
  if (threadIdx.x != 0) return;
  const AccArgs &a = *S.acc;
  double dMp = 0.0, dPx = 0.0, dPy = 0.0;
  if (a.nb > 0) { dMp = S.scal[SC_ACC_DM]; dPx = S.scal[SC_ACC_DPX]; dPy = S.scal[SC_ACC_DPY]; }
  if (S.accret_heating) {
    int idx;
    double add;
    if (pl_heating1(S.c, S.g.r.Rsup, S.g.r.Surf, S.g.ctl[CTL_TIME], a.Mp, dMp, a.Xp, a.Yp, S.g.ctl[CTL_DT], &idx, &add)) {
      S.heat_idx[k] = idx;
      S.heat_val[k] += add;
    }
  }
  pl_pebble_acc_finish(S.sys, k, a, dMp, dPx, dPy);
}

// dtemp += dt (SourceEuler.c:249), then FillForcesArrays' per-planet
// constants, the planets' indirect term and each planet's ring for
// DampingTW04.
__global__ void k_g_force_prep(StepDev S)
{
  if (threadIdx.x != 0) return;
  double *ctl = S.g.ctl;
  ctl[CTL_DTEMP] += ctl[CTL_DT];
  double axs = 0.0, ays = 0.0;
  for (int k = 0; k < S.npl; k++) {
    pl_force_planet(S.c, S.g.r.Rsup, S.g.r.csmean, S.g.r.OmegaInv, S.sys, k, ctl[CTL_MASS_TAPER], &S.pl[k], &axs,
                    &ays);
    const double x = S.sys->x[k], y = S.sys->y[k];
    const double r = sqrt(x * x + y * y);
    const int i = (r >= S.c.rin && r <= S.c.rout) ? pl_ring_of(S.g.r.Rsup, S.c.nr, r) : -1;
    S.ring_info[2 + k] = i;
    // the planet step runs beside the hydro substep, which rewrites the
    // ring means of c_s at its end: DampingTW04's value is taken now
    S.scal[SC_RCS + k] = (i >= 0) ? S.g.r.csmean[i] : 0.0;
  }
  ctl[CTL_INDX_PL] = S.indirect_term ? -axs : 0.0;
  ctl[CTL_INDY_PL] = S.indirect_term ? -ays : 0.0;
}

// AdvanceSystemFromDisk with DampingTW04, the N-body step and RotatePsys
// (SourceEuler.c:251-268).
__global__ void k_g_planet_step(StepDev S)
{
  if (threadIdx.x != 0) return;
  double rrho[MAXPL_DEV], rcs[MAXPL_DEV];
  thorin_planets *sys = S.sys;
  for (int k = 0; k < S.npl; k++) {
    sys->ax[k] = S.scal[SC_PLANET_A + 2 * k];
    sys->ay[k] = S.scal[SC_PLANET_A + 2 * k + 1];
    const int i = S.ring_info[2 + k];
    rrho[k] = (i >= 0) ? S.scal[SC_PLANET_A + 2 * MAXPL_DEV + k] : 0.0;
    rcs[k] = (i >= 0) ? S.scal[SC_RCS + k] : 0.0;
  }
  const double dt = S.g.ctl[CTL_DT];
  const double ind[2] = {S.scal[SC_INDX], S.scal[SC_INDY]};
  pl_advance_from_disk(S.c, sys, dt, ind, rrho, rcs);
  pl_nbody_step(sys, dt);
  pl_rotate(sys, S.g.ctl[CTL_OMEGA_FRAME] * dt);
}

// The omega schedule before a solve (EnergySources.c:298-305); arms the
// sweep loop's condition, whose default is applied only once per launch of
// the whole graph.
__global__ void k_g_sor_begin(StepDev S)
{
  if (threadIdx.x != 0) return;
  double *ctl = S.g.ctl;
  double omega = ctl[CTL_SOR_OMEGA] + ctl[CTL_SOR_DOMEGA], domega = ctl[CTL_SOR_DOMEGA];
  if (omega > TH_OMEGAUPPER) { omega = TH_OMEGAUPPER; domega = -domega; }
  if (omega < 1.0) { omega = 1.0; domega = -domega; }
  ctl[CTL_SOR_OMEGA] = omega;
  ctl[CTL_SOR_DOMEGA] = domega;
  cudaGraphSetConditional(S.h_sor, 1u);
}

// After a solve (EnergySources.c:306-317): counters, and the schedule's
// reversal when the solve took more sweeps than the last.
__global__ void k_g_sor_end(StepDev S)
{
  if (threadIdx.x != 0) return;
  GraphStats *st = S.st;
  const int done = *S.sor.done, n = *S.sor.niter;
  if (!done || n < 1) st->error = 1;
  if (done == 2) st->capped = 1;
  st->sor_calls++;
  st->sor_sweeps += n;
  st->sor_last_niter = n;
  st->omega_used = S.g.ctl[CTL_SOR_OMEGA];
  if (n > st->niterlast) S.g.ctl[CTL_SOR_DOMEGA] = -S.g.ctl[CTL_SOR_DOMEGA];
  st->niterlast = n;
}

// End of a substep: the clock, the counters and the loop condition
// (dtemp < 0.999999999 DT, SourceEuler.c:229).
__global__ void k_g_sub_end(StepDev S)
{
  if (threadIdx.x != 0) return;
  double *ctl = S.g.ctl;
  GraphStats *st = S.st;
  const double dt = ctl[CTL_DT];
  ctl[CTL_TIME] += dt;
  st->nsub++;
  st->crashed = S.iscal[IS_CRASH];
  unsigned more = (ctl[CTL_DTEMP] < 0.999999999 * S.DT) ? 1u : 0u;
  if (!(dt > 0.0)) { st->error = 3; more = 0u; }
  if (st->nsub >= GRAPH_MAX_SUBSTEPS) { st->error = 2; more = 0u; }
  if (st->error) more = 0u;
  cudaGraphSetConditional(S.h_sub, more);
}

#define ONE_BLOCK <<<1, 32, 0, s>>>
void graph_dt_begin(const StepDev &S, cudaStream_t s) { k_g_dt_begin ONE_BLOCK(S); g_thorin_launches++; }
void graph_sub_begin(const StepDev &S, cudaStream_t s) { k_g_sub_begin ONE_BLOCK(S); g_thorin_launches++; }
void graph_acc_init(const StepDev &S, cudaStream_t s) { k_g_acc_init ONE_BLOCK(S); g_thorin_launches++; }
void graph_acc_prep(const StepDev &S, int k, cudaStream_t s) { k_g_acc_prep ONE_BLOCK(S, k); g_thorin_launches++; }
void graph_acc_finish(const StepDev &S, int k, cudaStream_t s) { k_g_acc_finish ONE_BLOCK(S, k); g_thorin_launches++; }
void graph_force_prep(const StepDev &S, cudaStream_t s) { k_g_force_prep ONE_BLOCK(S); g_thorin_launches++; }
void graph_planet_step(const StepDev &S, cudaStream_t s) { k_g_planet_step ONE_BLOCK(S); g_thorin_launches++; }
void graph_sor_begin(const StepDev &S, cudaStream_t s) { k_g_sor_begin ONE_BLOCK(S); g_thorin_launches++; }
void graph_sor_end(const StepDev &S, cudaStream_t s) { k_g_sor_end ONE_BLOCK(S); g_thorin_launches++; }
void graph_sub_end(const StepDev &S, cudaStream_t s) { k_g_sub_end ONE_BLOCK(S); g_thorin_launches++; }

// kernels_aux.cu -- ring means, viscosity per ring, CFL, pebble source terms,
// damping boundaries, disk forces with their reductions, pebble accretion,
// conservation integrals.
#include "thorin_kernels.cuh"
#include "thorin_graph.cuh"

static inline dim3 grid2d(int ns, int rows, int bx) { return dim3((ns + bx - 1) / bx, rows); }
static const int BX = 128;

#define CELL_LOOP_2D                                                        \
  const int j = blockIdx.x * blockDim.x + threadIdx.x;                      \
  const int i = blockIdx.y;                                                 \
  if (j >= ns) return;                                                      \
  const int l = j + i * ns;

// ---------------------------------------------------------------------------
// Ring (azimuthal) means, mpi_make1Dprofile (mpiTasks.c:26-32) and the
// other azimuthal averages of the loop.  One warp per ring sums in a fixed
// tree (lanes take strided columns, then a butterfly), so results are
// deterministic; they differ from the reference's left-to-right sum in the
// last bits.  The only integer decision fed by a ring mean, the FARGO shift,
// re-sums its ring in order when the mean lands near a rounding tie (see
// k_azimuthal).  Output index is relative to ring0.
// One warp's fixed-tree sum of a ring (all lanes return it).
__device__ __forceinline__ double warp_ring_sum(const double *__restrict__ row, int ns, int lane)
{
  double a = 0.0;
  for (int j = lane; j < ns; j += 32) a += row[j];
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(TH_FULL, a, o);
  return a;
}

__global__ void __launch_bounds__(256) k_ring_means(int ns, const double *__restrict__ f0,
                                                    const double *__restrict__ f1, double *__restrict__ o0,
                                                    double *__restrict__ o1, int ring0, int nrings, int nf)
{
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= nrings) return;                         // whole warp
  const size_t base = (size_t)(ring0 + w) * ns;
  const double a0 = warp_ring_sum(f0 + base, ns, lane);
  const double a1 = (nf > 1) ? warp_ring_sum(f1 + base, ns, lane) : 0.0;
  if (lane == 0) {
    o0[w] = a0 / (double)ns;
    if (nf > 1) o1[w] = a1 / (double)ns;
  }
}

// The same ring means at rings chosen on the device: ring info[slot] and,
// with two, info[slot + 1] rings from there (else one ring when
// info[slot] >= 0, none when it is negative).
__global__ void __launch_bounds__(64) k_ring_means_at(int ns, const double *__restrict__ f, double *__restrict__ o,
                                                      const int *__restrict__ info, int slot, int two)
{
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ring0 = info[slot];
  const int nrings = two ? info[slot + 1] : (ring0 >= 0 ? 1 : 0);
  if (ring0 < 0 || w >= nrings) return;
  const double a = warp_ring_sum(f + (size_t)(ring0 + w) * ns, ns, lane);
  if (lane == 0) o[w] = a / (double)ns;
}

void graph_ring_means_at(const DevGrid &g, const double *f, double *out, const int *ring_info, int slot, int two_slots,
                         cudaStream_t s)
{
  k_ring_means_at<<<1, 64, 0, s>>>(g.ns, f, out, ring_info, slot, two_slots);
  g_thorin_launches++;
}

void aux_ring_means(const DevGrid &g, const double *f0, double *o0, const double *f1, double *o1, int ring0, int nrings,
                    cudaStream_t s)
{
  if (nrings <= 0) return;
  const int blocks = (nrings * 32 + 255) / 256;
  k_ring_means<<<blocks, 256, 0, s>>>(g.ns, f0, f1 ? f1 : f0, o0, o1 ? o1 : o0, ring0, nrings, f1 ? 2 : 1);
  g_thorin_launches++;
}

__global__ void k_set_ctl(double *__restrict__ ctl, CtlSet v)
{
  if (threadIdx.x < (unsigned)v.n) ctl[v.idx[threadIdx.x]] = v.val[threadIdx.x];
}

void aux_set_ctl(double *ctl, const CtlSet &v, cudaStream_t s)
{
  k_set_ctl<<<1, 32, 0, s>>>(ctl, v);
  g_thorin_launches++;
}

void aux_ring_mean(const DevGrid &g, const double *f, double *out, cudaStream_t s)
{
  aux_ring_means(g, f, out, nullptr, nullptr, 0, g.nr, s);
}

void aux_ring_mean_at(const DevGrid &g, const double *f, int ring, double *out, cudaStream_t s)
{
  aux_ring_means(g, f, out, nullptr, nullptr, ring, 1, s);
}

// FViscosity at Rmed[i] and Rinf[i] (Viscosity.c:26-54).  The ring index
// found by the reference's linear search is i for both radii; pow(r, 1.5)
// comes precomputed from the host.

__device__ __forceinline__ double fvisc(const ViscParams &v, double rad, double cs, double tmean, double r15)
{
  double nu = v.viscosity;
  if (v.viscosity_alpha) nu = v.alpha * cs * cs * r15;
  if (v.alpha_flock) {
    double a = (v.alpha_mri - v.alpha_dead) * (1.0 - tanh((v.tmri - tmean * v.t2si) / v.twidth)) / 2.0 + v.alpha_dead;
    nu = a * cs * cs * r15;
  }
  if (rad < v.cav_rmin) nu *= v.cav_ratio;
  if ((rad >= v.cav_rmin) && (rad <= v.cav_rmax)) nu *= exp((v.cav_rmax - rad) / (v.cav_rmax - v.cav_rmin) * v.log_cav_ratio);
  return nu;
}

__global__ void k_viscosity_rings(DevGrid g, ViscParams v)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.nr) return;
  const double cs = g.r.csmean[i], tm = g.r.tempmean[i];
  g.r.nu_med[i] = fvisc(v, g.r.Rmed[i], cs, tm, g.r.Rmed15[i]);
  g.r.nu_inf[i] = fvisc(v, g.r.Rinf[i], cs, tm, g.r.Rinf15[i]);
}

void aux_viscosity_rings(const DevGrid &g, const ViscParams &v, cudaStream_t s)
{
  k_viscosity_rings<<<(g.nr + 127) / 128, 128, 0, s>>>(g, v);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// PebbleStokesNumbers (Pebbles.c:280-300).
__global__ void k_stokes(DevGrid g, const double *__restrict__ rho, const double *__restrict__ psize,
                         double *__restrict__ tau)
{
  const int ns = g.ns;
  CELL_LOOP_2D
  tau[l] = div_fast(2.0 * g.k.pebbulkdens * psize[l], rho[l]) * g.k.sqrt_adiabind_inv;
}

void aux_stokes(const DevGrid &g, const double *rho, const double *psize, double *tau, cudaStream_t s)
{
  k_stokes<<<grid2d(g.ns, g.nr, BX), BX, 0, s>>>(g, rho, psize, tau);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// CFL: ConditionCFL (SourceEuler.c:589-712) and CriticalCharTime
// (Pebbles.c:729-767).  Because x -> CFLSECURITY/sqrt((x + a) + b) is
// monotone, the minimum over cells of the per-cell step equals the step of
// the cell with the largest sum of squared rates, so block maxima of that
// sum are reduced (exactly, in any order) and the step is formed once.

#define CFL_CPT 4       // cells per thread

// The sums of squared rates are >= 0, so their maxima are taken on the bit
// patterns as 64-bit integers (same order, integer pipe).
struct OpMaxI64 { __device__ long long operator()(long long a, long long b) const { return b > a ? b : a; } };

__global__ void __launch_bounds__(256) k_cfl_cells(DevGrid g, const double *__restrict__ vr,
                                                   const double *__restrict__ vt, const double *__restrict__ cs,
                                                   const double *__restrict__ pvr, const double *__restrict__ pvt,
                                                   CflRings cr, int pebbles, int fast, int viscous,
                                                   double *__restrict__ part)
{
  const int ns = g.ns;
  const int i = blockIdx.y + 1;                    // rings One_or_active .. Max_or_active-1
  const double dxrad = cr.dxrad[i], dxtheta = cr.dxtheta[i], mindx = cr.mindx[i];
  const double invdt5 = viscous ? div_fast(g.r.nu_med[i] * 4., cr.den5[i]) : 1e-30;
  // the per-cell rates divide by ring constants: multiply by their reciprocals
  const double idxrad = div_fast(1.0, dxrad), idxtheta = div_fast(1.0, dxtheta), imindx = div_fast(1.0, mindx);
  long long gas = 0, peb = 0;
  for (int m = 0; m < CFL_CPT; m++) {
    const int j = (blockIdx.x * CFL_CPT + m) * blockDim.x + threadIdx.x;
    if (j >= ns) break;
    const int l = j + i * ns, lip = l + ns;
    const int ljp = (j == ns - 1) ? i * ns : l + 1;
    const double vres = fast ? vt[l] - cr.vmoy[i] : vt[l];
    const double invdt1 = cs[l] * imindx;
    const double invdt2 = fabs(vr[l]) * idxrad;
    const double invdt3 = fabs(vres) * idxtheta;
    double dvr = vr[lip] - vr[l], dvt = vt[ljp] - vt[l];
    dvr = (dvr >= 0.0) ? 1e-10 : -dvr;
    dvt = (dvt >= 0.0) ? 1e-10 : -dvt;
    const double a = dvr * idxrad, b = dvt * idxtheta;
    double invdt4 = (b > a) ? b : a;
    invdt4 *= 4.0 * TH_CVNR * TH_CVNR;
    const double sg = invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 + invdt4 * invdt4 + invdt5 * invdt5;
    const long long bg = __double_as_longlong(sg);
    gas = bg > gas ? bg : gas;
    if (pebbles) {
      const double p1 = fabs(pvr[l]) * idxrad;
      const double vrp = fast ? pvt[l] - cr.pvtmed[i] : pvt[l];
      const double p2 = fabs(vrp) * idxtheta;
      const double p3 = fabs(pvr[l] - vr[l]) * idxrad;
      const double p4 = fabs(pvt[l] - vt[l]) * idxtheta;
      const long long bp = __double_as_longlong(p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4);
      peb = bp > peb ? bp : peb;
    }
  }
  const long long mg = block_reduce(gas, OpMaxI64(), 0LL);
  const long long mp = pebbles ? block_reduce(peb, OpMaxI64(), 0LL) : 0LL;
  if (threadIdx.x == 0) {
    const int b = blockIdx.x + blockIdx.y * gridDim.x;
    part[2 * b] = __longlong_as_double(mg);
    part[2 * b + 1] = pebbles ? __longlong_as_double(mp) : -1.0e30;
  }
}

__global__ void __launch_bounds__(1024) k_cfl_final(DevGrid g, const double *__restrict__ part, CflRings cr, CflFinal f,
                            double *__restrict__ scal, int *__restrict__ iscal)
{
  // the remaining part of the DT and MinStepForRebound's rate come from the
  // disk's control block; so does the CFL's substep length, written back
  const double deltaT = g.ctl[CTL_DELTAT], invdtreb_sq = g.ctl[CTL_INVDTREB];
  double mg = 0.0, mp = -1.0e30, shear = 1e30;
  for (int b = threadIdx.x; b < f.nb; b += blockDim.x) {
    const double a = part[2 * b], c = part[2 * b + 1];
    if (a > mg) mg = a;
    if (c > mp) mp = c;
  }
  for (int i = threadIdx.x; i < g.nr - 1; i += blockDim.x) {
    const double dt = f.twopi_cfl_ns / fabs(cr.vmoy[i] * g.r.InvRmed[i] - cr.vmoy[i + 1] * g.r.InvRmed[i + 1]);
    if (dt < shear) shear = dt;
  }
  mg = block_reduce(mg, OpMax(), 0.0);
  mp = block_reduce(mp, OpMax(), -1.0e30);
  shear = block_reduce(shear, OpMin(), 1e30);
  if (threadIdx.x == 0) {
    double newdt;
    if (!f.pebbles) newdt = TH_CFLSECURITY / sqrt(mg + invdtreb_sq);
    else newdt = TH_CFLSECURITY / sqrt(mg + mp + invdtreb_sq);
    if (newdt > 1e30) newdt = 1e30;
    if (shear < newdt) newdt = shear;
    const double dts = scal[SC_DTSTELLAR];
    if (newdt > dts) {
      const double m = (1.0 * dts > f.minimum_step) ? 1.0 * dts : f.minimum_step;
      newdt = (newdt < m) ? newdt : m;
    }
    newdt = (newdt < f.maximum_step) ? newdt : f.maximum_step;
    if (f.first_call && f.first_step > 0.0) newdt = f.first_step;
    if (deltaT < newdt) newdt = deltaT;
    scal[SC_NEWDT] = newdt;
    scal[SC_INVDTPEB] = mp;
    const int n = (int)(ceil(deltaT / newdt));
    iscal[IS_NSUB] = n;
    g.ctl[CTL_DT] = deltaT / (double)n;
  }
}

void aux_cfl(const DevGrid &g, const double *vr, const double *vt, const double *cs, const double *pvr, const double *pvt,
             const CflRings &cr, int pebbles, int fast, int viscous, double *part, const CflFinal &f0, double *scal,
             int *iscal, cudaStream_t s)
{
  if (pebbles && fast) aux_ring_means(g, vt, cr.vmoy, pvt, cr.pvtmed, 0, g.nr, s);
  else aux_ring_means(g, vt, cr.vmoy, nullptr, nullptr, 0, g.nr, s);
  dim3 grid = grid2d(g.ns, g.nr - 1, 256 * CFL_CPT);
  k_cfl_cells<<<grid, 256, 0, s>>>(g, vr, vt, cs, pvr, pvt, cr, pebbles, fast, viscous, part);
  g_thorin_launches++;
  CflFinal f = f0;
  f.nb = grid.x * grid.y;
  k_cfl_final<<<1, 1024, 0, s>>>(g, part, cr, f, scal, iscal);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// EvaporatePebbles (Pebbles.c:834-864).
__global__ void k_evaporate(DevGrid g, const double *__restrict__ T, double *__restrict__ pdens)
{
  const double facc = g.ctl[CTL_FACC_EVAP];
  const int ns = g.ns;
  CELL_LOOP_2D
  if (T[l] > g.k.evaptemp) {
    double d = pdens[l] * (1.0 - facc);
    if (d < 1.0e-8) d = 1.0e-8;
    pdens[l] = d;
  }
}

void aux_evaporate(const DevGrid &g, const double *T, double *pdens, cudaStream_t s)
{
  k_evaporate<<<grid2d(g.ns, g.nr, BX), BX, 0, s>>>(g, T, pdens);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// Damping boundaries (DampingBoundary, SideEuler.c:368-419, and DampPebbles,
// SideEuler.c:423-456).  Only rings inside the damping zones are launched.
__global__ void k_damp_gas(DevGrid g, double *__restrict__ vrad, double *__restrict__ rho, double *__restrict__ vtheta,
                           double *__restrict__ energy, const int *__restrict__ rings, const double *__restrict__ vr0r, int damp_init, int damp_flux, int energy_eq)
{
  const double dt = g.ctl[CTL_DT], omega_frame = g.ctl[CTL_OMEGA_FRAME];
  const int ns = g.ns;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ns) return;
  const int i = rings[blockIdx.y];
  const int l = j + i * ns;
  const double lambda = g.r.WaveKiller[i] * dt;
  const double vrad0 = damp_flux ? vr0r[i] : 0.0;
  vrad[l] = div_fast(vrad[l] + lambda * vrad0, 1.0 + lambda);
  if (damp_init) {
    const double rho0 = g.r.SigmaMed[i], e0 = g.r.EnergyMed[i];
    const double vt0 = g.r.VthetaMed[i] - g.r.Rmed[i] * omega_frame;
    rho[l] = div_fast(rho[l] + lambda * rho0, 1.0 + lambda);
    vtheta[l] = div_fast(vtheta[l] + lambda * vt0, 1.0 + lambda);
    if (energy_eq) energy[l] = div_fast(energy[l] + lambda * e0, 1.0 + lambda);
  }
  if (damp_flux) rho[l] = div_fast(rho[l] + lambda * g.r.SigmaMed[i], 1.0 + lambda);
}

void aux_damp_gas(const DevGrid &g, double *vrad, double *rho, double *vtheta, double *energy, const int *rings,
                  int nrings, const double *vr0r, int damp_init, int damp_flux,
                  int energy_eq, cudaStream_t s)
{
  if (nrings <= 0) return;
  k_damp_gas<<<grid2d(g.ns, nrings, BX), BX, 0, s>>>(g, vrad, rho, vtheta, energy, rings, vr0r,
                                                     damp_init, damp_flux, energy_eq);
  g_thorin_launches++;
}

// Isothermal equation of state (ComputeSoundSpeed, ComputePressureField,
// ComputeTemperatureField without the energy equation, SourceEuler.c:
// 715-792): c_s is the ring profile AspectRatio(r) sqrt(G/r) r^f, P = Sigma
// c_s^2, T = mu P / (Sigma R).  Each part is done only when asked for: the
// reference forms P at the start of a substep and T from that P and the
// transported Sigma at its end.
__global__ void k_iso_eos(DevGrid g, const double *__restrict__ rho, const double *__restrict__ csr,
                          double *__restrict__ cs, double *__restrict__ press, double *__restrict__ temper, int set_cs,
                          int set_press, int set_temper)
{
  const int ns = g.ns;
  CELL_LOOP_2D
  if (set_cs) cs[l] = csr[i];
  if (set_press) press[l] = rho[l] * cs[l] * cs[l];
  if (set_temper) temper[l] = (1.0 * press[l]) * div_fast(1.0, rho[l] * 1.0);
}

void aux_iso_eos(const DevGrid &g, const double *rho, const double *csr, double *cs, double *press, double *temper,
                 int set_cs, int set_press, int set_temper, cudaStream_t s)
{
  k_iso_eos<<<grid2d(g.ns, g.nr, BX), BX, 0, s>>>(g, rho, csr, cs, press, temper, set_cs, set_press, set_temper);
  g_thorin_launches++;
}

__global__ void k_damp_peb(DevGrid g, double *__restrict__ pd, double *__restrict__ pvr, double *__restrict__ pvt,
                           const int *__restrict__ rings)
{
  const double dt = g.ctl[CTL_DT], omega_frame = g.ctl[CTL_OMEGA_FRAME];
  const int ns = g.ns;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ns) return;
  const int i = rings[blockIdx.y];
  const int l = j + i * ns;
  const double lambda = g.r.WaveKiller[i] * dt;
  const double d0 = g.r.PebDensInit[i], vr0 = g.r.PebVradInit[i];
  const double vt0 = g.r.PebVthetaInit[i] - g.r.Rmed[i] * omega_frame;
  pd[l] = div_fast(pd[l] + lambda * d0, 1.0 + lambda);
  pvr[l] = div_fast(pvr[l] + lambda * vr0, 1.0 + lambda);
  pvt[l] = div_fast(pvt[l] + lambda * vt0, 1.0 + lambda);
}

void aux_damp_peb(const DevGrid &g, double *pd, double *pvr, double *pvt, const int *rings, int nrings, cudaStream_t s)
{
  if (nrings <= 0) return;
  k_damp_peb<<<grid2d(g.ns, nrings, BX), BX, 0, s>>>(g, pd, pvr, pvt, rings);
  g_thorin_launches++;
}

// DetectCrash (SourceEuler.c:48-66): any negative value in rows 0..nr-1.
__global__ void k_crash(int n, const double *__restrict__ f, int *flag)
{
  int bad = 0;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n; l += gridDim.x * blockDim.x)
    if (f[l] < 0.0) bad = 1;
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

void aux_crash(const DevGrid &g, const double *f, int *flag, cudaStream_t s)
{
  const int n = g.nr * g.ns;
  int blocks = (n + 255) / 256;
  if (blocks > 1216) blocks = 1216;
  k_crash<<<blocks, 256, 0, s>>>(n, f, flag);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// SourceTermsPebbles (Pebbles.c:550-613), after DampPebbles.
__global__ void k_pebble_sources(DevGrid g, const double *__restrict__ pd, const double *__restrict__ pvr,
                                 const double *__restrict__ pvt, const double *__restrict__ tau,
                                 const double *__restrict__ vr, const double *__restrict__ vt,
                                 const double *__restrict__ pagr, const double *__restrict__ pagt,
                                 double *__restrict__ paccr, double *__restrict__ pacct, double *__restrict__ dragr,
                                 double *__restrict__ dragt, int back_reaction)
{
  const double omega_frame = g.ctl[CTL_OMEGA_FRAME];
  const int ns = g.ns;
  CELL_LOOP_2D
  const double Omega = g.r.Omega[i];
  const int ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
  const double otau = back_reaction ? div_fast(Omega, tau[l]) : 0.0;    // Omega / tau_s
  if (i >= 1) {
    const int lim = l - ns;
    const int ljp = (j == ns - 1) ? i * ns : l + 1;
    double vt2 = pvt[l] + pvt[ljp] + pvt[lim] + pvt[ljp - ns];
    vt2 = vt2 / 4.0 + g.r.Rinf[i] * omega_frame;
    vt2 = vt2 * vt2;
    paccr[l] = vt2 * g.r.InvRinf[i] + 0.5 * (pagr[l] + pagr[lim]);
    if (back_reaction) {
      const double drag = (pvr[l] - vr[l]) * otau;
      dragr[l] = 0.5 * (pd[l] + pd[lim]) * drag;
    }
  }
  pacct[l] = 0.5 * (pagt[l] + pagt[ljm]);
  if (back_reaction) {
    const double drag = (pvt[l] - vt[l]) * otau;
    dragt[l] = 0.5 * (pd[l] + pd[ljm]) * drag;
  }
}

void aux_pebble_sources(const DevGrid &g, const double *pd, const double *pvr, const double *pvt, const double *tau,
                        const double *vr, const double *vt, const double *pagr, const double *pagt, double *paccr,
                        double *pacct, double *dragr, double *dragt, int back_reaction,
                        cudaStream_t s)
{
  k_pebble_sources<<<grid2d(g.ns, g.nr, BX), BX, 0, s>>>(g, pd, pvr, pvt, tau, vr, vt, pagr, pagt, paccr, pacct, dragr,
                                                         dragt, back_reaction);
  g_thorin_launches++;
}

// SubStep1Pebbles (Pebbles.c:617-652) followed by ParticleDiffusion
// (Pebbles.c:656-698): both only change the pebble velocities of cell l.
__global__ void k_pebble_substep1(DevGrid g, double *__restrict__ pvr, double *__restrict__ pvt,
                                  const double *__restrict__ tau, const double *__restrict__ vr,
                                  const double *__restrict__ vt, const double *__restrict__ paccr,
                                  const double *__restrict__ pacct, const double *__restrict__ gaccr,
                                  const double *__restrict__ gacct, const double *__restrict__ rho,
                                  const double *__restrict__ pd, int diffusion, double schmidt,
                                  const double *__restrict__ invdxtheta_r)
{
  const double dt = g.ctl[CTL_DT];
  const int ns = g.ns;
  CELL_LOOP_2D
  const double Omega = g.r.Omega[i];
  const double t = tau[l];
  const double efac = exp(div_fast(-dt * Omega, t));
  double a = pvr[l], b = pvt[l];
  const double oinv = g.r.OmegaInv[i];               // x / Omega as x * OmegaInv
  if (i > 0) a = a * efac + gaccr[l] * dt + (vr[l] + (paccr[l] - gaccr[l]) * t * oinv) * (1.0 - efac);
  b = b * efac + gacct[l] * dt + (vt[l] + (pacct[l] - gacct[l]) * t * oinv) * (1.0 - efac);
  if (diffusion) {
    if (i >= 1) {
      const int lim = l - ns;
      double corr = div_fast(-g.r.nu_inf[i], schmidt);
      corr *= div_fast(rho[l] + rho[lim], pd[l] + pd[lim]);
      corr *= (div_fast(pd[l], rho[l]) - div_fast(pd[lim], rho[lim])) * g.r.InvDiffRmed[i];
      a += corr;
    }
    const int ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
    double corr = div_fast(-g.r.nu_med[i], schmidt);
    corr *= div_fast(rho[l] + rho[ljm], pd[l] + pd[ljm]);
    corr *= (div_fast(pd[l], rho[l]) - div_fast(pd[ljm], rho[ljm])) * invdxtheta_r[i];
    b += corr;
  }
  pvr[l] = a;
  pvt[l] = b;
}

void aux_pebble_substep1(const DevGrid &g, double *pvr, double *pvt, const double *tau, const double *vr, const double *vt,
                         const double *paccr, const double *pacct, const double *gaccr, const double *gacct,
                         const double *rho, const double *pd, int diffusion, double schmidt,
                         const double *invdxtheta_r, cudaStream_t s)
{
  k_pebble_substep1<<<grid2d(g.ns, g.nr, BX), BX, 0, s>>>(g, pvr, pvt, tau, vr, vt, paccr, pacct, gaccr, gacct, rho, pd, diffusion, schmidt, invdxtheta_r);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// FillForcesArrays (Pframeforce.c:43-510).  Per ring: the azimuthal mean
// sound speed and Stokes number (sums in order) and the 10-node vertical
// averages of the star's pull for the ring-mean scale height.

__global__ void k_force_rings(DevGrid g, ForceRings fr, int pebbles, double pebble_alpha)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.nr) return;
  const double cs_avr = g.r.csmean[i];       // the ring mean of c_s, summed in order
  const double H_avr = cs_avr * g.r.OmegaInv[i] * g.k.sqrt_adiabind_inv;
  double tau_avr = 0.0, p_H_avr = 0.0, p_int = 0.0;
  if (pebbles) {
    tau_avr = fr.tau_avr[i];
    p_H_avr = H_avr * sqrt(pebble_alpha / tau_avr);
  }
  const double r2 = g.r.Rmed2[i];
  const double H2 = H_avr * H_avr, zmax = 3.0 * H_avr, deltaz = zmax / 10.0;
  double sig = 0.0, ist = 0.0;
  for (int m = 1; m <= 10; m++) {
    const double znode = ((double)m - 0.5) * deltaz;
    double znode2 = znode * znode;
    const double sum = exp(-(0.5 * znode2 / H2));
    sig += sum;
    double d2 = r2 + znode2, d = sqrt(d2), denom = d * d2;
    ist += sum / denom;
    if (pebbles) {
      znode2 *= pebble_alpha / tau_avr;
      d2 = r2 + znode2; d = sqrt(d2); denom = d * d2;
      p_int += sum / denom;
    }
  }
  fr.H_avr[i] = H_avr;
  fr.sigma_avr[i] = sig;
  fr.isigma_avr[i] = div_fast(1.0, sig);
  fr.integstar_avr[i] = ist;
  fr.p_H_avr[i] = p_H_avr;
  fr.p_integstar_avr[i] = p_int;
}

// One quadrature node of a planet's potential (FillForcesArrays,
// Pframeforce.c:300-372): cubic-spline taper inside rst, softened 1/d^3.
__device__ __forceinline__ double planet_node(double s2, double dz, double mx, const DevPlanet &P)
{
  double d2 = s2 + dz * dz, taper = 1.0;
  if (d2 < P.rst2) {
    const double dd = sqrt(d2);
    taper = div_fast(-3.0 * d2 * d2, P.rst4) + div_fast(4.0 * dd * d2, P.rst3);
  }
  const double iv = rsqrt(d2 + mx);
  return iv * iv * iv * taper;
}

// Vertical quadrature of one cell (FillForcesArrays, Pframeforce.c:260-372)
// over NV nodes z_m = (m - 1/2) 3H/NV.  The Gaussian weights depend only on
// m and NV and come precomputed; 1/d^3 comes from one reciprocal square root.
template <int NV>
__device__ __forceinline__ void vert_quad(const double (&wq)[NV], double H, double r2, double Hcorr, double pH, int peb,
                                          int npl, const int *with, const double *s2, double Rsup_Rinf2,
                                          const DevPlanet *pl, double &integstar, double &p_integstar,
                                          double *integpl, double *p_integpl)
{
  const double deltaz = 3.0 * H / (double)NV;
  const double hc2 = Hcorr * Hcorr;
  double is = 0.0, pis = 0.0;
#pragma unroll
  for (int m = 1; m <= NV; m++) {
    const double znode = ((double)m - 0.5) * deltaz, znode2 = znode * znode;
    const double sum = wq[m - 1];
    double iv = rsqrt(r2 + znode2);
    is += sum * iv * iv * iv;
    if (peb) {
      iv = rsqrt(r2 + znode2 * hc2);
      pis += sum * iv * iv * iv;
    }
    for (int k = 0; k < npl; k++) {
      if (!with[k]) continue;
      const DevPlanet P = pl[k];
      const double mx = (P.rsm2 > Rsup_Rinf2) ? P.rsm2 : Rsup_Rinf2;
      integpl[k] += sum * planet_node(s2[k], znode - P.z, mx, P);
      if (P.z < -0.05 * H || P.z > 0.05 * H) integpl[k] += sum * planet_node(s2[k], -znode - P.z, mx, P);
      if (peb) {
        const double zp = znode * Hcorr;
        p_integpl[k] += sum * planet_node(s2[k], zp - P.z, mx, P);
        if (P.z < -0.05 * pH || P.z > 0.05 * pH) p_integpl[k] += sum * planet_node(s2[k], -zp - P.z, mx, P);
      }
    }
  }
  integstar = is;
  p_integstar = pis;
}

#define FORCE_CPT 4     // cells per thread: one block reduction per 4*128 cells

__global__ void __launch_bounds__(128) k_forces(DevGrid g, ForceArgs a, ForceRings fr)
{
  const double mass_taper = g.ctl[CTL_MASS_TAPER];
  const int full_mass = (mass_taper == 1.0) ? 1 : 0;
  const int ns = g.ns;
  const int i = blockIdx.y;
  const int npl = a.npl, peb = a.pebbles;
  double acc[2 + 2 * MAXPL_DEV];
  for (int q = 0; q < 2 + 2 * npl; q++) acc[q] = 0.0;
  for (int mc = 0; mc < FORCE_CPT; mc++) {
    const int j = (blockIdx.x * FORCE_CPT + mc) * blockDim.x + threadIdx.x;
    if (j >= ns) break;
    const int l = j + i * ns;
    const double omegainv = g.r.OmegaInv[i], r2 = g.r.Rmed2[i];
    const double Rsup_Rinf2 = fr.drsq[i];
    const double x = g.r.Rmed[i] * g.r.costab[j];
    const double y = g.r.Rmed[i] * g.r.sintab[j];
    const double mcell = a.rho[l] * g.r.Surf[i];
    const double H = a.cs[l] * omegainv * g.k.sqrt_adiabind_inv;
    const double H_avr = fr.H_avr[i];
    int local = (fabs(H - H_avr) > 0.05 * H_avr) ? 1 : 0;      // |H - H_avr| / H_avr > 0.05
    double Hcorr = 0.0, pH = 0.0, pmcell = 0.0;
    if (peb) {
      pmcell = a.pdens[l] * g.r.Surf[i];
      Hcorr = a.sqrt_pebble_alpha * rsqrt(a.tau[l]);        // sqrt(alpha / tau) without the division
      pH = H * Hcorr;
      const double p_H_avr = fr.p_H_avr[i];
      if (fabs(pH - p_H_avr) > 0.05 * p_H_avr) local = 1;
    }
    double s2[MAXPL_DEV], integpl[MAXPL_DEV], p_integpl[MAXPL_DEV], hillcut[MAXPL_DEV];
    int with[MAXPL_DEV];
    int Nvert = 10;
    for (int k = 0; k < npl; k++) {
      const DevPlanet P = a.pl[k];
      s2[k] = (x - P.x) * (x - P.x) + (y - P.y) * (y - P.y);
      hillcut[k] = 1.0;
      integpl[k] = 0.0;
      p_integpl[k] = 0.0;
      if (full_mass && (s2[k] < P.near_h2 || s2[k] < P.near_hill2)) {
        local = 1;
        with[k] = 1;
        if (a.exclude_hill) {
          const double d2 = s2[k] + P.z * P.z;
          hillcut[k] = 1.0 / (exp(-(sqrt(d2) / P.rhill - a.hillcut) / a.hillcut * 10.0) + 1.0);
        }
      } else {
        with[k] = 0;
      }
      if (s2[k] < P.rmorevert2) Nvert = 30;
    }
    double isig, integstar, p_integstar = 0.0;       // 1 / sigma from tables
    if (local) {
      if (Nvert == 10) {
        isig = a.isig10;
        vert_quad<10>(a.wq10, H, r2, Hcorr, pH, peb, npl, with, s2, Rsup_Rinf2, a.pl, integstar, p_integstar,
                      integpl, p_integpl);
      } else {
        isig = a.isig30;
        vert_quad<30>(a.wq30, H, r2, Hcorr, pH, peb, npl, with, s2, Rsup_Rinf2, a.pl, integstar, p_integstar,
                      integpl, p_integpl);
      }
    } else {
      isig = fr.isigma_avr[i];
      integstar = fr.integstar_avr[i];
      if (peb) p_integstar = fr.p_integstar_avr[i];
    }
    double tmp = integstar * isig;
    double agr = -g.r.Rmed[i] * tmp;            // 0.0 + ar
    acc[0] += mcell * tmp * x;
    acc[1] += mcell * tmp * y;
    double pagr = 0.0;
    if (peb) { const double pt = p_integstar * isig; pagr = -g.r.Rmed[i] * pt; }
    double ax = 0.0, ay = 0.0, pax = 0.0, pay = 0.0;
    for (int k = 0; k < npl; k++) {
      const DevPlanet P = a.pl[k];
      double mpl = P.m;
      if (with[k]) {
        const bool off = (P.z < -0.05 * H || P.z > 0.05 * H);
        tmp = (x - P.x) * integpl[k] * (off ? 0.5 * isig : isig);
        ax += -mpl * tmp;
        if (a.exclude_hill) tmp *= hillcut[k];
        acc[2 + 2 * k] += mcell * tmp;
        tmp = (y - P.y) * integpl[k] * (off ? 0.5 * isig : isig);
        ay += -mpl * tmp;
        if (a.exclude_hill) tmp *= hillcut[k];
        acc[3 + 2 * k] += mcell * tmp;
        if (peb) {
          const bool poff = (P.z < -0.05 * pH || P.z > 0.05 * pH);
          tmp = (x - P.x) * p_integpl[k] * (poff ? 0.5 * isig : isig);
          pax += -mpl * tmp;
          if (a.pebble_gravity) { if (a.exclude_hill) tmp *= hillcut[k]; acc[2 + 2 * k] += pmcell * tmp; }
          tmp = (y - P.y) * p_integpl[k] * (poff ? 0.5 * isig : isig);
          pay += -mpl * tmp;
          if (a.pebble_gravity) { if (a.exclude_hill) tmp *= hillcut[k]; acc[3 + 2 * k] += pmcell * tmp; }
        }
      } else {
        mpl *= mass_taper;
        double d2 = s2[k] + P.z * P.z + P.smoothing2, iv = rsqrt(d2), id3 = iv * iv * iv;
        tmp = (x - P.x) * id3;
        ax += -mpl * tmp;
        if (a.exclude_hill) tmp *= hillcut[k];
        acc[2 + 2 * k] += mcell * tmp;
        tmp = (y - P.y) * id3;
        ay += -mpl * tmp;
        if (a.exclude_hill) tmp *= hillcut[k];
        acc[3 + 2 * k] += mcell * tmp;
        if (peb) {
          d2 += -P.smoothing2 + P.smoothing2 * Hcorr * Hcorr;
          iv = rsqrt(d2); id3 = iv * iv * iv;
          tmp = (x - P.x) * id3;
          pax += -mpl * tmp;
          if (a.pebble_gravity) { if (a.exclude_hill) tmp *= hillcut[k]; acc[2 + 2 * k] += pmcell * tmp; }
          tmp = (y - P.y) * id3;
          pay += -mpl * tmp;
          if (a.pebble_gravity) { if (a.exclude_hill) tmp *= hillcut[k]; acc[3 + 2 * k] += pmcell * tmp; }
        }
      }
    }
    const double ir = g.r.InvRmed[i];
    a.agr[l] = agr + (x * ax + y * ay) * ir;
    a.agt[l] = 0.0 + (x * ay - y * ax) * ir;
    if (peb) {
      a.pagr[l] = pagr + (x * pax + y * pay) * ir;
      a.pagt[l] = 0.0 + (x * pay - y * pax) * ir;
    }
  }
  const int nq = 2 + 2 * npl;
  const int b = blockIdx.x + blockIdx.y * gridDim.x;
  for (int q = 0; q < nq; q++) {
    const double v = block_reduce_smem<128>(acc[q], OpAdd());
    if (threadIdx.x == 0) a.part[(size_t)b * nq + q] = v;
  }
}

__global__ void __launch_bounds__(1024) k_forces_final(const double *__restrict__ part, int nb, int nq, double *__restrict__ scal)
{
  // one block; quantity q summed over blocks in a fixed order
  for (int q = 0; q < nq; q++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[(size_t)b * nq + q];
    s = block_reduce(s, OpAdd(), 0.0);
    if (threadIdx.x == 0) {
      if (q == 0) scal[SC_INDX] = -s;
      else if (q == 1) scal[SC_INDY] = -s;
      else scal[SC_PLANET_A + (q - 2)] = s;
    }
    __syncthreads();
  }
}

// Indirect term added to every cell (Pframeforce.c:488-509).
__global__ void k_forces_indirect(DevGrid g, double *__restrict__ agr, double *__restrict__ agt,
                                  double *__restrict__ pagr, double *__restrict__ pagt, const double *__restrict__ scal, int pebbles)
{
  const double indx_pl = g.ctl[CTL_INDX_PL], indy_pl = g.ctl[CTL_INDY_PL];
  const int ns = g.ns;
  CELL_LOOP_2D
  const double axi = scal[SC_INDX] + indx_pl, ayi = scal[SC_INDY] + indy_pl;
  const double x = g.r.Rmed[i] * g.r.costab[j], y = g.r.Rmed[i] * g.r.sintab[j];
  const double ar = (x * axi + y * ayi) * g.r.InvRmed[i];
  const double at = (x * ayi - y * axi) * g.r.InvRmed[i];
  agr[l] += ar;
  agt[l] += at;
  if (pebbles) { pagr[l] += ar; pagt[l] += at; }
}

void aux_forces(const DevGrid &g, const ForceArgs &a0, const ForceRings &fr,
                double *scal, cudaStream_t s)
{
  if (a0.pebbles) aux_ring_means(g, a0.tau, fr.tau_avr, nullptr, nullptr, 0, g.nr, s);
  k_force_rings<<<(g.nr + 127) / 128, 128, 0, s>>>(g, fr, a0.pebbles, a0.pebble_alpha);
  g_thorin_launches++;
  ForceArgs a = a0;
  for (int pass = 0; pass < 2; pass++) {
    const int nv = pass ? 30 : 10;
    double *w = pass ? a.wq30 : a.wq10, sig = 0.0;
    const double deltaz = 3.0 / (double)nv;          // H = 1
    for (int m = 1; m <= nv; m++) {
      const double z = ((double)m - 0.5) * deltaz;
      w[m - 1] = exp(-(0.5 * (z * z)));
      sig += w[m - 1];
    }
    if (pass) { a.sig30 = sig; a.isig30 = 1.0 / sig; }
    else { a.sig10 = sig; a.isig10 = 1.0 / sig; }
  }
  dim3 grid = grid2d(g.ns, g.nr, 128 * FORCE_CPT);
  k_forces<<<grid, 128, 0, s>>>(g, a, fr);
  g_thorin_launches++;
  k_forces_final<<<1, 1024, 0, s>>>(a0.part, grid.x * grid.y, 2 + 2 * a0.npl, scal);
  g_thorin_launches++;
  k_forces_indirect<<<grid2d(g.ns, g.nr, BX), BX, 0, s>>>(g, a0.agr, a0.agt, a0.pagr, a0.pagt, scal,
                                                          a0.pebbles);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// AccretePebblesOntoPlanets for one planet (Pebbles.c:353-539), one block.
// The annulus [imin, imax] holding the Hill sphere is searched; cells within
// the effective accretion radius give up pebbles up to the model rate.

// Trapzd and IntegrateColumnMass (Pebbles.c:302-349) for one cell, evaluated
// by a whole warp: the it = 2^(n-2) midpoints of level n are spread over the
// lanes (lane k takes points k, k + 32, ...), point j at a + (j + 1/2)
// spacing, and the level's sum is an xor butterfly over the lanes' partial
// sums, so every lane holds the same bits of the integral and takes the same
// exit.  The levels, the refinement integral = (integral + (b - a) sum / it)
// / 2 and the exit test after level 5 are the reference's; only the order of
// the midpoint sum and the rounding of the abscissae differ from its
// sequential loop (x += spacing), by relative amounts of order 1e-16.  Before
// this the reference's loop ran in one thread per cell, up to 2^14
// dependent exponentials each.
__device__ double column_mass_warp(double a, double b, double Hpeb)
{
  const int lane = threadIdx.x & 31;
  const double H2 = Hpeb * Hpeb;
  double integral = 0.5 * (b - a) * (exp(div_fast(-0.5 * a * a, H2)) + exp(div_fast(-0.5 * b * b, H2)));
  double iold = integral;
  for (int n = 2; n <= 16; n++) {
    const int it = 1 << (n - 2);
    const double iter = it, spacing = (b - a) / iter;
    double sum = 0.0;
    for (int j = lane; j < it; j += 32) {
      const double x = a + ((double)j + 0.5) * spacing;
      sum += exp(div_fast(-0.5 * x * x, H2));
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) sum += __shfl_xor_sync(TH_FULL, sum, o);
    integral = 0.5 * (integral + (b - a) * sum / iter);
    if (n > 5)
      if (fabs(integral - iold) < 1.0e-4 * fabs(iold) || (integral == 0.0 && iold == 0.0)) return integral;
    iold = integral;
  }
  return __longlong_as_double(0x7ff8000000000000ULL);   // the reference aborts here
}

// The annulus work runs on many blocks in three grid passes (mean Stokes
// number, upper limits per cell, application of the limiter), each followed
// by a one-block kernel that sums the block partials in a fixed order and
// does the scalar steps of the reference.
// acc[] scalars: 0 Reff, 1 vrel, 2 Mt, 3 limiter.

__global__ void __launch_bounds__(ACC_BX) k_acc_tau(DevGrid g, const AccArgs *__restrict__ ap)
{
  const AccArgs &a = *ap;
  if ((int)blockIdx.x >= a.nb) return;           // grid sized for the widest annulus
  const int ncells = (a.imax - a.imin + 1) * g.ns;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  double t = (q < ncells) ? a.tau[(size_t)a.imin * g.ns + q] : 0.0;
  t = block_reduce(t, OpAdd(), 0.0);
  if (threadIdx.x == 0) a.part[blockIdx.x] = t;
}

__global__ void __launch_bounds__(ACC_BX) k_acc_reff(DevGrid g, const AccArgs *__restrict__ ap)
{
  const AccArgs &a = *ap;
  const int nb = a.nb;
  if (nb == 0) return;                       // no annulus (only the device-resident DT launches this)
  const int ns = g.ns;
  __shared__ double sh[2];
  if (threadIdx.x == 0) {                    // vt1D at the two rings bracketing the planet
    sh[0] = a.acc[4];
    sh[1] = (a.iflow + 1 < g.nr) ? a.acc[5] : 0.0;   // vt1D[nrad] is zero in the reference
  }
  double ts = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) ts += a.part[b];
  ts = block_reduce(ts, OpAdd(), 0.0);
  if (threadIdx.x == 0) {
    const int ncells = (a.imax - a.imin + 1) * ns;
    const double tau_mean = ts / (double)ncells;
    const double flow = sh[0] * (1.0 - a.frac) + sh[1] * a.frac + a.Rp * a.omega_frame;
    const double flowx = -flow * a.Yp / a.Rp, flowy = flow * a.Xp / a.Rp;
    const double vrel = sqrt((a.VXp - flowx) * (a.VXp - flowx) + (a.VYp - flowy) * (a.VYp - flowy) + a.VZp * a.VZp);
    const double Mt = sqrt(1.0 / 3.0) * cube_rn(vrel) / a.Omegap;
    double Reff;
    if (a.Mp < Mt) {
      const double Rbondi = a.Mp / vrel / vrel, tbondi = Rbondi / vrel;
      Reff = Rbondi * sqrt(tau_mean * a.Rp15 / tbondi);
    } else {
      Reff = a.Rhill * pow(tau_mean / 0.1, 1.0 / 3.0);
    }
    if (Reff > a.Rhill) Reff = a.Rhill;
    a.acc[0] = Reff;
    a.acc[1] = vrel;
    a.acc[2] = Mt;
  }
}

// Annulus cell q (0 .. (imax - imin + 1) ns - 1) of the accretion step: true
// when its midplane distance to the planet is within the effective accretion
// radius, with the pebble scale height and the column's ends inside the
// sphere (Pebbles.c:445-453).  The operations are spelled out as
// round-to-nearest intrinsics so that the two kernels that call this get the
// same bits.
__device__ __forceinline__ bool acc_cell(const DevGrid &g, const AccArgs &a, int q, int &i, int &l, double &Hpeb,
                                         double &zmin, double &zmax)
{
  const int ns = g.ns;
  i = a.imin + q / ns;
  const int j = q - (q / ns) * ns;
  l = j + i * ns;
  const double Reff = a.acc[0], Reff2 = __dmul_rn(Reff, Reff);
  const double dx = __dsub_rn(__dmul_rn(g.r.Rmed[i], g.r.costab[j]), a.Xp);
  const double dy = __dsub_rn(__dmul_rn(g.r.Rmed[i], g.r.sintab[j]), a.Yp);
  const double R2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  if (!(R2 <= Reff2)) return false;
  const double H = __dmul_rn(__dmul_rn(a.cs[l], g.r.OmegaInv[i]), g.k.sqrt_adiabind_inv);
  Hpeb = __dmul_rn(H, __dsqrt_rn(__ddiv_rn(a.pebble_alpha, a.tau[l])));
  const double h = __dsqrt_rn(__dsub_rn(Reff2, R2));
  zmin = __dsub_rn(a.Zp, h);
  zmax = __dadd_rn(a.Zp, h);
  return true;
}

// Column integrals of the annulus cells inside the sphere (IntegrateColumnMass
// of Pebbles.c:456), one warp per cell, into macc[l] (zero outside the
// accretion step).  Warp w of the grid takes the annulus cells w, w + W,
// w + 2W, ... (W warps in all), 32 of them tested at a time, so the cells of
// the sphere, which lie together around the planet, fall on many
// multiprocessors.
__global__ void __launch_bounds__(ACC_BX) k_acc_column(DevGrid g, const AccArgs *__restrict__ ap)
{
  const AccArgs &a = *ap;
  if (a.nb == 0) return;                         // no annulus
  const int ncells = (a.imax - a.imin + 1) * g.ns;
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (ACC_BX / 32);
  const int gw = blockIdx.x * (ACC_BX / 32) + (threadIdx.x >> 5);
  for (long long base = gw; base < ncells; base += 32LL * nw) {   // warp-uniform
    const long long c = base + (long long)lane * nw;
    int i = 0, l = 0;
    double Hpeb = 0.0, zmin = 0.0, zmax = 0.0;
    const bool inside = c < ncells && acc_cell(g, a, (int)c, i, l, Hpeb, zmin, zmax);
    unsigned bal = __ballot_sync(TH_FULL, inside);
    while (bal) {
      const int src = __ffs(bal) - 1;
      bal &= bal - 1u;
      const double cm = column_mass_warp(__shfl_sync(TH_FULL, zmin, src), __shfl_sync(TH_FULL, zmax, src),
                                         __shfl_sync(TH_FULL, Hpeb, src));
      if (lane == src) a.macc[l] = cm;
    }
  }
}

// Upper limit of the mass each annulus cell inside the sphere can give up
// (Pebbles.c:454-462), from its column integral (k_acc_column), and the
// block partials of the limit, the scale height, the pebble density and the
// cell count.
__global__ void __launch_bounds__(ACC_BX) k_acc_upper(DevGrid g, const AccArgs *__restrict__ ap)
{
  const AccArgs &a = *ap;
  if ((int)blockIdx.x >= a.nb) return;           // grid sized for the widest annulus
  const int ncells = (a.imax - a.imin + 1) * g.ns;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  double dmu = 0.0, hpm = 0.0, pdm = 0.0, nc = 0.0;
  int i = 0, l = 0;
  double Hpeb = 0.0, zmin = 0.0, zmax = 0.0;
  if (q < ncells && acc_cell(g, a, q, i, l, Hpeb, zmin, zmax)) {
    const double pd = a.pdens[l];
    const double mcell = g.r.Surf[i] * pd;
    const double vdp = pd / Hpeb * g.k.sqrt2pi_inv;
    double dM = vdp * g.r.Surf[i] * a.macc[l];
    if (dM > mcell) dM = 0.99999999 * mcell;
    a.macc[l] = dM;
    dmu = dM; hpm = Hpeb; pdm = pd; nc = 1.0;
  }
  dmu = block_reduce(dmu, OpAdd(), 0.0);
  hpm = block_reduce(hpm, OpAdd(), 0.0);
  pdm = block_reduce(pdm, OpAdd(), 0.0);
  nc = block_reduce(nc, OpAdd(), 0.0);
  if (threadIdx.x == 0) {
    a.part[4 * blockIdx.x + 0] = dmu; a.part[4 * blockIdx.x + 1] = hpm;
    a.part[4 * blockIdx.x + 2] = pdm; a.part[4 * blockIdx.x + 3] = nc;
  }
}

__global__ void __launch_bounds__(ACC_BX) k_acc_limiter(const AccArgs *__restrict__ ap, double pi, double sqrt2pi_inv)
{
  const AccArgs &a = *ap;
  const int nb = a.nb;
  if (nb == 0) return;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int k = 0; k < 4; k++) v[k] += a.part[4 * b + k];
  for (int k = 0; k < 4; k++) v[k] = block_reduce(v[k], OpAdd(), 0.0);
  if (threadIdx.x == 0) {
    const double dmu = v[0];
    double Hpeb_mean = v[1], pdens_mean = v[2];
    const int nc = (int)v[3];
    if (nc > 0) { Hpeb_mean /= (double)nc; pdens_mean /= (double)nc; }
    const double Reff = a.acc[0], vrel = a.acc[1], Mt = a.acc[2];
    const double veloc = (a.Mp < Mt) ? vrel : Reff * a.Omegap;
    double dM_model;
    if (Hpeb_mean < Reff) dM_model = 2.0 * Reff * veloc * pdens_mean;
    else dM_model = pi * Reff * Reff * veloc * pdens_mean / Hpeb_mean * sqrt2pi_inv;
    dM_model *= a.dt;
    a.acc[3] = (dmu > dM_model) ? dM_model / dmu : 1.0;
  }
}

__global__ void __launch_bounds__(ACC_BX) k_acc_apply(DevGrid g, const AccArgs *__restrict__ ap)
{
  const AccArgs &a = *ap;
  if ((int)blockIdx.x >= a.nb) return;           // grid sized for the widest annulus
  const int ns = g.ns;
  const int ncells = (a.imax - a.imin + 1) * ns;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const double limiter = a.acc[3];
  double dM_s = 0.0, dPx = 0.0, dPy = 0.0;
  if (q < ncells) {
    const int i = a.imin + q / ns, j = q - (q / ns) * ns, l = j + i * ns;
    if (a.macc[l] > 0.0) {
      const double xc = g.r.Rmed[i] * g.r.costab[j], yc = g.r.Rmed[i] * g.r.sintab[j];
      const double vtcorr = g.r.Rmed[i] * a.omega_frame;
      const double vrc = a.pvr[l], vtc = a.pvt[l] + vtcorr;
      const double vxc = (vrc * xc - vtc * yc) * g.r.InvRmed[i], vyc = (vrc * yc + vtc * xc) * g.r.InvRmed[i];
      const double dM = a.macc[l] * limiter;
      a.macc[l] = 0.0;
      const double mcell = g.r.Surf[i] * a.pdens[l];
      double pd = (mcell - dM) / g.r.Surf[i];
      if (pd < 0.0) pd = 1.e-20;
      a.pdens[l] = pd;
      dM_s = dM; dPx = dM * vxc; dPy = dM * vyc;
    }
  }
  dM_s = block_reduce(dM_s, OpAdd(), 0.0);
  dPx = block_reduce(dPx, OpAdd(), 0.0);
  dPy = block_reduce(dPy, OpAdd(), 0.0);
  if (threadIdx.x == 0) {
    a.part[3 * blockIdx.x + 0] = dM_s; a.part[3 * blockIdx.x + 1] = dPx; a.part[3 * blockIdx.x + 2] = dPy;
  }
}

__global__ void __launch_bounds__(ACC_BX) k_acc_sum(const AccArgs *__restrict__ ap, double *__restrict__ scal)
{
  const AccArgs &a = *ap;
  const int nb = a.nb;
  double v[3] = {0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int k = 0; k < 3; k++) v[k] += a.part[3 * b + k];
  for (int k = 0; k < 3; k++) v[k] = block_reduce(v[k], OpAdd(), 0.0);
  if (threadIdx.x == 0) { scal[SC_ACC_DM] = v[0]; scal[SC_ACC_DPX] = v[1]; scal[SC_ACC_DPY] = v[2]; }
}

int aux_accrete_blocks(const DevGrid &g, int imin, int imax)
{
  const int ncells = (imax - imin + 1) * g.ns;
  return (ncells + ACC_BX - 1) / ACC_BX;
}

__global__ void k_set_accargs(AccArgs a, AccArgs *__restrict__ dst)
{
  if (threadIdx.x == 0) *dst = a;
}

void aux_accrete(const DevGrid &g, const AccArgs &a0, AccArgs *a_dev, double *scal, cudaStream_t s)
{
  AccArgs a = a0;
  a.nb = aux_accrete_blocks(g, a.imin, a.imax);
  k_set_accargs<<<1, 32, 0, s>>>(a, a_dev);
  g_thorin_launches++;
  aux_ring_means(g, a.vt, a.acc + 4, nullptr, nullptr, a.iflow, (a.iflow + 1 < g.nr) ? 2 : 1, s);
  aux_accrete_kernels(g, a_dev, a.nb, scal, s);
}

void aux_accrete_kernels(const DevGrid &g, const AccArgs *a_dev, int nb_grid, double *scal, cudaStream_t s)
{
  k_acc_tau<<<nb_grid, ACC_BX, 0, s>>>(g, a_dev);
  g_thorin_launches++;
  k_acc_reff<<<1, ACC_BX, 0, s>>>(g, a_dev);
  g_thorin_launches++;
  k_acc_column<<<2 * g.nsm, ACC_BX, 0, s>>>(g, a_dev);
  g_thorin_launches++;
  k_acc_upper<<<nb_grid, ACC_BX, 0, s>>>(g, a_dev);
  g_thorin_launches++;
  k_acc_limiter<<<1, ACC_BX, 0, s>>>(a_dev, TH_PI, g.k.sqrt2pi_inv);
  g_thorin_launches++;
  k_acc_apply<<<nb_grid, ACC_BX, 0, s>>>(g, a_dev);
  g_thorin_launches++;
  k_acc_sum<<<1, ACC_BX, 0, s>>>(a_dev, scal);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// Conservation integrals (GasTotalMass, GasMomentum, GasTotalEnergy,
// SideEuler.c:26-80,523-565) and the same mass/momentum sums for pebbles.
__global__ void k_integrals(DevGrid g, const double *__restrict__ rho, const double *__restrict__ vr,
                            const double *__restrict__ vt, const double *__restrict__ e, const double *__restrict__ pd,
                            const double *__restrict__ pvt, double omega_frame, int pebbles, double *__restrict__ part)
{
  const int ns = g.ns;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  double m = 0, am = 0, en = 0, pm = 0, pam = 0;
  if (j < ns) {
    const int l = j + i * ns;
    const int ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
    const int ljp = (j == ns - 1) ? i * ns : l + 1;
    const double S = g.r.Surf[i], rm = g.r.Rmed[i];
    m = S * rho[l];
    am = S * (rho[l] + rho[ljm]) * rm * (vt[l] + omega_frame * rm);
    double vrc = (rm - g.r.Rinf[i]) * vr[l + ns] + (g.r.Rsup[i] - rm) * vr[l];
    vrc /= (g.r.Rsup[i] - g.r.Rinf[i]);
    const double vtc = 0.5 * (vt[l] + vt[ljp]) + rm * omega_frame;
    en = 0.5 * S * rho[l] * (vrc * vrc + vtc * vtc) + S * e[l];
    if (pebbles) {
      pm = S * pd[l];
      pam = S * (pd[l] + pd[ljm]) * rm * (pvt[l] + omega_frame * rm);
    }
  }
  m = block_reduce(m, OpAdd(), 0.0);
  am = block_reduce(am, OpAdd(), 0.0);
  en = block_reduce(en, OpAdd(), 0.0);
  pm = block_reduce(pm, OpAdd(), 0.0);
  pam = block_reduce(pam, OpAdd(), 0.0);
  if (threadIdx.x == 0) {
    const int b = blockIdx.x + blockIdx.y * gridDim.x;
    part[5 * b + 0] = m; part[5 * b + 1] = am; part[5 * b + 2] = en; part[5 * b + 3] = pm; part[5 * b + 4] = pam;
  }
}

__global__ void __launch_bounds__(1024) k_integrals_final(const double *__restrict__ part, int nb, double *__restrict__ scal)
{
  for (int q = 0; q < 5; q++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[5 * b + q];
    s = block_reduce(s, OpAdd(), 0.0);
    if (threadIdx.x == 0) {
      if (q == 1 || q == 4) s *= 0.5;
      scal[SC_MASS + q] = s;
    }
    __syncthreads();
  }
}

void aux_integrals(const DevGrid &g, const double *rho, const double *vr, const double *vt, const double *e,
                   const double *pd, const double *pvt, double omega_frame, int pebbles, double *part, double *scal,
                   cudaStream_t s)
{
  dim3 grid = grid2d(g.ns, g.nr, 256);
  k_integrals<<<grid, 256, 0, s>>>(g, rho, vr, vt, e, pd, pvt, omega_frame, pebbles, part);
  g_thorin_launches++;
  k_integrals_final<<<1, 1024, 0, s>>>(part, grid.x * grid.y, scal);
  g_thorin_launches++;
}

// Final minimum of block partials (DiffusionTimestep's MPI_MIN).
__global__ void __launch_bounds__(1024) k_min_final(const double *__restrict__ part, int nb, double *__restrict__ out)
{
  double m = 1.0e38;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) m = (part[b] < m) ? part[b] : m;
  m = block_reduce(m, OpMin(), 1.0e38);
  if (threadIdx.x == 0) *out = m;
}

void aux_min_final(const double *part, int nb, double *out, cudaStream_t s)
{
  k_min_final<<<1, 1024, 0, s>>>(part, nb, out);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// Open, non-reflecting and source-mass boundaries (ApplyBoundaryCondition,
// SideEuler.c:133-337, 458-486).  The reference's floors of the open inner
// ghost ring (SideEuler.c:15-16):
#define TH_DENSITYFLOOR 1.0e-16
#define TH_ENERGYFLOOR 1.0e-16

// OpenInnerBoundary (SideEuler.c:133-178): ring 0 is the ghost ring.
__global__ void k_open_inner(DevGrid g, double *__restrict__ rho, double *__restrict__ vr,
                             double *__restrict__ energy, int energy_eq, int damp_flux, double gasflux)
{
  const int ns = g.ns, i = 1;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ns) return;
  const int l = j + i * ns;
  const double a = rho[l] + (rho[l] - rho[l + ns]);
  rho[l - ns] = (a > TH_DENSITYFLOOR) ? a : TH_DENSITYFLOOR;
  if (energy_eq) {
    const double b = energy[l] + (energy[l] - energy[l + ns]);
    energy[l - ns] = (b > TH_ENERGYFLOOR) ? b : TH_ENERGYFLOOR;
  }
  if (vr[l + ns] > 0.0) { vr[l] = 0.0; vr[l - ns] = 0.0; }
  else { vr[l] = vr[l + ns]; vr[l - ns] = vr[l]; }
  if (damp_flux) {
    double rhoinf = 0.5 * (rho[l] + rho[l - ns]);
    vr[l] = div_fast(-gasflux, 2.0 * TH_PI * g.r.Rinf[i] * rhoinf);
    rhoinf = rho[l - ns] - 0.5 * (rho[l] - rho[l - ns]);
    vr[l - ns] = div_fast(-gasflux, 2.0 * TH_PI * g.r.Rinf[i - 1] * rhoinf);
  }
}

// OpenOuterBoundary (SideEuler.c:193-232): ring nrad is the ghost ring.
__global__ void k_open_outer(DevGrid g, double *__restrict__ rho, double *__restrict__ vr,
                             double *__restrict__ energy, int energy_eq, int damp_flux, double gasflux)
{
  const int ns = g.ns, i = g.nr - 1;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ns) return;
  const int l = j + i * ns;
  rho[l + ns] = rho[l] + (rho[l] - rho[l - ns]);
  if (energy_eq) energy[l + ns] = energy[l] + (energy[l] - energy[l - ns]);
  if (vr[l] > 0.0) { vr[l] = 0.0; vr[l + ns] = 0.0; }
  else { vr[l] = vr[l - ns]; vr[l + ns] = vr[l]; }
  if (damp_flux) {
    double rhoinf = 0.5 * (rho[l] + rho[l + ns]);
    vr[l + ns] = div_fast(-gasflux, 2.0 * TH_PI * g.r.Rinf[i + 1] * rhoinf);
    rhoinf = rho[l + ns] + 0.5 * (rho[l + ns] - rho[l]);
    vr[l + 2 * ns] = div_fast(-gasflux, 2.0 * TH_PI * g.r.Rsup[i + 1] * rhoinf);
  }
}

// Block-wide sum of a ring, valid in every thread (fixed tree order).
__device__ double ring_sum_block(const double *__restrict__ row, int ns)
{
  __shared__ double sh;
  double a = 0.0;
  for (int j = threadIdx.x; j < ns; j += blockDim.x) a += row[j];
  a = block_reduce(a, OpAdd(), 0.0);
  if (threadIdx.x == 0) sh = a;
  __syncthreads();
  a = sh;
  __syncthreads();
  return a;
}

// NonReflectingBoundary (SideEuler.c:234-337): block 0 the inner edge,
// block 1 the outer edge.  Each block copies the ring next to the edge into
// the edge ring rotated by the Keplerian shear over one cell, sets v_r from
// the outgoing characteristic, and restores the edge ring's mean density and
// energy to the initial profile.
__global__ void __launch_bounds__(1024) k_nonreflecting(DevGrid g, double *__restrict__ rho,
                                                        double *__restrict__ vr, double *__restrict__ energy,
                                                        const double *__restrict__ cs)
{
  const int ns = g.ns, nr = g.nr;
  const bool inner = (blockIdx.x == 0);
  const int ia = inner ? 0 : nr - 2, ib = inner ? 1 : nr - 1;     // rings whose c_s are averaged
  const double csin = ring_sum_block(cs + (size_t)ia * ns, ns) / (double)ns;
  const double csout = ring_sum_block(cs + (size_t)ib * ns, ns) / (double)ns;
  double dangle;
  if (inner) dangle = (pow(g.r.Rinf[1], -1.5) - 1.0) / (.5 * (csin + csout)) * (g.r.Rmed[1] - g.r.Rmed[0]);
  else dangle = (pow(g.r.Rinf[nr - 2], -1.5) - 1.0) / (.5 * (csin + csout)) * (g.r.Rmed[nr - 1] - g.r.Rmed[nr - 2]);
  const int i_angle = (int)(dangle / 2.0 / TH_PI * (double)ns + .5);
  const int i = inner ? 1 : nr - 1;
  const int edge = inner ? 0 : nr - 1;
  const double sig = inner ? g.r.SigmaMed[1] : g.r.SigmaMed[nr - 2];
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    const int l = j + i * ns;
    int jp = inner ? j + i_angle : j - i_angle;
    if (jp >= ns) jp -= ns;
    if (jp < 0) jp += ns;
    if (inner) {
      const int lp = jp;
      rho[lp] = rho[l];
      energy[lp] = energy[l];
      const double vr_med = div_fast(-cs[l] * (rho[l] - sig), sig);
      vr[l] = 2. * vr_med - vr[l + ns];
    } else {
      const int lp = jp + (i - 1) * ns;
      rho[l] = rho[lp];
      energy[l] = energy[lp];
      const double vr_med = div_fast(cs[l] * (rho[l - ns] - sig), sig);
      vr[l] = 2. * vr_med - vr[l - ns];
    }
  }
  __syncthreads();
  double *re = rho + (size_t)edge * ns, *ee = energy + (size_t)edge * ns;
  const double mr = ring_sum_block(re, ns) / (double)ns;
  for (int j = threadIdx.x; j < ns; j += blockDim.x) re[j] += g.r.SigmaMed[edge] - mr;
  __syncthreads();
  const double me = ring_sum_block(ee, ns) / (double)ns;
  for (int j = threadIdx.x; j < ns; j += blockDim.x) ee[j] += g.r.EnergyMed[edge] - me;
}

// ApplyOuterSourceMass (SideEuler.c:458-486), one block.
__global__ void __launch_bounds__(1024) k_outer_source_mass(DevGrid g, double *__restrict__ rho,
                                                            double *__restrict__ vr, double penul_vr)
{
  const int ns = g.ns, i = g.nr - 1;
  double *row = rho + (size_t)i * ns;
  const double avg = g.r.SigmaMed[i] - ring_sum_block(row, ns) / (double)ns;
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    row[j] += avg;
    vr[j + i * ns] = penul_vr;
  }
}

void aux_open_inner(const DevGrid &g, double *rho, double *vr, double *energy, int energy_eq, int damp_flux,
                    double gasflux, cudaStream_t s)
{
  k_open_inner<<<(g.ns + BX - 1) / BX, BX, 0, s>>>(g, rho, vr, energy, energy_eq, damp_flux, gasflux);
  g_thorin_launches++;
}

void aux_open_outer(const DevGrid &g, double *rho, double *vr, double *energy, int energy_eq, int damp_flux,
                    double gasflux, cudaStream_t s)
{
  k_open_outer<<<(g.ns + BX - 1) / BX, BX, 0, s>>>(g, rho, vr, energy, energy_eq, damp_flux, gasflux);
  g_thorin_launches++;
}

void aux_nonreflecting(const DevGrid &g, double *rho, double *vr, double *energy, const double *cs, cudaStream_t s)
{
  k_nonreflecting<<<2, 1024, 0, s>>>(g, rho, vr, energy, cs);
  g_thorin_launches++;
}

void aux_outer_source_mass(const DevGrid &g, double *rho, double *vr, double penul_vr, cudaStream_t s)
{
  k_outer_source_mass<<<1, 1024, 0, s>>>(g, rho, vr, penul_vr);
  g_thorin_launches++;
}

// Parametric cooling of SubStep3 (SourceEuler.c:569-582): the energy relaxes
// towards the initial profile on the cooling time, heated by Q+.
__global__ void k_parametric_cooling(DevGrid g, const double *__restrict__ rho, const double *__restrict__ eint,
                                     const double *__restrict__ qplus, const double *__restrict__ divv,
                                     const double *__restrict__ coolt, const double *__restrict__ qplusmed,
                                     double *__restrict__ enew, double gm1)
{
  const double dt = g.ctl[CTL_DT];
  const int ns = g.ns;
  CELL_LOOP_2D
  const double tc = coolt[i], sm = g.r.SigmaMed[i];
  const double tmp1 = div_fast(g.r.EnergyMed[i] * dt * rho[l], sm) + tc * eint[l] +
                      dt * tc * (qplus[l] - div_fast(qplusmed[i] * rho[l], sm));
  const double tmp2 = dt + tc + gm1 * dt * tc * divv[l];
  enew[l] = div_fast(tmp1, tmp2);
}

void aux_parametric_cooling(const DevGrid &g, const double *rho, const double *eint, const double *qplus,
                            const double *divv, const double *coolt, const double *qplusmed, double *enew,
                            double gm1, cudaStream_t s)
{
  k_parametric_cooling<<<grid2d(g.ns, g.nr, BX), BX, 0, s>>>(g, rho, eint, qplus, divv, coolt, qplusmed, enew, gm1);
  g_thorin_launches++;
}

// ---------------------------------------------------------------------------
// Gas accretion onto a planet, Kley's prescription (AccreteOntoPlanets,
// Planet.c:34-166): within frac1 = 0.75 and frac2 = 0.45 Roche radii a cell
// loses facc1 times the Gaussian column between the planet's height +/- the
// chord (trapezoid rule refined to 1e-4, at most 16 levels: qtrap,
// Planet.c:172-211) and then the fraction facc2.  One block per planet over
// the window [i_min, i_max] x [j_min, j_max] (narrower than a ring, so no cell
// is visited twice); the mass and momentum taken are block sums written to
// out[0..2].
__device__ double qtrap_gauss(double a, double b)
{
  double s = 0.0, olds = 0.0;
  for (int n = 1; n <= 16; n++) {
    if (n == 1) {
      s = 0.5 * (b - a) * (exp(-a * a) + exp(-b * b));
    } else {
      int it = 1;
      for (int j = 1; j < n - 1; j++) it <<= 1;
      const double tnm = it, del = div_fast(b - a, tnm);
      double x = a + 0.5 * del, sum = 0.0;
      for (int j = 1; j <= it; j++, x += del) sum += exp(-x * x);
      s = 0.5 * (s + div_fast((b - a) * sum, tnm));
    }
    if (n > 5)
      if (fabs(s - olds) < 1.e-4 * fabs(olds) || (s == 0.0 && olds == 0.0)) return s;
    olds = s;
  }
  return s;
}

__global__ void __launch_bounds__(256) k_gas_accrete(DevGrid g, double *__restrict__ dens,
                                                     const double *__restrict__ vrad,
                                                     const double *__restrict__ vtheta,
                                                     const double *__restrict__ cs, GasAccArgs a,
                                                     double *__restrict__ out)
{
  const int ns = g.ns;
  const int nj = a.j_max - a.j_min + 1;
  const int ncell = (a.i_max - a.i_min + 1) * nj;
  double dM = 0.0, dPx = 0.0, dPy = 0.0;
  for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
    const int i = a.i_min + c / nj;
    const int j = a.j_min + c % nj;
    int jf = j;
    while (jf < 0) jf += ns;
    while (jf >= ns) jf -= ns;
    const int l = jf + i * ns, lip = l + ns;
    const int ljp = (jf == ns - 1) ? i * ns : l + 1;
    const double rm = g.r.Rmed[i];
    const double xc = rm * g.r.costab[jf], yc = rm * g.r.sintab[jf];
    const double dx = a.Xp - xc, dy = a.Yp - yc;
    const double distance = sqrt(dx * dx + dy * dy);
    const double vtcell = 0.5 * (vtheta[l] + vtheta[ljp]) + rm * a.omega_frame;
    const double vrcell = 0.5 * (vrad[l] + vrad[lip]);
    const double vxcell = div_fast(vrcell * xc - vtcell * yc, rm);
    const double vycell = div_fast(vrcell * yc + vtcell * xc, rm);
    const double H = cs[l] * g.r.OmegaInv[i] * g.k.sqrt_adiabind_inv;
    const double sq2H = sqrt(2.0) * H;
    for (int pass = 0; pass < 2; pass++) {
      const double fr = pass ? 0.45 : 0.75;
      if (distance < fr * a.RRoche) {
        const double dz = sqrt((fr * a.RRoche) * (fr * a.RRoche) - distance * distance);
        double factor = qtrap_gauss(div_fast(a.Zp - dz, sq2H), div_fast(a.Zp + dz, sq2H));
        factor *= div_fast(1.0, sqrt(2.0 * TH_PI) * H);
        const double fa = pass ? a.facc2 : a.facc1;
        const double deltaM = fa * factor * dens[l] * g.r.Surf[i];
        dens[l] *= pass ? (1.0 - fa) : (1.0 - fa * factor);
        dPx += deltaM * vxcell;
        dPy += deltaM * vycell;
        dM += deltaM;
      }
    }
  }
  dM = block_reduce(dM, OpAdd(), 0.0);
  dPx = block_reduce(dPx, OpAdd(), 0.0);
  dPy = block_reduce(dPy, OpAdd(), 0.0);
  if (threadIdx.x == 0) { out[0] = dM; out[1] = dPx; out[2] = dPy; }
}

void aux_gas_accrete(const DevGrid &g, double *dens, const double *vrad, const double *vtheta, const double *cs,
                     const GasAccArgs &a, double *out, cudaStream_t s)
{
  k_gas_accrete<<<1, 256, 0, s>>>(g, dens, vrad, vtheta, cs, a, out);
  g_thorin_launches++;
}

// The gas state of one cell for the planet's aerodynamic drag (StokesDrag,
// Drag.c:17-95): Sigma, c_s, v_r at l and l+nsec, v_theta at l and l+1.
__global__ void k_drag_cell(const double *__restrict__ rho, const double *__restrict__ cs,
                            const double *__restrict__ vrad, const double *__restrict__ vtheta, int l, int ns,
                            double *__restrict__ out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  out[0] = rho[l];
  out[1] = cs[l];
  out[2] = vrad[l];
  out[3] = vrad[l + ns];
  out[4] = vtheta[l];
  out[5] = vtheta[l + 1];
}

void aux_drag_cell(const double *rho, const double *cs, const double *vrad, const double *vtheta, int l, int ns,
                   double *out, cudaStream_t s)
{
  k_drag_cell<<<1, 32, 0, s>>>(rho, cs, vrad, vtheta, l, ns, out);
  g_thorin_launches++;
}

// CorrectVtheta (SideEuler.c:505-519): v_theta -= domega * Rmed when the
// frame's rotation rate changes by domega.
__global__ void k_correct_vtheta(DevGrid g, double *__restrict__ vt, double domega)
{
  const int ns = g.ns;
  CELL_LOOP_2D
  vt[l] -= domega * g.r.Rmed[i];
}

void aux_correct_vtheta(const DevGrid &g, double *vt, double domega, cudaStream_t s)
{
  k_correct_vtheta<<<grid2d(g.ns, g.nr, BX), BX, 0, s>>>(g, vt, domega);
  g_thorin_launches++;
}

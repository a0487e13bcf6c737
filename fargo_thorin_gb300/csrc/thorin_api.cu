// thorin_api.cu -- the C ABI of include/thorin_gpu.h: device state of one
// disk, host-side set-up that the reference performs once on the host
// (grid, profiles, initial fields: SourceEuler.c:68-175, Theo.c,
// Pframeforce.c:620-751, Pebbles.c:37-275), the substep driver of AlgoGas
// (SourceEuler.c:210-317), the SOR control loop and omega schedule
// (EnergySources.c:298-403), and the host N-body step standing in for
// REBOUND (ReboundInterface.c:262-385, Psys.c:336).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <initializer_list>
#include <string>
#include <vector>
#include "thorin_kernels.cuh"
#include "thorin_planet.cuh"
#include "thorin_graph.cuh"
#include "../../include/thorin_warmnet.h"

// learned SOR warm start (warmnet.cu)
int wn_sor_predict(thorin_warmnet *n, int nr, int ns, int fc, double *T, const double *ml, const double *mlip,
                   const double *mlim, const double *mljp, const double *mljm, const double *rhs, const double *prev,
                   double *jac, const double *jscale, double omega, const double *omega_dev, cudaStream_t s);
int wn_sor_train(thorin_warmnet *n, int nr, int ns, int fc, const double *tk, const double *tconv, const double *ml,
                 const double *mlip, const double *mlim, const double *mljp, const double *mljm, const double *rhs,
                 const double *prev, double *jac, float lr, double *scratch, cudaStream_t s);
int wn_record_update(int nr, int ns, const double *tconv, const double *tstart, double *hist, int nh,
                     const double *dt, double *dts, cudaStream_t s);
int ws_extrapolate(int nr, int ns, double *T, const double *hist, int order, const double *dt, const double *dts,
                   const double *ml, const double *mlip, const double *mlim, const double *mljp, const double *mljm,
                   const double *rhs, const double *cw, const double *omega, double *scratch, double *vq,
                   double *part, double *step, int nsm, cudaStream_t s);
int wn_last_loss(thorin_warmnet *n, double *loss);
int wn_dims(const thorin_warmnet *n, int *nr, int *ns);

// Unit constants (src_main/fondam.h), evaluated with the host libm.
#define H_PI 3.14159265358979323844
#define H_MPI 3.14159265358979323846
#define MSOL_SI 1.98855e30
#define GM_SI 1.32712440018e20
#define AU_SI 149597870700.0
#define R_STANDARD 8.3144598
#define MMW 2.4
#define R_SI (R_STANDARD / (MMW * 0.001))
#define OPA2CU (MSOL_SI * 1000.0 / pow(AU_SI * 100.0, 2.0))
#define T2SI (GM_SI / R_SI / AU_SI)
#define TIME2SI (sqrt(pow(AU_SI, 3.0) / GM_SI))
#define RHO2CGS (MSOL_SI * 1000.0 / pow(AU_SI * 100.0, 3.0))
#define STEFANBOLTZMANN (5.670367e-8 * (1.0 / MSOL_SI) * pow(1.0 / TIME2SI, -3.0) * pow(1.0 / T2SI, -4.0))
#define FLUX2CU (0.000003 / (2.0 * H_PI))
#define SQRT2PI_INV (1.0 / sqrt(2.0 * H_PI))

thread_local std::string g_last_error;
std::atomic<long long> g_thorin_launches{0};

#define CUCHK(call)                                                                     \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      g_last_error = std::string(#call) + ": " + cudaGetErrorString(e_);                \
      return THORIN_ERR_CUDA;                                                           \
    }                                                                                   \
  } while (0)

#define RCHK(expr)                     \
  do {                                 \
    int r_ = (expr);                   \
    if (r_ != THORIN_OK) return r_;    \
  } while (0)

extern "C" const char *thorin_gpu_last_error(void) { return g_last_error.c_str(); }

// Launch-time errors of the kernels enqueued so far (bad configuration,
// resources) surface here; faults of running kernels at the next sync.
#define KCHECK(where)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = cudaGetLastError();                                                \
    if (e_ != cudaSuccess) {                                                            \
      g_last_error = std::string(where) + ": " + cudaGetErrorString(e_);                \
      return THORIN_ERR_CUDA;                                                           \
    }                                                                                   \
  } while (0)

extern "C" void thorin_params_default(thorin_params *p, int nrad, int nsec)
{
  // src_main/var.c:17-141 defaults and the derived switches of Interpret.c.
  memset(p, 0, sizeof(*p));
  p->nrad = nrad; p->nsec = nsec;
  p->rmin = 1.0; p->rmax = 1.0;
  p->sigma0 = 173.0; p->aspect_ratio = 0.05;
  p->scaling_factor = 1.0;
  p->cavity_ratio = 1.0; p->cavity_width = 1.0;
  p->transition_ratio = 1.0; p->transition_width = 1.0;
  p->tmri = 1000.0; p->twidth = 25.0;
  p->adiabind = 1.4; p->cooling_time = -1.0;
  p->opacity_drop = 0.6; p->effective_temperature = 5656.0; p->stellar_radius = 3.0; p->disc_albedo = 0.5;
  p->hillcut = 0.8; p->indirect_term = 1; p->mass_taper = 0.0000001; p->vertical_damping = 0.1;
  p->planetary_density = 1.0;
  p->fast_transport = 1;
  p->damp_vrad = 1;
  p->damping_rmin_frac = 1.25; p->damping_rmax_frac = 0.84; p->damping_period_frac = 1.0;
  p->dt = 1.0; p->first_step = -1.0; p->minimum_step = 1.0e-3; p->maximum_step = 1.0e6;
  p->diffusive_particles = 1;
  p->pebble_flux = 2.0e-4; p->pebble_alpha = 1.0e-4; p->pebble_coagulation = 0.5; p->pebble_bulk_dens = 1.0;
  p->schmidt_number = 1.0; p->heating_delay = 100; p->pebble_to_gas_max = 0.01;
  p->fragment_factor = 1.0; p->fragment_threshold = 1.0; p->fragment_alpha = 1.0e-3;
  p->evaporation_temperature = 1000.0; p->evaporation_rate = 1.0e-3;
  p->sor_eps = 1.0e-6; p->sor_maxiters = 100000;
}

// ---------------------------------------------------------------------------
enum {  // ring arrays kept on the device
  R_RINF, R_RSUP, R_RMED, R_SURF, R_INVRMED, R_INVSURF, R_INVDIFFRMED, R_INVDIFFRSUP, R_INVRINF, R_OMEGAINV, R_RMED2,
  R_WAVEKILLER, R_RMED15, R_RINF15, R_RSUP15, R_COSTAB, R_SINTAB, R_SIGMAMED, R_ENERGYMED, R_VTHETAMED, R_PEBDENS0,
  R_PEBVRAD0, R_PEBVTHETA0, R_CSMEAN, R_TEMPMEAN, R_NUMED, R_NUINF, R_INVDXTHETA, R_INVDXTHETA2, R_SUPPTORQUE,
  R_DELTAR2, R_CFLDXRAD, R_CFLDXTHETA, R_CFLMINDX, R_CFLDEN5, R_VMOY, R_PVTMED, R_HAVR, R_SIGAVR, R_ISTAVR, R_PHAVR,
  R_PISTAVR, R_VMED, R_TAUAVR, R_VTEMP, R_DAMPVR0, R_CSISO, R_COOLT, R_QPLUSMED, R_ISIGAVR, R_DRSQ, R_OMEGA,
  R_COUNT
};

struct thorin_disk {
  thorin_params p;
  int nr, ns;
  size_t fsize;                      // doubles per field allocation
  cudaStream_t s;
  DevGrid g;
  std::vector<void *> allocs;
  double *ring[R_COUNT];
  // fields
  double *rho, *vrad, *vtheta, *energy, *vrad_new, *vtheta_new, *energy_new, *vrad_int, *vtheta_int, *energy_int;
  double *cs, *temper, *qplus, *qminus, *opacity, *divv, *trr, *trp, *tpp, *agr, *agt, *pagr, *pagt, *dcen;
  double *ml, *mlip, *mlim, *mljp, *mljm, *rhs, *sor_cw, *tbackup, *flaring, *qirr;   // sor_cw = omega / ml
  double *press = nullptr;   // pressure field of isothermal runs (formed at the start of each substep)
  double *label = nullptr;   // passive tracer (LabelAdvection)
  double *pdens, *pvrad, *pvtheta, *psize, *tau, *paccr, *pacct, *gaccr, *gacct, *dragr, *dragt, *macc;
  double *t_rho_gas, *t_e_gas, *t_rho_peb;
  TransportScratch ts;
  // the pebble fluid's transport runs on its own stream with its own scratch,
  // concurrently with SubStep2, the energy step and the gas transport
  TransportScratch ts_peb;
  cudaStream_t s_peb = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  double *partials, *scal;
  int *iscal, *nshift, *heat_idx_d, *damp_rings_d;
  double *heat_val_d;
  unsigned int *ticket;
  DevPlanet *planets_d;
  double *ctl;                       // control block (CTL_*), also d->g.ctl
  PlConst plc;                       // constants of the planet side (thorin_planet.cuh)
  // device-resident DT (thorin_gpu_algogas_graph): the instantiated graph of
  // one DT, the planets and counters it keeps on the device, and the state
  // of the capture that builds it
  cudaGraphExec_t dt_graph = nullptr;
  thorin_planets *sys_d = nullptr, *sys_h = nullptr;   // device copy, pinned staging copy
  GraphStats *gst_d = nullptr, *gst_h = nullptr;
  int *ring_info_d = nullptr;
  AccArgs *acc_args_g = nullptr;     // the graph's own accretion arguments (its buffers' pointers)
  double *ctl_h = nullptr;           // pinned staging of the control block
  int graph_npl = -1;                // planets the graph was built for
  int capturing = 0;                 // launches are being captured into the DT graph
  StepDev capS;
  cudaGraph_t capture_sor_body = nullptr;   // body of the SOR loop node, filled after the substep capture
  cudaStream_t s_pl = nullptr;       // the planet step's branch of the substep graph
  double *cap_ptr[11] = {};          // the buffers the DT graph was captured with (graph_roles order)
  cudaEvent_t ev_pl_fork = nullptr, ev_pl_join = nullptr;
  AccArgs *acc_args_d;               // pebble accretion arguments on the device
  SorCtl sor;
  CflRings cfl;
  ForceRings fr;
  // pinned host mirrors
  double *scal_h, *csmean_h;
  int *iscal_h;
  // host ring arrays
  std::vector<double> Radii, GlobalRmed, Rinf, Rsup, Rmed, Surf, InvRmed, InvSurf, InvDiffRmed, InvDiffRsup, InvRinf,
      OmegaInv, Rmed2, WaveKiller, SigmaMed, SigmaInf, EnergyMed, VthetaMed, PebDensInit, PebVradInit, PebVthetaInit;
  int *nshift_h = nullptr;           // pinned: the per-substep copy must not block the host
  int ndamp;
  // scalars carried between substeps (static variables in the reference)
  double PhysicalTime, PhysicalTimeInitial, OmegaFrame, MassTaper;
  int cfl_first;
  int sor_first, Niterlast, Niterbest;
  int torque_pending = 0, ntorque = 0;
  int sloppy_pass = 0;           // the once-per-DT CFL of SloppyCFL runs
  double doubling = 0.0;         // ParametricAccretion's doubling time, fixed at its first call
  thorin_torque torques[THORIN_MAXPLANETS];
  double omega, domega, omegabest;
  // learned warm start of the SOR solve (off unless attached)
  thorin_warmnet *ws_net = nullptr;
  int ws_mode = THORIN_WS_OFF;
  float ws_lr = 0.f;
  thorin_ws_stats ws_st = {0, 0, 0.0, 0.0, 0.0, 0.0};
  // the last ws_nh solves' updates T_conv - T_start, newest first (slot 0
  // is the network's input), and their time steps (THORIN_WS_MAX_ORDER
  // device doubles, 0 = not recorded)
  double *ws_prev = nullptr;
  double *ws_dts = nullptr;
  double *ws_part = nullptr;     // block partials of the extrapolated start's step length (4 nsm + 2)
  double *ws_vq = nullptr;       // its per-cell terms of the Jacobi step (2 fields)
  double *ws_step = nullptr;     // its step length and the running sum of the steps
  int ws_nh = 0;                 // slots of ws_prev
  int ws_order = 2;              // order of the extrapolated start
  double *ws_jac = nullptr;      // the Jacobi step of the solve's start, per cell
  int ws_f = 1;                  // disk cells per network cell along each axis (1 or 2)
  // the SOR sweep loop: one CUDA graph whose WHILE node repeats the two
  // colour passes until the completion step clears its condition
  cudaGraphExec_t sor_loop = nullptr;
  int sor_loop_k = 8;            // sweeps per run of the loop body
  int sor_direct = 0;            // sweeps as plain stream launches (for kernel profilers)
  double heatsrc[THORIN_MAXPLANETS];
  int heatsrc_index[THORIN_MAXPLANETS], heatsrc_max;
  double gm1, gg1, drin, drout, invdphi, lr01, lr12, taueff_c, tirr4fac, rstar;
  double vkep_in, vkep_out;      // Keplerian edge velocities (ImposeKeplerianEdges) in the inertial frame
  ViscParams vp;
  thorin_stats st;
  int timing;
  cudaEvent_t ev[4];
};

static int dalloc(thorin_disk *d, void **ptr, size_t bytes)
{
  CUCHK(cudaMalloc(ptr, bytes));
  CUCHK(cudaMemsetAsync(*ptr, 0, bytes, d->s));
  d->allocs.push_back(*ptr);
  return THORIN_OK;
}

static int dfield(thorin_disk *d, double **ptr) { return dalloc(d, (void **)ptr, d->fsize * sizeof(double)); }

static int upload_ring(thorin_disk *d, int id, const std::vector<double> &v)
{
  CUCHK(cudaMemcpyAsync(d->ring[id], v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, d->s));
  return THORIN_OK;
}

// FillPolar1DArrays (SourceEuler.c:68-131) and the per-ring constants of the
// kernels, each with the expression the reference uses at that place.
static void fill_rings(thorin_disk *d)
{
  const thorin_params &p = d->p;
  const int nr = d->nr, ns = d->ns, n1 = nr + 2;
  auto Z = [&](std::vector<double> &v) { v.assign(n1, 0.0); };
  Z(d->Radii); Z(d->GlobalRmed); Z(d->Rinf); Z(d->Rsup); Z(d->Rmed); Z(d->Surf); Z(d->InvRmed); Z(d->InvSurf);
  Z(d->InvDiffRmed); Z(d->InvDiffRsup); Z(d->InvRinf); Z(d->OmegaInv); Z(d->Rmed2); Z(d->WaveKiller);
  Z(d->SigmaMed); Z(d->SigmaInf); Z(d->EnergyMed); Z(d->VthetaMed); Z(d->PebDensInit); Z(d->PebVradInit);
  Z(d->PebVthetaInit);
  const double drrsep = (p.rmax - p.rmin) / (double)nr;
  for (int i = 0; i <= nr; i++)
    d->Radii[i] = p.log_grid ? p.rmin * exp((double)i / (double)nr * log(p.rmax / p.rmin)) : p.rmin + drrsep * (double)i;
  for (int i = 0; i < nr; i++) {
    const double a = d->Radii[i], b = d->Radii[i + 1];
    d->GlobalRmed[i] = 2.0 / 3.0 * (b * b * b - a * a * a);
    d->GlobalRmed[i] = d->GlobalRmed[i] / (b * b - a * a);
    d->Rinf[i] = a;
    d->Rsup[i] = b;
    d->Rmed[i] = 2.0 / 3.0 * (b * b * b - a * a * a);
    d->Rmed[i] = d->Rmed[i] / (b * b - a * a);
    d->Surf[i] = H_PI * (b * b - a * a) / (double)ns;
    d->InvRmed[i] = 1.0 / d->Rmed[i];
    d->InvSurf[i] = 1.0 / d->Surf[i];
    d->InvDiffRsup[i] = 1.0 / (b - a);
    d->InvRinf[i] = 1.0 / a;
    d->OmegaInv[i] = pow(d->Rmed[i], 1.5);
    d->Rmed2[i] = d->Rmed[i] * d->Rmed[i];
  }
  d->Rinf[nr] = d->Radii[nr];
  for (int i = 1; i < nr; i++) d->InvDiffRmed[i] = 1.0 / (d->Rmed[i] - d->Rmed[i - 1]);
  // SetWaveKillingZones (SideEuler.c:341-362)
  d->drin = p.rmin * p.damping_rmin_frac;
  d->drout = p.rmax * p.damping_rmax_frac;
  const double tauin = p.damping_period_frac * 2.0 * H_PI * pow(p.rmin, 1.5);
  const double tauout = p.damping_period_frac * 2.0 * H_PI * pow(d->drout, 1.5);
  if (p.damping || p.pebbles)
    for (int i = 0; i < nr; i++) {
      double damp;
      d->WaveKiller[i] = 0.0;
      if (d->Rmed[i] < d->drin) { damp = (d->drin - d->Rmed[i]) / (d->drin - p.rmin); d->WaveKiller[i] = damp * damp / tauin; }
      if (d->Rmed[i] > d->drout) { damp = (d->Rmed[i] - d->drout) / (p.rmax - d->drout); d->WaveKiller[i] = damp / tauout; }
    }
}

static double fviscosity_host(const thorin_disk *d, int i_ring, double rad, const std::vector<double> &csm)
{
  // FViscosity (Viscosity.c:26-54) for the ring the reference's search finds.
  const thorin_params &p = d->p;
  double nu = p.viscosity;
  if (p.viscosity_alpha) nu = p.alpha_viscosity * csm[i_ring] * csm[i_ring] * pow(rad, 1.5);
  const double rmin = (p.cavity_radius - p.cavity_width * p.aspect_ratio);
  const double rmax = (p.cavity_radius + p.cavity_width * p.aspect_ratio);
  if (rad < rmin) nu *= p.cavity_ratio;
  if ((rad >= rmin) && (rad <= rmax)) nu *= exp((rmax - rad) / (rmax - rmin) * log(p.cavity_ratio));
  return nu;
}

static int upload_all_rings(thorin_disk *d)
{
  const int nr = d->nr, ns = d->ns, n1 = nr + 2;
  const thorin_params &p = d->p;
  std::vector<double> v(n1, 0.0);
  RCHK(upload_ring(d, R_RINF, d->Rinf)); RCHK(upload_ring(d, R_RSUP, d->Rsup)); RCHK(upload_ring(d, R_RMED, d->Rmed));
  RCHK(upload_ring(d, R_SURF, d->Surf)); RCHK(upload_ring(d, R_INVRMED, d->InvRmed));
  RCHK(upload_ring(d, R_INVSURF, d->InvSurf)); RCHK(upload_ring(d, R_INVDIFFRMED, d->InvDiffRmed));
  RCHK(upload_ring(d, R_INVDIFFRSUP, d->InvDiffRsup)); RCHK(upload_ring(d, R_INVRINF, d->InvRinf));
  RCHK(upload_ring(d, R_OMEGAINV, d->OmegaInv)); RCHK(upload_ring(d, R_RMED2, d->Rmed2));
  {
    std::vector<double> om(n1, 0.0);           // Omega = 1 / OmegaInv, correctly rounded
    for (int i = 0; i < n1; i++)
      if (d->OmegaInv[i] != 0.0) om[i] = 1.0 / d->OmegaInv[i];
    RCHK(upload_ring(d, R_OMEGA, om));
  }
  RCHK(upload_ring(d, R_WAVEKILLER, d->WaveKiller));
  for (int i = 0; i < nr; i++) v[i] = pow(d->Rmed[i], 1.5);
  RCHK(upload_ring(d, R_RMED15, v));
  std::fill(v.begin(), v.end(), 0.0);
  for (int i = 0; i <= nr; i++) v[i] = pow(d->Rinf[i], 1.5);
  RCHK(upload_ring(d, R_RINF15, v));
  std::fill(v.begin(), v.end(), 0.0);
  for (int i = 0; i < nr; i++) v[i] = pow(d->Rsup[i], 1.5);
  RCHK(upload_ring(d, R_RSUP15, v));
  // trigonometric tables of InitComputeAccel (SideEuler.c:101-118):
  // abscissa = Rmed[i] * cos(2 pi j / ns) is a single product.
  std::vector<double> c(ns), sn(ns);
  for (int j = 0; j < ns; j++) { c[j] = cos(2.0 * H_PI * (double)j / (double)ns); sn[j] = sin(2.0 * H_PI * (double)j / (double)ns); }
  CUCHK(cudaMemcpyAsync(d->ring[R_COSTAB], c.data(), ns * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(d->ring[R_SINTAB], sn.data(), ns * sizeof(double), cudaMemcpyHostToDevice, d->s));
  // per-ring expressions of SubStep1/2, ImplicitRadiativeDiffusion, DiffusionTimestep, ConditionCFL
  std::vector<double> a(n1, 0.0), b(n1, 0.0), st(n1, 0.0), dr2(n1, 0.0), cdx(n1, 0.0), cdt(n1, 0.0), cmin(n1, 0.0),
      cden(n1, 0.0), drsq(n1, 0.0);
  for (int i = 0; i < nr; i++) {
    const double dxtheta = 2.0 * H_PI / (double)ns * d->Rmed[i];
    a[i] = 1.0 / dxtheta;
    b[i] = 1.0 / dxtheta / dxtheta;
    st[i] = p.imposed_disk_drift * .5 * pow(d->Rmed[i], -2.5 + p.sigma_slope);
    double dr = d->Rsup[i] - d->Rinf[i];
    dr2[i] = dr * dr / 2.0;
    drsq[i] = dr * dr;
    const double dxrad = d->Rsup[i] - d->Rinf[i];
    const double dxth = d->Rmed[i] * 2.0 * H_PI / (double)ns;
    cdx[i] = dxrad;
    cdt[i] = dxth;
    cmin[i] = (dxth < dxrad) ? dxth : dxrad;
    cden[i] = pow(cmin[i], 2);
  }
  RCHK(upload_ring(d, R_INVDXTHETA, a)); RCHK(upload_ring(d, R_INVDXTHETA2, b));
  RCHK(upload_ring(d, R_SUPPTORQUE, st)); RCHK(upload_ring(d, R_DELTAR2, dr2)); RCHK(upload_ring(d, R_DRSQ, drsq));
  RCHK(upload_ring(d, R_CFLDXRAD, cdx)); RCHK(upload_ring(d, R_CFLDXTHETA, cdt));
  RCHK(upload_ring(d, R_CFLMINDX, cmin)); RCHK(upload_ring(d, R_CFLDEN5, cden));
  RCHK(upload_ring(d, R_SIGMAMED, d->SigmaMed)); RCHK(upload_ring(d, R_ENERGYMED, d->EnergyMed));
  RCHK(upload_ring(d, R_VTHETAMED, d->VthetaMed)); RCHK(upload_ring(d, R_PEBDENS0, d->PebDensInit));
  RCHK(upload_ring(d, R_PEBVRAD0, d->PebVradInit)); RCHK(upload_ring(d, R_PEBVTHETA0, d->PebVthetaInit));
  // DampingBoundary's v_r target with DampTowards GASFLUX (SideEuler.c:395-398)
  std::vector<double> vr0(n1, 0.0);
  if (p.damp_flux)
    for (int i = 0; i < nr; i++) vr0[i] = -p.gasflux / (2.0 * H_PI * d->Rinf[i] * d->SigmaInf[i]);
  RCHK(upload_ring(d, R_DAMPVR0, vr0));
  return THORIN_OK;
}

static void build_grid(thorin_disk *d)
{
  DevGrid &g = d->g;
  g.nr = d->nr; g.ns = d->ns;
  g.sor_tpsm = 1536;
  int dev = 0;
  g.nsm = 1;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&g.nsm, cudaDevAttrMultiProcessorCount, dev);
  DevRings &r = g.r;
  double **R = d->ring;
  r.Rinf = R[R_RINF]; r.Rsup = R[R_RSUP]; r.Rmed = R[R_RMED]; r.Surf = R[R_SURF]; r.InvRmed = R[R_INVRMED];
  r.InvSurf = R[R_INVSURF]; r.InvDiffRmed = R[R_INVDIFFRMED]; r.InvDiffRsup = R[R_INVDIFFRSUP];
  r.InvRinf = R[R_INVRINF]; r.OmegaInv = R[R_OMEGAINV]; r.Omega = R[R_OMEGA]; r.Rmed2 = R[R_RMED2]; r.WaveKiller = R[R_WAVEKILLER];
  r.Rmed15 = R[R_RMED15]; r.Rinf15 = R[R_RINF15]; r.costab = R[R_COSTAB]; r.sintab = R[R_SINTAB];
  r.SigmaMed = R[R_SIGMAMED]; r.EnergyMed = R[R_ENERGYMED]; r.VthetaMed = R[R_VTHETAMED];
  r.PebDensInit = R[R_PEBDENS0]; r.PebVradInit = R[R_PEBVRAD0]; r.PebVthetaInit = R[R_PEBVTHETA0];
  r.csmean = R[R_CSMEAN]; r.tempmean = R[R_TEMPMEAN]; r.nu_med = R[R_NUMED]; r.nu_inf = R[R_NUINF];
  DevConst &k = g.k;
  const thorin_params &p = d->p;
  k.dpns = 2.0 * H_PI / (double)d->ns;
  r.InvDxtheta = R[R_INVDXTHETA];
  k.opa2cu = OPA2CU; k.t2si = T2SI; k.rho2cgs = RHO2CGS; k.sigma_sb = STEFANBOLTZMANN; k.sqrt2pi_inv = SQRT2PI_INV;
  k.pebbulkdens = p.pebble_bulk_dens / RHO2CGS;
  k.cv = 1.0 / (1.0 * (p.adiabind - 1.0));
  k.sqrt_adiabind_inv = 1.0 / sqrt(p.adiabind);
  k.evaptemp = p.evaporation_temperature / T2SI;
  k.sqrt3 = sqrt(3.0);
  d->cfl.dxrad = R[R_CFLDXRAD]; d->cfl.dxtheta = R[R_CFLDXTHETA]; d->cfl.mindx = R[R_CFLMINDX];
  d->cfl.den5 = R[R_CFLDEN5]; d->cfl.vmoy = R[R_VMOY]; d->cfl.pvtmed = R[R_PVTMED];
  d->fr.H_avr = R[R_HAVR]; d->fr.sigma_avr = R[R_SIGAVR]; d->fr.integstar_avr = R[R_ISTAVR];
  d->fr.p_H_avr = R[R_PHAVR]; d->fr.p_integstar_avr = R[R_PISTAVR]; d->fr.tau_avr = R[R_TAUAVR];
  d->fr.isigma_avr = R[R_ISIGAVR]; d->fr.drsq = R[R_DRSQ];
}

static int check_supported(const thorin_params &p)
{
  const char *bad = nullptr;
  if (p.nrad < 4 || p.nsec < 4 || (p.nsec & 1)) bad = "nrad, nsec >= 4 and nsec even (red-black SOR)";
  if (bad) {
    g_last_error = std::string("unsupported option: ") + bad;
    return THORIN_ERR_ARG;
  }
  return THORIN_OK;
}

extern "C" int thorin_gpu_create(const thorin_params *pin, thorin_disk **out)
{
  if (!pin || !out) return THORIN_ERR_ARG;
  RCHK(check_supported(*pin));
  thorin_disk *d = new thorin_disk();
  d->p = *pin;
  d->nr = pin->nrad;
  d->ns = pin->nsec;
  d->fsize = (size_t)(d->nr + 3) * (size_t)(d->ns + 1) + 5;
  CUCHK(cudaStreamCreateWithFlags(&d->s, cudaStreamNonBlocking));
  const int n1 = d->nr + 2;
  for (int q = 0; q < R_COUNT; q++) {
    size_t n = (q == R_COSTAB || q == R_SINTAB) ? (size_t)d->ns : (size_t)n1;
    RCHK(dalloc(d, (void **)&d->ring[q], n * sizeof(double)));
  }
  build_grid(d);
  RCHK(dalloc(d, (void **)&d->ctl, CTL_COUNT * sizeof(double)));
  d->g.ctl = d->ctl;
  RCHK(dalloc(d, (void **)&d->acc_args_d, sizeof(AccArgs)));
  double **F[] = {&d->rho, &d->vrad, &d->vtheta, &d->energy, &d->vrad_new, &d->vtheta_new, &d->energy_new,
                  &d->vrad_int, &d->vtheta_int, &d->energy_int, &d->cs, &d->temper, &d->qplus, &d->qminus,
                  &d->opacity, &d->divv, &d->trr, &d->trp, &d->tpp, &d->agr, &d->agt, &d->dcen, &d->ml, &d->mlip,
                  &d->mlim, &d->mljp, &d->mljm, &d->rhs, &d->sor_cw, &d->tbackup, &d->t_rho_gas, &d->t_e_gas};
  for (auto f : F) RCHK(dfield(d, f));
  if (!d->p.energy_eq) RCHK(dfield(d, &d->press));
  if (d->p.stellar_irradiation) { RCHK(dfield(d, &d->flaring)); RCHK(dfield(d, &d->qirr)); }
  else { d->flaring = d->qirr = nullptr; }
  if (d->p.pebbles) {
    double **P[] = {&d->pagr, &d->pagt, &d->pdens, &d->pvrad, &d->pvtheta, &d->psize, &d->tau, &d->paccr, &d->pacct,
                    &d->gaccr, &d->gacct, &d->dragr, &d->dragt, &d->macc, &d->t_rho_peb};
    for (auto f : P) RCHK(dfield(d, f));
  } else {
    d->pagr = d->pagt = d->pdens = d->pvrad = d->pvtheta = d->psize = d->tau = nullptr;
    d->paccr = d->pacct = d->gaccr = d->gacct = d->dragr = d->dragt = d->macc = d->t_rho_peb = nullptr;
  }
  for (int q = 0; q < 4; q++) RCHK(dfield(d, &d->ts.mom[q]));
  for (int q = 0; q < 6; q++) RCHK(dfield(d, &d->ts.w[q]));
  for (int q = 0; q < 8; q++) {
    if (q == 6 && !d->p.label_advection) { d->ts.d[q] = d->ts.f[q] = nullptr; continue; }
    RCHK(dfield(d, &d->ts.d[q]));
    RCHK(dfield(d, &d->ts.f[q]));
  }
  d->ts.w[6] = d->ts.ext = d->ts.ext_new = nullptr;
  if (d->p.label_advection) {
    RCHK(dfield(d, &d->ts.w[6]));
    RCHK(dfield(d, &d->ts.ext));
    RCHK(dfield(d, &d->ts.ext_new));
    RCHK(dfield(d, &d->label));
  }
  RCHK(dalloc(d, (void **)&d->nshift, n1 * sizeof(int)));
  d->ts.nshift = d->nshift;
  d->ts.vmed = d->ring[R_VMED];
  d->ts.vtemp = d->ring[R_VTEMP];
  if (d->p.pebbles) {
    TransportScratch &P = d->ts_peb;
    P = TransportScratch{};
    for (int q = 0; q < 4; q++) RCHK(dfield(d, &P.mom[q]));
    for (int q = 0; q < 6; q++) RCHK(dfield(d, &P.w[q]));
    // pebbles carry the four momenta (slots 0-3) and the density (slot 5,
    // its slope in slot 7): no energy or tracer slots, no slope of the
    // density quotient
    for (int q = 0; q < 8; q++) {
      const bool used = q < 4 || q == 5 || q == 7;
      P.d[q] = P.f[q] = nullptr;
      if (used && q != 5) RCHK(dfield(d, &P.d[q]));
      if (used) RCHK(dfield(d, &P.f[q]));
    }
    P.w[6] = P.ext = P.ext_new = nullptr;
    RCHK(dalloc(d, (void **)&P.nshift, n1 * sizeof(int)));
    RCHK(dalloc(d, (void **)&P.vmed, n1 * sizeof(double)));
    RCHK(dalloc(d, (void **)&P.vtemp, n1 * sizeof(double)));
    CUCHK(cudaStreamCreateWithFlags(&d->s_peb, cudaStreamNonBlocking));
    CUCHK(cudaEventCreateWithFlags(&d->ev_fork, cudaEventDisableTiming));
    CUCHK(cudaEventCreateWithFlags(&d->ev_join, cudaEventDisableTiming));
  }
  // reduction scratch: enough partials for every reduction kernel
  const size_t nb = (size_t)((d->ns + 127) / 128 + 2) * (size_t)(d->nr + 2);
  RCHK(dalloc(d, (void **)&d->partials, nb * (2 + 2 * MAXPL_DEV + 6) * sizeof(double)));
  RCHK(dalloc(d, (void **)&d->scal, 256 * sizeof(double)));
  RCHK(dalloc(d, (void **)&d->iscal, 64 * sizeof(int)));
  RCHK(dalloc(d, (void **)&d->ticket, 16 * sizeof(unsigned int)));
  RCHK(dalloc(d, (void **)&d->heat_idx_d, THORIN_MAXPLANETS * sizeof(int)));
  RCHK(dalloc(d, (void **)&d->heat_val_d, THORIN_MAXPLANETS * sizeof(double)));
  RCHK(dalloc(d, (void **)&d->damp_rings_d, n1 * sizeof(int)));
  RCHK(dalloc(d, (void **)&d->planets_d, MAXPL_DEV * sizeof(DevPlanet)));
  CUCHK(cudaMallocHost((void **)&d->scal_h, 256 * sizeof(double)));
  CUCHK(cudaMallocHost((void **)&d->iscal_h, 64 * sizeof(int)));
  CUCHK(cudaMallocHost((void **)&d->csmean_h, n1 * sizeof(double)));
  // SOR control block
  const int sb = sor_blocks(d->g);
  double *sp;
  int *ip;
  RCHK(dalloc(d, (void **)&sp, (size_t)(2 * sb + 8) * sizeof(double)));
  RCHK(dalloc(d, (void **)&ip, (size_t)(2 * sb + 8) * sizeof(int)));
  d->sor.part = sp + 8;
  d->sor.normres0 = sp;
  d->sor.normres = sp + 1;
  d->sor.jscale = sp + 2;
  d->sor.ipart = ip + 8;
  d->sor.done = ip;
  d->sor.niter = ip + 1;
  d->sor.changed = ip + 2;
  d->sor.ticket = d->ticket;
  d->sor.cond = 0;
  d->sor.has_cond = 0;
  if (const char *ek = getenv("THORIN_SOR_LOOP_SWEEPS")) {
    const int k = atoi(ek);
    if (k >= 1 && k <= 64) d->sor_loop_k = k;
  }
  if (const char *ed = getenv("THORIN_SOR_DIRECT")) d->sor_direct = (atoi(ed) != 0);
  const int ng = (sb + SOR_GROUP - 1) / SOR_GROUP;
  RCHK(dalloc(d, (void **)&d->sor.gpart, (size_t)ng * sizeof(double)));
  RCHK(dalloc(d, (void **)&d->sor.gipart, (size_t)ng * sizeof(int)));
  RCHK(dalloc(d, (void **)&d->sor.gticket, (size_t)ng * SOR_TSTRIDE * sizeof(unsigned int)));
  fill_rings(d);
  {
    PlConst &c = d->plc;                 // constants of the planet side of a substep
    const thorin_params &q = d->p;
    c.nr = d->nr; c.ns = d->ns;
    c.rin = d->Rinf[0]; c.rout = d->Rsup[d->nr - 1];
    c.plrho = q.planetary_density / RHO2CGS;
    c.tdelay = 4.0 * q.dt * (double)q.heating_delay;
    c.thickness_smoothing = q.thickness_smoothing;
    c.sqrt_adiabind_inv = 1.0 / sqrt(q.adiabind);
    c.adiabind = q.adiabind;
    c.pebble_alpha = q.pebble_alpha;
    c.vertical_damping = q.vertical_damping;
    c.mass_taper_param = q.mass_taper;
    c.indirect_term = q.indirect_term;
    c.accret_heating = q.accret_heating;
    c.feel_disk_any = q.feel_disk;
  }
  // damping rings (rows with Rmed outside [DRin, DRout])
  std::vector<int> rings;
  for (int i = 0; i < d->nr; i++)
    if (d->Rmed[i] < d->drin || d->Rmed[i] > d->drout) rings.push_back(i);
  d->ndamp = (int)rings.size();
  if (d->ndamp) CUCHK(cudaMemcpyAsync(d->damp_rings_d, rings.data(), d->ndamp * sizeof(int), cudaMemcpyHostToDevice, d->s));
  RCHK(upload_all_rings(d));
  const thorin_params &p = d->p;
  d->gm1 = p.adiabind - 1.0;
  d->gg1 = p.adiabind * (p.adiabind - 1.0);
  d->invdphi = 1.0 / (2.0 * H_MPI / (double)d->ns);
  d->lr01 = log(d->Rmed[0] / d->Rmed[1]);
  d->lr12 = log(d->Rmed[1] / d->Rmed[2]);
  d->taueff_c = p.stellar_irradiation ? 0.5 : 0.25 * sqrt(3.0);
  {
    // ImposeKeplerianEdges (Viscosity.c:221-260) with AspectRatio (:56-71)
    auto aspect = [&](double rad) {
      double ar = p.aspect_ratio;
      const double rmin = p.transition_radius - p.transition_width * p.aspect_ratio;
      const double rmax = p.transition_radius + p.transition_width * p.aspect_ratio;
      if (rad < rmin) ar *= p.transition_ratio;
      if ((rad >= rmin) && (rad <= rmax)) ar *= exp((rmax - rad) / (rmax - rmin) * log(p.transition_ratio));
      return ar;
    };
    const double r0 = d->Rmed[0], r1 = d->Rmed[d->nr - 1];
    const double vin = sqrt(1.0 * 1.0 / r0) *
                       sqrt(1.0 - pow(aspect(r0), 2.0) * pow(r0, 2.0 * p.flaring_index) *
                                      (1. + p.sigma_slope - 2.0 * p.flaring_index));
    const double vout = sqrt(1.0 * 1.0 / r1) *
                        sqrt(1.0 - pow(aspect(r1), 2.0) * pow(r1, 2.0 * p.flaring_index) *
                                       (1. + p.sigma_slope - 2.0 * p.flaring_index));
    d->vkep_in = vin;                      // inertial; the frame's rotation is taken off per substep
    d->vkep_out = vout;
  }
  d->rstar = p.stellar_radius * 6.957e8 / AU_SI;
  {
    double Teff4 = pow(p.effective_temperature / T2SI, 4.0);
    double Rstar2 = pow(p.stellar_radius * (6.957e8 / AU_SI), 2.0);
    d->tirr4fac = (1.0 - p.disc_albedo) * Teff4 * Rstar2;
  }
  d->vp.viscosity = p.viscosity; d->vp.alpha = p.alpha_viscosity; d->vp.alpha_mri = p.alpha_mri;
  d->vp.alpha_dead = p.alpha_dead; d->vp.tmri = p.tmri; d->vp.twidth = p.twidth; d->vp.t2si = T2SI;
  d->vp.cav_rmin = p.cavity_radius - p.cavity_width * p.aspect_ratio;
  d->vp.cav_rmax = p.cavity_radius + p.cavity_width * p.aspect_ratio;
  d->vp.cav_ratio = p.cavity_ratio; d->vp.log_cav_ratio = log(p.cavity_ratio);
  d->vp.viscosity_alpha = p.viscosity_alpha; d->vp.alpha_flock = p.alpha_flock;
  if (p.lambda_doubling != 0.0) { g_last_error = "LambdaDoubling is not supported"; return THORIN_ERR_ARG; }
  d->OmegaFrame = p.omega_frame;
  d->MassTaper = 1.0;
  d->cfl_first = 1;
  d->sor_first = 1;
  d->heatsrc_max = 0;
  for (int k = 0; k < THORIN_MAXPLANETS; k++) { d->heatsrc[k] = 0.0; d->heatsrc_index[k] = -1; }
  memset(&d->st, 0, sizeof(d->st));
  d->scal_h[SC_DTSTELLAR] = 1.0e38;                   // global.h:47
  CUCHK(cudaMemcpyAsync(d->scal + SC_DTSTELLAR, d->scal_h + SC_DTSTELLAR, sizeof(double), cudaMemcpyHostToDevice, d->s));
  for (int q = 0; q < 4; q++) CUCHK(cudaEventCreate(&d->ev[q]));
  d->timing = 0;
  CUCHK(cudaStreamSynchronize(d->s));
  CUCHK(cudaMallocHost((void **)&d->nshift_h, (size_t)d->nr * sizeof(int)));
  memset(d->nshift_h, 0, (size_t)d->nr * sizeof(int));
  *out = d;
  return THORIN_OK;
}

// Update history of the warm start with at least nh slots (zeroed, no time
// step recorded); a larger history replaces the old one.
static int ws_history(thorin_disk *d, int nh)
{
  const size_t cells = (size_t)d->nr * d->ns;
  if (!d->ws_jac) {
    RCHK(dalloc(d, (void **)&d->ws_jac, cells * sizeof(double)));
    RCHK(dalloc(d, (void **)&d->ws_dts, THORIN_WS_MAX_ORDER * sizeof(double)));
    RCHK(dalloc(d, (void **)&d->ws_part, (size_t)(4 * d->g.nsm + 2) * sizeof(double)));
    RCHK(dalloc(d, (void **)&d->ws_step, 2 * sizeof(double)));
  }
  if (nh <= d->ws_nh) return THORIN_OK;
  if (d->ws_prev) {
    d->allocs.erase(std::find(d->allocs.begin(), d->allocs.end(), (void *)d->ws_prev));
    CUCHK(cudaStreamSynchronize(d->s));
    cudaFree(d->ws_prev);
    d->ws_prev = nullptr;
  }
  if (d->dt_graph) {                               // the DT graph holds the old history's address
    cudaGraphExecDestroy(d->dt_graph);
    d->dt_graph = nullptr;
  }
  RCHK(dalloc(d, (void **)&d->ws_prev, (size_t)nh * cells * sizeof(double)));
  CUCHK(cudaMemsetAsync(d->ws_dts, 0, THORIN_WS_MAX_ORDER * sizeof(double), d->s));
  d->ws_nh = nh;
  return THORIN_OK;
}

extern "C" int thorin_gpu_warmstart(thorin_disk *d, thorin_warmnet *n, int mode, float lr)
{
  if (!d || mode < THORIN_WS_OFF || mode > THORIN_WS_EXTRAPOLATE ||
      ((mode == THORIN_WS_PREDICT || mode == THORIN_WS_TRAIN) && !n) ||
      (mode == THORIN_WS_TRAIN && !(lr > 0.f))) {
    g_last_error = "warmstart: mode OFF/PREDICT/TRAIN/EXTRAPOLATE, a network to predict or train, lr > 0 to train";
    return THORIN_ERR_ARG;
  }
  if (mode == THORIN_WS_EXTRAPOLATE || mode == THORIN_WS_OFF) n = nullptr;
  int f = 1;
  if (n) {
    int nr = 0, ns = 0;
    wn_dims(n, &nr, &ns);
    if (nr == d->nr && ns == d->ns) f = 1;
    else if (2 * nr == d->nr && 2 * ns == d->ns) f = 2;
    else {
      g_last_error = "warmstart: the network's grid must be the disk's or half of it in both directions";
      return THORIN_ERR_ARG;
    }
  }
  if (mode != THORIN_WS_OFF)
    RCHK(ws_history(d, mode == THORIN_WS_EXTRAPOLATE ? d->ws_order : 1));
  if (mode == THORIN_WS_EXTRAPOLATE && !d->ws_vq)
    RCHK(dalloc(d, (void **)&d->ws_vq, 2 * (size_t)d->nr * d->ns * sizeof(double)));
  if (d->ws_dts)                                   // every attach starts without recorded updates
    CUCHK(cudaMemsetAsync(d->ws_dts, 0, THORIN_WS_MAX_ORDER * sizeof(double), d->s));
  d->ws_f = f;
  if (d->dt_graph && (d->ws_net != n || d->ws_mode != mode)) {
    cudaGraphExecDestroy(d->dt_graph);            // the DT graph holds the warm start's launches or not
    d->dt_graph = nullptr;
  }
  d->ws_net = n;
  d->ws_mode = mode;
  d->ws_lr = lr;
  return THORIN_OK;
}

extern "C" int thorin_gpu_warmstart_order(thorin_disk *d, int order)
{
  if (!d || order < 1 || order > THORIN_WS_MAX_ORDER) {
    g_last_error = "warmstart order: 1 .. THORIN_WS_MAX_ORDER";
    return THORIN_ERR_ARG;
  }
  if (order == d->ws_order) return THORIN_OK;
  d->ws_order = order;
  if (d->ws_mode == THORIN_WS_EXTRAPOLATE) RCHK(ws_history(d, order));
  if (d->dt_graph) {                               // the order is baked into the DT graph's launch
    cudaGraphExecDestroy(d->dt_graph);
    d->dt_graph = nullptr;
  }
  return THORIN_OK;
}

extern "C" int thorin_gpu_warmstart_stats(thorin_disk *d, thorin_ws_stats *out)
{
  if (!d || !out) return THORIN_ERR_ARG;
  CUCHK(cudaStreamSynchronize(d->s));
  if (d->ws_net && d->ws_st.train_steps > 0) {
    double l[3];
    RCHK(wn_last_loss(d->ws_net, l));
    d->ws_st.last_loss = l[0];
    d->ws_st.last_res_loss = l[1];
    d->ws_st.last_sup_loss = l[2];
  }
  if (d->ws_step) CUCHK(cudaMemcpy(&d->ws_st.step_sum, d->ws_step + 1, sizeof(double), cudaMemcpyDeviceToHost));
  *out = d->ws_st;
  return THORIN_OK;
}

extern "C" int thorin_gpu_destroy(thorin_disk *d)
{
  if (!d) return THORIN_OK;
  cudaStreamSynchronize(d->s);
  for (void *a : d->allocs) cudaFree(a);
  cudaFreeHost(d->scal_h);
  cudaFreeHost(d->iscal_h);
  cudaFreeHost(d->csmean_h);
  if (d->nshift_h) cudaFreeHost(d->nshift_h);
  if (d->sor_loop) cudaGraphExecDestroy(d->sor_loop);
  if (d->dt_graph) cudaGraphExecDestroy(d->dt_graph);
  if (d->sys_h) cudaFreeHost(d->sys_h);
  if (d->gst_h) cudaFreeHost(d->gst_h);
  if (d->ctl_h) cudaFreeHost(d->ctl_h);
  if (d->s_pl) {
    cudaStreamSynchronize(d->s_pl);
    cudaEventDestroy(d->ev_pl_fork);
    cudaEventDestroy(d->ev_pl_join);
    cudaStreamDestroy(d->s_pl);
  }
  for (int q = 0; q < 4; q++) cudaEventDestroy(d->ev[q]);
  if (d->s_peb) {
    cudaStreamSynchronize(d->s_peb);
    cudaEventDestroy(d->ev_fork);
    cudaEventDestroy(d->ev_join);
    cudaStreamDestroy(d->s_peb);
  }
  cudaStreamDestroy(d->s);
  delete d;
  return THORIN_OK;
}

static double *field_ptr(thorin_disk *d, int id)
{
  switch (id) {
  case THORIN_DENS: return d->rho;
  case THORIN_VRAD: return d->vrad;
  case THORIN_VTHETA: return d->vtheta;
  case THORIN_ENERGY: return d->energy;
  case THORIN_PEBDENS: return d->pdens;
  case THORIN_PEBVRAD: return d->pvrad;
  case THORIN_PEBVTHETA: return d->pvtheta;
  case THORIN_PEBSIZE: return d->psize;
  case THORIN_TEMPER: return d->temper;
  case THORIN_SOUNDSPEED: return d->cs;
  case THORIN_STOKES: return d->tau;
  case THORIN_QPLUS: return d->qplus;
  case THORIN_DIVV: return d->divv;
  case THORIN_OPACITY: return d->opacity;
  case THORIN_QMINUS: return d->qminus;
  case THORIN_LABEL: return d->label;
  }
  return nullptr;
}

extern "C" int thorin_gpu_upload(thorin_disk *d, int field, const double *host)
{
  if (!d || !host) return THORIN_ERR_ARG;
  double *f = field_ptr(d, field);
  if (!f || field == THORIN_PRESSURE) { g_last_error = "field not available"; return THORIN_ERR_ARG; }
  CUCHK(cudaMemcpyAsync(f, host, (size_t)(d->nr + 1) * d->ns * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

// pressure (SourceEuler.c:740-762) is formed on the fly in the kernels; it
// is rebuilt here from the energy when asked for.
extern "C" int thorin_gpu_download(thorin_disk *d, int field, double *host)
{
  if (!d || !host) return THORIN_ERR_ARG;
  const size_t n = (size_t)(d->nr + 1) * d->ns;
  if (field == THORIN_PRESSURE) {
    CUCHK(cudaMemcpyAsync(host, d->energy, n * sizeof(double), cudaMemcpyDeviceToHost, d->s));
    CUCHK(cudaStreamSynchronize(d->s));
    for (size_t l = 0; l < (size_t)d->nr * d->ns; l++) host[l] = d->gm1 * host[l];
    for (size_t l = (size_t)d->nr * d->ns; l < n; l++) host[l] = 0.0;
    return THORIN_OK;
  }
  double *f = field_ptr(d, field);
  if (!f) { g_last_error = "field not available"; return THORIN_ERR_ARG; }
  CUCHK(cudaMemcpyAsync(host, f, n * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

static std::vector<double> *profile_vec(thorin_disk *d, int id, int *ring)
{
  switch (id) {
  case THORIN_SIGMAMED: *ring = R_SIGMAMED; return &d->SigmaMed;
  case THORIN_SIGMAINF: *ring = -1; return &d->SigmaInf;
  case THORIN_ENERGYMED: *ring = R_ENERGYMED; return &d->EnergyMed;
  case THORIN_VTHETAMED: *ring = R_VTHETAMED; return &d->VthetaMed;
  case THORIN_PEBDENSINIT: *ring = R_PEBDENS0; return &d->PebDensInit;
  case THORIN_PEBVRADINIT: *ring = R_PEBVRAD0; return &d->PebVradInit;
  case THORIN_PEBVTHETAINIT: *ring = R_PEBVTHETA0; return &d->PebVthetaInit;
  }
  return nullptr;
}

extern "C" int thorin_gpu_set_profile(thorin_disk *d, int profile, const double *host)
{
  int ring;
  std::vector<double> *v = profile_vec(d, profile, &ring);
  if (!v || !host) return THORIN_ERR_ARG;
  for (int i = 0; i < d->nr; i++) (*v)[i] = host[i];
  if (ring >= 0) RCHK(upload_ring(d, ring, *v));
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

extern "C" int thorin_gpu_get_profile(thorin_disk *d, int profile, double *host)
{
  int ring;
  std::vector<double> *v = profile_vec(d, profile, &ring);
  if (!v || !host) return THORIN_ERR_ARG;
  for (int i = 0; i < d->nr; i++) host[i] = (*v)[i];
  return THORIN_OK;
}

extern "C" int thorin_gpu_get_rings(thorin_disk *d, double *rinf, double *rsup, double *rmed, double *surf)
{
  if (!d) return THORIN_ERR_ARG;
  for (int i = 0; i < d->nr; i++) {
    if (rinf) rinf[i] = d->Rinf[i];
    if (rsup) rsup[i] = d->Rsup[i];
    if (rmed) rmed[i] = d->Rmed[i];
    if (surf) surf[i] = d->Surf[i];
  }
  return THORIN_OK;
}

extern "C" int thorin_gpu_set_time(thorin_disk *d, double t)
{
  d->PhysicalTime = t;
  d->PhysicalTimeInitial = t;
  return THORIN_OK;
}

extern "C" int thorin_gpu_get_nshift(thorin_disk *d, int *host)
{
  if (!d || !host) return THORIN_ERR_ARG;
  CUCHK(cudaStreamSynchronize(d->s));      // the last transport's copy has landed
  for (int i = 0; i < d->nr; i++) host[i] = d->nshift_h[i];
  return THORIN_OK;
}

extern "C" int thorin_gpu_set_opacity_table(thorin_disk *d, int rows, int cols, const double *pgrid, const double *tgrid,
                                            const double *planck, const double *rosseland)
{
  if (!d || rows < 2 || cols < 3 || !pgrid || !tgrid || !rosseland) {
    g_last_error = "opacity table: rows >= 2, cols >= 3 and the grids and the Rosseland table are required";
    return THORIN_ERR_ARG;
  }
  (void)planck;                                   // the hydro uses Rosseland means only (opacity_SM03)
  double *pg, *tg, *ro;
  RCHK(dalloc(d, (void **)&pg, rows * sizeof(double)));
  RCHK(dalloc(d, (void **)&tg, cols * sizeof(double)));
  RCHK(dalloc(d, (void **)&ro, (size_t)rows * cols * sizeof(double)));
  CUCHK(cudaMemcpyAsync(pg, pgrid, rows * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(tg, tgrid, cols * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(ro, rosseland, (size_t)rows * cols * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  d->g.k.sm_pgrid = pg; d->g.k.sm_tgrid = tg; d->g.k.sm_ross = ro;
  d->g.k.sm_rows = rows; d->g.k.sm_cols = cols;
  return THORIN_OK;
}

extern "C" int thorin_gpu_set_frame(thorin_disk *d, double omega_frame)
{
  if (!d) return THORIN_ERR_ARG;
  d->OmegaFrame = omega_frame;
  return THORIN_OK;
}

extern "C" int thorin_gpu_get_stats(thorin_disk *d, thorin_stats *s)
{
  *s = d->st;
  s->physical_time = d->PhysicalTime;
  s->omega_frame = d->OmegaFrame;
  s->kernel_launches = g_thorin_launches.load();
  return THORIN_OK;
}

// EOS refresh of the state, ring-mean sound speed (and temperature), and the
// viscosity per ring; the ring means are mirrored to the host.
// AspectRatio (Viscosity.c:56-71) at the current time.
static double aspect_ratio_host(const thorin_disk *d, double rad)
{
  const thorin_params &p = d->p;
  double ar = p.aspect_ratio;
  double rmin = p.transition_radius - p.transition_width * p.aspect_ratio;
  double rmax = p.transition_radius + p.transition_width * p.aspect_ratio;
  const double scale = 1.0 + (d->PhysicalTime - d->PhysicalTimeInitial) * p.lambda_doubling;
  rmin *= scale;
  rmax *= scale;
  if (rad < rmin) ar *= p.transition_ratio;
  if ((rad >= rmin) && (rad <= rmax)) ar *= exp((rmax - rad) / (rmax - rmin) * log(p.transition_ratio));
  return ar;
}

// Isothermal sound speed of ring i (ComputeSoundSpeed, SourceEuler.c:729-731).
static double cs_iso_host(const thorin_disk *d, int i)
{
  const double r = d->Rmed[i];
  return aspect_ratio_host(d, r) * sqrt(1.0 * 1.0 / r) * pow(r, d->p.flaring_index);
}

// ComputeSoundSpeed, ComputePressureField, ComputeTemperatureField and the
// ring means that depend on them (Init.c:131-133).
static int eos_refresh(thorin_disk *d)
{
  if (d->p.energy_eq) {
    hydro_eos(d->g, d->rho, d->energy, d->temper, d->cs, d->gm1, d->gg1, d->s);
  } else {
    std::vector<double> c(d->nr + 2, 0.0);
    for (int i = 0; i < d->nr; i++) c[i] = cs_iso_host(d, i);
    RCHK(upload_ring(d, R_CSISO, c));
    aux_iso_eos(d->g, d->rho, d->ring[R_CSISO], d->cs, d->press, d->temper, 1, 1, 1, d->s);
  }
  aux_ring_mean(d->g, d->cs, d->ring[R_CSMEAN], d->s);
  if (d->p.alpha_flock) aux_ring_mean(d->g, d->temper, d->ring[R_TEMPMEAN], d->s);
  aux_viscosity_rings(d->g, d->vp, d->s);
  CUCHK(cudaMemcpyAsync(d->csmean_h, d->ring[R_CSMEAN], d->nr * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  return THORIN_OK;
}

// ---------------------------------------------------------------------------
// Default initial state, built on the host like the reference does once
// (InitEuler, SourceEuler.c:133-175; main.c:168-170).
// EtaPressureSupport + InitPebblesViaFlux (Pebbles.c:80-275): the pebble disk
// in a coagulation-drift equilibrium with the given gas state (host copies
// of Sigma, v_r, v_theta and c_s in the PolarGrid layout).
static int init_pebbles_host(thorin_disk *d, const std::vector<double> &rho, const std::vector<double> &vr,
                             const std::vector<double> &vt, const std::vector<double> &cs)
{
  const thorin_params &p = d->p;
  const int nr = d->nr, ns = d->ns;
  const size_t n = (size_t)(nr + 1) * ns;
  std::vector<double> etacc(n, 0.0), etafc(n, 0.0), pd(n, 0.0), pvr(n, 0.0), pvt(n, 0.0), ps(n, 0.0), tau(n, 0.0);
  for (int i = 0; i < nr; i++) {
    const double vtcorr = d->Rmed[i] * d->OmegaFrame, vkinv = sqrt(d->Rmed[i]);
    for (int j = 0; j < ns; j++) {
      const int l = j + i * ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      const double vtcc = 0.5 * (vt[l] + vt[ljp]);
      etacc[l] = 1.0 - (vtcc + vtcorr) * vkinv;
    }
  }
  for (int i = 1; i < nr; i++)
    for (int j = 0; j < ns; j++) { const int l = j + i * ns; etafc[l] = 0.5 * (etacc[l] + etacc[l - ns]); }
  for (int j = 0; j < ns; j++) etafc[j] = etafc[j + ns];
  const double pebbleflux = p.pebble_flux * FLUX2CU, Ndf = 0.5, pb = p.pebble_bulk_dens / RHO2CGS;
  for (int i = 0; i < nr; i++) {
    double rho1 = 0, vr1 = 0, etafc1 = 0, etacc1 = 0, cs1 = 0;
    for (int j = 0; j < ns; j++) {
      const int l = j + i * ns;
      rho1 += rho[l]; vr1 += vr[l]; etafc1 += etafc[l]; etacc1 += etacc[l]; cs1 += cs[l];
    }
    rho1 /= (double)ns; vr1 /= (double)ns; etafc1 /= (double)ns; etacc1 /= (double)ns; cs1 /= (double)ns;
    double tau1 = sqrt(3.0) * p.pebble_coagulation * pebbleflux / (32.0 * H_PI * pow(d->Rmed[i], -1.5) * rho1);
    tau1 = sqrt(tau1) / (d->Rmed[i] * etacc1);
    double psize1 = fabs(tau1) * sqrt(p.adiabind) * rho1 / (2.0 * pb);
    const double taudf = p.fragment_threshold * sqrt(d->Rmed[i]) / (2.0 * etacc1 * (1.0 - Ndf));
    const double adf = fabs(taudf) * sqrt(p.adiabind) * rho1 / (2.0 * pb);
    const double taufrag = p.fragment_factor / (3.0 * p.fragment_alpha) * pow(p.fragment_threshold / cs1, 2);
    const double afrag = fabs(taufrag) * sqrt(p.adiabind) * rho1 / (2.0 * pb);
    if ((psize1 < adf) && (psize1 < afrag)) {
    } else if ((taudf > 0.0) && (adf < psize1) && (adf < afrag)) {
      tau1 = taudf; psize1 = adf;
    } else {
      tau1 = taufrag; psize1 = afrag;
    }
    const double vtcorr = d->Rmed[i] * d->OmegaFrame, vkepl = pow(d->Rmed[i], -0.5);
    const double fac = 1.0 / (tau1 * tau1 + 1.0);
    double etaterm = etafc1 * vkepl;
    const double pvr1 = -2.0 * tau1 * fac * (etaterm - 0.5 / tau1 * vr1);
    etaterm = etacc1 * vkepl;
    const double pvrtemp = -2.0 * tau1 * fac * (etaterm - 0.5 / tau1 * vr1);
    double pvt1 = -fac * (etaterm - 0.5 * tau1 * vr1);
    pvt1 += (vkepl - vtcorr);
    double pdens1 = pebbleflux / (2.0 * H_PI * d->Rmed[i] * fabs(pvrtemp));
    if (pdens1 / rho1 > p.pebble_to_gas_max) pdens1 = rho1 * p.pebble_to_gas_max;
    for (int j = 0; j < ns; j++) {
      const int l = j + i * ns;
      ps[l] = psize1; tau[l] = tau1; pd[l] = pdens1; pvr[l] = pvr1; pvt[l] = pvt1;
    }
    d->PebDensInit[i] = pdens1;
    d->PebVradInit[i] = pvr1;
    d->PebVthetaInit[i] = pvt1 + d->Rmed[i] * d->OmegaFrame;
  }
  CUCHK(cudaMemcpyAsync(d->pdens, pd.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(d->pvrad, pvr.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(d->pvtheta, pvt.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(d->psize, ps.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(d->tau, tau.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

extern "C" int thorin_gpu_init_default(thorin_disk *d)
{
  const thorin_params &p = d->p;
  const int nr = d->nr, ns = d->ns;
  const size_t n = (size_t)(nr + 1) * ns;
  std::vector<double> rho(n, 0.0), e(n, 0.0), vr(n, 0.0), vt(n, 0.0), cs(n, 0.0);
  auto sigma = [&](double r) {            // Theo.c:15-23
    double cavity = 1.0;
    if (r < p.cavity_radius) cavity = 1.0 / p.cavity_ratio;
    return cavity * p.scaling_factor * p.sigma0 * pow(r, -p.sigma_slope);
  };
  auto energy = [&](double r) {           // Theo.c:60-74
    double fac = 1.0 / (1.0 * (p.adiabind - 1.0));
    double power = -p.sigma_slope - 1.0 + 2.0 * p.flaring_index;
    return 1.0 * p.sigma0 * pow(p.aspect_ratio, 2.0) * pow(r, power) * fac;
  };
  for (int i = 0; i < nr; i++) {
    d->SigmaMed[i] = sigma(d->Rmed[i]);
    d->SigmaInf[i] = sigma(d->Rinf[i]);
    d->EnergyMed[i] = energy(d->Rmed[i]);
  }
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) { rho[j + i * ns] = d->SigmaMed[i]; e[j + i * ns] = d->EnergyMed[i]; }
  std::vector<double> csm(nr + 2, 0.0);
  for (int i = 0; i < nr; i++) {
    double sacc = 0.0;
    const double csi = p.energy_eq ? 0.0 : cs_iso_host(d, i);
    for (int j = 0; j < ns; j++) {
      const int l = j + i * ns;
      cs[l] = p.energy_eq ? sqrt(p.adiabind * (p.adiabind - 1.0) * fabs(e[l]) / rho[l]) : csi;
      sacc += cs[l];
    }
    csm[i] = sacc / (double)ns;
  }
  if (p.parametric_cooling) {             // FillCoolingTime, FillQplus (Theo.c:103-129)
    std::vector<double> ct(nr + 2, 0.0), qm(nr + 2, 0.0);
    for (int i = 0; i < nr; i++) {
      ct[i] = p.cooling_time * pow(d->Rmed[i], 2.0 + 2.0 * p.flaring_index);
      qm[i] = 2.25 * fviscosity_host(d, i, d->Rmed[i], csm) * p.sigma0 * pow(d->Rmed[i], -p.sigma_slope - 3.0);
    }
    RCHK(upload_ring(d, R_COOLT, ct));
    RCHK(upload_ring(d, R_QPLUSMED, qm));
  }
  // -b: v_theta from the radial balance of pressure, gravity and rotation
  // (InitGasVelocity, Pframeforce.c:666-688, with ConstructSequence :605-617)
  std::vector<double> vt_cent(nr + 2, 0.0);
  if (p.centrifugal_balance) {
    std::vector<double> gp(nr + 2, 0.0), vt_int(nr + 2, 0.0);
    for (int i = 0; i < nr; i++) {
      double acc = 0.0;
      for (int j = 0; j < ns; j++) {
        const int l = j + i * ns;
        acc += p.energy_eq ? (p.adiabind - 1.0) * e[l] : rho[l] * cs[l] * cs[l];
      }
      gp[i] = acc / (double)ns;
    }
    const std::vector<double> &GR = d->GlobalRmed;
    for (int i = 1; i < nr; i++) {
      vt_int[i] = (gp[i] - gp[i - 1]) / (.5 * (sigma(GR[i]) + sigma(GR[i - 1]))) / (GR[i] - GR[i - 1]) +
                  1.0 * (1.0 / GR[i - 1] - 1.0 / GR[i]) / (GR[i] - GR[i - 1]);
      vt_int[i] = sqrt(vt_int[i] * d->Radii[i]) - d->Radii[i] * d->OmegaFrame;
    }
    auto construct = [&](void) {
      for (int i = 1; i < nr; i++) vt_cent[i] = 2.0 * vt_int[i] - vt_cent[i - 1];
      double lapl = 0.0;
      for (int i = 1; i < nr - 1; i++) lapl += fabs(vt_cent[i + 1] + vt_cent[i - 1] - 2.0 * vt_cent[i]);
      return lapl;
    };
    double t1 = vt_cent[0] = vt_int[1] + .75 * (vt_int[1] - vt_int[2]);
    const double r1 = construct();
    vt_cent[0] += .25 * (vt_int[1] - vt_int[2]);
    const double t2 = vt_cent[0];
    const double r2 = construct();
    t1 = t1 - r1 / (r2 - r1) * (t2 - t1);
    vt_cent[0] = t1;
    construct();
    vt_cent[nr] = vt_cent[nr - 1];
  }
  // InitGasVelocity (Pframeforce.c:696-750)
  for (int i = 0; i <= nr; i++) {
    double r, ri;
    int ir;
    if (i == nr) { r = d->Rmed[nr - 1]; ri = d->Rinf[nr - 1]; ir = nr - 1; }
    else { r = d->Rmed[i]; ri = d->Rinf[i]; ir = i; }
    const double viscosity = fviscosity_host(d, ir, r, csm);
    for (int j = 0; j < ns; j++) {
      const int l = j + i * ns;
      const double rg = r, omega = sqrt(1.0 * 1.0 / rg / rg / rg);
      const double csl = (i == nr) ? 0.0 : cs[l];   // SoundSpeed row nrad is never set (zero)
      vt[l] = omega * r * sqrt(1.0 - csl * csl * r / p.adiabind);
      vt[l] -= d->OmegaFrame * r;
      if (p.centrifugal_balance) vt[l] = vt_cent[i];
      vr[l] = p.imposed_disk_drift * p.sigma0 / d->SigmaInf[i] / ri;
      if (p.damp_flux) {                   // steady inflow of GASFLUX (Pframeforce.c:735-740)
        const double rhoinf = (i == 0) ? d->SigmaMed[i] - 0.5 * (d->SigmaMed[i + 1] - d->SigmaMed[i])
                                       : 0.5 * (d->SigmaMed[i - 1] + d->SigmaMed[i]);
        vr[l] -= p.gasflux / (2.0 * H_PI * ri * rhoinf);
      } else if (p.viscosity_alpha) {
        vr[l] -= 3.0 * viscosity / r * (-p.sigma_slope + 2.0 * p.flaring_index + 1.0);
      } else {
        vr[l] -= 3.0 * viscosity / r * (-p.sigma_slope + .5);
      }
    }
  }
  if (!p.damp_flux)
    for (int j = 0; j < ns; j++) vr[j] = vr[j + ns * nr] = 0.0;
  if (p.damp_init)                         // FillVtheta (Theo.c:132-151)
    for (int i = 0; i < nr; i++) {
      double moy = 0.0;
      const double vtcorr = d->Rmed[i] * d->OmegaFrame;
      for (int j = 0; j < ns; j++) moy += vt[j + i * ns] + vtcorr;
      d->VthetaMed[i] = moy / (double)ns;
    }
  CUCHK(cudaMemcpyAsync(d->rho, rho.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(d->energy, e.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(d->vrad, vr.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaMemcpyAsync(d->vtheta, vt.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  std::vector<double> lab;
  if (p.label_advection) {                 // InitLabel (Init.c:59-72), rows 0..nrad
    lab.assign(n, 0.0);
    for (int i = 0; i <= nr; i++)
      for (int j = 0; j < ns; j++) lab[j + i * ns] = (d->Rmed[i] - p.rmin) / (p.rmax - p.rmin);
    CUCHK(cudaMemcpyAsync(d->label, lab.data(), n * sizeof(double), cudaMemcpyHostToDevice, d->s));
  }
  CUCHK(cudaStreamSynchronize(d->s));
  if (p.pebbles) RCHK(init_pebbles_host(d, rho, vr, vt, cs));
  RCHK(upload_all_rings(d));
  RCHK(eos_refresh(d));
  KCHECK("initial EOS kernels");
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

// Ring means of a device field (warp tree sums) to the host.
static int ring_means_host(thorin_disk *d, const double *f, std::vector<double> &out)
{
  aux_ring_mean(d->g, f, d->ring[R_VMOY], d->s);
  out.assign(d->nr + 2, 0.0);
  CUCHK(cudaMemcpyAsync(out.data(), d->ring[R_VMOY], d->nr * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

extern "C" int thorin_gpu_refresh(thorin_disk *d, int flags)
{
  const thorin_params &p = d->p;
  const int nr = d->nr;
  if (flags == THORIN_REFRESH_RING_MEANS) {
    // a state put back as it was at the end of a DT (fields, c_s and T
    // included): the ring means and viscosities the next substep reads
    aux_ring_mean(d->g, d->cs, d->ring[R_CSMEAN], d->s);
    if (p.alpha_flock) aux_ring_mean(d->g, d->temper, d->ring[R_TEMPMEAN], d->s);
    aux_viscosity_rings(d->g, d->vp, d->s);
    CUCHK(cudaMemcpyAsync(d->csmean_h, d->ring[R_CSMEAN], d->nr * sizeof(double), cudaMemcpyDeviceToHost, d->s));
    CUCHK(cudaStreamSynchronize(d->s));
    return THORIN_OK;
  }
  if (flags & THORIN_REFILL_GAS) {
    std::vector<double> m;
    RCHK(ring_means_host(d, d->rho, m));                    // RefillSigma, Theo.c:33-57
    for (int i = 0; i < nr; i++) d->SigmaMed[i] = m[i];
    d->SigmaInf[0] = d->SigmaMed[0];
    for (int i = 1; i < nr; i++)
      d->SigmaInf[i] = (d->SigmaMed[i - 1] * (d->Rmed[i] - d->Rinf[i]) + d->SigmaMed[i] * (d->Rinf[i] - d->Rmed[i - 1])) /
                       (d->Rmed[i] - d->Rmed[i - 1]);
    if (p.energy_eq) {
      RCHK(ring_means_host(d, d->energy, m));               // RefillEnergy, Theo.c:82-100
      for (int i = 0; i < nr; i++) d->EnergyMed[i] = m[i];
    }
    if (p.damp_init) {
      RCHK(ring_means_host(d, d->vtheta, m));               // FillVtheta, Theo.c:132-151
      for (int i = 0; i < nr; i++) d->VthetaMed[i] = m[i] + d->Rmed[i] * d->OmegaFrame;
    }
  }
  if ((flags & THORIN_REFILL_PEBBLES) && p.pebbles) {       // BckpFieldsForBC, Pebbles.c:208-232
    std::vector<double> m;
    RCHK(ring_means_host(d, d->pdens, m));
    for (int i = 0; i < nr; i++) d->PebDensInit[i] = m[i];
    RCHK(ring_means_host(d, d->pvrad, m));
    for (int i = 0; i < nr; i++) d->PebVradInit[i] = m[i];
    RCHK(ring_means_host(d, d->pvtheta, m));
    for (int i = 0; i < nr; i++) d->PebVthetaInit[i] = m[i] + d->Rmed[i] * d->OmegaFrame;
  }
  RCHK(upload_all_rings(d));
  RCHK(eos_refresh(d));
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

// EquilPebbleDisk on the current gas state, for runs that load the gas from
// files (Init.c:144-148): after the gas fields are uploaded.
extern "C" int thorin_gpu_init_pebbles(thorin_disk *d)
{
  if (!d) return THORIN_ERR_ARG;
  if (!d->p.pebbles) return THORIN_OK;
  const size_t n = (size_t)(d->nr + 1) * d->ns;
  RCHK(eos_refresh(d));
  std::vector<double> rho(n), vr(n), vt(n), cs(n);
  CUCHK(cudaMemcpyAsync(rho.data(), d->rho, n * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaMemcpyAsync(vr.data(), d->vrad, n * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaMemcpyAsync(vt.data(), d->vtheta, n * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaMemcpyAsync(cs.data(), d->cs, n * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  RCHK(init_pebbles_host(d, rho, vr, vt, cs));
  RCHK(upload_all_rings(d));
  RCHK(eos_refresh(d));
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

// ---------------------------------------------------------------------------
// Host N-body step standing in for REBOUND's IAS15 (ReboundInterface.c:
// 262-325): heliocentric -> barycentric, star + planets with mutual gravity
// over dt (classical RK4 with 256 substeps), back to heliocentric.




extern "C" int thorin_planet_from_elements(thorin_planets *sys, int k, float mass, float gas, float solid, float a,
                                           float e, float inc, float Omega, float omega, float f)
{
  // SetupReboundSimulation (ReboundInterface.c:137-192) with
  // reb_tools_orbit_to_particle (Murray & Dermott eqs. 2.122, 2.36).
  if (!sys || k < 0 || k >= THORIN_MAXPLANETS) return THORIN_ERR_ARG;
  const double rad = H_PI / 180.0;
  const double m = mass, aa = a, ee = e, in = (double)inc * rad, Om = (double)Omega * rad, om = (double)omega * rad,
               ff = (double)f * rad;
  const double r = aa * (1 - ee * ee) / (1 + ee * cos(ff));
  const double v0 = sqrt(1.0 * (m + 1.0) / aa / (1. - ee * ee));
  const double cO = cos(Om), sO = sin(Om), co = cos(om), so = sin(om), cf = cos(ff), sf = sin(ff), ci = cos(in),
               si = sin(in);
  sys->mass[k] = m; sys->gas[k] = gas; sys->solid[k] = solid;
  sys->x[k] = 0.0 + r * (cO * (co * cf - so * sf) - sO * (so * cf + co * sf) * ci);
  sys->y[k] = 0.0 + r * (sO * (co * cf - so * sf) + cO * (so * cf + co * sf) * ci);
  sys->z[k] = 0.0 + r * (so * cf + co * sf) * si;
  sys->vx[k] = 0.0 + v0 * ((ee + cf) * (-ci * co * sO - cO * so) - sf * (co * cO - ci * so * sO));
  sys->vy[k] = 0.0 + v0 * ((ee + cf) * (ci * co * cO - sO * so) - sf * (co * sO + ci * so * cO));
  sys->vz[k] = 0.0 + v0 * ((ee + cf) * co * si - sf * si * so);
  sys->ax[k] = sys->ay[k] = sys->az[k] = 0.0;
  if (k >= sys->nb) sys->nb = k + 1;
  return THORIN_OK;
}

// Writes control-block values (stream-ordered) for the kernels that follow.
static void set_ctl(thorin_disk *d, std::initializer_list<std::pair<int, double>> kv, cudaStream_t s = nullptr)
{
  CtlSet v;
  v.n = 0;
  for (const auto &e : kv) { v.idx[v.n] = e.first; v.val[v.n] = e.second; v.n++; }
  aux_set_ctl(d->ctl, v, s ? s : d->s);
}

// ---------------------------------------------------------------------------
// Substep pieces
// ConditionCFL's fixed arguments (the interval and the rebound rate are in
// the control block).
static CflFinal cfl_args(const thorin_disk *d)
{
  const thorin_params &p = d->p;
  CflFinal f;
  memset(&f, 0, sizeof(f));
  f.pebbles = p.pebbles && !d->sloppy_pass && !p.sloppy_cfl;   // SloppyCFL: CriticalCharTime is never called (rate 0)
  f.first_call = d->cfl_first;
  f.minimum_step = p.minimum_step;
  f.maximum_step = p.maximum_step;
  f.first_step = p.first_step;
  f.twopi_cfl_ns = 2.0 * H_PI * 0.5 / (double)d->ns;
  return f;
}

static void cfl_launches(thorin_disk *d)
{
  const thorin_params &p = d->p;
  if (p.pebbles) aux_stokes(d->g, d->rho, d->psize, d->tau, d->s);       // PebbleStokesNumbers
  aux_cfl(d->g, d->vrad, d->vtheta, d->cs, d->pvrad, d->pvtheta, d->cfl, p.pebbles, p.fast_transport,
          (p.viscosity_alpha || p.viscosity != 0.0), d->partials, cfl_args(d), d->scal, d->iscal, d->s);
}

extern "C" int thorin_gpu_cfl(thorin_disk *d, double dt_remaining, double invdtreb_sq, int *n_sub)
{
  set_ctl(d, {{CTL_DELTAT, dt_remaining}, {CTL_INVDTREB, invdtreb_sq}});
  cfl_launches(d);
  d->cfl_first = 0;
  KCHECK("cfl kernels");
  CUCHK(cudaMemcpyAsync(d->iscal_h, d->iscal, sizeof(int) * IS_COUNT, cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  *n_sub = d->iscal_h[IS_NSUB];
  return THORIN_OK;
}

extern "C" int thorin_gpu_stokes(thorin_disk *d)
{
  if (!d) return THORIN_ERR_ARG;
  if (d->p.pebbles) aux_stokes(d->g, d->rho, d->psize, d->tau, d->s);
  KCHECK("Stokes kernel");
  return THORIN_OK;
}



static int ring_of(const thorin_disk *d, double r) { return pl_ring_of(d->Rsup.data(), d->nr, r); }
static double global_ifrac(const thorin_disk *d, double r) { return pl_global_ifrac(d->GlobalRmed.data(), d->nr, r); }
static void heating1(thorin_disk *d, double Mp, double dMp, double Xp, double Yp, double dt, int k)
{
  int idx;
  double add;
  if (pl_heating1(d->plc, d->Rsup.data(), d->Surf.data(), d->PhysicalTime, Mp, dMp, Xp, Yp, dt, &idx, &add)) {
    d->heatsrc_index[k] = idx;
    d->heatsrc[k] += add;
  }
}

// Heating1 (Planet.c:222-247): accretion luminosity into the planet's cell.

extern "C" int thorin_gpu_accrete(thorin_disk *d, thorin_planets *sys, double dt)
{
  const thorin_params &p = d->p;
  {
    double facc = p.evaporation_rate * dt;                         // EvaporatePebbles' fraction
    if (facc > 1.0) facc = 1.0;
    set_ctl(d, {{CTL_DT, dt}, {CTL_OMEGA_FRAME, d->OmegaFrame}, {CTL_FACC_EVAP, facc}});
  }
  for (int k = 0; k < sys->nb; k++) { d->heatsrc[k] = 0.0; d->heatsrc_index[k] = -1; }   // InitHeating
  // AccreteOntoPlanets (Planet.c:34-166)
  for (int k = 0; k < sys->nb; k++) {
    if (!(sys->acc[k] > 1e-10)) continue;
    const double facc = fabs(dt) * sys->acc[k];
    GasAccArgs a;
    a.facc1 = 1.0 / 3.0 * facc; a.facc2 = 2.0 / 3.0 * facc;
    if (a.facc1 > 1.0) a.facc1 = 1.0;
    if (a.facc2 > 1.0) a.facc2 = 1.0;
    a.Xp = sys->x[k]; a.Yp = sys->y[k]; a.Zp = sys->z[k];
    const double VX = sys->vx[k], VY = sys->vy[k];
    double M = sys->mass[k];
    const double Rperp = sqrt(a.Xp * a.Xp + a.Yp * a.Yp);
    const double Rplanet = sqrt(a.Xp * a.Xp + a.Yp * a.Yp + a.Zp * a.Zp);
    a.RRoche = pow((1.0 / 3.0 * M * d->MassTaper), (1.0 / 3.0)) * Rplanet;
    a.i_min = 0; a.i_max = d->nr - 1;
    while ((a.i_min < d->nr) && (d->Rsup[a.i_min] < Rperp - a.RRoche)) a.i_min++;
    while ((d->Rinf[a.i_max] > Rperp + a.RRoche) && (a.i_max > 0)) a.i_max--;
    const double angle = atan2(a.Yp, a.Xp);
    a.j_min = (int)((double)d->ns / 2.0 / H_PI * (angle - 2.0 * a.RRoche / Rperp));
    a.j_max = (int)((double)d->ns / 2.0 / H_PI * (angle + 2.0 * a.RRoche / Rperp));
    a.omega_frame = d->OmegaFrame;
    if (a.j_max - a.j_min + 1 > d->ns) {
      g_last_error = "gas accretion: the planet's Roche window is wider than a ring";
      return THORIN_ERR_ARG;
    }
    double dM = 0.0, dPx = 0.0, dPy = 0.0;
    if (a.i_min <= a.i_max) {
      aux_gas_accrete(d->g, d->rho, d->vrad, d->vtheta, d->cs, a, d->scal + SC_GASACC, d->s);
      KCHECK("gas accretion kernel");
      CUCHK(cudaMemcpyAsync(d->scal_h + SC_GASACC, d->scal + SC_GASACC, 3 * sizeof(double), cudaMemcpyDeviceToHost, d->s));
      CUCHK(cudaStreamSynchronize(d->s));
      dM = d->scal_h[SC_GASACC]; dPx = d->scal_h[SC_GASACC + 1]; dPy = d->scal_h[SC_GASACC + 2];
    }
    if (p.gas_accret_heating) heating1(d, M, dM, a.Xp, a.Yp, dt, k);
    const double PX = M * VX + dPx, PY = M * VY + dPy;
    M += dM;
    if (sys->feel_disk[k]) { sys->vx[k] = PX / M; sys->vy[k] = PY / M; }
    sys->mass[k] = M;
  }
  // ParametricAccretion (Pebbles.c:806-828)
  if (p.prescribed_accretion) {
    if (d->doubling == 0.0) d->doubling = p.parametric_accretion * 1000.0 * 2.0 * H_PI;
    if (p.accret_heating) d->heatsrc_max = sys->nb;
    for (int k = 0; k < sys->nb; k++) {
      const double M = sys->mass[k], dM = M * dt / d->doubling;
      if (p.accret_heating) heating1(d, M, dM, sys->x[k], sys->y[k], dt, k);
      sys->mass[k] = M + dM;
    }
  }
  if (!p.pebbles) return THORIN_OK;
  if (p.accret_heating) d->heatsrc_max = sys->nb;
  for (int k = 0; k < sys->nb; k++) {
    AccArgs a;
    a.pdens = d->pdens; a.macc = d->macc; a.pvr = d->pvrad; a.pvt = d->pvtheta; a.tau = d->tau; a.cs = d->cs;
    a.vt = d->vtheta;
    a.part = d->partials;
    a.acc = d->scal + 64;
    pl_pebble_acc_prep(d->plc, d->Rinf.data(), d->Rsup.data(), d->GlobalRmed.data(), sys, k, d->OmegaFrame, dt,
                       ACC_BX, &a);
    const int imin = a.imin, imax = a.imax;
    double dMp = 0, dPx = 0, dPy = 0;
    if (imin <= imax) {
      aux_accrete(d->g, a, d->acc_args_d, d->scal, d->s);
      KCHECK("accretion kernel");
      CUCHK(cudaMemcpyAsync(d->scal_h + SC_ACC_DM, d->scal + SC_ACC_DM, 3 * sizeof(double), cudaMemcpyDeviceToHost, d->s));
      CUCHK(cudaStreamSynchronize(d->s));
      dMp = d->scal_h[SC_ACC_DM]; dPx = d->scal_h[SC_ACC_DPX]; dPy = d->scal_h[SC_ACC_DPY];
    }
    if (p.accret_heating) heating1(d, a.Mp, dMp, a.Xp, a.Yp, dt, k);
    pl_pebble_acc_finish(sys, k, a, dMp, dPx, dPy);
  }
  if (p.evaporation_rate > 0.0)                                    // EvaporatePebbles
    aux_evaporate(d->g, d->temper, d->pdens, d->s);
  return THORIN_OK;
}

// FillForcesArrays' fixed arguments for npl planets (their constants are in
// d->planets_d, the mass taper and the planets' indirect term in the
// control block).
static ForceArgs force_args(const thorin_disk *d, int npl)
{
  const thorin_params &p = d->p;
  ForceArgs a;
  a.rho = d->rho; a.cs = d->cs; a.tau = d->tau; a.pdens = d->pdens;
  a.agr = d->agr; a.agt = d->agt; a.pagr = d->pagr; a.pagt = d->pagt;
  a.part = d->partials;
  a.pl = d->planets_d;
  a.npl = npl; a.pebbles = p.pebbles; a.exclude_hill = p.exclude_hill; a.pebble_gravity = p.pebble_gravity;
  a.pebble_alpha = p.pebble_alpha; a.hillcut = p.hillcut;
  a.sqrt_pebble_alpha = sqrt(p.pebble_alpha);
  return a;
}

extern "C" int thorin_gpu_forces(thorin_disk *d, thorin_planets *sys, double mass_taper, double indirect[2],
                                 double *ring_rho, double *ring_cs)
{
  const thorin_params &p = d->p;
  const int npl = sys->nb;
  if (npl > MAXPL_DEV) { g_last_error = "more planets than the force kernel handles"; return THORIN_ERR_ARG; }
  DevPlanet pl[MAXPL_DEV];
  double axs = 0.0, ays = 0.0;
  CUCHK(cudaStreamSynchronize(d->s));        // csmean_h is current
  for (int k = 0; k < npl; k++)
    pl_force_planet(d->plc, d->Rsup.data(), d->csmean_h, d->OmegaInv.data(), sys, k, mass_taper, &pl[k], &axs, &ays);
  if (npl > 0) CUCHK(cudaMemcpyAsync(d->planets_d, pl, npl * sizeof(DevPlanet), cudaMemcpyHostToDevice, d->s));
  const double indx_pl = p.indirect_term ? -axs : 0.0, indy_pl = p.indirect_term ? -ays : 0.0;
  set_ctl(d, {{CTL_MASS_TAPER, mass_taper}, {CTL_INDX_PL, indx_pl}, {CTL_INDY_PL, indy_pl}});
  aux_forces(d->g, force_args(d, npl), d->fr, d->scal, d->s);
  KCHECK("force kernels");
  // DampingTW04 needs the ring means of Sigma (and c_s) at each planet
  for (int k = 0; k < npl; k++) {
    const double r = sqrt(sys->x[k] * sys->x[k] + sys->y[k] * sys->y[k]);
    if (ring_rho) ring_rho[k] = 0.0;
    if (ring_cs) ring_cs[k] = 0.0;
    if (r >= d->Rinf[0] && r <= d->Rsup[d->nr - 1]) {
      const int i = ring_of(d, r);
      aux_ring_mean_at(d->g, d->rho, i, d->scal + SC_PLANET_A + 2 * MAXPL_DEV + k, d->s);
      if (ring_cs) ring_cs[k] = d->csmean_h[i];
    }
  }
  // UpdateLog (Force.c:27-70) needs Sigma's ring means either side of each planet
  int tq_ring[MAXPL_DEV];
  const int torques = d->torque_pending;
  if (torques) {
    for (int k = 0; k < npl; k++) {
      const double r = sqrt(sys->x[k] * sys->x[k] + sys->y[k] * sys->y[k]);
      tq_ring[k] = (int)global_ifrac(d, r);
      aux_ring_mean_at(d->g, d->rho, tq_ring[k], d->scal + SC_TORQUE + 2 * k, d->s);
      if (tq_ring[k] + 1 <= d->nr) aux_ring_mean_at(d->g, d->rho, tq_ring[k] + 1, d->scal + SC_TORQUE + 2 * k + 1, d->s);
    }
  }
  CUCHK(cudaMemcpyAsync(d->scal_h, d->scal, 128 * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  for (int k = 0; k < npl; k++) {
    sys->ax[k] = d->scal_h[SC_PLANET_A + 2 * k];
    sys->ay[k] = d->scal_h[SC_PLANET_A + 2 * k + 1];
    const double r = sqrt(sys->x[k] * sys->x[k] + sys->y[k] * sys->y[k]);
    if (ring_rho && r >= d->Rinf[0] && r <= d->Rsup[d->nr - 1]) ring_rho[k] = d->scal_h[SC_PLANET_A + 2 * MAXPL_DEV + k];
  }
  if (torques) {
    for (int k = 0; k < npl; k++) {
      const double x = sys->x[k], y = sys->y[k], ax = sys->ax[k], ay = sys->ay[k], m = sys->mass[k];
      const double r2 = x * x + y * y, r = sqrt(r2);
      const double ifrac = global_ifrac(d, r), frac = ifrac - floor(ifrac);
      const int ii = tq_ring[k];
      const double rho_hi = (ii + 1 <= d->nr) ? d->scal_h[SC_TORQUE + 2 * k + 1] : 0.0;
      const double cs_hi = (ii + 1 <= d->nr) ? d->csmean_h[ii + 1] : 0.0;
      const double rhopl = d->scal_h[SC_TORQUE + 2 * k] * (1.0 - frac) + rho_hi * frac;
      const double cspl = d->csmean_h[ii] * (1.0 - frac) + cs_hi * frac;
      const double omega = pow(r, -1.5);
      const double h = cspl / (omega * r) * (1.0 / sqrt(p.adiabind));
      double norm = m * omega * r2 / h;
      norm *= norm;
      norm *= rhopl;
      const double tq = x * ay - y * ax;
      thorin_torque &t = d->torques[k];
      t.time = d->PhysicalTime;
      t.torque = tq;
      t.torque_norm = tq * m * p.adiabind / norm;
      t.x = x; t.y = y; t.ax = ax; t.ay = ay;
    }
    d->ntorque = npl;
    d->torque_pending = 0;
  }
  // IndirectTerm of the disk (the planets' part is only added to the gas)
  indirect[0] = d->scal_h[SC_INDX];
  indirect[1] = d->scal_h[SC_INDY];
  return THORIN_OK;
}

extern "C" int thorin_gpu_request_torques(thorin_disk *d)
{
  if (!d) return THORIN_ERR_ARG;
  d->torque_pending = 1;
  return THORIN_OK;
}

extern "C" int thorin_gpu_get_torques(thorin_disk *d, thorin_torque *out, int max, int *n)
{
  if (!d || !n || (max > 0 && !out)) return THORIN_ERR_ARG;
  const int m = d->ntorque < max ? d->ntorque : max;
  for (int k = 0; k < m; k++) out[k] = d->torques[k];
  *n = d->ntorque;
  return THORIN_OK;
}

// `count` SOR sweeps on the disk's stream: a CUDA graph of the 2*count pass
// launches, captured the first time this count is asked for.
// The sweep loop as one graph: a WHILE conditional node (default value 1 at
// every launch) whose body is sor_loop_k red-black sweeps.  Each sweep's
// completion step sets the condition from the exit tests (converged, or the
// iteration cap): 0 with done, else 1.  Sweeps after the one that set done
// return at once and leave the condition at 0, so one launch runs the sweeps
// the solve needs plus fewer than sor_loop_k no-op sweeps, with no host round
// trip.  A body of several sweeps keeps the loop's per-run restart, which
// costs more than a kernel node of a linear graph, off most sweeps
// (THORIN_SOR_LOOP_SWEEPS, 1..64, sets sor_loop_k; default 8, measured
// level with 16 and ahead of 2 and 4 on the 1024x3072 disk).
static int sor_loop_graph(thorin_disk *d)
{
  if (d->sor_loop) return THORIN_OK;
  cudaGraph_t gr;
  CUCHK(cudaGraphCreate(&gr, 0));
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams np = {};
  cudaGraphNode_t node;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, gr, 1u, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    e = cudaGraphAddNode(&node, gr, nullptr, nullptr, 0, &np);
  }
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(d->s, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    SorCtl c = d->sor;
    c.cond = h;
    c.has_cond = 1;
    hydro_sor_sweeps(d->g, d->temper, d->ml, d->mlip, d->mlim, d->mljp, d->mljm, d->rhs, d->sor_cw, c,
                     d->p.sor_eps, d->sor_loop_k, d->p.sor_maxiters, d->s);
    cudaGraph_t body;
    e = cudaStreamEndCapture(d->s, &body);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&d->sor_loop, gr, 0);
  cudaGraphDestroy(gr);
  if (e != cudaSuccess) {
    d->sor_loop = nullptr;
    g_last_error = std::string("SOR loop graph: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  return THORIN_OK;
}

// SuccessiveOverrelaxation driver: the start residual (and the learned warm
// start), then the sweep loop graph; one read of the exit state per solve.
static int sor_solve(thorin_disk *d, double omega, int *niter, int *capped, bool learned = false)
{
  // normres0 and the threshold always come from the start temperature as
  // the reference has it; a learned start only moves T before the sweeps
  set_ctl(d, {{CTL_SOR_OMEGA, omega}});
  hydro_sor_resid0(d->g, d->temper, d->ml, d->mlip, d->mlim, d->mljp, d->mljm, d->rhs, d->sor_cw, d->sor, d->s);
  KCHECK("SOR residual kernel");
  if (learned && d->ws_net && d->ws_mode == THORIN_WS_PREDICT) {
    // keep the start (for the update record after the solve), then move it
    CUCHK(cudaMemcpyAsync(d->tbackup, d->temper, (size_t)d->nr * d->ns * sizeof(double), cudaMemcpyDeviceToDevice,
                          d->s));
    RCHK(wn_sor_predict(d->ws_net, d->nr, d->ns, d->ws_f, d->temper, d->ml, d->mlip, d->mlim, d->mljp, d->mljm,
                        d->rhs, d->ws_prev, d->ws_jac, d->sor.jscale, omega, nullptr, d->s));
    d->ws_st.predictions++;
  } else if (learned && d->ws_mode == THORIN_WS_EXTRAPOLATE) {
    CUCHK(cudaMemcpyAsync(d->tbackup, d->temper, (size_t)d->nr * d->ns * sizeof(double), cudaMemcpyDeviceToDevice,
                          d->s));
    RCHK(ws_extrapolate(d->nr, d->ns, d->temper, d->ws_prev, d->ws_order, d->ctl + CTL_DT, d->ws_dts, d->ml, d->mlip,
                          d->mlim, d->mljp, d->mljm, d->rhs, d->sor_cw, d->ctl + CTL_SOR_OMEGA, d->ws_jac,
                          d->ws_vq, d->ws_part, d->ws_step, d->g.nsm, d->s));
    d->ws_st.predictions++;
  }
  if (d->timing) CUCHK(cudaEventRecord(d->ev[0], d->s));
  if (d->sor_direct) {
    // THORIN_SOR_DIRECT: the same kernels (no graph condition) as plain
    // launches in chunks of sor_loop_k sweeps, the done flag read after each
    // chunk; kernel profilers list these, not kernels inside conditional
    // graph nodes.  The sweep count and the results are the same.
    for (int first = 1;; first += d->sor_loop_k) {
      hydro_sor_sweeps(d->g, d->temper, d->ml, d->mlip, d->mlim, d->mljp, d->mljm, d->rhs, d->sor_cw, d->sor,
                       d->p.sor_eps, d->sor_loop_k, d->p.sor_maxiters, d->s);
      KCHECK("SOR sweep kernels");
      CUCHK(cudaMemcpyAsync(d->iscal_h + IS_SOR_DONE, d->sor.done, sizeof(int), cudaMemcpyDeviceToHost, d->s));
      CUCHK(cudaStreamSynchronize(d->s));
      if (d->iscal_h[IS_SOR_DONE] || first + d->sor_loop_k > d->p.sor_maxiters) break;
    }
  } else {
    RCHK(sor_loop_graph(d));
    CUCHK(cudaGraphLaunch(d->sor_loop, d->s));
    KCHECK("SOR sweep kernels");
  }
  if (d->timing) CUCHK(cudaEventRecord(d->ev[1], d->s));
  CUCHK(cudaMemcpyAsync(d->iscal_h + IS_SOR_DONE, d->sor.done, 2 * sizeof(int), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  const int done = d->iscal_h[IS_SOR_DONE], n = d->iscal_h[IS_SOR_DONE + 1];
  if (!done || n < 1) {
    g_last_error = "SOR loop ended without an exit decision";
    return THORIN_ERR_CUDA;
  }
  *niter = n;
  *capped = (done == 2);
  g_thorin_launches += 2LL * n;
  if (d->timing) {
    float ms = 0.f;
    CUCHK(cudaEventElapsedTime(&ms, d->ev[0], d->ev[1]));
    d->st.sor_time_ms += ms;
    d->st.sor_passes += 2LL * n;
  }
  return THORIN_OK;
}

// IterateRelaxationParameter (EnergySources.c:340-403).
static int iterate_relaxation(thorin_disk *d)
{
  const thorin_params &p = d->p;
  const int nsplit = 9;
  int count = 0, Niter, capped;
  double omegamin = 1.0, omega = 1.0, omegamax = TH_OMEGAUPPER;
  const size_t bytes = (size_t)d->nr * d->ns * sizeof(double);
  CUCHK(cudaMemcpyAsync(d->tbackup, d->temper, bytes, cudaMemcpyDeviceToDevice, d->s));
  d->domega = (omegamax - omegamin) / nsplit;
  d->Niterbest = p.sor_maxiters;
  d->omegabest = 1.0;
  for (int outer = 0;; outer++) {
    if (outer >= 1000) { g_last_error = "omega calibration did not settle"; return THORIN_ERR_OMEGA; }
    for (int n = 0; n <= nsplit; n++) {
      RCHK(sor_solve(d, omega, &Niter, &capped));
      d->st.sor_sweeps += Niter;
      if (Niter == d->Niterbest) count++;
      if (Niter < d->Niterbest) { d->Niterbest = Niter; d->omegabest = omega; }
      omega += d->domega;
      CUCHK(cudaMemcpyAsync(d->temper, d->tbackup, bytes, cudaMemcpyDeviceToDevice, d->s));
    }
    if (d->Niterbest == p.sor_maxiters) { g_last_error = "SOR did not converge when estimating omega"; return THORIN_ERR_OMEGA; }
    if (count == nsplit + 1) { d->domega = omegamax - omegamin; return THORIN_OK; }
    count = 0;
    omegamin = d->omegabest - d->domega;
    omegamax = d->omegabest + d->domega;
    if (omegamin < 1.0) omegamin = 1.0;
    if (omegamax > TH_OMEGAUPPER) omegamax = TH_OMEGAUPPER;
    d->domega = (omegamax - omegamin) / nsplit;
    omega = omegamin;
  }
}

// SubStep3 + ImplicitRadiativeDiffusion (SourceEuler.c:508-586,
// EnergySources.c:201-335).  Leaves the new energy in d->energy.
static int capture_sor(thorin_disk *d);

static int energy_step(thorin_disk *d, double dt)
{
  const thorin_params &p = d->p;
  hydro_qplus(d->g, d->vrad, d->vtheta, d->rho, d->divv, d->qplus, d->invdphi, d->lr01, d->lr12, d->s);
  if (p.parametric_cooling) {
    aux_parametric_cooling(d->g, d->rho, d->energy_int, d->qplus, d->divv, d->ring[R_COOLT], d->ring[R_QPLUSMED],
                           d->energy_new, d->gm1, d->s);
    KCHECK("cooling kernel");
    std::swap(d->energy, d->energy_new);
    return THORIN_OK;
  }
  if (p.opacity_law == THORIN_OPA_SM03 && !d->g.k.sm_ross) {
    g_last_error = "OpacityTable SM03 needs the gas opacity table (thorin_gpu_set_opacity_table)";
    return THORIN_ERR_STATE;
  }
  hydro_eos(d->g, d->rho, d->energy_int, d->temper, d->cs, d->gm1, d->gg1, d->s);
  hydro_diffcoef(d->g, d->rho, d->temper, d->cs, d->opacity, d->qminus, d->dcen, d->partials, p.opacity_law,
                 p.parametric_opacity * OPA2CU, p.parametric_opacity, p.opacity_drop, d->taueff_c,
                 d->ring[R_INVDXTHETA], d->ring[R_DELTAR2], d->s);
  aux_min_final(d->partials, hydro_diffcoef_blocks(d->g), d->scal + SC_DTSTELLAR, d->s);
  if (p.stellar_irradiation)
    hydro_irradiation(d->g, d->rho, d->cs, d->opacity, d->flaring, d->qirr, d->rstar, d->tirr4fac, p.opacity_drop,
                      d->taueff_c, d->ring[R_RINF15], d->ring[R_RSUP15], d->s);
  int nheat = 0;
  if (d->capturing) {
    nheat = d->capS.accret_heating ? d->capS.npl : 0;      // written on the device by the accretion step
  } else if (p.accret_heating || p.gas_accret_heating) {
    nheat = d->heatsrc_max;
    if (nheat > 0) {
      CUCHK(cudaMemcpyAsync(d->heat_idx_d, d->heatsrc_index, nheat * sizeof(int), cudaMemcpyHostToDevice, d->s));
      CUCHK(cudaMemcpyAsync(d->heat_val_d, d->heatsrc, nheat * sizeof(double), cudaMemcpyHostToDevice, d->s));
    }
  }
  hydro_matrix(d->g, d->rho, d->temper, d->cs, d->dcen, d->divv, d->qminus, d->qplus, d->qirr, d->ml, d->mlip, d->mlim,
               d->mljp, d->mljm, d->rhs, d->gm1, d->ring[R_INVDXTHETA2], p.stellar_irradiation, nheat,
               d->heat_idx_d, d->heat_val_d, d->s);
  KCHECK("energy kernels");
  if (d->capturing) {                  // device-resident DT: schedule, solve loop and counters on the device
    RCHK(capture_sor(d));
    hydro_energy_from_t(d->g, d->rho, d->temper, d->energy_new, d->s);
    std::swap(d->energy, d->energy_new);
    return THORIN_OK;
  }
  if (d->sor_first) {
    d->sor_first = 0;
    RCHK(iterate_relaxation(d));
    d->omega = d->omegabest;
    d->Niterlast = d->Niterbest;
  }
  d->omega += d->domega;
  if (d->omega > TH_OMEGAUPPER) { d->omega = TH_OMEGAUPPER; d->domega = -d->domega; }
  if (d->omega < 1.0) { d->omega = 1.0; d->domega = -d->domega; }
  int Niter, capped;
  const bool train = d->ws_net && d->ws_mode == THORIN_WS_TRAIN;
  const size_t tbytes = (size_t)d->nr * d->ns * sizeof(double);
  if (train) CUCHK(cudaMemcpyAsync(d->tbackup, d->temper, tbytes, cudaMemcpyDeviceToDevice, d->s));
  RCHK(sor_solve(d, d->omega, &Niter, &capped, true));
  if (train) {
    // fit the network to this solve; energy_new is free until the energy is formed below
    RCHK(wn_sor_train(d->ws_net, d->nr, d->ns, d->ws_f, d->tbackup, d->temper, d->ml, d->mlip, d->mlim, d->mljp,
                      d->mljm, d->rhs, d->ws_prev, d->ws_jac, d->ws_lr, d->energy_new, d->s));
    d->ws_st.train_steps++;
  }
  if (d->ws_mode != THORIN_WS_OFF && d->ws_prev)   // this solve's update, an input of the next prediction
    RCHK(wn_record_update(d->nr, d->ns, d->temper, d->tbackup, d->ws_prev, d->ws_nh, d->ctl + CTL_DT, d->ws_dts, d->s));
  d->st.sor_calls++;
  d->st.sor_sweeps += Niter;
  d->st.sor_last_niter = Niter;
  d->st.sor_omega = d->omega;
  if (Niter > d->Niterlast) d->domega = -d->domega;
  d->Niterlast = Niter;
  hydro_energy_from_t(d->g, d->rho, d->temper, d->energy_new, d->s);
  std::swap(d->energy, d->energy_new);
  return capped ? THORIN_ERR_SOR_MAXIT : THORIN_OK;
}

static void transport_fluid(thorin_disk *d, double **rho, double *vr, double *vt, double **energy, double **rho_scratch,
                            double dt, int gas, const TransportScratch &scratch, cudaStream_t stream)
{
  TransportScratch S = scratch;
  S.rho_new = *rho_scratch;
  S.e_new = energy ? d->t_e_gas : nullptr;
  // the v_r damping of the boundary call after the transport is fused into
  // the velocity kernel when it is the only boundary condition
  const thorin_params &p = d->p;
  const int fused = p.damping && p.damp_vrad && !(p.open_inner || p.open_outer || p.non_reflecting || p.outer_source_mass);
  hydro_transport(d->g, rho, vr, vt, energy, (gas && p.label_advection) ? d->label : nullptr, S,
                  p.fast_transport, gas && fused, d->drin, d->drout, gas ? d->temper : nullptr, d->cs, d->gm1, d->gg1,
                  stream);
  std::swap(*rho, *rho_scratch);
  if (energy) std::swap(*energy, d->t_e_gas);
}

extern "C" int thorin_gpu_hydro(thorin_disk *d, double dt)
{
  const thorin_params &p = d->p;
  if (!d->capturing) set_ctl(d, {{CTL_DT, dt}, {CTL_OMEGA_FRAME, d->OmegaFrame}});
  const int damp = p.damping;
  auto boundary = [&]() {                // ApplyBoundaryCondition (SideEuler.c:490-503)
    if (p.open_inner) aux_open_inner(d->g, d->rho, d->vrad, d->energy, p.energy_eq, p.damp_flux, p.gasflux, d->s);
    if (p.open_outer) aux_open_outer(d->g, d->rho, d->vrad, d->energy, p.energy_eq, p.damp_flux, p.gasflux, d->s);
    if (p.non_reflecting) {
      if (p.energy_eq) {                   // ComputeSoundSpeed: c_s, its ring means and the viscosity
        hydro_eos(d->g, d->rho, d->energy, nullptr, d->cs, d->gm1, d->gg1, d->s);
        aux_ring_mean(d->g, d->cs, d->ring[R_CSMEAN], d->s);
        aux_viscosity_rings(d->g, d->vp, d->s);
      }
      aux_nonreflecting(d->g, d->rho, d->vrad, d->energy, d->cs, d->s);
    }
    if (p.outer_source_mass)
      aux_outer_source_mass(d->g, d->rho, d->vrad, p.imposed_disk_drift * pow((d->Rinf[d->nr - 1] / 1.0), -p.sigma_slope),
                            d->s);
    if (damp) aux_damp_gas(d->g, d->vrad, d->rho, d->vtheta, d->energy, d->damp_rings_d, d->ndamp, d->ring[R_DAMPVR0], p.damp_init, p.damp_flux, p.energy_eq, d->s);
  };
  // ApplyBoundaryCondition, DetectCrash, ComputePressureField (SourceEuler.c:271-292)
  boundary();
  CUCHK(cudaMemsetAsync(d->iscal + IS_CRASH, 0, sizeof(int), d->s));
  aux_crash(d->g, p.pebbles ? d->pdens : d->energy, d->iscal + IS_CRASH, d->s);
  if (!p.energy_eq) aux_iso_eos(d->g, d->rho, nullptr, d->cs, d->press, d->temper, 0, 1, 0, d->s);
  // SourceTermsPebbles (Pebbles.c:550-613)
  if (p.pebbles) {
    aux_damp_peb(d->g, d->pdens, d->pvrad, d->pvtheta, d->damp_rings_d, d->ndamp, d->s);
    aux_pebble_sources(d->g, d->pdens, d->pvrad, d->pvtheta, d->tau, d->vrad, d->vtheta, d->pagr, d->pagt, d->paccr,
                       d->pacct, d->dragr, d->dragt, p.back_reaction, d->s);
  }
  // SubStep1 with viscous terms (SourceEuler.c:319-415)
  hydro_substep1(d->g, d->rho, d->vrad, d->vtheta, d->energy, p.energy_eq ? nullptr : d->press, d->agr, d->agt, d->dragr, d->dragt, d->vrad_int,
                 d->vtheta_int, d->gaccr, d->gacct, d->gm1, p.pebbles, p.back_reaction,
                 d->ring[R_SUPPTORQUE], d->ring[R_INVDXTHETA], d->s);
  hydro_stress(d->g, d->vrad_int, d->vtheta_int, d->rho, d->divv, d->trr, d->tpp, d->trp, d->invdphi, d->s);
  const int kepler = (!p.damping) || (p.damping && p.damp_vrad);
  hydro_visc_update(d->g, d->vrad_int, d->vtheta_int, d->rho, d->trr, d->tpp, d->trp, d->invdphi, kepler,
                    d->vkep_in - d->Rmed[0] * d->OmegaFrame, d->vkep_out - d->Rmed[d->nr - 1] * d->OmegaFrame, d->s);
  if (p.pebbles) {
    aux_pebble_substep1(d->g, d->pvrad, d->pvtheta, d->tau, d->vrad, d->vtheta, d->paccr, d->pacct, d->gaccr, d->gacct,
                        d->rho, d->pdens, p.diffusive_particles, p.schmidt_number, d->ring[R_INVDXTHETA], d->s);
    // EvolvePebbleDisk (Pebbles.c:702-708).  From here on the pebble fields
    // are read and written only by the pebble transport and the gas side
    // touches none of them, so it runs on the pebble stream while the gas
    // goes through SubStep2, the energy step and its own transport; the
    // streams join before this call returns.
    CUCHK(cudaEventRecord(d->ev_fork, d->s));
    CUCHK(cudaStreamWaitEvent(d->s_peb, d->ev_fork, 0));
    aux_damp_peb(d->g, d->pdens, d->pvrad, d->pvtheta, d->damp_rings_d, d->ndamp, d->s_peb);
    transport_fluid(d, &d->pdens, d->pvrad, d->pvtheta, nullptr, &d->t_rho_peb, dt, 0, d->ts_peb, d->s_peb);
    aux_damp_peb(d->g, d->pdens, d->pvrad, d->pvtheta, d->damp_rings_d, d->ndamp, d->s_peb);
    CUCHK(cudaEventRecord(d->ev_join, d->s_peb));
  }
  // SubStep2, ActualiseGas, ApplyBoundaryCondition
  hydro_substep2(d->g, d->rho, d->vrad_int, d->vtheta_int, d->energy, d->vrad_new, d->vtheta_new, d->energy_int,
                 p.energy_eq, d->ring[R_INVDXTHETA], d->s);
  std::swap(d->vrad, d->vrad_new);
  std::swap(d->vtheta, d->vtheta_new);
  boundary();
  int status = THORIN_OK;
  if (p.energy_eq) {
    int s = energy_step(d, dt);
    if (s != THORIN_OK && s != THORIN_ERR_SOR_MAXIT) {
      if (p.pebbles) cudaStreamWaitEvent(d->s, d->ev_join, 0);
      return s;
    }
    status = s;
  }
  // Transport, ApplyBoundaryCondition, ComputeTemperatureField, ComputeSoundSpeed
  transport_fluid(d, &d->rho, d->vrad, d->vtheta, p.energy_eq ? &d->energy : nullptr, &d->t_rho_gas, dt, 1, d->ts, d->s);
  if (!d->capturing)
    CUCHK(cudaMemcpyAsync(d->nshift_h, d->nshift, d->nr * sizeof(int), cudaMemcpyDeviceToHost, d->s));
  if ((damp && !p.damp_vrad) || p.open_inner || p.open_outer || p.non_reflecting || p.outer_source_mass) {
    // damping towards INIT / GASFLUX changes Sigma (and e): the boundary
    // call, then ComputeTemperatureField and ComputeSoundSpeed
    boundary();
    if (p.energy_eq) hydro_eos(d->g, d->rho, d->energy, d->temper, d->cs, d->gm1, d->gg1, d->s);
  }
  if (!p.energy_eq) aux_iso_eos(d->g, d->rho, nullptr, d->cs, d->press, d->temper, 0, 0, 1, d->s);
  aux_ring_mean(d->g, d->cs, d->ring[R_CSMEAN], d->s);
  if (p.alpha_flock) aux_ring_mean(d->g, d->temper, d->ring[R_TEMPMEAN], d->s);
  aux_viscosity_rings(d->g, d->vp, d->s);
  if (!d->capturing)
    CUCHK(cudaMemcpyAsync(d->csmean_h, d->ring[R_CSMEAN], d->nr * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  if (p.pebbles) CUCHK(cudaStreamWaitEvent(d->s, d->ev_join, 0));     // join the pebble transport
  KCHECK("hydro kernels");
  if (d->capturing) return status;     // clock and crash flag stay on the device
  CUCHK(cudaMemcpyAsync(d->iscal_h + IS_CRASH, d->iscal + IS_CRASH, sizeof(int), cudaMemcpyDeviceToHost, d->s));
  d->PhysicalTime += dt;
  d->st.last_dt = dt;
  return status;
}

// AdvanceSystemFromDisk (Pframeforce.c:514-566) with DampingTW04 (:571-603).
static void advance_from_disk(thorin_disk *d, thorin_planets *sys, double dt, const double ind[2], const double *rrho,
                              const double *rcs)
{
  pl_advance_from_disk(d->plc, sys, dt, ind, rrho, rcs);
}

extern "C" int thorin_advance_from_disk(const thorin_disk *d, thorin_planets *sys, double dt, const double indirect[2],
                                        const double *ring_rho, const double *ring_cs)
{
  if (!d || !sys || !indirect || !ring_rho || !ring_cs || sys->nb > MAXPL_DEV) return THORIN_ERR_ARG;
  advance_from_disk(const_cast<thorin_disk *>(d), sys, dt, indirect, ring_rho, ring_cs);
  return THORIN_OK;
}

extern "C" int thorin_gpu_correct_vtheta(thorin_disk *d, double domega)
{
  if (!d) return THORIN_ERR_ARG;
  aux_correct_vtheta(d->g, d->vtheta, domega, d->s);
  if (d->p.pebbles) aux_correct_vtheta(d->g, d->pvtheta, domega, d->s);
  KCHECK("CorrectVtheta kernel");
  d->OmegaFrame += domega;
  return THORIN_OK;
}

// StokesDrag + AdvanceSystemFromDrag (Drag.c:17-119): the drag of the gas in
// the planet's own cell (its v_theta neighbour is l+1 without wrapping, as in
// the reference).
extern "C" int thorin_gpu_drag(thorin_disk *d, thorin_planets *sys, double dt)
{
  if (!d || !sys) return THORIN_ERR_ARG;
  const thorin_params &p = d->p;
  const int nr = d->nr, ns = d->ns;
  for (int k = 0; k < sys->nb; k++) {
    if (!sys->feel_disk[k]) continue;
    const double m = sys->mass[k], x = sys->x[k], y = sys->y[k], z = sys->z[k];
    const double vx = sys->vx[k], vy = sys->vy[k], vz = sys->vz[k];
    double ax = 0.0, ay = 0.0, az = 0.0;
    const double Rperp = sqrt(x * x + y * y);
    if (Rperp >= d->Rinf[0] && Rperp <= d->Rsup[nr - 1]) {
      int i = 0;
      while (d->Rsup[i] < Rperp) i++;
      double ang = atan2(y, x);
      if (ang < 0.0) ang += 2.0 * H_PI;
      int j = (int)floor((double)ns / 2.0 / H_PI * ang + 0.5);
      if (j == ns) j = 0;
      const int l = j + i * ns;
      aux_drag_cell(d->rho, d->cs, d->vrad, d->vtheta, l, ns, d->scal + SC_DRAGCELL, d->s);
      CUCHK(cudaMemcpyAsync(d->scal_h + SC_DRAGCELL, d->scal + SC_DRAGCELL, 6 * sizeof(double), cudaMemcpyDeviceToHost,
                            d->s));
      CUCHK(cudaStreamSynchronize(d->s));
      const double *c = d->scal_h + SC_DRAGCELL;
      const double xc = d->Rmed[i] * cos(2.0 * H_PI * (double)j / (double)ns);
      const double yc = d->Rmed[i] * sin(2.0 * H_PI * (double)j / (double)ns);
      const double vtcell = 0.5 * (c[4] + c[5]) + d->Rmed[i] * d->OmegaFrame;
      const double vrcell = 0.5 * (c[2] + c[3]);
      const double vxcell = (vrcell * xc - vtcell * yc) / d->Rmed[i];
      const double vycell = (vrcell * yc + vtcell * xc) / d->Rmed[i];
      const double H = c[1] * d->OmegaInv[i] * (1.0 / sqrt(p.adiabind));
      double factor = exp(-(z / (sqrt(2.0) * H)) * (z / (sqrt(2.0) * H)));
      factor *= 1.0 / (sqrt(2.0 * H_PI) * H);
      const double plrho = p.planetary_density / RHO2CGS;
      const double plradius = pow(3.0 * m / (4.0 * H_PI * plrho), 1.0 / 3.0);
      const double dvx = vx - vxcell, dvy = vy - vycell, dvz = vz - 0.0;
      const double dvsq = dvx * dvx + dvy * dvy + dvz * dvz;
      const double tmp = -0.5 * 0.48 * H_PI * plradius * plradius / m * factor * c[0] * dvsq * 1.0 / sqrt(dvsq);
      ax = tmp * dvx; ay = tmp * dvy; az = tmp * dvz;
    }
    sys->vx[k] += dt * ax;
    sys->vy[k] += dt * ay;
    sys->vz[k] += dt * az;
  }
  return THORIN_OK;
}

/* The point whose angle a corotating frame follows (GetPsysInfo and
 * GetPsysInfoFromRsim, Psys.c:195-330): planet 0 itself, or with Frame
 * GUIDINGCENTER and an orbit both eccentric and inclined (e, inc > 1e-8),
 * its guiding centre a (cos, sin)(M + periapsis angle) cos(inc).  a, e, inc
 * and the mean anomaly M are REBOUND's reb_tools_particle_to_orbit
 * (src_reb/tools.c:578-686) for a unit-mass primary at rest at the origin
 * and G = 1. */
static double frame_acos(double num, double den, double sign)   /* acos2, tools.c:563-576 */
{
  double c = num / den;
  if (c > -1.0 && c < 1.0) {
    double v = acos(c);
    return sign < 0.0 ? -v : v;
  }
  return (c <= -1.0) ? H_MPI : 0.0;
}

static void frame_point(int guiding_center, const thorin_planets *sys, double *xc, double *yc)
{
  double x = sys->x[0], y = sys->y[0], z = sys->z[0], vx = sys->vx[0], vy = sys->vy[0], vz = sys->vz[0];
  double m = sys->mass[0] + 1.0;
  *xc = x;
  *yc = y;
  if (!guiding_center) return;
  double d = sqrt(x * x + y * y + z * z);
  double v2 = vx * vx + vy * vy + vz * vz, vc2 = m / d;
  double a = -m / (v2 - 2.0 * vc2);
  double hx = y * vz - z * vy, hy = z * vx - x * vz, hz = x * vy - y * vx;
  double h = sqrt(hx * hx + hy * hy + hz * hz);
  double vr = (x * vx + y * vy + z * vz) / d, rvr = d * vr, muinv = 1.0 / m, vd2 = v2 - vc2;
  double ex = muinv * (vd2 * x - rvr * vx), ey = muinv * (vd2 * y - rvr * vy), ez = muinv * (vd2 * z - rvr * vz);
  double e = sqrt(ex * ex + ey * ey + ez * ez);
  double inc = frame_acos(hz, h, 1.0), M;
  if (e < 1.0) {
    double ea = frame_acos(1.0 - d / a, e, vr);
    M = ea - e * sin(ea);
  } else {
    double ea = acosh((1.0 - d / a) / e);
    if (vr < 0.0) ea = -ea;
    M = e * sinh(ea) - ea;
  }
  if (e > 1e-8 && inc > 1e-8) {
    double Ax = vy * hz - vz * hy - m * x / d, Ay = vz * hx - vx * hz - m * y / d;
    double pa = (Ax * Ax + Ay * Ay > 0.0) ? atan2(Ay, Ax) : atan2(y, x);
    *xc = a * cos(M + pa) * cos(inc);
    *yc = a * sin(M + pa) * cos(inc);
  }
}

extern "C" int thorin_gpu_algogas(thorin_disk *d, thorin_planets *sys)
{
  const thorin_params &p = d->p;
  const double DT = p.dt;
  double dtemp = 0.0, dt;
  int nsub = 0, status = THORIN_OK;
  if (!sys || sys->nb > MAXPL_DEV) { g_last_error = "planetary system missing or too large"; return THORIN_ERR_ARG; }
  if (p.corotating && sys->nb < 1) { g_last_error = "Frame COROTATING needs a planet"; return THORIN_ERR_ARG; }
  if (d->timing) CUCHK(cudaEventRecord(d->ev[2], d->s));
  d->torque_pending = 1;                       // DumpTorqueNow: log the first substep's torques
  if (p.sloppy_cfl) {
    // SloppyCFL (-c): one CFL per DT, with the rebound and pebble rates of
    // MinStepForRebound/CriticalCharTime, which are then never called (0),
    // SourceEuler.c:221-226
    int n;
    d->sloppy_pass = 1;
    const int rc = thorin_gpu_cfl(d, DT - dtemp, 0.0, &n);
    d->sloppy_pass = 0;
    RCHK(rc);
    dt = DT / (double)n;
  }
  while (dtemp < 0.999999999 * DT) {
    d->MassTaper = pl_mass_taper(d->PhysicalTime, p.mass_taper);
    if (!p.sloppy_cfl) {
      const double invdtreb_sq = pl_min_step_for_rebound(sys);
      int n;
      RCHK(thorin_gpu_cfl(d, DT - dtemp, invdtreb_sq, &n));
      dt = (DT - dtemp) / (double)n;
    } else if (p.pebbles) {
      aux_stokes(d->g, d->rho, d->psize, d->tau, d->s);       // PebbleStokesNumbers, every substep
    }
    RCHK(thorin_gpu_accrete(d, sys, dt));
    dtemp += dt;
    double ind[2], rrho[THORIN_MAXPLANETS], rcs[THORIN_MAXPLANETS];
    double xmark, ymark;                                     // GetPsysInfo (MARK)
    frame_point(p.guiding_center, sys, &xmark, &ymark);
    RCHK(thorin_gpu_forces(d, sys, d->MassTaper, ind, rrho, rcs));
    advance_from_disk(d, sys, dt, ind, rrho, rcs);
    if (p.aerodynamic_drag) RCHK(thorin_gpu_drag(d, sys, dt));
    pl_nbody_step(sys, dt);
    if (p.corotating) {
      // GetPsysInfo (GET): the angle planet 0 (or its guiding centre) moved
      // through; the frame follows it and the azimuthal velocities are
      // corrected (SourceEuler.c:261-267, CorrectVtheta SideEuler.c:505-519)
      double x, y;
      frame_point(p.guiding_center, sys, &x, &y);
      const double d2 = sqrt(x * x + y * y), d1 = sqrt(xmark * xmark + ymark * ymark);
      const double cross = xmark * y - x * ymark;
      const double OmegaNew = asin(cross / (d1 * d2)) / dt;
      const double domega = OmegaNew - d->OmegaFrame;
      aux_correct_vtheta(d->g, d->vtheta, domega, d->s);
      if (p.pebbles) aux_correct_vtheta(d->g, d->pvtheta, domega, d->s);
      d->OmegaFrame = OmegaNew;
    }
    pl_rotate(sys, d->OmegaFrame * dt);
    int s = thorin_gpu_hydro(d, dt);
    if (s != THORIN_OK && s != THORIN_ERR_SOR_MAXIT) return s;
    if (s != THORIN_OK) status = s;
    nsub++;
  }
  if (d->timing) CUCHK(cudaEventRecord(d->ev[3], d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  if (d->timing) {
    float ms = 0.f;
    CUCHK(cudaEventElapsedTime(&ms, d->ev[2], d->ev[3]));
    d->st.step_time_ms = ms;
  }
  d->st.substeps = nsub;
  d->st.crashed = d->iscal_h[IS_CRASH];
  d->st.kernel_launches = g_thorin_launches.load();
  return status;
}

// ---------------------------------------------------------------------------
// Device-resident DT: one CUDA graph per disk runs a whole DT of AlgoGas.
//
//   [k_g_dt_begin] -> WHILE(h_sub) {  one substep:
//       k_g_sub_begin, Stokes numbers, CFL (dt into the control block),
//       InitHeating, per planet: accretion set-up, v_theta ring means,
//       accretion kernels, Heating1 + planet update; evaporation,
//       force constants, FillForcesArrays, DampingTW04 ring means,
//       planet kick + N-body step + rotation (a branch beside the hydro),
//       the hydro substep of the host path (pebble transport on a parallel
//       branch) with the SOR solve as   k_g_sor_begin, residual,
//       WHILE(h_sor) { sweeps }, k_g_sor_end,
//       copies that put the state back into the buffers the next run of the
//       body reads, k_g_sub_end (clock, counters, loop condition)  }
//
// The launches are the host path's own, captured with the control block in
// place of host values.  Pointer swaps of the host path (ActualiseGas, the
// transport's output buffers) would change buffers between runs of the loop
// body, so the body ends by copying each state field back into the buffer it
// started in.  The first DT of a disk (omega calibration) runs on the host
// path; planets are kept on the device for the DT.

// Inserts the SOR sweep loop into the capture: the omega schedule, the start
// residual, a WHILE node whose body (captured later into d->capS) holds the
// sweeps, then the counters.
static int capture_sor(thorin_disk *d)
{
  StepDev &S = d->capS;
  graph_sor_begin(S, d->s);
  hydro_sor_resid0(d->g, d->temper, d->ml, d->mlip, d->mlim, d->mljp, d->mljm, d->rhs, d->sor_cw, d->sor, d->s);
  const bool predict = d->ws_net && d->ws_mode == THORIN_WS_PREDICT;
  const bool extrap = d->ws_mode == THORIN_WS_EXTRAPOLATE;
  if (predict || extrap) {  // the warm start moves T before the sweeps, as on the host path
    CUCHK(cudaMemcpyAsync(d->tbackup, d->temper, (size_t)d->nr * d->ns * sizeof(double), cudaMemcpyDeviceToDevice,
                          d->s));
    if (predict)
      RCHK(wn_sor_predict(d->ws_net, d->nr, d->ns, d->ws_f, d->temper, d->ml, d->mlip, d->mlim, d->mljp, d->mljm,
                          d->rhs, d->ws_prev, d->ws_jac, d->sor.jscale, 0.0, d->ctl + CTL_SOR_OMEGA, d->s));
    else
      RCHK(ws_extrapolate(d->nr, d->ns, d->temper, d->ws_prev, d->ws_order, d->ctl + CTL_DT, d->ws_dts, d->ml, d->mlip,
                          d->mlim, d->mljp, d->mljm, d->rhs, d->sor_cw, d->ctl + CTL_SOR_OMEGA, d->ws_jac,
                          d->ws_vq, d->ws_part, d->ws_step, d->g.nsm, d->s));
  }
  cudaStreamCaptureStatus cs;
  cudaGraph_t cg;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *edges = nullptr;
  size_t ndeps = 0;
  CUCHK(cudaStreamGetCaptureInfo(d->s, &cs, nullptr, &cg, &deps, &edges, &ndeps));
  if (cs != cudaStreamCaptureStatusActive) { g_last_error = "SOR loop outside a capture"; return THORIN_ERR_STATE; }
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = S.h_sor;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  CUCHK(cudaGraphAddNode(&node, cg, deps, edges, ndeps, &np));
  d->capture_sor_body = np.conditional.phGraph_out[0];
  CUCHK(cudaStreamUpdateCaptureDependencies(d->s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  graph_sor_end(S, d->s);
  if ((predict || extrap) && d->ws_prev)   // this solve's update, an input of the next prediction
    RCHK(wn_record_update(d->nr, d->ns, d->temper, d->tbackup, d->ws_prev, d->ws_nh, d->ctl + CTL_DT, d->ws_dts, d->s));
  return THORIN_OK;
}

// Inserts a WHILE node with handle h into the capture of stream s; returns
// its body graph.
static int capture_while(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraph_t *body)
{
  cudaStreamCaptureStatus cs;
  cudaGraph_t cg;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *edges = nullptr;
  size_t ndeps = 0;
  CUCHK(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, &edges, &ndeps));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  CUCHK(cudaGraphAddNode(&node, cg, deps, edges, ndeps, &np));
  *body = np.conditional.phGraph_out[0];
  CUCHK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return THORIN_OK;
}

// The launches of one substep (the loop body), on d->s.
static int capture_substep(thorin_disk *d)
{
  const thorin_params &p = d->p;
  StepDev &S = d->capS;
  const int npl = S.npl;
  graph_sub_begin(S, d->s);
  cfl_launches(d);
  if (p.pebbles) {
    graph_acc_init(S, d->s);
    const int nb_max = aux_accrete_blocks(d->g, 0, d->nr - 1);
    for (int k = 0; k < npl; k++) {
      graph_acc_prep(S, k, d->s);
      graph_ring_means_at(d->g, d->vtheta, d->scal + 64 + 4, d->ring_info_d, 0, 1, d->s);
      aux_accrete_kernels(d->g, S.acc, nb_max, d->scal, d->s);
      graph_acc_finish(S, k, d->s);
    }
    if (p.evaporation_rate > 0.0) aux_evaporate(d->g, d->temper, d->pdens, d->s);
  }
  graph_force_prep(S, d->s);
  aux_forces(d->g, force_args(d, npl), d->fr, d->scal, d->s);
  for (int k = 0; k < npl; k++)
    graph_ring_means_at(d->g, d->rho, d->scal + SC_PLANET_A + 2 * MAXPL_DEV + k, d->ring_info_d, 2 + k, 0, d->s);
  // the planet kick and N-body step run beside the hydro substep, which does
  // not read the planets; the next substep's CFL waits for them
  CUCHK(cudaEventRecord(d->ev_pl_fork, d->s));
  CUCHK(cudaStreamWaitEvent(d->s_pl, d->ev_pl_fork, 0));
  graph_planet_step(S, d->s_pl);
  CUCHK(cudaEventRecord(d->ev_pl_join, d->s_pl));
  // the hydro substep, with the buffers' roles restored at the end
  double *const f0[5] = {d->rho, d->vrad, d->vtheta, d->energy, d->pdens};
  double *const sc0[6] = {d->vrad_new, d->vtheta_new, d->energy_new, d->t_rho_gas, d->t_e_gas, d->t_rho_peb};
  const int rc = thorin_gpu_hydro(d, 0.0);
  double *f1[5] = {d->rho, d->vrad, d->vtheta, d->energy, d->pdens};
  const size_t bytes = d->fsize * sizeof(double);
  for (int q = 0; q < 5; q++)
    if (f1[q] && f1[q] != f0[q]) CUCHK(cudaMemcpyAsync(f0[q], f1[q], bytes, cudaMemcpyDeviceToDevice, d->s));
  d->rho = f0[0]; d->vrad = f0[1]; d->vtheta = f0[2]; d->energy = f0[3]; d->pdens = f0[4];
  d->vrad_new = sc0[0]; d->vtheta_new = sc0[1]; d->energy_new = sc0[2];
  d->t_rho_gas = sc0[3]; d->t_e_gas = sc0[4]; d->t_rho_peb = sc0[5];
  CUCHK(cudaStreamWaitEvent(d->s, d->ev_pl_join, 0));
  if (rc != THORIN_OK) return rc;
  graph_sub_end(S, d->s);
  KCHECK("device-resident substep");
  return THORIN_OK;
}

// The state fields and their scratch partners, whose buffers the host path
// swaps (ActualiseGas, the transport's output buffers).
static void graph_roles(thorin_disk *d, double **r[11])
{
  double **q[11] = {&d->rho, &d->vrad, &d->vtheta, &d->energy, &d->pdens, &d->vrad_new, &d->vtheta_new,
                    &d->energy_new, &d->t_rho_gas, &d->t_e_gas, &d->t_rho_peb};
  for (int k = 0; k < 11; k++) r[k] = q[k];
}

// Options the device-resident DT covers; the others stay on the host path.
static const char *graph_unsupported(const thorin_disk *d, const thorin_planets *sys)
{
  const thorin_params &p = d->p;
  if (p.sloppy_cfl) return "SloppyCFL";
  if (p.corotating) return "corotating frames";
  if (p.accretion_rate > 0.0) return "gas accretion onto planets";
  if (p.prescribed_accretion) return "ParametricAccretion";
  if (p.aerodynamic_drag) return "AerodynamicDrag";
  if (!p.energy_eq || p.parametric_cooling) return "runs without SOR radiative diffusion";
  if (d->ws_net && d->ws_mode == THORIN_WS_TRAIN) return "warm-start training";
  if (d->sor_direct) return "THORIN_SOR_DIRECT";
  if (sys->nb > MAXPL_DEV) return "more than 8 planets";
  return nullptr;
}

static int build_dt_graph(thorin_disk *d, int npl)
{
  const thorin_params &p = d->p;
  if (d->dt_graph) { cudaGraphExecDestroy(d->dt_graph); d->dt_graph = nullptr; }
  if (!d->sys_d) {
    RCHK(dalloc(d, (void **)&d->sys_d, sizeof(thorin_planets)));
    RCHK(dalloc(d, (void **)&d->gst_d, sizeof(GraphStats)));
    RCHK(dalloc(d, (void **)&d->ring_info_d, (2 + MAXPL_DEV) * sizeof(int)));
    RCHK(dalloc(d, (void **)&d->acc_args_g, sizeof(AccArgs)));
    CUCHK(cudaMallocHost((void **)&d->sys_h, sizeof(thorin_planets)));
    CUCHK(cudaMallocHost((void **)&d->gst_h, sizeof(GraphStats)));
    CUCHK(cudaMallocHost((void **)&d->ctl_h, CTL_COUNT * sizeof(double)));
    CUCHK(cudaStreamCreateWithFlags(&d->s_pl, cudaStreamNonBlocking));
    CUCHK(cudaEventCreateWithFlags(&d->ev_pl_fork, cudaEventDisableTiming));
    CUCHK(cudaEventCreateWithFlags(&d->ev_pl_join, cudaEventDisableTiming));
  }
  // the accretion arguments' device pointers (the scalars are set per
  // planet): the buffers the graph is captured with, in a block of the
  // graph's own (the host path rewrites acc_args_d with its current buffers)
  AccArgs a;
  memset(&a, 0, sizeof(a));
  a.pdens = d->pdens; a.macc = d->macc; a.pvr = d->pvrad; a.pvt = d->pvtheta; a.tau = d->tau; a.cs = d->cs;
  a.vt = d->vtheta;
  a.part = d->partials;
  a.acc = d->scal + 64;
  CUCHK(cudaMemcpyAsync(d->acc_args_g, &a, sizeof(a), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  StepDev &S = d->capS;
  S.g = d->g; S.c = d->plc; S.sys = d->sys_d; S.scal = d->scal; S.iscal = d->iscal; S.acc = d->acc_args_g;
  S.ring_info = d->ring_info_d; S.pl = d->planets_d; S.heat_idx = d->heat_idx_d; S.heat_val = d->heat_val_d;
  S.st = d->gst_d; S.sor = d->sor; S.DT = p.dt; S.evaporation_rate = p.evaporation_rate; S.npl = npl;
  S.pebbles = p.pebbles; S.accret_heating = p.pebbles && p.accret_heating; S.indirect_term = p.indirect_term;
  cudaGraph_t G = nullptr, body = nullptr;
  cudaGraphExec_t exec = nullptr;
  int rc = THORIN_OK;
  cudaError_t e = cudaGraphCreate(&G, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&S.h_sub, G, 1u, cudaGraphCondAssignDefault);
  // top level: counters, then the substep loop
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(d->s, G, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    graph_dt_begin(S, d->s);
    rc = capture_while(d->s, S.h_sub, &body);
    cudaGraph_t tmp;
    const cudaError_t e2 = cudaStreamEndCapture(d->s, &tmp);
    if (rc == THORIN_OK && e2 != cudaSuccess) e = e2;
  }
  // the substep body, with the SOR loop's node inside it
  if (e == cudaSuccess && rc == THORIN_OK) e = cudaGraphConditionalHandleCreate(&S.h_sor, body, 1u, cudaGraphCondAssignDefault);
  if (e == cudaSuccess && rc == THORIN_OK) e = cudaStreamBeginCaptureToGraph(d->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess && rc == THORIN_OK) {
    d->capturing = 1;
    d->capture_sor_body = nullptr;
    rc = capture_substep(d);
    d->capturing = 0;
    cudaGraph_t tmp;
    const cudaError_t e2 = cudaStreamEndCapture(d->s, &tmp);
    if (rc == THORIN_OK && e2 != cudaSuccess) e = e2;
    if (rc == THORIN_OK && e == cudaSuccess && !d->capture_sor_body) { g_last_error = "no SOR loop in the substep"; rc = THORIN_ERR_STATE; }
  }
  // the sweeps inside the SOR loop
  if (e == cudaSuccess && rc == THORIN_OK) e = cudaStreamBeginCaptureToGraph(d->s, d->capture_sor_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess && rc == THORIN_OK) {
    SorCtl c = d->sor;
    c.cond = S.h_sor;
    c.has_cond = 1;
    hydro_sor_sweeps(d->g, d->temper, d->ml, d->mlip, d->mlim, d->mljp, d->mljm, d->rhs, d->sor_cw, c, p.sor_eps,
                     d->sor_loop_k, p.sor_maxiters, d->s);
    cudaGraph_t tmp;
    e = cudaStreamEndCapture(d->s, &tmp);
  }
  if (e == cudaSuccess && rc == THORIN_OK) e = cudaGraphInstantiate(&exec, G, 0);
  if (G) cudaGraphDestroy(G);
  cudaGetLastError();
  if (rc != THORIN_OK) return rc;
  if (e != cudaSuccess) {
    g_last_error = std::string("device-resident DT graph: ") + cudaGetErrorString(e);
    return THORIN_ERR_CUDA;
  }
  d->dt_graph = exec;
  d->graph_npl = npl;
  double **roles[11];
  graph_roles(d, roles);
  for (int k = 0; k < 11; k++) d->cap_ptr[k] = *roles[k];
  return THORIN_OK;
}

// Uploads what the graph reads (planets, clock, frame, omega schedule) and
// launches one DT on the disk's stream; thorin_gpu_graph_finish reads back.
static int graph_launch(thorin_disk *d, const thorin_planets *sys)
{
  if (!d->dt_graph || d->graph_npl != sys->nb) RCHK(build_dt_graph(d, sys->nb));
  // the host path swaps buffers between the state fields and their scratch
  // partners; the graph reads the buffers it was captured with, so the state
  // goes back into those first (each field's buffers are its own, so no copy
  // overwrites another field)
  double **roles[11];
  graph_roles(d, roles);
  const size_t bytes = d->fsize * sizeof(double);
  for (int k = 0; k < 5; k++)
    if (*roles[k] && *roles[k] != d->cap_ptr[k])
      CUCHK(cudaMemcpyAsync(d->cap_ptr[k], *roles[k], bytes, cudaMemcpyDeviceToDevice, d->s));
  for (int k = 0; k < 11; k++) *roles[k] = d->cap_ptr[k];
  *d->sys_h = *sys;
  CUCHK(cudaMemcpyAsync(d->sys_d, d->sys_h, sizeof(thorin_planets), cudaMemcpyHostToDevice, d->s));
  set_ctl(d, {{CTL_TIME, d->PhysicalTime}, {CTL_OMEGA_FRAME, d->OmegaFrame}, {CTL_SOR_OMEGA, d->omega},
              {CTL_SOR_DOMEGA, d->domega}});
  d->gst_h->niterlast = d->Niterlast;
  CUCHK(cudaMemcpyAsync(&d->gst_d->niterlast, &d->gst_h->niterlast, sizeof(int), cudaMemcpyHostToDevice, d->s));
  if (d->timing) CUCHK(cudaEventRecord(d->ev[2], d->s));
  CUCHK(cudaGraphLaunch(d->dt_graph, d->s));
  if (d->timing) CUCHK(cudaEventRecord(d->ev[3], d->s));
  CUCHK(cudaMemcpyAsync(d->sys_h, d->sys_d, sizeof(thorin_planets), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaMemcpyAsync(d->gst_h, d->gst_d, sizeof(GraphStats), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaMemcpyAsync(d->ctl_h, d->ctl, CTL_COUNT * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaMemcpyAsync(d->nshift_h, d->nshift, d->nr * sizeof(int), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaMemcpyAsync(d->csmean_h, d->ring[R_CSMEAN], d->nr * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  return THORIN_OK;
}

static int graph_finish(thorin_disk *d, thorin_planets *sys)
{
  CUCHK(cudaStreamSynchronize(d->s));
  d->cfl_first = 0;
  const GraphStats &g = *d->gst_h;
  *sys = *d->sys_h;
  d->PhysicalTime = d->ctl_h[CTL_TIME];
  d->omega = d->ctl_h[CTL_SOR_OMEGA];
  d->domega = d->ctl_h[CTL_SOR_DOMEGA];
  d->Niterlast = g.niterlast;
  d->MassTaper = d->ctl_h[CTL_MASS_TAPER];
  d->st.substeps = g.nsub;
  d->st.crashed = g.crashed;
  d->st.sor_calls += g.sor_calls;
  if ((d->ws_net && d->ws_mode == THORIN_WS_PREDICT) || d->ws_mode == THORIN_WS_EXTRAPOLATE)
    d->ws_st.predictions += g.sor_calls;
  d->st.sor_sweeps += g.sor_sweeps;
  if (g.sor_calls) { d->st.sor_last_niter = g.sor_last_niter; d->st.sor_omega = g.omega_used; }
  d->st.last_dt = d->ctl_h[CTL_DT];
  d->st.kernel_launches = g_thorin_launches.load();
  if (d->timing) {
    float ms = 0.f;
    CUCHK(cudaEventElapsedTime(&ms, d->ev[2], d->ev[3]));
    d->st.step_time_ms = ms;
  }
  if (g.error == 1) { g_last_error = "SOR loop ended without an exit decision"; return THORIN_ERR_CUDA; }
  if (g.error == 2) { g_last_error = "substep bound of the device-resident DT reached"; return THORIN_ERR_STATE; }
  if (g.error == 3) { g_last_error = "non-positive substep length"; return THORIN_ERR_STATE; }
  return g.capped ? THORIN_ERR_SOR_MAXIT : THORIN_OK;
}

extern "C" int thorin_gpu_set_launch_shape(thorin_disk *d, int sor_loop_sweeps, int sor_threads_per_sm)
{
  if (!d || sor_loop_sweeps < 1 || sor_loop_sweeps > 64 || sor_threads_per_sm < 128 || sor_threads_per_sm > 2048 ||
      sor_threads_per_sm % 128) {
    g_last_error = "launch shape: 1..64 sweeps per loop body, 128..2048 SOR threads per SM in steps of 128";
    return THORIN_ERR_ARG;
  }
  CUCHK(cudaStreamSynchronize(d->s));
  d->sor_loop_k = sor_loop_sweeps;
  d->g.sor_tpsm = sor_threads_per_sm;
  if (d->sor_loop) { cudaGraphExecDestroy(d->sor_loop); d->sor_loop = nullptr; }
  if (d->dt_graph) { cudaGraphExecDestroy(d->dt_graph); d->dt_graph = nullptr; }
  return THORIN_OK;
}

extern "C" int thorin_gpu_get_launch_shape(thorin_disk *d, int *sor_loop_sweeps, int *sor_threads_per_sm)
{
  if (!d || !sor_loop_sweeps || !sor_threads_per_sm) return THORIN_ERR_ARG;
  *sor_loop_sweeps = d->sor_loop_k;
  *sor_threads_per_sm = d->g.sor_tpsm;
  return THORIN_OK;
}

static bool graph_host_dt(const thorin_disk *d)
{
  return d->sor_first || (d->cfl_first && d->p.first_step > 0.0);
}

extern "C" int thorin_gpu_graph_supported(thorin_disk *d, const thorin_planets *sys)
{
  if (!d || !sys) return THORIN_ERR_ARG;
  const char *why = graph_unsupported(d, sys);
  if (why) { g_last_error = std::string("device-resident DT: not with ") + why; return THORIN_ERR_ARG; }
  return THORIN_OK;
}

extern "C" int thorin_gpu_algogas_graph(thorin_disk *d, thorin_planets *sys)
{
  RCHK(thorin_gpu_graph_supported(d, sys));
  // the omega calibration of a disk's first solve runs on the host path (so
  // does a first DT with FirstStep set, which only the first CFL reads)
  if (graph_host_dt(d)) return thorin_gpu_algogas(d, sys);
  RCHK(graph_launch(d, sys));
  return graph_finish(d, sys);
}

// One DT of n disks: every disk's graph is launched on its own stream before
// the first is waited for, so the disks run side by side on the GPU.
extern "C" int thorin_ensemble_algogas_graph(thorin_disk **disks, thorin_planets **systems, int n, int *status)
{
  if (!disks || !systems || n < 1) return THORIN_ERR_ARG;
  for (int k = 0; k < n; k++)
    if (!disks[k] || !systems[k]) return THORIN_ERR_ARG;
  int worst = THORIN_OK;
  std::vector<int> launched(n, 0);
  for (int k = 0; k < n; k++) {
    thorin_disk *d = disks[k];
    int rc = thorin_gpu_graph_supported(d, systems[k]);
    if (rc == THORIN_OK && graph_host_dt(d)) rc = thorin_gpu_algogas(d, systems[k]);
    else if (rc == THORIN_OK) { rc = graph_launch(d, systems[k]); launched[k] = (rc == THORIN_OK); }
    if (status) status[k] = rc;
    if (rc != THORIN_OK && rc != THORIN_ERR_SOR_MAXIT) worst = rc;
  }
  for (int k = 0; k < n; k++) {
    if (!launched[k]) continue;
    const int rc = graph_finish(disks[k], systems[k]);
    if (status) status[k] = rc;
    if (rc != THORIN_OK && rc != THORIN_ERR_SOR_MAXIT) worst = rc;
  }
  return worst;
}

extern "C" int thorin_gpu_get_sor_state(thorin_disk *d, double *omega, double *domega, int *niterlast, int *calibrated)
{
  if (!d) return THORIN_ERR_ARG;
  if (omega) *omega = d->omega;
  if (domega) *domega = d->domega;
  if (niterlast) *niterlast = d->Niterlast;
  if (calibrated) *calibrated = !d->sor_first;
  return THORIN_OK;
}

extern "C" int thorin_gpu_set_sor_state(thorin_disk *d, double omega, double domega, int niterlast)
{
  if (!d || !(omega >= 1.0 && omega <= TH_OMEGAUPPER)) return THORIN_ERR_ARG;
  d->omega = omega;
  d->domega = domega;
  d->Niterlast = niterlast;
  d->sor_first = 0;
  return THORIN_OK;
}

// The one scalar a DT hands to the next besides the fields and the omega
// schedule: DiffusionTimestep's dt_stellar of the last energy step, which
// bounds the next CFL (SourceEuler.c:680-690).
extern "C" int thorin_gpu_get_dt_stellar(thorin_disk *d, double *dt_stellar)
{
  if (!d || !dt_stellar) return THORIN_ERR_ARG;
  CUCHK(cudaMemcpyAsync(d->scal_h + SC_DTSTELLAR, d->scal + SC_DTSTELLAR, sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  *dt_stellar = d->scal_h[SC_DTSTELLAR];
  return THORIN_OK;
}

extern "C" int thorin_gpu_set_dt_stellar(thorin_disk *d, double dt_stellar)
{
  if (!d) return THORIN_ERR_ARG;
  d->scal_h[SC_DTSTELLAR] = dt_stellar;
  CUCHK(cudaMemcpyAsync(d->scal + SC_DTSTELLAR, d->scal_h + SC_DTSTELLAR, sizeof(double), cudaMemcpyHostToDevice, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  return THORIN_OK;
}

extern "C" int thorin_gpu_set_timing(thorin_disk *d, int on)
{
  if (!d) return THORIN_ERR_ARG;
  d->timing = on ? 1 : 0;
  d->st.sor_time_ms = 0.0;
  d->st.sor_passes = 0;
  return THORIN_OK;
}

// cells of a disk's grid (the ensemble scheduler orders disks by it)
long long thorin_disk_cells(const thorin_disk *d) { return (long long)d->nr * d->ns; }

extern "C" int thorin_gpu_get_stream(thorin_disk *d, void **stream)
{
  if (!d || !stream) return THORIN_ERR_ARG;
  *stream = (void *)d->s;
  return THORIN_OK;
}

extern "C" int thorin_gpu_integrals(thorin_disk *d, double *mass, double *momentum, double *energy, double *peb_mass,
                                    double *peb_momentum)
{
  aux_integrals(d->g, d->rho, d->vrad, d->vtheta, d->energy, d->pdens, d->pvtheta, d->OmegaFrame, d->p.pebbles,
                d->partials, d->scal, d->s);
  KCHECK("integral kernels");
  CUCHK(cudaMemcpyAsync(d->scal_h + SC_MASS, d->scal + SC_MASS, 5 * sizeof(double), cudaMemcpyDeviceToHost, d->s));
  CUCHK(cudaStreamSynchronize(d->s));
  if (mass) *mass = d->scal_h[SC_MASS];
  if (momentum) *momentum = d->scal_h[SC_MOM];
  if (energy) *energy = d->scal_h[SC_ENER];
  if (peb_mass) *peb_mass = d->scal_h[SC_PMASS];
  if (peb_momentum) *peb_momentum = d->scal_h[SC_PMOM];
  return THORIN_OK;
}

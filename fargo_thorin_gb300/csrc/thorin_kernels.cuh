// thorin_kernels.cuh -- argument structs and host launchers of the kernels.
#pragma once
#include <atomic>
#include "thorin_dev.cuh"

#define MAXPL_DEV 8            // planets handled by the force kernel (per-thread arrays)
#define ACC_BX 256             // threads per block of the pebble accretion kernels

// Planet data seen by the kernels (per-planet constants from the host).
struct DevPlanet {
  double x, y, z, m, rhill, Hpl, smoothing2, rst2, rst3, rst4, rsm2, rmorevert2;
  double near_h2, near_hill2;   // (10 Hpl)^2 and (5 rhill)^2: the vertical-quadrature zone
};

// Indices into the small device scalar buffer.
enum {
  SC_NEWDT = 0, SC_INVDTPEB, SC_DTSTELLAR, SC_INDX, SC_INDY, SC_ACC_DM, SC_ACC_DPX, SC_ACC_DPY, SC_RINGRHO,
  SC_MASS, SC_MOM, SC_ENER, SC_PMASS, SC_PMOM, SC_NORMRES0, SC_NORMRES,
  SC_PLANET_A = 32,           // 2 per planet: ax, ay (then the ring means of Sigma for DampingTW04)
  SC_TORQUE = 56,             // 2 per planet: ring means of Sigma either side of the planet (UpdateLog)
  SC_GASACC = 80,             // dM, dPx, dPy of the gas accretion onto one planet
  SC_DRAGCELL = 84,           // 6 values of the planet's cell for the aerodynamic drag
  SC_RCS = 96                 // device-resident DT: ring mean of c_s at each planet, taken before the hydro
};
enum { IS_NSUB = 0, IS_SOR_DONE, IS_SOR_NITER, IS_SOR_CHANGED, IS_CRASH, IS_COUNT };

// Red-black SOR control block (device pointers).
#define SOR_GROUP 64      // blocks per completion group of a SOR pass
#define SOR_TSTRIDE 32    // group tickets 128 bytes apart

struct SorCtl {
  double *part;           // [2][nblocks] partial |resid| sums
  int *ipart;             // [2][nblocks] partial changed counts
  double *gpart;          // [ngroups] group sums of both colours
  int *gipart;            // [ngroups]
  unsigned int *gticket;  // [ngroups * SOR_TSTRIDE] group tickets
  unsigned int *ticket;
  int *done;              // 1 converged, 2 iteration cap; later sweeps are no-ops
  int *niter;
  double *normres0;
  double *normres;
  int *changed;
  double *jscale;         // sum over the start of |resid| * omega/Ml (k_sor_resid0)
  // Condition of the graph's WHILE node around the sweeps: the completion
  // step sets it to 0 together with done (has_cond 0: no such node)
  cudaGraphConditionalHandle cond;
  int has_cond;
};

// Transport scratch (device fields).
struct TransportScratch {
  double *mom[4];          // RadMomP, RadMomM, ThetaMomP, ThetaMomM (updated in place)
  double *rho_new, *e_new;
  double *ext, *ext_new;   // rho * label before and after the transport (LabelAdvection)
  double *w[7], *d[8], *f[8];
  int *nshift;
  double *vmed, *vtemp;
};

struct PtrPack8 { const double *src[8]; double *dst[8]; int n; };
struct AziIO { const double *src[7]; double *dst[7]; int n; };   // index n-1 is the density

struct ViscParams {
  double viscosity, alpha, alpha_mri, alpha_dead, tmri, twidth, t2si;
  double cav_rmin, cav_rmax, cav_ratio, log_cav_ratio;
  int viscosity_alpha, alpha_flock;
};

struct CflRings {
  const double *dxrad, *dxtheta, *mindx, *den5;    // per ring, ConditionCFL's expressions
  double *vmoy, *pvtmed;                           // ring means (scratch)
};

struct CflFinal {
  int nb, pebbles, first_call;
  double deltaT, invdtreb_sq, minimum_step, maximum_step, first_step, twopi_cfl_ns;
};

struct ForceRings {
  double *H_avr, *sigma_avr, *integstar_avr, *p_H_avr, *p_integstar_avr, *tau_avr;
  double *isigma_avr;          // 1 / sigma_avr
  const double *drsq;          // (Rsup - Rinf)^2
};

struct ForceArgs {
  const double *rho, *cs, *tau, *pdens;
  double *agr, *agt, *pagr, *pagt;
  double *part;               // [nblocks][2 + 2*npl]
  const DevPlanet *pl;
  int npl, pebbles, exclude_hill, pebble_gravity;
  double pebble_alpha, hillcut;   // the mass taper is read from the control block
  double sqrt_pebble_alpha;   // sqrt(pebble_alpha)
  // vertical quadrature weights exp(-z_m^2 / 2H^2) at z_m = (m - 1/2) 3H/N,
  // which do not depend on H, and their sums (filled by aux_forces)
  double wq10[10], wq30[30], sig10, sig30;
  double isig10, isig30;      // 1 / sig10, 1 / sig30
};

struct GasAccArgs {           // one planet of AccreteOntoPlanets (Planet.c:34-166)
  double Xp, Yp, Zp, RRoche, facc1, facc2, omega_frame;
  int i_min, i_max, j_min, j_max;
};

struct AccArgs {
  double *pdens, *macc;
  double *part;               // block partials (4 per block)
  double *acc;                // scalars: Reff, vrel, Mt, limiter
  const double *pvr, *pvt, *tau, *cs, *vt;
  double Xp, Yp, Zp, VXp, VYp, VZp, Mp, Rp, Rhill, Omegap, Rp15, omega_frame, dt, pebble_alpha, frac;
  int imin, imax, iflow;
  int nb;                     // blocks over the annulus imin..imax (aux_accrete_blocks)
};

// Number of kernels launched by this library (host-side bookkeeping; every
// launcher below adds the launches it issues).  Atomic: disks of an ensemble
// are advanced from several host threads.
extern std::atomic<long long> g_thorin_launches;

// kernels_hydro.cu
void hydro_substep1(const DevGrid &g, const double *rho, const double *vrad, const double *vtheta,
                    const double *energy, const double *press, const double *agr, const double *agt, const double *dragr, const double *dragt,
                    double *vradint, double *vthetaint, double *gaccr, double *gacct,
                    double gm1, int pebbles, int back_reaction, const double *supp_torque, const double *invdxtheta_r,
                    cudaStream_t s);
void hydro_stress(const DevGrid &g, const double *vr, const double *vt, const double *rho, double *divv, double *trr,
                  double *tpp, double *trp, double invdphi, cudaStream_t s);
void hydro_visc_update(const DevGrid &g, double *vr, double *vt, const double *rho, const double *trr, const double *tpp,
                       const double *trp, double invdphi, int kepler, double vkin, double vkout,
                       cudaStream_t s);
void hydro_substep2(const DevGrid &g, const double *rho, const double *vr, const double *vt, const double *energy,
                    double *vrnew, double *vtnew, double *eint, int energy_eq, const double *invdxtheta_r,
                    cudaStream_t s);
void hydro_qplus(const DevGrid &g, const double *vr, const double *vt, const double *rho, double *divv, double *qplus,
                 double invdphi, double lr01, double lr12, cudaStream_t s);
void hydro_eos(const DevGrid &g, const double *rho, const double *energy, double *temper, double *cs, double gm1,
               double gg1, cudaStream_t s);
int hydro_diffcoef_blocks(const DevGrid &g);
void hydro_diffcoef(const DevGrid &g, const double *rho, const double *T, const double *cs, double *opacity,
                    double *qminus, double *dcen, double *dtmin_part, int law, double parametric_cu,
                    double parametric_raw, double opacity_drop, double taueff_c, const double *invdxtheta_r,
                    const double *deltar2_r, cudaStream_t s);
void hydro_irradiation(const DevGrid &g, const double *rho, const double *cs, const double *opacity, double *flaring,
                       double *qirr, double rstar, double tirr4fac, double opacity_drop, double taueff_c,
                       const double *rinf15, const double *rsup15, cudaStream_t s);
void hydro_matrix(const DevGrid &g, const double *rho, const double *T, const double *cs, const double *dcen,
                  const double *divv, const double *qminus, const double *qplus, const double *qirr, double *ml,
                  double *mlip, double *mlim, double *mljp, double *mljm, double *rhs,
                  double gm1, const double *invdxtheta2_r, int irradiation, int nheat, const int *heat_idx,
                  const double *heat_val, cudaStream_t s);
int sor_blocks(const DevGrid &g);
void hydro_sor_resid0(const DevGrid &g, const double *T, const double *ml, const double *mlip, const double *mlim,
                      const double *mljp, const double *mljm, const double *rhs, double *cw,
                      const SorCtl &c, cudaStream_t s);
// `count` sweeps (two colour passes each).  The sweep number lives on the
// device, so every call with the same count issues identical launches (the
// caller may capture and replay them as a CUDA graph); the launch counter is
// left to the caller.
void hydro_sor_sweeps(const DevGrid &g, double *T, const double *ml, const double *mlip, const double *mlim,
                      const double *mljp, const double *mljm, const double *rhs, const double *cw, const SorCtl &c,
                      double eps, int count, int maxiters, cudaStream_t s);
void hydro_energy_from_t(const DevGrid &g, const double *rho, double *T, double *enew, cudaStream_t s);
void hydro_transport(const DevGrid &g, double **rho, double *vr, double *vt, double **energy, double *label,
                     const TransportScratch &S, int fast, int damp_vrad, double drin,
                     double drout, double *temper, double *cs, double gm1, double gg1, cudaStream_t s);

// kernels_aux.cu
void aux_ring_means(const DevGrid &g, const double *f0, double *o0, const double *f1, double *o1, int ring0, int nrings,
                    cudaStream_t s);
void aux_ring_mean(const DevGrid &g, const double *f, double *out, cudaStream_t s);
void aux_ring_mean_at(const DevGrid &g, const double *f, int ring, double *out, cudaStream_t s);
void aux_viscosity_rings(const DevGrid &g, const ViscParams &v, cudaStream_t s);
void aux_stokes(const DevGrid &g, const double *rho, const double *psize, double *tau, cudaStream_t s);
void aux_cfl(const DevGrid &g, const double *vr, const double *vt, const double *cs, const double *pvr, const double *pvt,
             const CflRings &cr, int pebbles, int fast, int viscous, double *part, const CflFinal &f0, double *scal,
             int *iscal, cudaStream_t s);
void aux_evaporate(const DevGrid &g, const double *T, double *pdens, cudaStream_t s);
void aux_damp_gas(const DevGrid &g, double *vrad, double *rho, double *vtheta, double *energy, const int *rings,
                  int nrings, const double *vr0r, int damp_init, int damp_flux,
                  int energy_eq, cudaStream_t s);
void aux_open_inner(const DevGrid &g, double *rho, double *vr, double *energy, int energy_eq, int damp_flux,
                    double gasflux, cudaStream_t s);
void aux_open_outer(const DevGrid &g, double *rho, double *vr, double *energy, int energy_eq, int damp_flux,
                    double gasflux, cudaStream_t s);
void aux_nonreflecting(const DevGrid &g, double *rho, double *vr, double *energy, const double *cs, cudaStream_t s);
void aux_outer_source_mass(const DevGrid &g, double *rho, double *vr, double penul_vr, cudaStream_t s);
void aux_parametric_cooling(const DevGrid &g, const double *rho, const double *eint, const double *qplus,
                            const double *divv, const double *coolt, const double *qplusmed, double *enew,
                            double gm1, cudaStream_t s);
void aux_gas_accrete(const DevGrid &g, double *dens, const double *vrad, const double *vtheta, const double *cs,
                     const GasAccArgs &a, double *out, cudaStream_t s);
void aux_drag_cell(const double *rho, const double *cs, const double *vrad, const double *vtheta, int l, int ns,
                   double *out, cudaStream_t s);
void aux_correct_vtheta(const DevGrid &g, double *vt, double domega, cudaStream_t s);
void aux_iso_eos(const DevGrid &g, const double *rho, const double *csr, double *cs, double *press, double *temper,
                 int set_cs, int set_press, int set_temper, cudaStream_t s);
void aux_damp_peb(const DevGrid &g, double *pd, double *pvr, double *pvt, const int *rings, int nrings, cudaStream_t s);
void aux_crash(const DevGrid &g, const double *f, int *flag, cudaStream_t s);
void aux_pebble_sources(const DevGrid &g, const double *pd, const double *pvr, const double *pvt, const double *tau,
                        const double *vr, const double *vt, const double *pagr, const double *pagt, double *paccr,
                        double *pacct, double *dragr, double *dragt, int back_reaction,
                        cudaStream_t s);
void aux_pebble_substep1(const DevGrid &g, double *pvr, double *pvt, const double *tau, const double *vr, const double *vt,
                         const double *paccr, const double *pacct, const double *gaccr, const double *gacct,
                         const double *rho, const double *pd, int diffusion, double schmidt,
                         const double *invdxtheta_r, cudaStream_t s);
void aux_forces(const DevGrid &g, const ForceArgs &a0, const ForceRings &fr,
                double *scal, cudaStream_t s);
// AccArgs go to the device first (a_dev), the kernels read them there.
void aux_accrete(const DevGrid &g, const AccArgs &a, AccArgs *a_dev, double *scal, cudaStream_t s);
// The accretion kernels alone over a grid of nb_grid blocks (at least the
// annulus' aux_accrete_blocks; blocks beyond it return at once), arguments
// and the two ring means of v_theta already on the device.
void aux_accrete_kernels(const DevGrid &g, const AccArgs *a_dev, int nb_grid, double *scal, cudaStream_t s);
// Control block writes (host path): up to 6 (index, value) pairs.
struct CtlSet { int n; int idx[6]; double val[6]; };
void aux_set_ctl(double *ctl, const CtlSet &v, cudaStream_t s);
int aux_accrete_blocks(const DevGrid &g, int imin, int imax);
void aux_integrals(const DevGrid &g, const double *rho, const double *vr, const double *vt, const double *e,
                   const double *pd, const double *pvt, double omega_frame, int pebbles, double *part, double *scal,
                   cudaStream_t s);
void aux_min_final(const double *part, int nb, double *out, cudaStream_t s);

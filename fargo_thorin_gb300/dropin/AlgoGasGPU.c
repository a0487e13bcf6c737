/* AlgoGasGPU.c -- the per-DT hydro loop of FARGO_THORIN with every disk
 * operation on the GPU, as a drop-in for AlgoGas (src_main/SourceEuler.c:
 * 210-317).
 *
 * This file is compiled against the reference's own headers (fargo.h) and
 * linked with its src_main and src_reb sources and libthorin_gpu.so; main.c
 * is compiled with -DAlgoGas=AlgoGasGPU so that its call at main.c:201 lands
 * here (dropin.mk).  Everything else stays the reference's: the in.par
 * reader, the initial state, the output files, REBOUND and the planet
 * bookkeeping.  The disk lives on the GPU from the first call on.  The
 * host PolarGrids are brought up to date after a DT whenever the reference
 * reads them next: the outputs of the next iteration (main.c:177-181), the
 * -a integrals (main.c:216-220) and a crash dump.
 *
 * The order of one substep is the reference's: CFL, accretion, forces and
 * the torque log, the planet kick, REBOUND, the frame, then the hydro
 * substep (boundaries, DetectCrash, SubStep1-3, SOR, transport, pebbles).
 * Two deviations: the crash dump (gas*999.dat) holds the state after the
 * substep in which the crash was found, not before it; and the SOR
 * tolerance is the compile-time THORIN_DROPIN_SOREPS, like SOREPS of
 * EnergySources.c:23.
 */
#include "fargo.h"
#include "thorin_gpu.h"
#include "thorin_warmnet.h"

#ifndef THORIN_DROPIN_SOREPS
#define THORIN_DROPIN_SOREPS 1.0e-6      /* SOREPS, EnergySources.c:23 */
#endif
#define THORIN_DROPIN_SORMAXITERS 100000  /* SORMAXITERS, EnergySources.c:22 */

/* switches the reference keeps as globals outside its headers */
extern boolean OpenInner, OpenOuter, NonReflecting, OuterSourceMass, FastTransport, IsDisk, Corotating;
extern boolean Indirect_Term, Restart, DumpTorqueNow, GuidingCenter;
extern int begin_i;
extern real ScalingFactor;

static thorin_disk *g_disk = NULL;
static long g_iter = -1;                 /* main.c's loop index i of the current call */
static int g_crashed_before = 0;         /* AlreadyCrashed of SourceEuler.c:42 */

static void die(const char *what, int rc)
{
  mastererr("AlgoGasGPU: %s failed (status %d): %s\n", what, rc, thorin_gpu_last_error());
  prs_exit(1);
}

#define CALL(expr)                          \
  do {                                      \
    int rc_ = (expr);                       \
    if (rc_ != THORIN_OK) die(#expr, rc_);  \
  } while (0)

/* thorin_params from the reference's parameters and the switches that
 * Interpret.c (149-265) and main.c derived from them. */
static void params_from_reference(thorin_params *p)
{
  thorin_params_default(p, NRAD, NSEC);
  p->log_grid = LogGrid;
  p->rmin = RMIN;
  p->rmax = RMAX;
  p->sigma0 = SIGMA0;
  p->sigma_slope = SIGMASLOPE;
  p->aspect_ratio = ASPECTRATIO;
  p->flaring_index = FLARINGINDEX;
  p->scaling_factor = ScalingFactor;
  p->cavity_radius = CAVITYRADIUS;
  p->cavity_ratio = CAVITYRATIO;
  p->cavity_width = CAVITYWIDTH;
  p->lambda_doubling = LAMBDADOUBLING;
  p->transition_radius = TRANSITIONRADIUS;
  p->transition_ratio = TRANSITIONRATIO;
  p->transition_width = TRANSITIONWIDTH;
  p->viscosity = VISCOSITY;
  p->alpha_viscosity = ALPHAVISCOSITY;
  p->viscosity_alpha = ViscosityAlpha;
  p->alpha_flock = AlphaFlock;
  p->alpha_mri = ALPHAMRI;
  p->alpha_dead = ALPHADEAD;
  p->tmri = TMRI;
  p->twidth = TWIDTH;
  p->energy_eq = EnergyEq;
  p->adiabind = ADIABIND;
  p->cooling_time = COOLINGTIME;
  p->parametric_cooling = ParametricCooling;
  p->stellar_irradiation = StellarIrradiation;
  p->opacity_drop = OPACITYDROP;
  p->effective_temperature = EFFECTIVETEMPERATURE;
  p->stellar_radius = STELLARRADIUS;
  p->disc_albedo = DISCALBEDO;
  p->parametric_opacity = PARAMETRICOPACITY;
  /* the opacity law Interpret.c:250-265 picked */
  if (opacity_func == opacity_const) p->opacity_law = THORIN_OPA_CONST;
  else if (opacity_func == opacity_ZHU12) p->opacity_law = THORIN_OPA_ZHU12;
  else if (opacity_func == opacity_LP85) p->opacity_law = THORIN_OPA_LP85;
  else if (opacity_func == opacity_SM03) p->opacity_law = THORIN_OPA_SM03;
  else p->opacity_law = THORIN_OPA_BL94;
  p->thickness_smoothing = THICKNESSSMOOTHING;
  p->exclude_hill = ExcludeHill;
  p->hillcut = HILLCUT;
  p->indirect_term = Indirect_Term;
  p->mass_taper = MASSTAPER;
  p->vertical_damping = VERTICALDAMPING;
  p->feel_disk = FeelDisk;
  p->accretion_rate = ACCRETIONRATE;
  p->gas_accret_heating = GasAccretHeating;
  p->planetary_density = PLANETARYDENSITY;
  p->aerodynamic_drag = AerodynamicDrag;
  p->omega_frame = OmegaFrame;             /* main.c:160-165 set it (corotating, restart) */
  p->fast_transport = FastTransport;
  p->damping = Damping;
  p->damp_vrad = DampVrad;
  p->damp_init = DampInit;
  p->damp_flux = DampFlux;
  p->damping_rmin_frac = DAMPINGRMINFRAC;
  p->damping_rmax_frac = DAMPINGRMAXFRAC;
  p->damping_period_frac = DAMPINGPERIODFRAC;
  p->gasflux = GASFLUX;
  p->open_inner = OpenInner;
  p->open_outer = OpenOuter;
  p->non_reflecting = NonReflecting;
  p->outer_source_mass = OuterSourceMass;
  p->imposed_disk_drift = IMPOSEDDISKDRIFT;
  p->dt = DT;
  p->first_step = FIRSTSTEP;
  p->minimum_step = MINIMUMSTEP;
  p->maximum_step = MAXIMUMSTEP;
  p->sloppy_cfl = SloppyCFL;
  p->pebbles = Pebbles;
  p->back_reaction = BackReaction;
  p->accret_heating = AccretHeating;
  p->diffusive_particles = DiffusiveParticles;
  p->pebble_gravity = PebbleGravity;
  p->pebble_alpha = PEBBLEALPHA;
  p->pebble_bulk_dens = PEBBLEBULKDENS;
  p->schmidt_number = SCHMIDTNUMBER;
  p->pebble_flux = PEBBLEFLUX;
  p->pebble_coagulation = PEBBLECOAGULATION;
  p->pebble_to_gas_max = PEBBLETOGASMAX;
  p->fragment_factor = FRAGMENTFACTOR;
  p->fragment_threshold = FRAGMENTTHRESHOLD;
  p->fragment_alpha = FRAGMENTALPHA;
  p->evaporation_rate = EVAPORATIONRATE;
  p->evaporation_temperature = EVAPORATIONTEMPERATURE;
  p->heating_delay = HEATINGDELAY;
  p->parametric_accretion = PARAMETRICACCRETION;
  p->prescribed_accretion = PrescribedAccretion;
  p->sor_eps = THORIN_DROPIN_SOREPS;
  p->sor_maxiters = THORIN_DROPIN_SORMAXITERS;
  p->centrifugal_balance = CentrifugalBalance;
  p->label_advection = AdvecteLabel;
  p->corotating = Corotating;
  p->guiding_center = GuidingCenter;
}

/* A raw field file of the output directory (nrad x nsec doubles, the layout
 * of WriteDiskPolar, Output.c:153-189) into the first rows of buf. */
static void read_field_file(const char *name, double *buf)
{
  char path[1024];
  FILE *f;
  snprintf(path, sizeof(path), "%s%s", OUTPUTDIR, name);
  f = fopen(path, "rb");
  if (!f || fread(buf, sizeof(double), (size_t)NRAD * NSEC, f) != (size_t)NRAD * NSEC) {
    mastererr("AlgoGasGPU: cannot read %s\n", path);
    prs_exit(1);
  }
  fclose(f);
}

/* OpacityTable SM03: the gas table InitOpacities (Opacity2.c:250-297)
 * reads, handed to the GPU. */
static void upload_sm03_table(void)
{
  char path[1024];
  FILE *f;
  int rows, cols, k, n;
  double *v;
  snprintf(path, sizeof(path), "%s%s", INPUTDIR, "data_gasopacity_malygin.txt");
  f = fopen(path, "r");
  if (!f || fscanf(f, "%d %d", &rows, &cols) != 2 || rows < 2 || cols < 2) {
    mastererr("AlgoGasGPU: cannot read the gas opacity table %s\n", path);
    prs_exit(1);
  }
  n = rows + cols + 2 * rows * cols;
  v = (double *)malloc(sizeof(double) * (size_t)n);
  for (k = 0; k < n; k++)
    if (fscanf(f, "%lf", &v[k]) != 1) {
      mastererr("AlgoGasGPU: short gas opacity table %s\n", path);
      prs_exit(1);
    }
  fclose(f);
  CALL(thorin_gpu_set_opacity_table(g_disk, rows, cols, v, v + rows, v + rows + cols, v + rows + cols + rows * cols));
  free(v);
}

/* First call: create the GPU disk and give it the reference's state -- the
 * fields Initialization (or the restart) built, the ring profiles that
 * serve as damping targets, the clock and the frame. */
static void dropin_init(PolarGrid *Rho, PolarGrid *Vrad, PolarGrid *Vtheta, PolarGrid *Energy, PolarGrid *Label)
{
  thorin_params p;
  const char *dump = getenv("THORIN_DROPIN_PARAMS");
  double *buf;
  if (IsDisk != YES) {
    mastererr("AlgoGasGPU: runs without a disk (Disk NO) have no GPU path\n");
    prs_exit(1);
  }
  params_from_reference(&p);
  if (dump && *dump) {                    /* the parameters as built, for checking the translation */
    FILE *f = fopen(dump, "wb");
    if (f) {
      fwrite(&p, sizeof(p), 1, f);
      fclose(f);
    }
  }
  CALL(thorin_gpu_create(&p, &g_disk));
  CALL(thorin_gpu_init_default(g_disk));
  if (p.opacity_law == THORIN_OPA_SM03) upload_sm03_table();
  CALL(thorin_gpu_upload(g_disk, THORIN_DENS, Rho->Field));
  CALL(thorin_gpu_upload(g_disk, THORIN_VRAD, Vrad->Field));
  CALL(thorin_gpu_upload(g_disk, THORIN_VTHETA, Vtheta->Field));
  CALL(thorin_gpu_upload(g_disk, THORIN_ENERGY, Energy->Field));
  if (AdvecteLabel) CALL(thorin_gpu_upload(g_disk, THORIN_LABEL, Label->Field));
  if (Pebbles) {
    CALL(thorin_gpu_upload(g_disk, THORIN_PEBDENS, PebbleDens->Field));
    CALL(thorin_gpu_upload(g_disk, THORIN_PEBVRAD, PebbleVrad->Field));
    CALL(thorin_gpu_upload(g_disk, THORIN_PEBVTHETA, PebbleVtheta->Field));
    /* the pebble size grid is private to Pebbles.c; both of its set-ups
     * (InitPebblesViaFlux and RestartPebbleDisk) leave it in
     * gaspebblesize0.dat of the output directory */
    buf = (double *)calloc((size_t)(NRAD + 1) * NSEC, sizeof(double));
    read_field_file("gaspebblesize0.dat", buf);
    CALL(thorin_gpu_upload(g_disk, THORIN_PEBSIZE, buf));
    free(buf);
    CALL(thorin_gpu_set_profile(g_disk, THORIN_PEBDENSINIT, PebDensInit));
    CALL(thorin_gpu_set_profile(g_disk, THORIN_PEBVRADINIT, PebVradInit));
    CALL(thorin_gpu_set_profile(g_disk, THORIN_PEBVTHETAINIT, PebVthetaInit));
  }
  CALL(thorin_gpu_set_profile(g_disk, THORIN_SIGMAMED, SigmaMed));
  CALL(thorin_gpu_set_profile(g_disk, THORIN_SIGMAINF, SigmaInf));
  CALL(thorin_gpu_set_profile(g_disk, THORIN_ENERGYMED, EnergyMed));
  CALL(thorin_gpu_set_profile(g_disk, THORIN_VTHETAMED, VthetaMed));
  CALL(thorin_gpu_set_time(g_disk, PhysicalTime));
  CALL(thorin_gpu_set_frame(g_disk, OmegaFrame));
  CALL(thorin_gpu_refresh(g_disk, 0));   /* EOS of the uploaded state */
  {
    /* opt-in, no reference counterpart: THORIN_SOR_EXTRAPOLATE=<order 1..4>
     * starts every SOR solve from the extrapolated update (the exit tests
     * and the threshold stay SuccessiveOverrelaxation's; only the number of
     * sweeps changes) */
    const char *ex = getenv("THORIN_SOR_EXTRAPOLATE");
    if (ex && atoi(ex) > 0) {
      CALL(thorin_gpu_warmstart_order(g_disk, atoi(ex)));
      CALL(thorin_gpu_warmstart(g_disk, NULL, THORIN_WS_EXTRAPOLATE, 0.f));
    }
  }
  g_iter = begin_i;
}

static void to_gpu_planets(const PlanetarySystem *sys, thorin_planets *tp)
{
  int k;
  if (sys->nb > THORIN_MAXPLANETS) {
    mastererr("AlgoGasGPU: %d planets, at most %d\n", sys->nb, THORIN_MAXPLANETS);
    prs_exit(1);
  }
  tp->nb = sys->nb;
  for (k = 0; k < sys->nb; k++) {
    tp->mass[k] = sys->mass[k]; tp->gas[k] = sys->gas[k]; tp->solid[k] = sys->solid[k];
    tp->x[k] = sys->x[k]; tp->y[k] = sys->y[k]; tp->z[k] = sys->z[k];
    tp->vx[k] = sys->vx[k]; tp->vy[k] = sys->vy[k]; tp->vz[k] = sys->vz[k];
    tp->ax[k] = sys->ax[k]; tp->ay[k] = sys->ay[k]; tp->az[k] = sys->az[k];
    tp->acc[k] = sys->acc[k];
    tp->feel_disk[k] = sys->FeelDisk[k];
  }
}

static void from_gpu_planets(const thorin_planets *tp, PlanetarySystem *sys)
{
  int k;
  for (k = 0; k < sys->nb; k++) {
    sys->mass[k] = tp->mass[k]; sys->gas[k] = tp->gas[k]; sys->solid[k] = tp->solid[k];
    sys->x[k] = tp->x[k]; sys->y[k] = tp->y[k]; sys->z[k] = tp->z[k];
    sys->vx[k] = tp->vx[k]; sys->vy[k] = tp->vy[k]; sys->vz[k] = tp->vz[k];
    sys->ax[k] = tp->ax[k]; sys->ay[k] = tp->ay[k]; sys->az[k] = tp->az[k];
  }
}

/* UpdateLog's line for each planet (Force.c:27-70), from the GPU's records. */
static void write_torque_log(void)
{
  thorin_torque t[THORIN_MAXPLANETS];
  int n = 0, k;
  char name[1024];
  FILE *out;
  CALL(thorin_gpu_get_torques(g_disk, t, THORIN_MAXPLANETS, &n));
  for (k = 0; k < n && k < THORIN_MAXPLANETS; k++) {
    snprintf(name, sizeof(name), "%stqwk%d.dat", OUTPUTDIR, k);
    out = fopenp(name, "a");
    fprintf(out, "%#.18g\t%#.18g\t%#.18g\t%#.18g\t%#.18g\t%#.18g\t%#.18g\n", t[k].time, t[k].torque, t[k].torque_norm,
            t[k].x, t[k].y, t[k].ax, t[k].ay);
    fclose(out);
  }
}

/* The host copies of the fields the reference's outputs and monitors read. */
static void download_state(PolarGrid *Rho, PolarGrid *Vrad, PolarGrid *Vtheta, PolarGrid *Energy, PolarGrid *Label)
{
  CALL(thorin_gpu_download(g_disk, THORIN_DENS, Rho->Field));
  CALL(thorin_gpu_download(g_disk, THORIN_VRAD, Vrad->Field));
  CALL(thorin_gpu_download(g_disk, THORIN_VTHETA, Vtheta->Field));
  CALL(thorin_gpu_download(g_disk, THORIN_ENERGY, Energy->Field));
  CALL(thorin_gpu_download(g_disk, THORIN_TEMPER, Temperature->Field));
  CALL(thorin_gpu_download(g_disk, THORIN_SOUNDSPEED, SoundSpeed->Field));
  CALL(thorin_gpu_download(g_disk, THORIN_PRESSURE, Pressure->Field));
  if (AdvecteLabel) CALL(thorin_gpu_download(g_disk, THORIN_LABEL, Label->Field));
  if (EnergyEq) {
    CALL(thorin_gpu_download(g_disk, THORIN_DIVV, DivergenceVelocity->Field));
    CALL(thorin_gpu_download(g_disk, THORIN_QPLUS, Qplus->Field));
    CALL(thorin_gpu_download(g_disk, THORIN_QMINUS, Qminus->Field));
    CALL(thorin_gpu_download(g_disk, THORIN_OPACITY, Opacity->Field));
  }
  if (Pebbles) {
    CALL(thorin_gpu_download(g_disk, THORIN_PEBDENS, PebbleDens->Field));
    CALL(thorin_gpu_download(g_disk, THORIN_PEBVRAD, PebbleVrad->Field));
    CALL(thorin_gpu_download(g_disk, THORIN_PEBVTHETA, PebbleVtheta->Field));
    CALL(thorin_gpu_download(g_disk, THORIN_STOKES, StokesNumber->Field));
  }
}

void AlgoGasGPU(PolarGrid *Rho, PolarGrid *Vrad, PolarGrid *Vtheta, PolarGrid *Energy, PolarGrid *Label,
                PlanetarySystem *sys, struct reb_simulation *rsim)
{
  real dt = DT, dtemp = 0.0, OmegaNew, domega;
  double ind[2], rrho[THORIN_MAXPLANETS], rcs[THORIN_MAXPLANETS];
  thorin_planets tp;
  thorin_stats st;
  int n = 1, rc, crashed_now = 0;
  if (!g_disk) dropin_init(Rho, Vrad, Vtheta, Energy, Label);
  if (SloppyCFL == YES) {                  /* one CFL per DT (SourceEuler.c:221-228) */
    CALL(thorin_gpu_cfl(g_disk, DT - dtemp, 0.0, &n));
    dt = DT / (real)n;
  }
  while (dtemp < 0.999999999 * DT) {
    MassTaper = PhysicalTime / (MASSTAPER * 2.0 * M_PI);
    MassTaper = (MassTaper > 1.0 ? 1.0 : pow(sin(MassTaper * M_PI / 2.0), 2.0));
    if (SloppyCFL == NO) {
      MinStepForRebound(rsim);             /* sets invdtreb_sq */
      CALL(thorin_gpu_cfl(g_disk, DT - dtemp, invdtreb_sq, &n));
      dt = (DT - dtemp) / (real)n;
    } else if (Pebbles) {
      CALL(thorin_gpu_stokes(g_disk));
    }
    to_gpu_planets(sys, &tp);
    CALL(thorin_gpu_accrete(g_disk, &tp, dt));
    from_gpu_planets(&tp, sys);
    dtemp += dt;
    if (Corotating == YES) GetPsysInfo(sys, MARK);
    if (DumpTorqueNow) CALL(thorin_gpu_request_torques(g_disk));
    CALL(thorin_gpu_forces(g_disk, &tp, MassTaper, ind, rrho, rcs));
    if (DumpTorqueNow) {
      DumpTorqueNow = NO;
      write_torque_log();
    }
    CALL(thorin_advance_from_disk(g_disk, &tp, dt, ind, rrho, rcs));
    if (AerodynamicDrag == YES) CALL(thorin_gpu_drag(g_disk, &tp, dt));
    from_gpu_planets(&tp, sys);
    AdvanceSystemRebound(sys, rsim, dt);
    if (Corotating == YES) {
      OmegaNew = GetPsysInfoFromRsim(rsim, GET) / dt;
      domega = OmegaNew - OmegaFrame;
      CALL(thorin_gpu_correct_vtheta(g_disk, domega));
      OmegaFrame = OmegaNew;
    }
    RotatePsys(rsim, OmegaFrame * dt);
    SynchronizeFargoRebound(sys, rsim);
    rc = thorin_gpu_hydro(g_disk, dt);
    if (rc == THORIN_ERR_SOR_MAXIT)
      masterprint("SOR: iteration cap reached\n");   /* the reference only warns */
    else if (rc != THORIN_OK)
      die("thorin_gpu_hydro", rc);
    CALL(thorin_gpu_get_stats(g_disk, &st));
    if (st.crashed) {
      if (g_crashed_before == 0) {
        fprintf(stdout, "\nCrash! at time %.12g\n", PhysicalTime);
        download_state(Rho, Vrad, Vtheta, Energy, Label);
        WriteDiskPolar(Rho, 999);
        WriteDiskPolar(Vrad, 999);
        WriteDiskPolar(Vtheta, 999);
        WriteDiskPolar(Temperature, 999);
      }
      g_crashed_before++;
      crashed_now = 1;
      masterprint("c");
    } else {
      masterprint(".");
    }
    fflush(stdout);
    PhysicalTime += dt;
  }
  masterprint("\n");
  /* the next iteration writes outputs (main.c:177), or -a reads the fields */
  g_iter++;
  if (MonitorIntegral == YES || crashed_now || (g_iter <= NTOT && NINTERM * (g_iter / NINTERM) == g_iter))
    download_state(Rho, Vrad, Vtheta, Energy, Label);
}

/*
 * thorin_gpu.h -- C ABI of the GB300 (sm_103a) FP64 implementation of the
 * FARGO_THORIN per-timestep hydrodynamics loop.
 *
 * The reference has no plugin/FFI layer: its driver calls
 *   void AlgoGas(PolarGrid *Rho, *Vrad, *Vtheta, *Energy, *Label,
 *                PlanetarySystem *sys, struct reb_simulation *rsim)
 * once per DT (src_main/main.c:201, src_main/SourceEuler.c:210-317), and the
 * physics routines communicate through globals (src_main/global.h,
 * src_main/param.h).  This header replaces that link-level interface with
 * plain C entry points (no C++/torch types): parameters are passed in one
 * struct that mirrors the in.par variables (src_main/var.c:17-141) and the
 * switches derived from them (src_main/Interpret.c:149-265); fields are passed
 * as host double arrays in the reference's PolarGrid layout
 * (l = j + i*nsec, rows 0..nrad, src_main/LowTasks.c:73-103).
 *
 * All entry points return a status code (THORIN_OK == 0).  Device memory is
 * owned by the library; host arrays are owned by the caller.
 */
#ifndef THORIN_GPU_H
#define THORIN_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define THORIN_OK               0
#define THORIN_ERR_ARG          1   /* bad argument or unsupported option      */
#define THORIN_ERR_CUDA         2   /* a CUDA call failed                       */
#define THORIN_ERR_CRASH        3   /* negative density/energy (DetectCrash)    */
#define THORIN_ERR_SOR_MAXIT    4   /* SOR hit its iteration cap                */
#define THORIN_ERR_TIMEOUT      5   /* a bounded device wait gave up            */
#define THORIN_ERR_STATE        6   /* call out of order                        */
#define THORIN_ERR_NOMEM        7   /* allocation failed                        */
#define THORIN_ERR_OMEGA        8   /* SOR omega calibration did not converge   */

#define THORIN_MAXPLANETS     120   /* src_main/types.h:67 */

/* Opacity laws (src_main/Interpret.c:250-265). */
#define THORIN_OPA_BL94   0
#define THORIN_OPA_ZHU12  1
#define THORIN_OPA_LP85   2
#define THORIN_OPA_CONST  3
#define THORIN_OPA_SM03   4   /* Semenov et al. (2003) dust + Malygin et al. (2014) gas table */

/* Field identifiers for upload/download.  Sizes are (nrad+1)*nsec doubles
 * (the reference allocates nrad+1 rows; row nrad is the outer v_rad face). */
enum thorin_field {
  THORIN_DENS = 0,        /* gas surface density Sigma                 */
  THORIN_VRAD,            /* gas radial velocity (inner face of cell)  */
  THORIN_VTHETA,          /* gas azimuthal velocity (left face of cell)*/
  THORIN_ENERGY,          /* gas internal energy per unit area         */
  THORIN_PEBDENS,         /* pebble surface density                    */
  THORIN_PEBVRAD,
  THORIN_PEBVTHETA,
  THORIN_PEBSIZE,         /* dominant pebble size (code units)         */
  THORIN_TEMPER,          /* temperature (output only)                 */
  THORIN_SOUNDSPEED,      /* sound speed (output only)                 */
  THORIN_PRESSURE,        /* pressure (output only)                    */
  THORIN_STOKES,          /* Stokes number (output only)               */
  THORIN_QPLUS,           /* viscous heating (output only)             */
  THORIN_DIVV,            /* velocity divergence (output only)         */
  THORIN_OPACITY,         /* opacity in code units (output only)       */
  THORIN_QMINUS,          /* radiative cooling term (output only)      */
  THORIN_LABEL,           /* passive tracer (LabelAdvection YES)       */
  THORIN_NFIELDS
};

/* Ring (1D radial) profiles kept by the reference as globals and used as
 * damping targets / ring means.  Each has nrad entries. */
enum thorin_profile {
  THORIN_SIGMAMED = 0,    /* SigmaMed   (Theo.c:25, RefillSigma Theo.c:33) */
  THORIN_SIGMAINF,        /* SigmaInf                                      */
  THORIN_ENERGYMED,       /* EnergyMed  (Theo.c:76, RefillEnergy Theo.c:82)*/
  THORIN_VTHETAMED,       /* VthetaMed  (Theo.c:132)                       */
  THORIN_PEBDENSINIT,     /* PebDensInit   (Pebbles.c:182,208)             */
  THORIN_PEBVRADINIT,     /* PebVradInit                                   */
  THORIN_PEBVTHETAINIT,   /* PebVthetaInit                                 */
  THORIN_NPROFILES
};

/* Parameters: the in.par variables (src_main/var.c) and derived switches
 * (src_main/Interpret.c:149-265) read by the hydro loop.  Integers are 0/1
 * switches unless noted.  thorin_params_default() fills the reference's
 * defaults. */
typedef struct thorin_params {
  /* mesh */
  int    nrad, nsec;
  int    log_grid;               /* RadialSpacing Logarithmic           */
  double rmin, rmax;
  /* disk profiles */
  double sigma0, sigma_slope, aspect_ratio, flaring_index;
  double scaling_factor;         /* -f command-line factor (main.c:100) */
  double cavity_radius, cavity_ratio, cavity_width, lambda_doubling;
  double transition_radius, transition_ratio, transition_width;
  /* viscosity */
  double viscosity, alpha_viscosity;
  int    viscosity_alpha;        /* ALPHAVISCOSITY != 0                 */
  int    alpha_flock;
  double alpha_mri, alpha_dead, tmri, twidth;
  /* energy equation */
  int    energy_eq;
  double adiabind;
  double cooling_time;           /* > 0 selects parametric cooling      */
  int    parametric_cooling;
  int    stellar_irradiation;
  double opacity_drop, effective_temperature, stellar_radius, disc_albedo;
  double parametric_opacity;
  int    opacity_law;            /* THORIN_OPA_*                        */
  /* planets and disk forces */
  double thickness_smoothing;
  int    exclude_hill;
  double hillcut;
  int    indirect_term;
  double mass_taper;             /* MASSTAPER                           */
  double vertical_damping;
  int    feel_disk;
  double accretion_rate;         /* ACCRETIONRATE (gas accretion)       */
  int    gas_accret_heating;
  double planetary_density;
  int    aerodynamic_drag;
  /* frame and transport */
  double omega_frame;
  int    fast_transport;         /* FARGO (1) or standard (0)           */
  /* boundaries */
  int    damping, damp_vrad, damp_init, damp_flux;
  double damping_rmin_frac, damping_rmax_frac, damping_period_frac;
  double gasflux;
  int    open_inner, open_outer, non_reflecting, outer_source_mass;
  double imposed_disk_drift;
  /* time stepping */
  double dt;                     /* DT                                  */
  double first_step, minimum_step, maximum_step;
  int    sloppy_cfl;
  /* pebbles */
  int    pebbles, back_reaction, accret_heating, diffusive_particles, pebble_gravity;
  double pebble_alpha, pebble_bulk_dens, schmidt_number;
  double pebble_flux, pebble_coagulation, pebble_to_gas_max;
  double fragment_factor, fragment_threshold, fragment_alpha;
  double evaporation_rate, evaporation_temperature;
  int    heating_delay;
  double parametric_accretion;
  int    prescribed_accretion;
  /* SOR (EnergySources.c:22-27; the tolerance is a compile-time constant
   * there and a parameter here) */
  double sor_eps;                /* SOREPS                              */
  int    sor_maxiters;           /* SORMAXITERS                         */
  /* command-line switches of main.c:56-100 */
  int    centrifugal_balance;    /* -b: v_theta from the radial force balance */
  int    label_advection;        /* LabelAdvection YES: a passive tracer    */
  int    corotating;             /* Frame COROTATING: the frame follows planet 0
                                    (omega_frame starts at its angular speed) */
  int    guiding_center;         /* Frame GUIDINGCENTER (implies corotating): the
                                    frame follows planet 0's guiding centre when its
                                    orbit is eccentric and inclined (Psys.c:195-262) */
} thorin_params;

/* The planetary system as seen by the hydro loop (src_main/types.h:96-115). */
typedef struct thorin_planets {
  int    nb;
  double mass[THORIN_MAXPLANETS], gas[THORIN_MAXPLANETS], solid[THORIN_MAXPLANETS];
  double x[THORIN_MAXPLANETS], y[THORIN_MAXPLANETS], z[THORIN_MAXPLANETS];
  double vx[THORIN_MAXPLANETS], vy[THORIN_MAXPLANETS], vz[THORIN_MAXPLANETS];
  double ax[THORIN_MAXPLANETS], ay[THORIN_MAXPLANETS], az[THORIN_MAXPLANETS];
  double acc[THORIN_MAXPLANETS];
  int    feel_disk[THORIN_MAXPLANETS];
} thorin_planets;

/* One line of the torque log tqwk<k>.dat (UpdateLog, src_main/Force.c:27-70):
 * the disk's torque on planet k at the first substep of a DT. */
typedef struct thorin_torque {
  double time;                   /* PhysicalTime at the start of the DT          */
  double torque;                 /* x a_y - y a_x                                */
  double torque_norm;            /* torque * m * gamma / (m Omega r^2 / h)^2 / Sigma */
  double x, y, ax, ay;           /* planet position and disk acceleration        */
} thorin_torque;

/* Run statistics of the last call. */
typedef struct thorin_stats {
  int    substeps;               /* hydro substeps done in the last DT          */
  int    sor_calls;              /* SOR solves so far                           */
  long long sor_sweeps;          /* SOR sweeps so far (sum of Niter)            */
  int    sor_last_niter;         /* Niter of the last solve                     */
  double sor_omega;              /* omega used by the last solve                */
  int    crashed;                /* DetectCrash result of the last substep      */
  double physical_time;
  double last_dt;
  double sor_time_ms;            /* device time of SOR sweeps (timing on)       */
  long long sor_passes;          /* colour passes that did work (timing on)     */
  double step_time_ms;           /* device time of the last thorin_gpu_algogas  */
  long long kernel_launches;     /* kernels launched by the library so far      */
  double omega_frame;            /* OmegaFrame now (changes in corotating runs) */
} thorin_stats;

/* Fill p with the reference defaults of src_main/var.c and nrad x nsec. */
void thorin_params_default(thorin_params *p, int nrad, int nsec);

typedef struct thorin_disk thorin_disk;   /* one disk resident on one GPU */

/* Allocate all device state for one disk on the current CUDA device.
 * Replaces InitEuler's allocations (SourceEuler.c:133-175) and
 * CreatePolarGrid (LowTasks.c:73). */
int thorin_gpu_create(const thorin_params *p, thorin_disk **out);
int thorin_gpu_destroy(thorin_disk *d);

/* Build the 1D grid arrays (FillPolar1DArrays, SourceEuler.c:68-131), the
 * default initial state (FillSigma/FillEnergy/InitGasDensityEnergy,
 * ComputeSoundSpeed/Pressure/Temperature, InitGasVelocity,
 * SetWaveKillingZones: SourceEuler.c:133-175, Pframeforce.c:620-751,
 * SideEuler.c:341-362) and, with pebbles, the flux-equilibrium pebble disk
 * (EquilPebbleDisk, Pebbles.c:58-204).  Fields are left on the device. */
int thorin_gpu_init_default(thorin_disk *d);

/* Host<->device copies of one field, (nrad+1)*nsec doubles. */
int thorin_gpu_upload(thorin_disk *d, int field, const double *host);
int thorin_gpu_download(thorin_disk *d, int field, double *host);

/* After fields were uploaded (the InitializeFromFile / restart paths of
 * Init.c:81-136 and Pebbles.c:66-75): recompute c_s, P, T and the ring means
 * from the resident fields.  flags: THORIN_REFILL_GAS redoes RefillSigma,
 * RefillEnergy and FillVtheta (Theo.c:33-151); THORIN_REFILL_PEBBLES redoes
 * BckpFieldsForBC (Pebbles.c:208-232). */
#define THORIN_REFILL_GAS     1
#define THORIN_REFILL_PEBBLES 2
/* Alone (not combined with the others): only the ring means of c_s (and
 * of T) and the viscosity per ring, from the resident c_s and T, as the end
 * of a substep leaves them; for a state restored from a snapshot taken
 * between DTs that includes c_s and T. */
#define THORIN_REFRESH_RING_MEANS 4
int thorin_gpu_refresh(thorin_disk *d, int flags);

/* Ring profiles (nrad doubles each). */
int thorin_gpu_set_profile(thorin_disk *d, int profile, const double *host);
int thorin_gpu_get_profile(thorin_disk *d, int profile, double *host);

/* The disk's ring geometry as FillPolar1DArrays builds it
 * (src_main/SourceEuler.c:68-131): inner and outer interface radius, the
 * cell-centre radius and the cell area of every ring (nrad doubles each;
 * any pointer may be NULL).  Host copies. */
int thorin_gpu_get_rings(thorin_disk *d, double *rinf, double *rsup, double *rmed, double *surf);

/* Rotation rate of the frame, e.g. OmegaFrame of omegaframe.dat at a
 * restart (GetOmegaFrame, Output.c:280-310). */
int thorin_gpu_set_frame(thorin_disk *d, double omega_frame);

/* Simulation clock (PhysicalTime / PhysicalTimeInitial, main.c:166). */
int thorin_gpu_set_time(thorin_disk *d, double physical_time);

/* ---- phase API: the pieces of one AlgoGas substep, for a host driver that
 * keeps REBOUND on the host (SourceEuler.c:229-315). ---- */

/* PebbleStokesNumbers + CriticalCharTime + ConditionCFL
 * (Pebbles.c:280,729; SourceEuler.c:589-712).  invdtreb_sq comes from
 * MinStepForRebound (ReboundInterface.c:360).  Returns the substep count
 * for the remaining interval dt_remaining. */
int thorin_gpu_cfl(thorin_disk *d, double dt_remaining, double invdtreb_sq, int *n_sub);

/* PebbleStokesNumbers alone (Pebbles.c:280-300), for the substeps of a
 * SloppyCFL run, where thorin_gpu_cfl is called once per DT
 * (SourceEuler.c:221-235).  Without pebbles it does nothing. */
int thorin_gpu_stokes(thorin_disk *d);

/* InitHeating + AccretePebblesOntoPlanets + Heating1 + EvaporatePebbles
 * (Planet.c:222-258, Pebbles.c:353-539, Pebbles.c:834-864).  Updates the
 * planets' masses and velocities in sys. */
int thorin_gpu_accrete(thorin_disk *d, thorin_planets *sys, double dt);

/* FillForcesArrays (Pframeforce.c:43-510) incl. ThicknessSmoothing
 * (Force.c:75): fills the disk accelerations on the device and returns the
 * disk-on-planet accelerations in sys->ax/ay, the indirect term in
 * indirect[2] and, for DampingTW04 (Pframeforce.c:571), the ring means of
 * Sigma and c_s at each planet (ring_rho/ring_cs, may be NULL). */
int thorin_gpu_forces(thorin_disk *d, thorin_planets *sys, double mass_taper,
                      double indirect[2], double *ring_rho, double *ring_cs);

/* Everything after the planet update in one substep: boundaries, crash test,
 * pressure, pebble sources, SubStep1/2/3, implicit radiative diffusion with
 * SOR, transport, EOS refresh, pebble transport (SourceEuler.c:270-313).
 * Advances the clock by dt. */
int thorin_gpu_hydro(thorin_disk *d, double dt);

/* AdvanceSystemFromDisk with DampingTW04 (Pframeforce.c:514-603): kicks the
 * velocities of the planets that feel the disk by dt times the disk and
 * indirect accelerations of the last thorin_gpu_forces call, which also
 * returned indirect, ring_rho and ring_cs.  Host arithmetic only. */
int thorin_advance_from_disk(const thorin_disk *d, thorin_planets *sys, double dt, const double indirect[2],
                             const double *ring_rho, const double *ring_cs);

/* CorrectVtheta and CorrectPebblesVtheta (SideEuler.c:505-519) of a
 * corotating frame whose rate changes by domega: v_theta -= domega * Rmed
 * for the gas (and the pebbles), and OmegaFrame += domega. */
int thorin_gpu_correct_vtheta(thorin_disk *d, double domega);

/* ---- whole-DT driver ---- */

/* One call of AlgoGas (SourceEuler.c:210-317) with the planets integrated on
 * the host by the library's own N-body integrator (standing in for
 * REBOUND's IAS15, ReboundInterface.c:262-325).  sys is updated in place. */
int thorin_gpu_algogas(thorin_disk *d, thorin_planets *sys);

/* The same DT as one CUDA graph launch: the substep loop, the planet side
 * (accretion, forces, kick, N-body step) and the SOR omega schedule run on
 * the device, with no host round trip inside the DT.  The disk's first DT
 * (the omega calibration) runs as thorin_gpu_algogas.  Covers fixed frames,
 * SOR radiative diffusion, pebbles, pebble accretion with heating, all
 * boundaries and opacity laws; other options are rejected with
 * THORIN_ERR_ARG (thorin_gpu_graph_supported says which).  No torque log
 * records are made.  The graph is built at the first call for the current
 * number of planets. */
int thorin_gpu_algogas_graph(thorin_disk *d, thorin_planets *sys);

/* THORIN_OK if thorin_gpu_algogas_graph covers this disk and system, else
 * THORIN_ERR_ARG with the reason in thorin_gpu_last_error(). */
int thorin_gpu_graph_supported(thorin_disk *d, const thorin_planets *sys);

/* Launch shape of the SOR sweeps (no counterpart in the reference): sweeps
 * per run of the sweep loop's body (1..64, default 8) and the resident
 * threads per multiprocessor of a colour pass (128..2048 in steps of 128,
 * default 1536).  Results do not depend on either; the ensemble autotuner
 * picks them per disk size.  The disk's graphs are rebuilt at their next
 * use. */
int thorin_gpu_set_launch_shape(thorin_disk *d, int sor_loop_sweeps, int sor_threads_per_sm);
int thorin_gpu_get_launch_shape(thorin_disk *d, int *sor_loop_sweeps, int *sor_threads_per_sm);

/* Conservation integrals (SideEuler.c:26-80,523-565), summed on the device. */
int thorin_gpu_integrals(thorin_disk *d, double *mass, double *momentum,
                         double *energy, double *peb_mass, double *peb_momentum);

/* Per-ring FARGO shifts of the last gas transport (TransportEuler.c:70-111),
 * nrad ints. */
int thorin_gpu_get_nshift(thorin_disk *d, int *host);

int thorin_gpu_get_stats(thorin_disk *d, thorin_stats *s);

/* SOR over-relaxation schedule (EnergySources.c:298-317).  The reference
 * calibrates omega on its first solve (IterateRelaxationParameter,
 * :340-403) and then nudges it by +-domega each call; get/set lets a
 * restarted run continue the schedule instead of recalibrating. */
int thorin_gpu_get_sor_state(thorin_disk *d, double *omega, double *domega, int *niterlast, int *calibrated);
int thorin_gpu_set_sor_state(thorin_disk *d, double omega, double domega, int niterlast);

/* Device timing of the SOR sweeps and of whole DTs with CUDA events on the
 * library's stream (counters in thorin_stats). */
int thorin_gpu_set_timing(thorin_disk *d, int on);

/* DiffusionTimestep's dt_stellar (EnergySources.c:833), which the last
 * energy step leaves for the next CFL (SourceEuler.c:680-690): with the
 * fields and the SOR state, what a snapshot between DTs must carry for the
 * next DT to repeat. */
int thorin_gpu_get_dt_stellar(thorin_disk *d, double *dt_stellar);
int thorin_gpu_set_dt_stellar(thorin_disk *d, double dt_stellar);

/* The CUDA stream all work of this disk is issued on (cudaStream_t). */
int thorin_gpu_get_stream(thorin_disk *d, void **stream);

/* Gas mass, angular momentum and total energy (the sums of GasTotalMass,
 * GasMomentum and GasTotalEnergy) of fields the caller already holds in
 * device memory, computed without allocating any device memory.  No
 * counterpart in the reference: it is for callers that cannot allocate, such
 * as a host program whose pool allocator already owns all free GPU memory, or
 * a hook inside a latency-critical loop where a cudaMalloc (which can
 * synchronise the device) is not acceptable.
 * Inputs: rho, vrad, vtheta, energy in the PolarGrid layout ((nrad+1)*nsec
 * doubles; vrad row nrad is read), and per-ring surf, rinf, rsup, rmed (nrad
 * doubles) -- all device pointers.  Output: out[0..2] = mass, momentum,
 * energy, a device pointer.  Work is issued on stream (a cudaStream_t, or
 * NULL for the default stream); the call returns without waiting.
 * Limit: 1 <= nrad <= 16384 (the reference's MAX1D); larger grids are
 * rejected with THORIN_ERR_ARG.  The partial sums use one fixed device array
 * per GPU, found on the first call made while that GPU is current (make that
 * call before any stream capture) and found again when the GPU's context
 * has changed since (after a cudaDeviceReset, say); concurrent calls on one
 * GPU race on it. */
int thorin_integrals_static(const double *rho, const double *vrad, const double *vtheta, const double *energy,
                            const double *surf, const double *rinf, const double *rsup, const double *rmed,
                            int nrad, int nsec, double omega_frame, double *out, void *stream);

/* Gas opacity table of OpacityTable SM03 (InitOpacities, Opacity2.c:247-297:
 * the file data_gasopacity_malygin.txt holds rows, cols, the pressure grid
 * (rows values), the temperature grid (cols values), then the Planck and the
 * Rosseland tables, rows*cols values each, pressure-major).  Copied to the
 * device; required before the first step of an SM03 run. */
int thorin_gpu_set_opacity_table(thorin_disk *d, int rows, int cols, const double *pgrid, const double *tgrid,
                                 const double *planck, const double *rosseland);

/* AdvanceSystemFromDrag (Drag.c:97-119): velocity kicks of the planets that
 * feel the disk from the Stokes drag of the gas in their own cell, for
 * AerodynamicDrag YES.  thorin_gpu_algogas calls it after the disk's pull;
 * a phase-API driver calls it after AdvanceSystemFromDisk. */
int thorin_gpu_drag(thorin_disk *d, thorin_planets *sys, double dt);

/* EquilPebbleDisk (Pebbles.c:54-60) on the gas state now on the device:
 * for runs that upload their gas from files before the pebbles are set up
 * (Init.c:144-148).  No-op without pebbles. */
int thorin_gpu_init_pebbles(thorin_disk *d);

/* Torque log of the last thorin_gpu_algogas call (one record per planet,
 * taken at its first substep like UpdateLog, which AdvanceSystemFromDisk
 * calls once per DT, Pframeforce.c:523-526).  Phase-API drivers call
 * thorin_gpu_request_torques before the thorin_gpu_forces call whose
 * accelerations should be logged.  *n receives the number of records. */
int thorin_gpu_request_torques(thorin_disk *d);
int thorin_gpu_get_torques(thorin_disk *d, thorin_torque *out, int max, int *n);

/* Self-test of the kernels' division routine (reciprocal estimate, one
 * Newton-Raphson step, Markstein correction) against IEEE division on the
 * current GPU: n random quotients of values with exponents uniform in
 * [-max_exponent, max_exponent]; returns how many differ and the largest
 * difference in ulps.  No counterpart in the reference (its divisions are
 * the C operator). */
int thorin_selftest_division(long long n, unsigned long long seed, double max_exponent,
                             unsigned long long *mismatches, unsigned long long *max_ulp);

/* Self-test of the van Leer slopes' shorter division (reciprocal estimate
 * and one Newton-Raphson step, no correction) against IEEE division: n
 * random quotients as above; returns the largest difference in ulps.  No
 * counterpart in the reference. */
int thorin_selftest_slope_division(long long n, unsigned long long seed, double max_exponent,
                                   unsigned long long *max_ulp);

/* Self-test of the conditional CUDA graph nodes behind the SOR sweep loop:
 * a kernel that sets an IF node's condition to 0 must skip its body
 * (*if_zero = 0) and to 1 run it once (*if_one = 1); only then a WHILE node
 * whose body clears the condition on its fifth run is launched
 * (*while_count = 5; -1 when not run).  No counterpart in the reference. */
int thorin_selftest_graph_conditional(int *if_zero, int *if_one, int *while_count);

/* Nested conditional graph nodes (a WHILE node inside a WHILE node's body),
 * bounded: an outer loop of 3 runs, each running an inner loop of 4.  On
 * success outer = 3 and inner_total = 12.  No counterpart in the reference. */
int thorin_selftest_graph_nested(int *outer, int *inner_total);

/* FP64 fused multiply-add throughput of the current GPU in GFLOP/s (two
 * flops per FMA), measured with a short kernel of independent FMA chains:
 * the FP64-pipe ceiling for the roofline of the kernels.  No counterpart in
 * the reference. */
int thorin_selftest_fp64_peak(double *gflops);

/* Last CUDA error string (thread-local, for diagnostics). */
const char *thorin_gpu_last_error(void);

/* ---- host N-body (stands in for REBOUND) ---- */

/* reb_tools_orbit_to_particle semantics: planet k from orbital elements
 * (degrees), heliocentric.  mass etc. are read as float like
 * SetupReboundSimulation does (ReboundInterface.c:137-170). */
int thorin_planet_from_elements(thorin_planets *sys, int k, float mass, float gas,
                                float solid, float a, float e, float inc,
                                float Omega, float omega, float f);

#ifdef __cplusplus
}
#endif
#endif /* THORIN_GPU_H */

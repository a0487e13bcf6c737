/*
 * thorin_oracle.c -- CPU restatement of FARGO_THORIN's per-timestep hydro loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests, the smoke
 * check and the CPU-baseline leg of bench.py load it as the checker.  The
 * product (fargo_thorin_gb300/) never links, loads or calls it.
 *
 * It restates, in plain C99 with the reference's own per-cell arithmetic and
 * loop order, the algorithm of the reference's sequential build for the
 * AlgoGas path (src_main/SourceEuler.c:210-317) and the host pieces around it.
 * Every function cites the reference file:line it follows.  Parity is pinned
 * against outputs of the reference binary (built by oracle/ref.mk) committed
 * under tests/golden/.
 *
 * Build: -O2 -std=c99 (no FP contraction, like the reference's -std=c99
 * build); -fopenmp adds the reference's OpenMP loop parallelism for the CPU
 * baseline.  Sums that the reference performs sequentially stay sequential.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include "../include/thorin_gpu.h"

#define PI 3.14159265358979323844                      /* fondam.h:14 */
#ifndef M_PI
#define M_PI 3.14159265358979323846                     /* glibc math.h */
#endif
#define G 1.0
#define GASCONST 1.0
#define MOLWEIGHT 1.0
#define SQRT2PI_INV (1.0/sqrt(2.0*PI))
#define MSOL_SI 1.98855e30
#define GM_SI 1.32712440018e20
#define AU_SI 149597870700.0
#define R_STANDARD 8.3144598
#define MMW 2.4
#define R_SI (R_STANDARD/(MMW*0.001))
#define OPA2CU (MSOL_SI*1000.0/pow(AU_SI*100.0,2.0))
#define T2SI (GM_SI/R_SI/AU_SI)
#define TIME2SI (sqrt(pow(AU_SI,3.0)/GM_SI))
#define RHO2CGS (MSOL_SI*1000.0/pow(AU_SI*100.0,3.0))
#define STEFANBOLTZMANN (5.670367e-8*(1.0/MSOL_SI)*pow(1.0/TIME2SI,-3.0)*pow(1.0/T2SI,-4.0))
#define FLUX2CU (0.000003/(2.0*PI))
#define CFLSECURITY 0.5                                 /* SourceEuler.c:16 */
#define CVNR 1.41                                       /* SourceEuler.c:19 */
#define SORMIN 1.0e-15                                  /* EnergySources.c:24 */
#define SORPRECISION 1.0e-15                            /* EnergySources.c:25 */
#define OMEGAUPPER 1.9                                  /* EnergySources.c:27 */
#define TRAPEZMAX 16                                    /* Pebbles.c:21 */
#define TRAPEZEPS 1.0e-4
#define EVAPOREDSIGMA 1.0e-8                            /* Pebbles.c:832 */
#define KAPPAFLOOR 1.0e-12                              /* Opacity.c:29 */

/* The OpenMP build (the CPU baseline) parallelises the same loops as the
 * reference's OpenMP build; the sequential build ignores the pragmas. */
#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

typedef struct ora_disk {
  thorin_params p;
  int nr, ns;
  /* 1D arrays, nr+2 entries, zero-filled like the reference's MAX1D globals */
  double *Radii, *GlobalRmed, *Rinf, *Rsup, *Rmed, *Surf, *InvRmed, *InvSurf;
  double *InvDiffRmed, *InvDiffRsup, *InvRinf, *OmegaInv, *Rmed2;
  double *SigmaMed, *SigmaInf, *EnergyMed, *VthetaMed, *WaveKiller;
  double *CoolingTimeMed, *QplusMed;
  double *globcsvec, *globtempervec, *globpressvec, *vt1D;
  double *PebDensInit, *PebVradInit, *PebVthetaInit;
  double *VMed, *Vmoy; int *Nshift, *NshiftGas;
  /* hydro fields, (nr+3)*(ns+1)+5 doubles each (LowTasks.c:85) */
  double *rho, *vrad, *vtheta, *energy, *label, *ExtLabel;
  double *RhoStar, *RhoInt, *VradNew, *VradInt, *VthetaNew, *VthetaInt, *TemperInt;
  double *agr, *agt, *pagr, *pagt, *EnergyInt, *EnergyNew;
  double *cs, *press, *temper, *qplus, *qminus, *opacity;
  double *divv, *Drr, *Drp, *Dpp, *Trr, *Trp, *Tpp;
  double *RadMomP, *RadMomM, *ThetaMomP, *ThetaMomM, *Work, *QRStar, *VthetaRes;
  double *TempShift, *dq;
  double *abscissa, *ordinate;
  /* energy sources */
  double *GradTr, *GradTt, *GradTm, *Dcen, *Dr, *Dt, *voldens, *flaring, *qirr;
  double *A, *B, *Ml, *Mlip, *Mlim, *Mljp, *Mljm, *RHS;
  double *TsorStart;             /* T handed to the last SOR solve (its start) */
  /* pebbles */
  double *pdens, *pvrad, *pvtheta, *psize, *tau, *paccr, *pacct, *gaccr, *gacct;
  double *etafc, *etacc, *macc, *dragr, *dragt;
  /* scalars carried between calls (file-static in the reference) */
  double PhysicalTime, PhysicalTimeInitial, MassTaper, OmegaFrame;
  double dt_stellar, invdtpeb_sq, invdtreb_sq, pebbulkdens, CV, SQRT_ADIABIND_INV;
  double doubling;               /* ParametricAccretion's static doubling time */
  double indirect_x, indirect_y;
  double heatsrc[THORIN_MAXPLANETS]; int heatsrc_index[THORIN_MAXPLANETS]; int heatsrc_max;
  int cfl_count;                 /* ConditionCFL's static count  */
  int sor_first; double omega, domega, omegabest; int Niterlast, Niterbest;
  int jchess1st, jchess2nd;
  double Tirr4fac, Rstar;
  thorin_stats st;
} ora_disk;

static double *vec(int n) { return (double *)calloc((size_t)n, sizeof(double)); }
static double *grid(const ora_disk *d) { return vec((d->nr + 3) * (d->ns + 1) + 5); }

/* ------------------------------------------------------------------ */
/* FViscosity / AspectRatio: Viscosity.c:26-71                          */
static double FViscosity(const ora_disk *d, double rad)
{
  const thorin_params *p = &d->p;
  double viscosity, rmin, rmax, scale, alpha;
  int i = 0;
  viscosity = p->viscosity;
  if (p->viscosity_alpha) {
    while (d->GlobalRmed[i] < rad) i++;
    viscosity = p->alpha_viscosity * d->globcsvec[i] * d->globcsvec[i] * pow(rad, 1.5);
  }
  if (p->alpha_flock) {
    while (d->GlobalRmed[i] < rad) i++;
    alpha = (p->alpha_mri - p->alpha_dead) * (1.0 - tanh((p->tmri - d->globtempervec[i] * T2SI) / p->twidth)) / 2.0 + p->alpha_dead;
    viscosity = alpha * d->globcsvec[i] * d->globcsvec[i] * pow(rad, 1.5);
  }
  rmin = p->cavity_radius - p->cavity_width * p->aspect_ratio;
  rmax = p->cavity_radius + p->cavity_width * p->aspect_ratio;
  scale = 1.0 + (d->PhysicalTime - d->PhysicalTimeInitial) * p->lambda_doubling;
  rmin *= scale; rmax *= scale;
  if (rad < rmin) viscosity *= p->cavity_ratio;
  if ((rad >= rmin) && (rad <= rmax)) viscosity *= exp((rmax - rad) / (rmax - rmin) * log(p->cavity_ratio));
  return viscosity;
}

static double AspectRatio(const ora_disk *d, double rad)
{
  const thorin_params *p = &d->p;
  double ar = p->aspect_ratio, rmin, rmax, scale;
  rmin = p->transition_radius - p->transition_width * p->aspect_ratio;
  rmax = p->transition_radius + p->transition_width * p->aspect_ratio;
  scale = 1.0 + (d->PhysicalTime - d->PhysicalTimeInitial) * p->lambda_doubling;
  rmin *= scale; rmax *= scale;
  if (rad < rmin) ar *= p->transition_ratio;
  if ((rad >= rmin) && (rad <= rmax)) ar *= exp((rmax - rad) / (rmax - rmin) * log(p->transition_ratio));
  return ar;
}

/* mpi_make1Dprofile, sequential build: mpiTasks.c:12-36 */
static void make1Dprofile(const ora_disk *d, const double *f, double *axi)
{
  OMP_FOR
  for (int i = 0; i < d->nr; i++) {
    double s = 0.0;
    for (int j = 0; j < d->ns; j++) s += f[i * d->ns + j];
    axi[i] = s / (double)d->ns;
  }
}

/* ------------------------------------------------------------------ */
/* Opacity laws: Opacity.c                                             */
#define TEMP(i, j) pow(kappa[j] / kappa[i] * pow(rho, a[j] - a[i]), 1.0 / (b[i] - b[j]))
static double opacity_BL94(double rho, double T)          /* Opacity.c:31-75 */
{
  static const double kappa[] = {2.0e-4, 2.0e16, 0.1, 2.0e81, 1.0e-8, 1.0e-36, 1.5e20, 0.348};
  static const double a[] = {0.0, 0.0, 0.0, 1.0, 2.0 / 3.0, 1.0 / 3.0, 1.0, 0.0};
  static const double b[] = {2.0, -7.0, 0.5, -24.0, 3.0, 10.0, -2.5, 0.0};
  double k = KAPPAFLOOR, k1, k2, k3, t1, t2;
  if (T <= TEMP(2, 3)) {
    k1 = kappa[0] * pow(T, b[0]);
    k2 = kappa[1] * pow(T, b[1]);
    k3 = kappa[2] * pow(T, b[2]);
    t1 = 1.0 / (k1 * k1) + 1.0 / (k2 * k2);
    t1 = 1.0 / (t1 * t1);
    t2 = pow(k3 / (1.0 + 1.0e22 * pow(T, -10.0)), 4.0);
    k = pow(t1 + t2, 0.25);
  } else if ((T > TEMP(2, 3)) && (T <= TEMP(3, 4))) {
    k = kappa[3] * pow(rho, a[3]) * pow(T, b[3]);
  } else if ((T > TEMP(3, 4)) && (T <= TEMP(4, 5))) {
    k = kappa[4] * pow(rho, a[4]) * pow(T, b[4]);
  } else if ((T > TEMP(4, 5)) && (T <= TEMP(5, 6))) {
    k = kappa[5] * pow(rho, a[5]) * pow(T, b[5]);
  } else if ((T > TEMP(5, 6)) && (T <= TEMP(6, 7))) {
    k = kappa[6] * pow(rho, a[6]) * pow(T, b[6]);
  } else {
    k = kappa[7];
  }
  return k;
}
#undef TEMP

static double opacity_ZHU12(double rho, double T)         /* Opacity.c:145-199 */
{
  double xlop, xlp, xlt, pre;
  pre = R_STANDARD * 1.0e7 / MMW * rho * T;
  xlp = log10(pre);
  xlt = log10(T);
  if (xlt < 2.23567 + 0.01899 * (xlp - 5.)) xlop = 1.5 * (xlt - 1.16331) - 0.736364;
  else if (xlt < 2.30713 + 0.01899 * (xlp - 5.)) xlop = -3.53154212 * xlt + 8.767726 - (7.24786 - 8.767726) * (xlp - 5.) / 16.;
  else if (xlt < (17.7 - 0.62 + 1.5 * 2.30713) / (1.5 + 5.832)) xlop = 1.5 * (xlt - 2.30713) + 0.62;
  else if (xlt < (5.9398 + 17.7) / (5.832 + 2.129)) xlop = -5.832 * xlt + 17.7;
  else if (xlt < (129.88071 + 5.9398 + (142.996475 - 129.88071) * 0.1 * (xlp + 4.)) / (2.129 + 42.98075)) xlop = 2.129 * xlt - 5.9398;
  else if (xlt < (129.88071 + 15.0125 + (142.996475 - 129.88071) * 0.1 * (xlp + 4.)) / (4.0625 + 42.98075)) xlop = 129.88071 - 42.98075 * xlt + (142.996475 - 129.88071) * 0.1 * (xlp + 4.0);
  else if (xlt < 3.28 + xlp / 4. * 0.12) xlop = -15.0125 + 4.0625 * xlt;
  else if (xlt < 3.41 + 0.03328 * xlp / 4.) xlop = 58.9294 - 18.4808 * xlt + (61.6346 - 58.9294) * xlp / 4.;
  else if (xlt < 3.76 + (xlp - 4) / 2. * 0.03) xlop = -12.002 + 2.90477 * xlt + (xlp - 4) / 4. * (13.9953 - 12.002);
  else if (xlt < 4.07 + (xlp - 4) / 2. * 0.08) xlop = -39.4077 + 10.1935 * xlt + (xlp - 4) / 2. * (40.1719 - 39.4077);
  else if (xlt < 5.3715 + (xlp - 6) / 2. * 0.5594) xlop = 17.5935 - 3.3647 * xlt + (xlp - 6) / 2. * (17.5935 - 15.7376);
  else xlop = -0.48;
  if (xlop < 3.586 * xlt - 16.85 && xlt < 4.) xlop = 3.586 * xlt - 16.85;
  return pow(10., xlop);
}

static double opacity_LP85(double rho, double T)          /* Opacity.c:201-227 */
{
  double kappa;
  if (T < pow(2.0e-4 / 2.0e16, -1.0 / 9.0)) kappa = 2.0e-4 * T * T;
  else if (T < pow(2.0e16 / 5.0e-3, 1.0 / 8.0)) kappa = 2.0e16 * pow(T, -7.0);
  else if (T < pow(5.0e-3 / 2.0e34, -1.0 / 10.0) * pow(rho, 1.0 / 15.0)) kappa = 5.0e-3 * T;
  else if (T < pow(2.0e34 / 2.0e-8, 1.0 / 12.0)) kappa = 2.0e34 * pow(rho, 2.0 / 3.0) * pow(T, -9.0);
  else if (T < pow(2.0e-8 / 1.0e-36, 1.0 / 7.0) * pow(rho, 1.0 / 21.0)) kappa = 2.0e-8 * pow(rho, 2.0 / 3.0) * T * T * T;
  else if (T < pow(1.0e-36 / 1.5e20, -1.0 / 12.5) * pow(rho, 4.0 / 75.0)) kappa = 1.0e-36 * pow(rho, 1.0 / 3.0) * pow(T, 10.0);
  else kappa = 1.5e20 * rho * pow(T, -5.0 / 2.0);
  return kappa;
}

/* Semenov et al. (2003) dust and Malygin et al. (2014) gas opacities
 * (Opacity2.c:25-245), Rosseland means.  The dust part is a fifth-order
 * polynomial in T per temperature regime with the evaporation temperatures
 * interpolated in log rho and sine smoothing across each transition; the
 * gas part interpolates the tabulated Rosseland opacity bilinearly in
 * pressure and temperature.  The reference's integer abs() of the
 * temperature difference in the smoothing test is kept. */
static int sm_rows, sm_cols;
static double *sm_pgrid, *sm_tgrid, *sm_planck, *sm_rosseland;

void ora_set_opacity_table(int rows, int cols, const double *pgrid, const double *tgrid, const double *planck,
                           const double *rosseland)
{
  sm_rows = rows; sm_cols = cols;
  sm_pgrid = (double *)malloc(sizeof(double) * rows);
  sm_tgrid = (double *)malloc(sizeof(double) * cols);
  sm_planck = (double *)malloc(sizeof(double) * rows * cols);
  sm_rosseland = (double *)malloc(sizeof(double) * rows * cols);
  memcpy(sm_pgrid, pgrid, sizeof(double) * rows);
  memcpy(sm_tgrid, tgrid, sizeof(double) * cols);
  memcpy(sm_planck, planck, sizeof(double) * rows * cols);
  memcpy(sm_rosseland, rosseland, sizeof(double) * rows * cols);
}

static double sm_interp(const double *x, const double *y, int n, double x0)   /* Opacity2.c:28-41 */
{
  if (n <= 1) return y[0];
  if (x0 < x[0]) return y[0];
  if (x0 > x[n - 1]) return y[n - 1];
  int i = 1;
  while ((x[i] < x0) && (i < n - 1)) i++;
  return y[i - 1] + (y[i] - y[i - 1]) * (x0 - x[i - 1]) / (x[i] - x[i - 1]);
}

static double opacity_malygin(double rho, double T_gas)     /* Opacity2.c:45-92, Rosseland */
{
  const int rows = sm_rows, cols = sm_cols;
  const double *array = sm_rosseland;
  double tP = 8.3144598 * 1.0e7 / 2.4 * rho * T_gas, tT = T_gas;
  int Tlow = 0, Thigh = 1, Plow, Phigh;
  if (tT < sm_tgrid[0]) return 0.0;
  else if (tT > sm_tgrid[cols - 1]) tT = sm_tgrid[cols - 1];
  if (tP < sm_pgrid[0]) tP = sm_pgrid[0];
  else if (tP > sm_pgrid[rows - 1]) tP = sm_pgrid[rows - 1];
  for (int i = 0; i < cols - 2; i++)
    if (tT >= sm_tgrid[i]) { Tlow = i; Thigh = i + 1; }
  double fac = ((double)rows) / log10(sm_pgrid[rows - 1] / sm_pgrid[0]);
  Plow = (int)(fac * log10(tP / sm_pgrid[0]));
  Plow = (Plow > 0) ? Plow : 0;
  Plow = (Plow < rows - 2) ? Plow : rows - 2;
  Phigh = Plow + 1;
  double denom = 1.0 / ((sm_tgrid[Thigh] - sm_tgrid[Tlow]) * (sm_pgrid[Phigh] - sm_pgrid[Plow]));
  double mul1 = (sm_tgrid[Thigh] - tT) * (sm_pgrid[Phigh] - tP);
  double mul2 = (tT - sm_tgrid[Tlow]) * (sm_pgrid[Phigh] - tP);
  double mul3 = (sm_tgrid[Thigh] - tT) * (tP - sm_pgrid[Plow]);
  double mul4 = (tT - sm_tgrid[Tlow]) * (tP - sm_pgrid[Plow]);
  return denom * (mul1 * array[Tlow + Plow * cols] + mul2 * array[Thigh + Plow * cols] +
                  mul3 * array[Tlow + Phigh * cols] + mul4 * array[Thigh + Phigh * cols]);
}

/* Semenov et al. (2003) Rosseland dust coefficients (5 regimes x 6) and the
 * evaporation temperatures log T_ev(log rho) of water ice, iron,
 * orthopyroxene and olivine at 8 densities (published tables). */
static const double SM_DUST_ROSS[6][6] = {
  {0.244153190819473e-03, -0.191588103585833e-03, 0.229132294521843e-03, 0.454088516995579e-06, -0.389280273285906e-08,
   0.319006401785413e-11},
  {0.292517586013911e+01, -0.801305197566973e-01, 0.923001367150898e-03, -0.349287851393541e-05, 0.587151269508960e-08,
   -0.371333580736933e-11},
  {-0.125893536782728e+02, 0.160197849829283e+00, -0.582601311634824e-03, 0.110792133181219e-05, -0.105506373600323e-08,
   0.404997080931974e-12},
  {-0.192550086994197e+01, 0.354301116460647e-01, -0.127355043519226e-03, 0.233773506650911e-06, -0.207587683535083e-09,
   0.728005983960845e-13},
  {0.165244978116957e+01, -0.260479348963077e-02, 0.590717655258634e-05, -0.300202906476749e-08, 0.803836688553263e-12,
   -0.916709776405312e-16},
  {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}};
static const double SM_LOGTT[8][4] = {
  {2.03742650, 2.92168648, 2.95520654, 2.96801571}, {2.07188201, 2.95808585, 2.99122608, 2.99869516},
  {2.11058971, 2.99738638, 3.02077549, 3.03181227}, {2.15533604, 3.04139269, 3.05269394, 3.06744284},
  {2.20139712, 3.08990511, 3.08707121, 3.10619090}, {2.25527251, 3.14457421, 3.12417806, 3.14860265},
  {2.31597035, 3.20736504, 3.16494737, 3.19589965}, {2.38738983, 3.28057837, 3.20978301, 3.24895362}};
static const double SM_LOGRR[8] = {-18.0, -16.0, -14.0, -12.0, -10.0, -8.0, -6.0, -4.0};

static double opacity_SM03(double rho, double T_dust)       /* Opacity2.c:96-245, Rosseland */
{
  const double *eD = &SM_DUST_ROSS[0][0];
  double T_ev[4], temp[8], dT[5], T[5], aKext = 0.0;
  if (T_dust <= 0.9) return 0.9;
  double logrho = log10(rho);
  for (int i = 0; i < 4; i++) {
    for (int j = 0; j < 8; j++) temp[j] = SM_LOGTT[j][i];
    T_ev[i] = pow(10.0, sm_interp(SM_LOGRR, temp, 8, logrho));
  }
  T[0] = T_ev[0]; T[1] = 275.0; T[2] = 425.0; T[3] = 680.0;
  double tmax1 = (T_ev[1] > T_ev[2]) ? T_ev[1] : T_ev[2];
  double tmax2 = (T_ev[2] > T_ev[3]) ? T_ev[2] : T_ev[3];
  T[4] = (tmax1 < tmax2) ? tmax1 : tmax2;
  dT[0] = 5.0; dT[1] = 5.0; dT[2] = 15.0; dT[3] = 5.0; dT[4] = 100.0;
  int KK = 5;
  if (T_dust <= (T[0] + dT[0])) KK = 0;
  for (int i = 1; i < 5; i++)
    if ((T_dust > (T[i - 1] + dT[i - 1])) && (T_dust <= (T[i] + dT[i]))) KK = i;
  if (KK != 5) {
    int smooth = 0;
    for (int i = 0; i < 5; i++)
      if (abs((int)(T_dust - T[i])) < dT[i]) smooth = 1;
    if (smooth == 1) {
      double T1 = T[KK] - dT[KK], T2 = T[KK] + dT[KK], TD = T_dust - T[KK], aKrL, aKrR;
      int j = (KK + 1) * 6;
      aKrL = ((((eD[j - 1] * T1 + eD[j - 2]) * T1 + eD[j - 3]) * T1 + eD[j - 4]) * T1 + eD[j - 5]) * T1 + eD[j - 6];
      if (KK == 4) aKrR = 0.0;
      else {
        j = (KK + 2) * 6;
        aKrR = ((((eD[j - 1] * T2 + eD[j - 2]) * T2 + eD[j - 3]) * T2 + eD[j - 4]) * T2 + eD[j - 5]) * T2 + eD[j - 6];
      }
      double AA = 0.5e0 * (aKrL - aKrR), BB = 0.5e0 * (aKrL + aKrR), FF = PI / 2.0 / dT[KK];
      aKext = BB - AA * sin(FF * TD);
    } else {
      int j = (KK + 1) * 6;
      aKext = ((((eD[j - 1] * T_dust + eD[j - 2]) * T_dust + eD[j - 3]) * T_dust + eD[j - 4]) * T_dust + eD[j - 5]) *
                  T_dust + eD[j - 6];
    }
  }
  double kappa_dust = aKext, kappa_gas = opacity_malygin(rho, T_dust);
  return (kappa_dust > kappa_gas) ? kappa_dust : kappa_gas;
}

static double opacity_func(const ora_disk *d, double rho, double T)
{
  switch (d->p.opacity_law) {
  case THORIN_OPA_SM03: return opacity_SM03(rho, T);
  case THORIN_OPA_ZHU12: return opacity_ZHU12(rho, T);
  case THORIN_OPA_LP85: return opacity_LP85(rho, T);
  case THORIN_OPA_CONST: return d->p.parametric_opacity;
  default: return opacity_BL94(rho, T);
  }
}

/* ------------------------------------------------------------------ */
/* EOS: SourceEuler.c:715-792                                           */
static void ComputeSoundSpeed(ora_disk *d, const double *rho, const double *energy)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      if (!p->energy_eq)
        d->cs[l] = AspectRatio(d, d->Rmed[i]) * sqrt(G * 1.0 / d->Rmed[i]) * pow(d->Rmed[i], p->flaring_index);
      else
        d->cs[l] = sqrt(p->adiabind * (p->adiabind - 1.0) * fabs(energy[l]) / rho[l]);
    }
  make1Dprofile(d, d->cs, d->globcsvec);
}

static void ComputePressureField(ora_disk *d, const double *rho, const double *energy)
{
  int nr = d->nr, ns = d->ns;
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      if (!d->p.energy_eq) d->press[l] = rho[l] * d->cs[l] * d->cs[l];
      else d->press[l] = (d->p.adiabind - 1.0) * energy[l];
    }
}

static void ComputeTemperatureField(ora_disk *d, const double *rho, const double *energy)
{
  int nr = d->nr, ns = d->ns;
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      double t2 = 1.0 / (rho[l] * GASCONST), t1;
      if (d->p.energy_eq) { t1 = energy[l] * MOLWEIGHT * (d->p.adiabind - 1.0); d->temper[l] = t1 * t2; }
      else { t1 = MOLWEIGHT * d->press[l]; d->temper[l] = t1 * t2; }
    }
  make1Dprofile(d, d->temper, d->globtempervec);
}

/* ------------------------------------------------------------------ */
/* Initialisation                                                       */
static void FillPolar1DArrays(ora_disk *d)                 /* SourceEuler.c:68-131 */
{
  const thorin_params *p = &d->p;
  int nr = d->nr;
  double drrsep = (p->rmax - p->rmin) / (double)nr;
  for (int i = 0; i <= nr; i++) {
    if (p->log_grid) d->Radii[i] = p->rmin * exp((double)i / (double)nr * log(p->rmax / p->rmin));
    else d->Radii[i] = p->rmin + drrsep * (double)i;
  }
  for (int i = 0; i < nr; i++) {
    d->GlobalRmed[i] = 2.0 / 3.0 * (d->Radii[i + 1] * d->Radii[i + 1] * d->Radii[i + 1] - d->Radii[i] * d->Radii[i] * d->Radii[i]);
    d->GlobalRmed[i] = d->GlobalRmed[i] / (d->Radii[i + 1] * d->Radii[i + 1] - d->Radii[i] * d->Radii[i]);
  }
  for (int i = 0; i < nr; i++) {
    d->Rinf[i] = d->Radii[i];
    d->Rsup[i] = d->Radii[i + 1];
    d->Rmed[i] = 2.0 / 3.0 * (d->Rsup[i] * d->Rsup[i] * d->Rsup[i] - d->Rinf[i] * d->Rinf[i] * d->Rinf[i]);
    d->Rmed[i] = d->Rmed[i] / (d->Rsup[i] * d->Rsup[i] - d->Rinf[i] * d->Rinf[i]);
    d->Surf[i] = PI * (d->Rsup[i] * d->Rsup[i] - d->Rinf[i] * d->Rinf[i]) / (double)d->ns;
    d->InvRmed[i] = 1.0 / d->Rmed[i];
    d->InvSurf[i] = 1.0 / d->Surf[i];
    d->InvDiffRsup[i] = 1.0 / (d->Rsup[i] - d->Rinf[i]);
    d->InvRinf[i] = 1.0 / d->Rinf[i];
    d->OmegaInv[i] = pow(d->Rmed[i], 1.5);
    d->Rmed2[i] = d->Rmed[i] * d->Rmed[i];
  }
  d->Rinf[nr] = d->Radii[nr];
  for (int i = 1; i < nr; i++) d->InvDiffRmed[i] = 1.0 / (d->Rmed[i] - d->Rmed[i - 1]);
}

static double SigmaProfile(const ora_disk *d, double r)    /* Theo.c:15-23 */
{
  const thorin_params *p = &d->p;
  double cavity = 1.0;
  if (r < p->cavity_radius) cavity = 1.0 / p->cavity_ratio;
  return cavity * p->scaling_factor * p->sigma0 * pow(r, -p->sigma_slope);
}

static double EnergyProfile(const ora_disk *d, double r)   /* Theo.c:60-74 */
{
  const thorin_params *p = &d->p;
  double fac = 1.0 / (MOLWEIGHT * (p->adiabind - 1.0));
  double power = -p->sigma_slope - 1.0 + 2.0 * p->flaring_index;
  return GASCONST * p->sigma0 * pow(p->aspect_ratio, 2.0) * pow(r, power) * fac;
}

static double ConstructSequence(double *u, const double *v, int n)  /* Pframeforce.c:605-617 */
{
  double lapl = 0.0;
  for (int i = 1; i < n; i++) u[i] = 2.0 * v[i] - u[i - 1];
  for (int i = 1; i < n - 1; i++) lapl += fabs(u[i + 1] + u[i - 1] - 2.0 * u[i]);
  return lapl;
}

static void InitGasVelocity(ora_disk *d)                   /* Pframeforce.c:644-751 */
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  double *vt_int = vec(nr + 2), *vt_cent = vec(nr + 2);
  make1Dprofile(d, d->press, d->globpressvec);
  for (int i = 1; i < nr; i++) {
    vt_int[i] = (d->globpressvec[i] - d->globpressvec[i - 1]) /
                (.5 * (SigmaProfile(d, d->GlobalRmed[i]) + SigmaProfile(d, d->GlobalRmed[i - 1]))) / (d->GlobalRmed[i] - d->GlobalRmed[i - 1]) +
                G * (1.0 / d->GlobalRmed[i - 1] - 1.0 / d->GlobalRmed[i]) / (d->GlobalRmed[i] - d->GlobalRmed[i - 1]);
    vt_int[i] = sqrt(vt_int[i] * d->Radii[i]) - d->Radii[i] * d->OmegaFrame;
  }
  {
    double t1, t2, r1, r2;
    t1 = vt_cent[0] = vt_int[1] + .75 * (vt_int[1] - vt_int[2]);
    r1 = ConstructSequence(vt_cent, vt_int, nr);
    vt_cent[0] += .25 * (vt_int[1] - vt_int[2]);
    t2 = vt_cent[0];
    r2 = ConstructSequence(vt_cent, vt_int, nr);
    t1 = t1 - r1 / (r2 - r1) * (t2 - t1);
    vt_cent[0] = t1;
    ConstructSequence(vt_cent, vt_int, nr);
    vt_cent[nr] = vt_cent[nr - 1];
  }
  if (p->parametric_cooling)                                 /* FillCoolingTime, FillQplus (Theo.c:103-129) */
    for (int i = 0; i < nr; i++) {
      d->CoolingTimeMed[i] = p->cooling_time * pow(d->Rmed[i], 2.0 + 2.0 * p->flaring_index);
      d->QplusMed[i] = 2.25 * FViscosity(d, d->Rmed[i]) * p->sigma0 * pow(d->Rmed[i], -p->sigma_slope - 3.0);
    }
  for (int i = 0; i <= nr; i++) {
    double r, ri, viscosity;
    if (i == nr) { r = d->Rmed[nr - 1]; ri = d->Rinf[nr - 1]; }
    else { r = d->Rmed[i]; ri = d->Rinf[i]; }
    viscosity = FViscosity(d, r);
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      double rg = r, omega = sqrt(G * 1.0 / rg / rg / rg), rhoinf;
      d->vtheta[l] = omega * r * sqrt(1.0 - d->cs[l] * d->cs[l] * r / p->adiabind);
      d->vtheta[l] -= d->OmegaFrame * r;
      if (p->centrifugal_balance) d->vtheta[l] = vt_cent[i];      /* -b, IMIN = 0 */
      d->vrad[l] = p->imposed_disk_drift * p->sigma0 / d->SigmaInf[i] / ri;
      if (p->damp_flux) {
        if (i == 0) rhoinf = d->SigmaMed[i] - 0.5 * (d->SigmaMed[i + 1] - d->SigmaMed[i]);
        else rhoinf = 0.5 * (d->SigmaMed[i - 1] + d->SigmaMed[i]);
        d->vrad[l] -= p->gasflux / (2.0 * PI * ri * rhoinf);
      } else if (p->viscosity_alpha) {
        d->vrad[l] -= 3.0 * viscosity / r * (-p->sigma_slope + 2.0 * p->flaring_index + 1.0);
      } else {
        d->vrad[l] -= 3.0 * viscosity / r * (-p->sigma_slope + .5);
      }
    }
  }
  if (!p->damp_flux)
    for (int j = 0; j < ns; j++) d->vrad[j] = d->vrad[j + ns * nr] = 0.0;
  free(vt_int); free(vt_cent);
}

static void SetWaveKillingZones(ora_disk *d)               /* SideEuler.c:341-362 */
{
  const thorin_params *p = &d->p;
  double DRin = p->rmin * p->damping_rmin_frac, DRout = p->rmax * p->damping_rmax_frac;
  double tauin = p->damping_period_frac * 2.0 * PI * pow(p->rmin, 1.5);
  double tauout = p->damping_period_frac * 2.0 * PI * pow(DRout, 1.5);
  for (int i = 0; i < d->nr; i++) {
    double damp;
    d->WaveKiller[i] = 0.0;
    if (d->Rmed[i] < DRin) { damp = (DRin - d->Rmed[i]) / (DRin - p->rmin); d->WaveKiller[i] = damp * damp / tauin; }
    if (d->Rmed[i] > DRout) { damp = (d->Rmed[i] - DRout) / (p->rmax - DRout); d->WaveKiller[i] = damp / tauout; }
  }
}

static void FillVtheta(ora_disk *d)                         /* Theo.c:132-151 */
{
  for (int i = 0; i < d->nr; i++) {
    double moy = 0.0, vtcorr = d->Rmed[i] * d->OmegaFrame;
    for (int j = 0; j < d->ns; j++) moy += d->vtheta[j + i * d->ns] + vtcorr;
    d->VthetaMed[i] = moy / (double)d->ns;
  }
}

static void EtaPressureSupport(ora_disk *d)                 /* Pebbles.c:235-275 */
{
  int nr = d->nr, ns = d->ns;
  for (int i = 0; i < nr; i++) {
    double vtcorr = d->Rmed[i] * d->OmegaFrame, vkinv = sqrt(d->Rmed[i]);
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      double vtcc = 0.5 * (d->vtheta[l] + d->vtheta[ljp]);
      d->etacc[l] = 1.0 - (vtcc + vtcorr) * vkinv;
    }
  }
  for (int i = 1; i < nr; i++)
    for (int j = 0; j < ns; j++) { int l = j + i * ns; d->etafc[l] = 0.5 * (d->etacc[l] + d->etacc[l - ns]); }
  for (int j = 0; j < ns; j++) d->etafc[j] = d->etafc[j + ns];
}

static void InitPebblesViaFlux(ora_disk *d)                 /* Pebbles.c:80-204 */
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  double pebbleflux = p->pebble_flux * FLUX2CU, Ndf = 0.5;
  for (int i = 0; i < nr; i++) {
    double rho1 = 0, vr1 = 0, etafc1 = 0, etacc1 = 0, cs1 = 0;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      rho1 += d->rho[l]; vr1 += d->vrad[l]; etafc1 += d->etafc[l]; etacc1 += d->etacc[l]; cs1 += d->cs[l];
    }
    rho1 /= (double)ns; vr1 /= (double)ns; etafc1 /= (double)ns; etacc1 /= (double)ns; cs1 /= (double)ns;
    double tau1 = sqrt(3.0) * p->pebble_coagulation * pebbleflux / (32.0 * PI * pow(d->Rmed[i], -1.5) * rho1);
    tau1 = sqrt(tau1) / (d->Rmed[i] * etacc1);
    double psize1 = fabs(tau1) * sqrt(p->adiabind) * rho1 / (2.0 * d->pebbulkdens);
    double taudf = p->fragment_threshold * sqrt(d->Rmed[i]) / (2.0 * etacc1 * (1.0 - Ndf));
    double adf = fabs(taudf) * sqrt(p->adiabind) * rho1 / (2.0 * d->pebbulkdens);
    double taufrag = p->fragment_factor / (3.0 * p->fragment_alpha) * pow(p->fragment_threshold / cs1, 2);
    double afrag = fabs(taufrag) * sqrt(p->adiabind) * rho1 / (2.0 * d->pebbulkdens);
    if ((psize1 < adf) && (psize1 < afrag)) {
    } else if ((taudf > 0.0) && (adf < psize1) && (adf < afrag)) {
      tau1 = taudf; psize1 = adf;
    } else {
      tau1 = taufrag; psize1 = afrag;
    }
    double vtcorr = d->Rmed[i] * d->OmegaFrame, vkepl = pow(d->Rmed[i], -0.5);
    double fac = 1.0 / (tau1 * tau1 + 1.0), etaterm = etafc1 * vkepl;
    double pvr1 = -2.0 * tau1 * fac * (etaterm - 0.5 / tau1 * vr1);
    etaterm = etacc1 * vkepl;
    double pvrtemp = -2.0 * tau1 * fac * (etaterm - 0.5 / tau1 * vr1);
    double pvt1 = -fac * (etaterm - 0.5 * tau1 * vr1);
    pvt1 += (vkepl - vtcorr);
    double pdens1 = pebbleflux / (2.0 * PI * d->Rmed[i] * fabs(pvrtemp));
    if (pdens1 / rho1 > p->pebble_to_gas_max) pdens1 = rho1 * p->pebble_to_gas_max;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      d->psize[l] = psize1; d->tau[l] = tau1; d->pdens[l] = pdens1; d->pvrad[l] = pvr1; d->pvtheta[l] = pvt1;
    }
    d->PebDensInit[i] = pdens1;
    d->PebVradInit[i] = pvr1;
    d->PebVthetaInit[i] = pvt1 + d->Rmed[i] * d->OmegaFrame;
  }
}

static void BckpFieldsForBC(ora_disk *d)                    /* Pebbles.c:208-232 */
{
  for (int i = 0; i < d->nr; i++) {
    double a = 0, b = 0, c = 0;
    for (int j = 0; j < d->ns; j++) {
      int l = j + i * d->ns;
      a += d->pdens[l]; b += d->pvrad[l]; c += d->pvtheta[l];
    }
    d->PebDensInit[i] = a / (double)d->ns;
    d->PebVradInit[i] = b / (double)d->ns;
    d->PebVthetaInit[i] = c / (double)d->ns + d->Rmed[i] * d->OmegaFrame;
  }
}

static void InitComputeAccel(ora_disk *d)                   /* SideEuler.c:101-118 */
{
  for (int i = 0; i < d->nr; i++)
    for (int j = 0; j < d->ns; j++) {
      int l = j + i * d->ns;
      d->abscissa[l] = d->Rmed[i] * cos(2.0 * PI * (double)j / (double)d->ns);
      d->ordinate[l] = d->Rmed[i] * sin(2.0 * PI * (double)j / (double)d->ns);
    }
}

/* ------------------------------------------------------------------ */
/* Public: create / init                                                */
ora_disk *ora_create(const thorin_params *p)
{
  ora_disk *d = (ora_disk *)calloc(1, sizeof(ora_disk));
  d->p = *p;
  d->nr = p->nrad; d->ns = p->nsec;
  int n1 = d->nr + 2;
  double **v1[] = {&d->Radii, &d->GlobalRmed, &d->Rinf, &d->Rsup, &d->Rmed, &d->Surf, &d->InvRmed, &d->InvSurf,
                   &d->InvDiffRmed, &d->InvDiffRsup, &d->InvRinf, &d->OmegaInv, &d->Rmed2, &d->SigmaMed, &d->SigmaInf,
                   &d->EnergyMed, &d->VthetaMed, &d->WaveKiller, &d->globcsvec, &d->globtempervec, &d->globpressvec,
                   &d->vt1D, &d->PebDensInit, &d->PebVradInit, &d->PebVthetaInit, &d->VMed, &d->Vmoy,
                   &d->CoolingTimeMed, &d->QplusMed};
  for (size_t k = 0; k < sizeof(v1) / sizeof(v1[0]); k++) *v1[k] = vec(n1);
  d->Nshift = (int *)calloc((size_t)n1, sizeof(int));
  d->NshiftGas = (int *)calloc((size_t)n1, sizeof(int));
  double **v2[] = {&d->rho, &d->vrad, &d->vtheta, &d->energy, &d->label, &d->ExtLabel, &d->RhoStar, &d->RhoInt, &d->VradNew, &d->VradInt,
                   &d->VthetaNew, &d->VthetaInt, &d->TemperInt, &d->agr, &d->agt, &d->pagr, &d->pagt, &d->EnergyInt,
                   &d->EnergyNew, &d->cs, &d->press, &d->temper, &d->qplus, &d->qminus, &d->opacity, &d->divv,
                   &d->Drr, &d->Drp, &d->Dpp, &d->Trr, &d->Trp, &d->Tpp, &d->RadMomP, &d->RadMomM, &d->ThetaMomP,
                   &d->ThetaMomM, &d->Work, &d->QRStar, &d->VthetaRes, &d->TempShift, &d->dq, &d->abscissa,
                   &d->ordinate, &d->GradTr, &d->GradTt, &d->GradTm, &d->Dcen, &d->Dr, &d->Dt, &d->voldens,
                   &d->flaring, &d->qirr, &d->A, &d->B, &d->Ml, &d->Mlip, &d->Mlim, &d->Mljp, &d->Mljm, &d->RHS, &d->TsorStart,
                   &d->pdens, &d->pvrad, &d->pvtheta, &d->psize, &d->tau, &d->paccr, &d->pacct, &d->gaccr,
                   &d->gacct, &d->etafc, &d->etacc, &d->macc, &d->dragr, &d->dragt};
  for (size_t k = 0; k < sizeof(v2) / sizeof(v2[0]); k++) *v2[k] = grid(d);
  d->OmegaFrame = p->omega_frame;
  d->dt_stellar = 1.0e38;                                  /* global.h:47 */
  d->MassTaper = 1.0;                                      /* ReboundInterface.c:199 */
  d->SQRT_ADIABIND_INV = 1.0 / sqrt(p->adiabind);          /* SourceEuler.c:136 */
  d->pebbulkdens = p->pebble_bulk_dens / RHO2CGS;           /* Pebbles.c:54 */
  d->CV = GASCONST / (MOLWEIGHT * (p->adiabind - 1.0));   /* EnergySources.c:69 */
  d->sor_first = 1; d->jchess1st = 0; d->jchess2nd = 1;
  d->Rstar = p->stellar_radius * 6.957e8 / AU_SI;
  d->heatsrc_max = 0;
  for (int k = 0; k < THORIN_MAXPLANETS; k++) d->heatsrc_index[k] = -1;
  FillPolar1DArrays(d);
  InitComputeAccel(d);
  return d;
}

void ora_destroy(ora_disk *d) { (void)d; /* process-lifetime test object */ }

/* InitEuler (SourceEuler.c:133-175) plus EquilPebbleDisk (Pebbles.c:58-63)
 * and the ComputeSoundSpeed of main.c:168-170. */
void ora_init_default(ora_disk *d)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  for (int i = 0; i < nr; i++) {                           /* FillSigma, Theo.c:25 */
    d->SigmaMed[i] = SigmaProfile(d, d->Rmed[i]);
    d->SigmaInf[i] = SigmaProfile(d, d->Rinf[i]);
  }
  for (int i = 0; i < nr; i++) d->EnergyMed[i] = EnergyProfile(d, d->Rmed[i]);   /* Theo.c:76 */
  for (int i = 0; i < nr; i++)                              /* Pframeforce.c:620-642 */
    for (int j = 0; j < ns; j++) { d->rho[j + i * ns] = d->SigmaMed[i]; d->energy[j + i * ns] = d->EnergyMed[i]; }
  ComputeSoundSpeed(d, d->rho, d->energy);
  ComputePressureField(d, d->rho, d->energy);
  ComputeTemperatureField(d, d->rho, d->energy);
  InitGasVelocity(d);
  for (int i = 0; i <= nr; i++)                               /* InitLabel, Init.c:59-72 */
    for (int j = 0; j < ns; j++) d->label[j + i * ns] = (d->Rmed[i] - p->rmin) / (p->rmax - p->rmin);
  if (p->damp_init) FillVtheta(d);
  if (p->damping || p->pebbles) SetWaveKillingZones(d);
  if (p->pebbles) { EtaPressureSupport(d); InitPebblesViaFlux(d); }
  if (p->energy_eq) ComputeSoundSpeed(d, d->rho, d->energy);
}

/* After fields were set from files (Init.c:81-136): flags bit 0 redoes
 * RefillSigma/RefillEnergy/FillVtheta (Theo.c:33-151, InitializeFromFile
 * path), bit 1 redoes BckpFieldsForBC (Pebbles.c:208, pebble restart path);
 * then the EOS refresh of Init.c:131-133 and main.c:168-170. */
void ora_refresh(ora_disk *d, int flags)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  if (flags & 1) {
    for (int i = 0; i < nr; i++) {                          /* RefillSigma, Theo.c:33 */
      double moy = 0.0;
      for (int j = 0; j < ns; j++) moy += d->rho[j + i * ns];
      d->SigmaMed[i] = moy / (double)ns;
    }
    d->SigmaInf[0] = d->SigmaMed[0];
    for (int i = 1; i < nr; i++)
      d->SigmaInf[i] = (d->SigmaMed[i - 1] * (d->Rmed[i] - d->Rinf[i]) + d->SigmaMed[i] * (d->Rinf[i] - d->Rmed[i - 1])) / (d->Rmed[i] - d->Rmed[i - 1]);
    if (p->energy_eq)
      for (int i = 0; i < nr; i++) {                        /* RefillEnergy, Theo.c:82 */
        double moy = 0.0;
        for (int j = 0; j < ns; j++) moy += d->energy[j + i * ns];
        d->EnergyMed[i] = moy / (double)ns;
      }
    if (p->damp_init) FillVtheta(d);
  }
  if ((flags & 2) && p->pebbles) BckpFieldsForBC(d);
  ComputeSoundSpeed(d, d->rho, d->energy);
  ComputePressureField(d, d->rho, d->energy);
  ComputeTemperatureField(d, d->rho, d->energy);
  if (p->energy_eq) ComputeSoundSpeed(d, d->rho, d->energy);
}

double *ora_field(ora_disk *d, int id)
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
  case THORIN_PRESSURE: return d->press;
  case THORIN_STOKES: return d->tau;
  case THORIN_QPLUS: return d->qplus;
  case THORIN_DIVV: return d->divv;
  case THORIN_OPACITY: return d->opacity;
  case THORIN_QMINUS: return d->qminus;
  case THORIN_LABEL: return d->label;
  }
  return NULL;
}

double *ora_profile(ora_disk *d, int id)
{
  switch (id) {
  case THORIN_SIGMAMED: return d->SigmaMed;
  case THORIN_SIGMAINF: return d->SigmaInf;
  case THORIN_ENERGYMED: return d->EnergyMed;
  case THORIN_VTHETAMED: return d->VthetaMed;
  case THORIN_PEBDENSINIT: return d->PebDensInit;
  case THORIN_PEBVRADINIT: return d->PebVradInit;
  case THORIN_PEBVTHETAINIT: return d->PebVthetaInit;
  }
  return NULL;
}

double *ora_radii(ora_disk *d) { return d->Radii; }
int *ora_nshift(ora_disk *d) { return d->NshiftGas; }

/* The last SOR system: 0..5 = Ml, Mlip, Mlim, Mljp, Mljm, RHS; 6 = the
 * temperature the solve started from.  Rows 1..nr-2 are the unknowns. */
double *ora_sor_array(ora_disk *d, int k)
{
  double *a[] = {d->Ml, d->Mlip, d->Mlim, d->Mljp, d->Mljm, d->RHS, d->TsorStart};
  return (k >= 0 && k < 7) ? a[k] : NULL;
}
double ora_sor_omega(ora_disk *d) { return d->omega; }
void ora_set_time(ora_disk *d, double t) { d->PhysicalTime = t; d->PhysicalTimeInitial = t; }
void ora_get_stats(ora_disk *d, thorin_stats *s)
{
  *s = d->st;
  s->physical_time = d->PhysicalTime;
  s->omega_frame = d->OmegaFrame;
}

/* ------------------------------------------------------------------ */
/* Boundaries: SideEuler.c                                              */
static void DampingBoundary(ora_disk *d, double step)       /* SideEuler.c:368-419 */
{
  const thorin_params *p = &d->p;
  double DRin = p->rmin * p->damping_rmin_frac, DRout = p->rmax * p->damping_rmax_frac;
  OMP_FOR
  for (int i = 0; i < d->nr; i++) {
    if (d->Rmed[i] < DRin || d->Rmed[i] > DRout) {
      double vrad0 = 0.0, vtheta0 = 0.0, rho0 = 0.0, energy0 = 0.0, lambda;
      if (p->damp_init) { rho0 = d->SigmaMed[i]; energy0 = d->EnergyMed[i]; vtheta0 = d->VthetaMed[i] - d->Rmed[i] * d->OmegaFrame; }
      if (p->damp_flux) { vrad0 = -p->gasflux / (2.0 * PI * d->Rinf[i] * d->SigmaInf[i]); rho0 = d->SigmaMed[i]; }
      lambda = d->WaveKiller[i] * step;
      for (int j = 0; j < d->ns; j++) {
        int l = j + i * d->ns;
        d->vrad[l] = (d->vrad[l] + lambda * vrad0) / (1.0 + lambda);
        if (p->damp_init) {
          d->rho[l] = (d->rho[l] + lambda * rho0) / (1.0 + lambda);
          d->vtheta[l] = (d->vtheta[l] + lambda * vtheta0) / (1.0 + lambda);
          if (p->energy_eq) d->energy[l] = (d->energy[l] + lambda * energy0) / (1.0 + lambda);
        }
        if (p->damp_flux) d->rho[l] = (d->rho[l] + lambda * rho0) / (1.0 + lambda);
      }
    }
  }
}

#define DENSITYFLOOR 1.0e-16                                /* SideEuler.c:15-16 */
#define ENERGYFLOOR 1.0e-16

static void OpenInnerBoundary(ora_disk *d)                 /* SideEuler.c:133-178 */
{
  const thorin_params *p = &d->p;
  int ns = d->ns, i = 1;
  double *rho = d->rho, *vr = d->vrad, *energy = d->energy;
  for (int j = 0; j < ns; j++) {
    int l = j + i * ns;
    double a = rho[l] + (rho[l] - rho[l + ns]);
    rho[l - ns] = (a > DENSITYFLOOR) ? a : DENSITYFLOOR;
    if (p->energy_eq) {
      double b = energy[l] + (energy[l] - energy[l + ns]);
      energy[l - ns] = (b > ENERGYFLOOR) ? b : ENERGYFLOOR;
    }
    if (vr[l + ns] > 0.0) { vr[l] = 0.0; vr[l - ns] = 0.0; }
    else { vr[l] = vr[l + ns]; vr[l - ns] = vr[l]; }
    if (p->damp_flux) {
      double rhoinf = 0.5 * (rho[l] + rho[l - ns]);
      vr[l] = -p->gasflux / (2.0 * PI * d->Rinf[i] * rhoinf);
      rhoinf = rho[l - ns] - 0.5 * (rho[l] - rho[l - ns]);
      vr[l - ns] = -p->gasflux / (2.0 * PI * d->Rinf[i - 1] * rhoinf);
    }
  }
}

static void OpenOuterBoundary(ora_disk *d)                 /* SideEuler.c:193-232 */
{
  const thorin_params *p = &d->p;
  int ns = d->ns, i = d->nr - 1;
  double *rho = d->rho, *vr = d->vrad, *energy = d->energy;
  for (int j = 0; j < ns; j++) {
    int l = j + i * ns;
    rho[l + ns] = rho[l] + (rho[l] - rho[l - ns]);
    if (p->energy_eq) energy[l + ns] = energy[l] + (energy[l] - energy[l - ns]);
    if (vr[l] > 0.0) { vr[l] = 0.0; vr[l + ns] = 0.0; }
    else { vr[l] = vr[l - ns]; vr[l + ns] = vr[l]; }
    if (p->damp_flux) {
      double rhoinf = 0.5 * (rho[l] + rho[l + ns]);
      vr[l + ns] = -p->gasflux / (2.0 * PI * d->Rinf[i + 1] * rhoinf);
      rhoinf = rho[l + ns] + 0.5 * (rho[l + ns] - rho[l]);
      vr[l + 2 * ns] = -p->gasflux / (2.0 * PI * d->Rsup[i + 1] * rhoinf);
    }
  }
}

static void NonReflectingBoundary(ora_disk *d)             /* SideEuler.c:234-337 */
{
  int ns = d->ns, nr = d->nr;
  double *rho = d->rho, *vr = d->vrad, *energy = d->energy, *cs = d->cs;
  double csin = 0.0, csout = 0.0, dangle, mean;
  int i, i_angle;
  for (int j = 0; j < ns; j++) { csin += cs[j]; csout += cs[ns + j]; }
  csin /= (double)ns;
  csout /= (double)ns;
  i = 1;
  dangle = (pow(d->Rinf[1], -1.5) - 1.0) / (.5 * (csin + csout));
  dangle *= (d->Rmed[1] - d->Rmed[0]);
  i_angle = (int)(dangle / 2.0 / PI * (double)ns + .5);
  for (int j = 0; j < ns; j++) {
    int l = j + i * ns, jp = j + i_angle;
    if (jp >= ns) jp -= ns;
    if (jp < 0) jp += ns;
    int lp = jp;
    rho[lp] = rho[l];
    energy[lp] = energy[l];
    double vr_med = -cs[l] * (rho[l] - d->SigmaMed[1]) / d->SigmaMed[1];
    vr[l] = 2. * vr_med - vr[l + ns];
  }
  mean = 0.0;
  for (int j = 0; j < ns; j++) mean += rho[j];
  mean /= (double)ns;
  for (int j = 0; j < ns; j++) rho[j] += d->SigmaMed[0] - mean;
  mean = 0.0;
  for (int j = 0; j < ns; j++) mean += energy[j];
  mean /= (double)ns;
  for (int j = 0; j < ns; j++) energy[j] += d->EnergyMed[0] - mean;
  csin = 0.0;
  csout = 0.0;
  for (int j = 0; j < ns; j++) { csin += cs[(nr - 2) * ns + j]; csout += cs[(nr - 1) * ns + j]; }
  csin /= (double)ns;
  csout /= (double)ns;
  i = nr - 1;
  dangle = (pow(d->Rinf[nr - 2], -1.5) - 1.0) / (.5 * (csin + csout));
  dangle *= (d->Rmed[nr - 1] - d->Rmed[nr - 2]);
  i_angle = (int)(dangle / 2.0 / PI * (double)ns + .5);
  for (int j = 0; j < ns; j++) {
    int l = j + i * ns, jp = j - i_angle;
    if (jp >= ns) jp -= ns;
    if (jp < 0) jp += ns;
    int lp = jp + (i - 1) * ns;
    rho[l] = rho[lp];
    energy[l] = energy[lp];
    double vr_med = cs[l] * (rho[l - ns] - d->SigmaMed[nr - 2]) / d->SigmaMed[nr - 2];
    vr[l] = 2. * vr_med - vr[l - ns];
  }
  mean = 0.0;
  for (int j = 0; j < ns; j++) mean += rho[j + ns * (nr - 1)];
  mean /= (double)ns;
  for (int j = 0; j < ns; j++) rho[j + (nr - 1) * ns] += d->SigmaMed[nr - 1] - mean;
  mean = 0.0;
  for (int j = 0; j < ns; j++) mean += energy[j + ns * (nr - 1)];
  mean /= (double)ns;
  for (int j = 0; j < ns; j++) energy[j + (nr - 1) * ns] += d->EnergyMed[nr - 1] - mean;
}

static void ApplyOuterSourceMass(ora_disk *d)              /* SideEuler.c:458-486 */
{
  const thorin_params *p = &d->p;
  int ns = d->ns, nr = d->nr, i = nr - 1;
  double average_rho = 0.0, penul_vr;
  for (int j = 0; j < ns; j++) average_rho += d->rho[j + i * ns];
  average_rho /= (double)ns;
  average_rho = d->SigmaMed[nr - 1] - average_rho;
  for (int j = 0; j < ns; j++) d->rho[j + i * ns] += average_rho;
  penul_vr = p->imposed_disk_drift * pow((d->Rinf[nr - 1] / 1.0), -p->sigma_slope);
  for (int j = 0; j < ns; j++) d->vrad[j + i * ns] = penul_vr;
}

static void ApplyBoundaryCondition(ora_disk *d, double dt)  /* SideEuler.c:490-503 */
{
  const thorin_params *p = &d->p;
  if (p->open_inner) OpenInnerBoundary(d);
  if (p->open_outer) OpenOuterBoundary(d);
  if (p->non_reflecting) {
    if (p->energy_eq) ComputeSoundSpeed(d, d->rho, d->energy);
    NonReflectingBoundary(d);
  }
  if (p->outer_source_mass) ApplyOuterSourceMass(d);
  if (p->damping) DampingBoundary(d, dt);
}

static void DampPebbles(ora_disk *d, double dt)             /* SideEuler.c:423-456 */
{
  const thorin_params *p = &d->p;
  double DRin = p->rmin * p->damping_rmin_frac, DRout = p->rmax * p->damping_rmax_frac;
  OMP_FOR
  for (int i = 0; i < d->nr; i++) {
    if (d->Rmed[i] < DRin || d->Rmed[i] > DRout) {
      double lambda = d->WaveKiller[i] * dt;
      double pdens0 = d->PebDensInit[i], pvr0 = d->PebVradInit[i], pvt0 = d->PebVthetaInit[i] - d->Rmed[i] * d->OmegaFrame;
      for (int j = 0; j < d->ns; j++) {
        int l = j + i * d->ns;
        d->pdens[l] = (d->pdens[l] + lambda * pdens0) / (1.0 + lambda);
        d->pvrad[l] = (d->pvrad[l] + lambda * pvr0) / (1.0 + lambda);
        d->pvtheta[l] = (d->pvtheta[l] + lambda * pvt0) / (1.0 + lambda);
      }
    }
  }
}

static int DetectCrash(const ora_disk *d, const double *f)  /* SourceEuler.c:48-66 */
{
  int bad = 0;
  for (int l = 0; l < d->nr * d->ns; l++) if (f[l] < 0.0) bad = 1;
  return bad;
}

/* ------------------------------------------------------------------ */
/* CFL: SourceEuler.c:589-712, Pebbles.c:729-767                        */
static void CriticalCharTime(ora_disk *d)
{
  int ns = d->ns;
  double mx = -1.e30;
#ifdef _OPENMP
#pragma omp parallel for reduction(max : mx)
#endif
  for (int i = 1; i < d->nr; i++) {
    double dxrad = d->Rsup[i] - d->Rinf[i], dxtheta = d->Rmed[i] * 2.0 * PI / (double)ns, pvtmed = 0.0;
    if (d->p.fast_transport) {
      for (int j = 0; j < ns; j++) pvtmed += d->pvtheta[j + i * ns];
      pvtmed /= (double)ns;
    }
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      double invdt1 = fabs(d->pvrad[l]) / dxrad;
      double vres = d->p.fast_transport ? d->pvtheta[l] - pvtmed : d->pvtheta[l];
      double invdt2 = fabs(vres) / dxtheta;
      double invdt3 = fabs(d->pvrad[l] - d->vrad[l]) / dxrad;
      double invdt4 = fabs(d->pvtheta[l] - d->vtheta[l]) / dxtheta;
      double temp = invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 + invdt4 * invdt4;
      if (temp > mx) mx = temp;   /* max2 */
    }
  }
  d->invdtpeb_sq = mx;
}

static int ConditionCFL(ora_disk *d, double deltaT)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  double newdt = 1e30;
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double s = 0.0;
    for (int j = 0; j < ns; j++) s += d->vtheta[j + i * ns];
    d->Vmoy[i] = s / (double)ns;
  }
#ifdef _OPENMP
#pragma omp parallel for reduction(min : newdt)
#endif
  for (int i = 1; i < nr; i++) {
    double dxrad = d->Rsup[i] - d->Rinf[i], dxtheta = d->Rmed[i] * 2.0 * PI / (double)ns, invdt5 = 1e-30;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      double cs = d->cs[l], mindx = (dxtheta < dxrad) ? dxtheta : dxrad;   /* min2(dxrad,dxtheta) */
      double invdt1 = cs / mindx;
      double invdt2 = fabs(d->vrad[l]) / dxrad;
      double invdt3 = fabs(p->fast_transport ? d->vtheta[l] - d->Vmoy[i] : d->vtheta[l]) / dxtheta;
      double dvr = d->vrad[lip] - d->vrad[l], dvt = d->vtheta[ljp] - d->vtheta[l], invdt4, dt;
      if (dvr >= 0.0) dvr = 1e-10; else dvr = -dvr;
      if (dvt >= 0.0) dvt = 1e-10; else dvt = -dvt;
      invdt4 = (dvt / dxtheta > dvr / dxrad) ? dvt / dxtheta : dvr / dxrad;   /* max2 */
      invdt4 *= 4.0 * CVNR * CVNR;
      if (p->viscosity_alpha || (p->viscosity != 0.0)) invdt5 = FViscosity(d, d->Rmed[i]) * 4. / pow(mindx, 2);
      if (!p->pebbles)
        dt = CFLSECURITY / sqrt(invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 + invdt4 * invdt4 + invdt5 * invdt5 + d->invdtreb_sq);
      else
        dt = CFLSECURITY / sqrt(invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 + invdt4 * invdt4 + invdt5 * invdt5 + d->invdtpeb_sq + d->invdtreb_sq);
      if (dt < newdt) newdt = dt;
    }
  }
  for (int i = 0; i < nr - 1; i++) {
    double dt = 2.0 * PI * CFLSECURITY / (double)ns / fabs(d->Vmoy[i] * d->InvRmed[i] - d->Vmoy[i + 1] * d->InvRmed[i + 1]);
    if (dt < newdt) newdt = dt;
  }
  if (newdt > d->dt_stellar) {
    double m = (1.0 * d->dt_stellar > p->minimum_step) ? 1.0 * d->dt_stellar : p->minimum_step;
    newdt = (newdt < m) ? newdt : m;
  }
  newdt = (newdt < p->maximum_step) ? newdt : p->maximum_step;
  if (d->cfl_count == 0) { if (p->first_step > 0.0) newdt = p->first_step; d->cfl_count = 1; }
  if (deltaT < newdt) newdt = deltaT;
  return (int)(ceil(deltaT / newdt));
}

/* ------------------------------------------------------------------ */
/* Viscosity: Viscosity.c:85-260                                        */
static void UpdateDivVelocAndStressTensor(ora_disk *d, const double *vr, const double *vt, const double *rho)
{
  int nr = d->nr, ns = d->ns;
  double dphi = 2.0 * M_PI / (double)ns, invdphi = 1.0 / dphi, onethird = 1.0 / 3.0;
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      d->Drr[l] = (vr[lip] - vr[l]) * d->InvDiffRsup[i];
      d->Dpp[l] = (vt[ljp] - vt[l]) * invdphi * d->InvRmed[i] + 0.5 * (vr[lip] + vr[l]) * d->InvRmed[i];
      d->divv[l] = (vr[lip] * d->Rsup[i] - vr[l] * d->Rinf[i]) * d->InvDiffRsup[i] * d->InvRmed[i];
      d->divv[l] += (vt[ljp] - vt[l]) * invdphi * d->InvRmed[i];
    }
  OMP_FOR
  for (int i = 1; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1, lim = l - ns;
      d->Drp[l] = 0.5 * (d->Rinf[i] * (vt[l] * d->InvRmed[i] - vt[lim] * d->InvRmed[i - 1]) * d->InvDiffRmed[i] +
                         (vr[l] - vr[ljm]) * invdphi * d->InvRinf[i]);
    }
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double viscosity = FViscosity(d, d->Rmed[i]);
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      d->Trr[l] = 2.0 * rho[l] * viscosity * (d->Drr[l] - onethird * d->divv[l]);
      d->Tpp[l] = 2.0 * rho[l] * viscosity * (d->Dpp[l] - onethird * d->divv[l]);
    }
  }
  OMP_FOR
  for (int i = 1; i < nr; i++) {
    double viscosity = FViscosity(d, d->Rinf[i]);
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1, ljmim = ljm - ns;
      d->Trp[l] = 2.0 * 0.25 * (rho[l] + rho[lim] + rho[ljm] + rho[ljmim]) * viscosity * d->Drp[l];
    }
  }
}

static void UpdateVelocityWithViscousTerms(ora_disk *d, double *vr, double *vt, const double *rho, double DeltaT)
{
  int nr = d->nr, ns = d->ns;
  double invdphi = 1.0 / (2.0 * M_PI / (double)ns);
  OMP_FOR
  for (int i = 1; i < nr - 1; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      vt[l] += DeltaT * d->InvRmed[i] * ((d->Rsup[i] * d->Trp[lip] - d->Rinf[i] * d->Trp[l]) * d->InvDiffRsup[i] +
                                         (d->Tpp[l] - d->Tpp[ljm]) * invdphi + 0.5 * (d->Trp[l] + d->Trp[lip])) /
               (0.5 * (rho[l] + rho[ljm]));
    }
  OMP_FOR
  for (int i = 1; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      vr[l] += DeltaT * d->InvRinf[i] * ((d->Rmed[i] * d->Trr[l] - d->Rmed[i - 1] * d->Trr[lim]) * d->InvDiffRmed[i] +
                                         (d->Trp[ljp] - d->Trp[l]) * invdphi - 0.5 * (d->Tpp[l] + d->Tpp[lim])) /
               (0.5 * (rho[l] + rho[lim]));
    }
}

static void ImposeKeplerianEdges(ora_disk *d, double *vt)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  double VKepIn = sqrt(G * 1.0 / d->Rmed[0]) * sqrt(1.0 - pow(AspectRatio(d, d->Rmed[0]), 2.0) * pow(d->Rmed[0], 2.0 * p->flaring_index) * (1. + p->sigma_slope - 2.0 * p->flaring_index));
  double VKepOut = sqrt(G * 1.0 / d->Rmed[nr - 1]) * sqrt(1.0 - pow(AspectRatio(d, d->Rmed[nr - 1]), 2.0) * pow(d->Rmed[nr - 1], 2.0 * p->flaring_index) * (1. + p->sigma_slope - 2.0 * p->flaring_index));
  for (int j = 0; j < ns; j++) vt[j] = VKepIn - d->Rmed[0] * d->OmegaFrame;
  for (int j = 0; j < ns; j++) vt[j + (nr - 1) * ns] = VKepOut - d->Rmed[nr - 1] * d->OmegaFrame;
}

/* ------------------------------------------------------------------ */
/* Source substeps: SourceEuler.c:319-586                               */
static void SubStep1(ora_disk *d, double dt)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  const double *rho = d->rho, *vrad = d->vrad, *vtheta = d->vtheta, *press = d->press;
  OMP_FOR
  for (int i = 1; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      double gradp = (press[l] - press[lim]) * 2.0 / (rho[l] + rho[lim]) * d->InvDiffRmed[i];
      double vt2 = vtheta[l] + vtheta[ljp] + vtheta[lim] + vtheta[ljp - ns];
      vt2 = vt2 / 4.0 + d->Rinf[i] * d->OmegaFrame;
      vt2 = vt2 * vt2;
      double tmp = -gradp + 0.5 * (d->agr[l] + d->agr[lim]) + vt2 * d->InvRinf[i];
      d->VradInt[l] = vrad[l] + dt * tmp;
      if (p->pebbles) {
        d->gaccr[l] = tmp;
        if (p->back_reaction) {
          tmp = d->dragr[l] * 2.0 / (rho[l] + rho[lim]);
          d->VradInt[l] += dt * tmp;
          d->gaccr[l] += tmp;
        }
      }
    }
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double supp_torque = p->imposed_disk_drift * .5 * pow(d->Rmed[i], -2.5 + p->sigma_slope);
    double dxtheta = 2.0 * PI / (double)ns * d->Rmed[i], invdxtheta = 1.0 / dxtheta;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      double gradp = (press[l] - press[ljm]) * 2.0 / (rho[l] + rho[ljm]) * invdxtheta;
      double tmp = -gradp + 0.5 * (d->agt[l] + d->agt[ljm]);
      d->VthetaInt[l] = vtheta[l] + dt * tmp;
      d->VthetaInt[l] += dt * supp_torque;
      if (p->pebbles) {
        d->gacct[l] = tmp + supp_torque;
        if (p->back_reaction) {
          tmp = d->dragt[l] * 2.0 / (rho[l] + rho[ljm]);
          d->VthetaInt[l] += dt * tmp;
          d->gacct[l] += tmp;
        }
      }
    }
  }
  UpdateDivVelocAndStressTensor(d, d->VradInt, d->VthetaInt, rho);
  UpdateVelocityWithViscousTerms(d, d->VradInt, d->VthetaInt, rho, dt);
  if ((!p->damping) || (p->damping && p->damp_vrad)) ImposeKeplerianEdges(d, d->VthetaInt);
}

static void SubStep2(ora_disk *d, double dt)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  const double *rho = d->rho, *vrad = d->VradInt, *vtheta = d->VthetaInt;
  double *qr = d->RhoInt, *qt = d->TemperInt;
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      double dv = vrad[lip] - vrad[l];
      qr[l] = (dv < 0.0) ? CVNR * CVNR * rho[l] * dv * dv : 0.0;
      dv = vtheta[ljp] - vtheta[l];
      qt[l] = (dv < 0.0) ? CVNR * CVNR * rho[l] * dv * dv : 0.0;
    }
  OMP_FOR
  for (int i = 1; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns;
      d->VradNew[l] = vrad[l] - dt * 2.0 / (rho[l] + rho[lim]) * (qr[l] - qr[lim]) * d->InvDiffRmed[i];
    }
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double dxtheta = 2.0 * PI / (double)ns * d->Rmed[i], invdxtheta = 1.0 / dxtheta;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      d->VthetaNew[l] = vtheta[l] - dt * 2.0 / (rho[l] + rho[ljm]) * (qt[l] - qt[ljm]) * invdxtheta;
    }
  }
  if (p->energy_eq)
    for (int i = 0; i < nr; i++) {
      double dxtheta = 2.0 * PI / (double)ns * d->Rmed[i], invdxtheta = 1.0 / dxtheta;
      for (int j = 0; j < ns; j++) {
        int l = j + i * ns, lip = l + ns, ljp = (j == ns - 1) ? i * ns : l + 1;
        d->EnergyInt[l] = d->energy[l] - dt * qr[l] * (vrad[lip] - vrad[l]) * d->InvDiffRsup[i] -
                          dt * qt[l] * (vtheta[ljp] - vtheta[l]) * invdxtheta;
      }
    }
}

static void ActualiseGas(const ora_disk *d, double *dst, const double *src)   /* SourceEuler.c:192-208 */
{
  memcpy(dst, src, sizeof(double) * (size_t)(d->nr + 1) * (size_t)d->ns);
}

/* ------------------------------------------------------------------ */
/* Energy sources and SOR: EnergySources.c                              */
static double FluxLimiterValue(double s)                    /* EnergySources.c:684-696 */
{
  if (s <= 2.0) return 2.0 / (3.0 + sqrt(9.0 + 10.0 * s * s));
  return 10.0 / (10.0 * s + 9.0 + sqrt(81.0 + 180.0 * s));
}

static double EffectiveOpticalDepth(const ora_disk *d, double tau)   /* EnergySources.c:701-711 */
{
  if (d->p.stellar_irradiation) return 0.375 * tau + 0.5 + 0.25 / tau;
  return 0.375 * tau + 0.25 * sqrt(3.0) + 0.25 / tau;
}

static void MidplaneVolumeDensity(ora_disk *d)              /* EnergySources.c:658-680 */
{
  OMP_FOR
  for (int i = 0; i < d->nr; i++)
    for (int j = 0; j < d->ns; j++) {
      int l = j + i * d->ns;
      double H = d->cs[l] * d->OmegaInv[i] * d->SQRT_ADIABIND_INV;
      d->voldens[l] = d->rho[l] / H * SQRT2PI_INV;
    }
}

static void OpacityProfile(ora_disk *d)                     /* Opacity.c:231-266 */
{
  if (d->p.parametric_opacity > 0.0) {
    double tmp = d->p.parametric_opacity * OPA2CU;
    for (int l = 0; l < d->nr * d->ns; l++) d->opacity[l] = tmp;
    return;
  }
  OMP_FOR
  for (int l = 0; l < d->nr * d->ns; l++)
    d->opacity[l] = opacity_func(d, d->voldens[l] * RHO2CGS, d->temper[l] * T2SI) * OPA2CU;
}

static void CalculateQminus(ora_disk *d)                    /* EnergySources.c:75-99 */
{
  OMP_FOR
  for (int l = 0; l < d->nr * d->ns; l++) {
    double tau = d->p.opacity_drop * 0.5 * d->opacity[l] * d->rho[l];
    double taueff = EffectiveOpticalDepth(d, tau);
    d->qminus[l] = 2.0 * STEFANBOLTZMANN * pow(d->temper[l], 3.0) / taueff;
  }
}

static void CalculateFlaring(ora_disk *d)                   /* EnergySources.c:146-198 */
{
  int nr = d->nr, ns = d->ns;
  double *cs = d->cs, *fl = d->flaring, Rstar = d->Rstar;
  OMP_FOR
  for (int i = 1; i < nr - 1; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, lim = l - ns;
      double csin = 0.5 * (cs[l] + cs[lim]), csout = 0.5 * (cs[l] + cs[lip]);
      double Hin = csin * pow(d->Rinf[i], 1.5) * d->SQRT_ADIABIND_INV;
      double Hout = csout * pow(d->Rsup[i], 1.5) * d->SQRT_ADIABIND_INV;
      double dHdr = (Hout - Hin) * d->InvDiffRsup[i];
      double H = cs[l] * d->OmegaInv[i] * d->SQRT_ADIABIND_INV;
      fl[l] = atan(dHdr) - atan((H - 0.4 * Rstar) * d->InvRmed[i]);
      fl[l] = (fl[l] >= 0.0) ? sin(fl[l]) : 0.0;
      if (i == 1) {
        H = cs[lim] * d->OmegaInv[i - 1] * d->SQRT_ADIABIND_INV;
        fl[lim] = atan(dHdr) - atan((H - 0.4 * Rstar) / d->Rmed[i - 1]);
        fl[lim] = (fl[lim] >= 0.0) ? sin(fl[lim]) : 0.0;
      }
      if (i == nr - 2) {
        H = cs[lip] * d->OmegaInv[i + 1] * d->SQRT_ADIABIND_INV;
        fl[lip] = atan(dHdr) - atan((H - 0.4 * Rstar) / d->Rmed[i + 1]);
        fl[lip] = (fl[lip] >= 0.0) ? sin(fl[lip]) : 0.0;
      }
    }
}

static void CalculateQirr(ora_disk *d)                      /* EnergySources.c:103-141 */
{
  const thorin_params *p = &d->p;
  if (d->Tirr4fac == 0.0) {
    double Teff4 = pow(p->effective_temperature / T2SI, 4.0);
    double Rstar2 = pow(p->stellar_radius * (6.957e8 / AU_SI), 2.0);
    d->Tirr4fac = (1.0 - p->disc_albedo) * Teff4 * Rstar2;
  }
  OMP_FOR
  for (int i = 0; i < d->nr; i++) {
    double r2inv = 1.0 / d->Rmed2[i];
    for (int j = 0; j < d->ns; j++) {
      int l = j + i * d->ns;
      if (d->flaring[l] > 0.0) {
        double tau = p->opacity_drop * 0.5 * d->opacity[l] * d->rho[l];
        double taueff = EffectiveOpticalDepth(d, tau);
        d->qirr[l] = 2.0 * STEFANBOLTZMANN * (d->Tirr4fac * r2inv * d->flaring[l]) / taueff;
      } else d->qirr[l] = 0.0;
    }
  }
}

static void TemperatureGradient(ora_disk *d)                /* EnergySources.c:609-653 */
{
  int nr = d->nr, ns = d->ns;
  const double *T = d->temper;
  OMP_FOR
  for (int i = 1; i < nr; i++) {
    double dxtheta = 2.0 * PI / (double)ns * d->Rmed[i], invdxtheta = 1.0 / dxtheta;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      d->GradTr[l] = (T[l] - T[lim]) * d->InvDiffRmed[i];
      d->GradTt[l] = (T[l] - T[ljm]) * invdxtheta;
    }
  }
  OMP_FOR
  for (int i = 1; i < nr - 1; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      double r = 0.5 * (d->GradTr[lip] + d->GradTr[l]), t = 0.5 * (d->GradTt[ljp] + d->GradTt[l]);
      d->GradTm[l] = sqrt(r * r + t * t);
    }
}

static void DiffusionCoefs(ora_disk *d)                     /* EnergySources.c:556-605 */
{
  int nr = d->nr, ns = d->ns;
  TemperatureGradient(d);
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      double gradt = (i == 0) ? d->GradTm[l + ns] : (i == nr - 1) ? d->GradTm[l - ns] : d->GradTm[l];
      double fac = 1.0 / (d->voldens[l] * d->opacity[l]);
      double s = 4.0 * gradt * fac / d->temper[l];
      d->Dcen[l] = FluxLimiterValue(s) * 16.0 * STEFANBOLTZMANN * pow(d->temper[l], 3.0) * fac;
    }
  OMP_FOR
  for (int i = 1; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      d->Dr[l] = 0.5 * (d->Dcen[l] + d->Dcen[lim]);
      d->Dt[l] = 0.5 * (d->Dcen[l] + d->Dcen[ljm]);
    }
}

static void DiffusionTimestep(ora_disk *d)                  /* EnergySources.c:833-856 */
{
  double dtmin = 1.0e38;
#ifdef _OPENMP
#pragma omp parallel for reduction(min : dtmin)
#endif
  for (int i = 0; i < d->nr; i++) {
    double dr2 = d->Rsup[i] - d->Rinf[i];
    dr2 = dr2 * dr2 / 2.0;
    for (int j = 0; j < d->ns; j++) {
      double dttmp = dr2 / d->Dcen[j + i * d->ns];
      if (dttmp < dtmin) dtmin = dttmp;
    }
  }
  d->dt_stellar = dtmin;
}

/* SuccessiveOverrelaxation, EnergySources.c:406-511 (sequential build). */
static int SuccessiveOverrelaxation(ora_disk *d, double omega, int *maxed)
{
  int nr = d->nr, ns = d->ns, n;
  double *T = d->temper, normres0 = 0.0, normres = 0.0;
  const double *Ml = d->Ml, *Mlip = d->Mlip, *Mlim = d->Mlim, *Mljp = d->Mljp, *Mljm = d->Mljm, *RHS = d->RHS;
  *maxed = 0;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : normres0)
#endif
  for (int i = 1; i < nr - 1; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, lim = l - ns, ljp = (j == ns - 1) ? i * ns : l + 1, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      double resid = T[l] * Ml[l] + T[lip] * Mlip[l] + T[lim] * Mlim[l] + T[ljp] * Mljp[l] + T[ljm] * Mljm[l] - RHS[l];
      normres0 += fabs(resid);
    }
  for (n = 1; n <= d->p.sor_maxiters; n++) {
    int changed = 0;
    normres = 0.0;
    for (int ipass = 1; ipass <= 2; ipass++) {
      const int jstart = (ipass == 1) ? d->jchess1st : d->jchess2nd;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : normres, changed)
#endif
      for (int i = 1; i < nr - 1; i++) {
        const int jchess = jstart ^ ((i - 1) & 1);   /* flips every ring */
        for (int j = jchess; j < ns; j += 2) {
          int l = j + i * ns, lip = l + ns, lim = l - ns, ljp = (j == ns - 1) ? i * ns : l + 1, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
          double resid = T[l] * Ml[l] + T[lip] * Mlip[l] + T[lim] * Mlim[l] + T[ljp] * Mljp[l] + T[ljm] * Mljm[l] - RHS[l];
          normres += fabs(resid);
          double delta = omega * resid / Ml[l];
          T[l] -= delta;
          if (delta > T[l] * SORPRECISION) changed++;
        }
      }
    }
    if (normres < d->p.sor_eps * normres0) return n;
    if (normres < SORMIN) return n;
    if (changed == 0) return n;
  }
  *maxed = 1;
  return n;
}

/* IterateRelaxationParameter, EnergySources.c:340-403.  Returns 0, or -1
 * when no omega converged (the reference then exits). */
static int IterateRelaxationParameter(ora_disk *d)
{
  int nr = d->nr, ns = d->ns, nsplit = 9, Niter, count = 0, maxed;
  double omegamin = 1.0, omega = 1.0, omegamax = OMEGAUPPER;
  size_t bytes = sizeof(double) * (size_t)nr * (size_t)ns;
  double *bk = (double *)malloc(bytes);
  memcpy(bk, d->temper, bytes);
  d->domega = (omegamax - omegamin) / nsplit;
  d->Niterbest = d->p.sor_maxiters;
  d->omegabest = 1.0;
  for (;;) {
    for (int n = 0; n <= nsplit; n++) {
      Niter = SuccessiveOverrelaxation(d, omega, &maxed);
      d->st.sor_sweeps += Niter;
      if (Niter == d->Niterbest) count++;
      if (Niter < d->Niterbest) { d->Niterbest = Niter; d->omegabest = omega; }
      omega += d->domega;
      memcpy(d->temper, bk, bytes);
    }
    if (d->Niterbest == d->p.sor_maxiters) { free(bk); return -1; }
    if (count == nsplit + 1) { d->domega = omegamax - omegamin; free(bk); return 0; }
    count = 0;
    omegamin = d->omegabest - d->domega;
    omegamax = d->omegabest + d->domega;
    if (omegamin < 1.0) omegamin = 1.0;
    if (omegamax > OMEGAUPPER) omegamax = OMEGAUPPER;
    d->domega = (omegamax - omegamin) / nsplit;
    omega = omegamin;
  }
}

static int ImplicitRadiativeDiffusion(ora_disk *d, double dt)   /* EnergySources.c:201-335 */
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns, Niter, maxed, status = THORIN_OK;
  ComputeTemperatureField(d, d->rho, d->EnergyInt);
  ComputeSoundSpeed(d, d->rho, d->EnergyInt);
  MidplaneVolumeDensity(d);
  OpacityProfile(d);
  CalculateQminus(d);
  if (p->stellar_irradiation) { CalculateFlaring(d); CalculateQirr(d); }
  DiffusionCoefs(d);
  DiffusionTimestep(d);
  OMP_FOR
  for (int i = 1; i < nr; i++) {
    double dxtheta = 2.0 * PI / (double)ns * d->Rmed[i], invdxtheta2 = 1.0 / dxtheta / dxtheta;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      d->A[l] = d->Dr[l] * d->Rinf[i] * d->InvDiffRmed[i];
      double H = d->cs[l] * d->OmegaInv[i] * d->SQRT_ADIABIND_INV;
      d->B[l] = d->Dt[l] * invdxtheta2 * 2.0 * H;
    }
  }
  OMP_FOR
  for (int i = 1; i < nr - 1; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      double H = d->cs[l] * d->OmegaInv[i] * d->SQRT_ADIABIND_INV;
      double bfac = dt / (d->rho[l] * d->CV);
      double afac = bfac * d->InvDiffRsup[i] * 2.0 * H / d->Rmed[i];
      d->Ml[l] = 1.0 + d->divv[l] * (p->adiabind - 1.0) * dt + 4.0 * bfac * d->qminus[l] + afac * (d->A[lip] + d->A[l]) + bfac * (d->B[ljp] + d->B[l]);
      d->Mlip[l] = -afac * d->A[lip];
      d->Mlim[l] = -afac * d->A[l];
      d->Mljp[l] = -bfac * d->B[ljp];
      d->Mljm[l] = -bfac * d->B[l];
      d->RHS[l] = d->temper[l] + bfac * (d->qplus[l] + 3.0 * d->qminus[l] * d->temper[l]);
      if (p->stellar_irradiation) d->RHS[l] += bfac * d->qirr[l];
      if (p->accret_heating || p->gas_accret_heating)
        for (int k = 0; k < d->heatsrc_max; k++)
          if (l == d->heatsrc_index[k]) d->RHS[l] += bfac * d->heatsrc[k];
    }
  if (d->sor_first) {
    d->sor_first = 0;
    if (IterateRelaxationParameter(d) != 0) return THORIN_ERR_OMEGA;
    d->omega = d->omegabest;
    d->Niterlast = d->Niterbest;
  }
  d->omega += d->domega;
  if (d->omega > OMEGAUPPER) { d->omega = OMEGAUPPER; d->domega = -d->domega; }
  if (d->omega < 1.0) { d->omega = 1.0; d->domega = -d->domega; }
  memcpy(d->TsorStart, d->temper, sizeof(double) * (size_t)nr * (size_t)ns);
  Niter = SuccessiveOverrelaxation(d, d->omega, &maxed);
  if (maxed) status = THORIN_ERR_SOR_MAXIT;       /* reference only warns */
  d->st.sor_calls++; d->st.sor_sweeps += Niter; d->st.sor_last_niter = Niter; d->st.sor_omega = d->omega;
  if (Niter > d->Niterlast) d->domega = -d->domega;
  d->Niterlast = Niter;
  OMP_FOR
  for (int j = 0; j < ns; j++) d->temper[j] = d->temper[j + ns];
  OMP_FOR
  for (int j = 0; j < ns; j++) d->temper[j + (nr - 1) * ns] = d->temper[j + (nr - 2) * ns];
  OMP_FOR
  for (int l = 0; l < nr * ns; l++) d->EnergyNew[l] = d->rho[l] * d->temper[l] * d->CV;
  return status;
}

static int SubStep3(ora_disk *d, double dt)                 /* SourceEuler.c:508-586 */
{
  int nr = d->nr, ns = d->ns;
  const double *rho = d->rho;
  double r0 = d->Rmed[0], r1 = d->Rmed[1], r2 = d->Rmed[2], viscosity;
  OMP_FOR
  for (int i = 1; i < nr; i++) {
    const double viscosity = FViscosity(d, d->Rmed[i]);
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      if (viscosity != 0.0) {
        d->qplus[l] = 0.5 / viscosity / rho[l] * (d->Trr[l] * d->Trr[l] + 2.0 * d->Trp[l] * d->Trp[l] + d->Tpp[l] * d->Tpp[l]);
        d->qplus[l] += (2.0 / 9.0) * viscosity * rho[l] * d->divv[l] * d->divv[l];
      } else d->qplus[l] = 0.0;
    }
  }
  viscosity = FViscosity(d, d->Rmed[0]);
  OMP_FOR
  for (int j = 0; j < ns; j++) {
    double q1 = d->qplus[j + ns], q2 = d->qplus[j + 2 * ns];
    if (viscosity != 0.0) d->qplus[j] = q1 * exp(log(q1 / q2) * log(r0 / r1) / log(r1 / r2));
    else d->qplus[j] = 0.0;
  }
  if (d->p.parametric_cooling) {                             /* SourceEuler.c:569-582 */
    const double *energy = d->EnergyInt;
    OMP_FOR
    for (int i = 0; i < nr; i++)
      for (int j = 0; j < ns; j++) {
        int l = j + i * ns;
        double tmp1 = d->EnergyMed[i] * dt * rho[l] / d->SigmaMed[i] + d->CoolingTimeMed[i] * energy[l] +
                      dt * d->CoolingTimeMed[i] * (d->qplus[l] - d->QplusMed[i] * rho[l] / d->SigmaMed[i]);
        double tmp2 = dt + d->CoolingTimeMed[i] + (d->p.adiabind - 1.0) * dt * d->CoolingTimeMed[i] * d->divv[l];
        d->EnergyNew[l] = tmp1 / tmp2;
      }
    return THORIN_OK;
  }
  return ImplicitRadiativeDiffusion(d, dt);
}

/* ------------------------------------------------------------------ */
/* Transport: TransportEuler.c                                          */
static void ComputeLRMomenta(ora_disk *d, const double *rho, const double *vr, const double *vt)   /* :318-347 */
{
  int nr = d->nr, ns = d->ns;
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      d->RadMomP[l] = rho[l] * vr[lip];
      d->RadMomM[l] = rho[l] * vr[l];
      d->ThetaMomP[l] = rho[l] * (vt[ljp] + d->Rmed[i] * d->OmegaFrame) * d->Rmed[i];
      d->ThetaMomM[l] = rho[l] * (vt[l] + d->Rmed[i] * d->OmegaFrame) * d->Rmed[i];
    }
}

static void ComputeVelocities(ora_disk *d, const double *rho, double *vr, double *vt)   /* :350-381 */
{
  int nr = d->nr, ns = d->ns;
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      if (i == 0) vr[l] = 0.0;
      else vr[l] = (d->RadMomP[lim] + d->RadMomM[l]) / (rho[l] + rho[lim] + 1e-20);
      vt[l] = (d->ThetaMomP[ljm] + d->ThetaMomM[l]) / (rho[l] + rho[ljm] + 1e-15) / d->Rmed[i] - d->Rmed[i] * d->OmegaFrame;
    }
}

static void DivisePolarGrid(const ora_disk *d, const double *num, const double *den, double *res)   /* SideEuler.c:82-99 */
{
  /* The reference swaps Nrad/Nsec in the bounds; the covered index range is
   * l < (nsec+1)*nrad.  Only rows 0..nrad-1 are read afterwards. */
  int cnt = (d->ns + 1) * d->nr;
  OMP_FOR
  for (int l = 0; l < cnt; l++) res[l] = num[l] / (den[l] + 1e-20);
}

static void ComputeStarRad(ora_disk *d, const double *qb, const double *vr, double *qs, double dt)   /* :232-273 */
{
  int nr = d->nr, ns = d->ns;
  double *dq = d->dq;
  OMP_FOR
  for (int j = 0; j < ns; j++) {
    for (int i = 0; i < nr; i++) {
      int l = j + i * ns, lq = i + j * nr, lip = l + ns, lim = l - ns;
      if ((i == 0) || (i == nr - 1)) dq[lq] = 0.0;
      else {
        double dqm = (qb[l] - qb[lim]) * d->InvDiffRmed[i];
        double dqp = (qb[lip] - qb[l]) * d->InvDiffRmed[i + 1];
        dq[lq] = (dqp * dqm > 0.0) ? 2.0 * dqp * dqm / (dqp + dqm) : 0.0;
      }
    }
    for (int i = 1; i < nr; i++) {
      int l = j + i * ns, lq = i + j * nr, lim = l - ns;
      if (vr[l] > 0.0) qs[l] = qb[lim] + (d->Rmed[i] - d->Rmed[i - 1] - vr[l] * dt) * 0.5 * dq[lq - 1];
      else qs[l] = qb[l] - (d->Rmed[i + 1] - d->Rmed[i] + vr[l] * dt) * 0.5 * dq[lq];
    }
    qs[j] = qs[j + ns * nr] = 0.0;
  }
}

static void ComputeStarTheta(ora_disk *d, const double *qb, const double *vt, double *qs, double dt)   /* :275-316 */
{
  int nr = d->nr, ns = d->ns;
  double *dq = d->dq;
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double dxtheta = 2.0 * PI / (double)ns * d->Rmed[i], invdxtheta = 1.0 / dxtheta;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljp = (j == ns - 1) ? i * ns : l + 1, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      double dqm = qb[l] - qb[ljm], dqp = qb[ljp] - qb[l];
      dq[l] = ((dqp * dqm > 0.0) && (dqp + dqm != 0.0)) ? dqp * dqm / (dqp + dqm) * invdxtheta : 0.0;
    }
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljm = ((j == 0) ? ns - 1 : j - 1) + i * ns;
      double ksi = vt[l] * dt;
      if (ksi > 0.0) qs[l] = qb[ljm] + (dxtheta - ksi) * dq[ljm];
      else qs[l] = qb[l] - (dxtheta + ksi) * dq[l];
    }
  }
}

static void VanLeerRadial(ora_disk *d, const double *vr, double *qb, double dt)   /* :384-415 */
{
  int nr = d->nr, ns = d->ns;
  double dtheta = 2.0 * PI / (double)ns;
  DivisePolarGrid(d, qb, d->RhoInt, d->Work);
  ComputeStarRad(d, d->Work, vr, d->QRStar, dt);
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lip = l + ns;
      double varq = dt * dtheta * d->Rinf[i] * d->QRStar[l] * d->RhoStar[l] * vr[l];
      varq -= dt * dtheta * d->Rsup[i] * d->QRStar[lip] * d->RhoStar[lip] * vr[lip];
      qb[l] += varq * d->InvSurf[i];
    }
}

static void VanLeerTheta(ora_disk *d, const double *vt, double *qb, double dt)   /* :417-445 */
{
  int nr = d->nr, ns = d->ns;
  DivisePolarGrid(d, qb, d->RhoInt, d->Work);
  ComputeStarTheta(d, d->Work, vt, d->QRStar, dt);
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double dxrad = (d->Rsup[i] - d->Rinf[i]) * dt, invsurf = 1.0 / d->Surf[i];
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      double varq = dxrad * d->QRStar[l] * d->RhoStar[l] * vt[l];
      varq -= dxrad * d->QRStar[ljp] * d->RhoStar[ljp] * vt[ljp];
      qb[l] += varq * invsurf;
    }
  }
}

static void ComputeResiduals(ora_disk *d, double *vt, double dt)   /* :70-111 */
{
  int nr = d->nr, ns = d->ns;
  double invdt = 1.0 / dt, dpinvns = 2.0 * PI / (double)ns;
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double moy = 0.0;
    for (int j = 0; j < ns; j++) moy += vt[j + i * ns];
    d->VMed[i] = moy / (double)ns;
    double Ntilde = d->VMed[i] * d->InvRmed[i] * dt * (double)ns / 2.0 / PI;
    double Nround = floor(Ntilde + 0.5);
    long nitemp = (long)Nround;
    d->Nshift[i] = (int)nitemp;
    if (d->p.fast_transport) {
      double vtemp = (Ntilde - Nround) * d->Rmed[i] * invdt * dpinvns;
      for (int j = 0; j < ns; j++) { int l = j + i * ns; d->VthetaRes[l] = vt[l] - d->VMed[i]; vt[l] = vtemp; }
    } else {
      for (int j = 0; j < ns; j++) { int l = j + i * ns; d->VthetaRes[l] = vt[l]; vt[l] = 0.0; }
    }
  }
}

static void AdvectSHIFT(ora_disk *d, double *val)           /* :113-136 */
{
  int nr = d->nr, ns = d->ns;
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    for (int j = 0; j < ns; j++) {
      int ji = j - d->Nshift[i];
      while (ji < 0) ji += ns;
      while (ji >= ns) ji -= ns;
      d->TempShift[j + i * ns] = val[ji + i * ns];
    }
    for (int j = 0; j < ns; j++) val[j + i * ns] = d->TempShift[j + i * ns];
  }
}

/* Transport (TransportEuler.c:34-47) and TransportPebbles (:449-505):
 * with_energy selects the gas (energy transported) variant. */
/* Transport (TransportEuler.c:34-47): the gas with its energy and, with
 * LabelAdvection, the tracer as rho*label (ComputeExtQty, :177-195); the
 * pebbles without either. */
static void TransportFluid(ora_disk *d, double *rho, double *vr, double *vt, double *energy, double dt)
{
  double *ext = (rho == d->rho && d->p.label_advection) ? d->ExtLabel : NULL;
  ComputeLRMomenta(d, rho, vr, vt);
  if (ext)
    for (int i = 0; i < d->nr; i++)
      for (int j = 0; j < d->ns; j++) { int l = j + i * d->ns; ext[l] = rho[l] * d->label[l]; }
  /* OneWindRad */
  ComputeStarRad(d, rho, vr, d->RhoStar, dt);
  ActualiseGas(d, d->RhoInt, rho);
  VanLeerRadial(d, vr, d->RadMomP, dt);
  VanLeerRadial(d, vr, d->RadMomM, dt);
  VanLeerRadial(d, vr, d->ThetaMomP, dt);
  VanLeerRadial(d, vr, d->ThetaMomM, dt);
  if (energy) VanLeerRadial(d, vr, energy, dt);
  if (ext) VanLeerRadial(d, vr, ext, dt);
  VanLeerRadial(d, vr, rho, dt);
  /* OneWindTheta */
  ComputeResiduals(d, vt, dt);
  for (int pass = 0; pass < (d->p.fast_transport ? 2 : 1); pass++) {
    const double *v = (pass == 0) ? d->VthetaRes : vt;
    ComputeStarTheta(d, rho, v, d->RhoStar, dt);
    ActualiseGas(d, d->RhoInt, rho);
    VanLeerTheta(d, v, d->RadMomP, dt);
    VanLeerTheta(d, v, d->RadMomM, dt);
    VanLeerTheta(d, v, d->ThetaMomP, dt);
    VanLeerTheta(d, v, d->ThetaMomM, dt);
    if (energy) VanLeerTheta(d, v, energy, dt);
    if (ext) VanLeerTheta(d, v, ext, dt);
    VanLeerTheta(d, v, rho, dt);
  }
  if (d->p.fast_transport) {
    AdvectSHIFT(d, d->RadMomP);
    AdvectSHIFT(d, d->RadMomM);
    AdvectSHIFT(d, d->ThetaMomP);
    AdvectSHIFT(d, d->ThetaMomM);
    if (energy) AdvectSHIFT(d, energy);
    if (ext) AdvectSHIFT(d, ext);
    AdvectSHIFT(d, rho);
  }
  ComputeVelocities(d, rho, vr, vt);
  if (ext)                                                    /* ComputeSpeQty, TransportEuler.c:197-215 */
    for (int i = 0; i < d->nr; i++)
      for (int j = 0; j < d->ns; j++) { int l = j + i * d->ns; d->label[l] = ext[l] / rho[l]; }
}

/* ------------------------------------------------------------------ */
/* Pebbles: Pebbles.c                                                    */
static void PebbleStokesNumbers(ora_disk *d)                /* :280-300 */
{
  OMP_FOR
  for (int l = 0; l < d->nr * d->ns; l++)
    d->tau[l] = 2.0 * d->pebbulkdens * d->psize[l] / d->rho[l] * d->SQRT_ADIABIND_INV;
}

static double Trapzd(int n, double a, double b, double H2, double *integral)   /* :305-328 */
{
  if (n == 1) {
    *integral = 0.5 * (b - a) * (exp(-0.5 * a * a / H2) + exp(-0.5 * b * b / H2));
    return *integral;
  }
  int it = 1;
  for (int j = 1; j < n - 1; j++) it <<= 1;
  double iter = it, spacing = (b - a) / iter, x = a + 0.5 * spacing, sum = 0.0;
  for (int j = 1; j <= it; j++) { sum += exp(-0.5 * x * x / H2); x += spacing; }
  *integral = 0.5 * (*integral + (b - a) * sum / iter);
  return *integral;
}

static double IntegrateColumnMass(double a, double b, double Hpeb)   /* :333-349 */
{
  double integral = 0.0, iold = 0.0, H2 = Hpeb * Hpeb, state = 0.0;
  for (int n = 1; n <= TRAPEZMAX; n++) {
    integral = Trapzd(n, a, b, H2, &state);
    if (n > 5)
      if (fabs(integral - iold) < TRAPEZEPS * fabs(iold) || (integral == 0.0 && iold == 0.0)) return integral;
    iold = integral;
  }
  return NAN;   /* the reference exits here */
}

static double GetGlobalIFrac(const ora_disk *d, double r)   /* LowTasks.c:21-31 */
{
  int i = 0;
  if (r < d->GlobalRmed[0]) return 0.0;
  if (r > d->GlobalRmed[d->nr - 1]) return (double)d->nr - 1.0;
  while (d->GlobalRmed[i] <= r) i++;
  return (double)i + (r - d->GlobalRmed[i - 1]) / (d->GlobalRmed[i] - d->GlobalRmed[i - 1]) - 1.0;
}

static void Heating1(ora_disk *d, double Mplanet, double dMplanet, double Xp, double Yp, double dt, int k)   /* Planet.c:222-247 */
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  double Rperp = sqrt(Xp * Xp + Yp * Yp);
  if (Rperp < d->Rinf[0] || Rperp > d->Rsup[nr - 1]) return;
  double tdelay = 4.0 * p->dt * (double)p->heating_delay;
  double taper = d->PhysicalTime / tdelay;
  if (taper > 1.0) taper = 1.0;
  double plrho = p->planetary_density / RHO2CGS;
  double plradius = pow(3.0 * Mplanet / (4.0 * PI * plrho), 1.0 / 3.0);
  double L = Mplanet * dMplanet / dt / plradius;
  double ang = atan2(Yp, Xp);
  if (ang < 0.0) ang += 2.0 * PI;
  int i = 0;
  while (d->Rsup[i] < Rperp) i++;
  int j = (int)floor((double)ns / 2.0 / PI * ang + 0.5);
  if (j == ns) j = 0;
  d->heatsrc_index[k] = j + i * ns;
  d->heatsrc[k] += L * taper / d->Surf[i];
}

/* Kley's gas accretion (Planet.c:34-210): within 0.75 and 0.45 Roche radii
 * the density loses the fractions dt*acc/3 and 2 dt*acc/3 of the column
 * between the planet's height +/- the chord, integrated by the trapezoid
 * rule refined to a relative precision of 1e-4 (qtrap, at most 16 levels). */
#define QTRAPEPS 1.e-4
#define QTRAPMAX 16
static double rho_func(double z) { return exp(-z * z); }

static double trapzd_g(double a, double b, int n, double *s)
{
  if (n == 1) return (*s = 0.5 * (b - a) * (rho_func(a) + rho_func(b)));
  int it = 1;
  for (int j = 1; j < n - 1; j++) it <<= 1;
  double tnm = it, del = (b - a) / tnm, x = a + 0.5 * del, sum = 0.0;
  for (int j = 1; j <= it; j++, x += del) sum += rho_func(x);
  *s = 0.5 * (*s + (b - a) * sum / tnm);
  return *s;
}

static double qtrap_g(double a, double b, double eps)
{
  double s = 0.0, olds = 0.0, st = 0.0;
  for (int j = 1; j <= QTRAPMAX; j++) {
    s = trapzd_g(a, b, j, &st);
    if (j > 5)
      if (fabs(s - olds) < eps * fabs(olds) || (s == 0.0 && olds == 0.0)) return s;
    olds = s;
  }
  return s;
}

static void AccreteOntoPlanets(ora_disk *d, thorin_planets *sys, double dt)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  double *dens = d->rho, *vrad = d->vrad, *vtheta = d->vtheta;
  for (int k = 0; k < sys->nb; k++) {
    if (!(sys->acc[k] > 1e-10)) continue;
    double dMplanet = 0.0, dPxPlanet = 0.0, dPyPlanet = 0.0;
    double facc = fabs(dt) * (sys->acc[k]);
    double facc1 = 1.0 / 3.0 * facc, facc2 = 2.0 / 3.0 * facc, frac1 = 0.75, frac2 = 0.45;
    facc1 = (facc1 < 1.0) ? facc1 : 1.0;
    facc2 = (facc2 < 1.0) ? facc2 : 1.0;
    double Xplanet = sys->x[k], Yplanet = sys->y[k], Zplanet = sys->z[k];
    double VXplanet = sys->vx[k], VYplanet = sys->vy[k], Mplanet = sys->mass[k];
    double Rperp = sqrt(Xplanet * Xplanet + Yplanet * Yplanet);
    double Rplanet = sqrt(Xplanet * Xplanet + Yplanet * Yplanet + Zplanet * Zplanet);
    double RRoche = pow((1.0 / 3.0 * Mplanet * d->MassTaper), (1.0 / 3.0)) * Rplanet;
    int i_min = 0, i_max = nr - 1;
    while ((d->Rsup[i_min] < Rperp - RRoche) && (i_min < nr)) i_min++;
    while ((d->Rinf[i_max] > Rperp + RRoche) && (i_max > 0)) i_max--;
    double angle = atan2(Yplanet, Xplanet);
    int j_min = (int)((double)ns / 2.0 / PI * (angle - 2.0 * RRoche / Rperp));
    int j_max = (int)((double)ns / 2.0 / PI * (angle + 2.0 * RRoche / Rperp));
    double PxPlanet = Mplanet * VXplanet, PyPlanet = Mplanet * VYplanet;
    for (int i = i_min; i <= i_max; i++)
      for (int j = j_min; j <= j_max; j++) {
        int jf = j;
        while (jf < 0) jf += ns;
        while (jf >= ns) jf -= ns;
        int l = jf + i * ns, lip = l + ns, ljp = l + 1;
        if (jf == ns - 1) ljp = i * ns;
        double xc = d->abscissa[l], yc = d->ordinate[l];
        double dx = Xplanet - xc, dy = Yplanet - yc, distance = sqrt(dx * dx + dy * dy);
        double vtcell = 0.5 * (vtheta[l] + vtheta[ljp]) + d->Rmed[i] * d->OmegaFrame;
        double vrcell = 0.5 * (vrad[l] + vrad[lip]);
        double vxcell = (vrcell * xc - vtcell * yc) / d->Rmed[i];
        double vycell = (vrcell * yc + vtcell * xc) / d->Rmed[i];
        double H = d->cs[l] * d->OmegaInv[i] * d->SQRT_ADIABIND_INV;
        if (distance < frac1 * RRoche) {
          double dz = sqrt(pow(frac1 * RRoche, 2) - pow(distance, 2));
          double z1 = Zplanet - dz, z2 = Zplanet + dz;
          double factor = qtrap_g(z1 / (sqrt(2.0) * H), z2 / (sqrt(2.0) * H), QTRAPEPS);
          factor *= 1.0 / (sqrt(2.0 * PI) * H);
          double deltaM = facc1 * factor * dens[l] * d->Surf[i];
          if (i < 0) deltaM = 0.0;                              /* Zero_or_active = 0 */
          if (i >= nr) deltaM = 0.0;                            /* Max_or_active = nr */
          dens[l] *= (1.0 - facc1 * factor);
          dPxPlanet += deltaM * vxcell;
          dPyPlanet += deltaM * vycell;
          dMplanet += deltaM;
        }
        if (distance < frac2 * RRoche) {
          double dz = sqrt(pow(frac2 * RRoche, 2) - pow(distance, 2));
          double z1 = Zplanet - dz, z2 = Zplanet + dz;
          double factor = qtrap_g(z1 / (sqrt(2.0) * H), z2 / (sqrt(2.0) * H), QTRAPEPS);
          factor *= 1.0 / (sqrt(2.0 * PI) * H);
          double deltaM = facc2 * factor * dens[l] * d->Surf[i];
          if (i < 0) deltaM = 0.0;
          if (i >= nr) deltaM = 0.0;
          dens[l] *= (1.0 - facc2);
          dPxPlanet += deltaM * vxcell;
          dPyPlanet += deltaM * vycell;
          dMplanet += deltaM;
        }
      }
    if (p->gas_accret_heating) Heating1(d, Mplanet, dMplanet, Xplanet, Yplanet, dt, k);
    PxPlanet += dPxPlanet;
    PyPlanet += dPyPlanet;
    Mplanet += dMplanet;
    if (sys->feel_disk[k]) {
      sys->vx[k] = PxPlanet / Mplanet;
      sys->vy[k] = PyPlanet / Mplanet;
    }
    sys->mass[k] = Mplanet;
  }
}

/* ParametricAccretion (Pebbles.c:806-828): mass doubling every
 * PARAMETRICACCRETION kyr; the doubling time is fixed at the first call. */
static void ParametricAccretion(ora_disk *d, thorin_planets *sys, double dt)
{
  const thorin_params *p = &d->p;
  if (d->doubling == 0.0) d->doubling = p->parametric_accretion * 1000.0 * 2.0 * PI;
  if (p->accret_heating) d->heatsrc_max = sys->nb;
  for (int k = 0; k < sys->nb; k++) {
    double Mplanet = sys->mass[k];
    double dMplanet = Mplanet * dt / d->doubling;
    if (p->accret_heating) Heating1(d, Mplanet, dMplanet, sys->x[k], sys->y[k], dt, k);
    sys->mass[k] = Mplanet + dMplanet;
  }
}

/* StokesDrag + AdvanceSystemFromDrag (Drag.c:17-119): drag of the gas in
 * the planet's cell (the cell's v_theta neighbour is l+1 without wrapping,
 * as in the reference). */
#define DRAGCOEFF 0.48
static void AdvanceSystemFromDrag(ora_disk *d, thorin_planets *sys, double dt)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  for (int k = 0; k < sys->nb; k++) {
    if (!sys->feel_disk[k]) continue;
    double m = sys->mass[k], x = sys->x[k], y = sys->y[k], z = sys->z[k];
    double vx = sys->vx[k], vy = sys->vy[k], vz = sys->vz[k], ax = 0.0, ay = 0.0, az = 0.0;
    double Rperp = sqrt(x * x + y * y);
    if (Rperp >= d->Rinf[0] && Rperp <= d->Rsup[nr - 1]) {
      int i = 0;
      while (d->Rsup[i] < Rperp) i++;
      double ang = atan2(y, x);
      if (ang < 0.0) ang += 2.0 * PI;
      int j = (int)floor((double)ns / 2.0 / PI * ang + 0.5);
      if (j == ns) j = 0;
      int l = j + i * ns, lip = l + ns, ljp = l + 1;
      double xc = d->abscissa[l], yc = d->ordinate[l];
      double vtcell = 0.5 * (d->vtheta[l] + d->vtheta[ljp]) + d->Rmed[i] * d->OmegaFrame;
      double vrcell = 0.5 * (d->vrad[l] + d->vrad[lip]);
      double vxcell = (vrcell * xc - vtcell * yc) / d->Rmed[i];
      double vycell = (vrcell * yc + vtcell * xc) / d->Rmed[i];
      double vzcell = 0.0;
      double H = d->cs[l] * d->OmegaInv[i] * d->SQRT_ADIABIND_INV;
      double factor = rho_func(z / (sqrt(2.0) * H));
      factor *= 1.0 / (sqrt(2.0 * PI) * H);
      double plrho = p->planetary_density / RHO2CGS;
      double plradius = pow(3.0 * m / (4.0 * PI * plrho), 1.0 / 3.0);
      double dvx = vx - vxcell, dvy = vy - vycell, dvz = vz - vzcell;
      double dvsq = dvx * dvx + dvy * dvy + dvz * dvz;
      double tmp = -0.5 * DRAGCOEFF * PI * plradius * plradius / m * factor * d->rho[l] * dvsq * 1.0 / sqrt(dvsq);
      ax = tmp * dvx; ay = tmp * dvy; az = tmp * dvz;
    }
    sys->vx[k] += dt * ax;
    sys->vy[k] += dt * ay;
    sys->vz[k] += dt * az;
  }
}

static void AccretePebblesOntoPlanets(ora_disk *d, thorin_planets *sys, double dt)   /* :353-539 */
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  double *pdens = d->pdens, *tau = d->tau, *cs = d->cs, *macc = d->macc;
  if (p->accret_heating) d->heatsrc_max = sys->nb;
  make1Dprofile(d, d->vtheta, d->vt1D);
  for (int k = 0; k < sys->nb; k++) {
    double dMp = 0, dPXp = 0, dPYp = 0;
    double Xp = sys->x[k], Yp = sys->y[k], Zp = sys->z[k], VXp = sys->vx[k], VYp = sys->vy[k], VZp = sys->vz[k];
    double Mp = sys->mass[k], Msolid = sys->solid[k], PXp = VXp * Mp, PYp = VYp * Mp;
    double Rp = Xp * Xp + Yp * Yp, Rp3D = sqrt(Rp + Zp * Zp);
    Rp = sqrt(Rp);
    double Rhill = Rp3D * pow(1.0 / 3.0 * Mp, 1.0 / 3.0);
    double Omegap = pow(Rp, -1.5);
    double ifrac = GetGlobalIFrac(d, Rp), frac = ifrac - floor(ifrac);
    int i = (int)ifrac;
    double flow = d->vt1D[i] * (1.0 - frac) + d->vt1D[i + 1] * frac + Rp * d->OmegaFrame;
    double flowx = -flow * Yp / Rp, flowy = flow * Xp / Rp;
    double vrel = sqrt((VXp - flowx) * (VXp - flowx) + (VYp - flowy) * (VYp - flowy) + VZp * VZp);
    double Mt = sqrt(1.0 / 3.0) * pow(vrel, 3.0) / Omegap;
    int imax = nr - 1, imin = 0;
    while (d->Rinf[imax] > (Rp + Rhill) && imax >= imin) imax--;
    while (d->Rsup[imin] < (Rp - Rhill) && imin <= imax) imin++;
    int ncell = 0;
    double tau_mean = 0.0;
    for (i = imin; i <= imax; i++)
      for (int j = 0; j < ns; j++) { tau_mean += tau[j + i * ns]; ncell++; }
    tau_mean /= (double)ncell;
    double Reff, fac;
    if (Mp < Mt) {
      double Rbondi = Mp / vrel / vrel, tbondi = Rbondi / vrel;
      fac = sqrt(tau_mean * pow(Rp, 1.5) / tbondi);
      Reff = Rbondi * fac;
    } else {
      fac = pow(tau_mean / 0.1, 1.0 / 3.0);
      Reff = Rhill * fac;
    }
    if (Reff > Rhill) Reff = Rhill;
    double Reff2 = Reff * Reff, dM_upper = 0.0, Hpeb_mean = 0.0, pdens_mean = 0.0;
    ncell = 0;
    for (i = imin; i <= imax; i++)
      for (int j = 0; j < ns; j++) {
        int l = j + i * ns;
        double xc = d->abscissa[l], yc = d->ordinate[l];
        double R2 = (xc - Xp) * (xc - Xp) + (yc - Yp) * (yc - Yp);
        if (R2 <= Reff2) {
          double H = cs[l] * d->OmegaInv[i] * d->SQRT_ADIABIND_INV;
          double Hpeb = H * sqrt(p->pebble_alpha / tau[l]);
          double zmin = Zp - sqrt(Reff2 - R2), zmax = Zp + sqrt(Reff2 - R2);
          double mcell = d->Surf[i] * pdens[l];
          double vdp = pdens[l] / Hpeb * SQRT2PI_INV;
          double dM = vdp * d->Surf[i] * IntegrateColumnMass(zmin, zmax, Hpeb);
          if (dM > mcell) dM = 0.99999999 * mcell;
          macc[l] = dM;
          dM_upper += dM; Hpeb_mean += Hpeb; pdens_mean += pdens[l]; ncell++;
        }
      }
    if (ncell > 0) { Hpeb_mean /= (double)ncell; pdens_mean /= (double)ncell; }
    double veloc = (Mp < Mt) ? vrel : Reff * Omegap, dM_model, limiter;
    if (Hpeb_mean < Reff) dM_model = 2.0 * Reff * veloc * pdens_mean;
    else dM_model = PI * Reff * Reff * veloc * pdens_mean / Hpeb_mean * SQRT2PI_INV;
    dM_model *= dt;
    limiter = (dM_upper > dM_model) ? dM_model / dM_upper : 1.0;
    for (i = imin; i <= imax; i++) {
      double vtcorr = d->Rmed[i] * d->OmegaFrame;
      for (int j = 0; j < ns; j++) {
        int l = j + i * ns;
        if (macc[l] > 0.0) {
          double xc = d->abscissa[l], yc = d->ordinate[l];
          double vrc = d->pvrad[l], vtc = d->pvtheta[l] + vtcorr;
          double vxc = (vrc * xc - vtc * yc) * d->InvRmed[i], vyc = (vrc * yc + vtc * xc) * d->InvRmed[i];
          double dM = macc[l] * limiter;
          macc[l] = 0.0;
          double mcell = d->Surf[i] * pdens[l];
          pdens[l] = (mcell - dM) / d->Surf[i];
          if (pdens[l] < 0.0) pdens[l] = 1.e-20;
          dMp += dM; dPXp += dM * vxc; dPYp += dM * vyc;
        }
      }
    }
    if (p->accret_heating) Heating1(d, Mp, dMp, Xp, Yp, dt, k);
    PXp += dPXp; PYp += dPYp; Mp += dMp; Msolid += dMp;
    sys->mass[k] = Mp; sys->solid[k] = Msolid;
    sys->vx[k] = PXp / Mp; sys->vy[k] = PYp / Mp;
  }
}

static void EvaporatePebbles(ora_disk *d, double dt)        /* :834-864 */
{
  const thorin_params *p = &d->p;
  if (p->evaporation_rate <= 0.0) return;
  double facc = p->evaporation_rate * dt;
  if (facc > 1.0) facc = 1.0;
  double evaptemp = p->evaporation_temperature / T2SI;
  OMP_FOR
  for (int l = 0; l < d->nr * d->ns; l++)
    if (d->temper[l] > evaptemp) {
      d->pdens[l] *= (1.0 - facc);
      if (d->pdens[l] < EVAPOREDSIGMA) d->pdens[l] = EVAPOREDSIGMA;
    }
}

static void SourceTermsPebbles(ora_disk *d, double dt)      /* :550-613 */
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns;
  DampPebbles(d, dt);
  OMP_FOR
  for (int i = 1; i < nr; i++) {
    double Omega = 1.0 / d->OmegaInv[i];
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns, ljp = (j == ns - 1) ? i * ns : l + 1;
      double vt2 = d->pvtheta[l] + d->pvtheta[ljp] + d->pvtheta[lim] + d->pvtheta[ljp - ns];
      vt2 = vt2 / 4.0 + d->Rinf[i] * d->OmegaFrame;
      vt2 = vt2 * vt2;
      d->paccr[l] = vt2 * d->InvRinf[i] + 0.5 * (d->pagr[l] + d->pagr[lim]);
      if (p->back_reaction) {
        double drag = Omega * (d->pvrad[l] - d->vrad[l]) / d->tau[l];
        d->dragr[l] = 0.5 * (d->pdens[l] + d->pdens[lim]) * drag;
      }
    }
  }
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double Omega = 1.0 / d->OmegaInv[i];
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      d->pacct[l] = 0.5 * (d->pagt[l] + d->pagt[ljm]);
      if (p->back_reaction) {
        double drag = Omega * (d->pvtheta[l] - d->vtheta[l]) / d->tau[l];
        d->dragt[l] = 0.5 * (d->pdens[l] + d->pdens[ljm]) * drag;
      }
    }
  }
}

static void SubStep1Pebbles(ora_disk *d, double dt)         /* :617-652 */
{
  int nr = d->nr, ns = d->ns;
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double Omega = 1.0 / d->OmegaInv[i];
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      double efac = exp(-dt * Omega / d->tau[l]);
      if (i > 0)
        d->pvrad[l] = d->pvrad[l] * efac + d->gaccr[l] * dt + (d->vrad[l] + (d->paccr[l] - d->gaccr[l]) * d->tau[l] / Omega) * (1.0 - efac);
      d->pvtheta[l] = d->pvtheta[l] * efac + d->gacct[l] * dt + (d->vtheta[l] + (d->pacct[l] - d->gacct[l]) * d->tau[l] / Omega) * (1.0 - efac);
    }
  }
}

static void ParticleDiffusion(ora_disk *d)                  /* :656-698 */
{
  int nr = d->nr, ns = d->ns;
  const double *rho = d->rho, *pd = d->pdens;
  OMP_FOR
  for (int i = 1; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, lim = l - ns;
      double corr = -FViscosity(d, d->Rinf[i]) / d->p.schmidt_number;
      corr *= (rho[l] + rho[lim]) / (pd[l] + pd[lim]);
      corr *= (pd[l] / rho[l] - pd[lim] / rho[lim]) * d->InvDiffRmed[i];
      d->pvrad[l] += corr;
    }
  OMP_FOR
  for (int i = 0; i < nr; i++) {
    double dxtheta = 2.0 * PI / (double)ns * d->Rmed[i], invdxtheta = 1.0 / dxtheta;
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns, ljm = (j == 0) ? i * ns + ns - 1 : l - 1;
      double corr = -FViscosity(d, d->Rmed[i]) / d->p.schmidt_number;
      corr *= (rho[l] + rho[ljm]) / (pd[l] + pd[ljm]);
      corr *= (pd[l] / rho[l] - pd[ljm] / rho[ljm]) * invdxtheta;
      d->pvtheta[l] += corr;
    }
  }
}

/* ------------------------------------------------------------------ */
/* Disk forces: Pframeforce.c:43-510, Force.c:75-102                    */
static double ThicknessSmoothing(const ora_disk *d, double x, double y)
{
  double r = sqrt(x * x + y * y), sm = 0.0;
  if (r >= d->Rinf[0] && r <= d->Rsup[d->nr - 1]) {
    int i = 0;
    while (d->Rsup[i] < r) i++;
    double csavrg = 0.0;
    for (int j = 0; j < d->ns; j++) csavrg += d->cs[j + i * d->ns];
    csavrg /= (double)d->ns;
    sm = d->p.thickness_smoothing * (csavrg * d->OmegaInv[i] * d->SQRT_ADIABIND_INV);
  }
  return sm;
}

static void FillForcesArrays(ora_disk *d, thorin_planets *sys)
{
  const thorin_params *p = &d->p;
  int nr = d->nr, ns = d->ns, npl = sys->nb, peb = p->pebbles;
  double rsm2[THORIN_MAXPLANETS], rst2[THORIN_MAXPLANETS], rst3[THORIN_MAXPLANETS], rst4[THORIN_MAXPLANETS];
  double hillcut[THORIN_MAXPLANETS], rhill[THORIN_MAXPLANETS], smoothing2[THORIN_MAXPLANETS], Hpl[THORIN_MAXPLANETS];
  double s2[THORIN_MAXPLANETS], integpl[THORIN_MAXPLANETS], p_integpl[THORIN_MAXPLANETS], rmorevert2[THORIN_MAXPLANETS];
  double axpl[THORIN_MAXPLANETS], aypl[THORIN_MAXPLANETS];
  int IntegrateWithPlanet[THORIN_MAXPLANETS];
  double axstar = 0.0, aystar = 0.0, MassTaper = d->MassTaper;
  for (int k = 0; k < THORIN_MAXPLANETS; k++) axpl[k] = aypl[k] = 0.0;
  size_t bytes = sizeof(double) * (size_t)(nr + 1) * (size_t)ns;
  memset(d->agr, 0, bytes); memset(d->agt, 0, bytes);
  if (peb) { memset(d->pagr, 0, bytes); memset(d->pagt, 0, bytes); }
  for (int k = 0; k < npl; k++) {
    double xpl = sys->x[k], ypl = sys->y[k], zpl = sys->z[k], mpl = sys->mass[k];
    axpl[k] = aypl[k] = 0.0;
    hillcut[k] = 1.0;
    double dpl = sqrt(xpl * xpl + ypl * ypl + zpl * zpl);
    rhill[k] = dpl * pow((1.0 / 3.0 * mpl), 1.0 / 3.0);
    double smoothing = ThicknessSmoothing(d, xpl, ypl);
    Hpl[k] = smoothing / p->thickness_smoothing;
    smoothing2[k] = smoothing * smoothing;
    double rst = 0.5 * rhill[k];
    rst2[k] = rst * rst; rst3[k] = rst2[k] * rst; rst4[k] = rst3[k] * rst;
    double rsm = 0.05 * rhill[k];
    rsm2[k] = rsm * rsm;
    rmorevert2[k] = 2.0 * rhill[k];
    rmorevert2[k] *= rmorevert2[k];
    if (p->indirect_term) {
      double invdpl3 = 1.0 / (dpl * dpl * dpl);
      mpl *= MassTaper;
      axstar += mpl * invdpl3 * xpl;
      aystar += mpl * invdpl3 * ypl;
    }
  }
  double indpl_x = -axstar, indpl_y = -aystar;
  axstar = aystar = 0.0;
#ifdef _OPENMP
#pragma omp parallel for firstprivate(hillcut) private(s2, integpl, p_integpl, IntegrateWithPlanet) \
    reduction(+ : axstar, aystar, axpl[:THORIN_MAXPLANETS], aypl[:THORIN_MAXPLANETS])
#endif
  for (int i = 0; i < nr; i++) {
    double omegainv = d->OmegaInv[i], r2 = d->Rmed2[i], Rsup_Rinf2 = d->Rsup[i] - d->Rinf[i];
    Rsup_Rinf2 *= Rsup_Rinf2;
    int Nvert = 10;
    double cs_avr = 0.0, tau_avr = 0.0, p_H_avr = 0.0, p_integstar_avr = 0.0;
    for (int j = 0; j < ns; j++) { cs_avr += d->cs[j + i * ns]; if (peb) tau_avr += d->tau[j + i * ns]; }
    cs_avr /= (double)ns;
    double H_avr = cs_avr * omegainv * d->SQRT_ADIABIND_INV;
    if (peb) { tau_avr /= (double)ns; p_H_avr = H_avr * sqrt(p->pebble_alpha / tau_avr); p_integstar_avr = 0.0; }
    double H2 = H_avr * H_avr, zmax = 3.0 * H_avr, deltaz = zmax / (double)Nvert, sigma_avr = 0.0, integstar_avr = 0.0;
    for (int m = 1; m <= Nvert; m++) {
      double znode = ((double)m - 0.5) * deltaz, znode2 = znode * znode;
      double sum = exp(-(0.5 * znode2 / H2));
      sigma_avr += sum;
      double d2 = r2 + znode2, dd = sqrt(d2), denom = dd * d2;
      integstar_avr += sum / denom;
      if (peb) {
        znode2 *= p->pebble_alpha / tau_avr;
        d2 = r2 + znode2; dd = sqrt(d2); denom = dd * d2;
        p_integstar_avr += sum / denom;
      }
    }
    for (int j = 0; j < ns; j++) {
      int IntegrateLocally = 0, l = j + i * ns;
      double ax = 0.0, ay = 0.0, pax = 0.0, pay = 0.0, Hcorr = 0.0, pH = 0.0, pmcell = 0.0;
      double x = d->abscissa[l], y = d->ordinate[l], mcell = d->rho[l] * d->Surf[i];
      double H = d->cs[l] * omegainv * d->SQRT_ADIABIND_INV, sigma, integstar, p_integstar = 0.0, tmp, ar, at;
      Nvert = 10;
      H2 = H * H;
      if (fabs(H - H_avr) / H_avr > 0.05) IntegrateLocally = 1;
      if (peb) {
        pmcell = d->pdens[l] * d->Surf[i];
        Hcorr = sqrt(p->pebble_alpha / d->tau[l]);
        pH = H * Hcorr;
        if (fabs(pH - p_H_avr) / p_H_avr > 0.05) IntegrateLocally = 1;
      }
      for (int k = 0; k < npl; k++) {
        double xpl = sys->x[k], ypl = sys->y[k], zpl = sys->z[k];
        s2[k] = (x - xpl) * (x - xpl) + (y - ypl) * (y - ypl);
        double r2chk_1 = 10.0 * Hpl[k]; r2chk_1 *= r2chk_1;
        double r2chk_2 = 5.0 * rhill[k]; r2chk_2 *= r2chk_2;
        if (MassTaper == 1.0 && (s2[k] < r2chk_1 || s2[k] < r2chk_2)) {
          IntegrateLocally = 1;
          IntegrateWithPlanet[k] = 1;
          integpl[k] = 0.0;
          if (peb) p_integpl[k] = 0.0;
          double d2 = s2[k] + zpl * zpl;
          if (p->exclude_hill) hillcut[k] = 1.0 / (exp(-(sqrt(d2) / rhill[k] - p->hillcut) / p->hillcut * 10.0) + 1.0);
        } else IntegrateWithPlanet[k] = 0;
        if (s2[k] < rmorevert2[k]) Nvert = 30;
      }
      if (IntegrateLocally) {
        zmax = 3.0 * H; deltaz = zmax / (double)Nvert;
        sigma = 0.0; integstar = 0.0; p_integstar = 0.0;
        for (int m = 1; m <= Nvert; m++) {
          double znode = ((double)m - 0.5) * deltaz, znode2 = znode * znode;
          double sum = exp(-(0.5 * znode2 / H2));
          sigma += sum;
          double d2 = r2 + znode2, dd = sqrt(d2), denom = dd * d2;
          integstar += sum / denom;
          if (peb) { d2 = r2 + znode2 * Hcorr * Hcorr; dd = sqrt(d2); denom = dd * d2; p_integstar += sum / denom; }
          for (int k = 0; k < npl; k++) {
            if (!IntegrateWithPlanet[k]) continue;
            double zpl = sys->z[k], taper, mx = (rsm2[k] > Rsup_Rinf2) ? rsm2[k] : Rsup_Rinf2;
            d2 = s2[k] + (znode - zpl) * (znode - zpl);
            if (d2 < rst2[k]) { dd = sqrt(d2); taper = -3.0 * d2 * d2 / rst4[k] + 4.0 * dd * d2 / rst3[k]; } else taper = 1.0;
            d2 += mx; dd = sqrt(d2); denom = dd * d2;
            integpl[k] += sum / denom * taper;
            if (zpl < -0.05 * H || zpl > 0.05 * H) {
              d2 = s2[k] + (-znode - zpl) * (-znode - zpl);
              if (d2 < rst2[k]) { dd = sqrt(d2); taper = -3.0 * d2 * d2 / rst4[k] + 4.0 * dd * d2 / rst3[k]; } else taper = 1.0;
              d2 += mx; dd = sqrt(d2); denom = dd * d2;
              integpl[k] += sum / denom * taper;
            }
            if (peb) {
              d2 = s2[k] + (znode * Hcorr - zpl) * (znode * Hcorr - zpl);
              if (d2 < rst2[k]) { dd = sqrt(d2); taper = -3.0 * d2 * d2 / rst4[k] + 4.0 * dd * d2 / rst3[k]; } else taper = 1.0;
              d2 += mx; dd = sqrt(d2); denom = dd * d2;
              p_integpl[k] += sum / denom * taper;
              if (zpl < -0.05 * pH || zpl > 0.05 * pH) {
                d2 = s2[k] + (-znode * Hcorr - zpl) * (-znode * Hcorr - zpl);
                if (d2 < rst2[k]) { dd = sqrt(d2); taper = -3.0 * d2 * d2 / rst4[k] + 4.0 * dd * d2 / rst3[k]; } else taper = 1.0;
                d2 += mx; dd = sqrt(d2); denom = dd * d2;
                p_integpl[k] += sum / denom * taper;
              }
            }
          }
        }
      } else {
        sigma = sigma_avr; integstar = integstar_avr;
        if (peb) p_integstar = p_integstar_avr;
      }
      tmp = integstar / sigma;
      ar = -d->Rmed[i] * tmp;
      d->agr[l] += ar;
      axstar += mcell * tmp * x;
      aystar += mcell * tmp * y;
      if (peb) { tmp = p_integstar / sigma; ar = -d->Rmed[i] * tmp; d->pagr[l] += ar; }
      for (int k = 0; k < npl; k++) {
        double xpl = sys->x[k], ypl = sys->y[k], zpl = sys->z[k], mpl = sys->mass[k];
        if (IntegrateWithPlanet[k]) {
          if (zpl < -0.05 * H || zpl > 0.05 * H) tmp = (x - xpl) * integpl[k] / (2.0 * sigma);
          else tmp = (x - xpl) * integpl[k] / sigma;
          ax += -mpl * tmp;
          if (p->exclude_hill) tmp *= hillcut[k];
          axpl[k] += mcell * tmp;
          if (zpl < -0.05 * H || zpl > 0.05 * H) tmp = (y - ypl) * integpl[k] / (2.0 * sigma);
          else tmp = (y - ypl) * integpl[k] / sigma;
          ay += -mpl * tmp;
          if (p->exclude_hill) tmp *= hillcut[k];
          aypl[k] += mcell * tmp;
          if (peb) {
            if (zpl < -0.05 * pH || zpl > 0.05 * pH) tmp = (x - xpl) * p_integpl[k] / (2.0 * sigma);
            else tmp = (x - xpl) * p_integpl[k] / sigma;
            pax += -mpl * tmp;
            if (p->pebble_gravity) { if (p->exclude_hill) tmp *= hillcut[k]; axpl[k] += pmcell * tmp; }
            if (zpl < -0.05 * pH || zpl > 0.05 * pH) tmp = (y - ypl) * p_integpl[k] / (2.0 * sigma);
            else tmp = (y - ypl) * p_integpl[k] / sigma;
            pay += -mpl * tmp;
            if (p->pebble_gravity) { if (p->exclude_hill) tmp *= hillcut[k]; aypl[k] += pmcell * tmp; }
          }
        } else {
          mpl *= MassTaper;
          double d2 = s2[k] + zpl * zpl + smoothing2[k], dd = sqrt(d2), denom = dd * d2;
          tmp = (x - xpl) / denom;
          ax += -mpl * tmp;
          if (p->exclude_hill) tmp *= hillcut[k];
          axpl[k] += mcell * tmp;
          tmp = (y - ypl) / denom;
          ay += -mpl * tmp;
          if (p->exclude_hill) tmp *= hillcut[k];
          aypl[k] += mcell * tmp;
          if (peb) {
            d2 += -smoothing2[k] + smoothing2[k] * Hcorr * Hcorr;
            dd = sqrt(d2); denom = dd * d2;
            tmp = (x - xpl) / denom;
            pax += -mpl * tmp;
            if (p->pebble_gravity) { if (p->exclude_hill) tmp *= hillcut[k]; axpl[k] += pmcell * tmp; }
            tmp = (y - ypl) / denom;
            pay += -mpl * tmp;
            if (p->pebble_gravity) { if (p->exclude_hill) tmp *= hillcut[k]; aypl[k] += pmcell * tmp; }
          }
        }
      }
      ar = (x * ax + y * ay) * d->InvRmed[i];
      at = (x * ay - y * ax) * d->InvRmed[i];
      d->agr[l] += ar; d->agt[l] += at;
      if (peb) {
        ar = (x * pax + y * pay) * d->InvRmed[i];
        at = (x * pay - y * pax) * d->InvRmed[i];
        d->pagr[l] += ar; d->pagt[l] += at;
      }
    }
  }
  d->indirect_x = -axstar;
  d->indirect_y = -aystar;
  for (int k = 0; k < npl; k++) { sys->ax[k] = axpl[k]; sys->ay[k] = aypl[k]; }
  double axindir = d->indirect_x, ayindir = d->indirect_y;
  if (p->indirect_term) { axindir += indpl_x; ayindir += indpl_y; }
  OMP_FOR
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      double x = d->abscissa[l], y = d->ordinate[l];
      double ar = (x * axindir + y * ayindir) * d->InvRmed[i];
      double at = (x * ayindir - y * axindir) * d->InvRmed[i];
      d->agr[l] += ar; d->agt[l] += at;
      if (peb) { d->pagr[l] += ar; d->pagt[l] += at; }
    }
}

static double DampingTW04(const ora_disk *d, double m, double x, double y, double z, double vz)   /* Pframeforce.c:571-603 */
{
  double r = sqrt(x * x + y * y), damp = 0.0;
  if ((d->p.vertical_damping > 0.0) && (r >= d->Rinf[0] && r <= d->Rsup[d->nr - 1])) {
    int i = 0;
    while (d->Rsup[i] < r) i++;
    double rhoavr = 0.0, csavr = 0.0;
    for (int j = 0; j < d->ns; j++) { rhoavr += d->rho[j + i * d->ns]; csavr += d->cs[j + i * d->ns]; }
    csavr /= (double)d->ns; rhoavr /= (double)d->ns;
    double cs4inv = pow(csavr, -4.0), Omega = pow(r, -1.5);
    damp = d->p.vertical_damping * m * rhoavr * Omega * cs4inv * (-2.176 * vz - 0.871 * z * Omega);
  }
  return damp;
}

static void AdvanceSystemFromDisk(ora_disk *d, thorin_planets *sys, double dt)   /* Pframeforce.c:514-566 */
{
  for (int k = 0; k < sys->nb; k++)
    if (sys->feel_disk[k]) {
      double damp = DampingTW04(d, sys->mass[k], sys->x[k], sys->y[k], sys->z[k], sys->vz[k]);
      sys->vx[k] += dt * sys->ax[k];
      sys->vy[k] += dt * sys->ay[k];
      sys->vz[k] += dt * (sys->az[k] + damp);
      sys->vx[k] += dt * d->indirect_x;
      sys->vy[k] += dt * d->indirect_y;
    }
}

/* ------------------------------------------------------------------ */
/* N-body step standing in for REBOUND IAS15 (ReboundInterface.c:262-325):
 * heliocentric -> barycentric, integrate the star + planets with their
 * mutual gravity over dt, back to heliocentric.  The integrator here is
 * classical RK4 with many small substeps (error far below the tolerances
 * the tests use for fields). */
static void nbody_accel(int n, const double *m, const double *x, double *a)
{
  for (int i = 0; i < 3 * n; i++) a[i] = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) {
      double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1], dz = x[3 * j + 2] - x[3 * i + 2];
      double r2 = dx * dx + dy * dy + dz * dz, r = sqrt(r2), ir3 = 1.0 / (r2 * r);
      a[3 * i] += G * m[j] * dx * ir3; a[3 * i + 1] += G * m[j] * dy * ir3; a[3 * i + 2] += G * m[j] * dz * ir3;
      a[3 * j] -= G * m[i] * dx * ir3; a[3 * j + 1] -= G * m[i] * dy * ir3; a[3 * j + 2] -= G * m[i] * dz * ir3;
    }
}

static void AdvanceSystemNbody(thorin_planets *sys, double dt)
{
  int n = sys->nb + 1;
  double m[THORIN_MAXPLANETS + 1], x[3 * (THORIN_MAXPLANETS + 1)], v[3 * (THORIN_MAXPLANETS + 1)];
  double k1x[3 * (THORIN_MAXPLANETS + 1)], k1v[3 * (THORIN_MAXPLANETS + 1)], xt[3 * (THORIN_MAXPLANETS + 1)];
  double ax[3 * (THORIN_MAXPLANETS + 1)], sx[3 * (THORIN_MAXPLANETS + 1)], sv[3 * (THORIN_MAXPLANETS + 1)];
  m[0] = 1.0;
  for (int c = 0; c < 3; c++) { x[c] = 0.0; v[c] = 0.0; }
  for (int k = 0; k < sys->nb; k++) {
    m[k + 1] = sys->mass[k];
    x[3 * k + 3] = sys->x[k]; x[3 * k + 4] = sys->y[k]; x[3 * k + 5] = sys->z[k];
    v[3 * k + 3] = sys->vx[k]; v[3 * k + 4] = sys->vy[k]; v[3 * k + 5] = sys->vz[k];
  }
  double M = 0, cx[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
  for (int i = 0; i < n; i++) { M += m[i]; for (int c = 0; c < 3; c++) { cx[c] += m[i] * x[3 * i + c]; cv[c] += m[i] * v[3 * i + c]; } }
  for (int i = 0; i < n; i++) for (int c = 0; c < 3; c++) { x[3 * i + c] -= cx[c] / M; v[3 * i + c] -= cv[c] / M; }
  int nsteps = 256;
  double h = dt / nsteps;
  for (int s = 0; s < nsteps; s++) {
    /* RK4 on (x, v) */
    for (int q = 0; q < 3 * n; q++) { sx[q] = 0; sv[q] = 0; }
    static const double wts[4] = {1.0, 2.0, 2.0, 1.0}, cs[4] = {0.0, 0.5, 0.5, 1.0};
    for (int q = 0; q < 3 * n; q++) { k1x[q] = 0; k1v[q] = 0; }
    for (int stage = 0; stage < 4; stage++) {
      for (int q = 0; q < 3 * n; q++) xt[q] = x[q] + cs[stage] * h * k1x[q];
      nbody_accel(n, m, xt, ax);
      for (int q = 0; q < 3 * n; q++) {
        double vx = v[q] + cs[stage] * h * k1v[q];
        k1x[q] = vx; k1v[q] = ax[q];
        sx[q] += wts[stage] * k1x[q]; sv[q] += wts[stage] * k1v[q];
      }
    }
    for (int q = 0; q < 3 * n; q++) { x[q] += h / 6.0 * sx[q]; v[q] += h / 6.0 * sv[q]; }
  }
  for (int k = 0; k < sys->nb; k++) {
    sys->x[k] = x[3 * k + 3] - x[0]; sys->y[k] = x[3 * k + 4] - x[1]; sys->z[k] = x[3 * k + 5] - x[2];
    sys->vx[k] = v[3 * k + 3] - v[0]; sys->vy[k] = v[3 * k + 4] - v[1]; sys->vz[k] = v[3 * k + 5] - v[2];
  }
}

static void MinStepForRebound(ora_disk *d, const thorin_planets *sys)   /* ReboundInterface.c:360-385 */
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
  dt *= 0.25; dt *= dt;
  d->invdtreb_sq = 1.0 / dt;
}

static void RotatePsys(thorin_planets *sys, double angle)   /* Psys.c:336-355 */
{
  double sint = sin(angle), cost = cos(angle);
  for (int k = 0; k < sys->nb; k++) {
    double xt = sys->x[k], yt = sys->y[k];
    sys->x[k] = xt * cost + yt * sint; sys->y[k] = -xt * sint + yt * cost;
    xt = sys->vx[k]; yt = sys->vy[k];
    sys->vx[k] = xt * cost + yt * sint; sys->vy[k] = -xt * sint + yt * cost;
  }
}

/* ------------------------------------------------------------------ */
/* AlgoGas: SourceEuler.c:210-317 (fixed frame, SloppyCFL off).  Returns a
 * THORIN_* status. */
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
  return (c <= -1.0) ? M_PI : 0.0;
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

int ora_algogas(ora_disk *d, thorin_planets *sys)
{
  const thorin_params *p = &d->p;
  double dt, dtemp = 0.0, DT = p->dt;
  int status = THORIN_OK, nsub = 0;
  if (p->sloppy_cfl) dt = DT / (double)ConditionCFL(d, DT - dtemp);   /* SourceEuler.c:221-227 */
  while (dtemp < 0.999999999 * DT) {
    d->MassTaper = d->PhysicalTime / (p->mass_taper * 2.0 * M_PI);
    d->MassTaper = (d->MassTaper > 1.0 ? 1.0 : pow(sin(d->MassTaper * M_PI / 2.0), 2.0));
    if (p->pebbles) PebbleStokesNumbers(d);
    if (!p->sloppy_cfl) {
      MinStepForRebound(d, sys);
      if (p->pebbles) CriticalCharTime(d);
      int n = ConditionCFL(d, DT - dtemp);
      dt = (DT - dtemp) / (double)n;
    }
    for (int k = 0; k < sys->nb; k++) { d->heatsrc[k] = 0.0; d->heatsrc_index[k] = -1; }   /* InitHeating */
    AccreteOntoPlanets(d, sys, dt);
    if (p->prescribed_accretion) ParametricAccretion(d, sys, dt);
    if (p->pebbles) { AccretePebblesOntoPlanets(d, sys, dt); EvaporatePebbles(d, dt); }
    dtemp += dt;
    double xmark, ymark;                                       /* GetPsysInfo (MARK), Psys.c:240-244 */
    frame_point(p->guiding_center, sys, &xmark, &ymark);
    FillForcesArrays(d, sys);
    AdvanceSystemFromDisk(d, sys, dt);
    if (p->aerodynamic_drag) AdvanceSystemFromDrag(d, sys, dt);
    AdvanceSystemNbody(sys, dt);
    if (p->corotating) {                                       /* SourceEuler.c:261-267 */
      double x, y;
      frame_point(p->guiding_center, sys, &x, &y);             /* GetPsysInfoFromRsim (GET), Psys.c:313-322 */
      double d2 = sqrt(x * x + y * y), d1 = sqrt(xmark * xmark + ymark * ymark);
      double cross = xmark * y - x * ymark;
      double OmegaNew = asin(cross / (d1 * d2)) / dt;         /* GetPsysInfo (GET), Psys.c:245-254 */
      double domega = OmegaNew - d->OmegaFrame;
      for (int i = 0; i < d->nr; i++)                          /* CorrectVtheta, SideEuler.c:505-519 */
        for (int j = 0; j < d->ns; j++) {
          int l = j + i * d->ns;
          d->vtheta[l] -= domega * d->Rmed[i];
          if (p->pebbles) d->pvtheta[l] -= domega * d->Rmed[i];
        }
      d->OmegaFrame = OmegaNew;
    }
    RotatePsys(sys, d->OmegaFrame * dt);
    ApplyBoundaryCondition(d, dt);
    int crashed = DetectCrash(d, d->rho);
    crashed = DetectCrash(d, d->energy);
    if (p->pebbles) crashed = DetectCrash(d, d->pdens);
    d->st.crashed = crashed;
    ComputePressureField(d, d->rho, d->energy);
    if (p->pebbles) SourceTermsPebbles(d, dt);
    SubStep1(d, dt);
    if (p->pebbles) { SubStep1Pebbles(d, dt); if (p->diffusive_particles) ParticleDiffusion(d); }
    SubStep2(d, dt);
    ActualiseGas(d, d->vrad, d->VradNew);
    ActualiseGas(d, d->vtheta, d->VthetaNew);
    ApplyBoundaryCondition(d, dt);
    if (p->energy_eq) {
      UpdateDivVelocAndStressTensor(d, d->vrad, d->vtheta, d->rho);
      int s = SubStep3(d, dt);
      if (s == THORIN_ERR_OMEGA) return s;
      if (s != THORIN_OK) status = s;
      ActualiseGas(d, d->energy, d->EnergyNew);
    }
    TransportFluid(d, d->rho, d->vrad, d->vtheta, p->energy_eq ? d->energy : NULL, dt);
    memcpy(d->NshiftGas, d->Nshift, sizeof(int) * (size_t)d->nr);
    ApplyBoundaryCondition(d, dt);
    ComputeTemperatureField(d, d->rho, d->energy);
    if (p->energy_eq) ComputeSoundSpeed(d, d->rho, d->energy);
    if (p->pebbles) {                                        /* EvolvePebbleDisk, Pebbles.c:702-708 */
      DampPebbles(d, dt);
      TransportFluid(d, d->pdens, d->pvrad, d->pvtheta, NULL, dt);
      DampPebbles(d, dt);
    }
    d->PhysicalTime += dt;
    d->st.last_dt = dt;
    nsub++;
  }
  d->st.substeps = nsub;
  return status;
}

/* Conservation integrals: SideEuler.c:26-80, 523-565 (sequential sums). */
void ora_integrals(ora_disk *d, double *mass, double *mom, double *energy, double *pmass, double *pmom)
{
  int nr = d->nr, ns = d->ns;
  double m = 0, am = 0, e = 0, pm = 0, pam = 0;
  for (int i = 0; i < nr; i++) for (int j = 0; j < ns; j++) m += d->Surf[i] * d->rho[j + i * ns];
  for (int i = 0; i < nr; i++) {
    for (int j = 1; j < ns; j++)
      am += d->Surf[i] * (d->rho[j + i * ns] + d->rho[j - 1 + i * ns]) * d->Rmed[i] * (d->vtheta[j + i * ns] + d->OmegaFrame * d->Rmed[i]);
    am += d->Surf[i] * (d->rho[i * ns] + d->rho[i * ns + ns - 1]) * d->Rmed[i] * (d->vtheta[i * ns] + d->OmegaFrame * d->Rmed[i]);
  }
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < ns; j++) {
      int l = j + i * ns;
      double vr_c = ((d->Rmed[i] - d->Rinf[i]) * d->vrad[l + ns] + (d->Rsup[i] - d->Rmed[i]) * d->vrad[l]) / (d->Rsup[i] - d->Rinf[i]);
      double vt_c = (j < ns - 1) ? 0.5 * (d->vtheta[l] + d->vtheta[l + 1]) + d->Rmed[i] * d->OmegaFrame
                                 : 0.5 * (d->vtheta[l] + d->vtheta[i * ns]) + d->Rmed[i] * d->OmegaFrame;
      e += 0.5 * d->Surf[i] * d->rho[l] * (vr_c * vr_c + vt_c * vt_c) + d->Surf[i] * d->energy[l];
    }
  if (d->p.pebbles) {
    for (int i = 0; i < nr; i++) for (int j = 0; j < ns; j++) pm += d->Surf[i] * d->pdens[j + i * ns];
    for (int i = 0; i < nr; i++) {
      for (int j = 1; j < ns; j++)
        pam += d->Surf[i] * (d->pdens[j + i * ns] + d->pdens[j - 1 + i * ns]) * d->Rmed[i] * (d->pvtheta[j + i * ns] + d->OmegaFrame * d->Rmed[i]);
      pam += d->Surf[i] * (d->pdens[i * ns] + d->pdens[i * ns + ns - 1]) * d->Rmed[i] * (d->pvtheta[i * ns] + d->OmegaFrame * d->Rmed[i]);
    }
  }
  *mass = m; *mom = 0.5 * am; *energy = e; *pmass = pm; *pmom = 0.5 * pam;
}

/* DiffusionTimestep's dt_stellar carried from one DT to the next. */
void ora_set_dt_stellar(ora_disk *d, double v) { d->dt_stellar = v; }

/* The SOR omega schedule: omega, its step and the last iteration count. */
void ora_get_sor_state(const ora_disk *d, double *omega, double *domega, int *niterlast)
{
  *omega = d->omega;
  *domega = d->domega;
  *niterlast = d->Niterlast;
}

/* Continue an SOR omega schedule instead of calibrating it (used to time
 * steady-state substeps). */
void ora_set_sor_state(ora_disk *d, double omega, double domega, int niterlast)
{
  d->omega = omega;
  d->domega = domega;
  d->Niterlast = niterlast;
  d->sor_first = 0;
}

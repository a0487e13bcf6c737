"""Parameter handling: the in.par reader and the C-ABI structs.

Mirrors the reference's parameter layer so that an in.par file means the same
thing here as in FARGO_THORIN:

* ``VARIABLES`` restates the variable table of src_main/var.c:17-141 (name,
  type, mandatory flag, default string), parsed like var()/ReadVariables
  (src_main/Interpret.c:31-148): case-insensitive keys, the first token after
  the key read with ``%lf``, ints truncated from that double, strings taken
  verbatim, unknown keys only warn.
* ``derive()`` restates the switch derivation of src_main/Interpret.c:149-265
  (including its quirks: the PARTICLEDIFFUSION test is an assignment, so
  particle diffusion is always on; the OPACITYTABLE test is case-sensitive).
* ``ThorinParams``/``ThorinPlanets``/``ThorinStats`` are the ctypes mirrors of
  the structs in include/thorin_gpu.h.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings

MAXPLANETS = 120

# (name, type, mandatory, default) -- src_main/var.c:17-141
REAL, INT, STRING = "real", "int", "string"
VARIABLES = [
    ("DT", REAL, True, "1."), ("SIGMA0", REAL, True, "173."), ("NINTERM", INT, True, "10."),
    ("NTOT", INT, True, "1501."), ("OUTPUTDIR", STRING, True, "out"), ("INPUTDIR", STRING, False, "in"),
    ("INNERBOUNDARY", STRING, False, "WALL"), ("OUTERBOUNDARY", STRING, False, "WALL"),
    ("LABELADVECTION", STRING, False, "NO"), ("TRANSPORT", STRING, False, "FAST"),
    ("PLANETCONFIG", STRING, False, "Systems/SolarSystem.cfg"), ("MASSTAPER", REAL, False, "0.0000001"),
    ("RADIALSPACING", STRING, False, "ARITHMETIC"), ("NRAD", INT, True, "64.0"), ("NSEC", INT, True, "64.0"),
    ("RMIN", REAL, True, "1.0"), ("RMAX", REAL, True, "1.0"), ("THICKNESSSMOOTHING", REAL, False, "0.0"),
    ("ROCHESMOOTHING", REAL, False, "0.0"), ("ASPECTRATIO", REAL, True, "0.05"), ("VISCOSITY", REAL, False, "0.0"),
    ("ALPHAVISCOSITY", REAL, False, "0.0"), ("ALPHAFLOCK", STRING, False, "NO"), ("TMRI", REAL, False, "1000.0"),
    ("TWIDTH", REAL, False, "25.0"), ("ALPHAMRI", REAL, False, "0.0"), ("ALPHADEAD", REAL, False, "0.0"),
    ("SIGMASLOPE", REAL, True, "0.0"), ("RELEASERADIUS", REAL, False, "0.0"), ("RELEASEDATE", REAL, False, "0.0"),
    ("OMEGAFRAME", REAL, False, "0.0"), ("DISK", STRING, False, "YES"), ("FRAME", STRING, False, "FIXED"),
    ("OUTERSOURCEMASS", STRING, False, "NO"), ("WRITEDENSITY", STRING, False, "YES"),
    ("WRITEVELOCITY", STRING, False, "YES"), ("INDIRECTTERM", STRING, False, "YES"), ("EXCLUDEHILL", STRING, False, "NO"),
    ("IMPOSEDDISKDRIFT", REAL, False, "0.0"), ("FLARINGINDEX", REAL, False, "0.0"), ("ECCENTRICITY", REAL, False, "0.0"),
    ("CAVITYRADIUS", REAL, False, "0.0"), ("CAVITYRATIO", REAL, False, "1.0"), ("CAVITYWIDTH", REAL, False, "1.0"),
    ("TRANSITIONRADIUS", REAL, False, "0.0"), ("TRANSITIONRATIO", REAL, False, "1.0"),
    ("TRANSITIONWIDTH", REAL, False, "1.0"), ("LAMBDADOUBLING", REAL, False, "0.0"),
    ("ENERGYEQUATION", STRING, False, "NO"), ("WRITETEMPERATURE", STRING, False, "NO"),
    ("WRITEENERGY", STRING, False, "NO"), ("WRITEDIVV", STRING, False, "NO"), ("WRITEQPLUS", STRING, False, "NO"),
    ("WRITEQBALANCE", STRING, False, "NO"), ("WRITEOPACITY", STRING, False, "NO"), ("ADIABIND", REAL, False, "1.4"),
    ("COOLINGTIME", REAL, False, "-1.0"), ("STELLARIRRADIATION", STRING, False, "NO"),
    ("OPACITYDROP", REAL, False, "0.6"), ("EFFECTIVETEMPERATURE", REAL, False, "5656.0"),
    ("STELLARRADIUS", REAL, False, "3.0"), ("DISCALBEDO", REAL, False, "0.5"), ("PARAMETRICOPACITY", REAL, False, "0.0"),
    ("INITIALIZEFROMFILE", STRING, False, "NO"), ("DENSINFILE", STRING, False, "in/gasdens.cfg"),
    ("VRADINFILE", STRING, False, "in/gasvrad.cfg"), ("VTHETAINFILE", STRING, False, "in/gasvtheta.cfg"),
    ("TEMPERINFILE", STRING, False, "in/gastemper.cfg"), ("DAMPTOWARDS", STRING, False, "ZEROVRAD"),
    ("DAMPINGRMINFRAC", REAL, False, "1.25"), ("DAMPINGRMAXFRAC", REAL, False, "0.84"),
    ("DAMPINGPERIODFRAC", REAL, False, "1.0"), ("NOUTELEMENTS", INT, False, "1"),
    ("PLANETARYDENSITY", REAL, False, "1.0"), ("RESOLVECOLLISIONS", STRING, False, "NO"),
    ("TARGETNPL", INT, False, "-1.0"), ("IAS15PRECISSION", REAL, False, "1.e-9"), ("IAS15MINDT", REAL, False, "0.0"),
    ("DISCARDPLANETS", STRING, False, "NO"), ("WRITETORQUEFILES", STRING, False, "YES"), ("HILLCUT", REAL, False, "0.8"),
    ("VERTICALDAMPING", REAL, False, "0.1"), ("PLANETSFEELDISK", STRING, False, "NO"),
    ("ACCRETIONRATE", REAL, False, "0.0"), ("GASACCRETIONHEATING", STRING, False, "NO"),
    ("PEBBLEACCRETION", STRING, False, "NO"), ("BACKREACTION", STRING, False, "NO"),
    ("ACCRETIONALHEATING", STRING, False, "NO"), ("WRITEETA", STRING, False, "NO"), ("PEBBLEFLUX", REAL, False, "2.0e-4"),
    ("PEBBLEALPHA", REAL, False, "1.0e-4"), ("PEBBLECOAGULATION", REAL, False, "0.5"),
    ("PEBBLEBULKDENS", REAL, False, "1.0"), ("SCHMIDTNUMBER", REAL, False, "1.0"),
    ("PARTICLEDIFFUSION", STRING, False, "NO"), ("HEATINGDELAY", INT, False, "100"),
    ("PARAMETRICACCRETION", REAL, False, "0.0"), ("TORQUEMAPINFILE", STRING, False, "NO"),
    ("GETTORQUEFORPLANET", INT, False, "-1"), ("PEBBLETOGASMAX", REAL, False, "0.01"),
    ("FRAGMENTFACTOR", REAL, False, "1.0"), ("FRAGMENTTHRESHOLD", REAL, False, "1.0"),
    ("FRAGMENTALPHA", REAL, False, "1.0e-3"), ("OPACITYTABLE", STRING, False, "BL94"), ("GASFLUX", REAL, False, "0.0"),
    ("DAMPING", STRING, False, "NO"), ("EVAPORATIONTEMPERATURE", REAL, False, "1000.0"),
    ("EVAPORATIONRATE", REAL, False, "1.0e-3"), ("FIRSTSTEP", REAL, False, "-1.0"), ("MINIMUMSTEP", REAL, False, "1.0e-3"),
    ("MAXIMUMSTEP", REAL, False, "1.0e6"), ("AERODYNAMICDRAG", STRING, False, "NO"),
    ("ELEMENTSWITHDISK", STRING, False, "NO"), ("PEBBLEGRAVITY", STRING, False, "NO"),
]
_TABLE = {name: (typ, mand, dflt) for name, typ, mand, dflt in VARIABLES}

# SOR constants of src_main/EnergySources.c:22-23 (hard-coded there).
SORMAXITERS = 100000
SOREPS = 1.0e-6


def _scan_double(tok: str) -> float:
    """sscanf("%lf") on a token: the longest leading float literal, else 0."""
    best = None
    for end in range(len(tok), 0, -1):
        try:
            best = float(tok[:end])
            break
        except ValueError:
            continue
    return 0.0 if best is None else best


def _convert(typ, text):
    if typ == STRING:
        return text
    v = _scan_double(text)
    return int(v) if typ == INT else v


def read_inpar(text: str, overrides: dict | None = None) -> dict:
    """Parse in.par text into {VARIABLE: value} like ReadVariables
    (src_main/Interpret.c:64-148).  Missing mandatory keys raise."""
    values = {name: _convert(typ, dflt) for name, (typ, mand, dflt) in _TABLE.items() if not mand}
    seen = set()
    for line in text.splitlines():
        toks = line.split()
        if not toks or toks[0].startswith("#"):
            continue
        key = toks[0].upper()
        rest = line.strip()[len(toks[0]):].lstrip("\t :=>_")
        val = rest.split()[0] if rest.split() else ""
        if key not in _TABLE:
            warnings.warn(f"variable {key} defined but non-existent in code")
            continue
        typ = _TABLE[key][0]
        values[key] = _convert(typ, val)
        seen.add(key)
    for k, v in (overrides or {}).items():
        values[k.upper()] = v
        seen.add(k.upper())
    missing = [n for n, (t, m, d) in _TABLE.items() if m and n not in seen]
    if missing:
        raise ValueError(f"undefined mandatory variable(s): {missing}")
    return values


class ThorinParams(C.Structure):
    """ctypes mirror of thorin_params (include/thorin_gpu.h)."""
    _fields_ = [
        ("nrad", C.c_int), ("nsec", C.c_int), ("log_grid", C.c_int), ("rmin", C.c_double), ("rmax", C.c_double),
        ("sigma0", C.c_double), ("sigma_slope", C.c_double), ("aspect_ratio", C.c_double),
        ("flaring_index", C.c_double), ("scaling_factor", C.c_double),
        ("cavity_radius", C.c_double), ("cavity_ratio", C.c_double), ("cavity_width", C.c_double),
        ("lambda_doubling", C.c_double), ("transition_radius", C.c_double), ("transition_ratio", C.c_double),
        ("transition_width", C.c_double),
        ("viscosity", C.c_double), ("alpha_viscosity", C.c_double), ("viscosity_alpha", C.c_int),
        ("alpha_flock", C.c_int), ("alpha_mri", C.c_double), ("alpha_dead", C.c_double), ("tmri", C.c_double),
        ("twidth", C.c_double),
        ("energy_eq", C.c_int), ("adiabind", C.c_double), ("cooling_time", C.c_double),
        ("parametric_cooling", C.c_int), ("stellar_irradiation", C.c_int), ("opacity_drop", C.c_double),
        ("effective_temperature", C.c_double), ("stellar_radius", C.c_double), ("disc_albedo", C.c_double),
        ("parametric_opacity", C.c_double), ("opacity_law", C.c_int),
        ("thickness_smoothing", C.c_double), ("exclude_hill", C.c_int), ("hillcut", C.c_double),
        ("indirect_term", C.c_int), ("mass_taper", C.c_double), ("vertical_damping", C.c_double),
        ("feel_disk", C.c_int), ("accretion_rate", C.c_double), ("gas_accret_heating", C.c_int),
        ("planetary_density", C.c_double), ("aerodynamic_drag", C.c_int),
        ("omega_frame", C.c_double), ("fast_transport", C.c_int),
        ("damping", C.c_int), ("damp_vrad", C.c_int), ("damp_init", C.c_int), ("damp_flux", C.c_int),
        ("damping_rmin_frac", C.c_double), ("damping_rmax_frac", C.c_double), ("damping_period_frac", C.c_double),
        ("gasflux", C.c_double), ("open_inner", C.c_int), ("open_outer", C.c_int), ("non_reflecting", C.c_int),
        ("outer_source_mass", C.c_int), ("imposed_disk_drift", C.c_double),
        ("dt", C.c_double), ("first_step", C.c_double), ("minimum_step", C.c_double), ("maximum_step", C.c_double),
        ("sloppy_cfl", C.c_int),
        ("pebbles", C.c_int), ("back_reaction", C.c_int), ("accret_heating", C.c_int),
        ("diffusive_particles", C.c_int), ("pebble_gravity", C.c_int),
        ("pebble_alpha", C.c_double), ("pebble_bulk_dens", C.c_double), ("schmidt_number", C.c_double),
        ("pebble_flux", C.c_double), ("pebble_coagulation", C.c_double), ("pebble_to_gas_max", C.c_double),
        ("fragment_factor", C.c_double), ("fragment_threshold", C.c_double), ("fragment_alpha", C.c_double),
        ("evaporation_rate", C.c_double), ("evaporation_temperature", C.c_double), ("heating_delay", C.c_int),
        ("parametric_accretion", C.c_double), ("prescribed_accretion", C.c_int),
        ("sor_eps", C.c_double), ("sor_maxiters", C.c_int), ("centrifugal_balance", C.c_int),
        ("label_advection", C.c_int), ("corotating", C.c_int), ("guiding_center", C.c_int),
    ]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_PLANET_ARRAYS = ("mass", "gas", "solid", "x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "acc")


class ThorinPlanets(C.Structure):
    """ctypes mirror of thorin_planets."""
    _fields_ = [("nb", C.c_int)] + [(n, C.c_double * MAXPLANETS) for n in _PLANET_ARRAYS] + \
               [("feel_disk", C.c_int * MAXPLANETS)]

    def copy(self):
        c = ThorinPlanets()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(ThorinPlanets))
        return c

    def state(self):
        n = self.nb
        return {k: list(getattr(self, k)[:n]) for k in ("mass", "x", "y", "z", "vx", "vy", "vz")}


class ThorinTorque(C.Structure):
    """One line of tqwk<k>.dat (UpdateLog, src_main/Force.c:27-70)."""
    _fields_ = [("time", C.c_double), ("torque", C.c_double), ("torque_norm", C.c_double), ("x", C.c_double),
                ("y", C.c_double), ("ax", C.c_double), ("ay", C.c_double)]

    def row(self):
        return (self.time, self.torque, self.torque_norm, self.x, self.y, self.ax, self.ay)


class ThorinStats(C.Structure):
    _fields_ = [("substeps", C.c_int), ("sor_calls", C.c_int), ("sor_sweeps", C.c_longlong),
                ("sor_last_niter", C.c_int), ("sor_omega", C.c_double), ("crashed", C.c_int),
                ("physical_time", C.c_double), ("last_dt", C.c_double), ("sor_time_ms", C.c_double),
                ("sor_passes", C.c_longlong), ("step_time_ms", C.c_double), ("kernel_launches", C.c_longlong),
                ("omega_frame", C.c_double)]


def _yes(s: str, ch: str) -> bool:
    return len(s) > 0 and s[0] in (ch.lower(), ch.upper())


def derive(v: dict, *, sor_eps: float = SOREPS, sor_maxiters: int = SORMAXITERS,
           scaling_factor: float = 1.0, sloppy_cfl: bool = False, centrifugal_balance: bool = False) -> ThorinParams:
    """Build thorin_params from parsed variables with the switch logic of
    src_main/Interpret.c:149-265."""
    p = ThorinParams()
    p.nrad, p.nsec = v["NRAD"], v["NSEC"]
    p.log_grid = int(_yes(v["RADIALSPACING"], "L"))
    p.rmin, p.rmax = v["RMIN"], v["RMAX"]
    p.sigma0, p.sigma_slope, p.aspect_ratio = v["SIGMA0"], v["SIGMASLOPE"], v["ASPECTRATIO"]
    p.flaring_index = v["FLARINGINDEX"]
    p.scaling_factor = scaling_factor
    p.cavity_radius, p.cavity_ratio, p.cavity_width = v["CAVITYRADIUS"], v["CAVITYRATIO"], v["CAVITYWIDTH"]
    p.lambda_doubling = v["LAMBDADOUBLING"]
    p.transition_radius, p.transition_ratio = v["TRANSITIONRADIUS"], v["TRANSITIONRATIO"]
    p.transition_width = v["TRANSITIONWIDTH"]
    p.viscosity, p.alpha_viscosity = v["VISCOSITY"], v["ALPHAVISCOSITY"]
    if p.alpha_viscosity != 0.0 and p.viscosity != 0.0:
        raise ValueError("You cannot use at the same time VISCOSITY and ALPHAVISCOSITY.")
    p.viscosity_alpha = int(p.alpha_viscosity != 0.0)
    p.alpha_flock = int(_yes(v["ALPHAFLOCK"], "Y"))
    p.alpha_mri, p.alpha_dead, p.tmri, p.twidth = v["ALPHAMRI"], v["ALPHADEAD"], v["TMRI"], v["TWIDTH"]
    p.energy_eq = int(_yes(v["ENERGYEQUATION"], "Y"))
    p.adiabind = v["ADIABIND"]
    p.cooling_time = v["COOLINGTIME"]
    p.parametric_cooling = int(p.cooling_time > 0.0)
    p.stellar_irradiation = int(_yes(v["STELLARIRRADIATION"], "Y"))
    p.opacity_drop, p.effective_temperature = v["OPACITYDROP"], v["EFFECTIVETEMPERATURE"]
    p.stellar_radius, p.disc_albedo = v["STELLARRADIUS"], v["DISCALBEDO"]
    p.parametric_opacity = v["PARAMETRICOPACITY"]
    tab = v["OPACITYTABLE"]
    if p.parametric_opacity > 0.0:
        p.opacity_law = 3
    elif tab[:1] == "Z":
        p.opacity_law = 1
    elif tab[:1] == "L":
        p.opacity_law = 2
    elif tab[:1] == "S":
        p.opacity_law = 4
    else:
        p.opacity_law = 0
    ts, rs = v["THICKNESSSMOOTHING"], v["ROCHESMOOTHING"]
    if ts != 0.0 and rs != 0.0:
        raise ValueError("You cannot use at the same time ThicknessSmoothing and RocheSmoothing.")
    if ts <= 0.0 and rs <= 0.0:
        raise ValueError("A non-vanishing potential smoothing length is required.")
    p.thickness_smoothing = ts
    p.exclude_hill = int(_yes(v["EXCLUDEHILL"], "Y"))
    p.hillcut = v["HILLCUT"]
    p.indirect_term = int(not _yes(v["INDIRECTTERM"], "N"))
    p.mass_taper = v["MASSTAPER"]
    p.vertical_damping = v["VERTICALDAMPING"]
    p.feel_disk = int(_yes(v["PLANETSFEELDISK"], "Y"))
    p.accretion_rate = v["ACCRETIONRATE"]
    p.gas_accret_heating = int(_yes(v["GASACCRETIONHEATING"], "Y"))
    p.planetary_density = v["PLANETARYDENSITY"]
    p.aerodynamic_drag = int(_yes(v["AERODYNAMICDRAG"], "Y"))
    p.omega_frame = v["OMEGAFRAME"]
    p.guiding_center = int(_yes(v["FRAME"], "G"))          # Interpret.c:165-169
    p.corotating = int(_yes(v["FRAME"], "C") or p.guiding_center)
    p.fast_transport = int(not _yes(v["TRANSPORT"], "S"))
    ib, ob = v["INNERBOUNDARY"], v["OUTERBOUNDARY"]
    p.open_inner = int(_yes(ib, "O"))
    p.non_reflecting = int(_yes(ib, "N"))
    p.open_outer = int(_yes(ob, "O"))
    p.outer_source_mass = int(_yes(v["OUTERSOURCEMASS"], "Y"))
    p.damping = int(_yes(ib, "D") or _yes(ob, "D") or _yes(v["DAMPING"], "Y"))
    dtw = v["DAMPTOWARDS"]
    p.damp_vrad, p.damp_init, p.damp_flux = int(_yes(dtw, "Z")), int(_yes(dtw, "I")), int(_yes(dtw, "G"))
    p.damping_rmin_frac, p.damping_rmax_frac = v["DAMPINGRMINFRAC"], v["DAMPINGRMAXFRAC"]
    p.damping_period_frac = v["DAMPINGPERIODFRAC"]
    p.gasflux = v["GASFLUX"]
    p.imposed_disk_drift = v["IMPOSEDDISKDRIFT"]
    p.dt = v["DT"]
    p.first_step, p.minimum_step, p.maximum_step = v["FIRSTSTEP"], v["MINIMUMSTEP"], v["MAXIMUMSTEP"]
    p.sloppy_cfl = int(sloppy_cfl)
    p.pebbles = int(_yes(v["PEBBLEACCRETION"], "Y"))
    p.back_reaction = int(_yes(v["BACKREACTION"], "Y"))
    p.accret_heating = int(_yes(v["ACCRETIONALHEATING"], "Y"))
    p.diffusive_particles = 1          # Interpret.c:241 assigns 'Y' instead of comparing
    p.pebble_gravity = int(_yes(v["PEBBLEGRAVITY"], "Y"))
    p.pebble_alpha, p.pebble_bulk_dens = v["PEBBLEALPHA"], v["PEBBLEBULKDENS"]
    p.schmidt_number, p.pebble_flux = v["SCHMIDTNUMBER"], v["PEBBLEFLUX"]
    p.pebble_coagulation, p.pebble_to_gas_max = v["PEBBLECOAGULATION"], v["PEBBLETOGASMAX"]
    p.fragment_factor, p.fragment_threshold = v["FRAGMENTFACTOR"], v["FRAGMENTTHRESHOLD"]
    p.fragment_alpha = v["FRAGMENTALPHA"]
    p.evaporation_rate, p.evaporation_temperature = v["EVAPORATIONRATE"], v["EVAPORATIONTEMPERATURE"]
    p.heating_delay = v["HEATINGDELAY"]
    p.parametric_accretion = v["PARAMETRICACCRETION"]
    p.prescribed_accretion = int(p.parametric_accretion > 0.0)
    p.sor_eps, p.sor_maxiters = sor_eps, sor_maxiters
    p.centrifugal_balance = int(centrifugal_balance)
    p.label_advection = int(_yes(v["LABELADVECTION"], "Y"))
    return p


def check_supported(p: ThorinParams) -> None:
    """Raise for options outside the implemented hot path (fail loudly)."""
    bad = []
    if bad:
        raise NotImplementedError("unsupported options: " + ", ".join(bad))


def read_planet_config(text: str):
    """Planet lines of a planet config file as SetupReboundSimulation reads
    them (ReboundInterface.c:157-195): lines starting with a letter; nine
    floats after the name: mass gas solid a e inc Omega omega f."""
    out = []
    for line in text.splitlines():
        if not line[:1].isalpha():
            continue
        toks = line.split()
        vals = [float(t) for t in toks[1:10]]
        if len(vals) != 9:
            raise ValueError(f"Error reading planet line {line!r}")
        out.append(vals)
    return out


def orbit_elements(m, x, y, z, vx, vy, vz):
    """Semi-major axis, eccentricity, inclination and mean anomaly of a body
    of mass m about a unit-mass primary at rest at the origin (G = 1), as
    REBOUND's reb_tools_particle_to_orbit defines them (src_reb/tools.c:
    578-686; Murray & Dermott ch. 2)."""
    def acos_ratio(num, den, sign):
        c = num / den if den != 0.0 else math.nan
        if -1.0 < c < 1.0:
            v = math.acos(c)
            return -v if sign < 0.0 else v
        return math.pi if c <= -1.0 else 0.0
    mu = m + 1.0
    d = math.sqrt(x * x + y * y + z * z)
    v2 = vx * vx + vy * vy + vz * vz
    vc2 = mu / d
    a = -mu / (v2 - 2.0 * vc2)
    hx, hy, hz = y * vz - z * vy, z * vx - x * vz, x * vy - y * vx
    h = math.sqrt(hx * hx + hy * hy + hz * hz)
    vr = (x * vx + y * vy + z * vz) / d
    rvr, muinv, vd2 = d * vr, 1.0 / mu, v2 - vc2
    ex, ey, ez = (muinv * (vd2 * x - rvr * vx), muinv * (vd2 * y - rvr * vy), muinv * (vd2 * z - rvr * vz))
    e = math.sqrt(ex * ex + ey * ey + ez * ez)
    inc = acos_ratio(hz, h, 1.0)
    if e < 1.0:
        ea = acos_ratio(1.0 - d / a, e, vr)
        mean = ea - e * math.sin(ea)
    else:
        ea = math.acosh((1.0 - d / a) / e)
        ea = -ea if vr < 0.0 else ea
        mean = e * math.sinh(ea) - ea
    return a, e, inc, mean


def corotating_frame(p: ThorinParams, planets) -> None:
    """Frame COROTATING: the run starts in the frame of planet 0, rotating at
    its angular speed (x vy - y vx) / (x^2 + y^2); Frame GUIDINGCENTER: at
    the mean motion sqrt((1 + m) / a^3) of its orbit (GetPsysInfo FREQUENCY,
    Psys.c:195-262; main.c:161)."""
    if p.corotating:
        if planets.nb < 1:
            raise ValueError("Frame COROTATING needs a planet")
        x, y, vx, vy = planets.x[0], planets.y[0], planets.vx[0], planets.vy[0]
        if p.guiding_center:
            a = orbit_elements(planets.mass[0], x, y, planets.z[0], vx, vy, planets.vz[0])[0]
            p.omega_frame = math.sqrt((planets.mass[0] + 1.0) / (a * a * a))
        else:
            p.omega_frame = (x * vy - y * vx) / (x * x + y * y)


def read_opacity_table(path: str):
    """InitOpacities (Opacity2.c:247-297): rows, cols, pressure grid,
    temperature grid, Planck table, Rosseland table (whitespace-separated)."""
    import numpy as np
    with open(path) as f:
        tok = f.read().split()
    rows, cols = int(tok[0]), int(tok[1])
    v = np.array([float(t) for t in tok[2:2 + rows + cols + 2 * rows * cols]], dtype=np.float64)
    pgrid, tgrid = v[:rows], v[rows:rows + cols]
    planck = v[rows + cols:rows + cols + rows * cols]
    rosseland = v[rows + cols + rows * cols:]
    return rows, cols, pgrid, tgrid, planck, rosseland

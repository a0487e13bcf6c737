"""Named workloads and host-side set-up helpers.

The two plain-method workloads are the disk set-ups the hydro loop is
measured on:

* ``disk0``: gas-only non-isothermal disk, log-spaced r in [0.4, 2.5],
  Sigma = 5e-4 r^-0.5 (1 + 1e-4 u), h = 0.05, alpha = 1e-3, gamma = 1.4,
  Bell & Lin opacity, SOR radiative diffusion, damping boundaries, a
  zero-mass planet at r = 1 (128 x 384 by default).
* ``disk1``: the same profiles plus a pebble fluid with Sigma_p = 0.01 Sigma
  and Stokes number 0.1, outer-edge pebble inflow (damping towards the
  initial pebble state), and a 3e-5 M* embryo at r = 1 that feels the disk,
  accretes pebbles and heats the gas (1024 x 3072 by default).

The perturbed, v_r = 0 initial state is what the reference produces with
InitializeFromFile (src_main/Init.c:86-105) from its own initial dump; the
pebble state is what its restart path reads (Init.c:109-129,
Pebbles.c:66-75).  Both are reproduced here by overwriting the library's
default initial fields and refreshing the derived quantities.
"""
from __future__ import annotations

import math

import numpy as np

from .params import ThorinPlanets, derive, read_inpar

PI = 3.14159265358979323844          # src_main/fondam.h:14
RHO2CGS = 1.98855e30 * 1000.0 / (149597870700.0 * 100.0) ** 3

_DISK0 = """
AspectRatio 0.05
AlphaViscosity 1.0e-3
SigmaSlope 0.5
FlaringIndex 0.0
Sigma0 5.0e-4
OpacityTable BL94
EnergyEquation YES
Adiabind 1.4
CoolingTime -1.0
StellarIrradiation NO
ThicknessSmoothing 0.6
Transport FARGO
InnerBoundary DAMPING
DampTowards ZEROVRAD
Disk YES
OmegaFrame 0.0
Frame Fixed
IndirectTerm YES
Rmin 0.4
Rmax 2.5
RadialSpacing Logarithmic
Ntot 200
Ninterm 200
DT 0.0314159265358979
OutputDir out
PlanetsFeelDisk NO
"""

_DISK1_EXTRA = """
PlanetsFeelDisk YES
PebbleAccretion YES
BackReaction YES
AccretionalHeating YES
"""

PLANET0 = (0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0)        # zero-mass planet at r = 1
PLANET1 = (3.0e-5, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0)     # 10 Earth-mass embryo at r = 1


def inpar_text(kind: str, nrad: int, nsec: int) -> str:
    base = _DISK0 + f"Nrad {nrad}\nNsec {nsec}\n"
    if kind == "disk1":
        base += _DISK1_EXTRA
    return base


def params_for(kind: str, nrad: int, nsec: int, sor_eps: float | None = None, **over):
    v = read_inpar(inpar_text(kind, nrad, nsec), over or None)
    kw = {}
    if sor_eps is not None:
        kw["sor_eps"] = sor_eps
    return derive(v, **kw)


def planet_from_elements(mass, gas, solid, a, e, inc, Omega, omega, f):
    """Heliocentric planet state as SetupReboundSimulation builds it: the nine
    numbers are read as C floats (ReboundInterface.c:137-163), angles are in
    degrees (rad = PI/180, :144), and reb_tools_orbit_to_particle_err follows
    Murray & Dermott eqs. 2.122 and 2.36 for a unit-mass primary at the
    origin."""
    f32 = [float(np.float32(v)) for v in (mass, gas, solid, a, e, inc, Omega, omega, f)]
    m, g, s, a, e, inc, Om, om, f = f32
    rad = PI / 180.0
    inc, Om, om, f = inc * rad, Om * rad, om * rad, f * rad
    r = a * (1 - e * e) / (1 + e * math.cos(f))
    v0 = math.sqrt(1.0 * (m + 1.0) / a / (1. - e * e))
    cO, sO, co, so = math.cos(Om), math.sin(Om), math.cos(om), math.sin(om)
    cf, sf, ci, si = math.cos(f), math.sin(f), math.cos(inc), math.sin(inc)
    x = 0.0 + r * (cO * (co * cf - so * sf) - sO * (so * cf + co * sf) * ci)
    y = 0.0 + r * (sO * (co * cf - so * sf) + cO * (so * cf + co * sf) * ci)
    z = 0.0 + r * (so * cf + co * sf) * si
    vx = 0.0 + v0 * ((e + cf) * (-ci * co * sO - cO * so) - sf * (co * cO - ci * so * sO))
    vy = 0.0 + v0 * ((e + cf) * (ci * co * cO - sO * so) - sf * (co * sO + ci * so * cO))
    vz = 0.0 + v0 * ((e + cf) * co * si - sf * si * so)
    return dict(mass=m, gas=g, solid=s, x=x, y=y, z=z, vx=vx, vy=vy, vz=vz)


def make_planets(params, rows) -> ThorinPlanets:
    sys_ = ThorinPlanets()
    sys_.nb = len(rows)
    for k, row in enumerate(rows):
        st = planet_from_elements(*row)
        for key, val in st.items():
            getattr(sys_, key)[k] = val
        sys_.acc[k] = params.accretion_rate
        sys_.feel_disk[k] = params.feel_disk
    return sys_


def perturbation(nrad: int, nsec: int, seed: int = 0) -> np.ndarray:
    """u ~ U(-1, 1) per cell in row-major (l = j + i*nsec) order."""
    return np.random.default_rng(seed).uniform(-1.0, 1.0, nrad * nsec)


def perturbed_state(params, fields: dict, seed: int = 0) -> dict:
    """From the default initial fields (dens, vtheta, temper and, with
    pebbles, pebble velocities) build the measured initial state:
    Sigma' = Sigma (1 + 1e-4 u), v_r = 0, e = T Sigma' / (gamma - 1) with the
    initial T, and with pebbles Sigma_p = 0.01 Sigma' and a pebble size that
    gives Stokes number 0.1 through the Epstein law of Pebbles.c:297."""
    nr, ns = params.nrad, params.nsec
    n = nr * ns
    u = perturbation(nr, ns, seed)
    out = {}
    dens = fields["dens"][:n] * (1.0 + 1e-4 * u)
    out["dens"] = dens
    out["vrad"] = np.zeros(n)
    out["energy"] = fields["temper"][:n] * dens / (params.adiabind - 1.0)
    if params.pebbles:
        pebbulkdens = params.pebble_bulk_dens / RHO2CGS
        out["pebdens"] = 0.01 * dens
        out["pebsize"] = 0.1 * dens * math.sqrt(params.adiabind) / (2.0 * pebbulkdens)
    return out

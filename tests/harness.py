"""Shared set-up for the parity tests: golden cases and initial states."""
from __future__ import annotations

import os

import numpy as np

from fargo_thorin_gb300 import workloads
from fargo_thorin_gb300.params import corotating_frame, derive, read_inpar

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

FIELD_IDS = {"dens": 0, "vrad": 1, "vtheta": 2, "energy": 3, "pebbledens": 4, "pebblevrad": 5,
             "pebblevtheta": 6, "pebblesize": 7, "temper": 8, "soundspeed": 9, "pressure": 10,
             "pebblestokes": 11, "qplus": 12, "divv": 13, "opacity": 14, "qminus": 15, "label": 16}
GAS = ["dens", "vrad", "vtheta", "temper"]
PEB = ["pebbledens", "pebblevrad", "pebblevtheta"]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def case_params(g, **kw):
    flags = str(g["flags"]) if "flags" in g.files else ""
    if "soreps" in g.files:                           # a reference build with another SOR tolerance
        kw.setdefault("sor_eps", float(g["soreps"]))
    p = derive(read_inpar(str(g["inpar"])), centrifugal_balance="b" in flags, sloppy_cfl="c" in flags, **kw)
    if p.corotating:                                  # the frame of planet 0 (main.c:161)
        corotating_frame(p, workloads.make_planets(p, [tuple(g["planet"])]))
    return p


def opacity_table(disk, g):
    """Give the disk the golden run's SM03 gas-opacity table, if it has one."""
    if "sm_rows" in g.files:
        disk.set_opacity_table(int(g["sm_rows"]), int(g["sm_cols"]), g["sm_pgrid"], g["sm_tgrid"], g["sm_planck"],
                               g["sm_rosseland"])


def start_state(disk, params, init_fields, seed=0):
    """Apply the measured initial state (perturbed Sigma, v_r = 0, pebble
    overrides) on top of a disk that holds the default initial fields, then
    refresh derived quantities like the reference's InitializeFromFile
    (gas-only) or restart (pebbles) path."""
    st = workloads.perturbed_state(params, init_fields, seed=seed)
    disk.set(FIELD_IDS["dens"], st["dens"])
    disk.set(FIELD_IDS["vrad"], st["vrad"])
    if params.energy_eq:                            # isothermal runs do not read TemperInfile (Init.c:96)
        disk.set(FIELD_IDS["energy"], st["energy"])
    if params.pebbles:
        disk.set(FIELD_IDS["pebbledens"], st["pebdens"])
        disk.set(FIELD_IDS["pebblesize"], st["pebsize"])
        disk.refresh(2)
    else:
        disk.refresh(1)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def mass_momentum(rings, rho, vtheta, omega_frame=0.0):
    """GasTotalMass and GasMomentum (src_main/SideEuler.c:26-60) of a density
    and azimuthal velocity given as (nrad, nsec) arrays, summed by numpy; the
    reference applies the same two sums to the pebble fluid.  rings = (Rinf,
    Rsup, Rmed, Surf)."""
    _, _, rmed, surf = (np.asarray(a)[:, None] for a in rings)
    rho = np.asarray(rho)
    vt = np.asarray(vtheta) + omega_frame * rmed
    mass = float(np.sum(surf * rho))
    mom = 0.5 * float(np.sum(surf * (rho + np.roll(rho, 1, axis=1)) * rmed * vt))
    return mass, mom

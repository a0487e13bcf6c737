"""Generate golden fixtures from the reference FARGO_THORIN binary.

Builds the reference's sequential binary from its sources with
oracle/ref.mk (into oracle/_ref/), runs it on small disk set-ups and stores
its outputs as .npz fixtures next to this script.  Needs the reference tree
(the directory $THORIN_REFERENCE names); the fixtures it writes are
committed so that the tests never need the reference at run time.

Each case runs the reference twice, like the measured workloads prescribe:
``thorin -0`` dumps the default initial state, that state is perturbed
(Sigma (1 + 1e-4 u), v_r = 0, and for pebble cases Sigma_p = 0.01 Sigma with
Stokes number 0.1), and the perturbed state is fed back through the
reference's own InitializeFromFile (gas only) or restart (-s 0, pebbles)
path.  Recorded: the initial dump, field dumps after chosen DTs, the -a
integrals after every DT, the -d SOR iteration counts and CFL substep counts,
and the planet state of the torque log (tqwk0.dat, written every DT).

Usage: THORIN_REFERENCE=<reference tree> python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from fargo_thorin_gb300 import workloads  # noqa: E402

REF = os.environ.get("THORIN_REFERENCE", "")
REF_OUT = os.path.join(ROOT, "oracle", "_ref")

# Stellar irradiation and its parameters as the reference's shipped
# in_relax/in.par sets them (lines 9-21)
IRRADIATION = ("StellarIrradiation YES\nOpacityDrop 0.6\nEffectiveTemperature 4370.0\nStellarRadius 1.5\n"
               "DiscAlbedo 0.5\n")

# name: (kind, nrad, nsec, ntot, ninterm, extra in.par lines, full-field snapshots?
#        [, planet row [, command-line flags [, SOREPS of the reference build]]])
# full: True = every output in full; "last" = the last output in full and
# sampled rows + ring means before it; False = sampled rows + ring means only
CASES = {
    "disk0_24x72": ("disk0", 24, 72, 4, 1, "", True),
    "disk1_32x96": ("disk1", 32, 96, 3, 1, "", True),
    "disk0_128x384_200": ("disk0", 128, 384, 200, 100, "", "last"),
    "disk1_64x192_40": ("disk1", 64, 192, 40, 20, "", False),
    # in.par options beyond the two measured set-ups
    "iso_24x72": ("disk0", 24, 72, 6, 2, "EnergyEquation NO\nWriteTemperature YES\n", True),
    "iso_peb_32x96": ("disk1", 32, 96, 6, 2, "EnergyEquation NO\nWriteTemperature YES\n", True),
    "dampinit_24x72": ("disk0", 24, 72, 6, 2, "DampTowards INIT\n", True),
    "gasflux_24x72": ("disk0", 24, 72, 6, 2, "DampTowards GASFLUX\nGasFlux 1e-8\n", True),
    "frame_24x72": ("disk0", 24, 72, 6, 2, "OmegaFrame 1.0\n", True),
    "open_24x72": ("disk0", 24, 72, 6, 2, "InnerBoundary OPEN\nOuterBoundary OPEN\n", True),
    "nonrefl_24x72": ("disk0", 24, 72, 6, 2, "InnerBoundary NONREFLECTING\n", True),
    "srcmass_24x72": ("disk0", 24, 72, 6, 2, "OuterSourceMass YES\n", True),
    "cooling_24x72": ("disk0", 24, 72, 6, 2, "CoolingTime 10.0\n", True),
    # planets: a Jupiter-mass planet accreting gas (Kley), a pebble-disk embryo
    # growing at a prescribed rate, and a small body braked by gas drag
    "gasacc_24x72": ("disk0", 24, 72, 6, 2, "AccretionRate 1.0\nPlanetsFeelDisk YES\n", True,
                     (1.0e-3, 0.0, 0.0, 1.05, 0.0, 0.0, 0.0, 0.0, 0.0)),
    "paracc_32x96": ("disk1", 32, 96, 6, 2, "ParametricAccretion 10.0\n", True, None),
    "drag_24x72": ("disk0", 24, 72, 6, 2, "AerodynamicDrag YES\nPlanetsFeelDisk YES\n", True,
                   (1.0e-7, 0.0, 0.0, 1.05, 0.05, 0.0, 0.0, 0.0, 0.0)),
    # command-line switch -b: v_theta from the centrifugal balance
    "cbal_24x72": ("disk0", 24, 72, 6, 2, "", True, None, "b"),
    "label_24x72": ("disk0", 24, 72, 6, 2, "LabelAdvection YES\n", True),
    "corot_24x72": ("disk0", 24, 72, 6, 2, "Frame COROTATING\n", True),
    "corot_peb_32x96": ("disk1", 32, 96, 6, 2, "Frame COROTATING\n", True),
    # OpacityTable SM03 with a synthetic gas table (the run reads it from in/)
    "sm03_24x72": ("disk0", 24, 72, 6, 2, "OpacityTable SM03\n", True),
    # command-line switch -c: one CFL per DT (and a DT long enough to need substeps)
    "sloppy_peb_32x96": ("disk1", 32, 96, 6, 2, "DT 0.4\n", True, None, "c"),
    # the opacity laws and the stellar irradiation of the shipped examples
    "zhu12irr_24x72": ("disk0", 24, 72, 6, 2, "OpacityTable ZHU12\n" + IRRADIATION, True),
    "zhu12irr_peb_32x96": ("disk1", 32, 96, 6, 2, "OpacityTable ZHU12\n" + IRRADIATION, True),
    "lp85_24x72": ("disk0", 24, 72, 6, 2, "OpacityTable LP85\n", True),
    "lp85irr_24x72": ("disk0", 24, 72, 6, 2, "OpacityTable LP85\n" + IRRADIATION, True),
    "constopa_24x72": ("disk0", 24, 72, 6, 2, "ParametricOpacity 2.0\n", True),
    "bl94irr_24x72": ("disk0", 24, 72, 6, 2, IRRADIATION, True),
    # the pebble + embryo disk at the SOR tolerance of the measured workload
    # (SOREPS is a compile-time constant of the reference, EnergySources.c:23)
    "disk1_48x144_eps8": ("disk1", 48, 144, 10, 5, "", True, None, "", "1e-8"),
    # the guiding-centre frame follows an eccentric, inclined planet
    "gc_24x72": ("disk0", 24, 72, 6, 2, "Frame GUIDINGCENTER\nPlanetsFeelDisk YES\n", True,
                 (1.0e-5, 0.0, 0.0, 1.05, 0.03, 1.0, 0.0, 0.0, 30.0)),
    "gc_peb_32x96": ("disk1", 32, 96, 6, 2, "Frame GUIDINGCENTER\n", True,
                     (3.0e-5, 0.0, 0.0, 1.05, 0.03, 1.0, 0.0, 0.0, 30.0)),
}


def synthetic_gas_table(rows=40, cols=30):
    """A smooth made-up gas-opacity table in the layout of
    data_gasopacity_malygin.txt: log-spaced pressures and temperatures,
    Rosseland kappa = 1e-3 (T/100)^1.5 (P/1)^0.2, Planck twice that."""
    pgrid = np.logspace(-6.0, 8.0, rows)
    tgrid = np.logspace(np.log10(50.0), 4.0, cols)
    P, T = np.meshgrid(pgrid, tgrid, indexing="ij")
    ross = 1e-3 * (T / 100.0) ** 1.5 * P ** 0.2
    return rows, cols, pgrid, tgrid, 2.0 * ross.ravel(), ross.ravel()


def write_gas_table(path, table):
    rows, cols, pgrid, tgrid, planck, ross = table
    with open(path, "w") as f:
        f.write(f"{rows} {cols}\n")
        for arr in (pgrid, tgrid, planck, ross):
            f.write("\n".join("%.17g" % v for v in arr) + "\n")
GAS = ["dens", "vrad", "vtheta", "temper"]
PEB = ["pebbledens", "pebblevrad", "pebblevtheta"]
SAMPLE_ROWS_FRAC = [0.0, 0.3, 0.5, 0.75, 1.0]


def build_reference(soreps=""):
    if not REF or not os.path.isdir(os.path.join(REF, "src_main")):
        sys.exit("set THORIN_REFERENCE to the reference FARGO_THORIN source tree")
    extra = [f"SOREPS={soreps}"] if soreps else []
    subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref.mk"), f"REF={REF}", *extra], check=True)
    return os.path.join(REF_OUT, "thorin" + (f"_soreps{soreps}" if soreps else ""))


def read_dump(out, name, k, nr, ns):
    return np.fromfile(os.path.join(out, f"gas{name}{k}.dat"), dtype="<f8").reshape(nr, ns)


def run(cmd, cwd):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed: {r.stdout[-2000:]} {r.stderr[-2000:]}")
    return r.stdout


def parse_log(text):
    """Per-DT integrals, SOR Niter per solve, CFL substeps per DT."""
    mom, mass, ener, niter, subs = [], [], [], [], []
    cfl_calls = 0
    for line in text.splitlines():
        if "Limit time step adopted" in line:
            cfl_calls += 1
        m = re.search(r"SOR: Niter = (\d+)", line)
        if m and "omega" not in line:
            niter.append(int(m.group(1)))
        if line.startswith("Gas Momentum"):
            mom.append(float(line.split(":")[1]))
            subs.append(cfl_calls)
            cfl_calls = 0
        elif line.startswith("Gas total Mass"):
            mass.append(float(line.split(":")[1]))
        elif line.startswith("Gas total Energy"):
            ener.append(float(line.split(":")[1]))
    return dict(momentum=np.array(mom), mass=np.array(mass), energy=np.array(ener),
                sor_niter=np.array(niter, dtype=np.int64), substeps=np.array(subs, dtype=np.int64))


def make_case(name):
    kind, nr, ns, ntot, ninterm, extra, full = CASES[name][:7]
    planet_override = CASES[name][7] if len(CASES[name]) > 7 else None
    flags = CASES[name][8] if len(CASES[name]) > 8 else ""
    soreps = CASES[name][9] if len(CASES[name]) > 9 else ""
    THORIN = build_reference(soreps)
    work = tempfile.mkdtemp(prefix="thorin_golden_")
    try:
        out = os.path.join(work, "out")
        par = workloads.inpar_text(kind, nr, ns) + extra
        par = re.sub(r"Ntot \d+", f"Ntot {ntot}", par)
        par = re.sub(r"Ninterm \d+", f"Ninterm {ninterm}", par)
        par = par.replace("OutputDir out", f"OutputDir {out}")
        planet = workloads.PLANET1 if kind == "disk1" else workloads.PLANET0
        if planet_override is not None:
            planet = planet_override
        with open(os.path.join(work, "planet.cfg"), "w") as f:
            f.write("Embryo1 " + " ".join(repr(v) for v in planet) + "\n")
        par += f"PlanetConfig {os.path.join(work, 'planet.cfg')}\n"
        with open(os.path.join(work, "in.par"), "w") as f:
            f.write(par)
        table = None
        if "OpacityTable SM03" in extra:
            table = synthetic_gas_table()
            os.makedirs(os.path.join(work, "in"), exist_ok=True)
            write_gas_table(os.path.join(work, "in", "data_gasopacity_malygin.txt"), table)
        run([THORIN, "-0" + flags, "in.par"], work)
        init = {k: read_dump(out, k, 0, nr, ns) for k in GAS}
        if kind == "disk1":
            for k in PEB + ["pebblesize", "pebblestokes"]:
                init[k] = read_dump(out, k, 0, nr, ns)
        params = workloads.params_for(kind, nr, ns)
        st = workloads.perturbed_state(params, {"dens": init["dens"].ravel(), "temper": init["temper"].ravel()})
        if kind == "disk0":
            files = {"DensInfile": st["dens"], "VradInfile": st["vrad"],
                     "VthetaInfile": init["vtheta"].ravel(), "TemperInfile": init["temper"].ravel()}
            for key, arr in files.items():
                path = os.path.join(work, key + ".txt")
                np.savetxt(path, arr, fmt="%.17g")
                par += f"{key} {path}\n"
            par += "InitializeFromFile YES\n"
            with open(os.path.join(work, "in.par"), "w") as f:
                f.write(par)
            log = run([THORIN, "-ad" + flags, "in.par"], work)
        else:
            st["dens"].astype("<f8").tofile(os.path.join(out, "gasdens0.dat"))
            st["vrad"].astype("<f8").tofile(os.path.join(out, "gasvrad0.dat"))
            st["pebdens"].astype("<f8").tofile(os.path.join(out, "gaspebbledens0.dat"))
            st["pebsize"].astype("<f8").tofile(os.path.join(out, "gaspebblesize0.dat"))
            log = run([THORIN, "-ad" + flags, "-s", "0", "in.par"], work)
        res = {"inpar": np.array(par), "planet": np.array(planet), "flags": np.array(flags), "nrad": nr, "nsec": ns,
               "ntot": ntot, "ninterm": ninterm, "kind": np.array(kind)}
        if soreps:
            res["soreps"] = float(soreps)
        for k, v in init.items():
            res["init_" + k] = v
        if table is not None:
            for key, v in zip(("sm_rows", "sm_cols", "sm_pgrid", "sm_tgrid", "sm_planck", "sm_rosseland"), table):
                res[key] = v
        res.update(parse_log(log))
        names = GAS + (PEB if kind == "disk1" else []) + (["label"] if "LabelAdvection YES" in extra else [])
        rows = sorted({min(nr - 1, int(round(f * (nr - 1)))) for f in SAMPLE_ROWS_FRAC})
        res["sample_rows"] = np.array(rows)
        nout = ntot // ninterm
        for k in range(1, nout + 1):
            for fname in names:
                arr = read_dump(out, fname, k, nr, ns)
                if full is True or (full == "last" and k == nout):
                    res[f"out{k}_{fname}"] = arr
                else:
                    res[f"out{k}_{fname}_ringmean"] = arr.mean(axis=1)
                    res[f"out{k}_{fname}_rows"] = arr[rows]
                    res[f"out{k}_{fname}_l2"] = np.sqrt(np.sum(arr * arr))
        tq = np.loadtxt(os.path.join(out, "tqwk0.dat"), ndmin=2)
        res["tqwk"] = tq                      # t, tq, tq_norm, x, y, ax, ay (one line per DT)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "substeps", res["substeps"].tolist()[:10], "sor", res["sor_niter"].tolist()[:10])
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    for name in (sys.argv[1:] or list(CASES)):
        make_case(name)

"""Golden outputs of whole reference runs, for the host driver (run.py).

Runs the reference binary (built from its own sources by oracle/ref.mk into
oracle/_ref/thorin) the way a user does and records every file it writes:

* ``driver_init_disk1_20x60``: ``thorin -0 in.par`` (initial outputs only) of
  the pebble + embryo disk; the files' SHA-256 digests and the text files.
* ``driver_disk0_20x60``: the gas disk initialised from ASCII files
  (InitializeFromFile, perturbed Sigma, v_r = 0), ``thorin -a``, 5 DTs
  (Ntot 4), outputs every 2 DTs.
* ``driver_disk1_20x60``: the pebble + embryo disk restarted from output 0
  with overridden pebble fields (``thorin -a -s 0``), 5 DTs, outputs every 2.

The planet sits at a = 1.05, off the ring interfaces, so that the different
N-body integrators (REBOUND's IAS15 there, the library's RK4 here) give the
same cells near the planet.
Usage: THORIN_REFERENCE=<reference tree> python tests/golden/make_driver_golden.py
"""
from __future__ import annotations

import hashlib
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
THORIN = os.path.join(ROOT, "oracle", "_ref", "thorin")
NR, NS = 20, 60


def planet_row(kind):
    m = 3.0e-5 if kind == "disk1" else 0.0
    return (m, 0.0, 0.0, 1.05, 0.0, 0.0, 0.0, 0.0, 0.0)


def setup_dir(kind, ntot, ninterm):
    work = tempfile.mkdtemp(prefix="thorin_driver_")
    par = workloads.inpar_text(kind, NR, NS)
    par = re.sub(r"Ntot \d+", f"Ntot {ntot}", par)
    par = re.sub(r"Ninterm \d+", f"Ninterm {ninterm}", par)
    par = par.replace("OutputDir out", "OutputDir out")
    with open(os.path.join(work, "planet.cfg"), "w") as f:
        f.write("Embryo1 " + " ".join(repr(v) for v in planet_row(kind)) + "\n")
    par += "PlanetConfig planet.cfg\n"
    return work, par


def write_par(work, par):
    with open(os.path.join(work, "in.par"), "w") as f:
        f.write(par)


def run(cmd, cwd):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed: {r.stdout[-2000:]} {r.stderr[-2000:]}")
    return r.stdout


def integrals(log):
    out = {"momentum": [], "mass": [], "energy": []}
    for line in log.splitlines():
        if line.startswith("Gas Momentum"):
            out["momentum"].append(float(line.split(":")[1]))
        elif line.startswith("Gas total Mass"):
            out["mass"].append(float(line.split(":")[1]))
        elif line.startswith("Gas total Energy"):
            out["energy"].append(float(line.split(":")[1]))
    return {k: np.array(v) for k, v in out.items()}


def collect(outdir, res, binary_names, text_names):
    for name in binary_names:
        res["bin_" + name] = np.fromfile(os.path.join(outdir, name), dtype="<f8")
    for name in text_names:
        with open(os.path.join(outdir, name)) as f:
            res["txt_" + name] = np.array(f.read())


def make_init():
    work, par = setup_dir("disk1", 4, 2)
    try:
        write_par(work, par)
        run([THORIN, "-0", "in.par"], work)
        out = os.path.join(work, "out")
        res = {"inpar": np.array(par), "planet_cfg": np.array(open(os.path.join(work, "planet.cfg")).read())}
        for name in sorted(os.listdir(out)):
            with open(os.path.join(out, name), "rb") as f:
                res["sha256_" + name] = np.array(hashlib.sha256(f.read()).hexdigest())
        for name in ("used_rad.dat", "dims.dat"):
            with open(os.path.join(out, name)) as f:
                res["txt_" + name] = np.array(f.read())
        np.savez_compressed(os.path.join(HERE, "driver_init_disk1_20x60.npz"), **res)
    finally:
        shutil.rmtree(work, ignore_errors=True)


def make_run(kind):
    work, par = setup_dir(kind, 4, 2)
    try:
        out = os.path.join(work, "out")
        write_par(work, par)
        run([THORIN, "-0", "in.par"], work)
        rd = lambda n: np.fromfile(os.path.join(out, n), dtype="<f8")  # noqa: E731
        init = {"dens": rd("gasdens0.dat"), "temper": rd("gastemper0.dat")}
        params = workloads.params_for(kind, NR, NS)
        st = workloads.perturbed_state(params, init)
        res = {"kind": np.array(kind), "planet_cfg": np.array(open(os.path.join(work, "planet.cfg")).read())}
        if kind == "disk0":
            files = {"DensInfile": st["dens"], "VradInfile": st["vrad"], "VthetaInfile": rd("gasvtheta0.dat"),
                     "TemperInfile": init["temper"]}
            for key, arr in files.items():
                np.savetxt(os.path.join(work, key + ".txt"), arr, fmt="%.17g")
                res["ascii_" + key] = arr
                par += f"{key} {key}.txt\n"
            par += "InitializeFromFile YES\n"
            shutil.rmtree(out)
            write_par(work, par)
            log = run([THORIN, "-a", "in.par"], work)
        else:
            res["restart0_dens"] = st["dens"]
            res["restart0_vrad"] = st["vrad"]
            res["restart0_pebbledens"] = st["pebdens"]
            res["restart0_pebblesize"] = st["pebsize"]
            for name in ("vtheta", "temper", "pebblevrad", "pebblevtheta"):
                res["restart0_" + name] = rd(f"gas{name}0.dat")
            st["dens"].astype("<f8").tofile(os.path.join(out, "gasdens0.dat"))
            st["vrad"].astype("<f8").tofile(os.path.join(out, "gasvrad0.dat"))
            st["pebdens"].astype("<f8").tofile(os.path.join(out, "gaspebbledens0.dat"))
            st["pebsize"].astype("<f8").tofile(os.path.join(out, "gaspebblesize0.dat"))
            log = run([THORIN, "-a", "-s", "0", "in.par"], work)
        res["inpar"] = np.array(par)
        res.update({"int_" + k: v for k, v in integrals(log).items()})
        names = ["dens", "vrad", "vtheta", "temper"] + (["pebbledens", "pebblevrad", "pebblevtheta"]
                                                         if kind == "disk1" else [])
        binaries = [f"gas{n}{k}.dat" for n in names for k in (1, 2)]
        collect(out, res, binaries, ["tqwk0.dat", "used_rad.dat", "dims.dat"])
        np.savez_compressed(os.path.join(HERE, f"driver_{kind}_20x60.npz"), **res)
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    if not REF or not os.path.isdir(os.path.join(REF, "src_main")):
        sys.exit("set THORIN_REFERENCE to the reference FARGO_THORIN source tree")
    subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref.mk"), f"REF={REF}"], check=True)
    make_init()
    make_run("disk0")
    make_run("disk1")

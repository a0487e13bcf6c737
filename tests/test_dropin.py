"""The C drop-in (fargo_thorin_gb300/dropin/AlgoGasGPU.c): the reference's
own sequential build, with main.c's AlgoGas call switched to AlgoGasGPU and
linked against libthorin_gpu.so.

Needs the reference source tree ($THORIN_REFERENCE, or the one build()
recorded in oracle/_ref/REFERENCE); skipped where it is absent, e.g. on the
GPU machine.  Without a GPU the binary runs the reference's whole start-up (in.par,
initial state, outputs, REBOUND) and stops with an error at the first GPU
call, having written the thorin_params it built from the reference's globals;
these must equal what the Python in.par reader derives from the same file.
"""
import ctypes as C
import os
import subprocess

import pytest

from fargo_thorin_gb300 import workloads
from fargo_thorin_gb300.params import ThorinParams, derive, read_inpar

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MK = os.path.join(ROOT, "fargo_thorin_gb300", "dropin", "dropin.mk")
BIN = os.path.join(ROOT, "fargo_thorin_gb300", "_build", "dropin", "thorin_gpu")


def _reference():
    ref = os.environ.get("THORIN_REFERENCE", "")
    rec = os.path.join(ROOT, "oracle", "_ref", "REFERENCE")
    if not ref and os.path.exists(rec):
        ref = open(rec).read().strip()
    if not ref or not os.path.isdir(os.path.join(ref, "src_main")):
        pytest.skip("reference source tree not available")
    return ref


@pytest.fixture(scope="module")
def dropin():
    ref = _reference()
    lib = os.path.join(ROOT, "fargo_thorin_gb300", "libthorin_gpu.so")
    if not os.path.exists(lib):
        from fargo_thorin_gb300 import build
        build.build()
    subprocess.run(["make", "-s", "-f", MK, f"REF={ref}"], check=True, capture_output=True)
    assert os.path.exists(BIN)
    return BIN


def test_dropin_links_the_gpu_library(dropin):
    """The binary defines AlgoGasGPU, calls the library's C ABI and still
    contains the reference's own AlgoGas (which main.c no longer calls)."""
    syms = subprocess.run(["nm", dropin], capture_output=True, text=True, check=True).stdout
    defined = {l.split()[-1] for l in syms.splitlines() if " T " in l}
    undefined = {l.split()[-1] for l in syms.splitlines() if " U " in l}
    assert {"AlgoGasGPU", "AlgoGas", "AdvanceSystemRebound", "main"} <= defined
    for f in ("thorin_gpu_create", "thorin_gpu_cfl", "thorin_gpu_accrete", "thorin_gpu_forces", "thorin_gpu_hydro",
              "thorin_advance_from_disk", "thorin_gpu_download"):
        assert f in undefined, f
    ldd = subprocess.run(["ldd", dropin], capture_output=True, text=True).stdout
    assert "libthorin_gpu.so" in ldd and "not found" not in ldd.split("libthorin_gpu.so")[1].splitlines()[0]


CASES = {
    "disk0": ("disk0", ""),
    "disk1": ("disk1", ""),
    "zhu12_irradiation": ("disk0", "OpacityTable ZHU12\nStellarIrradiation YES\n"),
    "open_nonreflecting": ("disk0", "InnerBoundary NONREFLECTING\nOuterBoundary OPEN\n"),
    "corotating_pebbles": ("disk1", "Frame COROTATING\nParametricOpacity 2.0\n"),
    "cooling_label": ("disk0", "CoolingTime 10.0\nLabelAdvection YES\nDampTowards INIT\n"),
}


@pytest.mark.parametrize("case", list(CASES))
def test_dropin_builds_the_same_parameters(dropin, tmp_path, case):
    kind, extra = CASES[case]
    # paths relative to the run directory: the reference's pebble set-up
    # formats the output directory into fixed-size command buffers
    par = workloads.inpar_text(kind, 20, 60).replace("OutputDir out", "OutputDir out/") + extra
    par = par.replace("Ntot 200", "Ntot 4").replace("Ninterm 200", "Ninterm 2")
    (tmp_path / "planet.cfg").write_text("Embryo1 3e-5 0 0 1.05 0 0 0 0 0\n")
    par += "PlanetConfig planet.cfg\n"
    (tmp_path / "in.par").write_text(par)
    (tmp_path / "out").mkdir()
    dump = tmp_path / "params.bin"
    env = dict(os.environ, THORIN_DROPIN_PARAMS=str(dump), CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([dropin, "-a", "in.par"], cwd=tmp_path, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "AlgoGasGPU: thorin_gpu_create" in (r.stdout + r.stderr), r.stdout[-2000:]
    assert (tmp_path / "out" / "gasdens0.dat").exists()        # the reference's own start-up ran
    got = ThorinParams.from_buffer_copy(dump.read_bytes())
    want = derive(read_inpar(par))
    if want.corotating:                                        # main.c:161 sets the frame from planet 0
        from fargo_thorin_gb300.params import corotating_frame
        corotating_frame(want, workloads.make_planets(want, [(3e-5, 0, 0, 1.05, 0, 0, 0, 0, 0)]))
    diff = [(n, getattr(got, n), getattr(want, n)) for n, _ in ThorinParams._fields_
            if getattr(got, n) != getattr(want, n)]
    assert not diff, diff

"""Host-side logic and the C-ABI boundary, without a GPU: the library loads
and exports every function include/*.h declares, parameter handling
matches the reference's variable table, unsupported options are rejected
before any device work, and the multi-replica bench aggregation (max time,
summed updates) works across two gloo ranks."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include")))
           if h.endswith(".h")]
sys.path.insert(0, ROOT)

from fargo_thorin_gb300 import params as P  # noqa: E402
from fargo_thorin_gb300 import workloads  # noqa: E402


def _declared_functions():
    text = "".join(open(h).read() for h in HEADERS)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(thorin_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from fargo_thorin_gb300 import _lib
    from fargo_thorin_gb300 import build as B
    if not os.path.exists(_lib.LIB_PATH):
        B.build()
    return _lib.load()


def test_header_functions_exported(lib):
    from fargo_thorin_gb300 import _lib
    names = _declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), f"{n} declared in the header but not exported"
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_extrapolation_weights(lib):
    """The extrapolated SOR start's weights of the last update rates are the
    backward differences of an evenly spaced sequence: they reproduce
    polynomials of degree order-1 exactly at the next point."""
    import math
    for order in range(1, 5):
        c = (C.c_double * order)()
        assert lib.thorin_warmstart_coefficients(order, c) == 0
        want = [(-1) ** k * math.comb(order, k + 1) for k in range(order)]
        assert list(c) == want
        # samples p(-1), p(-2), ... of a degree order-1 polynomial extrapolate to p(0)
        for deg in range(order):
            coef = [0.3 * (d + 1) for d in range(deg + 1)]
            p = lambda x: sum(a * x ** d for d, a in enumerate(coef))
            assert abs(sum(c[k] * p(-(k + 1)) for k in range(order)) - p(0)) < 1e-12
    c = (C.c_double * 5)()
    assert lib.thorin_warmstart_coefficients(0, c) != 0
    assert lib.thorin_warmstart_coefficients(5, c) != 0


def test_params_default_matches_struct(lib):
    """thorin_params_default fills the grid size and the SOR controls the same
    way the Python in.par path does for an empty file plus mandatory keys."""
    p = P.ThorinParams()
    lib.thorin_params_default(C.byref(p), 128, 384)
    assert (p.nrad, p.nsec) == (128, 384)
    q = workloads.params_for("disk0", 128, 384)
    assert p.sor_maxiters == q.sor_maxiters
    assert p.adiabind == q.adiabind


def test_read_inpar_case_insensitive_and_defaults():
    text = workloads.inpar_text("disk1", 64, 192).replace("Nrad", "nRaD")
    v = P.read_inpar(text)
    assert v["NRAD"] == 64 and v["NSEC"] == 192
    assert v["INNERBOUNDARY"].upper() == "DAMPING"
    p = P.derive(v)
    assert p.pebbles == 1 and p.back_reaction == 1 and p.feel_disk == 1
    assert p.diffusive_particles == 1          # Interpret.c assigns instead of comparing
    with pytest.warns(UserWarning):
        P.read_inpar(text + "\nNoSuchKey 3\n")


def test_bad_options_rejected_before_cuda(lib):
    """Grids the red-black SOR cannot colour are refused by thorin_gpu_create
    before any CUDA call, with the reason in thorin_gpu_last_error."""
    p = P.derive(P.read_inpar(workloads.inpar_text("disk1", 32, 95)))
    h = C.c_void_p()
    rc = lib.thorin_gpu_create(C.byref(p), C.byref(h))
    assert rc == 1                                  # THORIN_ERR_ARG
    assert not h.value
    assert "nsec even" in lib.thorin_gpu_last_error().decode()


def test_guiding_centre_frame_is_corotating():
    """Frame GUIDINGCENTER sets both switches (Interpret.c:165-169), and the
    orbital elements behind its frame rate invert the planet set-up."""
    text = workloads.inpar_text("disk0", 24, 72) + "\nFrame GUIDINGCENTER\n"
    p = P.derive(P.read_inpar(text))
    assert p.corotating == 1 and p.guiding_center == 1
    m, a, e, inc_deg, f_deg = 1e-5, 1.05, 0.02, 0.5, 30.0
    st = workloads.planet_from_elements(m, 0.0, 0.0, a, e, inc_deg, 0.0, 0.0, f_deg)
    a2, e2, inc2, mean = P.orbit_elements(st["mass"], st["x"], st["y"], st["z"], st["vx"], st["vy"], st["vz"])
    a32, e32 = float(np.float32(a)), float(np.float32(e))     # the planet file is read as C floats
    assert abs(a2 - a32) < 1e-13 and abs(e2 - e32) < 1e-13
    assert abs(inc2 - float(np.float32(inc_deg)) * np.pi / 180.0) < 1e-13
    f = float(np.float32(f_deg)) * np.pi / 180.0               # true -> eccentric -> mean anomaly
    ea = 2.0 * np.arctan(np.sqrt((1 - e32) / (1 + e32)) * np.tan(f / 2.0))
    assert abs(mean - (ea - e32 * np.sin(ea))) < 1e-12
    sys_ = workloads.make_planets(p, [(m, 0.0, 0.0, a, e, inc_deg, 0.0, 0.0, f_deg)])
    P.corotating_frame(p, sys_)
    assert abs(p.omega_frame - np.sqrt((1.0 + sys_.mass[0]) / a2 ** 3)) < 1e-15


def test_corotating_frame_rate():
    """Frame COROTATING starts at planet 0's angular speed (GetPsysInfo)."""
    p = P.derive(P.read_inpar(workloads.inpar_text("disk0", 24, 72) + "\nFrame COROTATING\n"))
    assert p.corotating == 1
    sys_ = workloads.make_planets(p, [workloads.PLANET1])
    P.corotating_frame(p, sys_)
    x, y, vx, vy = sys_.x[0], sys_.y[0], sys_.vx[0], sys_.vy[0]
    assert p.omega_frame == (x * vy - y * vx) / (x * x + y * y)


def test_bad_grid_rejected(lib):
    p = workloads.params_for("disk0", 24, 71)      # odd nsec
    h = C.c_void_p()
    assert lib.thorin_gpu_create(C.byref(p), C.byref(h)) != 0


def test_planet_from_elements_circular(lib):
    s = P.ThorinPlanets()
    rc = lib.thorin_planet_from_elements(C.byref(s), 0, *[C.c_float(v) for v in (3e-5, 0, 0, 1.0, 0, 0, 0, 0, 0)])
    assert rc == 0
    py = workloads.planet_from_elements(3e-5, 0, 0, 1.0, 0, 0, 0, 0, 0)
    assert abs(s.x[0] - py["x"]) == 0.0 and abs(s.vy[0] - py["vy"]) < 1e-15
    assert abs(s.vy[0] - (1.0 + float(__import__("numpy").float32(3e-5))) ** 0.5) < 1e-15


def test_create_without_gpu_fails_loudly():
    """No CPU fallback: without a GPU the product path reports a CUDA error."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from fargo_thorin_gb300.disk import GpuDisk
    from fargo_thorin_gb300._lib import ThorinError
    with pytest.raises(ThorinError):
        GpuDisk(workloads.params_for("disk0", 24, 72))


def _gloo_rank(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    import bench
    out = bench.reduce_over_ranks([10.0 + rank, 3 + rank], ["max", "sum"], "cpu")
    dist.destroy_process_group()
    q.put((rank, out))


def test_replica_aggregation_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_gloo_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(60)
        assert pr.exitcode == 0
    assert res[0] == res[1] == [11.0, 7.0]


def test_reference_arm_nonzero_rank_exits():
    """Under torchrun only rank 0 runs the CPU reference arm."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_ensemble_partition_is_disjoint_balanced_and_deterministic():
    from fargo_thorin_gb300.sharding import partition
    rng = np.random.default_rng(3)
    nr = rng.choice([128, 192, 256, 384, 512], size=64)
    cells = [int(3 * n * n) for n in nr]
    for world in (1, 2, 3, 4, 8):
        shards = partition(cells, world)
        flat = sorted(k for s in shards for k in s)
        assert flat == list(range(len(cells)))                  # every disk exactly once
        loads = [sum(cells[k] for k in s) for s in shards]
        # LPT bound: no rank exceeds the mean load by more than the largest disk
        assert max(loads) <= sum(cells) / world + max(cells)
        assert partition(cells, world) == shards                # same answer on every rank


class _StubDisk:
    """A host stand-in for a GPU disk: one DT = a fixed number of substeps."""

    def __init__(self, cells, substeps):
        self.cells, self.substeps = cells, substeps

    def step(self):
        return self.cells * self.substeps


def _shard_rank(rank, ws, port, cells, q):
    import time
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    from fargo_thorin_gb300 import sharding
    mine = sharding.shard_of(cells, rank, ws)
    disks = [_StubDisk(cells[k], 2 + k % 3) for k in mine]
    t0 = time.perf_counter()
    upd = sum(d.step() for d in disks)
    local = {"disks": len(disks), "cells": sum(d.cells for d in disks), "cell_updates": upd,
             "seconds": time.perf_counter() - t0 + 1e-3 * (rank + 1), "indices": mine}
    got = sharding.gather_metrics(local)
    dist.destroy_process_group()
    q.put((rank, got))


def test_sharded_ensemble_gathers_metrics_gloo():
    """Two ranks take disjoint shards of an ensemble and gather their
    metrics on the host; no data-path collective is involved."""
    import multiprocessing as mp
    from fargo_thorin_gb300.sharding import combine
    cells = [3 * n * n for n in (128, 512, 256, 384, 192, 512, 128, 256, 384)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, cells, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(60)
        assert pr.exitcode == 0
    assert res[0] == res[1]                                     # every rank sees the same gather
    metrics = res[0]
    idx = metrics[0]["indices"] + metrics[1]["indices"]
    assert sorted(idx) == list(range(len(cells))) and not set(metrics[0]["indices"]) & set(metrics[1]["indices"])
    tot = combine(metrics)
    assert tot["disks"] == len(cells)
    assert tot["cell_updates"] == sum(c * (2 + k % 3) for k, c in enumerate(cells))
    assert tot["seconds"] == max(m["seconds"] for m in metrics)

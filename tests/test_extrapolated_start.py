"""The extrapolated SOR start (THORIN_WS_EXTRAPOLATE, include/thorin_warmnet.h).

Every solve starts from T_old + dt times the update rate of the last solves
extrapolated to this one; the exit tests and the threshold stay those of
SuccessiveOverrelaxation (src_main/EnergySources.c:406-511), eps times the L1
residual of T_old.  So the converged temperature meets the plain solve's
criterion and only the sweep count changes.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from fargo_thorin_gb300 import _lib, warmstart as WS  # noqa: E402

pytestmark = pytest.mark.gpu

SNAP = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 11]


def _settled_disk(nr=256, ns=768, settle=3):
    """The disk1 pebble + embryo set-up at SOR eps 1e-8 after a few DTs."""
    from fargo_thorin_gb300 import workloads
    from fargo_thorin_gb300.disk import GpuDisk
    p = workloads.params_for("disk1", nr, ns, sor_eps=1e-8)
    d = GpuDisk(p)
    d.init_default()
    st = workloads.perturbed_state(p, {"dens": d.get(0), "temper": d.get(8)})
    d.set(0, st["dens"]); d.set(1, st["vrad"]); d.set(3, st["energy"])
    d.set(4, st["pebdens"]); d.set(7, st["pebsize"])
    d.refresh(2)
    sys_ = workloads.make_planets(p, [workloads.PLANET1])
    for _ in range(settle):
        d.algogas(sys_)
    return d, sys_


def _replay(d, snap, sys0, mode, ndt, order=2, graph=False):
    d.restore(snap)
    s = sys0.copy()
    WS.set_order(d, order)
    WS.attach(d, None, mode)
    st0, p0 = d.stats(), WS.stats(d).predictions
    for _ in range(ndt):
        (d.algogas_graph if graph else d.algogas)(s)
    st1 = d.stats()
    solves = st1.sor_calls - st0.sor_calls
    out = {"sweeps": (st1.sor_sweeps - st0.sor_sweeps) / solves, "solves": solves,
           "predictions": WS.stats(d).predictions - p0, "T": d.get(8),
           "fields": [d.get(f) for f in (0, 1, 2, 3, 4)]}
    WS.attach(d, None, WS.OFF)
    return out


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_extrapolated_start_meets_the_same_threshold_with_fewer_sweeps():
    d, sys0 = _settled_disk()
    snap = d.snapshot(SNAP)
    plain = _replay(d, snap, sys0, WS.OFF, 4)
    ext = _replay(d, snap, sys0, WS.EXTRAPOLATE, 4)
    print(plain["sweeps"], ext["sweeps"], _rel(ext["T"], plain["T"]))
    assert ext["solves"] == plain["solves"]
    assert ext["predictions"] == ext["solves"]
    assert ext["sweeps"] < 0.9 * plain["sweeps"]
    assert _rel(ext["T"], plain["T"]) < 1e-9
    for a, b in zip(ext["fields"], plain["fields"]):
        assert _rel(a, b) < 1e-9
    d.close()


def test_step_length_keeps_the_start_no_worse_in_a_transient():
    """From the set-up's start (the first DTs are a fast transient, where
    extrapolating the last updates overshoots) the residual-minimising step
    keeps the extrapolated start's solves within a few sweeps of the plain
    ones, and on the settled disk it stays near 1 (the plain extrapolation)."""
    d, sys0 = _settled_disk(settle=1)
    snap = d.snapshot(SNAP)
    plain = _replay(d, snap, sys0, WS.OFF, 2)
    s0 = WS.stats(d).step_sum
    ext = _replay(d, snap, sys0, WS.EXTRAPOLATE, 2)
    steps = (WS.stats(d).step_sum - s0) / max(ext["predictions"], 1)
    print(plain["sweeps"], ext["sweeps"], steps)
    assert ext["sweeps"] <= plain["sweeps"] + 2
    assert _rel(ext["T"], plain["T"]) < 1e-9
    d.close()
    d, sys0 = _settled_disk()
    snap = d.snapshot(SNAP)
    s0 = WS.stats(d).step_sum
    ext = _replay(d, snap, sys0, WS.EXTRAPOLATE, 4)
    steps = (WS.stats(d).step_sum - s0) / max(ext["predictions"] - 1, 1)   # the first solve has no update
    print("settled mean step", steps)
    assert 0.5 < steps < 1.5
    d.close()


def test_linear_extrapolation_beats_the_previous_update():
    """Order 2 (the rate extrapolated linearly) against order 1 (the last
    update's rate) on the same DTs."""
    d, sys0 = _settled_disk()
    snap = d.snapshot(SNAP)
    o1 = _replay(d, snap, sys0, WS.EXTRAPOLATE, 4, order=1)
    o2 = _replay(d, snap, sys0, WS.EXTRAPOLATE, 4, order=2)
    print(o1["sweeps"], o2["sweeps"])
    assert o2["sweeps"] < o1["sweeps"]
    assert _rel(o2["T"], o1["T"]) < 1e-9
    d.close()


def test_extrapolated_start_in_the_dt_graph_matches_the_host_path():
    d, sys0 = _settled_disk()
    assert d.graph_supported(sys0)
    snap = d.snapshot(SNAP)
    host = _replay(d, snap, sys0, WS.EXTRAPOLATE, 3)
    gr = _replay(d, snap, sys0, WS.EXTRAPOLATE, 3, graph=True)
    assert gr["sweeps"] == host["sweeps"] and gr["solves"] == host["solves"]
    assert gr["predictions"] == host["predictions"]
    assert _rel(gr["T"], host["T"]) < 1e-12
    d.close()


def test_first_solve_after_attaching_starts_from_t_old():
    """Nothing is recorded when the mode is attached, so the first solve
    starts from T_old: a DT of one substep is the plain DT bit for bit.  The
    DT here is short enough for one substep."""
    p, d, sys0 = WS.make_training_disk(64, 192, {"alpha": 1e-3, "aspect": 0.05, "mplanet": 3e-5}, seed=3,
                                       dt_div=50.0)
    d.algogas(sys0)
    snap = d.snapshot(SNAP)
    s = sys0.copy()
    d.algogas(s)
    assert d.stats().substeps == 1
    plain = [d.get(f) for f in (0, 1, 2, 3, 4)] + [d.get(8)]
    ext = _replay(d, snap, sys0, WS.EXTRAPOLATE, 1)
    assert ext["predictions"] == 1
    for a, b in zip(ext["fields"] + [ext["T"]], plain):
        assert np.array_equal(a, b)
    d.close()


def test_order_is_checked():
    d, _ = _settled_disk(64, 192, settle=0)
    for bad in (0, 5):
        with pytest.raises(_lib.ThorinError):
            WS.set_order(d, bad)
    WS.set_order(d, 3)
    d.close()

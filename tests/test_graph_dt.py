"""The device-resident DT (thorin_gpu_algogas_graph): one CUDA graph per DT
with the substep loop, the planet side and the SOR omega schedule on the
device.

It runs the host path's own kernels with the control block filled on the
device, so it must give the host path's results: substep and SOR counts
exact, FARGO shifts exact, fields within 1e-12 (the transcendental functions
of the planet side, pow and atan2, are CUDA's on the device and glibc's on
the host), planets within 1e-13.  Against the reference's golden outputs it
meets the same 1e-10 as the host path.
"""
import ctypes as C

import numpy as np
import pytest

import harness as H
import oracle as O
from fargo_thorin_gb300 import workloads

pytestmark = pytest.mark.gpu
FIELDS = H.GAS + H.PEB + ["energy"]


def _disk(p):
    from fargo_thorin_gb300.disk import GpuDisk
    return GpuDisk(p)


def _start(d, p, g):
    d.init_default()
    H.opacity_table(d, g)
    H.start_state(d, p, {"dens": g["init_dens"].ravel(), "temper": g["init_temper"].ravel()})


@pytest.mark.parametrize("name", ["disk1_32x96", "disk1_48x144_eps8", "disk0_24x72", "zhu12irr_peb_32x96",
                                  "dampinit_24x72", "open_24x72", "nonrefl_24x72", "label_24x72", "frame_24x72"])
def test_graph_dt_matches_host_path(name):
    g = H.load(name)
    p = H.case_params(g)
    a, b = _disk(p), _disk(p)
    for d in (a, b):
        _start(d, p, g)
    sa = workloads.make_planets(p, [tuple(g["planet"])])
    sb = workloads.make_planets(p, [tuple(g["planet"])])
    assert b.graph_supported(sb)
    n = p.nrad * p.nsec
    fields = FIELDS if p.pebbles else H.GAS + ["energy"]
    for step in range(1, 6):
        a.algogas(sa)
        b.algogas_graph(sb)                    # DT 1 calibrates omega on the host path
        ta, tb = a.stats(), b.stats()
        assert ta.substeps == tb.substeps and ta.sor_sweeps == tb.sor_sweeps, f"counts at DT {step}"
        assert ta.sor_last_niter == tb.sor_last_niter and ta.crashed == tb.crashed
        assert abs(ta.physical_time - tb.physical_time) <= 1e-15 * abs(ta.physical_time)
        np.testing.assert_array_equal(a.nshift(), b.nshift())
        for f in fields + (["label"] if p.label_advection else []):
            err = H.rel_l2(b.get(H.FIELD_IDS[f])[:n], a.get(H.FIELD_IDS[f])[:n])
            assert err < 1e-12, (f, step, err)
        for k in ("x", "y", "vx", "vy", "mass"):
            assert abs(getattr(sa, k)[0] - getattr(sb, k)[0]) <= 1e-13 * max(1.0, abs(getattr(sa, k)[0])), k
        assert a.sor_state()[:3] == b.sor_state()[:3]
    a.close()
    b.close()


@pytest.mark.parametrize("name", ["disk1_64x192_40", "disk1_48x144_eps8", "zhu12irr_peb_32x96"])
def test_graph_dt_vs_reference_golden(name):
    """The whole golden run with every DT after the first as a graph: the
    reference's substep and SOR counts, fields within 1e-10 at the outputs."""
    g = H.load(name)
    p = H.case_params(g)
    d = _disk(p)
    _start(d, p, g)
    sys_ = workloads.make_planets(p, [tuple(g["planet"])])
    tq = g["tqwk"]
    ntot, ninterm = int(g["ntot"]), int(g["ninterm"])
    nr, ns = p.nrad, p.nsec
    for step in range(1, ntot + 1):
        sys_.x[0], sys_.y[0] = tq[step - 1][3], tq[step - 1][4]
        d.algogas_graph(sys_)
        st = d.stats()
        assert st.substeps == g["substeps"][step - 1]
        assert st.sor_last_niter == g["sor_niter"][step - 1], f"SOR iterations at DT {step}"
        m, mom, e, _, _ = d.integrals()
        assert abs(m / g["mass"][step - 1] - 1) < 1e-12 and abs(mom / g["momentum"][step - 1] - 1) < 1e-12
        assert abs(e / g["energy"][step - 1] - 1) < 1e-12
        if step % ninterm == 0:
            k = step // ninterm
            for f in H.GAS + H.PEB:
                a = d.get(H.FIELD_IDS[f])[:nr * ns].reshape(nr, ns)
                if f"out{k}_{f}" in g:
                    assert H.rel_l2(a, g[f"out{k}_{f}"]) < 1e-10, f
                else:
                    assert H.rel_l2(a[g["sample_rows"]], g[f"out{k}_{f}_rows"]) < 1e-10, f
    d.close()


def test_graph_dt_rejects_host_only_options():
    g = H.load("corot_24x72")
    p = H.case_params(g)
    d = _disk(p)
    _start(d, p, g)
    s = workloads.make_planets(p, [tuple(g["planet"])])
    assert not d.graph_supported(s)
    from fargo_thorin_gb300 import _lib
    with pytest.raises(_lib.ThorinError):
        d.algogas_graph(s)
    assert b"corotating" in d.L.thorin_gpu_last_error()
    d.close()


def test_launch_shape_does_not_change_results():
    """Sweeps per loop body and SOR threads per SM change the launches, not
    the arithmetic: bit-identical fields."""
    g = H.load("disk1_32x96")
    p = H.case_params(g)
    out = []
    for shape in ((8, 1536), (4, 768), (16, 2048)):
        d = _disk(p)
        _start(d, p, g)
        d.set_launch_shape(*shape)
        assert d.launch_shape() == shape
        s = workloads.make_planets(p, [tuple(g["planet"])])
        for _ in range(3):
            d.algogas_graph(s)
        out.append([d.get(H.FIELD_IDS[f]) for f in FIELDS])
        d.close()
    for other in out[1:]:
        for a, b in zip(out[0], other):
            np.testing.assert_array_equal(a, b)


def test_ensemble_graph_matches_single_disks():
    """Disks of uneven sizes advanced together as graphs on their own
    streams end bit-identical to each advanced alone."""
    from fargo_thorin_gb300.ensemble import Ensemble
    specs = [{"nrad": 32, "alpha": 1e-3, "sigma_scale": 1.0, "aspect": 0.05, "mplanet": 3e-5},
             {"nrad": 48, "alpha": 3e-4, "sigma_scale": 2.0, "aspect": 0.04, "mplanet": 1e-5},
             {"nrad": 40, "alpha": 1e-4, "sigma_scale": 1.5, "aspect": 0.07, "mplanet": 6e-5}]
    ens = Ensemble(specs, seed=5)
    for _ in range(3):
        assert ens.step_graph() == [0] * len(specs)
    together = [[d.get(f) for f in (0, 1, 2, 3, 4, 5, 6, 8)] for d in ens.disks]
    ens.close()
    for k, spec in enumerate(specs):
        one = Ensemble([spec], seed=5 + k)
        for _ in range(3):
            one.disks[0].algogas_graph(one.systems[0])
        alone = [one.disks[0].get(f) for f in (0, 1, 2, 3, 4, 5, 6, 8)]
        one.close()
        for a, b in zip(together[k], alone):
            np.testing.assert_array_equal(a, b)


def test_schedule_tuner_replays_identical_work():
    """The autotuner times every candidate schedule on the same DT from a
    snapshot; the chosen schedule and the sequential host path then do the
    same substeps and SOR sweeps on the same DTs, and end with the same
    fields to 1e-12."""
    from fargo_thorin_gb300.ensemble import Ensemble
    specs = [{"nrad": 32, "alpha": 1e-3, "sigma_scale": 1.0, "aspect": 0.05, "mplanet": 3e-5},
             {"nrad": 48, "alpha": 3e-4, "sigma_scale": 2.0, "aspect": 0.04, "mplanet": 1e-5},
             {"nrad": 64, "alpha": 1e-3, "sigma_scale": 1.0, "aspect": 0.05, "mplanet": 2e-5}]
    ens = Ensemble(specs, seed=7)
    ens.step(1)
    snaps = ens.snapshot()
    tune = ens.tune_schedule(snaps, shapes=((8, 1536), (4, 768)), pool_workers=(2,))
    assert tune["schedule"]["mode"] in ("graph", "pool") and len(tune["trials"]) >= 2
    ens.restore(snaps)
    a = ens.run_schedule(tune["schedule"], 2)
    fa = [d.get(0) for d in ens.disks]
    ens.restore(snaps)
    b = ens.run_schedule({"mode": "sequential"}, 2)
    fb = [d.get(0) for d in ens.disks]
    assert a["cell_updates"] == b["cell_updates"] and a["sweeps"] == b["sweeps"]
    for x, y in zip(fa, fb):
        assert H.rel_l2(x, y) < 1e-12
    ens.close()


def test_graph_and_host_dts_interleave():
    """Host-path DTs swap the buffers of the state fields; a graph DT after
    them still reads the current state: host, graph, host, graph DTs end
    where four host DTs end (counts exact, fields within 1e-12)."""
    g = H.load("disk1_32x96")
    p = H.case_params(g)
    a, b = _disk(p), _disk(p)
    for d in (a, b):
        _start(d, p, g)
    sa = workloads.make_planets(p, [tuple(g["planet"])])
    sb = workloads.make_planets(p, [tuple(g["planet"])])
    n = p.nrad * p.nsec
    for step in range(8):
        a.algogas(sa)
        (b.algogas if step in (0, 1, 3, 6) else b.algogas_graph)(sb)
        assert a.stats().substeps == b.stats().substeps and a.stats().sor_sweeps == b.stats().sor_sweeps
        for f in FIELDS:
            assert H.rel_l2(b.get(H.FIELD_IDS[f])[:n], a.get(H.FIELD_IDS[f])[:n]) < 1e-12, (f, step)
    a.close()
    b.close()


def test_graph_dt_with_learned_warm_start():
    """The warm start's prediction (network on the tensor cores) inside the
    device-resident DT gives the host path's result: same SOR counts,
    temperature within 1e-12."""
    from fargo_thorin_gb300 import warmstart as WS
    g = H.load("disk1_32x96")
    p = H.case_params(g)
    rng = np.random.default_rng(3)
    params = WS.init_params(1)
    import warmnet_oracle as WO
    params[WO.OFFSETS[7]:] = rng.standard_normal(params.size - WO.OFFSETS[7]).astype(np.float32) * 0.01
    out = []
    for use_graph in (False, True):
        d = _disk(p)
        _start(d, p, g)
        s = workloads.make_planets(p, [tuple(g["planet"])])
        d.algogas(s)                                    # calibration DT without the network
        net = WS.WarmNet(p.nrad, p.nsec, params=params)
        WS.attach(d, net, WS.PREDICT)
        counts = []
        for _ in range(3):
            (d.algogas_graph if use_graph else d.algogas)(s)
            counts.append((d.stats().substeps, d.stats().sor_sweeps))
        out.append((counts, d.get(H.FIELD_IDS["temper"]), WS.stats(d).predictions))
        WS.attach(d, None, WS.OFF)
        net.close()
        d.close()
    assert out[0][0] == out[1][0] and out[0][2] == out[1][2] > 0
    assert H.rel_l2(out[1][1], out[0][1]) < 1e-12

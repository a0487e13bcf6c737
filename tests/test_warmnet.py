"""The learned SOR warm start (include/thorin_warmnet.h).

CPU: the numpy restatement of the network (oracle/warmnet_oracle.py) has a
backward pass that matches finite differences of its float64 forward pass,
and its bfloat16 rounding is round-to-nearest-even.
GPU: the tcgen05 layout self-test GEMM is exact; the CUDA forward pass, loss
and parameter gradient match the oracle's bf16 emulation; gradients repeat
bit for bit; Adam steps on a fixed batch lower the loss.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import warmnet_oracle as WO  # noqa: E402
from fargo_thorin_gb300 import warmstart as WS  # noqa: E402


def _params(seed, out_std=0.05):
    p = WS.init_params(seed).astype(np.float64)
    o = WO.OFFSETS[7]
    rng = np.random.default_rng(seed + 1)
    p[o:] = rng.standard_normal(p.size - o) * out_std
    for k, (cin, cout) in enumerate(WO.LAYERS):      # small nonzero biases
        b0 = WO.OFFSETS[k] + cout * 9 * cin
        p[b0:b0 + cout] = rng.uniform(-0.05, 0.05, cout)
    return p


def _inputs(seed, B, H, W):
    rng = np.random.default_rng(seed)
    x = np.zeros((B, H, W, WO.INPUTS), np.float32)
    x[..., :WO.NIN] = rng.uniform(-1.0, 1.0, (B, H, W, WO.NIN))
    t = rng.standard_normal((B, H, W)).astype(np.float32) * 0.1
    return WO.bf16(x), t


def test_param_count_and_init():
    assert WO.NPARAMS == WS.NPARAMS == 57825
    p = WS.init_params(3)
    assert p.dtype == np.float32 and p.size == WS.NPARAMS
    assert np.all(p[WO.OFFSETS[7]:] == 0.0)            # output layer starts at zero


def test_bf16_rounding_ties_to_even():
    vals = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 3.0e-39], np.float32)
    got = WO.bf16(vals)
    assert got[0] == 1.0
    assert got[1] == 1.0                                # tie -> even mantissa
    assert got[2] == np.float32(1.0 + 4 * 2.0 ** -8)    # tie -> even (rounds up)
    assert got[3] == 1.0
    assert got[4] == -2.5
    assert np.all(WO.from_bits(WO.bf16_bits(vals)) == got)


def test_oracle_backward_matches_finite_differences():
    B, H, W = 1, 16, 16
    p = _params(5, out_std=0.2)
    x, t = _inputs(6, B, H, W)
    loss, g, _ = WO.loss_and_grad(p, x.astype(np.float64), t.astype(np.float64), bf=False)
    rng = np.random.default_rng(7)
    idx = np.concatenate([rng.integers(WO.OFFSETS[k], WO.OFFSETS[k + 1] if k < 7 else WO.NPARAMS, 3)
                          for k in range(8)])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = WO.loss_and_grad(pp, x.astype(np.float64), t.astype(np.float64), bf=False)[0]
        lm = WO.loss_and_grad(pm, x.astype(np.float64), t.astype(np.float64), bf=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(abs(fd), 1e-6), (i, fd, g[i])


# --------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def lib():
    from fargo_thorin_gb300 import _lib
    return _lib.load()


@pytest.mark.gpu
def test_umma_selftest_exact(lib):
    import ctypes as C
    rng = np.random.default_rng(0)
    a = WO.bf16(rng.uniform(-1, 1, (128, 64)).astype(np.float32))
    b = WO.bf16(rng.uniform(-1, 1, (32, 64)).astype(np.float32))
    ab, bb = WO.bf16_bits(a), WO.bf16_bits(b)
    d = np.zeros((128, 32), np.float32)
    from fargo_thorin_gb300 import _lib
    _lib.check(lib.thorin_selftest_umma(ab.ctypes.data_as(C.POINTER(C.c_uint16)),
                                        bb.ctypes.data_as(C.POINTER(C.c_uint16)),
                                        d.ctypes.data_as(C.POINTER(C.c_float))), "selftest_umma")
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    assert np.max(np.abs(d - ref)) <= 1e-5 * np.max(np.abs(ref)), np.max(np.abs(d - ref))


@pytest.mark.gpu
@pytest.mark.parametrize("B,H,W", [(1, 16, 32), (2, 24, 40)])
def test_forward_matches_oracle(B, H, W):
    p = _params(11)
    x, _ = _inputs(12, B, H, W)
    net = WS.WarmNet(H, W, max_batch=B, params=p.astype(np.float32))
    y = net.forward(WO.bf16_bits(x))
    yo, _ = WO.forward(p.astype(np.float32), x, bf=True)
    err = np.linalg.norm(y - yo) / np.linalg.norm(yo)
    assert err < 1e-2, err


@pytest.mark.gpu
def test_gradient_matches_oracle_and_repeats():
    B, H, W = 2, 16, 32
    p = _params(21)
    x, t = _inputs(22, B, H, W)
    net = WS.WarmNet(H, W, max_batch=B, params=p.astype(np.float32))
    loss, g = net.gradient(WO.bf16_bits(x), t)
    lo, go, _ = WO.loss_and_grad(p.astype(np.float32), x, t, bf=True)
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    for k in range(8):
        a, b = WO.OFFSETS[k], (WO.OFFSETS[k + 1] if k < 7 else WO.NPARAMS)
        err = np.linalg.norm(g[a:b] - go[a:b]) / np.linalg.norm(go[a:b])
        assert err < 3e-2, (k, err)
    loss2, g2 = net.gradient(WO.bf16_bits(x), t)
    assert loss2 == loss and np.array_equal(g2, g)


@pytest.mark.gpu
def test_adam_lowers_loss_on_fixed_batch():
    B, H, W = 2, 16, 32
    p = _params(31)
    x, t = _inputs(32, B, H, W)
    net = WS.WarmNet(H, W, max_batch=B, params=p.astype(np.float32))
    xb = WO.bf16_bits(x)
    l0, _ = net.gradient(xb, t)
    for _ in range(40):
        net.gradient(xb, t)
        net.adam(3e-3)
    l1, _ = net.gradient(xb, t)
    assert l1 < 0.5 * l0, (l0, l1)


def _small_disk():
    return WS.make_training_disk(64, 192, {"alpha": 1e-3, "aspect": 0.05, "mplanet": 3e-5}, seed=3)


@pytest.mark.gpu
def test_training_leaves_the_plain_solve_unchanged():
    """TRAIN mode fits the network after each solve; the disk's own fields
    stay bit-identical to a run without a network."""
    out = []
    for mode in (WS.OFF, WS.TRAIN):
        p, d, sys_ = _small_disk()
        net = WS.WarmNet(64, 192)
        if mode == WS.TRAIN:
            WS.attach(d, net, WS.TRAIN, 1e-3)
        for _ in range(2):
            d.algogas(sys_)
        out.append([d.get(f) for f in (0, 1, 2, 3, 4, 8)])
        if mode == WS.TRAIN:
            s = WS.stats(d)
            assert s.train_steps == d.stats().sor_calls and np.isfinite(s.last_loss)
        d.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_predicted_start_meets_the_same_threshold():
    """From an untrained network (prediction = one Jacobi step) the solve
    still converges to the plain solve's threshold: temperatures agree to the
    SOR tolerance."""
    temps, per = [], []
    for mode in (WS.OFF, WS.PREDICT):
        p, d, sys_ = _small_disk()
        d.algogas(sys_)
        net = WS.WarmNet(64, 192)
        WS.attach(d, net, mode)
        s0 = d.stats()
        d.algogas(sys_)
        s1 = d.stats()
        temps.append(d.get(8))
        per.append((s1.sor_sweeps - s0.sor_sweeps) / (s1.sor_calls - s0.sor_calls))
        if mode == WS.PREDICT:
            assert WS.stats(d).predictions == s1.sor_calls - s0.sor_calls
        d.close()
    assert np.linalg.norm(temps[1] - temps[0]) / np.linalg.norm(temps[0]) < 1e-9
    assert per[1] <= per[0] + 1


WEIGHTS = os.path.join(ROOT, "fargo_thorin_gb300", "warmnet_disk1_1024x3072.npy")


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained network file")
def test_trained_network_saves_sweeps_on_the_disk1_workload():
    """The committed network, trained on the plain solver's solves of drawn
    1024 x 3072 disks, against plain SOR on the measured disk1 workload: fewer
    sweeps per solve at the same threshold, the same temperatures to 1e-9."""
    from fargo_thorin_gb300 import workloads
    net = WS.WarmNet(1024, 3072, params=WS.WarmNet.load_params(WEIGHTS))
    r = WS.compare_sweeps(net, {"alpha": 1.0e-3, "aspect": 0.05, "mplanet": workloads.PLANET1[0]}, ndt=1)
    print(r)
    assert r["learned"] < r["plain"]
    assert r["t_rel_l2"] < 1e-9


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained network file")
def test_learned_start_stays_on_the_plain_solution_over_several_dts():
    """Over 5 DTs (40 solves) of the disk1 workload the learned start's
    temperatures stay within 1e-9 of the plain run's: every solve meets the
    plain solve's threshold, so the difference does not grow with the DTs."""
    from fargo_thorin_gb300 import workloads
    net = WS.WarmNet(1024, 3072, params=WS.WarmNet.load_params(WEIGHTS))
    r = WS.compare_sweeps(net, {"alpha": 1.0e-3, "aspect": 0.05, "mplanet": workloads.PLANET1[0]}, ndt=5, warm=2)
    print(r)
    assert r["learned"] < r["plain"]
    assert r["t_rel_l2"] < 1e-9 and r["t_rel_l2_last"] < 1e-9


@pytest.mark.gpu
def test_training_residual_uses_the_disks_packed_system():
    """The warm start reads the disk's SOR system, which k_matrix stores
    colour-packed.  With a zero output layer the prediction is the start plus
    one Jacobi step J = -r/Ml, and the training step records
    mean((A (T0 + J) - rhs)^2) / mean|r0|^2 over the unknowns.  Recomputed
    here from the oracle's system of the same solve (grid layout)."""
    import oracle as O
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import harness as H
    from fargo_thorin_gb300 import workloads
    p = workloads.params_for("disk1", 32, 96)
    o = O.OracleDisk(p)
    o.init_default()
    # 20% random structure in azimuth, so that cells of one ring have clearly
    # different coefficients (on a near-axisymmetric disk, reading another
    # cell of the same ring would go unnoticed)
    rng = np.random.default_rng(5)
    dens = o.get(H.FIELD_IDS["dens"]).copy()
    temper = o.get(H.FIELD_IDS["temper"]).copy()
    dens *= 1 + 0.2 * rng.uniform(-1, 1, dens.shape)
    temper *= 1 + 0.2 * rng.uniform(-1, 1, temper.shape)
    init = {"dens": dens, "temper": temper}
    from fargo_thorin_gb300.disk import GpuDisk
    d = GpuDisk(p)
    d.init_default()
    for x in (d, o):
        H.start_state(x, p, init)
    sg = workloads.make_planets(p, [workloads.PLANET1])
    so = workloads.make_planets(p, [workloads.PLANET1])
    d.algogas(sg)
    o.algogas(so)
    net = WS.WarmNet(32, 96, params=WS.init_params(0))
    WS.attach(d, net, WS.TRAIN, 1e-30)
    d.algogas(sg)
    o.algogas(so)
    got = WS.stats(d).last_res_loss
    s = o.sor_system()
    nr, ns = 32, 96
    A = {k: s[k].reshape(-1, ns)[:nr] for k in ("ml", "mlip", "mlim", "mljp", "mljm", "rhs")}
    T0 = s["tstart"].reshape(-1, ns)[:nr]

    def resid(T):
        r = (T * A["ml"] + np.roll(T, -1, axis=0) * A["mlip"] + np.roll(T, 1, axis=0) * A["mlim"]
             + np.roll(T, -1, axis=1) * A["mljp"] + np.roll(T, 1, axis=1) * A["mljm"] - A["rhs"])
        return r[1:nr - 1]

    r0 = resid(T0)
    T1 = T0.copy()
    T1[1:nr - 1] -= r0 / A["ml"][1:nr - 1]
    want = np.mean(resid(T1) ** 2) / np.mean(np.abs(r0)) ** 2
    assert abs(got / want - 1) < 1e-3, (got, want)
    WS.attach(d, None, WS.OFF)
    net.close()
    d.close()

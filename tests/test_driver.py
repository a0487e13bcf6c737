"""The host driver (fargo_thorin_gb300/run.py) against whole reference runs.

* CPU: the initial outputs of ``-0`` written from the oracle's initial state
  are byte-identical to the reference's own files (gas and pebble fields,
  used_rad.dat, dims.dat, omegaframe.dat).
* GPU: a gas disk initialised from ASCII files and a pebble + embryo disk
  restarted from output 0 run 5 DTs through the driver; every output file,
  the torque log and the -a integrals match the reference's run.  A restart
  from output 1 reproduces the continuous run's output 2.
"""
import hashlib
import os

import numpy as np
import pytest

import harness as H
import oracle as O
from fargo_thorin_gb300 import run as R

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _prepare(tmp_path, g, inpar_extra=""):
    (tmp_path / "planet.cfg").write_text(str(g["planet_cfg"]))
    (tmp_path / "in.par").write_text(str(g["inpar"]) + inpar_extra)
    return str(tmp_path / "in.par")


def test_initial_outputs_byte_identical(tmp_path, monkeypatch):
    g = _golden("driver_init_disk1_20x60")
    monkeypatch.chdir(tmp_path)
    par = _prepare(tmp_path, g)
    r = R.Run(par, disk_factory=O.OracleDisk)
    r.run(only_init=True, log=lambda *a: None, argv=["thorin", "-0", "in.par"])
    out = tmp_path / "out"
    for key in g.files:
        if not key.startswith("sha256_"):
            continue
        name = key[len("sha256_"):]
        if name.startswith("nbody.") or name == "run.commandline":
            continue                      # REBOUND's own files; the driver writes nbody.state<N>.dat instead
        data = (out / name).read_bytes()
        assert hashlib.sha256(data).hexdigest() == str(g[key]), name
    assert (out / "used_rad.dat").read_text() == str(g["txt_used_rad.dat"])
    assert (out / "dims.dat").read_text() == str(g["txt_dims.dat"])


def _run_like_reference(tmp_path, g, restart=None, ntot=None):
    """Lay out the reference's inputs in tmp_path and run the driver on them."""
    kind = str(g["kind"])
    extra = ""
    if kind == "disk0":
        for key in ("DensInfile", "VradInfile", "VthetaInfile", "TemperInfile"):
            np.savetxt(tmp_path / (key + ".txt"), g["ascii_" + key], fmt="%.17g")
    par = _prepare(tmp_path, g, extra)
    if ntot is not None:
        txt = (tmp_path / "in.par").read_text().replace("Ntot 4", f"Ntot {ntot}")
        (tmp_path / "in.par").write_text(txt)
    logs = []
    if kind == "disk1" and restart is None:
        # the reference's -0 run, then its overridden restart files
        R.Run(par).run(only_init=True, log=lambda *a: None)
        for name in ("dens", "vrad", "vtheta", "temper", "pebbledens", "pebblesize", "pebblevrad", "pebblevtheta"):
            g["restart0_" + name].astype("<f8").tofile(tmp_path / "out" / f"gas{name}0.dat")
        restart = 0
    R.Run(par).run(restart=restart, monitor=True, log=logs.append)
    return tmp_path / "out", logs


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["disk0", "disk1"])
def test_driver_matches_reference_run(tmp_path, monkeypatch, kind):
    g = _golden(f"driver_{kind}_20x60")
    monkeypatch.chdir(tmp_path)
    out, logs = _run_like_reference(tmp_path, g)
    for key in g.files:
        if key.startswith("bin_"):
            name = key[4:]
            a = np.fromfile(out / name, dtype="<f8")
            assert a.size == g[key].size, name
            assert H.rel_l2(a, g[key]) < 1e-9, name
    ref = np.loadtxt(str(g["txt_tqwk0.dat"]).splitlines(), ndmin=2)
    got = np.loadtxt(out / "tqwk0.dat", ndmin=2)
    assert got.shape == ref.shape
    amag = np.hypot(ref[:, 5], ref[:, 6])
    assert np.all(np.abs(got[:, 0] - ref[:, 0]) <= 1e-12)
    assert np.all(np.hypot(got[:, 5] - ref[:, 5], got[:, 6] - ref[:, 6]) < 1e-9 * amag)
    assert np.all(np.hypot(got[:, 3] - ref[:, 3], got[:, 4] - ref[:, 4]) < 1e-9)
    vals = {"momentum": [], "mass": [], "energy": []}
    for line in logs:
        for key, tag in (("momentum", "Gas Momentum"), ("mass", "Gas total Mass"), ("energy", "Gas total Energy")):
            if line.startswith(tag):
                vals[key].append(float(line.split(":")[1]))
    for key in ("mass", "momentum"):
        np.testing.assert_allclose(vals[key], g["int_" + key], rtol=1e-11)
    assert (out / "used_rad.dat").read_text() == str(g["txt_used_rad.dat"])


@pytest.mark.gpu
def test_driver_restart_reproduces_continuous_run(tmp_path, monkeypatch):
    g = _golden("driver_disk0_20x60")
    a = tmp_path / "a"
    a.mkdir()
    monkeypatch.chdir(a)
    out_a, _ = _run_like_reference(a, g)
    cont = np.fromfile(out_a / "gasdens2.dat", dtype="<f8")
    cont_t = np.fromfile(out_a / "gastemper2.dat", dtype="<f8")
    for name in ("gasdens2.dat", "gastemper2.dat", "gasvrad2.dat", "gasvtheta2.dat"):
        os.remove(out_a / name)
    R.Run(str(a / "in.par")).run(restart=1, log=lambda *x: None)
    assert H.rel_l2(np.fromfile(out_a / "gasdens2.dat", dtype="<f8"), cont) < 1e-12
    assert H.rel_l2(np.fromfile(out_a / "gastemper2.dat", dtype="<f8"), cont_t) < 1e-12

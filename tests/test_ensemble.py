"""Ensembles of disks (include/thorin_ensemble.h).

CPU: argument checks return THORIN_ERR_ARG before any device work.
GPU: disks of uneven sizes advanced concurrently on four worker threads,
largest first, end bit-identical to the same disks advanced one after the
other; the autotuner returns a schedule it measured.  (Every disk carries
an accreting embryo of nonzero mass: with pebble accretion and accretion
heating on, a zero-mass embryo has a zero Hill radius and the reference's
heating term turns the temperature NaN.)
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from fargo_thorin_gb300 import _lib  # noqa: E402


def test_ensemble_rejects_bad_arguments():
    L = _lib.load()
    assert L.thorin_ensemble_algogas(None, None, 0, 1, 0, None) == 1
    dp = (C.c_void_p * 1)(None)
    assert L.thorin_ensemble_algogas(dp, dp, 1, 1, 0, None) == 1          # missing disk
    assert L.thorin_ensemble_algogas(dp, dp, 1, 0, 0, None) == 1          # no workers
    assert L.thorin_ensemble_algogas(dp, dp, 1, 1, 7, None) == 1          # unknown order
    bw, bo = C.c_int(), C.c_int()
    bms = C.c_double()
    assert L.thorin_ensemble_tune(dp, dp, 1, 0, 1, C.byref(bw), C.byref(bo), C.byref(bms), None) == 1


SPECS = [{"nrad": 32, "alpha": 1e-3, "sigma_scale": 1.0, "aspect": 0.05, "mplanet": 3e-5},
         {"nrad": 48, "alpha": 3e-4, "sigma_scale": 2.0, "aspect": 0.04, "mplanet": 1e-5},
         {"nrad": 64, "alpha": 1e-3, "sigma_scale": 1.0, "aspect": 0.05, "mplanet": 2e-5},
         {"nrad": 40, "alpha": 1e-4, "sigma_scale": 1.5, "aspect": 0.07, "mplanet": 6e-5}]


def _fields(ens):
    return [[d.get(f) for f in (0, 1, 2, 3, 4, 5, 6, 8)] for d in ens.disks]


@pytest.mark.gpu
def test_concurrent_ensemble_matches_sequential_runs():
    from fargo_thorin_gb300.ensemble import GIVEN, LARGEST, Ensemble
    out = []
    for workers, order in ((1, GIVEN), (4, LARGEST)):
        ens = Ensemble(SPECS, seed=5)
        for _ in range(2):
            assert ens.step(workers, order) == [0] * len(SPECS)
        out.append(_fields(ens))
        ens.close()
    for a, b in zip(*out):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


@pytest.mark.gpu
def test_autotuner_returns_a_measured_schedule():
    from fargo_thorin_gb300.ensemble import Ensemble
    ens = Ensemble(SPECS, seed=6)
    ens.step(1)
    r = ens.tune(max_workers=4, ndt=1)
    assert r["workers"] in (1, 2, 4) and r["order_code"] in (0, 1)
    assert 0.0 < r["ms_per_dt"] <= r["sequential_ms_per_dt"]
    ens.close()

"""ctypes wrapper of the CPU oracle (oracle/thorin_oracle.c).

TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
from fargo_thorin_gb300.params import ThorinParams, ThorinPlanets, ThorinStats  # noqa: E402

SRC = os.path.join(HERE, "thorin_oracle.c")
LIB_SEQ = os.path.join(HERE, "liboracle.so")
LIB_OMP = os.path.join(HERE, "liboracle_omp.so")


def build(force: bool = False) -> None:
    """Compile the oracle: a sequential copy for parity and an OpenMP copy
    for the CPU baseline.  -std=c99 keeps FP contraction off, as in the
    reference build."""
    for out, extra in ((LIB_SEQ, []), (LIB_OMP, ["-fopenmp", "-DORACLE_OMP"])):
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
            continue
        cmd = ["gcc", "-O2", "-std=c99", "-Wno-unknown-pragmas", "-fPIC", "-shared", *extra, SRC, "-o", out + ".tmp",
               "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(out + ".tmp", out)


_libs = {}


def lib(omp: bool = False):
    path = LIB_OMP if omp else LIB_SEQ
    if path not in _libs:
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(SRC):
            build()
        L = C.CDLL(path)
        L.ora_create.restype = C.c_void_p
        L.ora_create.argtypes = [C.POINTER(ThorinParams)]
        L.ora_init_default.argtypes = [C.c_void_p]
        L.ora_refresh.argtypes = [C.c_void_p, C.c_int]
        L.ora_field.restype = C.POINTER(C.c_double)
        L.ora_field.argtypes = [C.c_void_p, C.c_int]
        L.ora_profile.restype = C.POINTER(C.c_double)
        L.ora_profile.argtypes = [C.c_void_p, C.c_int]
        L.ora_radii.restype = C.POINTER(C.c_double)
        L.ora_radii.argtypes = [C.c_void_p]
        L.ora_nshift.restype = C.POINTER(C.c_int)
        L.ora_nshift.argtypes = [C.c_void_p]
        L.ora_set_time.argtypes = [C.c_void_p, C.c_double]
        L.ora_get_stats.argtypes = [C.c_void_p, C.POINTER(ThorinStats)]
        L.ora_algogas.restype = C.c_int
        L.ora_algogas.argtypes = [C.c_void_p, C.POINTER(ThorinPlanets)]
        L.ora_integrals.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 5
        L.ora_sor_array.restype = C.POINTER(C.c_double)
        L.ora_sor_array.argtypes = [C.c_void_p, C.c_int]
        L.ora_sor_omega.restype = C.c_double
        L.ora_sor_omega.argtypes = [C.c_void_p]
        L.ora_set_sor_state.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int]
        L.ora_set_dt_stellar.argtypes = [C.c_void_p, C.c_double]
        L.ora_get_sor_state.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_int)]
        _D = C.POINTER(C.c_double)
        L.ora_set_opacity_table.argtypes = [C.c_int, C.c_int, _D, _D, _D, _D]
        _libs[path] = L
    return _libs[path]


class OracleDisk:
    """One disk advanced by the CPU restatement."""

    def __init__(self, params: ThorinParams, omp: bool = False):
        self.p = params
        self.L = lib(omp)
        self.h = self.L.ora_create(C.byref(params))
        self.nr, self.ns = params.nrad, params.nsec

    def init_default(self):
        self.L.ora_init_default(self.h)

    def refresh(self, flags: int):
        self.L.ora_refresh(self.h, flags)

    def field(self, fid: int) -> np.ndarray:
        ptr = self.L.ora_field(self.h, fid)
        return np.ctypeslib.as_array(ptr, shape=((self.nr + 1) * self.ns,))

    def get(self, fid: int) -> np.ndarray:
        return self.field(fid).copy()

    def set(self, fid: int, values: np.ndarray):
        f = self.field(fid)
        v = np.asarray(values, dtype=np.float64).ravel()
        f[: v.size] = v

    def profile(self, pid: int) -> np.ndarray:
        return np.ctypeslib.as_array(self.L.ora_profile(self.h, pid), shape=(self.nr,))

    def radii(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.L.ora_radii(self.h), shape=(self.nr + 1,)).copy()

    def nshift(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.L.ora_nshift(self.h), shape=(self.nr,)).copy()

    def set_time(self, t: float):
        self.L.ora_set_time(self.h, t)

    def stats(self) -> ThorinStats:
        s = ThorinStats()
        self.L.ora_get_stats(self.h, C.byref(s))
        return s

    def algogas(self, sys_: ThorinPlanets) -> int:
        return self.L.ora_algogas(self.h, C.byref(sys_))

    def integrals(self):
        vals = [C.c_double() for _ in range(5)]
        self.L.ora_integrals(self.h, *[C.byref(v) for v in vals])
        return tuple(v.value for v in vals)

    def set_dt_stellar(self, v: float):
        self.L.ora_set_dt_stellar(self.h, v)

    def sor_state(self):
        om, dom, nl = C.c_double(), C.c_double(), C.c_int()
        self.L.ora_get_sor_state(self.h, C.byref(om), C.byref(dom), C.byref(nl))
        return om.value, dom.value, nl.value

    def set_sor_state(self, omega: float, domega: float, niterlast: int):
        self.L.ora_set_sor_state(self.h, omega, domega, niterlast)

    def sor_system(self) -> dict:
        """The last SOR solve: its five coefficient arrays, RHS, start
        temperature and omega (copies)."""
        n = self.nr * self.ns
        names = ("ml", "mlip", "mlim", "mljp", "mljm", "rhs", "tstart")
        out = {k: np.ctypeslib.as_array(self.L.ora_sor_array(self.h, i), shape=(n,)).copy()
               for i, k in enumerate(names)}
        out["omega"] = self.L.ora_sor_omega(self.h)
        return out

    def set_opacity_table(self, rows, cols, pgrid, tgrid, planck, rosseland):
        """OpacityTable SM03 gas table (shared by all oracle disks)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (pgrid, tgrid, planck, rosseland)]
        self.L.ora_set_opacity_table(int(rows), int(cols), *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs])

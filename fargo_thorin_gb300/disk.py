"""Host-side handle of one disk resident on the GPU (C ABI wrapper)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .params import ThorinParams, ThorinPlanets, ThorinStats


class GpuDisk:
    """One FARGO_THORIN disk advanced by the sm_103a kernels.

    The methods mirror the reference's hydro entry points: ``algogas``
    advances one DT like AlgoGas (src_main/SourceEuler.c:210-317) with the
    planets integrated on the host; ``init_default`` builds the initial state
    of InitEuler; ``refresh`` recomputes derived fields after fields were
    replaced (InitializeFromFile / restart paths of src_main/Init.c)."""

    def __init__(self, params: ThorinParams):
        self.L = _lib.load()
        self.p = params
        self.nr, self.ns = params.nrad, params.nsec
        self.h = C.c_void_p()
        _lib.check(self.L.thorin_gpu_create(C.byref(params), C.byref(self.h)), "thorin_gpu_create")

    def close(self):
        if self.h:
            self.L.thorin_gpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_default(self):
        _lib.check(self.L.thorin_gpu_init_default(self.h), "thorin_gpu_init_default")

    def refresh(self, flags: int):
        _lib.check(self.L.thorin_gpu_refresh(self.h, flags), "thorin_gpu_refresh")

    def get(self, fid: int) -> np.ndarray:
        out = np.zeros((self.nr + 1) * self.ns)
        _lib.check(self.L.thorin_gpu_download(self.h, fid, out.ctypes.data_as(C.POINTER(C.c_double))), "download")
        return out

    def set(self, fid: int, values: np.ndarray):
        cur = self.get(fid)
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        cur[: v.size] = v
        _lib.check(self.L.thorin_gpu_upload(self.h, fid, cur.ctypes.data_as(C.POINTER(C.c_double))), "upload")

    def upload(self, fid: int, full: np.ndarray):
        a = np.ascontiguousarray(full, dtype=np.float64)
        assert a.size == (self.nr + 1) * self.ns
        _lib.check(self.L.thorin_gpu_upload(self.h, fid, a.ctypes.data_as(C.POINTER(C.c_double))), "upload")

    def rings(self):
        """Rinf, Rsup, Rmed and Surf of the disk's grid (FillPolar1DArrays)."""
        arrs = [np.zeros(self.nr) for _ in range(4)]
        _lib.check(self.L.thorin_gpu_get_rings(self.h, *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]),
                   "get_rings")
        return tuple(arrs)

    def set_opacity_table(self, rows, cols, pgrid, tgrid, planck, rosseland):
        """OpacityTable SM03 gas table (InitOpacities, Opacity2.c:247-297)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (pgrid, tgrid, planck, rosseland)]
        _lib.check(self.L.thorin_gpu_set_opacity_table(self.h, int(rows), int(cols),
                                                       *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]),
                   "set_opacity_table")

    def set_frame(self, omega_frame: float):
        """Rotation rate of the frame (OmegaFrame)."""
        _lib.check(self.L.thorin_gpu_set_frame(self.h, omega_frame), "set_frame")

    def set_time(self, t: float):
        _lib.check(self.L.thorin_gpu_set_time(self.h, t), "set_time")

    def algogas(self, sys_: ThorinPlanets) -> int:
        return _lib.check(self.L.thorin_gpu_algogas(self.h, C.byref(sys_)), "thorin_gpu_algogas", ok=(0, 4))

    def algogas_graph(self, sys_: ThorinPlanets) -> int:
        """One DT as a single CUDA graph launch (the disk's first DT runs
        through algogas, which calibrates the SOR omega)."""
        return _lib.check(self.L.thorin_gpu_algogas_graph(self.h, C.byref(sys_)), "thorin_gpu_algogas_graph",
                          ok=(0, 4))

    def graph_supported(self, sys_: ThorinPlanets) -> bool:
        return self.L.thorin_gpu_graph_supported(self.h, C.byref(sys_)) == 0

    def set_launch_shape(self, sor_loop_sweeps: int, sor_threads_per_sm: int):
        _lib.check(self.L.thorin_gpu_set_launch_shape(self.h, sor_loop_sweeps, sor_threads_per_sm), "set_launch_shape")

    def launch_shape(self):
        a, b = C.c_int(), C.c_int()
        _lib.check(self.L.thorin_gpu_get_launch_shape(self.h, C.byref(a), C.byref(b)), "get_launch_shape")
        return a.value, b.value

    def integrals(self):
        vals = [C.c_double() for _ in range(5)]
        _lib.check(self.L.thorin_gpu_integrals(self.h, *[C.byref(v) for v in vals]), "integrals")
        return tuple(v.value for v in vals)

    def nshift(self) -> np.ndarray:
        out = np.zeros(self.nr, dtype=np.int32)
        _lib.check(self.L.thorin_gpu_get_nshift(self.h, out.ctypes.data_as(C.POINTER(C.c_int))), "nshift")
        return out

    def stats(self) -> ThorinStats:
        s = ThorinStats()
        _lib.check(self.L.thorin_gpu_get_stats(self.h, C.byref(s)), "stats")
        return s

    def init_pebbles(self):
        """EquilPebbleDisk on the gas state now on the device."""
        _lib.check(self.L.thorin_gpu_init_pebbles(self.h), "init_pebbles")

    def torques(self):
        """Torque-log records (one per planet) of the last algogas call."""
        from .params import ThorinTorque
        out = (ThorinTorque * 120)()
        n = C.c_int()
        _lib.check(self.L.thorin_gpu_get_torques(self.h, out, 120, C.byref(n)), "get_torques")
        return [out[k] for k in range(min(n.value, 120))]

    def sor_state(self):
        om, dom, nl, cal = C.c_double(), C.c_double(), C.c_int(), C.c_int()
        _lib.check(self.L.thorin_gpu_get_sor_state(self.h, C.byref(om), C.byref(dom), C.byref(nl), C.byref(cal)),
                   "get_sor_state")
        return om.value, dom.value, nl.value, bool(cal.value)

    def set_sor_state(self, omega: float, domega: float, niterlast: int):
        _lib.check(self.L.thorin_gpu_set_sor_state(self.h, omega, domega, niterlast), "set_sor_state")

    def dt_stellar(self) -> float:
        v = C.c_double()
        _lib.check(self.L.thorin_gpu_get_dt_stellar(self.h, C.byref(v)), "get_dt_stellar")
        return v.value

    def set_dt_stellar(self, v: float):
        _lib.check(self.L.thorin_gpu_set_dt_stellar(self.h, v), "set_dt_stellar")

    def snapshot(self, fields) -> dict:
        """The state a later DT starts from: the given fields (with c_s and
        T), the SOR omega schedule, the clock and dt_stellar."""
        return {"fields": {f: self.get(f) for f in fields}, "sor": self.sor_state(),
                "time": self.stats().physical_time, "dt_stellar": self.dt_stellar()}

    def restore(self, snap: dict):
        for f, v in snap["fields"].items():
            self.upload(f, v)
        self.set_sor_state(*snap["sor"][:3])
        self.set_time(snap["time"])
        self.set_dt_stellar(snap["dt_stellar"])
        self.refresh(4)                   # THORIN_REFRESH_RING_MEANS

    def set_timing(self, on: bool):
        _lib.check(self.L.thorin_gpu_set_timing(self.h, 1 if on else 0), "set_timing")

    def stream(self) -> int:
        ptr = C.c_void_p()
        _lib.check(self.L.thorin_gpu_get_stream(self.h, C.byref(ptr)), "get_stream")
        return ptr.value or 0

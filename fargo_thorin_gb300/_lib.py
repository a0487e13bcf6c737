"""Loader of the in-tree CUDA library (libthorin_gpu.so) through its C ABI.

There is no CPU fallback: if the library is missing or cannot be loaded the
import fails with the reason.
"""
from __future__ import annotations

import ctypes as C
import os

from .params import ThorinParams, ThorinPlanets, ThorinStats, ThorinTorque

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libthorin_gpu.so")

# exported symbols: name -> (restype, argtypes)
_P = C.c_void_p
_D = C.POINTER(C.c_double)
SIGNATURES = {
    "thorin_params_default": (None, [C.POINTER(ThorinParams), C.c_int, C.c_int]),
    "thorin_gpu_create": (C.c_int, [C.POINTER(ThorinParams), C.POINTER(_P)]),
    "thorin_gpu_destroy": (C.c_int, [_P]),
    "thorin_gpu_init_default": (C.c_int, [_P]),
    "thorin_gpu_upload": (C.c_int, [_P, C.c_int, _D]),
    "thorin_gpu_download": (C.c_int, [_P, C.c_int, _D]),
    "thorin_gpu_refresh": (C.c_int, [_P, C.c_int]),
    "thorin_gpu_set_profile": (C.c_int, [_P, C.c_int, _D]),
    "thorin_gpu_get_profile": (C.c_int, [_P, C.c_int, _D]),
    "thorin_gpu_get_rings": (C.c_int, [_P, _D, _D, _D, _D]),
    "thorin_gpu_set_time": (C.c_int, [_P, C.c_double]),
    "thorin_gpu_cfl": (C.c_int, [_P, C.c_double, C.c_double, C.POINTER(C.c_int)]),
    "thorin_gpu_accrete": (C.c_int, [_P, C.POINTER(ThorinPlanets), C.c_double]),
    "thorin_gpu_forces": (C.c_int, [_P, C.POINTER(ThorinPlanets), C.c_double, _D, _D, _D]),
    "thorin_gpu_hydro": (C.c_int, [_P, C.c_double]),
    "thorin_advance_from_disk": (C.c_int, [_P, C.POINTER(ThorinPlanets), C.c_double, _D, _D, _D]),
    "thorin_gpu_correct_vtheta": (C.c_int, [_P, C.c_double]),
    "thorin_gpu_stokes": (C.c_int, [_P]),
    "thorin_gpu_algogas": (C.c_int, [_P, C.POINTER(ThorinPlanets)]),
    "thorin_gpu_algogas_graph": (C.c_int, [_P, C.POINTER(ThorinPlanets)]),
    "thorin_gpu_graph_supported": (C.c_int, [_P, C.POINTER(ThorinPlanets)]),
    "thorin_gpu_set_launch_shape": (C.c_int, [_P, C.c_int, C.c_int]),
    "thorin_gpu_get_launch_shape": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "thorin_ensemble_algogas_graph": (C.c_int, [C.POINTER(_P), C.POINTER(_P), C.c_int, C.POINTER(C.c_int)]),
    "thorin_gpu_integrals": (C.c_int, [_P, _D, _D, _D, _D, _D]),
    "thorin_gpu_get_nshift": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "thorin_gpu_get_stats": (C.c_int, [_P, C.POINTER(ThorinStats)]),
    "thorin_gpu_get_sor_state": (C.c_int, [_P, _D, _D, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "thorin_gpu_set_sor_state": (C.c_int, [_P, C.c_double, C.c_double, C.c_int]),
    "thorin_gpu_set_timing": (C.c_int, [_P, C.c_int]),
    "thorin_gpu_get_dt_stellar": (C.c_int, [_P, _D]),
    "thorin_gpu_set_dt_stellar": (C.c_int, [_P, C.c_double]),
    "thorin_gpu_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "thorin_integrals_static": (C.c_int, [_D, _D, _D, _D, _D, _D, _D, _D, C.c_int, C.c_int, C.c_double, _D, _P]),
    "thorin_selftest_division": (C.c_int, [C.c_longlong, C.c_ulonglong, C.c_double, C.POINTER(C.c_ulonglong),
                                           C.POINTER(C.c_ulonglong)]),
    "thorin_selftest_slope_division": (C.c_int, [C.c_longlong, C.c_ulonglong, C.c_double,
                                                 C.POINTER(C.c_ulonglong)]),
    "thorin_selftest_graph_conditional": (C.c_int, [C.POINTER(C.c_int)] * 3),
    "thorin_selftest_graph_nested": (C.c_int, [C.POINTER(C.c_int)] * 2),
    "thorin_selftest_fp64_peak": (C.c_int, [_D]),
    "thorin_gpu_request_torques": (C.c_int, [_P]),
    "thorin_gpu_init_pebbles": (C.c_int, [_P]),
    "thorin_gpu_drag": (C.c_int, [_P, C.POINTER(ThorinPlanets), C.c_double]),
    "thorin_gpu_set_frame": (C.c_int, [_P, C.c_double]),
    "thorin_gpu_set_opacity_table": (C.c_int, [_P, C.c_int, C.c_int, _D, _D, _D, _D]),
    "thorin_gpu_get_torques": (C.c_int, [_P, C.POINTER(ThorinTorque), C.c_int, C.POINTER(C.c_int)]),
    "thorin_gpu_last_error": (C.c_char_p, []),
    # learned SOR warm start (include/thorin_warmnet.h)
    "thorin_warmnet_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(_P)]),
    "thorin_warmnet_destroy": (C.c_int, [_P]),
    "thorin_warmnet_set_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_int]),
    "thorin_warmnet_get_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_int]),
    "thorin_warmnet_forward": (C.c_int, [_P, C.c_int, C.POINTER(C.c_uint16), C.POINTER(C.c_float)]),
    "thorin_warmnet_gradient": (C.c_int, [_P, C.c_int, C.POINTER(C.c_uint16), C.POINTER(C.c_float),
                                          C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "thorin_warmnet_adam": (C.c_int, [_P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]),
    "thorin_gpu_warmstart": (C.c_int, [_P, _P, C.c_int, C.c_float]),
    "thorin_gpu_warmstart_stats": (C.c_int, [_P, _P]),
    "thorin_gpu_warmstart_order": (C.c_int, [_P, C.c_int]),
    # ensembles (include/thorin_ensemble.h)
    "thorin_ensemble_algogas": (C.c_int, [C.POINTER(_P), C.POINTER(_P), C.c_int, C.c_int, C.c_int,
                                          C.POINTER(C.c_int)]),
    "thorin_ensemble_tune": (C.c_int, [C.POINTER(_P), C.POINTER(_P), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), _D, _D]),
    "thorin_warmstart_coefficients": (C.c_int, [C.c_int, _D]),
    "thorin_selftest_bounded_wait": (C.c_int, [C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "thorin_selftest_umma": (C.c_int, [C.POINTER(C.c_uint16), C.POINTER(C.c_uint16), C.POINTER(C.c_float)]),
    "thorin_planet_from_elements": (C.c_int, [C.POINTER(ThorinPlanets), C.c_int] + [C.c_float] * 9),
}

_lib = None


def load(path: str = LIB_PATH):
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise ImportError(f"{path} is missing: build it with fargo_thorin_gb300.build.build()")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class ThorinError(RuntimeError):
    CODES = {1: "ARG", 2: "CUDA", 3: "CRASH", 4: "SOR_MAXIT", 5: "TIMEOUT", 6: "STATE", 7: "NOMEM", 8: "OMEGA"}

    def __init__(self, code: int, where: str):
        msg = load().thorin_gpu_last_error().decode(errors="replace")
        super().__init__(f"{where}: THORIN_ERR_{self.CODES.get(code, code)} ({msg})")
        self.code = code


def check(code: int, where: str, ok=(0,)):
    if code not in ok:
        raise ThorinError(code, where)
    return code

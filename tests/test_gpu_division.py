"""The kernels divide with a reciprocal estimate, one Newton-Raphson step and
Markstein's correction instead of the IEEE divide sequence.  This checks the
routine against CUDA's IEEE division on the GPU over random operands: at
most one ulp apart, and in practice identical."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("max_exponent,seed", [(40.0, 1), (300.0, 2), (1000.0, 3)])
def test_division_matches_ieee(max_exponent, seed):
    from fargo_thorin_gb300 import _lib
    lib = _lib.load()
    n = 1 << 26
    mis, ulp = C.c_ulonglong(), C.c_ulonglong()
    _lib.check(lib.thorin_selftest_division(n, seed, max_exponent, C.byref(mis), C.byref(ulp)), "selftest_division")
    assert ulp.value <= 1
    assert mis.value <= n // 1000000


@pytest.mark.parametrize("max_exponent,seed", [(40.0, 4), (300.0, 5)])
def test_slope_division_bound(max_exponent, seed):
    """The van Leer slopes' division (no Markstein correction) stays within
    2^14 ulp of IEEE division, a relative error below 2^-38 (measured on
    GB300: 8696 ulp at most in 2^26 quotients)."""
    from fargo_thorin_gb300 import _lib
    lib = _lib.load()
    ulp = C.c_ulonglong()
    _lib.check(lib.thorin_selftest_slope_division(1 << 26, seed, max_exponent, C.byref(ulp)),
               "selftest_slope_division")
    print("slope division: max", ulp.value, "ulp")
    assert ulp.value <= 16384


def test_graph_conditional_nodes():
    """The SOR sweep loop is a WHILE graph node whose condition the last
    sweep's completion step clears; this checks the mechanism in bounded
    form first (IF nodes), then a WHILE node of five runs."""
    from fargo_thorin_gb300 import _lib
    lib = _lib.load()
    a, b, w = C.c_int(), C.c_int(), C.c_int()
    _lib.check(lib.thorin_selftest_graph_conditional(C.byref(a), C.byref(b), C.byref(w)),
               "selftest_graph_conditional")
    assert (a.value, b.value, w.value) == (0, 1, 5)


def test_graph_nested_conditional_nodes():
    """A WHILE node inside a WHILE node's body (the substep loop around the
    SOR sweep loop of a whole-DT graph), bounded: 3 outer runs of 4 inner."""
    from fargo_thorin_gb300 import _lib
    lib = _lib.load()
    o, i = C.c_int(), C.c_int()
    _lib.check(lib.thorin_selftest_graph_nested(C.byref(o), C.byref(i)), "selftest_graph_nested")
    assert (o.value, i.value) == (3, 12)

"""Failure detection without a GPU fault: the bounded mbarrier wait that
every tensor-core kernel uses gives up after its poll limit when nothing
arrives, the kernel returns normally, the host reads the outcome, and the
context stays usable for the next launches."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_on_a_barrier_nothing_arrives_at_gives_up():
    from fargo_thorin_gb300 import _lib
    lib = _lib.load()
    t, ok = C.c_int(-1), C.c_int(-1)
    _lib.check(lib.thorin_selftest_bounded_wait(1000, C.byref(t), C.byref(ok)), "selftest_bounded_wait")
    assert t.value == 1 and ok.value == 1
    # the context is still usable: the tensor-core layout check runs and is exact
    rng = np.random.default_rng(0)
    a = rng.integers(-8, 8, (128, 64)).astype(np.float32)
    b = rng.integers(-8, 8, (32, 64)).astype(np.float32)
    bits = lambda x: (x.view(np.uint32) >> 16).astype(np.uint16)   # small integers are exact in bf16
    d = np.zeros((128, 32), np.float32)
    _lib.check(lib.thorin_selftest_umma(bits(a).ctypes.data_as(C.POINTER(C.c_uint16)),
                                        bits(b).ctypes.data_as(C.POINTER(C.c_uint16)),
                                        d.ctypes.data_as(C.POINTER(C.c_float))), "selftest_umma")
    assert np.array_equal(d, a @ b.T)


def test_poll_limit_is_checked():
    from fargo_thorin_gb300 import _lib
    lib = _lib.load()
    t, ok = C.c_int(), C.c_int()
    assert lib.thorin_selftest_bounded_wait(0, C.byref(t), C.byref(ok)) != 0

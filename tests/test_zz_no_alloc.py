"""The allocation-free integrals entry point against the regular one.

thorin_integrals_static serves callers that cannot allocate device memory
(a host program whose own pool already owns the free GPU memory, or a hook in
a latency-critical loop where a cudaMalloc could synchronise the device).  It
reads fields the caller already keeps on the GPU and uses a fixed device
array for its partial sums.  This test gives it device copies of a disk's
fields and compares its mass, momentum and energy with those of
thorin_gpu_integrals on the same state, on two calls in a row (the second
after the disk has advanced, so a stale partials array would show).  It is
collected last so that a failure here never stops the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import harness as H

pytestmark = pytest.mark.gpu
TOL = 1e-12       # summation order differs from the regular entry point


def test_static_integrals_match_regular_entry_point():
    import torch
    from fargo_thorin_gb300 import _lib, workloads
    from fargo_thorin_gb300.disk import GpuDisk
    g = H.load("disk0_24x72")
    p = H.case_params(g)
    d = GpuDisk(p)
    d.init_default()
    H.start_state(d, p, {"dens": g["init_dens"].ravel(), "temper": g["init_temper"].ravel()})
    sys_ = workloads.make_planets(p, [tuple(g["planet"])])
    L = _lib.load()
    dev = torch.device("cuda", 0)
    # the disk's own ring geometry (FillPolar1DArrays), as the regular entry point uses it
    rinf, rsup, rmed, surf = (torch.tensor(a, dtype=torch.float64, device=dev) for a in d.rings())
    out = torch.full((3,), float("nan"), dtype=torch.float64, device=dev)
    ptr = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_double))
    for call in range(2):
        d.algogas(sys_)
        fields = [torch.tensor(d.get(f), dtype=torch.float64, device=dev) for f in (0, 1, 2, 3)]
        stream = torch.cuda.current_stream(dev)
        rc = L.thorin_integrals_static(*[ptr(t) for t in fields], ptr(surf), ptr(rinf), ptr(rsup), ptr(rmed),
                                       p.nrad, p.nsec, p.omega_frame, ptr(out), C.c_void_p(stream.cuda_stream))
        assert rc == 0, L.thorin_gpu_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        want = np.array(d.integrals()[:3])
        np.testing.assert_allclose(got, want, rtol=TOL, atol=0, err_msg=f"call {call + 1}")
        out.fill_(float("nan"))
    d.close()


def test_static_integrals_reject_too_many_rings():
    import torch
    from fargo_thorin_gb300 import _lib
    L = _lib.load()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    ptr = C.cast(x.data_ptr(), C.POINTER(C.c_double))
    rc = L.thorin_integrals_static(ptr, ptr, ptr, ptr, ptr, ptr, ptr, ptr, 16385, 4, 0.0, ptr, None)
    assert rc == 1
    assert b"16384" in L.thorin_gpu_last_error()

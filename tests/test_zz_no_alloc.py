"""The allocation-free branching entry point, called through the C ABI.

jqmc_branch_comb_noalloc exists for callers that may not allocate device
memory -- a host code whose own pool already owns the GPU's memory, or a driver
loop that must not wait on an allocation.  Its scratch is a fixed device array
inside the library, shared by every call.  This test checks that two calls in a
row give exactly the walker indices of jqmc_branch_comb (integer output, so the
tolerance is zero), which also shows that the shared array's leftovers from the
first call do not leak into the second.  The file is named to be collected
last, so a failure here cannot hide the results of the other GPU tests.
"""

import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_noalloc_branch_matches_branch_comb_twice():
    from jqmc_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(2024)
    for nwalk, zeta in ((8192, 0.731), (1000, 0.052)):   # the second call is smaller than the first
        w = torch.as_tensor(rng.uniform(0.05, 3.0, size=nwalk), device="cuda")
        ref = torch.empty(nwalk, dtype=torch.int32, device="cuda")
        cum = torch.empty(nwalk, dtype=torch.float64, device="cuda")
        _lib.check(L.jqmc_branch_comb(nwalk, C.c_void_p(w.data_ptr()), zeta, C.c_void_p(ref.data_ptr()),
                                      C.c_void_p(cum.data_ptr()), _stream()), "jqmc_branch_comb")
        got = torch.full((nwalk,), -1, dtype=torch.int32, device="cuda")
        _lib.check(L.jqmc_branch_comb_noalloc(nwalk, C.c_void_p(w.data_ptr()), zeta, C.c_void_p(got.data_ptr()),
                                              _stream()), "jqmc_branch_comb_noalloc")
        torch.cuda.synchronize()
        assert torch.equal(got, ref)


def test_noalloc_branch_rejects_oversize():
    from jqmc_gb300 import _lib
    L = _lib.lib()
    w = torch.ones(4, dtype=torch.float64, device="cuda")
    out = torch.empty(4, dtype=torch.int32, device="cuda")
    rc = L.jqmc_branch_comb_noalloc(262144 + 1, C.c_void_p(w.data_ptr()), 0.5, C.c_void_p(out.data_ptr()), _stream())
    assert rc == -2

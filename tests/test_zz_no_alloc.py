"""N_VDotProdMultiNoAlloc_GB300: the allocation-free dot products, for callers
that cannot let the library allocate device memory.

Called through the C ABI with raw device pointers, it must give the same
results as the regular fused DotProdMulti of the N_Vector ops table -- the
tolerance of the other reduction tests (1e-12 * sum|terms|) is checked, and
the bits are in fact identical -- on two calls in a row (the static scratch
keeps the previous call's contents).  This file is collected last so that a
run stopping at the first failure has run every other test first."""
import ctypes as ct

import numpy as np
import pytest

from sundials_gb300 import _lib
from sundials_gb300.nvector import NVector

pytestmark = pytest.mark.gpu
SUM_RTOL = 1e-12


def _fn(lib):
    f = lib.N_VDotProdMultiNoAlloc_GB300
    f.restype = ct.c_int
    f.argtypes = [ct.c_int, ct.c_void_p, ct.POINTER(ct.c_void_p), ct.c_int64, ct.c_void_p,
                  ct.c_void_p]
    return f


@pytest.mark.parametrize("n,nvec", [(100003, 5), ((1 << 20) + 1, 8), (33, 3), (1, 1)])
def test_no_alloc_matches_ops_table_twice(gb300_lib, n, nvec):
    f = _fn(gb300_lib)
    rng = np.random.default_rng(2024)
    x = rng.uniform(-1, 1, n)
    ys = [rng.uniform(-1, 1, n) for _ in range(nvec)]
    X = NVector.from_numpy(x)
    Ys = [NVector.from_numpy(y) for y in ys]
    ref = (ct.c_double * nvec)()
    assert X.ops["nvdotprodmulti"](nvec, X.v, _lib.nv_array([v.v for v in Ys]), ref) == 0
    out = NVector(nvec)  # receives the results (device array)
    ptrs = (ct.c_void_p * nvec)(*[v.device_ptr for v in Ys])
    for call in range(2):
        out.set(np.full(nvec, np.nan))
        rc = f(nvec, X.device_ptr, ptrs, n, out.device_ptr, None)
        assert rc == 0, gb300_lib.SUNGB300_GetLastErrorMessage()
        got = out.get()
        for k in range(nvec):
            bound = SUM_RTOL * float(np.sum(np.abs(x * ys[k]))) + 1e-300
            assert abs(got[k] - ref[k]) <= bound, (call, k)
        assert np.array_equal(got.view(np.int64), np.array(list(ref)).view(np.int64)), call


def test_no_alloc_rejects_too_many_vectors(gb300_lib):
    f = _fn(gb300_lib)
    X = NVector.from_numpy(np.ones(16))
    out = NVector(16)
    ptrs = (ct.c_void_p * 9)(*([X.device_ptr] * 9))
    rc = f(9, X.device_ptr, ptrs, 16, out.device_ptr, None)
    assert rc == -9997  # SUN_ERR_ARG_OUTOFRANGE
    assert b"must be 1..8" in gb300_lib.SUNGB300_GetLastErrorMessage()

"""CPU: the fixed-point solver restatement (oracle/fixedpoint_port.c) against
the reference's own SUNNonlinSol_FixedPoint on a small contraction, with
enough iterations (maxiters 25) that Anderson acceleration fills its
subspace and recycles it by Givens rotations -- a branch the integrators'
three iterations per solve never reach.  Both sides run on the reference's
NVECTOR_SERIAL with the same fixed-point function and convergence test:
every iterate, the iteration and failure counts and the status must be
identical, bit for bit."""
import ctypes as ct

import numpy as np
import pytest

from oracle import heat_cvode as hc
from oracle import port

needs_ref = pytest.mark.skipif(not hc.REF_LIB.exists(),
                               reason="reference library not built on this machine")
VP, D, I = ct.c_void_p, ct.c_double, ct.c_int
SYS_FN = ct.CFUNCTYPE(I, VP, VP, VP)                 # SUNNonlinSolSysFn(ycor, g, mem)
CTEST_FN = ct.CFUNCTYPE(I, VP, VP, VP, D, VP, VP)    # (NLS, ycor, del, tol, ewt, data)
PSYS_FN = ct.CFUNCTYPE(I, VP, VP, VP)                # port: (mem, ycor, g)
PCTEST_FN = ct.CFUNCTYPE(I, VP, VP, VP, D, I)        # port: (mem, ycor, del, tol, curiter)
N = 40


def _g(y):
    """A contraction with coupling: g_i = 0.5 cos(y_i) + 0.3 y_{i+1} + 0.1."""
    return 0.5 * np.cos(y) + 0.3 * np.roll(y, -1) + 0.1


def _libs():
    L = hc.ref_lib()
    for name, res, args in [("SUNNonlinSol_FixedPoint", VP, [VP, I, VP]),
                            ("SUNNonlinSolSetSysFn", I, [VP, VP]),
                            ("SUNNonlinSolSetConvTestFn", I, [VP, VP, VP]),
                            ("SUNNonlinSolSetMaxIters", I, [VP, I]),
                            ("SUNNonlinSolInitialize", I, [VP]),
                            ("SUNNonlinSolSolve", I, [VP, VP, VP, VP, D, I, VP]),
                            ("SUNNonlinSolGetNumIters", I, [VP, ct.POINTER(ct.c_long)]),
                            ("SUNNonlinSolGetNumConvFails", I, [VP, ct.POINTER(ct.c_long)]),
                            ("SUNNonlinSolFree", I, [VP]),
                            ("N_VWrmsNorm", D, [VP, VP])]:
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    P = port.lib()
    P.fp_port_create.restype, P.fp_port_create.argtypes = VP, [VP, I]
    P.fp_port_set_maxiters.restype, P.fp_port_set_maxiters.argtypes = None, [VP, I]
    P.fp_port_solve.restype, P.fp_port_solve.argtypes = I, [VP, VP, D, VP, VP, VP]
    P.fp_port_niters.restype, P.fp_port_niters.argtypes = ct.c_long, [VP]
    P.fp_port_nconvfails.restype, P.fp_port_nconvfails.argtypes = ct.c_long, [VP]
    P.fp_port_free.restype, P.fp_port_free.argtypes = None, [VP]
    return L, P


@needs_ref
@pytest.mark.parametrize("m,maxiters,tol", [(0, 25, 1e-12), (1, 25, 1e-12), (2, 25, 1e-13),
                                            (3, 25, 1e-14), (5, 25, 1e-14), (3, 4, 1e-14)])
def test_fixed_point_bit_identical_to_reference(m, maxiters, tol):
    L, P = _libs()
    ctx = VP()
    assert L.SUNContext_Create(0, ct.byref(ctx)) == 0
    vecs = [L.N_VNew_Serial(N, ctx) for _ in range(4)]
    y0, w, ycor_r, ycor_p = vecs
    arr = lambda v: np.ctypeslib.as_array(L.N_VGetArrayPointer(v), shape=(N,))  # noqa: E731
    rng = np.random.default_rng(5)
    arr(y0)[:] = 0.0
    arr(w)[:] = 1.0 / (1e-6 * np.abs(rng.uniform(0.5, 1.5, N)) + 1e-8)
    start = rng.uniform(-1.0, 1.0, N)
    iterates = {"ref": [], "port": []}

    def record(key, v):
        iterates[key].append(arr(v).copy())

    def sys_ref(ycor, g, mem):
        arr(g)[:] = _g(arr(ycor))
        return 0

    def ctest_ref(nls, ycor, dl, tl, ewt, data):
        record("ref", ycor)
        return 0 if L.N_VWrmsNorm(dl, ewt) <= tl else 901

    def sys_port(mem, ycor, g):
        arr(g)[:] = _g(arr(ycor))
        return 0

    def ctest_port(mem, ycor, dl, tl, curiter):
        record("port", ycor)
        return 0 if L.N_VWrmsNorm(dl, w) <= tl else 901

    cbs = (SYS_FN(sys_ref), CTEST_FN(ctest_ref), PSYS_FN(sys_port), PCTEST_FN(ctest_port))
    NLS = L.SUNNonlinSol_FixedPoint(y0, m, ctx)
    assert L.SUNNonlinSolSetSysFn(NLS, ct.cast(cbs[0], VP)) == 0
    assert L.SUNNonlinSolSetConvTestFn(NLS, ct.cast(cbs[1], VP), None) == 0
    assert L.SUNNonlinSolSetMaxIters(NLS, maxiters) == 0
    assert L.SUNNonlinSolInitialize(NLS) == 0
    arr(ycor_r)[:] = start
    flag_r = L.SUNNonlinSolSolve(NLS, y0, ycor_r, w, tol, 0, None)
    it_r, cf_r = ct.c_long(), ct.c_long()
    L.SUNNonlinSolGetNumIters(NLS, ct.byref(it_r))
    L.SUNNonlinSolGetNumConvFails(NLS, ct.byref(cf_r))
    fp = P.fp_port_create(y0, m)
    P.fp_port_set_maxiters(fp, maxiters)
    arr(ycor_p)[:] = start
    flag_p = P.fp_port_solve(fp, ycor_p, tol, ct.cast(cbs[2], VP), ct.cast(cbs[3], VP), None)
    try:
        assert flag_p == flag_r
        assert P.fp_port_niters(fp) == it_r.value and P.fp_port_nconvfails(fp) == cf_r.value
        assert len(iterates["port"]) == len(iterates["ref"])
        for a, b in zip(iterates["port"], iterates["ref"]):
            assert np.array_equal(a.view(np.int64), b.view(np.int64))
        if m > 0 and maxiters > m + 1:
            assert it_r.value > m + 1  # the recycling branch ran
    finally:
        P.fp_port_free(fp)
        L.SUNNonlinSolFree(NLS)
        for v in vecs:
            L.N_VDestroy(v)
        L.SUNContext_Free(ct.byref(ctx))

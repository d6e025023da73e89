"""TEST ORACLE (checker only): CVODE runs of user problems with SPGMR
(``run_reference_with`` / ``run_port`` / ``run_port_serial_with``, used by
oracle/robertson_cvode.py too), and the 2-D heat problem of
examples/cvode/CXX_serial/cv_heat2D.cpp -- 5-point stencil on the nx x ny
interior grid, zero Dirichlet boundaries, no forcing term, BDF + Newton +
SPGMR (left preconditioning, maxl 5) with the user J v and the Jacobi
preconditioner (cv_heat2D.cpp:371-408) -- by two drivers:

* ``run_reference``: the reference's own CVode and its NVECTOR_SERIAL /
  SUNLINSOL_SPGMR objects (``oracle/_ref``, built where the reference sources
  are present) with serial callbacks restated here in numpy;
* ``run_port``: the C restatement ``oracle/cvode_ls_port.c`` (in
  ``oracle/_build/liboracle.so``), which drives any N_Vector and
  SUNLinearSolver through their ops tables -- the reference's serial objects
  (to pin it against ``run_reference``) or NVECTOR_GB300 +
  SUNLinSol_SPGMR_GB300 with the device callbacks of include/heat2d_gb300.h.

Both return the counters after every output time (COUNTER_NAMES) and the
solutions there."""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

from . import heat2d_port as hp
from . import port

REF_LIB = Path(__file__).resolve().parent / "_ref" / "libsundials_ref.so"
COUNTER_NAMES = ("nst", "nfe", "nni", "nnf", "ncfn", "netf", "nsetups", "nli", "npe", "nps",
                 "njtimes", "ncfl", "qu", "q", "nfels", "nje")
REAL_NAMES = ("hu", "h", "tn", "h0u")
# CVLS getters, which fail when no linear solver is attached
LS_GETTERS = ("CVodeGetNumLinIters", "CVodeGetNumPrecEvals", "CVodeGetNumPrecSolves",
              "CVodeGetNumJtimesEvals", "CVodeGetNumLinConvFails")

VP, D, I, I64 = ct.c_void_p, ct.c_double, ct.c_int, ct.c_int64
RHS_FN = ct.CFUNCTYPE(I, D, VP, VP, VP)
JTIMES_FN = ct.CFUNCTYPE(I, VP, VP, D, VP, VP, VP, VP)
PSETUP_FN = ct.CFUNCTYPE(I, D, VP, VP, I, ct.POINTER(I), D, VP)
PSOLVE_FN = ct.CFUNCTYPE(I, D, VP, VP, VP, VP, D, D, I, VP)
JAC_FN = ct.CFUNCTYPE(I, D, VP, VP, VP, VP, VP, VP, VP)


def initial(nx: int, ny: int, seed: int = 1) -> np.ndarray:
    """u0 = sin(pi x) sin(pi y) + U(-1e-3, 1e-3) on the interior points, row by row."""
    x = np.arange(1, nx + 1) / (nx + 1)
    y = np.arange(1, ny + 1) / (ny + 1)
    u = np.sin(np.pi * y)[:, None] * np.sin(np.pi * x)[None, :]
    return (u + np.random.default_rng(seed).uniform(-1e-3, 1e-3, (ny, nx))).reshape(-1)


def ref_lib() -> ct.CDLL:
    L = ct.CDLL(str(REF_LIB))
    for name, res, args in [
        ("SUNContext_Create", I, [I, ct.POINTER(VP)]),
        ("SUNContext_Free", I, [ct.POINTER(VP)]),
        ("N_VNew_Serial", VP, [I64, VP]),
        ("N_VNew_OpenMP", VP, [I64, I, VP]),
        ("N_VDestroy", None, [VP]),
        ("N_VGetArrayPointer", ct.POINTER(D), [VP]),
        ("SUNLinSol_SPGMR", VP, [VP, I, I, VP]),
        ("SUNDenseMatrix", VP, [I64, I64, VP]),
        ("SUNDenseMatrix_Data", ct.POINTER(D), [VP]),
        ("SUNMatDestroy", None, [VP]),
        ("SUNLinSol_Dense", VP, [VP, VP, VP]),
        ("CVodeSetJacFn", I, [VP, VP]),
        ("SUNLinSolFree", I, [VP]),
        ("CVodeCreate", VP, [I, VP]),
        ("CVodeInit", I, [VP, VP, D, VP]),
        ("CVodeSStolerances", I, [VP, D, D]),
        ("CVodeSVtolerances", I, [VP, D, VP]),
        ("CVodeSetMaxNumSteps", I, [VP, ct.c_long]),
        ("CVodeSetLinearSolver", I, [VP, VP, VP]),
        ("CVodeSetJacTimes", I, [VP, VP, VP]),
        ("CVodeSetPreconditioner", I, [VP, VP, VP]),
        ("CVode", I, [VP, D, VP, ct.POINTER(D), I]),
        ("CVodeFree", None, [ct.POINTER(VP)]),
        ("SUNNonlinSol_FixedPoint", VP, [VP, I, VP]),
        ("CVodeSetNonlinearSolver", I, [VP, VP]),
        ("SUNNonlinSolFree", I, [VP]),
    ]:
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    for name in ("CVodeGetNumSteps", "CVodeGetNumRhsEvals", "CVodeGetNumNonlinSolvIters",
                 "CVodeGetNumNonlinSolvConvFails", "CVodeGetNumStepSolveFails",
                 "CVodeGetNumErrTestFails", "CVodeGetNumLinSolvSetups", "CVodeGetNumLinIters",
                 "CVodeGetNumPrecEvals", "CVodeGetNumPrecSolves", "CVodeGetNumJtimesEvals",
                 "CVodeGetNumLinConvFails", "CVodeGetNumLinRhsEvals", "CVodeGetNumJacEvals"):
        f = getattr(L, name)
        f.restype, f.argtypes = I, [VP, ct.POINTER(ct.c_long)]
    for name in ("CVodeGetLastOrder", "CVodeGetCurrentOrder"):
        f = getattr(L, name)
        f.restype, f.argtypes = I, [VP, ct.POINTER(I)]
    for name in ("CVodeGetLastStep", "CVodeGetCurrentStep", "CVodeGetCurrentTime",
                 "CVodeGetActualInitStep"):
        f = getattr(L, name)
        f.restype, f.argtypes = I, [VP, ct.POINTER(D)]
    return L


def port_lib() -> ct.CDLL:
    L = port.lib()
    if not getattr(L, "_cvls_declared", False):
        L.cvls_port_create.restype = VP
        L.cvls_port_create.argtypes = [VP, D, VP, D, D, ct.c_long, VP, VP, VP, VP, VP]
        L.cvls_port_solve.restype = I
        L.cvls_port_solve.argtypes = [VP, D, VP, ct.POINTER(D)]
        L.cvls_port_stats.restype = None
        L.cvls_port_stats.argtypes = [VP, ct.POINTER(ct.c_long), ct.POINTER(D)]
        L.cvls_port_free.restype = None
        L.cvls_port_free.argtypes = [VP]
        L.cvls_port_set_vabstol.restype = None
        L.cvls_port_set_vabstol.argtypes = [VP, D, VP]
        L.cvls_port_set_matrix.restype = None
        L.cvls_port_set_matrix.argtypes = [VP, VP, VP]
        L.cvls_port_set_fixed_point.restype = None
        L.cvls_port_set_fixed_point.argtypes = [VP, I]
        L.cvls_port_set_adams.restype = None
        L.cvls_port_set_adams.argtypes = [VP]
        L._cvls_declared = True
    return L


class SerialHeat:
    """The problem's callbacks on NVECTOR_SERIAL vectors of the reference
    library, rounded like the device callbacks (oracle/heat2d_port.py)."""

    def __init__(self, L, nx: int, ny: int):
        self.L, self.nx, self.ny, self.n = L, nx, ny, nx * ny
        self.cc = hp.coefficients(nx, ny)[2]
        self.d = 1.0

        def arr(v):
            return np.ctypeslib.as_array(L.N_VGetArrayPointer(v), shape=(self.n,))

        def f(t, y, ydot, data):
            arr(ydot)[:] = hp.jv(arr(y), nx, ny)
            return 0

        def jtimes(v, jv, t, y, fy, data, tmp):
            arr(jv)[:] = hp.jv(arr(v), nx, ny)
            return 0

        def psetup(t, y, fy, jok, jcur, gamma, data):
            self.d = 1.0 / (1.0 - gamma * self.cc)
            return 0

        def psolve(t, y, fy, r, z, gamma, delta, lr, data):
            arr(z)[:] = self.d * arr(r)
            return 0

        self.cbs = (RHS_FN(f), JTIMES_FN(jtimes), PSETUP_FN(psetup), PSOLVE_FN(psolve))
        self.arr = arr

    def addresses(self):
        return tuple(ct.cast(c, VP).value for c in self.cbs)


def run_reference(nx: int, ny: int, touts, rtol=1e-6, atol=1e-10, mxstep=100000, threads=None):
    """The reference's CVode on the heat problem with serial vectors (or,
    with threads = k, NVECTOR_OPENMP on k threads, whose reductions sum in
    another order): (counters [len(touts), 14], reals [len(touts), 4],
    solutions [len(touts), nx*ny], u0)."""
    u0 = initial(nx, ny)
    c, r, s = run_reference_with(lambda L: SerialHeat(L, nx, ny), u0, touts, rtol, atol, mxstep,
                                 threads)
    return c, r, s, u0


def run_reference_with(make_serial, u0, touts, rtol, atol, mxstep=100000, threads=None,
                       direct=False, fixed_point=None, adams=False):
    """The reference's CVode (BDF, Newton, SPGMR with left preconditioning and
    maxl 5, user J v and preconditioner) on the problem whose serial
    callbacks make_serial(L) builds (an object with .addresses() -> (f,
    jtimes, psetup, psolve) and .arr(N_Vector) -> numpy view).  atol: a
    scalar (CVodeSStolerances) or an array (CVodeSVtolerances).  direct:
    SUNDenseMatrix + SUNLINSOL_DENSE and the problem's .jac_address() instead
    (the matrix-based path of CVLS).  fixed_point = m: SUNNonlinSol_FixedPoint
    with Anderson depth m and no linear solver (the linear-solver counters
    are then 0).  adams: CVodeCreate(CV_ADAMS) instead of CV_BDF."""
    L = ref_lib()
    ctx = VP()
    assert L.SUNContext_Create(0, ct.byref(ctx)) == 0
    prob = make_serial(L)
    n = len(u0)
    y = L.N_VNew_Serial(n, ctx) if threads is None else L.N_VNew_OpenMP(n, threads, ctx)
    prob.arr(y)[:] = u0
    mem = L.CVodeCreate(1 if adams else 2, ctx)
    f, jt, ps, pv = prob.addresses()
    assert L.CVodeInit(mem, f, 0.0, y) == 0
    vatol = None
    if np.ndim(atol) == 0:
        assert L.CVodeSStolerances(mem, rtol, atol) == 0
    else:
        vatol = L.N_VNew_Serial(n, ctx)
        prob.arr(vatol)[:] = atol
        assert L.CVodeSVtolerances(mem, rtol, vatol) == 0
    assert L.CVodeSetMaxNumSteps(mem, mxstep) == 0
    A, LS, NLS = None, None, None
    if fixed_point is not None:
        NLS = L.SUNNonlinSol_FixedPoint(y, fixed_point, ctx)
        assert L.CVodeSetNonlinearSolver(mem, NLS) == 0
    elif direct:
        A = L.SUNDenseMatrix(n, n, ctx)
        LS = L.SUNLinSol_Dense(y, A, ctx)
        assert L.CVodeSetLinearSolver(mem, LS, A) == 0
        assert L.CVodeSetJacFn(mem, prob.jac_address()) == 0
    else:
        LS = L.SUNLinSol_SPGMR(y, 1, 5, ctx)
        assert L.CVodeSetLinearSolver(mem, LS, None) == 0
        if jt:
            assert L.CVodeSetJacTimes(mem, None, jt) == 0
        assert L.CVodeSetPreconditioner(mem, ps, pv) == 0
    cnt, real, sols = [], [], []
    t = D()
    for tout in touts:
        flag = L.CVode(mem, tout, y, ct.byref(t), 1)
        assert flag == 0, flag
        c, li, ri = ct.c_long(), I(), D()
        row = []
        for name in ("CVodeGetNumSteps", "CVodeGetNumRhsEvals", "CVodeGetNumNonlinSolvIters",
                     "CVodeGetNumNonlinSolvConvFails", "CVodeGetNumStepSolveFails",
                     "CVodeGetNumErrTestFails", "CVodeGetNumLinSolvSetups", "CVodeGetNumLinIters",
                     "CVodeGetNumPrecEvals", "CVodeGetNumPrecSolves", "CVodeGetNumJtimesEvals",
                     "CVodeGetNumLinConvFails"):
            if NLS and name in LS_GETTERS:
                row.append(0)
                continue
            getattr(L, name)(mem, ct.byref(c))
            row.append(c.value)
        for name in ("CVodeGetLastOrder", "CVodeGetCurrentOrder"):
            getattr(L, name)(mem, ct.byref(li))
            row.append(li.value)
        for name in ("CVodeGetNumLinRhsEvals", "CVodeGetNumJacEvals"):
            if NLS:
                row.append(0)
                continue
            getattr(L, name)(mem, ct.byref(c))
            row.append(c.value)
        rrow = []
        for name in ("CVodeGetLastStep", "CVodeGetCurrentStep", "CVodeGetCurrentTime",
                     "CVodeGetActualInitStep"):
            getattr(L, name)(mem, ct.byref(ri))
            rrow.append(ri.value)
        cnt.append(row)
        real.append(rrow)
        sols.append(prob.arr(y).copy())
    pm = VP(mem)
    L.CVodeFree(ct.byref(pm))
    if LS:
        L.SUNLinSolFree(LS)
    if NLS:
        L.SUNNonlinSolFree(NLS)
    if A:
        L.SUNMatDestroy(A)
    L.N_VDestroy(y)
    if vatol:
        L.N_VDestroy(vatol)
    L.SUNContext_Free(ct.byref(ctx))
    return np.array(cnt, np.int64), np.array(real), np.array(sols)


def run_port(y0_handle, LS_handle, callbacks, get, touts, rtol=1e-6, atol=1e-10, mxstep=100000,
             vatol_handle=None, matrix=None, fixed_point=None, adams=False):
    """The restated CVODE on whatever objects it is given: y0_handle (an
    N_Vector holding u0, also used for the outputs), LS_handle (a
    SUNLinearSolver built on it), callbacks = (f, jtimes, psetup, psolve,
    user_data) addresses, get(handle) -> numpy copy of a vector;
    vatol_handle: an N_Vector of absolute tolerances (else atol, a scalar);
    matrix = (SUNMatrix, CVLsJacFn address): the matrix-based path with a
    direct LS_handle (callbacks then only need f and the user data);
    fixed_point = m: the fixed-point solver with Anderson depth m and no
    linear solver (LS_handle None); adams: Adams-Moulton instead of BDF."""
    P = port_lib()
    f, jt, ps, pv, data = callbacks
    mem = P.cvls_port_create(f, 0.0, y0_handle, rtol, 0.0 if vatol_handle else atol, mxstep,
                             LS_handle, jt, ps, pv, data)
    assert mem
    if vatol_handle:
        P.cvls_port_set_vabstol(mem, rtol, vatol_handle)
    if matrix is not None:
        P.cvls_port_set_matrix(mem, matrix[0], matrix[1])
    if fixed_point is not None:
        P.cvls_port_set_fixed_point(mem, fixed_point)
    if adams:
        P.cvls_port_set_adams(mem)
    cnt, real, sols = [], [], []
    t = D()
    c = (ct.c_long * len(COUNTER_NAMES))()
    r = (D * 4)()
    try:
        for tout in touts:
            flag = P.cvls_port_solve(mem, tout, y0_handle, ct.byref(t))
            assert flag == 0, flag
            P.cvls_port_stats(mem, c, r)
            cnt.append(list(c))
            real.append(list(r))
            sols.append(get(y0_handle))
    finally:
        P.cvls_port_free(mem)
    return np.array(cnt, np.int64), np.array(real), np.array(sols)


def run_port_serial(nx: int, ny: int, touts, rtol=1e-6, atol=1e-10):
    """run_port on the reference's own serial vector and SPGMR (the pin)."""
    return run_port_serial_with(lambda L: SerialHeat(L, nx, ny), initial(nx, ny), touts, rtol,
                                atol)


def run_port_serial_with(make_serial, u0, touts, rtol, atol, direct=False, fixed_point=None,
                         adams=False):
    L = ref_lib()
    ctx = VP()
    assert L.SUNContext_Create(0, ct.byref(ctx)) == 0
    prob = make_serial(L)
    n = len(u0)
    y = L.N_VNew_Serial(n, ctx)
    prob.arr(y)[:] = u0
    A, matrix, LS = None, None, None
    if fixed_point is not None:
        cbs = (prob.addresses()[0], None, None, None, None)
    elif direct:
        A = L.SUNDenseMatrix(n, n, ctx)
        LS = L.SUNLinSol_Dense(y, A, ctx)
        matrix = (A, prob.jac_address())
        cbs = (prob.addresses()[0], None, None, None, None)
    else:
        LS = L.SUNLinSol_SPGMR(y, 1, 5, ctx)
        cbs = prob.addresses() + (None,)
    vatol = None
    if np.ndim(atol) != 0:
        vatol = L.N_VNew_Serial(n, ctx)
        prob.arr(vatol)[:] = atol
    try:
        return run_port(y, LS, cbs, lambda h: prob.arr(h).copy(), touts, rtol, atol,
                        vatol_handle=vatol, matrix=matrix, fixed_point=fixed_point,
                        adams=adams)
    finally:
        if LS:
            L.SUNLinSolFree(LS)
        if A:
            L.SUNMatDestroy(A)
        L.N_VDestroy(y)
        if vatol:
            L.N_VDestroy(vatol)
        L.SUNContext_Free(ct.byref(ctx))

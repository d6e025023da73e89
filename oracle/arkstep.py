"""TEST ORACLE (checker only): ARKStep runs with an implicit right-hand side
(DIRK) or an explicit + implicit splitting (ARK IMEX), Newton, SPGMR with
left preconditioning and the default maxl, the difference-quotient J v, a
preconditioner solve without setup -- the ARK-DIRK and ARK-IMEX
configurations of the 3-D advection-reaction benchmark
(benchmarks/advection_reaction_3D/raja/arkode_driver.cpp:51-160, 239-370,
default order 3) -- by two drivers:

* ``run_reference_with``: the reference's own ARKodeEvolve on its
  NVECTOR_SERIAL / SUNLINSOL_SPGMR objects (``oracle/_ref``), which also
  returns the Butcher tables the run used (ARKStepGetCurrentButcherTables);
* ``run_port``: the C restatement ``oracle/arkstep_port.c`` on whatever
  N_Vector and SUNLinearSolver it is given, with those tables as inputs.

Both return the counters after every output time (COUNTER_NAMES), the step
sizes and times (REAL_NAMES) and the solutions there."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import heat_cvode as hc
from . import port

COUNTER_NAMES = ("nst", "nst_attempts", "nfi", "netf", "ncfn", "nni", "nnf", "nli", "nps",
                 "njtimes", "nfeDQ", "ncfl", "nfe", "nnlfi", "nsetups", "nje", "npe")
REAL_NAMES = ("hold", "hnext", "tcur", "h0u")
TABLE_KEYS = ("A", "b", "c", "d", "orders")


def tables_from(g, prefix=""):
    """The tables dict of a fixture: keys <prefix>table_* (implicit, or the
    ERK method's with <prefix>erk set) and <prefix>etable_* (explicit,
    absent for a DIRK run)."""
    Ti = {k: g[prefix + "table_" + k] for k in TABLE_KEYS}
    Te = ({k: g[prefix + "etable_" + k] for k in TABLE_KEYS}
          if prefix + "etable_A" in g else None)
    return {"i": Ti, "e": Te, "erk": bool(g[prefix + "erk"]) if prefix + "erk" in g else False}


def tables_to_dict(tables, prefix=""):
    """Fixture entries of a tables dict (inverse of tables_from)."""
    out = {prefix + "table_" + k: v for k, v in tables["i"].items()}
    if tables.get("erk"):
        out[prefix + "erk"] = np.array(1)
    if tables["e"] is not None:
        out.update({prefix + "etable_" + k: v for k, v in tables["e"].items()})
    return out

VP, D, I, I64 = hc.VP, hc.D, hc.I, hc.I64


class _Table(ct.Structure):
    """struct ARKodeButcherTableMem (include/arkode/arkode_butcher.h:33-42)."""
    _fields_ = [("q", I), ("p", I), ("stages", I), ("A", ct.POINTER(ct.POINTER(D))),
                ("c", ct.POINTER(D)), ("b", ct.POINTER(D)), ("d", ct.POINTER(D))]


def ref_lib() -> ct.CDLL:
    L = hc.ref_lib()
    if getattr(L, "_ark_declared", False):
        return L
    for name, res, args in [
        ("ARKStepCreate", VP, [VP, VP, D, VP, VP]),
        ("ARKodeSetOrder", I, [VP, I]),
        ("ARKodeSStolerances", I, [VP, D, D]),
        ("ARKodeSVtolerances", I, [VP, D, VP]),
        ("ARKodeSetJacFn", I, [VP, VP]),
        ("ARKodeSetJacTimes", I, [VP, VP, VP]),
        ("ARKodeSetMaxNumSteps", I, [VP, ct.c_long]),
        ("SUNNonlinSol_Newton", VP, [VP, VP]),
        ("SUNNonlinSolFree", I, [VP]),
        ("ARKodeSetNonlinearSolver", I, [VP, VP]),
        ("ARKodeSetLinearSolver", I, [VP, VP, VP]),
        ("ARKodeSetPreconditioner", I, [VP, VP, VP]),
        ("ARKodeEvolve", I, [VP, D, VP, ct.POINTER(D), I]),
        ("ARKodeFree", None, [ct.POINTER(VP)]),
        ("ARKStepGetCurrentButcherTables", I, [VP, ct.POINTER(ct.POINTER(_Table)),
                                               ct.POINTER(ct.POINTER(_Table))]),
        ("ARKodeGetNumRhsEvals", I, [VP, I, ct.POINTER(ct.c_long)]),
        ("ARKodeGetNonlinearSystemData", I, [VP, ct.POINTER(D), ct.POINTER(VP), ct.POINTER(VP),
                                             ct.POINTER(VP), ct.POINTER(D), ct.POINTER(VP),
                                             ct.POINTER(VP)]),
        ("SUNNonlinSolNewEmpty", VP, [VP]),
        ("SUNNonlinSol_FixedPoint", VP, [VP, I, VP]),
        ("ERKStepCreate", VP, [VP, D, VP, VP]),
        ("ERKStepGetCurrentButcherTable", I, [VP, ct.POINTER(ct.POINTER(_Table))]),
        ("SUNNonlinSolFreeEmpty", None, [VP]),
        ("SUNNonlinSolSetSysFn", I, [VP, VP]),
        ("SUNNonlinSolSetLSolveFn", I, [VP, VP]),
        ("SUNNonlinSolSetConvTestFn", I, [VP, VP, VP]),
        ("SUNNonlinSolInitialize", I, [VP]),
        ("SUNNonlinSolSolve", I, [VP, VP, VP, VP, D, I, VP]),
        ("N_VLinearSum", None, [D, VP, D, VP, VP]),
        ("N_VLinearCombination", I, [I, ct.POINTER(D), ct.POINTER(VP), VP]),
    ]:
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    for name in ("ARKodeGetNumSteps", "ARKodeGetNumStepAttempts", "ARKodeGetNumErrTestFails",
                 "ARKodeGetNumStepSolveFails", "ARKodeGetNumNonlinSolvIters",
                 "ARKodeGetNumNonlinSolvConvFails", "ARKodeGetNumLinIters",
                 "ARKodeGetNumPrecSolves", "ARKodeGetNumJtimesEvals", "ARKodeGetNumLinRhsEvals",
                 "ARKodeGetNumLinConvFails", "ARKodeGetNumLinSolvSetups", "ARKodeGetNumJacEvals",
                 "ARKodeGetNumPrecEvals"):
        f = getattr(L, name)
        f.restype, f.argtypes = I, [VP, ct.POINTER(ct.c_long)]
    for name in ("ARKodeGetLastStep", "ARKodeGetCurrentStep", "ARKodeGetCurrentTime",
                 "ARKodeGetActualInitStep"):
        f = getattr(L, name)
        f.restype, f.argtypes = I, [VP, ct.POINTER(D)]
    L._ark_declared = True
    return L


def port_lib() -> ct.CDLL:
    L = port.lib()
    if not getattr(L, "_arkstep_declared", False):
        DP = ct.POINTER(D)
        L.arkstep_port_create.restype = VP
        L.arkstep_port_create.argtypes = [VP, VP, D, VP, D, D, ct.c_long, VP, VP, VP, VP, I, I,
                                          I, DP, DP, DP, DP, DP, DP, DP, DP]
        L.arkstep_port_solve.restype = I
        L.arkstep_port_solve.argtypes = [VP, D, VP, ct.POINTER(D)]
        L.arkstep_port_stats.restype = None
        L.arkstep_port_stats.argtypes = [VP, ct.POINTER(ct.c_long), ct.POINTER(D)]
        L.arkstep_port_free.restype = None
        L.arkstep_port_free.argtypes = [VP]
        L.arkstep_port_set_task_local.restype = None
        L.arkstep_port_set_task_local.argtypes = [VP, VP]
        L.arkstep_port_set_fixed_point.restype = None
        L.arkstep_port_set_fixed_point.argtypes = [VP, I]
        L.arkstep_port_set_erk.restype = None
        L.arkstep_port_set_erk.argtypes = [VP]
        L.arkstep_port_set_matrix.restype = None
        L.arkstep_port_set_matrix.argtypes = [VP, VP, VP]
        L.arkstep_port_set_vabstol.restype = None
        L.arkstep_port_set_vabstol.argtypes = [VP, D, VP]
        L.arkstep_port_set_psetup.restype = None
        L.arkstep_port_set_psetup.argtypes = [VP, VP]
        L._arkstep_declared = True
    return L


class _NLSOps(ct.Structure):
    """struct _generic_SUNNonlinearSolver_Ops (sundials_nonlinearsolver.h)."""
    _fields_ = [(n, VP) for n in ("gettype", "initialize", "setup", "solve", "free", "setsysfn",
                                  "setlsetupfn", "setlsolvefn", "setctestfn", "setoptions",
                                  "setmaxiters", "getnumiters", "getcuriter",
                                  "getnumconvfails")]


class _NLS(ct.Structure):
    _fields_ = [("content", VP), ("ops", ct.POINTER(_NLSOps)), ("sunctx", VP)]


_GETTYPE = ct.CFUNCTYPE(I, VP)
_INIT = ct.CFUNCTYPE(I, VP)
_SOLVE = ct.CFUNCTYPE(I, VP, VP, VP, VP, D, I, VP)
_SETSYS = ct.CFUNCTYPE(I, VP, VP)
_SETCTEST = ct.CFUNCTYPE(I, VP, VP, VP)
_GETNCF = ct.CFUNCTYPE(I, VP, ct.POINTER(ct.c_long))
_SYSFN = ct.CFUNCTYPE(I, VP, VP, VP)
_LSOLVEFN = ct.CFUNCTYPE(I, VP, VP)


class TaskLocalNewton:
    """The 3-D advection-reaction benchmark's TaskLocalNewton
    (arkode_driver.cpp:546-780) on one task, restated around the reference's
    own SUNNonlinSol_Newton: a SUNNonlinearSolver of type ROOTFIND whose
    initialize installs TaskLocalNlsResidual / TaskLocalLSolve on the inner
    Newton, whose solve returns the inner status (the MPI reductions over one
    task are the identity) and counts CONV_RECVR returns, and which forwards
    the system and convergence-test functions to the inner Newton.
    reaction(t, z, Fi) and block_solve(z, x, b, gamma) act on N_Vector
    handles (the benchmark's Reaction and SolveReactionLinSys)."""

    def __init__(self, L, ctx, y, reaction, block_solve):
        self.L, self.ncnf, self.nnlfi = L, 0, 0
        self.inner = L.SUNNonlinSol_Newton(y, ctx)
        self.nls = L.SUNNonlinSolNewEmpty(ctx)
        assert self.inner and self.nls

        def sysfn(ycor, F, mem):
            t, zpred, z, Fi, gamma, sdata, ud = D(), VP(), VP(), VP(), D(), VP(), VP()
            L.ARKodeGetNonlinearSystemData(mem, ct.byref(t), ct.byref(zpred), ct.byref(z),
                                           ct.byref(Fi), ct.byref(gamma), ct.byref(sdata),
                                           ct.byref(ud))
            L.N_VLinearSum(1.0, zpred, 1.0, ycor, z)
            r = reaction(t.value, z, Fi)
            self.nnlfi += 1
            if r != 0:
                return -1 if r < 0 else 1
            c = (D * 3)(1.0, -1.0, -gamma.value)
            X = (VP * 3)(ycor, sdata, Fi)
            return 0 if L.N_VLinearCombination(3, c, X, F) == 0 else -1

        def lsolve(delta, mem):
            t, zpred, z, Fi, gamma, sdata, ud = D(), VP(), VP(), VP(), D(), VP(), VP()
            L.ARKodeGetNonlinearSystemData(mem, ct.byref(t), ct.byref(zpred), ct.byref(z),
                                           ct.byref(Fi), ct.byref(gamma), ct.byref(sdata),
                                           ct.byref(ud))
            return block_solve(z, delta, delta, gamma.value)

        def initialize(nls):
            L.SUNNonlinSolSetSysFn(self.inner, self._cb["sys"])
            L.SUNNonlinSolSetLSolveFn(self.inner, self._cb["lsolve"])
            return L.SUNNonlinSolInitialize(self.inner)

        def solve(nls, y0, ycor, w, tol, call_lsetup, mem):
            status = L.SUNNonlinSolSolve(self.inner, y0, ycor, w, tol, call_lsetup, mem)
            if status < 0:
                return status
            if status == 902:  # SUN_NLS_CONV_RECVR
                self.ncnf += 1
            return status

        def getncf(nls, out):
            out[0] = self.ncnf
            return 0

        self._cb = {"sys": _SYSFN(sysfn), "lsolve": _LSOLVEFN(lsolve),
                    "gettype": _GETTYPE(lambda nls: 0), "init": _INIT(initialize),
                    "solve": _SOLVE(solve),
                    "setsys": _SETSYS(lambda nls, fn: L.SUNNonlinSolSetSysFn(self.inner, fn)),
                    "setctest": _SETCTEST(
                        lambda nls, fn, data: L.SUNNonlinSolSetConvTestFn(self.inner, fn, data)),
                    "getncf": _GETNCF(getncf)}
        ops = ct.cast(self.nls, ct.POINTER(_NLS)).contents.ops.contents
        for field, key in (("gettype", "gettype"), ("initialize", "init"), ("solve", "solve"),
                           ("setsysfn", "setsys"), ("setctestfn", "setctest"),
                           ("getnumconvfails", "getncf")):
            setattr(ops, field, ct.cast(self._cb[key], VP).value)

    def free(self):
        self.L.SUNNonlinSolFreeEmpty(self.nls)
        self.L.SUNNonlinSolFree(self.inner)


def _read_table(T: _Table) -> dict:
    s = T.stages
    A = np.array([[T.A[i][j] for j in range(s)] for i in range(s)])
    return {"A": A, "b": np.array([T.b[i] for i in range(s)]),
            "c": np.array([T.c[i] for i in range(s)]),
            "d": np.array([T.d[i] for i in range(s)]), "orders": np.array([T.q, T.p])}


def run_reference_with(make_serial, u0, touts, rtol, atol, order=3, mxstep=100000, threads=None,
                       imex=False, task_local=False, fixed_point=None, erk=False, direct=False):
    """The reference's ARKodeEvolve on the problem whose serial callbacks
    make_serial(L) builds (.addresses() -> (f, jtimes, psetup, psolve), with
    psetup None, .imex_addresses() -> (fe, fi), and .arr(N_Vector)):
    (counters, reals, solutions, tables) with tables = {"i": implicit table,
    "e": explicit table or None}.  imex: ARKStepCreate(fe, fi) instead of
    ARKStepCreate(NULL, f).  task_local (with imex): the benchmark's
    TaskLocalNewton (``--nls tl-newton``) instead of Newton + SPGMR, with the
    problem's .reaction_into / .block_solve; the counters then end with its
    nonlinear-residual evaluations.  fixed_point = m: SUNNonlinSol_FixedPoint
    with Anderson depth m and no linear solver (``--nls fixedpoint``).
    direct: SUNDenseMatrix + SUNLINSOL_DENSE and the problem's
    .jac_address() (ARKodeSetJacFn) instead of SPGMR: the matrix-based path
    of ARKLS.  atol: a scalar (ARKodeSStolerances) or an array
    (ARKodeSVtolerances).  erk: the benchmark's ERK configuration (ERKStepCreate(f), no nonlinear
    or linear solver; the method's table is returned as tables["i"] with
    tables["erk"] set).  threads = k: NVECTOR_OPENMP on k threads
    instead of NVECTOR_SERIAL (its reductions sum in another order)."""
    L = ref_lib()
    ctx = VP()
    assert L.SUNContext_Create(0, ct.byref(ctx)) == 0
    prob = make_serial(L)
    n = len(u0)
    y = L.N_VNew_Serial(n, ctx) if threads is None else L.N_VNew_OpenMP(n, threads, ctx)
    prob.arr(y)[:] = u0
    f, jt, ps, pv = prob.addresses()
    fe, fi = prob.imex_addresses() if imex else (None, f)
    mem = L.ERKStepCreate(f, 0.0, y, ctx) if erk else L.ARKStepCreate(fe, fi, 0.0, y, ctx)
    assert mem
    assert L.ARKodeSetOrder(mem, order) == 0
    vatol = None
    if np.ndim(atol) == 0:
        assert L.ARKodeSStolerances(mem, rtol, atol) == 0
    else:
        vatol = L.N_VNew_Serial(n, ctx)
        prob.arr(vatol)[:] = atol
        assert L.ARKodeSVtolerances(mem, rtol, vatol) == 0
    assert L.ARKodeSetMaxNumSteps(mem, mxstep) == 0
    TL, LS, NLS, A = None, None, None, None
    no_ls = task_local or fixed_point is not None or erk
    if erk:
        pass
    elif direct:
        NLS = L.SUNNonlinSol_Newton(y, ctx)
        assert L.ARKodeSetNonlinearSolver(mem, NLS) == 0
        A = L.SUNDenseMatrix(n, n, ctx)
        LS = L.SUNLinSol_Dense(y, A, ctx)
        assert L.ARKodeSetLinearSolver(mem, LS, A) == 0
        assert L.ARKodeSetJacFn(mem, prob.jac_address()) == 0
    elif fixed_point is not None:
        NLS = L.SUNNonlinSol_FixedPoint(y, fixed_point, ctx)
        assert L.ARKodeSetNonlinearSolver(mem, NLS) == 0
    elif task_local:
        assert imex
        TL = TaskLocalNewton(L, ctx, y, prob.reaction_into, prob.block_solve)
        NLS = TL.nls
        assert L.ARKodeSetNonlinearSolver(mem, NLS) == 0
    else:
        NLS = L.SUNNonlinSol_Newton(y, ctx)
        assert L.ARKodeSetNonlinearSolver(mem, NLS) == 0
        LS = L.SUNLinSol_SPGMR(y, 1, 0, ctx)
        assert L.ARKodeSetLinearSolver(mem, LS, None) == 0
        if jt:
            assert L.ARKodeSetJacTimes(mem, None, jt) == 0
        assert L.ARKodeSetPreconditioner(mem, ps, pv) == 0
    cnt, real, sols = [], [], []
    t, c, r = D(), ct.c_long(), D()
    table = None
    for tout in touts:
        flag = L.ARKodeEvolve(mem, tout, y, ct.byref(t), 1)
        assert flag == 0, flag
        if table is None and erk:
            B = ct.POINTER(_Table)()
            assert L.ERKStepGetCurrentButcherTable(mem, ct.byref(B)) == 0
            table = {"i": _read_table(B.contents), "e": None, "erk": True}
        if table is None:
            Bi, Be = ct.POINTER(_Table)(), ct.POINTER(_Table)()
            assert L.ARKStepGetCurrentButcherTables(mem, ct.byref(Bi), ct.byref(Be)) == 0
            assert Bi and (bool(Be) == imex)
            table = {"i": _read_table(Bi.contents),
                     "e": _read_table(Be.contents) if imex else None}
        row = []
        for name in ("ARKodeGetNumSteps", "ARKodeGetNumStepAttempts"):
            getattr(L, name)(mem, ct.byref(c))
            row.append(c.value)
        if erk:
            row.append(0)
        else:
            L.ARKodeGetNumRhsEvals(mem, 1, ct.byref(c))
            row.append(c.value)
        for name in ("ARKodeGetNumErrTestFails", "ARKodeGetNumStepSolveFails",
                     "ARKodeGetNumNonlinSolvIters", "ARKodeGetNumNonlinSolvConvFails",
                     "ARKodeGetNumLinIters", "ARKodeGetNumPrecSolves", "ARKodeGetNumJtimesEvals",
                     "ARKodeGetNumLinRhsEvals", "ARKodeGetNumLinConvFails"):
            if (no_ls and any(k in name for k in ("Lin", "Prec", "Jtimes", "Jac"))
                    or erk and "Nonlin" in name):
                row.append(0)  # no linear solver attached
                continue
            getattr(L, name)(mem, ct.byref(c))
            row.append(c.value)
        L.ARKodeGetNumRhsEvals(mem, 0, ct.byref(c))
        row.append(c.value)
        row.append(TL.nnlfi if TL else 0)
        for name in ("ARKodeGetNumLinSolvSetups", "ARKodeGetNumJacEvals", "ARKodeGetNumPrecEvals"):
            if LS:
                getattr(L, name)(mem, ct.byref(c))
                row.append(c.value)
            else:
                row.append(0)
        rrow = []
        for name in ("ARKodeGetLastStep", "ARKodeGetCurrentStep", "ARKodeGetCurrentTime",
                     "ARKodeGetActualInitStep"):
            getattr(L, name)(mem, ct.byref(r))
            rrow.append(r.value)
        cnt.append(row)
        real.append(rrow)
        sols.append(prob.arr(y).copy())
    pm = VP(mem)
    L.ARKodeFree(ct.byref(pm))
    if TL:
        TL.free()
    elif NLS:
        L.SUNNonlinSolFree(NLS)
    if LS:
        L.SUNLinSolFree(LS)
    if A:
        L.SUNMatDestroy(A)
    if vatol:
        L.N_VDestroy(vatol)
    L.N_VDestroy(y)
    L.SUNContext_Free(ct.byref(ctx))
    return np.array(cnt, np.int64), np.array(real), np.array(sols), table


def run_port(y0_handle, LS_handle, callbacks, get, touts, tables, rtol, atol, mxstep=100000,
             block_solve=None, fixed_point=None, matrix=None, vatol_handle=None, psetup=None):
    """The restated ARKStep on the objects it is given: y0_handle (an
    N_Vector holding u0, also used for the outputs), LS_handle (a
    SUNLinearSolver built on it), callbacks = (fe, fi, jtimes, psolve,
    user_data) addresses (fe None: implicit only; jtimes None: difference
    quotients), get(handle) -> numpy copy, tables = the Butcher tables of
    run_reference_with ({"i": ..., "e": ... or None}); block_solve: the
    address of a block solve (z, x, b, gamma, user_data) -> the task-local
    Newton, with LS_handle and the preconditioner None; fixed_point = m: the
    fixed-point solver with Anderson depth m, also without a linear solver;
    matrix = (SUNMatrix, ARKLsJacFn address): the matrix-based path with a
    direct LS_handle; vatol_handle: an N_Vector of absolute tolerances;
    psetup: a preconditioner setup (ARKLsPrecSetupFn address) beside psolve."""
    P = port_lib()
    fe, fi, jt, pv, data = callbacks
    DP = ct.POINTER(D)
    Ti, Te = tables["i"], tables["e"]
    if tables.get("erk"):  # ERKStep: the single right-hand side goes in fi's place
        fe, fi = None, fe or fi
    assert (fe is None) == (Te is None)
    keep = []

    def arrs(T):
        if T is None:
            return [None] * 4
        a = [np.ascontiguousarray(T[k], np.float64) for k in ("A", "b", "c", "d")]
        keep.extend(a)
        return [x.ctypes.data_as(DP) for x in a]

    q, p = (int(v) for v in Ti["orders"])
    mem = P.arkstep_port_create(fe, fi, 0.0, y0_handle, rtol, 0.0 if vatol_handle else atol,
                                mxstep, LS_handle, jt, pv,
                                data, len(Ti["b"]), q, p, *arrs(Ti), *arrs(Te))
    assert mem
    if block_solve is not None:
        P.arkstep_port_set_task_local(mem, block_solve)
    if fixed_point is not None:
        P.arkstep_port_set_fixed_point(mem, fixed_point)
    if tables.get("erk"):
        P.arkstep_port_set_erk(mem)
    if matrix is not None:
        P.arkstep_port_set_matrix(mem, matrix[0], matrix[1])
    if vatol_handle:
        P.arkstep_port_set_vabstol(mem, rtol, vatol_handle)
    if psetup:
        P.arkstep_port_set_psetup(mem, psetup)
    cnt, real, sols = [], [], []
    t = D()
    cbuf = (ct.c_long * len(COUNTER_NAMES))()
    rbuf = (D * len(REAL_NAMES))()
    try:
        for tout in touts:
            flag = P.arkstep_port_solve(mem, tout, y0_handle, ct.byref(t))
            assert flag == 0, flag
            P.arkstep_port_stats(mem, cbuf, rbuf)
            cnt.append(list(cbuf))
            real.append(list(rbuf))
            sols.append(get(y0_handle))
    finally:
        P.arkstep_port_free(mem)
    return np.array(cnt, np.int64), np.array(real), np.array(sols)


def run_port_serial_with(make_serial, u0, touts, tables, rtol, atol, task_local=False,
                         fixed_point=None, direct=False):
    """run_port on the reference's own serial vector and SPGMR (the pin)."""
    L = ref_lib()
    ctx = VP()
    assert L.SUNContext_Create(0, ct.byref(ctx)) == 0
    prob = make_serial(L)
    y = L.N_VNew_Serial(len(u0), ctx)
    prob.arr(y)[:] = u0
    no_ls = task_local or fixed_point is not None or tables.get("erk")
    A, matrix, vatol = None, None, None
    if direct:
        A = L.SUNDenseMatrix(len(u0), len(u0), ctx)
        LS = L.SUNLinSol_Dense(y, A, ctx)
        matrix = (A, prob.jac_address())
    else:
        LS = None if no_ls else L.SUNLinSol_SPGMR(y, 1, 0, ctx)
    if np.ndim(atol) != 0:
        vatol = L.N_VNew_Serial(len(u0), ctx)
        prob.arr(vatol)[:] = atol
    f, jt, ps, pv = prob.addresses()
    fe, fi = prob.imex_addresses() if tables["e"] is not None else (None, f)
    try:
        return run_port(y, LS, (fe, fi, None if direct else jt,
                                None if (no_ls or direct) else pv, None),
                        lambda h: prob.arr(h).copy(), touts, tables, rtol, atol,
                        block_solve=prob.block_solve_address() if task_local else None,
                        fixed_point=fixed_point, matrix=matrix, vatol_handle=vatol,
                        psetup=None if (no_ls or direct) else ps)
    finally:
        if LS:
            L.SUNLinSolFree(LS)
        if A:
            L.SUNMatDestroy(A)
        if vatol:
            L.N_VDestroy(vatol)
        L.N_VDestroy(y)
        L.SUNContext_Free(ct.byref(ctx))

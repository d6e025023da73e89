"""GPU: the 3-D advection-reaction benchmark's ARKODE configurations --
ARK-DIRK (its default, arkode_driver.cpp:51-160: implicit advection +
reaction) and ARK-IMEX (239-370: explicit advection, implicit reaction), order
3 -- with the GB300 modules plugged in: NVECTOR_GB300 for every vector,
SUNLinSol_SPGMR_GB300 (left preconditioning, maxl 5) as the linear solver,
and the device user functions of include/bruss3d_gb300.h as the right-hand
sides and the preconditioner solve; and ARK-IMEX with the benchmark's
task-local Newton (546-780, one task), whose linear solve is the device
per-cell reaction solve (SUNBruss3D_GB300_SolveReaction) with no
SUNLinearSolver at all.  Driven by the ARKStep restatement
oracle/arkstep_port.c (the reference's ARKodeEvolve bit for bit on serial
objects: tests/test_arkstep_port.py) with the reference's Butcher tables
from the fixture, and compared with the reference's own runs
(tests/golden/bruss3d_arkode_ref.npz).  The reference's own runs on
NVECTOR_OPENMP at 2-16 threads never moved a counter, so every counter after
every output must equal the reference's; the last solution within 3x the
reference's own weighted RMS deviation (in units of the tolerance)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import arkstep as ak

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "bruss3d_arkode_ref.npz"


@pytest.mark.parametrize("name,fused", [("dirk_", False), ("dirk_", True), ("imex_", False),
                                        ("imex_", True), ("tl_", None)],
                         ids=["dirk-unfused_gs", "dirk-fused_gs", "imex-unfused_gs",
                              "imex-fused_gs", "imex-tl_newton"])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_arkstep_bruss3d_matches_reference(name, fused, fma):
    from sundials_gb300.bruss3d import Bruss3D
    from sundials_gb300.nvector import NVector
    from sundials_gb300.spgmr import PREC_LEFT, SPGMR
    g = np.load(GOLDEN)
    rtol, atol = (float(v) for v in g["tol"])
    tables = ak.tables_from(g, name)
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    tl = name == "tl_"
    S = None if tl else SPGMR(y, pretype=PREC_LEFT, maxl=5)
    if S:
        assert S.set_fused(fused) == 0
    P = Bruss3D(*(int(v) for v in g["grid"]))
    try:
        fe, fi, jt, psolve, data = P.arkode_callbacks(imex=tables["e"] is not None)
        c, r, s = ak.run_port(y.v, S.S if S else None, (fe, fi, jt, None if tl else psolve, data),
                              lambda h: y.get(), [float(t) for t in g["touts"]], tables, rtol,
                              atol, block_solve=P.block_solve_address() if tl else None)
    finally:
        if S:
            S.free()
        P.free()
    ref = g[name + "counters"]
    assert np.array_equal(c, ref), dict(zip(ak.COUNTER_NAMES, (c[-1] - ref[-1]).tolist()))
    yr = g[name + "y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + atol)) ** 2)))
    assert w <= max(3.0 * float(g[name + "omp_wrms"].max()), 1e-6), w


@pytest.mark.parametrize("name", ["fpdirk_", "fpimex_"])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_arkstep_bruss3d_fixed_point_matches_reference(name, fma):
    """ARK-DIRK / ARK-IMEX with ``--nls fixedpoint`` (Anderson depth 3, no
    linear solver) over t in [0, 0.01] on the 16^3 grid: hundreds of steps
    and of nonlinear failures, which the reference's own summation order
    already moves (its NVECTOR_OPENMP runs).  Six such runs are a small
    sample of a spread that a chaotic iteration makes wide, so each counter
    must lie within twice the reference's own largest deviation + 1 (equal
    where it never moved) and the last solution within 3x its own weighted
    RMS deviation."""
    from sundials_gb300.bruss3d import Bruss3D
    from sundials_gb300.nvector import NVector
    g = np.load(GOLDEN)
    rtol, atol = (float(v) for v in g["tol"])
    tables = ak.tables_from(g, name)
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    P = Bruss3D(*(int(v) for v in g["grid"]))
    try:
        fe, fi, _, _, data = P.arkode_callbacks(imex=tables["e"] is not None)
        c, r, s = ak.run_port(y.v, None, (fe, fi, None, None, data), lambda h: y.get(),
                              [float(t) for t in g[name + "touts"]], tables, rtol, atol,
                              fixed_point=3)
    finally:
        P.free()
    ref = g[name + "counters"][-1]
    own = np.abs(g[name + "omp_counters"] - ref).max(axis=0)
    band = np.where(own == 0, 0, 2 * own + 1)
    dev = np.abs(c[-1] - ref)
    assert np.all(dev <= band), {n: (int(d), int(b)) for n, d, b in zip(ak.COUNTER_NAMES, dev, band)
                                 if d > b}
    yr = g[name + "y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + atol)) ** 2)))
    assert w <= max(3.0 * float(g[name + "omp_wrms"].max()), 1e-6), w


@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_erkstep_bruss3d_matches_reference(fma):
    """The benchmark's ERK configuration (ERKStep, order 3, explicit on the
    stiff reaction: ~800 steps over t in [0, 0.01]) on NVECTOR_GB300 with the
    device right-hand side.  The reference's own reduction-order runs never
    moved a counter, so every counter after every output must equal the
    reference's; the last solution within 3x its own weighted RMS deviation
    or 1e-3 tolerances (its own deviation, ~1e-5 tolerances, is below what
    one rounding per product in the FMA mode moves over the run)."""
    from sundials_gb300.bruss3d import Bruss3D
    from sundials_gb300.nvector import NVector
    g = np.load(GOLDEN)
    rtol, atol = (float(v) for v in g["tol"])
    tables = ak.tables_from(g, "erk_")
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    P = Bruss3D(*(int(v) for v in g["grid"]))
    try:
        _, f, _, _, data = P.arkode_callbacks()
        c, r, s = ak.run_port(y.v, None, (None, f, None, None, data), lambda h: y.get(),
                              [float(t) for t in g["erk_touts"]], tables, rtol, atol)
    finally:
        P.free()
    ref = g["erk_counters"]
    assert np.array_equal(c, ref), dict(zip(ak.COUNTER_NAMES, (c[-1] - ref[-1]).tolist()))
    yr = g["erk_y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + atol)) ** 2)))
    assert w <= max(3.0 * float(g["erk_omp_wrms"].max()), 1e-3), w


ROB_GOLDEN = Path(__file__).resolve().parent / "golden" / "robertson_arkode_ref.npz"


@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_arkstep_robertson_direct_block_lu_matches_reference(fma):
    """The batched Robertson cells (64) through ARKStep with
    SUNMatrix_BlockDiag_GB300 + SUNLinSol_BlockLU_GB300 (FP64) attached as
    ARKODE's direct linear solver (ARKodeSetLinearSolver(LS, A)) and the
    device Jacobian (ARKodeSetJacFn), per-species absolute tolerances, to
    t = 4e5: against the reference's ARKodeEvolve with SUNDenseMatrix +
    SUNLINSOL_DENSE.  Its own reduction-order runs never moved a counter, so
    every counter after every output must equal the reference's; the last
    solution within 3x its own weighted RMS deviation and 10 tolerances."""
    from sundials_gb300 import blockdiag as BD
    from sundials_gb300.nvector import NVector
    from sundials_gb300.robertson import LU_FP64, Robertson
    g = np.load(ROB_GOLDEN)
    ncells = int(g["cells"])
    rtol = float(g["rtol"])
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    vatol = NVector.from_numpy(g["atol"])
    prob = Robertson(g["k"], y, LU_FP64)
    M = BD.BlockDiag([3] * ncells)
    S = BD.BlockLU(y.v, M, LU_FP64)
    try:
        f = prob.cvode_callbacks()[0]
        c, r, s = ak.run_port(y.v, S.S, (None, f, None, None, prob.p), lambda h: y.get(),
                              [float(t) for t in g["touts"]], ak.tables_from(g), rtol, 0.0,
                              matrix=(M.A, prob.jac_address()), vatol_handle=vatol.v)
    finally:
        S.free()
        prob.free()
    ref = g["counters"]
    assert np.array_equal(c, ref), dict(zip(ak.COUNTER_NAMES, (c[-1] - ref[-1]).tolist()))
    yr = g["y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + g["atol"])) ** 2)))
    assert w <= max(3.0 * float(g["omp_wrms"].max()), 1e-6) and w <= 10.0, w


@pytest.mark.parametrize("fused", [False, True], ids=["unfused_gs", "fused_gs"])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_arkstep_robertson_preconditioned_matches_reference(fma, fused):
    """The same cells through ARKStep with SPGMR_GB300 (left, maxl 5), the
    device J v and the exact block-Jacobi preconditioner with its setup
    (ARKodeSetPreconditioner(psetup, psolve), the block LU inside): every
    counter after every output equal to the reference's (its own
    reduction-order runs never moved one), the last solution within 3x its
    own weighted RMS deviation and 10 tolerances."""
    from sundials_gb300.nvector import NVector
    from sundials_gb300.robertson import LU_FP64, Robertson
    from sundials_gb300.spgmr import PREC_LEFT, SPGMR
    g = np.load(ROB_GOLDEN)
    rtol = float(g["rtol"])
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    vatol = NVector.from_numpy(g["atol"])
    prob = Robertson(g["k"], y, LU_FP64)
    S = SPGMR(y, pretype=PREC_LEFT, maxl=5)
    assert S.set_fused(fused) == 0
    try:
        f, jt, ps, pv, data = prob.cvode_callbacks()
        c, r, s = ak.run_port(y.v, S.S, (None, f, jt, pv, data), lambda h: y.get(),
                              [float(t) for t in g["touts"]], ak.tables_from(g, "prec_"), rtol,
                              0.0, vatol_handle=vatol.v, psetup=ps)
    finally:
        S.free()
        prob.free()
    ref = g["prec_counters"]
    assert np.array_equal(c, ref), dict(zip(ak.COUNTER_NAMES, (c[-1] - ref[-1]).tolist()))
    yr = g["prec_y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + g["atol"])) ** 2)))
    assert w <= max(3.0 * float(g["prec_omp_wrms"].max()), 1e-6) and w <= 10.0, w

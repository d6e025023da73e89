"""GPU: whole CVODE integrations with the GB300 modules plugged in --
NVECTOR_GB300 for every vector, SUNLinSol_SPGMR_GB300 (left preconditioning,
maxl 5, modified Gram-Schmidt) as the linear solver, and device callbacks as
f / J v / psetup / psolve: the 2-D heat problem with its Jacobi
preconditioner (include/heat2d_gb300.h), and the batched Robertson problem
with the exact block-Jacobi preconditioner on SUNLinSol_BlockLU_GB300
(include/robertson_gb300.h) -- driven by the CVODE restatement
oracle/cvode_ls_port.c (the reference's CVode, bit for bit on serial objects:
tests/test_cvode_ls_port.py, tests/test_robertson_cvode.py) and compared with
the reference's own runs on NVECTOR_SERIAL + SUNLINSOL_SPGMR
(tests/golden/heat_cvode_ref.npz, robertson_cvode_ref.npz).

What differs from the serial objects is the summation order of the dot
products and norms (a fixed tree instead of a sequential loop), the fused
Gram-Schmidt kernels (deferred normalisation) and, with FMA on, one rounding
per contracted product.  The reference itself moves when only its summation
order changes: the fixture holds its own runs on NVECTOR_OPENMP at 2-16
threads.  The bar, per counter after the last output: equal to the serial
reference's where the reference's own runs never moved it (steps, error-test
and nonlinear failures, setups, orders, and every counter of the cases whose
linear solves converge well inside maxl), otherwise within the largest
deviation the reference showed plus one; the solutions at every output within
3x the reference's own largest weighted RMS deviation and within 10x the
error tolerance (weighted RMS in units of the tolerance, CVODE's weights at
the serial solution)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import heat_cvode as hc

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "heat_cvode_ref.npz"


def _run(name, fma, fused):
    from sundials_gb300.heat2d import Heat2D
    from sundials_gb300.nvector import NVector
    from sundials_gb300.spgmr import PREC_LEFT, SPGMR
    g = np.load(GOLDEN)
    nx, ny = (int(v) for v in g[f"{name}_grid"])
    rtol, atol = (float(v) for v in g[f"{name}_tol"])
    touts = [float(t) for t in g[f"{name}_touts"]]
    y = NVector.from_numpy(g[f"{name}_u0"])
    y.set_fma(fma)
    S = SPGMR(y, pretype=PREC_LEFT, maxl=5)
    assert S.set_fused(fused) == 0
    heat = Heat2D(nx, ny)
    try:
        c, r, s = hc.run_port(y.v, S.S, heat.cvode_callbacks(), lambda h: y.get(), touts, rtol,
                              atol)
    finally:
        S.free()
        heat.free()
    return g, c, r, s, rtol, atol


def _wrms(d, yref, rtol, atol):
    w = 1.0 / (rtol * np.abs(yref) + atol)
    return float(np.sqrt(np.mean((d * w) ** 2)))


@pytest.mark.parametrize("name", ["g32", "g48x32_tight", "g128"])
@pytest.mark.parametrize("fused", [False, True], ids=["unfused_gs", "fused_gs"])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_cvode_heat_matches_reference(name, fused, fma):
    g, c, r, s, rtol, atol = _run(name, fma, fused)
    c_ref, y_ref = g[f"{name}_counters"], g[f"{name}_y"]
    own = np.abs(g[f"{name}_omp_counters"] - c_ref[-1]).max(axis=0)
    band = np.where(own == 0, 0, own + 1)
    dev = np.abs(c[-1] - c_ref[-1])
    assert np.all(dev <= band), {n: (int(d), int(b)) for n, d, b in zip(hc.COUNTER_NAMES, dev, band)
                                 if d > b}
    if not own.any():  # the reference never moved: every output's counters are equal
        assert np.array_equal(c, c_ref)
    own_wrms = float(g[f"{name}_omp_wrms"].max())
    for k in range(len(y_ref)):
        w = _wrms(s[k] - y_ref[k], y_ref[k], rtol, atol)
        assert w <= 3.0 * own_wrms and w <= 10.0, (k, w, own_wrms)


ROB_GOLDEN = Path(__file__).resolve().parent / "golden" / "robertson_cvode_ref.npz"


def _run_robertson(name, fma, fused, lu, direct=False):
    from sundials_gb300 import blockdiag as BD
    from sundials_gb300.nvector import NVector
    from sundials_gb300.robertson import Robertson
    from sundials_gb300.spgmr import PREC_LEFT, SPGMR
    from oracle import robertson_cvode as rc
    g = np.load(ROB_GOLDEN)
    k = g[f"{name}_k"]
    ncells = len(k)
    y = NVector.from_numpy(rc.initial(ncells))
    y.set_fma(fma)
    vatol = NVector.from_numpy(rc.vector_atol(ncells))
    prob = Robertson(k, y, lu)
    touts = [float(t) for t in g[f"{name}_touts"]]
    rtol = float(g[f"{name}_rtol"])
    try:
        if direct:  # the reference example's configuration: direct block solve, user J
            M = BD.BlockDiag([3] * ncells)
            S = BD.BlockLU(y.v, M, lu)
            f = prob.cvode_callbacks()[0]
            c, r, s = hc.run_port(y.v, S.S, (f, None, None, None, prob.p), lambda h: y.get(),
                                  touts, rtol, 0.0, vatol_handle=vatol.v,
                                  matrix=(M.A, prob.jac_address()))
            S.free()
        else:
            S = SPGMR(y, pretype=PREC_LEFT, maxl=5)
            assert S.set_fused(fused) == 0
            c, r, s = hc.run_port(y.v, S.S, prob.cvode_callbacks(), lambda h: y.get(), touts,
                                  rtol, 0.0, vatol_handle=vatol.v)
            S.free()
    finally:
        prob.free()
    return g, c, r, s


def _check_against_reference(g, name, c, s, atol_vec, rtol):
    """Counters: equal at every output where the reference's own
    reduction-order runs never moved them, else within its largest deviation
    + 1 after the last output; solutions within 3x its own weighted RMS
    deviation (and 10x the tolerance)."""
    c_ref = g[f"{name}_counters"]
    own = np.abs(g[f"{name}_omp_counters"] - c_ref[-1]).max(axis=0)
    if not own.any():
        assert np.array_equal(c, c_ref), (c[-1] - c_ref[-1]).tolist()
    band = np.where(own == 0, 0, own + 1)
    dev = np.abs(c[-1] - c_ref[-1])
    assert np.all(dev <= band), {n: (int(d), int(b)) for n, d, b in zip(hc.COUNTER_NAMES, dev, band)
                                 if d > b}
    own_w = float(g[f"{name}_omp_wrms"].max())
    for j, k in enumerate(g[f"{name}_y_index"]):
        yr = g[f"{name}_y"][j]
        w = float(np.sqrt(np.mean(((s[k] - yr) / (rtol * np.abs(yr) + atol_vec)) ** 2)))
        assert w <= max(3.0 * own_w, 1e-6) and w <= 10.0, (k, w, own_w)


@pytest.mark.parametrize("name", ["r256", "r1024"])
@pytest.mark.parametrize("fused", [False, True], ids=["unfused_gs", "fused_gs"])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_cvode_robertson_block_preconditioner_matches_reference(name, fused, fma):
    """SPGMR with the exact block-Jacobi preconditioner on the FP64 block LU
    (bit-identical to SUNDlsMat_denseGETRF/GETRS per block)."""
    from oracle import robertson_cvode as rc
    from sundials_gb300.robertson import LU_FP64
    g, c, r, s = _run_robertson(name, fma, fused, LU_FP64)
    _check_against_reference(g, name, c, s, rc.vector_atol(len(g[f"{name}_k"])),
                             float(g[f"{name}_rtol"]))


@pytest.mark.parametrize("name", ["rd256", "rd1024"])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_cvode_robertson_direct_block_lu_matches_reference(name, fma):
    """The reference example's own configuration -- CVodeSetLinearSolver with
    SUNMatrix_BlockDiag_GB300 + SUNLinSol_BlockLU_GB300 (FP64) as the direct
    solver and the device Jacobian -- against the reference's CVode with
    SUNDenseMatrix + SUNLINSOL_DENSE (whose LU of the block-diagonal Newton
    matrix is the per-block LU, bit for bit)."""
    from oracle import robertson_cvode as rc
    from sundials_gb300.robertson import LU_FP64
    g, c, r, s = _run_robertson(name, fma, False, LU_FP64, direct=True)
    assert c[-1][list(hc.COUNTER_NAMES).index("nje")] > 0
    _check_against_reference(g, name, c, s, rc.vector_atol(len(g[f"{name}_k"])),
                             float(g[f"{name}_rtol"]))


def test_cvode_robertson_mixed_block_preconditioner():
    """The FP32-inverse + FP64-refinement block LU as the preconditioner.  Late
    in the run (t -> 4e10, gamma ~ 1e9) the Newton matrices' condition
    numbers (~1e13) exceed what an FP32 inverse can serve; those blocks fail
    the setup's probe and are factored in FP64.  The integration keeps the
    reference's step count within 5% and its solutions within the error
    tolerance at every stored output."""
    from oracle import robertson_cvode as rc
    from sundials_gb300.robertson import LU_MIXED
    g, c, r, s = _run_robertson("r1024", True, True, LU_MIXED)
    cr = g["r1024_counters"][-1]
    assert abs(int(c[-1][0]) - int(cr[0])) <= 0.05 * cr[0]
    atol = rc.vector_atol(1024)
    for j, k in enumerate(g["r1024_y_index"]):
        yr = g["r1024_y"][j]
        w = float(np.sqrt(np.mean(((s[k] - yr) / (1e-4 * np.abs(yr) + atol)) ** 2)))
        assert w <= 1.0, (k, w)


BR_GOLDEN = Path(__file__).resolve().parent / "golden" / "bruss3d_cvode_ref.npz"


@pytest.mark.parametrize("shape,c", [((6, 5, 7), 0.01), ((6, 5, 7), -0.02), ((4, 4, 4), 0.0),
                                     ((16, 16, 16), 0.01)])
def test_bruss3d_functions_bit_identical(shape, c):
    """Advection (both upwind directions and c = 0), reaction alone, the full
    right-hand side and the per-cell reaction solve: bit for bit the
    restatement of rhs3D.hpp."""
    from oracle import bruss3d_cvode as bc
    from sundials_gb300.bruss3d import Bruss3D
    from sundials_gb300.nvector import NVector
    q = bc.Params(*shape, c=c)
    rng = np.random.default_rng(7)
    y = rng.uniform(0.5, 4.0, q.n)
    b = rng.uniform(-1.0, 1.0, q.n)
    Y, B, O = NVector.from_numpy(y), NVector.from_numpy(b), NVector(q.n)
    P = Bruss3D(*shape, c=c)
    try:
        def beq(got, ref):
            return np.array_equal(got.view(np.int64), ref.view(np.int64))
        assert P.advection(Y, O) == 0 and beq(O.get(), bc.advection(q, y))
        assert P.reaction(Y, O) == 0 and beq(O.get(), bc.reaction(q, y))
        assert P.rhs(Y, O) == 0 and beq(O.get(), bc.rhs(q, y))
        for gamma in (1e-6, 3.7e-3, 0.25):
            assert P.solve_reaction(Y, O, B, gamma) == 0
            assert beq(O.get(), bc.solve_reaction(q, y, b, gamma)), gamma
        assert P.rhs(Y, Y) == -1  # the stencil needs distinct input and output
    finally:
        P.free()


@pytest.mark.parametrize("fused", [False, True], ids=["unfused_gs", "fused_gs"])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_cvode_bruss3d_matches_reference(fused, fma):
    """The benchmark's CVODE configuration on a 16^3 grid to t = 10: the
    reference's own reduction-order runs never moved a counter, so every
    counter after every output must equal the reference's; the last
    solution within 3x the reference's own weighted RMS deviation."""
    from sundials_gb300.bruss3d import Bruss3D
    from sundials_gb300.nvector import NVector
    from sundials_gb300.spgmr import PREC_LEFT, SPGMR
    g = np.load(BR_GOLDEN)
    rtol, atol = (float(v) for v in g["tol"])
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    S = SPGMR(y, pretype=PREC_LEFT, maxl=5)
    assert S.set_fused(fused) == 0
    P = Bruss3D(*(int(v) for v in g["grid"]))
    try:
        c, r, s = hc.run_port(y.v, S.S, P.cvode_callbacks(), lambda h: y.get(),
                              [float(t) for t in g["touts"]], rtol, atol)
    finally:
        S.free()
        P.free()
    assert np.array_equal(c, g["counters"]), (c[-1] - g["counters"][-1]).tolist()
    yr = g["y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + atol)) ** 2)))
    assert w <= max(3.0 * float(g["omp_wrms"].max()), 1e-6), w


@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_cvode_bruss3d_fixed_point_matches_reference(fma):
    """cvode_driver.cpp's ``--nls fixedpoint`` variant (Anderson depth 3, no
    linear solver: every operation is an NVECTOR_GB300 one, the fused dot
    products included) on the 16^3 grid to t = 10.  Here the reference is
    sensitive to its own summation order (its NVECTOR_OPENMP runs move steps
    and iterations by up to a few hundred and the solution by many
    tolerances), and six such runs are a small sample of that spread, so
    each counter must lie within twice the reference's own largest deviation
    + 1 (equal where it never moved) and the last solution within 3x its own
    weighted RMS deviation."""
    from sundials_gb300.bruss3d import Bruss3D
    from sundials_gb300.nvector import NVector
    g = np.load(BR_GOLDEN)
    rtol, atol = (float(v) for v in g["tol"])
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    P = Bruss3D(*(int(v) for v in g["grid"]))
    try:
        f, _, _, _, data = P.cvode_callbacks()
        c, r, s = hc.run_port(y.v, None, (f, None, None, None, data), lambda h: y.get(),
                              [float(t) for t in g["touts"]], rtol, atol, fixed_point=3)
    finally:
        P.free()
    ref = g["fp_counters"][-1]
    own = np.abs(g["fp_omp_counters"] - ref).max(axis=0)
    band = np.where(own == 0, 0, 2 * own + 1)
    dev = np.abs(c[-1] - ref)
    assert np.all(dev <= band), {n: (int(d), int(b)) for n, d, b in zip(hc.COUNTER_NAMES, dev, band)
                                 if d > b}
    yr = g["fp_y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + atol)) ** 2)))
    assert w <= max(3.0 * float(g["fp_omp_wrms"].max()), 1e-6), w


@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_cvode_bruss3d_adams_matches_reference(fma):
    """cvode_driver.cpp's CV-ADAMS configuration (Adams-Moulton with the
    fixed-point solver, Anderson depth 3, no linear solver) on the 16^3 grid
    over t in [0, 0.01] (some 3,200 steps: the stiff reaction bounds them).
    The reference's own reduction-order runs never moved a counter here, so
    every counter after every output must equal the reference's; the last
    solution within 3x its own weighted RMS deviation or 1e-3 tolerances
    (the own deviation is ~1e-6 here, below what one rounding per product
    in the FMA mode moves over thousands of steps)."""
    from sundials_gb300.bruss3d import Bruss3D
    from sundials_gb300.nvector import NVector
    g = np.load(BR_GOLDEN)
    rtol, atol = (float(v) for v in g["tol"])
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    P = Bruss3D(*(int(v) for v in g["grid"]))
    try:
        f, _, _, _, data = P.cvode_callbacks()
        c, r, s = hc.run_port(y.v, None, (f, None, None, None, data), lambda h: y.get(),
                              [float(t) for t in g["adams_touts"]], rtol, atol, fixed_point=3,
                              adams=True)
    finally:
        P.free()
    ref = g["adams_counters"]
    own = np.abs(g["adams_omp_counters"] - ref[-1]).max(axis=0)
    band = np.where(own == 0, 0, own + 1)
    dev = np.abs(c[-1] - ref[-1])
    assert np.all(dev <= band), {n: (int(d), int(b)) for n, d, b in zip(hc.COUNTER_NAMES, dev, band)
                                 if d > b}
    yr = g["adams_y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + atol)) ** 2)))
    assert w <= max(3.0 * float(g["adams_omp_wrms"].max()), 1e-3), w

"""CPU: the 3-D advection-reaction benchmark's CVODE configuration
(cvode_driver.cpp: SPGMR, difference-quotient J v, PSolve only) through the
CVODE restatement (oracle/cvode_ls_port.c) against the reference's own CVode
on the reference's serial vector and SPGMR, with the benchmark's user
functions restated in oracle/bruss3d_cvode.py."""
from pathlib import Path

import numpy as np
import pytest

from oracle import bruss3d_cvode as bc
from oracle import heat_cvode as hc

GOLDEN = Path(__file__).resolve().parent / "golden" / "bruss3d_cvode_ref.npz"
needs_ref = pytest.mark.skipif(not hc.REF_LIB.exists(),
                               reason="reference library not built on this machine")


def test_golden_layout():
    g = np.load(GOLDEN)
    n = 3 * int(np.prod(g["grid"]))
    assert g["u0"].shape == (n,) and g["y_last"].shape == (n,)
    assert g["counters"].shape == (len(g["touts"]), len(hc.COUNTER_NAMES))
    assert np.all(g["omp_counters"] == g["counters"][-1])  # order never moved a counter


def test_upwind_orders_differ_between_interior_and_faces():
    """The restated advection sums z, y, x inside and x, y, z on the upwind
    faces, as the reference's interior and face kernels do; the two orders
    give different bits somewhere on this grid, so the distinction is real."""
    q = bc.Params(6, 5, 7)
    y = np.random.default_rng(3).uniform(0.5, 4.0, q.n)
    a = bc.advection(q, y).reshape(6, 5, 7, 3)
    Y = y.reshape(6, 5, 7, 3)
    dx, dy, dz = (Y - np.roll(Y, 1, 0), Y - np.roll(Y, 1, 1), Y - np.roll(Y, 1, 2))
    xyz = (q.cx * dx + q.cy * dy) + q.cz * dz
    zyx = (q.cz * dz + q.cy * dy) + q.cx * dx
    assert np.array_equal(a[0], xyz[0]) and np.array_equal(a[1:, 1:, 1:], zyx[1:, 1:, 1:])
    assert not np.array_equal(xyz, zyx)


@needs_ref
def test_restatement_is_the_reference_cvode_small():
    q = bc.Params(8, 8, 8, tf=1.0, nout=4)
    c_ref, r_ref, y_ref = bc.run_reference(q)
    c, r, y = bc.run_port_serial(q)
    assert np.array_equal(c, c_ref)
    assert np.array_equal(r.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(y.view(np.int64), y_ref.view(np.int64))
    assert c_ref[-1][list(hc.COUNTER_NAMES).index("nfels")] > 0  # the DQ J v path ran


@needs_ref
def test_golden_is_the_reference_today():
    g = np.load(GOLDEN)
    q = bc.Params(*(int(v) for v in g["grid"]))
    assert np.array_equal(g["u0"].view(np.int64), bc.initial(q).view(np.int64))
    c, r, s = bc.run_reference(q)
    c2, r2, s2 = bc.run_port_serial(q)
    assert np.array_equal(c, g["counters"]) and np.array_equal(c2, c)
    assert np.array_equal(s[-1].view(np.int64), g["y_last"].view(np.int64))
    assert np.array_equal(s2.view(np.int64), s.view(np.int64))


@needs_ref
@pytest.mark.parametrize("shape,c", [((6, 5, 7), 0.01), ((8, 8, 8), -0.02)])
def test_fixed_point_restatement_is_the_reference_cvode(shape, c):
    """cvode_driver.cpp's ``--nls fixedpoint`` variant (SUNNonlinSol_FixedPoint,
    Anderson depth 3, no linear solver): the restatement
    (oracle/fixedpoint_port.c inside oracle/cvode_ls_port.c) bit for bit."""
    q = bc.Params(*shape, c=c)
    c_ref, r_ref, y_ref = bc.run_reference(q, fixed_point=3)
    c_p, r_p, y_p = bc.run_port_serial(q, fixed_point=3)
    assert np.array_equal(c_p, c_ref)
    assert np.array_equal(r_p.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(y_p.view(np.int64), y_ref.view(np.int64))
    last = dict(zip(hc.COUNTER_NAMES, c_ref[-1]))
    assert last["nni"] > 0 and last["nli"] == 0  # fixed point, no linear solver


def test_fixed_point_golden_layout():
    g = np.load(GOLDEN)
    assert g["fp_counters"].shape == g["counters"].shape
    assert g["fp_y_last"].shape == g["y_last"].shape
    assert g["fp_omp_counters"].shape == g["omp_counters"].shape
    last = dict(zip(hc.COUNTER_NAMES, g["fp_counters"][-1]))
    assert last["nni"] > 0 and last["nli"] == last["nps"] == last["nsetups"] == 0


@needs_ref
def test_fixed_point_golden_reproduced():
    g = np.load(GOLDEN)
    q = bc.Params(*(int(v) for v in g["grid"]))
    c, r, s = bc.run_port_serial(q, fixed_point=3)
    assert np.array_equal(c, g["fp_counters"])
    assert np.array_equal(r.view(np.int64), g["fp_reals"].view(np.int64))
    assert np.array_equal(s[-1].view(np.int64), g["fp_y_last"].view(np.int64))


@needs_ref
@pytest.mark.parametrize("shape,c,tf,k,rtol", [
    ((6, 5, 7), -0.02, 0.01, None, 1e-6),                 # the benchmark's stiff reaction
    ((6, 5, 7), -0.02, 10.0, (1, 1, 1, 1, 1, 1), 1e-10),  # non-stiff: orders up to 7
    ((5, 6, 4), 0.02, 5.0, (1, 1, 1, 1, 2, 2), 1e-12),
    ((4, 4, 4), 0.001, 10.0, (0.1, 0.1, 0.1, 0.1, 0.1, 0.1), 1e-14)])  # order 8
def test_adams_restatement_is_the_reference_cvode(shape, c, tf, k, rtol):
    """cvode_driver.cpp's CV-ADAMS configuration (Adams-Moulton with the
    fixed-point solver): the restatement bit for bit, including orders above
    BDF's 5 and order decreases (cvAdjustAdams)."""
    kw = {} if k is None else {"k": k, "rtol": rtol, "atol": rtol * 1e-3}
    q = bc.Params(*shape, c=c, tf=tf, nout=2 if k is None else 5, **kw)
    c_ref, r_ref, y_ref = bc.run_reference(q, fixed_point=3, adams=True)
    c_p, r_p, y_p = bc.run_port_serial(q, fixed_point=3, adams=True)
    assert np.array_equal(c_p, c_ref)
    assert np.array_equal(r_p.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(y_p.view(np.int64), y_ref.view(np.int64))
    if k is not None:
        assert c_ref[:, list(hc.COUNTER_NAMES).index("qu")].max() > 5


def test_adams_golden_layout():
    g = np.load(GOLDEN)
    assert len(g["adams_touts"]) == 2 and g["adams_touts"][-1] == 0.01
    assert g["adams_counters"].shape == (2, len(hc.COUNTER_NAMES))
    last = dict(zip(hc.COUNTER_NAMES, g["adams_counters"][-1]))
    assert last["nst"] > 1000 and last["nli"] == 0


@needs_ref
def test_adams_golden_reproduced():
    g = np.load(GOLDEN)
    q = bc.Params(*(int(v) for v in g["grid"]), tf=0.01, nout=2)
    c, r, s = bc.run_port_serial(q, fixed_point=3, adams=True)
    assert np.array_equal(c, g["adams_counters"])
    assert np.array_equal(r.view(np.int64), g["adams_reals"].view(np.int64))
    assert np.array_equal(s[-1].view(np.int64), g["adams_y_last"].view(np.int64))

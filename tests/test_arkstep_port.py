"""CPU: the ARKStep restatement (oracle/arkstep_port.c) against the
reference's own ARKodeEvolve, both on the reference's NVECTOR_SERIAL and
SUNLINSOL_SPGMR, on the 3-D advection-reaction benchmark's ARK-DIRK and
ARK-IMEX configurations (arkode_driver.cpp:51-160, 239-370) at orders 2-5 and
on ARK-IMEX with its task-local Newton (546-780, one task), and on both with
``--nls fixedpoint`` (SUNNonlinSol_FixedPoint, Anderson depth 3), with the
benchmark's user functions restated in oracle/bruss3d_cvode.py:
every counter, step size and solution value after every output time must be
identical, bit for bit."""
from pathlib import Path

import numpy as np
import pytest

from oracle import arkstep as ak
from oracle import bruss3d_cvode as bc
from oracle import heat_cvode as hc

GOLDEN = Path(__file__).resolve().parent / "golden" / "bruss3d_arkode_ref.npz"
needs_ref = pytest.mark.skipif(not hc.REF_LIB.exists(),
                               reason="reference library not built on this machine")


@pytest.mark.parametrize("name", ["dirk_", "imex_", "tl_"])
def test_golden_layout(name):
    g = np.load(GOLDEN)
    n = 3 * int(np.prod(g["grid"]))
    assert g["u0"].shape == (n,) and g[name + "y_last"].shape == (n,)
    assert g[name + "counters"].shape == (len(g["touts"]), len(ak.COUNTER_NAMES))
    assert g[name + "reals"].shape == (len(g["touts"]), len(ak.REAL_NAMES))
    T = ak.tables_from(g, name)
    Ti, Te = T["i"], T["e"]
    s = len(Ti["b"])
    assert Ti["A"].shape == (s, s) and tuple(Ti["orders"]) == (3, 2)
    # first stage explicit, lower-triangular implicit table, stiffly accurate
    assert Ti["A"][0, 0] == 0.0 and np.all(np.triu(Ti["A"], 1) == 0.0)
    assert np.array_equal(Ti["b"], Ti["A"][-1])
    if name != "dirk_":  # strictly lower-triangular explicit partner, same nodes
        assert Te["A"].shape == (s, s) and np.all(np.triu(Te["A"]) == 0.0)
        assert np.array_equal(Te["c"], Ti["c"])
        assert g[name + "counters"][-1][ak.COUNTER_NAMES.index("nfe")] > 0
    else:
        assert Te is None
    last = dict(zip(ak.COUNTER_NAMES, g[name + "counters"][-1]))
    if name == "tl_":  # no SUNLinearSolver; residuals counted by the solver itself
        assert last["nnlfi"] > 0 and last["nli"] == last["nps"] == last["nni"] == 0
        same = dict(zip(ak.COUNTER_NAMES, g["imex_counters"][-1]))
        assert last["nst"] == same["nst"] and last["nnlfi"] == same["nni"]
    else:
        assert last["nnlfi"] == 0 and last["nli"] > 0
    # the reference's own reduction-order runs never moved a counter
    assert np.all(g[name + "omp_counters"] == g[name + "counters"][-1])


@needs_ref
@pytest.mark.parametrize("imex,tl", [(False, False), (True, False), (True, True)],
                         ids=["dirk", "imex", "imex_tl_newton"])
@pytest.mark.parametrize("shape,c,order", [((6, 5, 7), 0.01, 3), ((6, 5, 7), -0.02, 4),
                                           ((5, 6, 4), 0.01, 2), ((8, 8, 8), 0.01, 3),
                                           ((6, 5, 7), 0.01, 5)])
def test_port_bit_identical_to_reference(shape, c, order, imex, tl):
    q = bc.Params(*shape, c=c)
    u0 = bc.initial(q)
    c_ref, r_ref, s_ref, tables = ak.run_reference_with(lambda L: bc.SerialBruss(L, q), u0,
                                                        q.touts, q.rtol, q.atol, order=order,
                                                        imex=imex, task_local=tl)
    c_p, r_p, s_p = ak.run_port_serial_with(lambda L: bc.SerialBruss(L, q), u0, q.touts, tables,
                                            q.rtol, q.atol, task_local=tl)
    assert np.array_equal(c_p, c_ref), (c_p[-1] - c_ref[-1]).tolist()
    assert np.array_equal(r_p.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(s_p.view(np.int64), s_ref.view(np.int64))


@needs_ref
@pytest.mark.parametrize("name", ["dirk_", "imex_", "tl_"])
def test_port_reproduces_golden(name):
    """The committed fixture (made by the reference) through the restatement,
    with the tables read from the fixture -- what the GPU test relies on."""
    g = np.load(GOLDEN)
    q = bc.Params(*(int(v) for v in g["grid"]))
    assert np.array_equal(bc.initial(q), g["u0"])
    c, r, s = bc.run_port_serial_arkode(q, ak.tables_from(g, name), task_local=name == "tl_")
    assert np.array_equal(c, g[name + "counters"])
    assert np.array_equal(r.view(np.int64), g[name + "reals"].view(np.int64))
    assert np.array_equal(s[-1].view(np.int64), g[name + "y_last"].view(np.int64))


@pytest.mark.parametrize("name", ["fpdirk_", "fpimex_"])
def test_fixed_point_golden_layout(name):
    g = np.load(GOLDEN)
    assert len(g[name + "touts"]) == 2 and g[name + "touts"][-1] == 0.01
    assert g[name + "counters"].shape == (2, len(ak.COUNTER_NAMES))
    last = dict(zip(ak.COUNTER_NAMES, g[name + "counters"][-1]))
    # the stiff reaction makes the iteration fail often; no linear solver
    assert last["nni"] > 0 and last["nnf"] > 0 and last["nli"] == last["nps"] == 0
    assert (ak.tables_from(g, name)["e"] is None) == (name == "fpdirk_")


@needs_ref
@pytest.mark.parametrize("imex", [False, True], ids=["dirk", "imex"])
@pytest.mark.parametrize("shape,c,order", [((6, 5, 7), 0.01, 3), ((6, 5, 7), -0.02, 4),
                                           ((5, 6, 4), 0.01, 2)])
def test_fixed_point_bit_identical_to_reference(shape, c, order, imex):
    """The fixed-point solver (oracle/fixedpoint_port.c) inside the ARKStep
    restatement, over t in [0, 0.01] (hundreds of steps and of nonlinear
    failures: the reaction is stiff)."""
    q = bc.Params(*shape, c=c, tf=0.01, nout=2)
    u0 = bc.initial(q)
    c_ref, r_ref, s_ref, tables = ak.run_reference_with(lambda L: bc.SerialBruss(L, q), u0,
                                                        q.touts, q.rtol, q.atol, order=order,
                                                        imex=imex, fixed_point=3)
    c_p, r_p, s_p = ak.run_port_serial_with(lambda L: bc.SerialBruss(L, q), u0, q.touts, tables,
                                            q.rtol, q.atol, fixed_point=3)
    assert np.array_equal(c_p, c_ref), (c_p[-1] - c_ref[-1]).tolist()
    assert np.array_equal(r_p.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(s_p.view(np.int64), s_ref.view(np.int64))


@needs_ref
@pytest.mark.parametrize("name", ["fpdirk_", "fpimex_"])
def test_fixed_point_golden_reproduced(name):
    g = np.load(GOLDEN)
    q = bc.Params(*(int(v) for v in g["grid"]), tf=0.01, nout=2)
    c, r, s = bc.run_port_serial_arkode(q, ak.tables_from(g, name), fixed_point=3)
    assert np.array_equal(c, g[name + "counters"])
    assert np.array_equal(r.view(np.int64), g[name + "reals"].view(np.int64))
    assert np.array_equal(s[-1].view(np.int64), g[name + "y_last"].view(np.int64))


def test_erk_golden_layout():
    g = np.load(GOLDEN)
    T = ak.tables_from(g, "erk_")
    assert T["erk"] and T["e"] is None and tuple(T["i"]["orders"]) == (3, 2)
    assert np.all(np.triu(T["i"]["A"]) == 0.0)  # explicit
    last = dict(zip(ak.COUNTER_NAMES, g["erk_counters"][-1]))
    assert last["nfe"] > 0 and last["nfi"] == last["nni"] == last["nli"] == 0
    assert np.all(g["erk_omp_counters"] == g["erk_counters"][-1])


@needs_ref
@pytest.mark.parametrize("order,shape,c,tf,k", [(3, (6, 5, 7), 0.01, 0.01, None),
                                                 (4, (6, 5, 7), -0.02, 0.01, None),
                                                 (2, (5, 6, 4), 0.01, 0.005, None),
                                                 (5, (6, 5, 7), 0.01, 0.01, None),
                                                 (6, (6, 5, 7), 0.01, 0.01, None),
                                                 (9, (6, 5, 7), -0.02, 0.01, None),
                                                 (3, (6, 5, 7), 0.01, 10.0, (1, 1, 1, 1, 1, 1))])
def test_erk_bit_identical_to_reference(order, shape, c, tf, k):
    """The benchmark's ERK configuration (ERKStepCreate, arkode_driver.cpp:
    441-540) through the restatement's ERKStep mode: stiff (steps held near
    1e-5 by stability, many error-test failures at order 2) and non-stiff;
    orders 6 and 9 take the quintic dense output."""
    q = bc.Params(*shape, c=c, tf=tf, nout=2, **({} if k is None else {"k": k}))
    u0 = bc.initial(q)
    c_ref, r_ref, s_ref, tables = ak.run_reference_with(lambda L: bc.SerialBruss(L, q), u0,
                                                        q.touts, q.rtol, q.atol, order=order,
                                                        erk=True)
    c_p, r_p, s_p = ak.run_port_serial_with(lambda L: bc.SerialBruss(L, q), u0, q.touts, tables,
                                            q.rtol, q.atol)
    assert np.array_equal(c_p, c_ref), (c_p[-1] - c_ref[-1]).tolist()
    assert np.array_equal(r_p.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(s_p.view(np.int64), s_ref.view(np.int64))


@needs_ref
def test_erk_golden_reproduced():
    g = np.load(GOLDEN)
    q = bc.Params(*(int(v) for v in g["grid"]), tf=0.01, nout=2)
    c, r, s = bc.run_port_serial_arkode(q, ak.tables_from(g, "erk_"))
    assert np.array_equal(c, g["erk_counters"])
    assert np.array_equal(r.view(np.int64), g["erk_reals"].view(np.int64))
    assert np.array_equal(s[-1].view(np.int64), g["erk_y_last"].view(np.int64))

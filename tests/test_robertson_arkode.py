"""CPU: the batched Robertson problem through ARKODE's ARKStep (DIRK, order
3, Newton) with the matrix-based direct path of ARKLS -- a SUNMatrix, a
direct SUNLinearSolver attached with ARKodeSetLinearSolver(LS, A), the user
Jacobian (ARKodeSetJacFn), per-species absolute tolerances -- in the ARKStep
restatement (oracle/arkstep_port.c: arkLsSetup, arkLsLinSys with the saved
Jacobian, the Newton setup / retry logic, the solution scaling of a direct
solve) against the reference's own ARKodeEvolve on SUNDenseMatrix +
SUNLINSOL_DENSE: every counter, step size and solution bit after every
output."""
from pathlib import Path

import numpy as np
import pytest

from oracle import arkstep as ak
from oracle import heat_cvode as hc
from oracle import robertson_cvode as rc

GOLDEN = Path(__file__).resolve().parent / "golden" / "robertson_arkode_ref.npz"
needs_ref = pytest.mark.skipif(not hc.REF_LIB.exists(),
                               reason="reference library not built on this machine")


def test_golden_layout():
    g = np.load(GOLDEN)
    n = 3 * int(g["cells"])
    assert g["u0"].shape == (n,) and g["y_last"].shape == (n,) and g["atol"].shape == (n,)
    assert g["counters"].shape == (len(g["touts"]), len(ak.COUNTER_NAMES))
    last = dict(zip(ak.COUNTER_NAMES, g["counters"][-1]))
    assert last["nsetups"] > 0 and last["nje"] > 0 and last["nli"] == 0  # direct solves
    assert np.all(g["omp_counters"] == g["counters"][-1])  # order never moved a counter
    assert tuple(ak.tables_from(g)["i"]["orders"]) == (3, 2)


@needs_ref
@pytest.mark.parametrize("ncells,nout", [(16, 12), (24, 7)])
def test_direct_path_bit_identical_to_reference(ncells, nout):
    touts = rc.TOUTS[:nout]
    c_ref, r_ref, s_ref, tables = rc.run_reference_arkode_direct(ncells, touts=touts)
    c_p, r_p, s_p = rc.run_port_serial_arkode_direct(ncells, tables, touts=touts)
    assert np.array_equal(c_p, c_ref), (c_p[-1] - c_ref[-1]).tolist()
    assert np.array_equal(r_p.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(s_p.view(np.int64), s_ref.view(np.int64))
    last = dict(zip(ak.COUNTER_NAMES, c_ref[-1]))
    assert last["nnf"] > 0 and last["netf"] > 0  # failure and retry paths ran


@needs_ref
def test_golden_reproduced():
    g = np.load(GOLDEN)
    c, r, s = rc.run_port_serial_arkode_direct(int(g["cells"]), ak.tables_from(g),
                                               touts=[float(t) for t in g["touts"]])
    assert np.array_equal(c, g["counters"])
    assert np.array_equal(r.view(np.int64), g["reals"].view(np.int64))
    assert np.array_equal(s[-1].view(np.int64), g["y_last"].view(np.int64))


@needs_ref
@pytest.mark.parametrize("ncells,nout", [(16, 12), (24, 7)])
def test_preconditioned_path_bit_identical_to_reference(ncells, nout):
    """ARKLS's iterative path with a preconditioner setup (arkLsSetup without
    a matrix, arkLsPSetup's jok / jcur logic): SPGMR with the user J v and
    the exact block-Jacobi preconditioner."""
    touts = rc.TOUTS[:nout]
    c_ref, r_ref, s_ref, tables = rc.run_reference_arkode(ncells, touts=touts)
    c_p, r_p, s_p = rc.run_port_serial_arkode(ncells, tables, touts=touts)
    assert np.array_equal(c_p, c_ref), (c_p[-1] - c_ref[-1]).tolist()
    assert np.array_equal(r_p.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(s_p.view(np.int64), s_ref.view(np.int64))
    last = dict(zip(ak.COUNTER_NAMES, c_ref[-1]))
    assert last["npe"] > 0 and last["nli"] > 0 and last["ncfl"] > 0


@needs_ref
def test_preconditioned_golden_reproduced():
    g = np.load(GOLDEN)
    c, r, s = rc.run_port_serial_arkode(int(g["cells"]), ak.tables_from(g, "prec_"),
                                        touts=[float(t) for t in g["touts"]])
    assert np.array_equal(c, g["prec_counters"])
    assert np.array_equal(r.view(np.int64), g["prec_reals"].view(np.int64))
    assert np.array_equal(s[-1].view(np.int64), g["prec_y_last"].view(np.int64))

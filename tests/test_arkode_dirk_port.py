"""CPU: the ARKStep DIRK restatement (oracle/arkode_dirk_port.c) against the
reference's own ARKodeEvolve, both on the reference's NVECTOR_SERIAL and
SUNLINSOL_SPGMR, on the 3-D advection-reaction benchmark's ARK-DIRK
configuration (arkode_driver.cpp:51-160) with the benchmark's user functions
restated in oracle/bruss3d_cvode.py: every counter, step size and solution
value after every output time must be identical, bit for bit."""
from pathlib import Path

import numpy as np
import pytest

from oracle import arkode_dirk as ad
from oracle import bruss3d_cvode as bc
from oracle import heat_cvode as hc

GOLDEN = Path(__file__).resolve().parent / "golden" / "bruss3d_arkode_ref.npz"
needs_ref = pytest.mark.skipif(not hc.REF_LIB.exists(),
                               reason="reference library not built on this machine")


def _table(g):
    return {k: g["table_" + k] for k in ad.TABLE_KEYS}


def test_golden_layout():
    g = np.load(GOLDEN)
    n = 3 * int(np.prod(g["grid"]))
    assert g["u0"].shape == (n,) and g["y_last"].shape == (n,)
    assert g["counters"].shape == (len(g["touts"]), len(ad.COUNTER_NAMES))
    assert g["reals"].shape == (len(g["touts"]), len(ad.REAL_NAMES))
    T = _table(g)
    s = len(T["b"])
    assert T["A"].shape == (s, s) and tuple(T["orders"]) == (3, 2)
    # ESDIRK (explicit first stage), stiffly accurate, lower triangular
    assert T["A"][0, 0] == 0.0 and np.array_equal(T["b"], T["A"][-1])
    assert np.all(np.triu(T["A"], 1) == 0.0)
    # the reference's own reduction-order runs never moved a counter
    assert np.all(g["omp_counters"] == g["counters"][-1])


@needs_ref
@pytest.mark.parametrize("shape,c,order", [((6, 5, 7), 0.01, 3), ((6, 5, 7), -0.02, 4),
                                           ((5, 6, 4), 0.01, 2), ((8, 8, 8), 0.01, 3)])
def test_port_bit_identical_to_reference(shape, c, order):
    q = bc.Params(*shape, c=c)
    u0 = bc.initial(q)
    c_ref, r_ref, s_ref, table = ad.run_reference_with(lambda L: bc.SerialBruss(L, q), u0,
                                                       q.touts, q.rtol, q.atol, order=order)
    c_p, r_p, s_p = ad.run_port_serial_with(lambda L: bc.SerialBruss(L, q), u0, q.touts, table,
                                            q.rtol, q.atol)
    assert np.array_equal(c_p, c_ref), (c_p[-1] - c_ref[-1]).tolist()
    assert np.array_equal(r_p.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(s_p.view(np.int64), s_ref.view(np.int64))


@needs_ref
def test_port_reproduces_golden():
    """The committed fixture (made by the reference) through the restatement,
    with the table read from the fixture -- what the GPU test relies on."""
    g = np.load(GOLDEN)
    q = bc.Params(*(int(v) for v in g["grid"]))
    assert np.array_equal(bc.initial(q), g["u0"])
    c, r, s = bc.run_port_serial_arkode(q, _table(g))
    assert np.array_equal(c, g["counters"])
    assert np.array_equal(r.view(np.int64), g["reals"].view(np.int64))
    assert np.array_equal(s[-1].view(np.int64), g["y_last"].view(np.int64))

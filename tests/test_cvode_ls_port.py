"""CPU: the CVODE restatement over generic objects (oracle/cvode_ls_port.c)
against the reference's own CVode (src/cvode/cvode.c, cvode_ls.c,
cvode_nls.c, sunnonlinsol_newton.c), both driving the reference's
NVECTOR_SERIAL and SUNLINSOL_SPGMR on the 2-D heat problem: every counter,
step size and solution bit must agree.  The GPU test
(tests/test_cvode_gb300_gpu.py) then runs the same restatement over
NVECTOR_GB300 + SUNLinSol_SPGMR_GB300, where the reference library does not
exist."""
from pathlib import Path

import numpy as np
import pytest

from oracle import heat_cvode as hc

GOLDEN = Path(__file__).resolve().parent / "golden" / "heat_cvode_ref.npz"
needs_ref = pytest.mark.skipif(not hc.REF_LIB.exists(),
                               reason="reference library not built on this machine")


def _case(g, name):
    nx, ny = (int(v) for v in g[f"{name}_grid"])
    rtol, atol = (float(v) for v in g[f"{name}_tol"])
    return nx, ny, rtol, atol, [float(t) for t in g[f"{name}_touts"]]


def test_golden_fixture_layout():
    g = np.load(GOLDEN)
    for name in g["names"]:
        nx, ny, rtol, atol, touts = _case(g, name)
        assert g[f"{name}_counters"].shape == (len(touts), len(hc.COUNTER_NAMES))
        assert g[f"{name}_y"].shape == (len(touts), nx * ny)
        assert g[f"{name}_u0"].shape == (nx * ny,)
        assert np.all(g[f"{name}_counters"][:, 0] > 0)
        # the reference's own summation-order sample
        oc = g[f"{name}_omp_counters"]
        assert oc.shape == (len(g[f"{name}_omp_threads"]), len(hc.COUNTER_NAMES))


@needs_ref
@pytest.mark.parametrize("name", ["g32", "g48x32_tight", "g128"])
def test_restatement_is_the_reference_cvode(name):
    g = np.load(GOLDEN)
    nx, ny, rtol, atol, touts = _case(g, name)
    c_ref, r_ref, y_ref, u0 = hc.run_reference(nx, ny, touts, rtol, atol)
    c, r, y = hc.run_port_serial(nx, ny, touts, rtol, atol)
    assert np.array_equal(c, c_ref)
    assert np.array_equal(r.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(y.view(np.int64), y_ref.view(np.int64))
    # and the committed fixture is what the reference prints today
    assert np.array_equal(g[f"{name}_counters"], c_ref)
    assert np.array_equal(g[f"{name}_y"].view(np.int64), y_ref.view(np.int64))
    assert np.array_equal(g[f"{name}_u0"].view(np.int64), u0.view(np.int64))


@needs_ref
def test_restatement_reaches_linear_solver_failures():
    """The 128^2 case takes the SPGMR 'residual reduced' path (ncfl > 0) and
    error-test failures, so those branches of the restatement are pinned."""
    g = np.load(GOLDEN)
    c = dict(zip(hc.COUNTER_NAMES, g["g128_counters"][-1]))
    assert c["ncfl"] > 0 and c["netf"] > 0

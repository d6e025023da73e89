"""CPU: the batched Robertson problem through CVODE + SPGMR with the exact
block-Jacobi preconditioner (examples/cvode/serial/cvDiurnal_kry.c pattern):
the CVODE restatement (oracle/cvode_ls_port.c) against the reference's own
CVode on the reference's serial vector and SPGMR, and the vectorised 3x3
GETRF/GETRS of the oracle against the dense LU restatement pinned to
SUNDlsMat_denseGETRF/GETRS (oracle/dense_port.c)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import heat_cvode as hc
from oracle import port
from oracle import robertson_cvode as rc

GOLDEN = Path(__file__).resolve().parent / "golden" / "robertson_cvode_ref.npz"
needs_ref = pytest.mark.skipif(not hc.REF_LIB.exists(),
                               reason="reference library not built on this machine")


def test_block_lu_restatement_is_dense_getrf():
    rng = np.random.default_rng(5)
    nb = 1500
    P = rng.standard_normal((nb, 3, 3))
    P[::7, 0, :] = 0.0          # pivot search past a zero
    P[::11, :, 0] = P[::11, :, 1]
    P[::13, 1, 2] = 0.0
    P[5] = 0.0                  # singular
    lu = P.copy()
    piv, fail = rc.getrf(lu)
    b = rng.standard_normal(3 * nb)
    good = np.nonzero(fail == 0)[0]
    x = rc.getrs(lu[good], piv[good], b.reshape(-1, 3)[good].reshape(-1)).reshape(-1, 3)
    assert (fail > 0).sum() > 100
    for c in range(nb):
        assert port.dense_lu(P[c].copy())[2] == fail[c]
    for gi, c in enumerate(good):
        ref_lu, ref_piv, _ = port.dense_lu(P[c].copy())
        assert np.array_equal(ref_lu.view(np.int64), lu[c].view(np.int64))
        assert np.array_equal(ref_piv, piv[c])
        ref_x = port.dense_solve(ref_lu, ref_piv, b[3 * c:3 * c + 3])
        assert np.array_equal(ref_x.view(np.int64), x[gi].view(np.int64))


def test_golden_layout():
    g = np.load(GOLDEN)
    for name in g["names"]:
        c = g[f"{name}_counters"]
        assert c.shape == (len(g[f"{name}_touts"]), len(hc.COUNTER_NAMES))
        assert g[f"{name}_y"].shape == (len(g[f"{name}_y_index"]), 3 * len(g[f"{name}_k"]))
        assert g[f"{name}_omp_counters"].shape == (len(g[f"{name}_omp_threads"]), c.shape[1])


@needs_ref
@pytest.mark.parametrize("name,ncells,direct", [("r256", 256, False), ("r1024", 1024, False),
                                                ("rd256", 256, True)])
def test_restatement_is_the_reference_cvode(name, ncells, direct):
    """SPGMR + block-Jacobi preconditioner (r*), and the matrix-based path
    with a direct solver and the user Jacobian (rd*: SUNDenseMatrix +
    SUNLINSOL_DENSE in both runs)."""
    g = np.load(GOLDEN)
    if direct:
        c_ref, r_ref, y_ref = rc.run_reference_direct(ncells)
        c, r, y = rc.run_port_serial(ncells, direct=True)
        assert c_ref[-1][list(hc.COUNTER_NAMES).index("nje")] > 0
    else:
        c_ref, r_ref, y_ref = rc.run_reference(ncells)
        c, r, y = rc.run_port_serial(ncells)
    assert np.array_equal(c, c_ref)
    assert np.array_equal(r.view(np.int64), r_ref.view(np.int64))
    assert np.array_equal(y.view(np.int64), y_ref.view(np.int64))
    assert np.array_equal(g[f"{name}_counters"], c_ref)
    keep = g[f"{name}_y_index"]
    assert np.array_equal(g[f"{name}_y"].view(np.int64), y_ref[keep].view(np.int64))
    assert np.array_equal(g[f"{name}_k"], rc.rates(ncells))

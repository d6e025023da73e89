"""GPU: the 3-D advection-reaction benchmark's default ARKODE configuration
(ARK-DIRK, order 3: arkode_driver.cpp:51-160) with the GB300 modules plugged
in -- NVECTOR_GB300 for every vector, SUNLinSol_SPGMR_GB300 (left
preconditioning, maxl 5) as the linear solver, and the device user functions
of include/bruss3d_gb300.h as the implicit right-hand side and the
preconditioner solve -- driven by the ARKStep restatement
oracle/arkode_dirk_port.c (the reference's ARKodeEvolve bit for bit on serial
objects: tests/test_arkode_dirk_port.py) with the reference's Butcher table
from the fixture, and compared with the reference's own run
(tests/golden/bruss3d_arkode_ref.npz).  The reference's own runs on
NVECTOR_OPENMP at 2-16 threads never moved a counter, so every counter after
every output must equal the reference's; the last solution within 3x the
reference's own weighted RMS deviation (in units of the tolerance)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import arkode_dirk as ad

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "bruss3d_arkode_ref.npz"


@pytest.mark.parametrize("fused", [False, True], ids=["unfused_gs", "fused_gs"])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_arkode_dirk_bruss3d_matches_reference(fused, fma):
    from sundials_gb300.bruss3d import Bruss3D
    from sundials_gb300.nvector import NVector
    from sundials_gb300.spgmr import PREC_LEFT, SPGMR
    g = np.load(GOLDEN)
    rtol, atol = (float(v) for v in g["tol"])
    table = {k: g["table_" + k] for k in ad.TABLE_KEYS}
    y = NVector.from_numpy(g["u0"])
    y.set_fma(fma)
    S = SPGMR(y, pretype=PREC_LEFT, maxl=5)
    assert S.set_fused(fused) == 0
    P = Bruss3D(*(int(v) for v in g["grid"]))
    try:
        c, r, s = ad.run_port(y.v, S.S, P.arkode_callbacks(), lambda h: y.get(),
                              [float(t) for t in g["touts"]], table, rtol, atol)
    finally:
        S.free()
        P.free()
    assert np.array_equal(c, g["counters"]), (c[-1] - g["counters"][-1]).tolist()
    yr = g["y_last"]
    w = float(np.sqrt(np.mean(((s[-1] - yr) / (rtol * np.abs(yr) + atol)) ** 2)))
    assert w <= max(3.0 * float(g["omp_wrms"].max()), 1e-6), w

"""CPU: pin the numpy SPGMR oracle (oracle/spgmr_port.py) to the reference's
own SPGMR (tests/golden/spgmr_ref.npz, made by tests/golden/gen_spgmr_golden.py
from SUNLinSol_SPGMR over NVECTOR_SERIAL), and check the solver's host-side
constants that need no GPU."""
from pathlib import Path

import numpy as np
import pytest

from oracle import spgmr_port as sp

GOLD = np.load(Path(__file__).parent / "golden" / "spgmr_ref.npz")
NAMES = [str(s) for s in GOLD["names"]]


def case(name):
    gs, pre, s1_on, s2_on, maxl, maxrs, n, zg = (int(v) for v in GOLD[f"{name}_params"])
    dg, lo, hi, delta = (float(v) for v in GOLD[f"{name}_op"])
    return dict(gs=gs, pre=pre, s1=GOLD[f"{name}_s1"] if s1_on else None,
                s2=GOLD[f"{name}_s2"] if s2_on else None, maxl=maxl, maxrs=maxrs, n=n,
                zg=bool(zg), dg=dg, lo=lo, hi=hi, delta=delta, b=GOLD[f"{name}_b"],
                x0=GOLD[f"{name}_x0"])


@pytest.mark.parametrize("name", NAMES)
def test_port_matches_reference_spgmr(name):
    c = case(name)
    s1 = c["s1"] if c["s1"] is not None else np.ones(c["n"])
    s2 = c["s2"] if c["s2"] is not None else np.ones(c["n"])

    def atimes(v):
        return sp.tridiag_apply(v, s1, s2, c["dg"], c["lo"], c["hi"])

    def psolve(r, lr):
        return r / c["dg"]
    flag, x, nli, res, _ = sp.spgmr_solve(
        atimes, psolve, c["x0"], c["b"], c["delta"], maxl=c["maxl"], max_restarts=c["maxrs"],
        gstype=c["gs"], pretype=c["pre"], s1=c["s1"], s2=c["s2"], zeroguess=c["zg"])
    assert flag == int(GOLD[f"{name}_flag"][0])
    assert nli == int(GOLD[f"{name}_nli"][0])
    xref = GOLD[f"{name}_x"]
    assert np.max(np.abs(x - xref)) <= 1e-12 * max(1.0, np.max(np.abs(xref)))
    rref = float(GOLD[f"{name}_resnorm"][0])
    assert abs(res - rref) <= 1e-7 * rref + 1e-300


def test_golden_covers_every_option():
    params = np.array([GOLD[f"{n}_params"] for n in NAMES])
    flags = {int(GOLD[f"{n}_flag"][0]) for n in NAMES}
    assert set(params[:, 0]) == {1, 2}            # modified and classical GS
    assert set(params[:, 1]) == {0, 1, 2, 3}      # every preconditioning side
    assert params[:, 2].any() and params[:, 3].any()  # both scaling vectors
    assert (params[:, 5] > 0).any()               # restarts
    assert flags == {0, 801, 802}                 # success, reduced, failure
    assert any(int(GOLD[f"{n}_nli"][0]) == 0 for n in NAMES)  # immediate return


def test_tridiag_operator_is_the_unit_test_operator():
    """With diag 5 and off-diagonals -1 the oracle's operator gives the bits of
    the reference unit test's ATimes expression, written out here per entry."""
    rng = np.random.default_rng(3)
    n = 9
    v, s1, s2 = rng.uniform(-1, 1, n), 1 + rng.uniform(0, 9, n), 1 + rng.uniform(0, 9, n)
    z = sp.tridiag_apply(v, s1, s2, 5.0, -1.0, -1.0)
    ref = np.empty(n)
    ref[0] = (5.0 * v[0] * s2[0] - v[1] * s2[1]) / s1[0]
    for i in range(1, n - 1):
        ref[i] = (-v[i - 1] * s2[i - 1] + 5.0 * v[i] * s2[i] - v[i + 1] * s2[i + 1]) / s1[i]
    ref[n - 1] = (-v[n - 2] * s2[n - 2] + 5.0 * v[n - 1] * s2[n - 1]) / s1[n - 1]
    assert np.array_equal(z, ref)

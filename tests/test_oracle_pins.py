"""Pin the oracle: the NVECTOR_SERIAL restatement (oracle/nvector_serial_port.c)
must reproduce, bit for bit, the outputs of the reference's own NVECTOR_SERIAL
stored in tests/golden/nvector_serial.npz (made by gen_nvector_golden.py from
oracle/_ref, i.e. the reference sources compiled by oracle/Makefile)."""
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "nvector_serial.npz"


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def beq(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("n", [1, 7, 1000])
def test_port_matches_reference_nvector_serial(oracle_lib, gold, n):
    from oracle import port
    P = port.ptr
    g = lambda k: gold[f"n{n}_{k}"]
    x, y, w, idm = g("in_x"), g("in_y"), g("in_w"), g("in_id")
    z = np.empty(n)
    for j, (a, b) in enumerate([(1, 1), (1, -1), (-1, 1), (1, 2.5), (0.3, 1), (-1, 0.7),
                                (0.3, -1), (2.5, 2.5), (2.5, -2.5), (0.3, 0.7)]):
        port.call("port_linearsum", a, P(x), b, P(y), P(z), n)
        assert beq(z, g(f"linearsum{j}")), (a, b)
    for name, args in [("prod", (P(x), P(y))), ("div", (P(x), P(y))), ("scale", (2.5, P(x))),
                       ("inv", (P(y),)), ("compare", (0.5, P(x)))]:
        port.call("port_" + name, *args, P(z), n)
        assert beq(z, g(name)), name
    port.call("port_addconst", P(x), -0.75, P(z), n)
    assert beq(z, g("addconst"))
    assert port.call("port_dotprod", P(x), P(y), n) == g("dotprod")[0]
    assert port.call("port_maxnorm", P(x), n) == g("maxnorm")[0]
    assert port.call("port_wrmsnorm", P(x), P(w), n) == g("wrmsnorm")[0]
    assert port.call("port_wrmsnormmask", P(x), P(w), P(idm), n) == g("wrmsnormmask")[0]
    assert port.call("port_min", P(x), n) == g("min")[0]
    assert port.call("port_wl2norm", P(x), P(w), n) == g("wl2norm")[0]
    assert port.call("port_l1norm", P(x), n) == g("l1norm")[0]
    assert port.call("port_minquotient", P(x), P(y), n) == g("minquotient")[0]
    zi = np.full(n, 7.0)
    assert port.call("port_invtest", P(g("in_xz")), P(zi), n) == g("invtest_flag")[0]
    assert beq(zi, g("invtest"))
    m = np.zeros(n)
    assert port.call("port_constrmask", P(g("in_cc")), P(x), P(m), n) == g("constrmask_flag")[0]
    assert beq(m, g("constrmask"))
    xs = [g(f"in_xs{k}") for k in range(5)]
    c5 = g("in_c5")
    port.call("port_linearcombination", 5, P(c5), port.ptrs(xs), P(z), n)
    assert beq(z, g("lincomb5"))
    Zs = [np.empty(n) for _ in range(5)]
    port.call("port_scaleaddmulti", 5, P(c5), P(x), port.ptrs(xs), port.ptrs(Zs), n)
    for k in range(5):
        assert beq(Zs[k], g(f"scaleaddmulti{k}"))
    d = np.empty(5)
    port.call("port_dotprodmulti", 5, P(x), port.ptrs(xs), P(d), n)
    assert beq(d, g("dotprodmulti5"))


DENSE = Path(__file__).resolve().parent / "golden" / "dense_lu.npz"


@pytest.mark.parametrize("case", ["1", "3", "8", "17", "33", "64", "singular"])
def test_dense_lu_port_matches_reference(oracle_lib, case):
    """GETRF / GETRS restatement (oracle/dense_port.c) against the reference's
    SUNDlsMat_denseGETRF / GETRS (tests/golden/dense_lu.npz): same bits."""
    from oracle import port
    g = dict(np.load(DENSE))
    lu, piv, flag = port.dense_lu(g[f"a_{case}"])
    assert flag == g[f"flag_{case}"][0]
    assert beq(lu, g[f"lu_{case}"]) and np.array_equal(piv[:len(piv)], g[f"piv_{case}"])
    if flag == 0:
        assert beq(port.dense_solve(lu, piv, g[f"b_{case}"]), g[f"x_{case}"])

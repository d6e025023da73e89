"""NVECTOR_GB300 parity against the NVECTOR_SERIAL restatement (oracle/).

Every operation is called through the vector's ops table, as CVODE does.
Tolerances:
  * elementwise, fused (LinearCombination, ScaleAddMulti) and vector-array
    operations: BIT-EXACT in the serial-order arithmetic mode
    (N_VSetFMA_GB300(v, 0)); in the default FMA mode within one rounding per
    term: |gpu - serial| <= 2.3e-16 * sum_k |c_k x_k|;
  * max / min reductions (MaxNorm, Min, MinQuotient, InvTest, ConstrMask):
    bit-exact (order-free);
  * sum reductions (DotProd, WrmsNorm, WL2Norm, L1Norm, DotProdMulti):
    |gpu - serial| <= 1e-12 * sum|terms|, because the GPU sums in a fixed tree
    order and the serial vector sequentially; and bitwise equal across reruns.
Known-answer cases mirror test/unit_tests/nvector/test_nvector.c.
"""
import ctypes as ct

import numpy as np
import pytest

from sundials_gb300 import _lib
from sundials_gb300.nvector import NVector

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 31, 33, 255, 257, 1000, 4097, 100003, (1 << 20) + 3]
SUM_RTOL = 1e-12


@pytest.fixture(scope="module")
def port(oracle_lib):
    from oracle import port as p
    return p


def rnd(n, seed, lo=-1.0, hi=1.0):
    return np.random.default_rng(seed).uniform(lo, hi, n)


def nv(a, exact=True):
    """Vectors of the bit-exact tests use the serial-order arithmetic mode."""
    v = NVector.from_numpy(a)
    v.set_fma(not exact)
    return v


def bits_equal(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def sum_close(g, s, terms):
    bound = SUM_RTOL * float(np.sum(np.abs(terms))) + 1e-300
    return abs(g - s) <= bound


@pytest.mark.parametrize("n", SIZES)
def test_linearsum_all_special_cases(gb300_lib, port, n):
    x, y = rnd(n, 1), rnd(n, 2)
    X, Y = nv(x), nv(y)
    Z = X.clone()
    ops = X.ops
    for a, b in [(1, 1), (1, -1), (-1, 1), (1, 2.5), (0.3, 1), (-1, 0.7), (0.3, -1),
                 (2.5, 2.5), (2.5, -2.5), (0.3, 0.7), (0.0, 0.7), (0.0, 0.0)]:
        ops["nvlinearsum"](a, X.v, b, Y.v, Z.v)
        ref = np.empty(n)
        port.call("port_linearsum", a, port.ptr(x), b, port.ptr(y), port.ptr(ref), n)
        assert bits_equal(Z.get(), ref), (a, b)
    # in-place axpy forms (z == y, b == 1) and (z == x, a == 1)
    ops["nvlinearsum"](0.25, X.v, 1.0, Y.v, Y.v)
    ref_y = np.empty(n)
    port.call("port_linearsum", 0.25, port.ptr(x), 1.0, port.ptr(y), port.ptr(ref_y), n)
    assert bits_equal(Y.get(), ref_y)
    ops["nvlinearsum"](1.0, X.v, -3.0, Y.v, X.v)
    ref_x = np.empty(n)
    port.call("port_linearsum", 1.0, port.ptr(x), -3.0, port.ptr(ref_y), port.ptr(ref_x), n)
    assert bits_equal(X.get(), ref_x)


@pytest.mark.parametrize("n", SIZES)
def test_streaming_ops_bitexact(gb300_lib, port, n):
    x, y = rnd(n, 3), rnd(n, 4)
    y[::7] += 2.0
    X, Y = nv(x), nv(y)
    Z = X.clone()
    ops = X.ops
    P = port.ptr
    ref = np.empty(n)

    ops["nvconst"](0.125, Z.v)
    port.call("port_const", 0.125, P(ref), n)
    assert bits_equal(Z.get(), ref)
    ops["nvprod"](X.v, Y.v, Z.v)
    port.call("port_prod", P(x), P(y), P(ref), n)
    assert bits_equal(Z.get(), ref)
    ops["nvdiv"](X.v, Y.v, Z.v)
    port.call("port_div", P(x), P(y), P(ref), n)
    assert bits_equal(Z.get(), ref)
    for c in (1.0, -1.0, 2.5):
        ops["nvscale"](c, X.v, Z.v)
        port.call("port_scale", c, P(x), P(ref), n)
        assert bits_equal(Z.get(), ref)
    ops["nvabs"](X.v, Z.v)
    port.call("port_abs", P(x), P(ref), n)
    assert bits_equal(Z.get(), ref)
    ops["nvinv"](Y.v, Z.v)
    port.call("port_inv", P(y), P(ref), n)
    assert bits_equal(Z.get(), ref)
    ops["nvaddconst"](X.v, -0.75, Z.v)
    port.call("port_addconst", P(x), -0.75, P(ref), n)
    assert bits_equal(Z.get(), ref)
    ops["nvcompare"](0.5, X.v, Z.v)
    port.call("port_compare", 0.5, P(x), P(ref), n)
    assert bits_equal(Z.get(), ref)
    # in place: z == x
    ops["nvscale"](3.0, X.v, X.v)
    port.call("port_scale", 3.0, P(x), P(ref), n)
    assert bits_equal(X.get(), ref)


@pytest.mark.parametrize("n", SIZES)
def test_reductions(gb300_lib, port, n):
    x, y = rnd(n, 5), rnd(n, 6)
    w = 1.0 / (1e-6 * np.abs(y) + 1e-10) * 1e-8
    idm = (rnd(n, 7) > 0).astype(np.float64)
    X, Y, W, ID = nv(x), nv(y), nv(w), nv(idm)
    ops = X.ops
    P = port.ptr

    g = ops["nvdotprod"](X.v, Y.v)
    assert sum_close(g, port.call("port_dotprod", P(x), P(y), n), x * y)
    g = ops["nvwrmsnorm"](X.v, W.v)
    s = port.call("port_wrmsnorm", P(x), P(w), n)
    assert abs(g - s) <= SUM_RTOL * s
    g = ops["nvwrmsnormmask"](X.v, W.v, ID.v)
    s = port.call("port_wrmsnormmask", P(x), P(w), P(idm), n)
    assert abs(g - s) <= SUM_RTOL * s + 1e-300
    g = ops["nvwl2norm"](X.v, W.v)
    s = port.call("port_wl2norm", P(x), P(w), n)
    assert abs(g - s) <= SUM_RTOL * s
    g = ops["nvl1norm"](X.v)
    s = port.call("port_l1norm", P(x), n)
    assert abs(g - s) <= SUM_RTOL * s
    assert ops["nvmaxnorm"](X.v) == port.call("port_maxnorm", P(x), n)
    assert ops["nvmin"](X.v) == port.call("port_min", P(x), n)
    assert ops["nvminquotient"](X.v, Y.v) == port.call("port_minquotient", P(x), P(y), n)
    # the *Local forms are the same reductions on one GPU
    assert ops["nvwsqrsumlocal"](X.v, W.v) == ops["nvwsqrsumlocal"](X.v, W.v)
    assert ops["nvdotprodlocal"](X.v, Y.v) == ops["nvdotprod"](X.v, Y.v)


@pytest.mark.parametrize("n", [257, 100003, (1 << 20) + 3])
def test_reductions_deterministic(gb300_lib, n):
    x, y = rnd(n, 8), rnd(n, 9)
    X, Y = nv(x), nv(y)
    vals = {X.ops["nvdotprod"](X.v, Y.v) for _ in range(5)}
    assert len(vals) == 1


@pytest.mark.parametrize("n", [1, 33, 4097, 100003])
def test_invtest_constrmask(gb300_lib, port, n):
    P = port.ptr
    x = rnd(n, 10)
    x[::5] = 0.0
    z0 = rnd(n, 11)
    X, Z = nv(x), nv(z0)
    ok = X.ops["nvinvtest"](X.v, Z.v)
    ref = z0.copy()
    ok_ref = port.call("port_invtest", P(x), P(ref), n)
    assert bool(ok) == bool(ok_ref) and bits_equal(Z.get(), ref)
    c = np.random.default_rng(12).choice([-2.0, -1.0, 0.0, 1.0, 2.0], n)
    xc = rnd(n, 13)
    xc[::9] = 0.0
    Cv, Xv, M = nv(c), nv(xc), nv(np.full(n, 7.0))
    ok = Cv.ops["nvconstrmask"](Cv.v, Xv.v, M.v)
    mref = np.empty(n)
    ok_ref = port.call("port_constrmask", P(c), P(xc), P(mref), n)
    assert bool(ok) == bool(ok_ref) and bits_equal(M.get(), mref)
    # no zero -> SUNTRUE
    xp = np.abs(rnd(n, 14)) + 0.5
    Xp = nv(xp)
    assert Xp.ops["nvinvtest"](Xp.v, Z.v) == 1


@pytest.mark.parametrize("n", [3, 1000, 100003])
@pytest.mark.parametrize("nvec", [1, 2, 3, 5, 8, 33])
def test_linearcombination(gb300_lib, port, n, nvec):
    P = port.ptr
    xs = [rnd(n, 20 + k) for k in range(nvec)]
    c = rnd(nvec, 99) * 2
    Xs = [nv(a) for a in xs]
    Z = nv(np.zeros(n))
    Z.ops["nvlinearcombination"](nvec, _lib.real_array(c), _lib.nv_array([v.v for v in Xs]), Z.v)
    ref = np.empty(n)
    port.call("port_linearcombination", nvec, P(c), port.ptrs(xs), P(ref), n)
    assert bits_equal(Z.get(), ref)
    if nvec >= 3:
        # aliasing: X[0] == z with c[0] == 1 and with c[0] != 1
        for c0 in (1.0, 0.5):
            cc = c.copy()
            cc[0] = c0
            z0 = xs[0].copy()
            Z0 = nv(z0)
            arr = _lib.nv_array([Z0.v] + [v.v for v in Xs[1:]])
            Z0.ops["nvlinearcombination"](nvec, _lib.real_array(cc), arr, Z0.v)
            refz = z0.copy()
            port.call("port_linearcombination", nvec, P(cc), port.ptrs([refz] + xs[1:]),
                      P(refz), n)
            assert bits_equal(Z0.get(), refz), c0


@pytest.mark.parametrize("n", [3, 1000, 100003])
@pytest.mark.parametrize("nvec", [1, 3, 5, 40])
def test_scaleaddmulti_dotprodmulti(gb300_lib, port, n, nvec):
    P = port.ptr
    x = rnd(n, 30)
    ys = [rnd(n, 31 + k) for k in range(nvec)]
    a = rnd(nvec, 77)
    X = nv(x)
    Ys = [nv(v) for v in ys]
    Zs = [nv(np.zeros(n)) for _ in range(nvec)]
    X.ops["nvscaleaddmulti"](nvec, _lib.real_array(a), X.v, _lib.nv_array([v.v for v in Ys]),
                             _lib.nv_array([v.v for v in Zs]))
    refs = [np.empty(n) for _ in range(nvec)]
    port.call("port_scaleaddmulti", nvec, P(a), P(x), port.ptrs(ys), port.ptrs(refs), n)
    for k in range(nvec):
        assert bits_equal(Zs[k].get(), refs[k])
    # in place Y == Z
    arr = _lib.nv_array([v.v for v in Ys])
    X.ops["nvscaleaddmulti"](nvec, _lib.real_array(a), X.v, arr, arr)
    for k in range(nvec):
        assert bits_equal(Ys[k].get(), refs[k])
    # DotProdMulti: x read once; each entry equals the single DotProd bit for bit
    d = (ct.c_double * nvec)()
    X.ops["nvdotprodmulti"](nvec, X.v, _lib.nv_array([v.v for v in Zs]), d)
    for k in range(nvec):
        single = X.ops["nvdotprod"](X.v, Zs[k].v)
        assert d[k] == single
        s = port.call("port_dotprod", P(x), P(refs[k]), n)
        assert sum_close(d[k], s, x * refs[k])


@pytest.mark.parametrize("n", [5, 1000, 100003])
def test_vector_array_ops(gb300_lib, port, n):
    P = port.ptr
    nvec = 4
    xs = [rnd(n, 40 + k) for k in range(nvec)]
    ys = [rnd(n, 50 + k) for k in range(nvec)]
    Xs, Ys = [nv(v) for v in xs], [nv(v) for v in ys]
    Zs = [nv(np.zeros(n)) for _ in range(nvec)]
    ops = Xs[0].ops
    arrX, arrY, arrZ = (_lib.nv_array([v.v for v in V]) for V in (Xs, Ys, Zs))
    for a, b in [(0.3, 0.7), (2.0, 2.0), (2.0, -2.0), (1.0, -1.0)]:
        ops["nvlinearsumvectorarray"](nvec, a, arrX, b, arrY, arrZ)
        for k in range(nvec):
            ref = np.empty(n)
            port.call("port_linearsum", a, P(xs[k]), b, P(ys[k]), P(ref), n)
            assert bits_equal(Zs[k].get(), ref)
    c = rnd(nvec, 60)
    ops["nvscalevectorarray"](nvec, _lib.real_array(c), arrX, arrZ)
    for k in range(nvec):
        assert bits_equal(Zs[k].get(), c[k] * xs[k])
    ops["nvconstvectorarray"](nvec, -1.5, arrZ)
    for k in range(nvec):
        assert bits_equal(Zs[k].get(), np.full(n, -1.5))
    ws = [np.abs(rnd(n, 70 + k)) + 0.1 for k in range(nvec)]
    Ws = [nv(v) for v in ws]
    arrW = _lib.nv_array([v.v for v in Ws])
    nrm = (ct.c_double * nvec)()
    ops["nvwrmsnormvectorarray"](nvec, arrX, arrW, nrm)
    idm = (rnd(n, 80) > -0.3).astype(np.float64)
    ID = nv(idm)
    nrmm = (ct.c_double * nvec)()
    ops["nvwrmsnormmaskvectorarray"](nvec, arrX, arrW, ID.v, nrmm)
    for k in range(nvec):
        s = port.call("port_wrmsnorm", P(xs[k]), P(ws[k]), n)
        assert abs(nrm[k] - s) <= SUM_RTOL * s
        assert nrm[k] == ops["nvwrmsnorm"](Xs[k].v, Ws[k].v)
        sm = port.call("port_wrmsnormmask", P(xs[k]), P(ws[k]), P(idm), n)
        assert abs(nrmm[k] - sm) <= SUM_RTOL * sm


@pytest.mark.parametrize("n", [7, 1000, 100003])
@pytest.mark.parametrize("nvec,nsum", [(1, 1), (1, 3), (3, 1), (3, 4), (2, 10)])
def test_scaleaddmulti_vectorarray(gb300_lib, port, n, nvec, nsum):
    P = port.ptr
    xs = [rnd(n, 100 + i) for i in range(nvec)]
    ys = [[rnd(n, 200 + 10 * j + i) for i in range(nvec)] for j in range(nsum)]
    a = rnd(nsum, 300)
    Xs = [nv(v) for v in xs]
    Ys = [[nv(v) for v in row] for row in ys]
    Zs = [[nv(np.zeros(n)) for _ in range(nvec)] for _ in range(nsum)]
    rowsY = [_lib.nv_array([v.v for v in row]) for row in Ys]
    rowsZ = [_lib.nv_array([v.v for v in row]) for row in Zs]
    PY = (_lib.P_NV * nsum)(*[ct.cast(r, _lib.P_NV) for r in rowsY])
    PZ = (_lib.P_NV * nsum)(*[ct.cast(r, _lib.P_NV) for r in rowsZ])
    Xs[0].ops["nvscaleaddmultivectorarray"](nvec, nsum, _lib.real_array(a),
                                            _lib.nv_array([v.v for v in Xs]), PY, PZ)
    for j in range(nsum):
        for i in range(nvec):
            assert bits_equal(Zs[j][i].get(), a[j] * xs[i] + ys[j][i])


@pytest.mark.parametrize("n", [7, 1000, 100003])
@pytest.mark.parametrize("nvec,nsum", [(1, 1), (1, 2), (1, 4), (3, 1), (3, 2), (3, 5), (2, 11)])
def test_linearcombination_vectorarray(gb300_lib, port, n, nvec, nsum):
    P = port.ptr
    xs = [[rnd(n, 400 + 10 * i + j) for j in range(nvec)] for i in range(nsum)]
    c = rnd(nsum, 500)
    Xs = [[nv(v) for v in row] for row in xs]
    Zs = [nv(np.zeros(n)) for _ in range(nvec)]
    rows = [_lib.nv_array([v.v for v in row]) for row in Xs]
    PX = (_lib.P_NV * nsum)(*[ct.cast(r, _lib.P_NV) for r in rows])
    Zs[0].ops["nvlinearcombinationvectorarray"](nvec, nsum, _lib.real_array(c), PX,
                                                _lib.nv_array([v.v for v in Zs]))
    for j in range(nvec):
        ref = np.empty(n)
        port.call("port_linearcombination", nsum, P(c), port.ptrs([xs[i][j] for i in range(nsum)]),
                  P(ref), n)
        assert bits_equal(Zs[j].get(), ref)


def test_unaligned_operands_take_scalar_path(gb300_lib, port):
    """A device pointer 8 bytes past a 16-byte boundary (a subvector view)."""
    lib = gb300_lib
    n = 10001
    base = NVector(n + 1)
    base.set_fma(False)
    x = rnd(n, 600)
    base.set(np.concatenate([[0.0], x]))
    view = lib.N_VMake_GB300(n, None, ct.cast(base.device_ptr + 8, _lib.P_real), None)
    V = NVector(n, handle=view)
    V.set_fma(False)
    Y = nv(rnd(n, 601))
    Z = Y.clone()
    V.ops["nvlinearsum"](0.3, V.v, 0.7, Y.v, Z.v)
    ref = np.empty(n)
    yy = Y.get()
    port.call("port_linearsum", 0.3, port.ptr(x), 0.7, port.ptr(yy), port.ptr(ref), n)
    assert bits_equal(Z.get(), ref)
    g = V.ops["nvdotprod"](V.v, Y.v)
    assert sum_close(g, port.call("port_dotprod", port.ptr(x), port.ptr(yy), n), x * yy)


def test_known_answers_from_reference_harness(gb300_lib):
    """Closed-form cases of test_nvector.c (WrmsNorm :1503, DotProdMulti :2613,
    LinearCombination :2155, ScaleAddMulti :2440)."""
    n = 1000
    X, W = nv(np.full(n, -0.5)), nv(np.full(n, 0.5))
    assert X.ops["nvwrmsnorm"](X.v, W.v) == 0.25
    x = NVector.from_numpy(np.full(n, 2.0))
    Ys = [nv(np.full(n, v)) for v in (-0.5, 0.5, 1.0)]
    d = (ct.c_double * 3)()
    x.ops["nvdotprodmulti"](3, x.v, _lib.nv_array([v.v for v in Ys]), d)
    assert list(d) == [-n, n, 2 * n]
    X1, X2, X3 = nv(np.full(n, 1.0)), nv(np.full(n, -2.0)), nv(np.full(n, 3.0))
    Z = nv(np.zeros(n))
    c = _lib.real_array([1.0, 0.5, -2.0])
    X1.ops["nvlinearcombination"](3, c, _lib.nv_array([X1.v, X2.v, X3.v]), Z.v)
    assert np.all(Z.get() == 1.0 - 1.0 - 6.0)
    A = _lib.real_array([2.0, 1.0])
    Y1, Y2 = nv(np.full(n, -1.0)), nv(np.full(n, 1.0))
    Z1, Z2 = nv(np.zeros(n)), nv(np.zeros(n))
    X1.ops["nvscaleaddmulti"](2, A, X1.v, _lib.nv_array([Y1.v, Y2.v]), _lib.nv_array([Z1.v, Z2.v]))
    assert np.all(Z1.get() == 1.0) and np.all(Z2.get() == 2.0)


def test_fused_ops_can_be_disabled(gb300_lib):
    v = NVector(10)
    assert v.ops["nvlinearcombination"] is not None
    gb300_lib.N_VEnableFusedOps_GB300(v.v, 0)
    ops = _lib.ops_of(v.v)
    for name in ("nvlinearcombination", "nvscaleaddmulti", "nvdotprodmulti",
                 "nvlinearsumvectorarray", "nvwrmsnormvectorarray"):
        assert ops[name] is None
    c = v.clone()  # clones copy the ops table
    assert c.ops["nvdotprodmulti"] is None


def test_fma_mode_within_one_rounding_per_term(gb300_lib, port):
    n = 100003
    x, y = rnd(n, 700), rnd(n, 701)
    X, Y = nv(x, exact=False), nv(y, exact=False)
    Z = X.clone()
    Z.ops["nvlinearsum"](0.3, X.v, 0.7, Y.v, Z.v)
    ref = np.empty(n)
    port.call("port_linearsum", 0.3, port.ptr(x), 0.7, port.ptr(y), port.ptr(ref), n)
    err = np.abs(Z.get() - ref)
    assert np.all(err <= 2.3e-16 * (np.abs(0.3 * x) + np.abs(0.7 * y)))
    # LinearCombination(5) and ScaleAddMulti(3) in the default FMA mode
    xs = [rnd(n, 710 + k) for k in range(5)]
    c = rnd(5, 720)
    Xs = [nv(a, exact=False) for a in xs]
    Zc = nv(np.zeros(n), exact=False)
    Zc.ops["nvlinearcombination"](5, _lib.real_array(c), _lib.nv_array([v.v for v in Xs]), Zc.v)
    port.call("port_linearcombination", 5, port.ptr(c), port.ptrs(xs), port.ptr(ref), n)
    bound = 2.3e-16 * 5 * sum(np.abs(c[k] * xs[k]) for k in range(5))
    assert np.all(np.abs(Zc.get() - ref) <= bound)
    Zs = [nv(np.zeros(n), exact=False) for _ in range(3)]
    X.ops["nvscaleaddmulti"](3, _lib.real_array(c[:3]), X.v, _lib.nv_array([v.v for v in Xs[:3]]),
                             _lib.nv_array([v.v for v in Zs]))
    for k in range(3):
        exact = c[k] * x + xs[k]
        assert np.all(np.abs(Zs[k].get() - exact) <= 2.3e-16 * (np.abs(c[k] * x) + np.abs(xs[k])))
    # reductions in FMA mode stay within the sum tolerance
    g = X.ops["nvdotprod"](X.v, Y.v)
    assert sum_close(g, port.call("port_dotprod", port.ptr(x), port.ptr(y), n), x * y)


def test_identity_and_utilities(gb300_lib):
    v = NVector(17)
    assert v.ops["nvgetvectorid"](v.v) == 16  # SUNDIALS_NVEC_CUSTOM
    assert v.ops["nvgetlength"](v.v) == 17
    assert v.ops["nvgetlocallength"](v.v) == 17
    assert v.ops["nvgetcommunicator"](v.v) == 0
    sz = _lib.idx()
    v.ops["nvbufsize"](v.v, ct.byref(sz))
    assert sz.value == 17 * 8
    data = rnd(17, 800)
    buf = data.copy()
    assert v.ops["nvbufunpack"](v.v, buf.ctypes.data) == 0
    out = np.zeros(17)
    assert v.ops["nvbufpack"](v.v, out.ctypes.data) == 0
    assert bits_equal(out, data)
    e = v.ops["nvcloneempty"](v.v)
    assert gb300_lib.N_VGetDeviceArrayPointer_GB300(e) is None
    v.ops["nvdestroy"](e)

"""GPU: CVODE's fused integrator kernels over NVECTOR_GB300
(include/cvode_fused_gb300.h) against the serial sequences they replace
(src/cvode/cvode_fused_stubs.c), composed here from the oracle's NVECTOR_SERIAL
restatement (oracle/nvector_serial_port.c, pinned to the reference's golden
vectors).  Exact mode: bit-identical.  FMA mode (one rounding less per
contracted product): element-wise relative error 1e-15 where no terms cancel
(tolerances, weights), else an absolute error of a few ulp of the operands'
magnitude (sums that may cancel), 1e-11 relative for buildM's quotient of a
difference."""
import ctypes as ct

import numpy as np
import pytest

from oracle import port

pytestmark = pytest.mark.gpu
N = 100003
D = ct.c_double
VP = ct.c_void_p


def _fn(lib, name, args):
    f = getattr(lib, name)
    f.restype = ct.c_int
    f.argtypes = args
    return f


def _vecs(arrs, fma):
    from sundials_gb300.nvector import NVector
    out = []
    for a in arrs:
        v = NVector.from_numpy(a)
        v.set_fma(fma)
        out.append(v)
    return out


def _p(a):
    return port.ptr(a)


def _check(got, ref, fma, rtol=1e-15, operand_scale=None):
    if not fma:
        assert np.array_equal(got.view(np.int64), ref.view(np.int64))
    elif operand_scale is None:
        scale = np.maximum(np.abs(ref), 1e-300)
        assert np.max(np.abs(got - ref) / scale) <= rtol
    else:
        assert np.max(np.abs(got - ref)) <= rtol * operand_scale


@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_ewt_ss_and_sv(gb300_lib, fma):
    rng = np.random.default_rng(1)
    y = rng.uniform(-2, 2, N)
    y[::97] = 0.0
    vabs = rng.uniform(1e-10, 1e-6, N)
    rel, sabs = 1e-6, 1e-10
    # serial sequences
    t = np.empty(N)
    port.call("port_abs", _p(y), _p(t), N)
    port.call("port_scale", rel, _p(t), _p(t), N)
    port.call("port_addconst", _p(t), sabs, _p(t), N)
    w = np.empty(N)
    port.call("port_inv", _p(t), _p(w), N)
    t2 = np.empty(N)
    port.call("port_abs", _p(y), _p(t2), N)
    port.call("port_linearsum", rel, _p(t2), 1.0, _p(vabs), _p(t2), N)
    w2 = np.empty(N)
    port.call("port_inv", _p(t2), _p(w2), N)
    Y, T, W, VA = _vecs([y, np.zeros(N), np.zeros(N), vabs], fma)
    ss = _fn(gb300_lib, "cvEwtSetSS_fused", [ct.c_int, D, D, VP, VP, VP])
    sv = _fn(gb300_lib, "cvEwtSetSV_fused", [ct.c_int, D, VP, VP, VP, VP])
    assert ss(1, rel, sabs, Y.v, T.v, W.v) == 0
    _check(T.get(), t, fma)
    _check(W.get(), w, fma)
    assert sv(0, rel, VA.v, Y.v, T.v, W.v) == 0
    _check(T.get(), t2, fma)
    _check(W.get(), w2, fma)
    # atolmin0: a zero tolerance entry makes the call fail
    assert ss(1, rel, 0.0, Y.v, T.v, W.v) == -1
    assert ss(0, rel, 0.0, Y.v, T.v, W.v) == 0


@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_check_constraints(gb300_lib, fma):
    rng = np.random.default_rng(2)
    c = rng.choice([-2.0, -1.0, 0.0, 1.0, 2.0], N)
    ewt = 1.0 / rng.uniform(1e-8, 1e-3, N)
    y = rng.uniform(-1, 1, N)
    mm = rng.choice([0.0, 1.0], N)
    t = np.empty(N)
    port.call("port_compare", 1.5, _p(c), _p(t), N)
    port.call("port_prod", _p(t), _p(c), _p(t), N)
    port.call("port_div", _p(t), _p(ewt), _p(t), N)
    port.call("port_linearsum", 1.0, _p(y), -0.1, _p(t), _p(t), N)
    port.call("port_prod", _p(t), _p(mm), _p(t), N)
    C, E, Y, M, T = _vecs([c, ewt, y, mm, np.zeros(N)], fma)
    f = _fn(gb300_lib, "cvCheckConstraints_fused", [VP] * 5)
    assert f(C.v, E.v, Y.v, M.v, T.v) == 0
    _check(T.get(), t, fma, rtol=4e-16, operand_scale=1.0)


@pytest.mark.parametrize("ngamma", [-0.37, -1.0, 1.0])
@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_nls_resid(gb300_lib, fma, ngamma):
    rng = np.random.default_rng(3)
    zn1, ycor, ft = (rng.uniform(-1, 1, N) for _ in range(3))
    rl1 = 0.61
    r = np.empty(N)
    port.call("port_linearsum", rl1, _p(zn1), 1.0, _p(ycor), _p(r), N)
    port.call("port_linearsum", ngamma, _p(ft), 1.0, _p(r), _p(r), N)
    Z, Yc, F, R = _vecs([zn1, ycor, ft, np.zeros(N)], fma)
    f = _fn(gb300_lib, "cvNlsResid_fused", [D, D, VP, VP, VP, VP])
    assert f(rl1, ngamma, Z.v, Yc.v, F.v, R.v) == 0
    _check(R.get(), r, fma, rtol=8e-16, operand_scale=3.0)


@pytest.mark.parametrize("fma", [False, True], ids=["exact", "fma"])
def test_diag_setup_and_solve(gb300_lib, fma):
    rng = np.random.default_rng(4)
    fpred, zn1, ypred = (rng.uniform(-1, 1, N) for _ in range(3))
    h, r, fract, uround = 3.7e-3, 0.1, 0.1, 2.220446049250313e-16
    # formY
    ft = np.empty(N)
    port.call("port_linearsum", h, _p(fpred), -1.0, _p(zn1), _p(ft), N)
    yy = np.empty(N)
    port.call("port_linearsum", r, _p(ft), 1.0, _p(ypred), _p(yy), N)
    FP, Z1, YP, FT, YV = _vecs([fpred, zn1, ypred, np.zeros(N), np.zeros(N)], fma)
    formy = _fn(gb300_lib, "cvDiagSetup_formY", [D, D, VP, VP, VP, VP, VP])
    assert formy(h, r, FP.v, Z1.v, YP.v, FT.v, YV.v) == 0
    _check(FT.get(), ft, fma, rtol=4e-16, operand_scale=1.0)
    _check(YV.get(), yy, fma, rtol=4e-16, operand_scale=2.0)
    # buildM (ftemp with entries whose weighted size is below uround)
    ftemp = rng.uniform(-1e-3, 1e-3, N)
    ftemp[::11] = 1e-30
    ewt = 1.0 / rng.uniform(1e-8, 1e-4, N)
    M0 = rng.uniform(-1, 1, N)
    m = M0.copy()
    port.call("port_linearsum", 1.0, _p(m), -1.0, _p(fpred), _p(m), N)
    port.call("port_linearsum", fract, _p(ftemp), -h, _p(m), _p(m), N)
    y2 = np.empty(N)
    port.call("port_prod", _p(ftemp), _p(ewt), _p(y2), N)
    bit = np.empty(N)
    port.call("port_compare", uround, _p(y2), _p(bit), N)
    bitc = np.empty(N)
    port.call("port_addconst", _p(bit), -1.0, _p(bitc), N)
    port.call("port_prod", _p(ftemp), _p(bit), _p(y2), N)
    port.call("port_linearsum", fract, _p(y2), -1.0, _p(bitc), _p(y2), N)
    port.call("port_div", _p(m), _p(y2), _p(m), N)
    port.call("port_prod", _p(m), _p(bit), _p(m), N)
    port.call("port_linearsum", 1.0, _p(m), -1.0, _p(bitc), _p(m), N)
    FT2, FP2, EW, B, BC, Y2, MV = _vecs([ftemp, fpred, ewt, np.zeros(N), np.zeros(N),
                                         np.zeros(N), M0], fma)
    buildm = _fn(gb300_lib, "cvDiagSetup_buildM", [D, D, D] + [VP] * 7)
    assert buildm(fract, uround, h, FT2.v, FP2.v, EW.v, B.v, BC.v, Y2.v, MV.v) == 0
    assert np.array_equal(B.get(), bit) and np.array_equal(BC.get(), bitc)
    _check(Y2.get(), y2, fma, rtol=1e-13)
    _check(MV.get(), m, fma, rtol=1e-11)
    # updateM
    mu = m.copy()
    port.call("port_inv", _p(mu), _p(mu), N)
    port.call("port_addconst", _p(mu), -1.0, _p(mu), N)
    port.call("port_scale", 0.83, _p(mu), _p(mu), N)
    port.call("port_addconst", _p(mu), 1.0, _p(mu), N)
    upd = _fn(gb300_lib, "cvDiagSolve_updateM", [D, VP])
    MV.set(m)
    assert upd(0.83, MV.v) == 0
    _check(MV.get(), mu, fma, rtol=4e-16,
           operand_scale=1.0 + float(np.max(np.abs(0.83 * (1.0 / m - 1.0)))))


def test_rejects_mismatched_vectors(gb300_lib):
    from sundials_gb300.nvector import NVector
    a, b = NVector(10), NVector(11)
    f = _fn(gb300_lib, "cvNlsResid_fused", [D, D, VP, VP, VP, VP])
    assert f(1.0, -1.0, a.v, a.v, b.v, a.v) == -1

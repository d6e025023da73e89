"""Generate tests/golden/nvector_serial.npz from the reference itself.

Runs the reference's NVECTOR_SERIAL (oracle/_ref/libsundials_ref.so, compiled
from the reference sources by oracle/Makefile) through its generic N_V* API on
seeded inputs and stores inputs and outputs.  The oracle restatement
(oracle/nvector_serial_port.c) must reproduce these bits on any machine.

Usage (in a checkout that has the reference sources):
    python -m sundials_gb300.build && python tests/golden/gen_nvector_golden.py
"""
import ctypes as ct
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
REF = ROOT / "oracle" / "_ref" / "libsundials_ref.so"
OUT = Path(__file__).resolve().parent / "nvector_serial.npz"


def main():
    L = ct.CDLL(str(REF))
    P = ct.POINTER(ct.c_double)
    vp = ct.c_void_p
    L.SUNContext_Create.argtypes = [ct.c_int, ct.POINTER(vp)]
    L.N_VMake_Serial.restype = vp
    L.N_VMake_Serial.argtypes = [ct.c_int64, P, vp]
    for nm, res, args in [
        ("N_VLinearSum", None, [ct.c_double, vp, ct.c_double, vp, vp]),
        ("N_VProd", None, [vp, vp, vp]), ("N_VDiv", None, [vp, vp, vp]),
        ("N_VScale", None, [ct.c_double, vp, vp]), ("N_VInv", None, [vp, vp]),
        ("N_VAddConst", None, [vp, ct.c_double, vp]), ("N_VCompare", None, [ct.c_double, vp, vp]),
        ("N_VDotProd", ct.c_double, [vp, vp]), ("N_VMaxNorm", ct.c_double, [vp]),
        ("N_VWrmsNorm", ct.c_double, [vp, vp]), ("N_VWrmsNormMask", ct.c_double, [vp, vp, vp]),
        ("N_VMin", ct.c_double, [vp]), ("N_VWL2Norm", ct.c_double, [vp, vp]),
        ("N_VL1Norm", ct.c_double, [vp]), ("N_VInvTest", ct.c_int, [vp, vp]),
        ("N_VConstrMask", ct.c_int, [vp, vp, vp]), ("N_VMinQuotient", ct.c_double, [vp, vp]),
        ("N_VLinearCombination", ct.c_int, [ct.c_int, P, ct.POINTER(vp), vp]),
        ("N_VScaleAddMulti", ct.c_int, [ct.c_int, P, vp, ct.POINTER(vp), ct.POINTER(vp)]),
        ("N_VDotProdMulti", ct.c_int, [ct.c_int, vp, ct.POINTER(vp), P]),
        ("N_VEnableFusedOps_Serial", ct.c_int, [vp, ct.c_int]),
    ]:
        f = getattr(L, nm)
        f.restype = res
        f.argtypes = args
    ctx = vp()
    assert L.SUNContext_Create(0, ct.byref(ctx)) == 0
    keep = []

    def mk(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        v = L.N_VMake_Serial(a.size, a.ctypes.data_as(P), ctx)
        L.N_VEnableFusedOps_Serial(v, 1)
        return v, a

    out = {}
    rng = np.random.default_rng(20251204)
    for n in (1, 7, 1000):
        x = rng.uniform(-1, 1, n)
        y = rng.uniform(-1, 1, n)
        y[::7] += 2.0
        w = 1.0 / (1e-6 * np.abs(y) + 1e-10) * 1e-8
        idm = (rng.uniform(-1, 1, n) > 0).astype(np.float64)
        xz = x.copy()
        xz[::5] = 0.0
        cc = rng.choice([-2.0, -1.0, 0.0, 1.0, 2.0], n)
        xs5 = [rng.uniform(-1, 1, n) for _ in range(5)]
        c5 = rng.uniform(-1, 1, 5)
        for k, v in dict(x=x, y=y, w=w, id=idm, xz=xz, cc=cc, c5=c5).items():
            out[f"n{n}_in_{k}"] = v
        for k in range(5):
            out[f"n{n}_in_xs{k}"] = xs5[k]
        X, _ = mk(x)
        Y, _ = mk(y)
        W, _ = mk(w)
        ID, _ = mk(idm)
        Z, z = mk(np.zeros(n))
        for j, (a, b) in enumerate([(1, 1), (1, -1), (-1, 1), (1, 2.5), (0.3, 1), (-1, 0.7),
                                    (0.3, -1), (2.5, 2.5), (2.5, -2.5), (0.3, 0.7)]):
            L.N_VLinearSum(a, X, b, Y, Z)
            out[f"n{n}_linearsum{j}"] = z.copy()
        L.N_VProd(X, Y, Z); out[f"n{n}_prod"] = z.copy()
        L.N_VDiv(X, Y, Z); out[f"n{n}_div"] = z.copy()
        L.N_VScale(2.5, X, Z); out[f"n{n}_scale"] = z.copy()
        L.N_VInv(Y, Z); out[f"n{n}_inv"] = z.copy()
        L.N_VAddConst(X, -0.75, Z); out[f"n{n}_addconst"] = z.copy()
        L.N_VCompare(0.5, X, Z); out[f"n{n}_compare"] = z.copy()
        out[f"n{n}_dotprod"] = np.array([L.N_VDotProd(X, Y)])
        out[f"n{n}_maxnorm"] = np.array([L.N_VMaxNorm(X)])
        out[f"n{n}_wrmsnorm"] = np.array([L.N_VWrmsNorm(X, W)])
        out[f"n{n}_wrmsnormmask"] = np.array([L.N_VWrmsNormMask(X, W, ID)])
        out[f"n{n}_min"] = np.array([L.N_VMin(X)])
        out[f"n{n}_wl2norm"] = np.array([L.N_VWL2Norm(X, W)])
        out[f"n{n}_l1norm"] = np.array([L.N_VL1Norm(X)])
        out[f"n{n}_minquotient"] = np.array([L.N_VMinQuotient(X, Y)])
        XZ, _ = mk(xz)
        Zi, zi = mk(np.full(n, 7.0))
        out[f"n{n}_invtest_flag"] = np.array([L.N_VInvTest(XZ, Zi)], dtype=np.float64)
        out[f"n{n}_invtest"] = zi.copy()
        CC, _ = mk(cc)
        M, m = mk(np.zeros(n))
        out[f"n{n}_constrmask_flag"] = np.array([L.N_VConstrMask(CC, X, M)], dtype=np.float64)
        out[f"n{n}_constrmask"] = m.copy()
        Xs = [mk(a)[0] for a in xs5]
        arr = (vp * 5)(*Xs)
        L.N_VLinearCombination(5, c5.ctypes.data_as(P), arr, Z)
        out[f"n{n}_lincomb5"] = z.copy()
        Zs = [mk(np.zeros(n)) for _ in range(5)]
        L.N_VScaleAddMulti(5, c5.ctypes.data_as(P), X, arr, (vp * 5)(*[v for v, _ in Zs]))
        for k in range(5):
            out[f"n{n}_scaleaddmulti{k}"] = Zs[k][1].copy()
        d = np.zeros(5)
        L.N_VDotProdMulti(5, X, arr, d.ctypes.data_as(P))
        out[f"n{n}_dotprodmulti5"] = d
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({len(out)} arrays)")


if __name__ == "__main__":
    sys.exit(main())

"""Generate tests/golden/spgmr_ref.npz from the reference itself: SPGMR solves
by SUNLinSol_SPGMR (src/sunlinsol/spgmr/sunlinsol_spgmr.c) over NVECTOR_SERIAL
from oracle/_ref/libsundials_ref.so, on the problem family of the reference's
unit test (test/unit_tests/sunlinsol/spgmr/serial/test_sunlinsol_spgmr_serial.c):
A = S1^{-1} T S2 with T tridiagonal, Jacobi preconditioner P^{-1} r = r / diag,
exact solution x = xhat / s2.  ATimes / PSolve are numpy callbacks rounded
like the unit test's C versions (oracle/spgmr_port.py:tridiag_apply).

Each case stores the inputs it needs (seeded vectors), the reference's flag,
iteration count, residual norm and solution.  A case is only kept if the
numpy port (oracle/spgmr_port.py) shows the residual norm of every iteration
at least 1% away from the tolerance, so the iteration count is not decided
by the last bit of a dot product.

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_spgmr_golden.py
"""
import ctypes as ct
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import spgmr_port as sp  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "libsundials_ref.so"
OUT = Path(__file__).resolve().parent / "spgmr_ref.npz"

# name, gstype, pretype, s1, s2, maxl, maxrs, (diag, lo, hi), n, delta, zeroguess
CASES = [
    ("mgs_none", 1, 0, False, False, 20, 0, (5.0, -1.0, -1.0), 1000, 1e-9, True),
    ("cgs_none", 2, 0, False, False, 20, 0, (5.0, -1.0, -1.0), 1000, 1e-9, True),
    ("mgs_left", 1, 1, False, False, 20, 0, (5.0, -1.0, -1.0), 1000, 1e-9, False),
    ("cgs_right", 2, 2, False, False, 20, 0, (5.0, -1.0, -1.0), 1000, 1e-9, True),
    ("cgs_both_s1s2", 2, 3, True, True, 20, 0, (5.0, -1.0, -1.0), 1000, 1e-9, False),
    ("mgs_right_s2", 1, 2, False, True, 20, 0, (5.0, -1.0, -1.0), 1000, 1e-9, True),
    ("mgs_left_s1", 1, 1, True, False, 20, 0, (5.0, -1.0, -1.0), 1000, 1e-9, True),
    ("cgs_restart", 2, 0, False, False, 5, 6, (2.2, -1.0, -0.8), 3001, 1e-8, True),
    ("mgs_restart_left", 1, 1, False, False, 5, 4, (2.2, -1.0, -0.8), 3001, 1e-8, False),
    ("cgs_res_reduced", 2, 0, False, False, 3, 1, (2.05, -1.0, -1.0), 2000, 1e-12, True),
    ("mgs_conv_fail", 1, 0, False, False, 1, 0, (0.0, -1.0, 1.0), 500, 1e-12, True),
    ("cgs_conv_fail", 2, 0, False, False, 1, 0, (0.0, -1.0, 1.0), 500, 1e-12, True),
    ("mgs_exact_guess", 1, 1, False, False, 5, 0, (5.0, -1.0, -1.0), 257, 1e-9, False),
    ("cgs_maxl12", 2, 1, True, True, 12, 2, (3.0, -1.0, -0.9), 4099, 1e-10, False),
]


def case_inputs(i, n, s1_on, s2_on):
    rng = np.random.default_rng(1000 + i)
    xhat = 1.0 + rng.uniform(0.0, 1.0, n)
    s1 = 1.0 + 1000.0 * rng.uniform(0.0, 1.0, n) if s1_on else np.ones(n)
    s2 = 1.0 + 1000.0 * rng.uniform(0.0, 1.0, n) if s2_on else np.ones(n)
    x0 = rng.uniform(-1.0, 1.0, n) / s2
    return xhat, s1, s2, x0


def main():
    L = ct.CDLL(str(REF))
    vp, i64, d, ci = ct.c_void_p, ct.c_int64, ct.c_double, ct.c_int
    sig = {
        "SUNContext_Create": (ci, [ci, ct.POINTER(vp)]),
        "SUNContext_Free": (ci, [ct.POINTER(vp)]),
        "N_VNew_Serial": (vp, [i64, vp]),
        "N_VGetArrayPointer": (ct.POINTER(d), [vp]),
        "N_VDestroy": (None, [vp]),
        "SUNLinSol_SPGMR": (vp, [vp, ci, ci, vp]),
        "SUNLinSol_SPGMRSetGSType": (ci, [vp, ci]),
        "SUNLinSol_SPGMRSetMaxRestarts": (ci, [vp, ci]),
        "SUNLinSolSetATimes": (ci, [vp, vp, vp]),
        "SUNLinSolSetPreconditioner": (ci, [vp, vp, vp, vp]),
        "SUNLinSolSetScalingVectors": (ci, [vp, vp, vp]),
        "SUNLinSolSetZeroGuess": (ci, [vp, ci]),
        "SUNLinSolInitialize": (ci, [vp]),
        "SUNLinSolSetup": (ci, [vp, vp]),
        "SUNLinSolSolve": (ci, [vp, vp, vp, vp, d]),
        "SUNLinSolNumIters": (ci, [vp]),
        "SUNLinSolResNorm": (d, [vp]),
        "SUNLinSolLastFlag": (i64, [vp]),
        "SUNLinSolFree": (ci, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    ATIMES = ct.CFUNCTYPE(ci, vp, vp, vp)
    PSOLVE = ct.CFUNCTYPE(ci, vp, vp, vp, d, ci)

    ctx = vp()
    assert L.SUNContext_Create(0, ct.byref(ctx)) == 0

    def arr(v, n):
        return np.ctypeslib.as_array(L.N_VGetArrayPointer(v), shape=(n,))

    out = {"names": np.array([c[0] for c in CASES])}
    for i, (name, gs, pre, s1_on, s2_on, maxl, maxrs, (dg, lo, hi), n, delta, zg) in enumerate(CASES):
        xhat, s1, s2, x0 = case_inputs(i, n, s1_on, s2_on)
        xtrue = xhat / s2
        b = sp.tridiag_apply(xtrue, s1, s2, dg, lo, hi)
        if name == "mgs_exact_guess":
            x0 = xtrue.copy()
        # numpy port: margins of the convergence test
        def at_np(v):
            return sp.tridiag_apply(v, s1, s2, dg, lo, hi)

        def ps_np(r, lr):
            return r / dg
        pflag, px, pnli, pres, hist = sp.spgmr_solve(
            at_np, ps_np, np.zeros(n) if zg else x0, b, delta, maxl=maxl, max_restarts=maxrs,
            gstype=gs, pretype=pre, s1=s1 if s1_on else None, s2=s2 if s2_on else None,
            zeroguess=zg)
        margin = min([abs(h / delta - 1.0) for h in hist], default=1.0)
        assert margin > 0.01, (name, margin)

        vx, vb, vs1, vs2 = (L.N_VNew_Serial(n, ctx) for _ in range(4))
        arr(vb, n)[:] = b
        arr(vs1, n)[:] = s1
        arr(vs2, n)[:] = s2
        arr(vx, n)[:] = 0.0 if zg else x0

        @ATIMES
        def atimes(data, v, z):
            arr(z, n)[:] = at_np(arr(v, n).copy())
            return 0

        @PSOLVE
        def psolve(data, r, z, tol, lr):
            arr(z, n)[:] = arr(r, n) / dg
            return 0

        LS = L.SUNLinSol_SPGMR(vx, pre, maxl, ctx)
        assert L.SUNLinSol_SPGMRSetGSType(LS, gs) == 0
        assert L.SUNLinSol_SPGMRSetMaxRestarts(LS, maxrs) == 0
        assert L.SUNLinSolSetATimes(LS, None, ct.cast(atimes, vp)) == 0
        assert L.SUNLinSolSetPreconditioner(LS, None, None, ct.cast(psolve, vp)) == 0
        assert L.SUNLinSolSetScalingVectors(LS, vs1 if s1_on else None, vs2 if s2_on else None) == 0
        assert L.SUNLinSolInitialize(LS) == 0
        assert L.SUNLinSolSetup(LS, None) == 0
        assert L.SUNLinSolSetZeroGuess(LS, 1 if zg else 0) == 0
        flag = L.SUNLinSolSolve(LS, None, vx, vb, delta)
        nli = L.SUNLinSolNumIters(LS)
        res = L.SUNLinSolResNorm(LS)
        lastflag = L.SUNLinSolLastFlag(LS)
        xs = arr(vx, n).copy()
        assert lastflag == flag
        print(f"{name:18s} n={n:5d} flag={flag:4d} nli={nli:3d} res={res:.3e} "
              f"port: flag={pflag} nli={pnli} margin={margin:.3f} "
              f"|x-xport|={np.max(np.abs(xs - px)):.2e}")
        out[f"{name}_flag"] = np.array([flag])
        out[f"{name}_nli"] = np.array([nli])
        out[f"{name}_resnorm"] = np.array([res])
        out[f"{name}_x"] = xs
        out[f"{name}_x0"] = x0 if not zg else np.zeros(n)
        out[f"{name}_b"] = b
        out[f"{name}_s1"] = s1
        out[f"{name}_s2"] = s2
        out[f"{name}_params"] = np.array([gs, pre, int(s1_on), int(s2_on), maxl, maxrs, n, int(zg)],
                                         dtype=np.int64)
        out[f"{name}_op"] = np.array([dg, lo, hi, delta])
        L.SUNLinSolFree(LS)
        for v in (vx, vb, vs1, vs2):
            L.N_VDestroy(v)
    L.SUNContext_Free(ct.byref(ctx))
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()

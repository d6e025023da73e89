"""Generate tests/golden/heat_cvode_ref.npz from the reference itself: the
reference's CVode (src/cvode/cvode.c) with NVECTOR_SERIAL and SUNLINSOL_SPGMR
from oracle/_ref/libsundials_ref.so on the 2-D heat problem of
examples/cvode/CXX_serial/cv_heat2D.cpp (no forcing term; BDF, Newton, SPGMR
with left Jacobi preconditioning, maxl 5, user J v), u0 = sin(pi x) sin(pi y)
+ U(-1e-3, 1e-3) (seed 1).  Per case: u0, the output times, the counters
after each output (oracle/heat_cvode.py:COUNTER_NAMES), hu / h / tn / h0u and
the solutions; and the reference's own sensitivity to the summation order of
its reductions: the same runs on NVECTOR_OPENMP with 2, 3, 4, 6, 8 and 16
threads (counters after the last output, and the largest weighted RMS
distance of their solutions from the serial ones, in units of the error
tolerance).  OpenMP combines its per-thread partial sums in an order that may
change from run to run, so these rows are a sample of that sensitivity, not
values to reproduce.

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_heat_cvode_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import heat_cvode as hc  # noqa: E402

OUT = Path(__file__).resolve().parent / "heat_cvode_ref.npz"
THREADS = (2, 3, 4, 6, 8, 16)

# name: (nx, ny, rtol, atol, output times)
CASES = {
    "g32": (32, 32, 1e-6, 1e-10, [0.01 * k for k in range(1, 11)]),
    "g128": (128, 128, 1e-6, 1e-10, [0.1]),
    "g48x32_tight": (48, 32, 1e-8, 1e-12, [0.02, 0.05, 0.1]),
}


def main():
    out = {}
    for name, (nx, ny, rtol, atol, touts) in CASES.items():
        c, r, s, u0 = hc.run_reference(nx, ny, touts, rtol, atol)
        out[f"{name}_grid"] = np.array([nx, ny])
        out[f"{name}_tol"] = np.array([rtol, atol])
        out[f"{name}_touts"] = np.array(touts)
        out[f"{name}_u0"] = u0
        out[f"{name}_counters"] = c
        out[f"{name}_reals"] = r
        out[f"{name}_y"] = s
        print(name, dict(zip(hc.COUNTER_NAMES, c[-1].tolist())))
        oc, ow = [], []
        for th in THREADS:
            c2, _, s2, _ = hc.run_reference(nx, ny, touts, rtol, atol, threads=th)
            w = 1.0 / (rtol * np.abs(s) + atol)
            oc.append(c2[-1])
            ow.append(float(np.sqrt(np.mean(((s2 - s) * w) ** 2, axis=1)).max()))
        out[f"{name}_omp_threads"] = np.array(THREADS)
        out[f"{name}_omp_counters"] = np.array(oc, np.int64)
        out[f"{name}_omp_wrms"] = np.array(ow)
        print("   order sensitivity:", {n: (int(np.min(np.array(oc)[:, k] - c[-1][k])),
                                            int(np.max(np.array(oc)[:, k] - c[-1][k])))
                                        for k, n in enumerate(hc.COUNTER_NAMES)},
              "wrms", max(ow))
    np.savez_compressed(OUT, names=np.array(list(CASES)), **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()

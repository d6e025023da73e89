"""Generate tests/golden/robertson_cvode_ref.npz from the reference itself:
the reference's CVode (src/cvode/cvode.c) with NVECTOR_SERIAL and
SUNLINSOL_SPGMR from oracle/_ref/libsundials_ref.so on the batched Robertson
problem of oracle/robertson_cvode.py (cells with k = (0.04, 3e7, 1e4) x
exp(0.1 z), y0 = (1, 0, 0), rtol 1e-4 and the per-species absolute
tolerances 1e-8 / 1e-14 / 1e-6 of cvRoberts_block_cusolversp_batchqr.cu,
outputs 0.4 * 10^k for k = 0..11; SPGMR with left preconditioning, maxl 5,
the user J v and the exact block-Jacobi preconditioner of cvDiurnal_kry.c;
the rd* cases: the example's own configuration, a direct solver on the
block-diagonal Newton matrix with the user Jacobian -- SUNDenseMatrix +
SUNLINSOL_DENSE on the CPU).
Per case: the rate constants, the counters after each output, hu / h / tn /
h0u, the solutions at the outputs listed in <case>_y_index, and the same runs on NVECTOR_OPENMP with 2, 3, 4, 6, 8 and 16 threads (a
sample of the reference's own sensitivity to the summation order of its
reductions: counters after the last output and the largest weighted RMS
distance of their solutions from the serial ones, in tolerance units).

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_robertson_cvode_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import heat_cvode as hc  # noqa: E402
from oracle import robertson_cvode as rc  # noqa: E402

OUT = Path(__file__).resolve().parent / "robertson_cvode_ref.npz"
THREADS = (2, 3, 4, 6, 8, 16)
# name: (cells, outputs whose solutions are stored, direct solver)
CASES = {"r256": (256, list(range(12)), False), "r1024": (1024, [5, 11], False),
         "rd256": (256, list(range(12)), True), "rd1024": (1024, [5, 11], True)}
RTOL = 1e-4


def main():
    out = {}
    for name, (ncells, keep, direct) in CASES.items():
        atol = rc.vector_atol(ncells)
        run = rc.run_reference_direct if direct else rc.run_reference
        c, r, s = run(ncells, rc.TOUTS, RTOL, atol)
        out[f"{name}_k"] = rc.rates(ncells)
        out[f"{name}_touts"] = np.array(rc.TOUTS)
        out[f"{name}_rtol"] = np.array(RTOL)
        out[f"{name}_counters"] = c
        out[f"{name}_reals"] = r
        out[f"{name}_y"] = s[keep]
        out[f"{name}_y_index"] = np.array(keep)
        print(name, dict(zip(hc.COUNTER_NAMES, c[-1].tolist())))
        oc, ow = [], []
        for th in THREADS:
            c2, _, s2 = run(ncells, rc.TOUTS, RTOL, atol, threads=th)
            w = 1.0 / (RTOL * np.abs(s) + atol)
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

"""Generate tests/golden/robertson_arkode_ref.npz from the reference itself:
the reference's ARKodeEvolve (src/arkode/arkode.c, ARKStep: DIRK of order 3,
Newton) with NVECTOR_SERIAL from oracle/_ref/libsundials_ref.so on the
batched Robertson problem of oracle/robertson_cvode.py (64 cells, rtol 1e-4,
per-species absolute tolerances 1e-8 / 1e-14 / 1e-6 through
ARKodeSVtolerances, outputs 0.4 * 10^k for k = 0..6), with the
matrix-based direct path of ARKLS -- ARKodeSetLinearSolver(LS, A) with
SUNDenseMatrix + SUNLINSOL_DENSE (whose LU of the block-diagonal Newton
matrix is the per-block LU) and the user Jacobian (ARKodeSetJacFn).  Stores
the Butcher table the run used, the counters after each output
(oracle/arkstep.py COUNTER_NAMES), last / next step, time and first step,
the solution at the last output, and the same run on NVECTOR_OPENMP with 2,
3, 4, 6, 8 and 16 threads (a sample of the reference's own sensitivity to the
summation order of its reductions).  The ``prec_`` entries are the same
for ARKLS's iterative path: SPGMR (left, maxl 5) with the user J v and the
exact block-Jacobi preconditioner with its setup (ARKodeSetPreconditioner).
The outputs stop at t = 4e5: beyond
4e6 the reference's own DIRK runs of this problem part ways when only the
summation order changes (steps by up to ~300, solutions by up to thousands
of tolerances at 4e7-4e10), so they pin nothing.

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_robertson_arkode_golden.py
    (``--only prec_`` or ``--only direct`` regenerates one configuration's
    entries and keeps the other's, its reduction-order sample included)
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import arkstep as ak  # noqa: E402
from oracle import robertson_cvode as rc  # noqa: E402

OUT = Path(__file__).resolve().parent / "robertson_arkode_ref.npz"
THREADS = (2, 3, 4, 6, 8, 16)
CELLS = 64
RTOL = 1e-4
TOUTS = rc.TOUTS[:7]


def run(out, prefix, runner):
    c, r, s, tables = runner(CELLS, touts=TOUTS)
    out.update({prefix + "counters": c, prefix + "reals": r, prefix + "y_last": s[-1],
                **ak.tables_to_dict(tables, prefix)})
    print(prefix or "direct", dict(zip(ak.COUNTER_NAMES, c[-1].tolist())))
    oc, ow = [], []
    w = 1.0 / (RTOL * np.abs(s) + rc.vector_atol(CELLS))
    for th in THREADS:
        c2, _, s2, _ = runner(CELLS, touts=TOUTS, threads=th)
        oc.append(c2[-1])
        ow.append(float(np.sqrt(np.mean(((s2 - s) * w) ** 2, axis=1)).max()))
    out[prefix + "omp_counters"] = np.array(oc, np.int64)
    out[prefix + "omp_wrms"] = np.array(ow)
    print("  order sensitivity:", (np.array(oc) - c[-1]).min(axis=0).tolist(),
          (np.array(oc) - c[-1]).max(axis=0).tolist(), "wrms", max(ow))


def main(only=None):
    out = {"cells": np.array(CELLS), "k": rc.rates(CELLS), "touts": np.array(TOUTS),
           "rtol": np.array(RTOL), "atol": rc.vector_atol(CELLS), "u0": rc.initial(CELLS),
           "omp_threads": np.array(THREADS)}
    if only:
        old = np.load(OUT)
        keep = (lambda k: not k.startswith("prec_")) if only == "prec_" else \
            (lambda k: k.startswith("prec_"))
        out.update({k: old[k] for k in old.files if keep(k) and k not in out})
    if only in (None, "direct"):
        run(out, "", rc.run_reference_arkode_direct)
    if only in (None, "prec_"):
        run(out, "prec_", rc.run_reference_arkode)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[2] if len(sys.argv) > 2 and sys.argv[1] == "--only" else None)

"""Generate tests/golden/bruss3d_arkode_ref.npz from the reference itself: the
reference's ARKodeEvolve (src/arkode/arkode.c, ARKStep) with NVECTOR_SERIAL
and SUNLINSOL_SPGMR from oracle/_ref/libsundials_ref.so, configured as the
3-D advection-reaction benchmark's default ARK-DIRK driver
(benchmarks/advection_reaction_3D/raja/arkode_driver.cpp:51-160: implicit
right-hand side = advection + reaction, order 3, Newton, SPGMR with left
preconditioning and the default maxl, the difference-quotient J v, PSolve =
the per-cell reaction solve), on the benchmark's defaults (rtol 1e-6, atol
1e-9, t in [0, 10], 10 outputs, c = 0.01) on a 16^3 grid, with the user
functions of oracle/bruss3d_cvode.py.  Stores u0, the Butcher table the run
used (read from the reference's table object), the counters after every
output (oracle/arkode_dirk.py COUNTER_NAMES), last / next step, time and
first step, the solution at the last output, and the same run on
NVECTOR_OPENMP with 2, 3, 4, 6, 8 and 16 threads (a sample of the
reference's own sensitivity to the summation order of its reductions).

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_bruss3d_arkode_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import arkode_dirk as ad  # noqa: E402
from oracle import bruss3d_cvode as bc  # noqa: E402

OUT = Path(__file__).resolve().parent / "bruss3d_arkode_ref.npz"
THREADS = (2, 3, 4, 6, 8, 16)
NPTS = 16


def main():
    q = bc.Params(NPTS, NPTS, NPTS)
    c, r, s, table = bc.run_reference_arkode(q)
    out = {"grid": np.array([NPTS] * 3), "touts": np.array(q.touts),
           "tol": np.array([q.rtol, q.atol]), "u0": bc.initial(q), "counters": c, "reals": r,
           "y_last": s[-1], **{"table_" + k: v for k, v in table.items()}}
    print(dict(zip(ad.COUNTER_NAMES, c[-1].tolist())))
    oc, ow = [], []
    for th in THREADS:
        c2, _, s2, _ = bc.run_reference_arkode(q, threads=th)
        w = 1.0 / (q.rtol * np.abs(s) + q.atol)
        oc.append(c2[-1])
        ow.append(float(np.sqrt(np.mean(((s2 - s) * w) ** 2, axis=1)).max()))
    out["omp_threads"] = np.array(THREADS)
    out["omp_counters"] = np.array(oc, np.int64)
    out["omp_wrms"] = np.array(ow)
    print("order sensitivity:", {n: (int(np.min(np.array(oc)[:, k] - c[-1][k])),
                                     int(np.max(np.array(oc)[:, k] - c[-1][k])))
                                 for k, n in enumerate(ad.COUNTER_NAMES)}, "wrms", max(ow))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()

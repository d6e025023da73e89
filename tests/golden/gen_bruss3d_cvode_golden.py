"""Generate tests/golden/bruss3d_cvode_ref.npz from the reference itself: the
reference's CVode (src/cvode/cvode.c) with NVECTOR_SERIAL and SUNLINSOL_SPGMR
from oracle/_ref/libsundials_ref.so, configured as the 3-D advection-reaction
benchmark's CVODE driver (benchmarks/advection_reaction_3D/raja/
cvode_driver.cpp: BDF, Newton, SPGMR with left preconditioning, the
difference-quotient J v, PSolve = the per-cell reaction solve), on its
defaults (rtol 1e-6, atol 1e-9, t in [0, 10], 10 outputs, c = 0.01, A = 1,
B = 3.5, k5 = k6 = 2e5) on a 16^3 grid, with the user functions of
oracle/bruss3d_cvode.py.  Stores u0 (its exp / pow are the host's), the
counters after every output, hu / h / tn / h0u, the solution at the last
output, and the same run on NVECTOR_OPENMP with 2, 3, 4, 6, 8 and 16 threads
(a sample of the reference's own sensitivity to the summation order of its
reductions).  The ``fp_`` entries are the same for the driver's
``--nls fixedpoint`` variant (SUNNonlinSol_FixedPoint, Anderson depth
``--fpaccel`` 3, no linear solver), and the ``adams_`` entries those of its
CV-ADAMS configuration (Adams-Moulton, always with that fixed-point solver),
whose steps the stiff reaction holds near 5e-6: over ``--tf 0.01 --nout 2``
(their own ``adams_touts``).

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_bruss3d_cvode_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import bruss3d_cvode as bc  # noqa: E402
from oracle import heat_cvode as hc  # noqa: E402

OUT = Path(__file__).resolve().parent / "bruss3d_cvode_ref.npz"
THREADS = (2, 3, 4, 6, 8, 16)
NPTS = 16


def main():
    q = bc.Params(NPTS, NPTS, NPTS)
    c, r, s = bc.run_reference(q)
    out = {"grid": np.array([NPTS] * 3), "touts": np.array(q.touts),
           "tol": np.array([q.rtol, q.atol]), "u0": bc.initial(q), "counters": c, "reals": r,
           "y_last": s[-1]}
    print(dict(zip(hc.COUNTER_NAMES, c[-1].tolist())))
    oc, ow = [], []
    for th in THREADS:
        c2, _, s2 = bc.run_reference(q, threads=th)
        w = 1.0 / (q.rtol * np.abs(s) + q.atol)
        oc.append(c2[-1])
        ow.append(float(np.sqrt(np.mean(((s2 - s) * w) ** 2, axis=1)).max()))
    out["omp_threads"] = np.array(THREADS)
    out["omp_counters"] = np.array(oc, np.int64)
    out["omp_wrms"] = np.array(ow)
    c, r, s = bc.run_reference(q, fixed_point=3)
    out.update({"fp_counters": c, "fp_reals": r, "fp_y_last": s[-1]})
    print("fixed point:", dict(zip(hc.COUNTER_NAMES, c[-1].tolist())))
    oc, ow = [], []
    for th in THREADS:
        c2, _, s2 = bc.run_reference(q, threads=th, fixed_point=3)
        w = 1.0 / (q.rtol * np.abs(s) + q.atol)
        oc.append(c2[-1])
        ow.append(float(np.sqrt(np.mean(((s2 - s) * w) ** 2, axis=1)).max()))
    out["fp_omp_counters"] = np.array(oc, np.int64)
    out["fp_omp_wrms"] = np.array(ow)
    print("  order sensitivity:", (np.array(oc) - c[-1]).min(axis=0).tolist(),
          (np.array(oc) - c[-1]).max(axis=0).tolist(), "wrms", max(ow))
    qa = bc.Params(NPTS, NPTS, NPTS, tf=0.01, nout=2)
    c, r, s = bc.run_reference(qa, fixed_point=3, adams=True)
    out.update({"adams_touts": np.array(qa.touts), "adams_counters": c, "adams_reals": r,
                "adams_y_last": s[-1]})
    print("adams:", dict(zip(hc.COUNTER_NAMES, c[-1].tolist())))
    oc, ow = [], []
    for th in THREADS:
        c2, _, s2 = bc.run_reference(qa, threads=th, fixed_point=3, adams=True)
        w = 1.0 / (qa.rtol * np.abs(s) + qa.atol)
        oc.append(c2[-1])
        ow.append(float(np.sqrt(np.mean(((s2 - s) * w) ** 2, axis=1)).max()))
    out["adams_omp_counters"] = np.array(oc, np.int64)
    out["adams_omp_wrms"] = np.array(ow)
    print("  order sensitivity:", (np.array(oc) - c[-1]).min(axis=0).tolist(),
          (np.array(oc) - c[-1]).max(axis=0).tolist(), "wrms", max(ow))
    print("order sensitivity:", {n: (int(np.min(np.array(oc)[:, k] - c[-1][k])),
                                     int(np.max(np.array(oc)[:, k] - c[-1][k])))
                                 for k, n in enumerate(hc.COUNTER_NAMES)}, "wrms", max(ow))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()

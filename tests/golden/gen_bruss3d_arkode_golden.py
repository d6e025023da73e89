"""Generate tests/golden/bruss3d_arkode_ref.npz from the reference itself: the
reference's ARKodeEvolve (src/arkode/arkode.c, ARKStep) with NVECTOR_SERIAL
and SUNLINSOL_SPGMR from oracle/_ref/libsundials_ref.so, configured as the
3-D advection-reaction benchmark's ARKODE drivers
(benchmarks/advection_reaction_3D/raja/arkode_driver.cpp):

* ``dirk_``: ARK-DIRK, the benchmark's default (51-160): implicit
  right-hand side = advection + reaction;
* ``imex_``: ARK-IMEX (239-370): explicit advection, implicit reaction;

both at order 3 with Newton, SPGMR (left preconditioning, default maxl), the
difference-quotient J v and PSolve = the per-cell reaction solve; and

* ``tl_``: ARK-IMEX with ``--nls tl-newton``: the benchmark's TaskLocalNewton
  (546-780) on one task -- the reference's Newton with the per-cell reaction
  solve as its linear solve and no SUNLinearSolver (the wrapper restated in
  oracle/arkstep.py around the reference's own SUNNonlinSol_Newton: the
  reference's build here has no MPI for the MPIPlusX vector it requires);
* ``erk_``: the ERK configuration (ERKStep, 441-540, order 3), explicit on
  the stiff reaction, so stability holds its steps near 1e-5: over
  ``--tf 0.01 --nout 2`` (its own ``touts``);
* ``fpdirk_`` / ``fpimex_``: ARK-DIRK / ARK-IMEX with ``--nls fixedpoint``
  (SUNNonlinSol_FixedPoint, Anderson depth 3, no linear solver), whose steps
  the stiff reaction limits to ~1e-5: over ``--tf 0.01 --nout 2`` (their own
  ``touts``);

on the benchmark's defaults (rtol 1e-6, atol 1e-9, t in [0, 10], 10 outputs,
c = 0.01) on a 16^3 grid, with the user functions of
oracle/bruss3d_cvode.py.  Stores u0, the Butcher tables each run used (read
from the reference's table objects), the counters after every output
(oracle/arkstep.py COUNTER_NAMES), last / next step, time and first step, the
solution at the last output, and the same runs on NVECTOR_OPENMP with 2, 3,
4, 6, 8 and 16 threads (a sample of the reference's own sensitivity to the
summation order of its reductions).

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_bruss3d_arkode_golden.py
    (``--only erk_`` regenerates one configuration's entries and keeps the
    file's others, their reduction-order samples included)
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import arkstep as ak  # noqa: E402
from oracle import bruss3d_cvode as bc  # noqa: E402

OUT = Path(__file__).resolve().parent / "bruss3d_arkode_ref.npz"
THREADS = (2, 3, 4, 6, 8, 16)
NPTS = 16


CONFIGS = (("dirk_", False, False, None, False), ("imex_", True, False, None, False),
           ("tl_", True, True, None, False), ("erk_", False, False, None, True),
           ("fpdirk_", False, False, 3, False), ("fpimex_", True, False, 3, False))


def main(only=None):
    q = bc.Params(NPTS, NPTS, NPTS)
    out = {"grid": np.array([NPTS] * 3), "touts": np.array(q.touts),
           "tol": np.array([q.rtol, q.atol]), "u0": bc.initial(q),
           "omp_threads": np.array(THREADS)}
    if only:
        old = np.load(OUT)
        out = {k: old[k] for k in old.files if not k.startswith(only)}
    qshort = bc.Params(NPTS, NPTS, NPTS, tf=0.01, nout=2)
    for name, imex, tl, fp, erk in CONFIGS:
        if only and name != only:
            continue
        qq = qshort if (fp or erk) else q
        if fp or erk:
            out[name + "touts"] = np.array(qq.touts)
        c, r, s, tables = bc.run_reference_arkode(qq, imex=imex, task_local=tl, fixed_point=fp,
                                                  erk=erk)
        out.update({name + "counters": c, name + "reals": r, name + "y_last": s[-1],
                    **ak.tables_to_dict(tables, name)})
        print(name, dict(zip(ak.COUNTER_NAMES, c[-1].tolist())))
        oc, ow = [], []
        for th in THREADS:
            c2, _, s2, _ = bc.run_reference_arkode(qq, threads=th, imex=imex, task_local=tl,
                                                   fixed_point=fp, erk=erk)
            w = 1.0 / (q.rtol * np.abs(s) + q.atol)
            oc.append(c2[-1])
            ow.append(float(np.sqrt(np.mean(((s2 - s) * w) ** 2, axis=1)).max()))
        out[name + "omp_counters"] = np.array(oc, np.int64)
        out[name + "omp_wrms"] = np.array(ow)
        print("  order sensitivity:", {n: (int(np.min(np.array(oc)[:, k] - c[-1][k])),
                                           int(np.max(np.array(oc)[:, k] - c[-1][k])))
                                       for k, n in enumerate(ak.COUNTER_NAMES)}, "wrms", max(ow))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[2] if len(sys.argv) > 2 and sys.argv[1] == "--only" else None)

"""Generate tests/golden/kinetics_cvode_ref.npz from the reference itself.

Systems 0, 64, 128, ... (1024 systems spread over the 65,536-system batch,
seed 1) and systems 0..255 at the looser tolerance rtol 1e-4 are integrated
by the reference's own CVODE (oracle/_ref/kinetics_cvode_ref, built from the
reference sources by oracle/Makefile): BDF, Newton, NVECTOR_SERIAL,
SUNLINSOL_DENSE, analytic Jacobian, one CVode(tout = 100, CV_NORMAL) call,
atol 1e-12, mxstep 10^6.  Stored: system ids, the counters and y(100).

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_kinetics_golden.py
"""
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from sundials_gb300 import kinetics as K  # noqa: E402

OUT = Path(__file__).resolve().parent / "kinetics_cvode_ref.npz"
DRIVER = ROOT / "oracle" / "_ref" / "kinetics_cvode_ref"


def run(batch, rtol, atol, tout):
    with tempfile.TemporaryDirectory() as d:
        p, o = Path(d) / "p.bin", Path(d) / "o.bin"
        K.write_bin(batch, p)
        subprocess.run([str(DRIVER), str(p), str(o), repr(rtol), repr(atol), repr(tout)],
                       check=True)
        return K.read_results(o, batch)


def main():
    full = K.generate(65536, seed=1)
    out = {}
    for tag, ids, rtol in [("r6", np.arange(0, 65536, 64), 1e-6), ("r4", np.arange(256), 1e-4)]:
        sub = full.subset(ids)
        st, ys = run(sub, rtol, 1e-12, 100.0)
        out[f"{tag}_ids"] = ids
        out[f"{tag}_rtol"] = np.array([rtol])
        for f in K.STATS_FIELDS + ["tn", "hu"]:
            out[f"{tag}_{f}"] = st[f]
        out[f"{tag}_y"] = np.concatenate(ys)
    # FP64 oracle solution of the rtol 1e-6 sample: the reference's CVODE at
    # rtol 1e-10, atol 1e-16 (errors of the rtol 1e-6 runs are measured
    # against it).
    sub = full.subset(out["r6_ids"])
    st, ys = run(sub, 1e-10, 1e-16, 100.0)
    assert np.all(st["flag"] == 0)
    out["truth_y"] = np.concatenate(ys)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()

"""Generate tests/golden/dense_lu.npz from the reference itself: LU factors,
pivots and solutions of SUNDlsMat_denseGETRF / SUNDlsMat_denseGETRS
(src/sundials/sundials_dense.c) from oracle/_ref/libsundials_ref.so on seeded
matrices of sizes 1, 3, 8, 17, 33 and 64, plus one singular matrix.

Usage (where the reference sources exist):
    python -m sundials_gb300.build && python tests/golden/gen_dense_golden.py
"""
import ctypes as ct
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
REF = ROOT / "oracle" / "_ref" / "libsundials_ref.so"
OUT = Path(__file__).resolve().parent / "dense_lu.npz"


def main():
    L = ct.CDLL(str(REF))
    PP = ct.POINTER(ct.POINTER(ct.c_double))
    L.SUNDlsMat_denseGETRF.restype = ct.c_int64
    L.SUNDlsMat_denseGETRF.argtypes = [PP, ct.c_int64, ct.c_int64, ct.POINTER(ct.c_int64)]
    L.SUNDlsMat_denseGETRS.argtypes = [PP, ct.c_int64, ct.POINTER(ct.c_int64),
                                       ct.POINTER(ct.c_double)]
    rng = np.random.default_rng(808)
    out = {}
    cases = [1, 3, 8, 17, 33, 64, "singular"]
    for c in cases:
        n = 5 if c == "singular" else c
        a = rng.uniform(-1, 1, (n, n))  # column-major storage: a[j] is column j
        if c == "singular":
            a[2] = a[0] * 2.0           # column 2 = 2 * column 0
        b = rng.uniform(-1, 1, n)
        cols = [np.ascontiguousarray(a[j].copy()) for j in range(n)]
        colp = (ct.POINTER(ct.c_double) * n)(*[x.ctypes.data_as(ct.POINTER(ct.c_double)) for x in cols])
        piv = np.zeros(n, np.int64)
        flag = L.SUNDlsMat_denseGETRF(colp, n, n, piv.ctypes.data_as(ct.POINTER(ct.c_int64)))
        x = b.copy()
        if flag == 0:
            L.SUNDlsMat_denseGETRS(colp, n, piv.ctypes.data_as(ct.POINTER(ct.c_int64)),
                                   x.ctypes.data_as(ct.POINTER(ct.c_double)))
        key = f"{c}"
        out[f"a_{key}"] = a
        out[f"b_{key}"] = b
        out[f"lu_{key}"] = np.stack(cols)
        out[f"piv_{key}"] = piv
        out[f"flag_{key}"] = np.array([flag])
        out[f"x_{key}"] = x
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()

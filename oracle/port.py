"""TEST ORACLE: ctypes access to ``oracle/_build/liboracle.so`` (the C
restatements of NVECTOR_SERIAL and friends).  Checker only."""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "liboracle.so"
_lib = None

_P = ct.POINTER(ct.c_double)
_I = ct.c_int64


def lib() -> ct.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from sundials_gb300.build import build_oracle
            build_oracle()
        _lib = ct.CDLL(str(LIB_PATH))
        d = ct.c_double
        sigs = {
            "port_linearsum": (None, [d, _P, d, _P, _P, _I]),
            "port_const": (None, [d, _P, _I]),
            "port_prod": (None, [_P, _P, _P, _I]),
            "port_div": (None, [_P, _P, _P, _I]),
            "port_scale": (None, [d, _P, _P, _I]),
            "port_abs": (None, [_P, _P, _I]),
            "port_inv": (None, [_P, _P, _I]),
            "port_addconst": (None, [_P, d, _P, _I]),
            "port_compare": (None, [d, _P, _P, _I]),
            "port_dotprod": (d, [_P, _P, _I]),
            "port_maxnorm": (d, [_P, _I]),
            "port_wsqrsum": (d, [_P, _P, _I]),
            "port_wsqrsummask": (d, [_P, _P, _P, _I]),
            "port_wrmsnorm": (d, [_P, _P, _I]),
            "port_wrmsnormmask": (d, [_P, _P, _P, _I]),
            "port_min": (d, [_P, _I]),
            "port_wl2norm": (d, [_P, _P, _I]),
            "port_l1norm": (d, [_P, _I]),
            "port_invtest": (ct.c_int, [_P, _P, _I]),
            "port_constrmask": (ct.c_int, [_P, _P, _P, _I]),
            "port_minquotient": (d, [_P, _P, _I]),
            "port_linearcombination": (None, [ct.c_int, _P, ct.POINTER(_P), _P, _I]),
            "port_scaleaddmulti": (None, [ct.c_int, _P, _P, ct.POINTER(_P), ct.POINTER(_P), _I]),
            "port_dotprodmulti": (None, [ct.c_int, _P, ct.POINTER(_P), _P, _I]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


def ptrs(arrs):
    arr = (_P * len(arrs))()
    for i, a in enumerate(arrs):
        arr[i] = ptr(a)
    return arr


def call(name, *args):
    return getattr(lib(), name)(*args)


def omp():
    """Multi-core timing variants (same arithmetic, NVECTOR_OPENMP-style sums)."""
    L = lib()
    d = ct.c_double
    for name, res, args in [
        ("omp_linearsum", None, [d, _P, d, _P, _P, _I]),
        ("omp_linearcombination", None, [ct.c_int, _P, ct.POINTER(_P), _P, _I]),
        ("omp_dotprodmulti", None, [ct.c_int, _P, ct.POINTER(_P), _P, _I]),
        ("omp_wrmsnorm", d, [_P, _P, _I]),
        ("omp_threads", ct.c_int, []),
    ]:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def bdf_batch(batch, rtol=1e-6, atol=1e-12, tout=100.0, mxstep=1000000, threads=0,
              first=0, count=None, dd_pow=False):
    """Run the CVODE restatement over systems [first, first+count) of a
    KineticsBatch; returns (stats structured array, yout flat array).
    dd_pow=True swaps the C library's pow for the correctly rounded one."""
    from sundials_gb300.kinetics import STATS_DTYPE
    L = lib()
    L.bdf_port_set_pow.argtypes = [ct.c_int]
    L.bdf_port_set_pow(1 if dd_pow else 0)
    if count is None:
        count = batch.nsys - first
    f = L.bdf_port_batch
    i32 = ct.POINTER(ct.c_int32)
    i64 = ct.POINTER(ct.c_int64)
    f.restype = None
    f.argtypes = [ct.c_int64, ct.c_int64, i32, i64, i64, i32, i32, i32, i32, _P, _P,
                  ct.c_double, ct.c_double, ct.c_double, ct.c_long, ct.c_int, _P, ct.c_void_p]
    c = lambda a, t: np.ascontiguousarray(a, dtype=t)
    n, yo, ro = c(batch.n, np.int32), c(batch.y_off, np.int64), c(batch.r_off, np.int64)
    rt, ra, rb, rc = (c(a, np.int32) for a in (batch.rtype, batch.ra, batch.rb, batch.rc))
    rk, y0 = c(batch.rk, np.float64), c(batch.y0, np.float64)
    yout = np.zeros_like(y0)
    stats = np.zeros(count, STATS_DTYPE)
    f(first, count, n.ctypes.data_as(i32), yo.ctypes.data_as(i64), ro.ctypes.data_as(i64),
      rt.ctypes.data_as(i32), ra.ctypes.data_as(i32), rb.ctypes.data_as(i32),
      rc.ctypes.data_as(i32), rk.ctypes.data_as(_P), y0.ctypes.data_as(_P), rtol, atol, tout,
      mxstep, threads, yout.ctypes.data_as(_P), stats.ctypes.data)
    L.bdf_port_set_pow(0)
    return stats, yout


def dense_lu(a_colmajor: np.ndarray):
    """(factors, pivots, flag) of the GETRF restatement; a is (n, n) with a[j] = column j."""
    L = lib()
    f = L.port_dense_getrf
    f.restype = ct.c_int
    f.argtypes = [_P, ct.c_int64, ct.POINTER(ct.c_int64)]
    n = a_colmajor.shape[0]
    lu = np.ascontiguousarray(a_colmajor, dtype=np.float64).copy()
    piv = np.zeros(n, np.int64)
    flag = f(lu.ctypes.data_as(_P), n, piv.ctypes.data_as(ct.POINTER(ct.c_int64)))
    return lu, piv, flag


def dense_solve(lu: np.ndarray, piv: np.ndarray, b: np.ndarray) -> np.ndarray:
    L = lib()
    f = L.port_dense_getrs
    f.restype = None
    f.argtypes = [_P, ct.c_int64, ct.POINTER(ct.c_int64), _P]
    x = np.ascontiguousarray(b, dtype=np.float64).copy()
    f(np.ascontiguousarray(lu).ctypes.data_as(_P), lu.shape[0],
      np.ascontiguousarray(piv, np.int64).ctypes.data_as(ct.POINTER(ct.c_int64)), x.ctypes.data_as(_P))
    return x

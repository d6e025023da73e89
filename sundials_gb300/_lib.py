"""ctypes view of the C ABI: loads ``lib/libsundials_gb300.so`` and mirrors the
SUNDIALS v7.5.0 object layouts (``include/sundials_gb300_abi.h``) so host code
and tests can call every operation through the ops table, exactly as CVODE's
generic dispatch does (``sundials_nvector.c:383-835``).

There is no fallback: if the library is missing, importing it raises.
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libsundials_gb300.so"

real = ct.c_double
idx = ct.c_int64
N_Vector = ct.c_void_p
P_real = ct.POINTER(ct.c_double)
P_NV = ct.POINTER(ct.c_void_p)

# (field name, restype, argtypes) in ABI order: sundials_nvector.h:101-195
NV_OPS_FIELDS = [
    ("nvgetvectorid", ct.c_int, [N_Vector]),
    ("nvclone", N_Vector, [N_Vector]),
    ("nvcloneempty", N_Vector, [N_Vector]),
    ("nvdestroy", None, [N_Vector]),
    ("nvspace", None, [N_Vector, ct.POINTER(idx), ct.POINTER(idx)]),
    ("nvgetarraypointer", P_real, [N_Vector]),
    ("nvgetdevicearraypointer", P_real, [N_Vector]),
    ("nvsetarraypointer", None, [P_real, N_Vector]),
    ("nvgetcommunicator", ct.c_int, [N_Vector]),
    ("nvgetlength", idx, [N_Vector]),
    ("nvgetlocallength", idx, [N_Vector]),
    ("nvlinearsum", None, [real, N_Vector, real, N_Vector, N_Vector]),
    ("nvconst", None, [real, N_Vector]),
    ("nvprod", None, [N_Vector, N_Vector, N_Vector]),
    ("nvdiv", None, [N_Vector, N_Vector, N_Vector]),
    ("nvscale", None, [real, N_Vector, N_Vector]),
    ("nvabs", None, [N_Vector, N_Vector]),
    ("nvinv", None, [N_Vector, N_Vector]),
    ("nvaddconst", None, [N_Vector, real, N_Vector]),
    ("nvdotprod", real, [N_Vector, N_Vector]),
    ("nvmaxnorm", real, [N_Vector]),
    ("nvwrmsnorm", real, [N_Vector, N_Vector]),
    ("nvwrmsnormmask", real, [N_Vector, N_Vector, N_Vector]),
    ("nvmin", real, [N_Vector]),
    ("nvwl2norm", real, [N_Vector, N_Vector]),
    ("nvl1norm", real, [N_Vector]),
    ("nvcompare", None, [real, N_Vector, N_Vector]),
    ("nvinvtest", ct.c_int, [N_Vector, N_Vector]),
    ("nvconstrmask", ct.c_int, [N_Vector, N_Vector, N_Vector]),
    ("nvminquotient", real, [N_Vector, N_Vector]),
    ("nvlinearcombination", ct.c_int, [ct.c_int, P_real, P_NV, N_Vector]),
    ("nvscaleaddmulti", ct.c_int, [ct.c_int, P_real, N_Vector, P_NV, P_NV]),
    ("nvdotprodmulti", ct.c_int, [ct.c_int, N_Vector, P_NV, P_real]),
    ("nvlinearsumvectorarray", ct.c_int, [ct.c_int, real, P_NV, real, P_NV, P_NV]),
    ("nvscalevectorarray", ct.c_int, [ct.c_int, P_real, P_NV, P_NV]),
    ("nvconstvectorarray", ct.c_int, [ct.c_int, real, P_NV]),
    ("nvwrmsnormvectorarray", ct.c_int, [ct.c_int, P_NV, P_NV, P_real]),
    ("nvwrmsnormmaskvectorarray", ct.c_int, [ct.c_int, P_NV, P_NV, N_Vector, P_real]),
    ("nvscaleaddmultivectorarray", ct.c_int,
     [ct.c_int, ct.c_int, P_real, P_NV, ct.POINTER(P_NV), ct.POINTER(P_NV)]),
    ("nvlinearcombinationvectorarray", ct.c_int,
     [ct.c_int, ct.c_int, P_real, ct.POINTER(P_NV), P_NV]),
    ("nvdotprodlocal", real, [N_Vector, N_Vector]),
    ("nvmaxnormlocal", real, [N_Vector]),
    ("nvminlocal", real, [N_Vector]),
    ("nvl1normlocal", real, [N_Vector]),
    ("nvinvtestlocal", ct.c_int, [N_Vector, N_Vector]),
    ("nvconstrmasklocal", ct.c_int, [N_Vector, N_Vector, N_Vector]),
    ("nvminquotientlocal", real, [N_Vector, N_Vector]),
    ("nvwsqrsumlocal", real, [N_Vector, N_Vector]),
    ("nvwsqrsummasklocal", real, [N_Vector, N_Vector, N_Vector]),
    ("nvdotprodmultilocal", ct.c_int, [ct.c_int, N_Vector, P_NV, P_real]),
    ("nvdotprodmultiallreduce", ct.c_int, [ct.c_int, N_Vector, P_real]),
    ("nvbufsize", ct.c_int, [N_Vector, ct.POINTER(idx)]),
    ("nvbufpack", ct.c_int, [N_Vector, ct.c_void_p]),
    ("nvbufunpack", ct.c_int, [N_Vector, ct.c_void_p]),
    ("nvprint", None, [N_Vector]),
    ("nvprintfile", None, [N_Vector, ct.c_void_p]),
]


class NVectorOps(ct.Structure):
    _fields_ = [(name, ct.c_void_p) for name, _, _ in NV_OPS_FIELDS]


class GenericNVector(ct.Structure):
    _fields_ = [("content", ct.c_void_p), ("ops", ct.POINTER(NVectorOps)),
                ("sunctx", ct.c_void_p)]


_OP_TYPES = {name: ct.CFUNCTYPE(res, *args) for name, res, args in NV_OPS_FIELDS}

_lib = None


def load() -> ct.CDLL:
    """Load the GB300 library; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m sundials_gb300.build` "
                "(there is no CPU fallback)")
        _lib = ct.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


def _declare(lib: ct.CDLL) -> None:
    sig = {
        "N_VNew_GB300": (N_Vector, [idx, ct.c_void_p]),
        "N_VNewWithStream_GB300": (N_Vector, [idx, ct.c_void_p, ct.c_void_p]),
        "N_VNewEmpty_GB300": (N_Vector, [ct.c_void_p]),
        "N_VMake_GB300": (N_Vector, [idx, P_real, P_real, ct.c_void_p]),
        "N_VCopyToDevice_GB300": (None, [N_Vector]),
        "N_VCopyFromDevice_GB300": (None, [N_Vector]),
        "N_VGetHostArrayPointer_GB300": (P_real, [N_Vector]),
        "N_VGetDeviceArrayPointer_GB300": (ct.c_void_p, [N_Vector]),
        "N_VSetDeviceArrayPointer_GB300": (None, [ct.c_void_p, N_Vector]),
        "N_VGetStream_GB300": (ct.c_void_p, [N_Vector]),
        "N_VEnableFusedOps_GB300": (ct.c_int, [N_Vector, ct.c_int]),
        "N_VSetFMA_GB300": (ct.c_int, [N_Vector, ct.c_int]),
        "SUNGB300_GetLastError": (ct.c_int, []),
        "SUNGB300_GetLastErrorMessage": (ct.c_char_p, []),
        "SUNGB300_KernelLaunchCount": (ct.c_longlong, []),
        "N_VDestroy_GB300": (None, [N_Vector]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


def ops_of(v: int) -> dict:
    """Callable view of an N_Vector's ops table (NULL entries -> None)."""
    gv = ct.cast(v, ct.POINTER(GenericNVector)).contents
    table = gv.ops.contents
    out = {}
    for name, _, _ in NV_OPS_FIELDS:
        addr = getattr(table, name)
        out[name] = _OP_TYPES[name](addr) if addr else None
    return out


def nv_array(vecs) -> ct.Array:
    arr = (ct.c_void_p * len(vecs))()
    for i, v in enumerate(vecs):
        arr[i] = v
    return arr


def real_array(vals) -> ct.Array:
    arr = (ct.c_double * len(vals))()
    for i, x in enumerate(vals):
        arr[i] = float(x)
    return arr

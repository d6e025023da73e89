"""Host-side handles for the block-diagonal SUNMatrix and the BlockLU
SUNLinearSolver (include/sunlinsol_blocklu_gb300.h), called through their
ops tables like CVODE's linear-solver interface does."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib

FP64, MIXED = 0, 1


class _MatOps(ct.Structure):
    _fields_ = [(n, ct.c_void_p) for n in ("getid", "clone", "destroy", "zero", "copy", "scaleadd",
                                           "scaleaddi", "matvecsetup", "matvec",
                                           "mathermitiantransposevec", "space")]


class _LSOps(ct.Structure):
    _fields_ = [(n, ct.c_void_p) for n in ("gettype", "getid", "setatimes", "setpreconditioner",
                                           "setscalingvectors", "setoptions", "setzeroguess",
                                           "initialize", "setup", "solve", "numiters", "resnorm",
                                           "lastflag", "space", "resid", "free")]


class _Obj(ct.Structure):
    _fields_ = [("content", ct.c_void_p), ("ops", ct.c_void_p), ("sunctx", ct.c_void_p)]


def _declare(lib):
    if getattr(lib, "_bd_declared", False):
        return
    vp, i64, d = ct.c_void_p, ct.c_int64, ct.c_double
    for name, res, args in [
        ("SUNMatrix_BlockDiag_GB300", vp, [i64, ct.POINTER(i64), vp]),
        ("SUNMatrix_BlockDiag_GB300_NNZ", i64, [vp]),
        ("SUNMatrix_BlockDiag_GB300_CopyToDevice", ct.c_int, [vp, vp]),
        ("SUNMatrix_BlockDiag_GB300_CopyFromDevice", ct.c_int, [vp, vp]),
        ("SUNLinSol_BlockLU_GB300", vp, [vp, vp, ct.c_int, vp]),
    ]:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._bd_declared = True


def _ops(ptr, cls):
    obj = ct.cast(ptr, ct.POINTER(_Obj)).contents
    return ct.cast(obj.ops, ct.POINTER(cls)).contents


class BlockDiag:
    def __init__(self, sizes, handle=None):
        self.lib = _lib.load()
        _declare(self.lib)
        self.sizes = np.asarray(sizes, np.int64)
        self.off = np.zeros(self.sizes.size + 1, np.int64)
        self.off[1:] = np.cumsum(self.sizes)
        self.boff = np.zeros(self.sizes.size + 1, np.int64)
        self.boff[1:] = np.cumsum(self.sizes ** 2)
        if handle is None:
            handle = self.lib.SUNMatrix_BlockDiag_GB300(
                self.sizes.size, self.off.ctypes.data_as(ct.POINTER(ct.c_int64)), None)
            if not handle:
                raise RuntimeError("SUNMatrix_BlockDiag_GB300 failed: "
                                   + self.lib.SUNGB300_GetLastErrorMessage().decode())
        self.A = handle
        o = _ops(handle, _MatOps)
        self.zero = ct.CFUNCTYPE(ct.c_int, ct.c_void_p)(o.zero)
        self.copy = ct.CFUNCTYPE(ct.c_int, ct.c_void_p, ct.c_void_p)(o.copy)
        self.scaleadd = ct.CFUNCTYPE(ct.c_int, ct.c_double, ct.c_void_p, ct.c_void_p)(o.scaleadd)
        self.scaleaddi = ct.CFUNCTYPE(ct.c_int, ct.c_double, ct.c_void_p)(o.scaleaddi)
        self.matvec = ct.CFUNCTYPE(ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p)(o.matvec)
        self.clone_fn = ct.CFUNCTYPE(ct.c_void_p, ct.c_void_p)(o.clone)
        self.destroy_fn = ct.CFUNCTYPE(None, ct.c_void_p)(o.destroy)
        self.getid = ct.CFUNCTYPE(ct.c_int, ct.c_void_p)(o.getid)

    @property
    def nnz(self):
        return int(self.boff[-1])

    def set_blocks(self, blocks):
        """blocks: list of (n_b, n_b) arrays in natural (row, col) indexing."""
        flat = np.concatenate([np.asarray(b, np.float64).T.ravel() for b in blocks])
        assert flat.size == self.nnz
        assert self.lib.SUNMatrix_BlockDiag_GB300_CopyToDevice(self.A, flat.ctypes.data) == 0

    def get_blocks(self):
        flat = np.zeros(self.nnz)
        assert self.lib.SUNMatrix_BlockDiag_GB300_CopyFromDevice(self.A, flat.ctypes.data) == 0
        return [flat[self.boff[b]:self.boff[b + 1]].reshape(n, n).T
                for b, n in enumerate(self.sizes)]

    def get_flat(self):
        flat = np.zeros(self.nnz)
        assert self.lib.SUNMatrix_BlockDiag_GB300_CopyFromDevice(self.A, flat.ctypes.data) == 0
        return flat

    def clone(self):
        return BlockDiag(self.sizes, handle=self.clone_fn(self.A))

    def destroy(self):
        if self.A:
            self.destroy_fn(self.A)
            self.A = None


class BlockLU:
    def __init__(self, y_handle, mat: BlockDiag, precision=FP64):
        self.lib = _lib.load()
        _declare(self.lib)
        self.S = self.lib.SUNLinSol_BlockLU_GB300(y_handle, mat.A, precision, None)
        if not self.S:
            raise RuntimeError("SUNLinSol_BlockLU_GB300 failed")
        o = _ops(self.S, _LSOps)
        self.gettype = ct.CFUNCTYPE(ct.c_int, ct.c_void_p)(o.gettype)
        self.initialize = ct.CFUNCTYPE(ct.c_int, ct.c_void_p)(o.initialize)
        self.setup = ct.CFUNCTYPE(ct.c_int, ct.c_void_p, ct.c_void_p)(o.setup)
        self.solve = ct.CFUNCTYPE(ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                  ct.c_double)(o.solve)
        self.lastflag = ct.CFUNCTYPE(ct.c_int64, ct.c_void_p)(o.lastflag)
        self.free_fn = ct.CFUNCTYPE(ct.c_int, ct.c_void_p)(o.free)

    def free(self):
        if self.S:
            self.free_fn(self.S)
            self.S = None

"""Host-side handle for the batched Robertson device user functions
(include/robertson_gb300.h): right-hand side, J v and the exact block-Jacobi
preconditioner on SUNLinSol_BlockLU_GB300, as the C callbacks a CVODE + SPGMR
run of the batch takes."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib

LU_FP64, LU_MIXED = 0, 1


def _declare(lib):
    if getattr(lib, "_rob_declared", False):
        return
    vp, i64 = ct.c_void_p, ct.c_int64
    lib.SUNRoberts_GB300_Create.restype = vp
    lib.SUNRoberts_GB300_Create.argtypes = [i64, ct.POINTER(ct.c_double), vp, ct.c_int, vp]
    lib.SUNRoberts_GB300_Free.restype = None
    lib.SUNRoberts_GB300_Free.argtypes = [vp]
    lib._rob_declared = True


class Robertson:
    def __init__(self, k, tmpl, lu_precision: int = LU_FP64):
        """k: (ncells, 3) rate constants k1, k2, k3; tmpl: an NVector of length 3*ncells."""
        self.lib = _lib.load()
        _declare(self.lib)
        k = np.ascontiguousarray(k, dtype=np.float64)
        self.ncells = k.shape[0]
        self.p = self.lib.SUNRoberts_GB300_Create(
            self.ncells, k.ctypes.data_as(ct.POINTER(ct.c_double)), tmpl.v, int(lu_precision), None)
        if not self.p:
            raise RuntimeError("SUNRoberts_GB300_Create failed: "
                               + self.lib.SUNGB300_GetLastErrorMessage().decode())

    def cvode_callbacks(self):
        """(CVRhsFn, CVLsJacTimesVecFn, CVLsPrecSetupFn, CVLsPrecSolveFn)
        addresses and the user-data pointer they take."""
        addr = lambda name: ct.cast(getattr(self.lib, name), ct.c_void_p).value
        return (addr("SUNRoberts_GB300_RHS"), addr("SUNRoberts_GB300_JTimes"),
                addr("SUNRoberts_GB300_CVPSetup"), addr("SUNRoberts_GB300_CVPSolve"), self.p)

    def jac_address(self) -> int:
        """CVLsJacFn filling a SUNMatrix_BlockDiag_GB300 of 3x3 blocks."""
        return ct.cast(self.lib.SUNRoberts_GB300_Jac, ct.c_void_p).value

    def free(self) -> None:
        if self.p:
            self.lib.SUNRoberts_GB300_Free(self.p)
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

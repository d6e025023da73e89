"""Host-side handle for the 3-D advection-reaction (Brusselator) device user
functions (include/bruss3d_gb300.h): the explicit, implicit and full
right-hand sides, the per-cell reaction solve and the preconditioner solve,
as the C callbacks CVODE / ARKODE runs of the benchmark take."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib

# the benchmark's defaults (advection_reaction_3D.cpp:454-464)
DEFAULTS = dict(xmax=1.0, A=1.0, B=3.5, k=(1.0, 1.0, 1.0, 1.0, 1.0 / 5.0e-6, 1.0 / 5.0e-6),
                c=0.01)


def _declare(lib):
    if getattr(lib, "_bruss_declared", False):
        return
    vp, i64, d = ct.c_void_p, ct.c_int64, ct.c_double
    lib.SUNBruss3D_GB300_Create.restype = vp
    lib.SUNBruss3D_GB300_Create.argtypes = [i64, i64, i64, d, d, d, ct.POINTER(d), d]
    lib.SUNBruss3D_GB300_Free.restype = None
    lib.SUNBruss3D_GB300_Free.argtypes = [vp]
    for name in ("SUNBruss3D_GB300_Advection", "SUNBruss3D_GB300_Reaction",
                 "SUNBruss3D_GB300_RHS"):
        f = getattr(lib, name)
        f.restype, f.argtypes = ct.c_int, [d, vp, vp, vp]
    lib.SUNBruss3D_GB300_SolveReaction.restype = ct.c_int
    lib.SUNBruss3D_GB300_SolveReaction.argtypes = [vp, vp, vp, d, vp]
    lib._bruss_declared = True


class Bruss3D:
    def __init__(self, nx: int, ny: int, nz: int, xmax=None, A=None, B=None, k=None, c=None):
        self.lib = _lib.load()
        _declare(self.lib)
        p = dict(DEFAULTS)
        for name, val in (("xmax", xmax), ("A", A), ("B", B), ("k", k), ("c", c)):
            if val is not None:
                p[name] = val
        kk = np.ascontiguousarray(p["k"], dtype=np.float64)
        self.shape = (int(nx), int(ny), int(nz))
        self.p = self.lib.SUNBruss3D_GB300_Create(
            self.shape[0], self.shape[1], self.shape[2], float(p["xmax"]), float(p["A"]),
            float(p["B"]), kk.ctypes.data_as(ct.POINTER(ct.c_double)), float(p["c"]))
        if not self.p:
            raise ValueError("SUNBruss3D_GB300_Create: bad arguments")

    def advection(self, y, ydot) -> int:
        return self.lib.SUNBruss3D_GB300_Advection(0.0, y.v, ydot.v, self.p)

    def reaction(self, y, ydot) -> int:
        return self.lib.SUNBruss3D_GB300_Reaction(0.0, y.v, ydot.v, self.p)

    def rhs(self, y, ydot) -> int:
        return self.lib.SUNBruss3D_GB300_RHS(0.0, y.v, ydot.v, self.p)

    def solve_reaction(self, y, x, b, gamma: float) -> int:
        return self.lib.SUNBruss3D_GB300_SolveReaction(y.v, x.v, b.v, float(gamma), self.p)

    def cvode_callbacks(self):
        """(CVRhsFn, None (difference-quotient J v), None (no psetup),
        CVLsPrecSolveFn) addresses and the user-data pointer: the benchmark's
        CVODE configuration (cvode_driver.cpp:51-103)."""
        addr = lambda name: ct.cast(getattr(self.lib, name), ct.c_void_p).value
        return (addr("SUNBruss3D_GB300_RHS"), None, None, addr("SUNBruss3D_GB300_CVPSolve"),
                self.p)

    def arkode_callbacks(self, imex: bool = False):
        """(fe, fi ARKRhsFn, None (difference-quotient J v), ARKLsPrecSolveFn)
        addresses and the user-data pointer: the benchmark's ARK-DIRK
        configuration (arkode_driver.cpp:51-160: fe None, fi = advection +
        reaction) or, imex, its ARK-IMEX one (239-370: fe = advection, fi =
        reaction).  The preconditioner solve is the same function as CVODE's:
        the two callback types have the same signature."""
        addr = lambda name: ct.cast(getattr(self.lib, name), ct.c_void_p).value
        f, _, _, psolve, p = self.cvode_callbacks()
        if imex:
            return (addr("SUNBruss3D_GB300_Advection"), addr("SUNBruss3D_GB300_Reaction"), None,
                    psolve, p)
        return None, f, None, psolve, p

    def block_solve_address(self):
        """SUNBruss3D_GB300_SolveReaction: the per-cell solve x = (I - gamma
        dg/dy)^{-1} b at the state y (x may be b), the linear solve of the
        benchmark's task-local Newton (arkode_driver.cpp:580-596)."""
        return ct.cast(self.lib.SUNBruss3D_GB300_SolveReaction, ct.c_void_p).value

    def free(self) -> None:
        if self.p:
            self.lib.SUNBruss3D_GB300_Free(self.p)
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

"""Host-side handle for the heat-2D device user functions
(include/heat2d_gb300.h): the C callbacks an SPGMR / CVODE run of the 5-point
heat problem hands to the solvers, so that their solves run without any
Python in the loop."""
from __future__ import annotations

import ctypes as ct

from . import _lib


def _declare(lib):
    if getattr(lib, "_heat_declared", False):
        return
    vp, i64, d = ct.c_void_p, ct.c_int64, ct.c_double
    for name, res, args in [
        ("SUNHeat2D_GB300_Create", vp, [i64, i64, d, d]),
        ("SUNHeat2D_GB300_Free", None, [vp]),
        ("SUNHeat2D_GB300_SetGamma", ct.c_int, [vp, d]),
        ("SUNHeat2D_GB300_RHS", ct.c_int, [d, vp, vp, vp]),
        ("SUNHeat2D_GB300_ATimes", ct.c_int, [vp, vp, vp]),
        ("SUNHeat2D_GB300_PSetup", ct.c_int, [vp]),
        ("SUNHeat2D_GB300_PSolve", ct.c_int, [vp, vp, vp, d, ct.c_int]),
    ]:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._heat_declared = True


class Heat2D:
    def __init__(self, nx: int, ny: int, kx: float = 1.0, ky: float = 1.0):
        self.lib = _lib.load()
        _declare(self.lib)
        self.nx, self.ny = int(nx), int(ny)
        self.p = self.lib.SUNHeat2D_GB300_Create(self.nx, self.ny, float(kx), float(ky))
        if not self.p:
            raise ValueError("SUNHeat2D_GB300_Create: bad grid")

    def set_gamma(self, gamma: float) -> None:
        self.lib.SUNHeat2D_GB300_SetGamma(self.p, float(gamma))

    def rhs(self, u, f) -> int:
        return self.lib.SUNHeat2D_GB300_RHS(0.0, u.v, f.v, self.p)

    def atimes(self, v, z) -> int:
        return self.lib.SUNHeat2D_GB300_ATimes(self.p, v.v, z.v)

    def psetup(self) -> int:
        return self.lib.SUNHeat2D_GB300_PSetup(self.p)

    def psolve(self, r, z) -> int:
        return self.lib.SUNHeat2D_GB300_PSolve(self.p, r.v, z.v, 0.0, 1)

    def c_callbacks(self):
        """(ATimes, Psetup, Psolve) addresses for SPGMR.set_*_c, and the data pointer."""
        addr = lambda name: ct.cast(getattr(self.lib, name), ct.c_void_p).value
        return (addr("SUNHeat2D_GB300_ATimes"), addr("SUNHeat2D_GB300_PSetup"),
                addr("SUNHeat2D_GB300_PSolve"), self.p)

    def cvode_callbacks(self):
        """(CVRhsFn, CVLsJacTimesVecFn, CVLsPrecSetupFn, CVLsPrecSolveFn)
        addresses for CVodeInit / CVodeSetJacTimes / CVodeSetPreconditioner,
        and the user-data pointer they take."""
        addr = lambda name: ct.cast(getattr(self.lib, name), ct.c_void_p).value
        return (addr("SUNHeat2D_GB300_RHS"), addr("SUNHeat2D_GB300_JTimes"),
                addr("SUNHeat2D_GB300_CVPSetup"), addr("SUNHeat2D_GB300_CVPSolve"), self.p)

    def free(self) -> None:
        if self.p:
            self.lib.SUNHeat2D_GB300_Free(self.p)
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

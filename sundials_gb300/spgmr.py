"""Host-side handle for SUNLinSol_SPGMR_GB300 (include/sunlinsol_spgmr_gb300.h):
every generic operation is called through the solver's ops table, as CVODE's
linear-solver interface does (src/cvode/cvode_ls.c), and ATimes / Psetup /
Psolve are Python callables wrapped as the C callback types of
src/sundials/sundials_iterative.h:100-140.

A callback receives N_Vector handles (ints); ``device_array(handle)`` gives
the vector's device pointer for whatever the callback launches.  Callbacks
must order their GPU work on the vectors' stream (the legacy default stream
for vectors made by N_VNew_GB300)."""
from __future__ import annotations

import ctypes as ct

from . import _lib
from .blockdiag import _LSOps, _ops

PREC_NONE, PREC_LEFT, PREC_RIGHT, PREC_BOTH = 0, 1, 2, 3
MODIFIED_GS, CLASSICAL_GS = 1, 2

ATIMES_FN = ct.CFUNCTYPE(ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p)
PSETUP_FN = ct.CFUNCTYPE(ct.c_int, ct.c_void_p)
PSOLVE_FN = ct.CFUNCTYPE(ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_double, ct.c_int)

_vp, _i = ct.c_void_p, ct.c_int
_OPS_SIG = {
    "gettype": (_i, [_vp]),
    "getid": (_i, [_vp]),
    "setatimes": (_i, [_vp, _vp, ATIMES_FN]),
    "setpreconditioner": (_i, [_vp, _vp, PSETUP_FN, PSOLVE_FN]),
    "setscalingvectors": (_i, [_vp, _vp, _vp]),
    "setzeroguess": (_i, [_vp, _i]),
    "initialize": (_i, [_vp]),
    "setup": (_i, [_vp, _vp]),
    "solve": (_i, [_vp, _vp, _vp, _vp, ct.c_double]),
    "numiters": (_i, [_vp]),
    "resnorm": (ct.c_double, [_vp]),
    "lastflag": (ct.c_int64, [_vp]),
    "space": (_i, [_vp, ct.POINTER(ct.c_long), ct.POINTER(ct.c_long)]),
    "resid": (_vp, [_vp]),
    "free": (_i, [_vp]),
}


def _declare(lib):
    if getattr(lib, "_spgmr_declared", False):
        return
    for name, res, args in [
        ("SUNLinSol_SPGMR_GB300", _vp, [_vp, _i, _i, _vp]),
        ("SUNLinSol_SPGMR_GB300SetPrecType", _i, [_vp, _i]),
        ("SUNLinSol_SPGMR_GB300SetGSType", _i, [_vp, _i]),
        ("SUNLinSol_SPGMR_GB300SetMaxRestarts", _i, [_vp, _i]),
        ("SUNLinSol_SPGMR_GB300SetFusedGS", _i, [_vp, _i]),
        ("SUNLinSol_SPGMR_GB300NumSyncs", ct.c_long, [_vp]),
        ("N_VGetDeviceArrayPointer_GB300", _vp, [_vp]),
    ]:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._spgmr_declared = True


def device_array(handle) -> int:
    """Device pointer of an NVECTOR_GB300 handle."""
    lib = _lib.load()
    _declare(lib)
    return lib.N_VGetDeviceArrayPointer_GB300(handle) or 0


class SPGMR:
    def __init__(self, y, pretype: int = PREC_NONE, maxl: int = 5):
        self.lib = _lib.load()
        _declare(self.lib)
        self.S = self.lib.SUNLinSol_SPGMR_GB300(y.v, int(pretype), int(maxl), None)
        if not self.S:
            raise RuntimeError("SUNLinSol_SPGMR_GB300 failed: "
                               + self.lib.SUNGB300_GetLastErrorMessage().decode())
        table = _ops(self.S, _LSOps)
        self.ops = {}
        for name, (res, args) in _OPS_SIG.items():
            addr = getattr(table, name)
            if addr:
                self.ops[name] = ct.CFUNCTYPE(res, *args)(addr)
        self._keep = []

    # ---- configuration (reference: SUNLinSol_SPGMRSet*, SUNLinSolSet*)
    def set_gs_type(self, gstype: int) -> int:
        return self.lib.SUNLinSol_SPGMR_GB300SetGSType(self.S, int(gstype))

    def set_prec_type(self, pretype: int) -> int:
        return self.lib.SUNLinSol_SPGMR_GB300SetPrecType(self.S, int(pretype))

    def set_max_restarts(self, maxrs: int) -> int:
        return self.lib.SUNLinSol_SPGMR_GB300SetMaxRestarts(self.S, int(maxrs))

    def set_fused(self, on: bool) -> int:
        return self.lib.SUNLinSol_SPGMR_GB300SetFusedGS(self.S, 1 if on else 0)

    def set_atimes(self, fn) -> int:
        cb = ATIMES_FN(lambda data, v, z: int(fn(v, z)))
        self._keep.append(cb)
        return self.ops["setatimes"](self.S, None, cb)

    def set_preconditioner(self, psolve, psetup=None) -> int:
        ps = PSOLVE_FN(lambda data, r, z, tol, lr: int(psolve(r, z, tol, lr)))
        pu = PSETUP_FN(lambda data: int(psetup())) if psetup else PSETUP_FN()
        self._keep += [ps, pu]
        return self.ops["setpreconditioner"](self.S, None, pu, ps)

    def set_atimes_c(self, fn_addr: int, data) -> int:
        """ATimes given as a C function (address of a SUNATimesFn) and its data."""
        cb = ATIMES_FN(fn_addr)
        self._keep.append(cb)
        return self.ops["setatimes"](self.S, data, cb)

    def set_preconditioner_c(self, psolve_addr: int, psetup_addr: int | None, data) -> int:
        """Psetup / Psolve given as C functions (SUNPSetupFn / SUNPSolveFn)."""
        ps = PSOLVE_FN(psolve_addr)
        pu = PSETUP_FN(psetup_addr) if psetup_addr else PSETUP_FN()
        self._keep += [ps, pu]
        return self.ops["setpreconditioner"](self.S, data, pu, ps)

    def set_scaling_vectors(self, s1=None, s2=None) -> int:
        return self.ops["setscalingvectors"](self.S, s1.v if s1 else None, s2.v if s2 else None)

    def set_zero_guess(self, on: bool) -> int:
        return self.ops["setzeroguess"](self.S, 1 if on else 0)

    # ---- operations
    def initialize(self) -> int:
        return self.ops["initialize"](self.S)

    def setup(self) -> int:
        return self.ops["setup"](self.S, None)

    def solve(self, x, b, delta: float) -> int:
        return self.ops["solve"](self.S, None, x.v, b.v, float(delta))

    @property
    def num_iters(self) -> int:
        return self.ops["numiters"](self.S)

    @property
    def res_norm(self) -> float:
        return self.ops["resnorm"](self.S)

    @property
    def last_flag(self) -> int:
        return self.ops["lastflag"](self.S)

    @property
    def num_syncs(self) -> int:
        return self.lib.SUNLinSol_SPGMR_GB300NumSyncs(self.S)

    def gettype(self) -> int:
        return self.ops["gettype"](self.S)

    def getid(self) -> int:
        return self.ops["getid"](self.S)

    def space(self):
        rw, iw = ct.c_long(), ct.c_long()
        self.ops["space"](self.S, ct.byref(rw), ct.byref(iw))
        return rw.value, iw.value

    def resid(self) -> int:
        return self.ops["resid"](self.S)

    def free(self) -> None:
        if self.S:
            self.ops["free"](self.S)
            self.S = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

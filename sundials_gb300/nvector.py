"""Host-side handle for NVECTOR_GB300 vectors.

A thin owner of an ``N_Vector`` created by ``N_VNew_GB300``: numpy data goes
in and out through the vector's own pinned host mirror and
``N_VCopyToDevice_GB300`` / ``N_VCopyFromDevice_GB300``; every operation is
called through the vector's ops table (``ops``), the way CVODE/ARKODE reach it.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib


class NVector:
    def __init__(self, n: int, *, stream=None, handle: int | None = None, own: bool = True):
        self.lib = _lib.load()
        if handle is None:
            if stream is None:
                handle = self.lib.N_VNew_GB300(int(n), None)
            else:
                handle = self.lib.N_VNewWithStream_GB300(int(n), ct.c_void_p(stream), None)
            if not handle:
                raise RuntimeError("N_VNew_GB300 failed: "
                                   + self.lib.SUNGB300_GetLastErrorMessage().decode())
        self.v = handle
        self.n = int(n)
        self.own = own
        self.ops = _lib.ops_of(handle)

    # --------------------------------------------------------------- data
    @classmethod
    def from_numpy(cls, a, **kw) -> "NVector":
        a = np.ascontiguousarray(a, dtype=np.float64)
        v = cls(a.size, **kw)
        v.set(a)
        return v

    def set(self, a) -> None:
        a = np.ascontiguousarray(a, dtype=np.float64)
        if self.n == 0:
            return
        h = self.ops["nvgetarraypointer"](self.v)
        ct.memmove(h, a.ctypes.data, 8 * self.n)
        self.lib.N_VCopyToDevice_GB300(self.v)

    def get(self) -> np.ndarray:
        if self.n == 0:
            return np.zeros(0)
        self.lib.N_VCopyFromDevice_GB300(self.v)
        h = self.ops["nvgetarraypointer"](self.v)
        return np.ctypeslib.as_array(h, shape=(self.n,)).copy()

    @property
    def device_ptr(self) -> int:
        return self.lib.N_VGetDeviceArrayPointer_GB300(self.v) or 0

    def clone(self) -> "NVector":
        h = self.ops["nvclone"](self.v)
        return NVector(self.n, handle=h)

    def set_fma(self, on: bool) -> None:
        self.lib.N_VSetFMA_GB300(self.v, 1 if on else 0)

    def destroy(self) -> None:
        if self.v and self.own:
            self.ops["nvdestroy"](self.v)
        self.v = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

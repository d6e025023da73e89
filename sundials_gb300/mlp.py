"""Host-side handle for the learned Newton predictor (include/sunmlp_gb300.h):
creation, parameters, batched inference and training steps, all through the
C ABI; device arrays are passed as raw pointers (torch tensors are used for
device memory by the training driver in sundials_gb300/learned.py)."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib

IN, IN_PAD, HID, OUT, TILE = 129, 144, 64, 64, 128
NPARAMS = IN_PAD * HID + HID + HID * HID + HID + HID * OUT + OUT
# offsets of the FP32 master parameters
P_W1, P_B1 = 0, IN_PAD * HID
P_W2 = P_B1 + HID
P_B2 = P_W2 + HID * HID
P_W3 = P_B2 + HID
P_B3 = P_W3 + HID * OUT


def _declare(lib):
    if getattr(lib, "_mlp_declared", False):
        return
    vp, i64, f = ct.c_void_p, ct.c_int64, ct.c_float
    for name, res, args in [
        ("SUNMLP_GB300_Create", vp, [ct.c_uint64, vp]),
        ("SUNMLP_GB300_Free", None, [vp]),
        ("SUNMLP_GB300_SetParams", ct.c_int, [vp, vp]),
        ("SUNMLP_GB300_GetParams", ct.c_int, [vp, vp]),
        ("SUNMLP_GB300_DeviceWeights", vp, [vp]),
        ("SUNMLP_GB300_DeviceBiases", vp, [vp]),
        ("SUNMLP_GB300_Forward", ct.c_int, [vp, i64, vp, vp]),
        ("SUNMLP_GB300_Gradients", ct.c_int, [vp, i64, vp, vp, vp, ct.POINTER(f)]),
        ("SUNMLP_GB300_TrainStep", ct.c_int, [vp, i64, vp, vp, f, ct.POINTER(f)]),
    ]:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    lib._mlp_declared = True


def split(params: np.ndarray):
    """(W1, b1, W2, b2, W3, b3) views of a flat FP32 parameter vector."""
    p = np.asarray(params)
    return (p[P_W1:P_B1].reshape(IN_PAD, HID), p[P_B1:P_W2], p[P_W2:P_B2].reshape(HID, HID),
            p[P_B2:P_W3], p[P_W3:P_B3].reshape(HID, OUT), p[P_B3:])


class MLP:
    def __init__(self, seed: int = 1, stream=None):
        self.lib = _lib.load()
        _declare(self.lib)
        self.h = self.lib.SUNMLP_GB300_Create(int(seed), stream)
        if not self.h:
            raise RuntimeError("SUNMLP_GB300_Create failed: "
                               + self.lib.SUNGB300_GetLastErrorMessage().decode())

    @property
    def device_weights(self) -> int:
        return self.lib.SUNMLP_GB300_DeviceWeights(self.h)

    @property
    def device_biases(self) -> int:
        return self.lib.SUNMLP_GB300_DeviceBiases(self.h)

    def get_params(self) -> np.ndarray:
        out = np.zeros(NPARAMS, np.float32)
        assert self.lib.SUNMLP_GB300_GetParams(self.h, out.ctypes.data) == 0
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == NPARAMS
        assert self.lib.SUNMLP_GB300_SetParams(self.h, p.ctypes.data) == 0

    def forward(self, rows: int, d_x: int, d_out: int) -> None:
        assert self.lib.SUNMLP_GB300_Forward(self.h, rows, d_x, d_out) == 0

    def gradients(self, rows: int, d_x: int, d_t: int, d_grad: int) -> float:
        loss = ct.c_float()
        rc = self.lib.SUNMLP_GB300_Gradients(self.h, rows, d_x, d_t, d_grad, ct.byref(loss))
        assert rc == 0, rc
        return loss.value

    def train_step(self, rows: int, d_x: int, d_t: int, lr: float, want_loss=False):
        loss = ct.c_float()
        rc = self.lib.SUNMLP_GB300_TrainStep(self.h, rows, d_x, d_t, lr,
                                             ct.byref(loss) if want_loss else None)
        assert rc == 0, rc
        return loss.value if want_loss else None

    def free(self):
        if self.h:
            self.lib.SUNMLP_GB300_Free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

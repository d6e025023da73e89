"""Host-side handle for SUNBatchBDF_GB300 (include/sunbatchbdf_gb300.h)."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib
from .kinetics import BATCH_STATS_DTYPE, KineticsBatch

FP64, FP64_EXACT, MIXED = 0, 1, 2
MODES = {"fp64": FP64, "fp64_exact": FP64_EXACT, "mixed": MIXED}


class _Problem(ct.Structure):
    _fields_ = [("nsys", ct.c_int64)] + [
        (name, ct.c_void_p) for name in ("n", "y_off", "r_off", "rtype", "ra", "rb", "rc", "rk")]


def _declare(lib):
    if getattr(lib, "_batch_declared", False):
        return
    vp = ct.c_void_p
    for name, res, args in [
        ("SUNBatchBDF_GB300_Create", vp, [ct.POINTER(_Problem), vp]),
        ("SUNBatchBDF_GB300_SetTolerances", ct.c_int, [vp, ct.c_double, ct.c_double]),
        ("SUNBatchBDF_GB300_SetMaxNumSteps", ct.c_int, [vp, ct.c_long]),
        ("SUNBatchBDF_GB300_SetMode", ct.c_int, [vp, ct.c_int]),
        ("SUNBatchBDF_GB300_SetRefinementSweeps", ct.c_int, [vp, ct.c_int]),
        ("SUNBatchBDF_GB300_Solve", ct.c_int, [vp, ct.c_double, vp, ct.c_double, vp, vp]),
        ("SUNBatchBDF_GB300_SolveAsync", ct.c_int, [vp, ct.c_double, vp, ct.c_double, vp, vp]),
        ("SUNBatchBDF_GB300_LastKernelMs", ct.c_double, [vp]),
        ("SUNBatchBDF_GB300_Free", None, [vp]),
        ("SUNBatchBDF_GB300_SetPredictor", ct.c_int, [vp, vp, vp]),
        ("SUNBatchBDF_GB300_GetPredictorCounts", ct.c_int,
         [vp, ct.POINTER(ct.c_longlong), ct.POINTER(ct.c_longlong)]),
        ("SUNBatchBDF_GB300_SetRecorder", ct.c_int, [vp, vp, vp, ct.c_longlong, vp]),
        ("SUNBatchBDF_GB300_SetRetryMode", ct.c_int, [vp, ct.c_int]),
        ("SUNBatchBDF_GB300_Autotune", ct.c_int, [vp, ct.c_double, vp, ct.c_double, ct.c_int, vp]),
        ("SUNBatchBDF_GB300_GetLaunchPlan", ct.c_int, [vp, ct.c_int, vp]),
        ("SUNBatchBDF_GB300_GetRetryCount", ct.c_int, [vp, ct.POINTER(ct.c_longlong)]),
    ]:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._batch_declared = True


class BatchBDF:
    def __init__(self, batch: KineticsBatch, stream=None):
        self.lib = _lib.load()
        _declare(self.lib)
        self.batch = batch
        self._keep = [np.ascontiguousarray(batch.n, np.int32),
                      np.ascontiguousarray(batch.y_off, np.int64),
                      np.ascontiguousarray(batch.r_off, np.int64),
                      np.ascontiguousarray(batch.rtype, np.int32),
                      np.ascontiguousarray(batch.ra, np.int32),
                      np.ascontiguousarray(batch.rb, np.int32),
                      np.ascontiguousarray(batch.rc, np.int32),
                      np.ascontiguousarray(batch.rk, np.float64)]
        prob = _Problem(batch.nsys, *[a.ctypes.data for a in self._keep])
        self.h = self.lib.SUNBatchBDF_GB300_Create(ct.byref(prob), stream)
        if not self.h:
            raise RuntimeError("SUNBatchBDF_GB300_Create failed: "
                               + self.lib.SUNGB300_GetLastErrorMessage().decode())

    def configure(self, rtol=1e-6, atol=1e-12, mode="fp64", mxstep=1000000, refine=1,
                  retry="other"):
        """retry: mode for systems that fail in a fast mode ("other" fast mode,
        "fp64_exact", "fp64", "mixed", or None for no retry)."""
        L = self.lib
        rmode = {None: -1, "other": -2}.get(retry, MODES.get(retry))
        self._mode = MODES[mode] if isinstance(mode, str) else mode
        assert L.SUNBatchBDF_GB300_SetRetryMode(self.h, rmode) == 0
        assert L.SUNBatchBDF_GB300_SetTolerances(self.h, rtol, atol) == 0
        assert L.SUNBatchBDF_GB300_SetMode(self.h, MODES[mode] if isinstance(mode, str) else mode) == 0
        assert L.SUNBatchBDF_GB300_SetMaxNumSteps(self.h, mxstep) == 0
        assert L.SUNBatchBDF_GB300_SetRefinementSweeps(self.h, refine) == 0
        return self

    def solve(self, tout=100.0, t0=0.0, y0=None):
        y0 = np.ascontiguousarray(self.batch.y0 if y0 is None else y0, np.float64)
        yout = np.zeros_like(y0)
        stats = np.zeros(self.batch.nsys, BATCH_STATS_DTYPE)
        rc = self.lib.SUNBatchBDF_GB300_Solve(self.h, t0, y0.ctypes.data, tout,
                                              yout.ctypes.data, stats.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"SUNBatchBDF_GB300_Solve failed ({rc}): "
                               + self.lib.SUNGB300_GetLastErrorMessage().decode())
        return yout, stats

    def solve_device(self, d_y0: int, d_yout: int, d_stats: int, tout=100.0, t0=0.0):
        rc = self.lib.SUNBatchBDF_GB300_SolveAsync(self.h, t0, d_y0, tout, d_yout, d_stats)
        if rc != 0:
            raise RuntimeError(f"SUNBatchBDF_GB300_SolveAsync failed ({rc})")

    def set_predictor(self, mlp) -> None:
        """Use a trained sundials_gb300.mlp.MLP as Newton predictor (None: off)."""
        if mlp is None:
            rc = self.lib.SUNBatchBDF_GB300_SetPredictor(self.h, None, None)
        else:
            rc = self.lib.SUNBatchBDF_GB300_SetPredictor(self.h, mlp.device_weights,
                                                         mlp.device_biases)
        if rc != 0:
            raise RuntimeError(f"SUNBatchBDF_GB300_SetPredictor failed ({rc})")
        self._mlp = mlp

    def autotune(self, stride=16, tout=100.0, t0=0.0, y0=None):
        """Time every launch plan on every stride-th system and keep the
        fastest for the configured mode; returns {plan widths: ms}."""
        y0 = np.ascontiguousarray(self.batch.y0 if y0 is None else y0, np.float64)
        ms = np.zeros(4)
        rc = self.lib.SUNBatchBDF_GB300_Autotune(self.h, t0, y0.ctypes.data, tout, int(stride),
                                                 ms.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"SUNBatchBDF_GB300_Autotune failed ({rc})")
        plans = ["32,64", "32,48,64", "48,64", "64"]
        return dict(zip(plans, ms.tolist()))

    def launch_plan(self, mode=None):
        w = np.zeros(3, np.int32)
        m = MODES[mode] if isinstance(mode, str) else (self._mode if mode is None else mode)
        assert self.lib.SUNBatchBDF_GB300_GetLaunchPlan(self.h, m, w.ctypes.data) == 0
        return [int(x) for x in w if x]

    @property
    def retry_count(self) -> int:
        n = ct.c_longlong()
        assert self.lib.SUNBatchBDF_GB300_GetRetryCount(self.h, ct.byref(n)) == 0
        return n.value

    def predictor_counts(self):
        calls, kept = ct.c_longlong(), ct.c_longlong()
        assert self.lib.SUNBatchBDF_GB300_GetPredictorCounts(self.h, ct.byref(calls),
                                                             ct.byref(kept)) == 0
        return calls.value, kept.value

    def set_recorder(self, d_x: int, d_t: int, capacity: int, d_count: int) -> None:
        """Record (features, converged corrector) rows into device buffers."""
        rc = self.lib.SUNBatchBDF_GB300_SetRecorder(self.h, d_x, d_t, capacity, d_count)
        if rc != 0:
            raise RuntimeError(f"SUNBatchBDF_GB300_SetRecorder failed ({rc})")

    @property
    def last_kernel_ms(self) -> float:
        return self.lib.SUNBatchBDF_GB300_LastKernelMs(self.h)

    def free(self):
        if self.h:
            self.lib.SUNBatchBDF_GB300_Free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _main(argv=None):
    """One solve of the seeded kinetics batch (a profiling and smoke entry):
    python -m sundials_gb300.batch --nsys 4096 --mode mixed"""
    import argparse
    import json

    from . import kinetics as K
    ap = argparse.ArgumentParser()
    ap.add_argument("--nsys", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--mode", choices=sorted(MODES), default="mixed")
    ap.add_argument("--rtol", type=float, default=1e-6)
    ap.add_argument("--atol", type=float, default=1e-12)
    ap.add_argument("--tout", type=float, default=100.0)
    args = ap.parse_args(argv)
    b = BatchBDF(K.generate(args.nsys, seed=args.seed)).configure(args.rtol, args.atol, args.mode)
    _, st = b.solve(args.tout)
    print(json.dumps({"nsys": args.nsys, "mode": args.mode, "kernel_ms": round(b.last_kernel_ms, 3),
                      "nst": int(st["nst"].sum()), "nni": int(st["nni"].sum()),
                      "nsetups": int(st["nsetups"].sum()), "failed": int((st["flag"] != 0).sum())}))


if __name__ == "__main__":
    _main()

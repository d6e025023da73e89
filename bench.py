#!/usr/bin/env python3
"""Benchmark of the GB300 SUNDIALS hot path.  Prints ONE JSON line on rank 0.

Headline (``value``): ODE systems solved per second on the uneven stiff
kinetics batch -- 65,536 independent mass-action networks, n ~ U{8..64}
species, 2n reactions each, rtol 1e-6, atol 1e-12, t in [0, 100] -- by the
batched per-system BDF integrator in its MIXED form (FP32 Newton-matrix
inverse with FP64 refinement; FP64 residuals, norms, error test and step
control).  One step = one full integration of the whole batch.  The plain
FP64 GPU form of the same solver is timed in the same run
(``plain_fp64_gpu``), and the error of both against the FP64 oracle solution
(the reference's own CVODE at rtol 1e-10) is reported on the 1,024-system
golden sample.  The 19 MB state fits in L2, so a 512 MB buffer is written
between timed steps (L2 flush, outside the timed region).

``nvector``: the N_Vector microbenchmark (FP64, length 2^28; LinearSum,
LinearCombination(5), DotProdMulti(5), WrmsNorm; 136 bytes per element),
with the HBM roofline of its dominant kernel.

``--impl reference``: the reference's CPU path on the host cores -- the
CVODE restatement (bit-identical to the reference's CVODE on the golden
systems) over all host threads, on a bounded sample of the same batch.
"""
from __future__ import annotations

import argparse
import ctypes as ct
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ODE systems solved/s vs plain FP64 GPU form at rtol 1e-6; N_Vector HBM GB/s"
NV_BYTES = {"LinearSum": 24, "LinearCombination5": 48, "DotProdMulti5": 48, "WrmsNorm": 16,
            "ScaleAddMulti5": 88}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, gpu_index=0):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(gpu_index):
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ distributed
# One process per GPU (torchrun); the batch is not split: every rank
# integrates its own seeded batch (weak scaling, no data-path collective), and
# only the timings meet, as the max over ranks.  The backend is NCCL on GPUs;
# the same helpers run over gloo on CPU for the multi-process tests.
_BACKEND = "nccl"


def dist_setup(n_gpus, backend="nccl"):
    global _BACKEND
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        _BACKEND = backend
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(world, x, op):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if _BACKEND == "nccl" else "cpu")
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(world, x):
    import torch.distributed as dist
    return x if world == 1 else _reduce(world, x, dist.ReduceOp.MAX)


def sum_over_ranks(world, x):
    import torch.distributed as dist
    return x if world == 1 else _reduce(world, x, dist.ReduceOp.SUM)


def rank_seed(rank):
    """Seed of rank's batch: rank 0 integrates the seed-1 batch the accuracy
    checks use; the others get distinct seeds."""
    return 1 if rank == 0 else 1 + rank * 1000003


def weak_value(units_per_rank, steps, world, max_elapsed):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    return units_per_rank * steps * world / max_elapsed


# --------------------------------------------------------- nvector workload
def gen_inputs(n, seed=1):
    rng = np.random.default_rng(seed)
    xs = [rng.uniform(-1.0, 1.0, n) for _ in range(6)]
    y = rng.uniform(-1.0, 1.0, n)
    w = 1.0 / (1e-6 * np.abs(y) + 1e-10)
    c5 = rng.uniform(-1.0, 1.0, 5)
    return xs, y, w, c5


def nvector_measure(args, rank, local, steps, warmup):
    """N_Vector microbenchmark on this GPU; returns a dict (per-op GB/s, the
    roofline of the dominant kernel, launch count)."""
    import torch
    from sundials_gb300 import _lib
    from sundials_gb300.nvector import NVector

    lib = _lib.load()
    n = 1 << args.log2n
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    xs, y, w, c5 = gen_inputs(n, seed=1 + rank)
    X = [NVector.from_numpy(a, stream=sp) for a in xs]
    Y = NVector.from_numpy(y, stream=sp)
    W = NVector.from_numpy(w, stream=sp)
    Z = NVector(n, stream=sp)
    Z2 = NVector(n, stream=sp)
    del xs, y, w
    ops = Z.ops
    c5a = _lib.real_array(c5)
    arrX = _lib.nv_array([v.v for v in X[:5]])
    dots = (ct.c_double * 5)()
    evs = {k: [] for k in NV_BYTES}

    a5 = _lib.real_array(c5[::-1].copy() * 1e-3)
    arrY = _lib.nv_array([v.v for v in X[1:6]])  # Y_k += a_k x in place, as CVODE calls it

    def step(timed):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(6)] if timed else None
        if timed:
            e[0].record(stream)
        ops["nvlinearsum"](0.3, X[0].v, 0.7, Y.v, Z.v)
        if timed:
            e[1].record(stream)
        ops["nvlinearcombination"](5, c5a, arrX, Z2.v)
        if timed:
            e[2].record(stream)
        ops["nvdotprodmulti"](5, X[5].v, arrX, dots)
        if timed:
            e[3].record(stream)
        ops["nvwrmsnorm"](X[0].v, W.v)
        if timed:
            e[4].record(stream)
        ops["nvscaleaddmulti"](5, a5, X[0].v, arrY, arrY)
        if timed:
            e[5].record(stream)
            for k, name in enumerate(NV_BYTES):
                evs[name].append((e[k], e[k + 1]))

    for _ in range(warmup):
        step(False)
    torch.cuda.synchronize()
    l0 = lib.SUNGB300_KernelLaunchCount()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        step(True)
    t1.record(stream)
    torch.cuda.synchronize()
    launches = lib.SUNGB300_KernelLaunchCount() - l0
    elapsed = t0.elapsed_time(t1) / 1e3
    bytes_step = sum(NV_BYTES.values()) * n
    per_op = {}
    for name, lst in evs.items():
        ms = float(np.mean([a.elapsed_time(b) for a, b in lst]))
        per_op[name] = {"ms": round(ms, 4), "GBs": round(NV_BYTES[name] * n / (ms / 1e3) / 1e9, 1)}
    hbm, src = peaks()
    achieved = per_op["LinearCombination5"]["GBs"]
    out = {
        "workload": "nvector_microbench_2^%d" % args.log2n, "vector_length": n,
        "GBs": round(bytes_step * steps / elapsed / 1e9, 1), "steps": steps,
        "bytes_per_elem_step": sum(NV_BYTES.values()), "per_op": per_op,
        "arithmetic": "FMA (default)",
        "l2": "inputs larger than L2 (2 GiB per vector), no flush",
        "roofline": {"bound": "hbm", "kernel": "k_lincomb (LinearCombination, 5 vectors)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "peak_source": src,
                     "traffic": None,
                     "note": "FP64-issue-bound on GB300 (~600 G FP64 instr/s): 5 FP64 "
                             "instructions per element cap this kernel at ~85% of HBM"},
        "gpu_launches": int(launches),
    }
    for v in X + [Y, W, Z, Z2]:
        v.destroy()
    out["sweep"] = nvector_sweep(rank)
    return out


def nvector_sweep(rank, log2s=(12, 16, 20, 22, 24, 26)):
    """The same five operations at 2^12 .. 2^26 elements, each timed over
    back-to-back calls with CUDA events (no flush).  Where an operation's
    operands fit in the 129 MB L2 (operands_fit_l2) the figure is L2
    bandwidth or launch latency; the reductions (DotProdMulti, WrmsNorm)
    return their result to the host on every call, so at small sizes their
    figure is that round trip (the "us" per call; the Python caller adds
    ~0.25 us).  From 2^24
    every operation streams from HBM, as at 2^28."""
    import torch
    from sundials_gb300 import _lib
    from sundials_gb300.nvector import NVector

    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    res = {}
    for lg in log2s:
        n = 1 << lg
        xs, y, w, c5 = gen_inputs(n, seed=11 + rank)
        X = [NVector.from_numpy(a, stream=sp) for a in xs]
        W = NVector.from_numpy(w, stream=sp)
        Z, Z2 = NVector(n, stream=sp), NVector(n, stream=sp)
        ops = Z.ops
        c5a = _lib.real_array(c5)
        a5 = _lib.real_array(c5[::-1].copy() * 1e-3)
        arrX = _lib.nv_array([v.v for v in X[:5]])
        arrY = _lib.nv_array([v.v for v in X[1:6]])
        dots = (ct.c_double * 5)()
        calls = {
            "LinearSum": lambda: ops["nvlinearsum"](0.3, X[0].v, 0.7, X[1].v, Z.v),
            "LinearCombination5": lambda: ops["nvlinearcombination"](5, c5a, arrX, Z2.v),
            "DotProdMulti5": lambda: ops["nvdotprodmulti"](5, X[5].v, arrX, dots),
            "WrmsNorm": lambda: ops["nvwrmsnorm"](X[0].v, W.v),
            "ScaleAddMulti5": lambda: ops["nvscaleaddmulti"](5, a5, X[0].v, arrY, arrY),
        }
        reps = max(10, min(400, (1 << 30) // (n * 48)))
        row = {}
        for name, fn in calls.items():
            for _ in range(3):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            us = e0.elapsed_time(e1) * 1e3 / reps
            row[name] = {"us": round(us, 2), "GBs": round(NV_BYTES[name] * n / (us * 1e-6) / 1e9, 1),
                         "operands_fit_l2": NV_BYTES[name] * n < 129e6}
        res["2^%d" % lg] = row
        for v in X + [W, Z, Z2]:
            v.destroy()
    return res


def spgmr_measure(nx=2048, solves=20, warmup=3):
    """SPGMR on the heat-2D Newton system (I - gamma J) x = b, 2048^2 interior
    points, maxl 5, left Jacobi preconditioning, no restarts (the CVODE
    configuration of the heat benchmark), with the operator and preconditioner
    as C callbacks (include/heat2d_gb300.h).  Each Gram-Schmidt type runs with
    the fused kernels and with the reference's sequence of N_Vector
    operations on the same GPU; wall time per solve includes the host's
    synchronisations, which is what the fusion removes."""
    import torch
    from sundials_gb300 import _lib
    from sundials_gb300.heat2d import Heat2D
    from sundials_gb300.nvector import NVector
    from sundials_gb300.spgmr import SPGMR

    lib = _lib.load()
    n = nx * nx
    gamma = 1e-6
    rng = np.random.default_rng(1)
    b = rng.uniform(-1.0, 1.0, n)
    delta = 1e-4 * float(np.linalg.norm(b))
    H = Heat2D(nx, nx)
    H.set_gamma(gamma)
    X, B = NVector(n), NVector.from_numpy(b)
    at, pset, psol, data = H.c_callbacks()
    out = {"workload": f"heat2d {nx}x{nx} Newton system, SPGMR maxl 5, left Jacobi",
           "vector_length": n, "gamma": gamma, "delta": delta}
    for gs, gname in ((1, "mgs"), (2, "cgs")):
        for fused in (True, False):
            S = SPGMR(X, 1, 5)
            S.set_gs_type(gs)
            S.set_fused(fused)
            S.set_atimes_c(at, data)
            S.set_preconditioner_c(psol, pset, data)
            S.initialize()
            S.setup()
            for _ in range(warmup):
                S.set_zero_guess(True)
                S.solve(X, B, delta)
            torch.cuda.synchronize()
            l0 = lib.SUNGB300_KernelLaunchCount()
            t0 = time.perf_counter()
            for _ in range(solves):
                S.set_zero_guess(True)
                flag = S.solve(X, B, delta)
            torch.cuda.synchronize()
            el = (time.perf_counter() - t0) / solves
            out[f"{gname}_{'fused' if fused else 'ops'}"] = {
                "ms_per_solve": round(el * 1e3, 4), "flag": int(flag), "nli": S.num_iters,
                "res_norm": S.res_norm, "syncs_per_solve": int(S.num_syncs),
                "launches_per_solve": int((lib.SUNGB300_KernelLaunchCount() - l0) // solves)}
            S.free()
    for g in ("mgs", "cgs"):
        out[f"{g}_fused_speedup"] = round(out[f"{g}_ops"]["ms_per_solve"]
                                          / out[f"{g}_fused"]["ms_per_solve"], 3)
    X.destroy()
    B.destroy()
    H.free()
    return out


def learned_measure(batch, steps=2):
    """The learned Newton predictor end to end: record training rows with the
    plain FP64 solver on training seeds 1001-1004 (8,192 systems each), train
    the BF16 network with the library's kernels, then solve a 16,384-system
    slice of the test batch (every 4th system) in the MIXED form with and
    without the predictor."""
    from sundials_gb300 import learned
    t0 = time.perf_counter()
    X, T = learned.record(8192, range(learned.TRAIN_SEED0, learned.TRAIN_SEED0 + 4), 1 << 20)
    t1 = time.perf_counter()
    from sundials_gb300.mlp import MLP
    net = MLP(seed=7)
    losses = learned.train(net, X, T, epochs=8)
    t2 = time.perf_counter()
    sub = batch.subset(np.arange(0, batch.nsys, 4))
    ev = learned.evaluate(sub, net, repeats=steps)
    out = {"training_rows": int(X.shape[0]), "record_s": round(t1 - t0, 3),
           "train_s": round(t2 - t1, 3), "loss_first_last": [losses[0], losses[-1]],
           "target_variance": round(float(T.var().item()), 4), "systems": int(sub.nsys)}
    for k in ("plain", "learned"):
        r = ev[k]
        out[k] = {"systems_per_s": round(sub.nsys / (r["kernel_ms"] / 1e3), 1),
                  "kernel_ms": round(r["kernel_ms"], 2), "nni": r["nni"], "nfe": r["nfe"],
                  "nst": r["nst"], "failed": r["failed"]}
        if k == "learned":
            out[k]["predictor_calls"], out[k]["learned_iterate_kept"] = r["calls"], r["kept"]
    out["speedup_learned_vs_plain"] = round(ev["plain"]["kernel_ms"] / ev["learned"]["kernel_ms"], 3)
    return out


def fp64_peak_tflops():
    """Dense FP64 rate of this GPU, measured live with a float64 matmul."""
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        a @ b
    e1.record()
    torch.cuda.synchronize()
    return 5 * 2 * 4096 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12


# --------------------------------------------------------- kinetics workload
GOLD = ROOT / "tests" / "golden" / "kinetics_cvode_ref.npz"
RTOL, ATOL, TOUT = 1e-6, 1e-12, 100.0


def fp64_flops_per_system(st, n, refine):
    """Algorithmic FP64 floating-point work of one system's integration in the
    MIXED form, from its counters: per Newton iteration the refinement
    residual (2n^2 per sweep) and the corrector algebra (~12n), per f
    evaluation ~6n (2n reactions), per setup the Newton-matrix formation
    (2n^2) and the Jacobian (~9n), per step ~(4q+12)n for prediction,
    history update, weights and norms (q ~ 3)."""
    n = n.astype(np.float64)
    return (st["nni"] * (2.0 * refine * n * n + 12.0 * n) + st["nfe"] * 6.0 * n
            + st["nsetups"] * (2.0 * n * n + 9.0 * n) + st["nst"] * 24.0 * n)


def wrms_rtol_units(y, yt):
    return float(np.sqrt(np.mean(((y - yt) / (RTOL * np.abs(yt) + ATOL)) ** 2)))


def accuracy_vs_oracle(batch, yout):
    """Error against the FP64 oracle on the golden sample (systems 0, 64, ...)."""
    if not GOLD.exists():
        return None
    g = np.load(GOLD)
    ids = g["r6_ids"]
    if ids.max() >= batch.nsys:
        return None
    sub_off = np.zeros(ids.size + 1, np.int64)
    sub_off[1:] = np.cumsum(batch.n[ids])
    errs, errs_ref = [], []
    for k, i in enumerate(ids):
        y = yout[batch.y_off[i]:batch.y_off[i + 1]]
        yt = g["truth_y"][sub_off[k]:sub_off[k + 1]]
        yr = g["r6_y"][sub_off[k]:sub_off[k + 1]]
        errs.append(wrms_rtol_units(y, yt))
        errs_ref.append(wrms_rtol_units(yr, yt))
    e, r = np.array(errs), np.array(errs_ref)
    return {"systems": int(ids.size), "unit": "WRMS error vs FP64 oracle, in units of rtol",
            "median": round(float(np.median(e)), 3), "p99": round(float(np.percentile(e, 99)), 3),
            "max": round(float(e.max()), 3),
            "reference_cvode": {"median": round(float(np.median(r)), 3),
                                "p99": round(float(np.percentile(r, 99)), 3),
                                "max": round(float(r.max()), 3)}}


def time_batch(B, d_y0, d_yout, d_stats, steps, warmup, flush):
    """Per-step kernel time (CUDA events on the integrator's stream, L2 flushed
    between steps outside the timed region); returns the list of seconds."""
    import torch
    for _ in range(warmup):
        B.solve_device(d_y0.data_ptr(), d_yout.data_ptr(), d_stats.data_ptr(), TOUT)
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        B.solve_device(d_y0.data_ptr(), d_yout.data_ptr(), d_stats.data_ptr(), TOUT)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    return times


def run_kinetics(args, world, rank, local):
    import torch
    from sundials_gb300 import _lib, kinetics as K
    from sundials_gb300.batch import BatchBDF

    lib = _lib.load()
    torch.cuda.set_device(local)
    # weak scaling: every rank integrates its own 65,536-system batch
    nsys = args.nsys
    batch = K.generate(nsys, seed=rank_seed(rank))
    stats_bytes = K.BATCH_STATS_DTYPE.itemsize * nsys
    d_y0 = torch.from_numpy(batch.y0.copy()).cuda()
    d_yout = torch.zeros_like(d_y0)
    d_stats = torch.zeros(stats_bytes, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # ---- headline: MIXED form (launch plan picked by the autotuner on every
    # 2nd system; the plain form below is tuned the same way)
    B = BatchBDF(batch).configure(RTOL, ATOL, "mixed", refine=args.refine)
    tune_mixed = B.autotune(stride=2)
    barrier(world)
    clocks = ClockSampler()
    if rank == 0:
        clocks.start()
    l0 = lib.SUNGB300_KernelLaunchCount()
    times = time_batch(B, d_y0, d_yout, d_stats, args.steps, args.warmup, flush)
    launches = (lib.SUNGB300_KernelLaunchCount() - l0) * args.steps // (args.steps + args.warmup)
    ck = clocks.stop(local) if rank == 0 else None
    elapsed = max_over_ranks(world, float(np.sum(times)))
    value = weak_value(nsys, args.steps, world, elapsed)
    yout_mixed = d_yout.cpu().numpy()
    st = np.frombuffer(d_stats.cpu().numpy().tobytes(), K.BATCH_STATS_DTYPE)

    # ---- e2e through the C ABI with host buffers (H2D y0, solve, D2H y, stats)
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    barrier(world)
    te = time.perf_counter()
    for _ in range(e2e_steps):
        y_host, st_host = B.solve(TOUT)
    e2e_el = max_over_ranks(world, time.perf_counter() - te)
    e2e = weak_value(nsys, e2e_steps, world, e2e_el)

    # ---- roofline of the integrator: FP64 work vs the live FP64 rate
    flops = float(np.sum(fp64_flops_per_system(st, batch.n, args.refine)))
    fp64_peak = fp64_peak_tflops()
    achieved_tf = flops / float(np.mean(times)) / 1e12

    # ---- plain FP64 GPU form of the same solver
    B64 = BatchBDF(batch).configure(RTOL, ATOL, "fp64")
    tune_fp64 = B64.autotune(stride=2)
    t64 = time_batch(B64, d_y0, d_yout, d_stats, max(1, args.steps // 2), 1, flush)
    plain = weak_value(nsys, 1, world, max_over_ranks(world, float(np.mean(t64))))
    yout_plain = d_yout.cpu().numpy()

    # ---- the N_Vector microbenchmark
    nv = nvector_measure(args, rank, local, steps=10, warmup=3) if not args.no_nvector else None
    spg = spgmr_measure() if not args.no_spgmr else None
    lrn = learned_measure(batch) if not args.no_learned else None

    if rank != 0:
        return None
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "systems/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(float(np.mean(times)) * 1e3, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (FP32 Newton-matrix inverse)",
        "data": "synthetic (seeded mass-action networks, sundials_gb300/kinetics.py)",
        "config": {"workload": f"uneven stiff kinetics batch: {nsys:,} mass-action systems, "
                               "n ~ U{8..64}, 2n reactions", "systems": nsys,
                   "species": "U{8..64}", "reactions_per_system": "2n", "rtol": RTOL,
                   "atol": ATOL, "t": [0.0, TOUT], "method": "BDF q<=5, Newton, dense",
                   "form": f"MIXED (FP32 Gauss-Jordan inverse + {args.refine} FP64 refinement sweep)",
                   "l2": "512 MB buffer written between timed steps (flush)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single"},
        "plain_fp64_gpu": {"value": round(plain, 1), "unit": "systems/s",
                           "ms_per_step": round(float(np.mean(t64)) * 1e3, 2),
                           "launch_plan": B64.launch_plan(),
                           "autotune_ms": {k: round(v, 2) for k, v in tune_fp64.items()}},
        "launch_plan": B.launch_plan(),
        "autotune_ms": {k: round(v, 2) for k, v in tune_mixed.items()},
        "speedup_vs_plain_fp64_gpu": round(value / plain, 3),
        "counters_mean": {f: round(float(st[f].mean()), 2) for f in
                          ("nst", "nfe", "nni", "nsetups", "nje", "netf", "ncfn")},
        "failed_systems": int(np.sum(st["flag"] != 0)),
        "accuracy": {"mixed": accuracy_vs_oracle(batch, yout_mixed),
                     "plain_fp64": accuracy_vs_oracle(batch, yout_plain)},
        "roofline": {"bound": "fp64", "kernel": "k_batch_bdf<MIXED> (both size buckets)",
                     "achieved": round(achieved_tf, 4), "peak": round(fp64_peak, 3),
                     "unit": "TFLOP/s", "frac": round(achieved_tf / fp64_peak, 4),
                     "peak_source": "float64 matmul measured live in this run",
                     "traffic": None,
                     "algorithmic_flops_per_step": flops},
        "e2e": {"value": round(e2e, 1), "unit": "systems/s",
                "h2d_bytes_per_step": int(8 * batch.y0.size),
                "d2h_bytes_per_step": int(8 * batch.y0.size + stats_bytes)},
        "gpu_launches": int(launches),
        "clocks": ck,
    }
    if nv:
        out["nvector"] = nv
    if spg:
        out["spgmr"] = spg
    if lrn:
        out["learned_predictor"] = lrn
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = kinetics_cpu_sample(batch, threads=1, target_s=args.cpu_seconds)
    return out


def kinetics_cpu_sample(batch, threads, target_s):
    """The CVODE restatement on host cores over a bounded sample of the batch
    (systems spread over the batch, every 16th), until target_s of CPU work."""
    from oracle import port
    idx = np.arange(0, batch.nsys, 16)
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    done, t_total = 0, 0.0
    chunk = 64 * cores
    for start in range(0, idx.size, chunk):
        sub = batch.subset(idx[start:start + chunk])
        t0 = time.perf_counter()
        port.bdf_batch(sub, RTOL, ATOL, TOUT, threads=cores)
        t_total += time.perf_counter() - t0
        done += sub.nsys
        if t_total >= target_s:
            break
    return {"value": round(done / t_total, 2), "unit": "systems/s", "cores": cores,
            "kind": "port",
            "sample": f"{done} systems (every 16th of the batch) in {t_total:.1f} s on {cores} "
                      "host thread(s); the CVODE restatement, bit-identical to the reference's "
                      "CVODE on the golden systems"}


def run_reference(args, world, rank):
    if rank != 0:
        return None
    from sundials_gb300 import kinetics as K
    batch = K.generate(args.nsys, seed=1)
    for _ in range(args.warmup):
        kinetics_cpu_sample(batch, threads=0, target_s=1.0)
    vals = []
    cb = None
    for _ in range(args.steps):
        cb = kinetics_cpu_sample(batch, threads=0, target_s=args.ref_seconds)
        vals.append(cb["value"])
    value = float(np.median(vals))
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": "systems/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(args.nsys / value * 1e3, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"uneven stiff kinetics batch: {args.nsys:,} mass-action systems, "
                               "n ~ U{8..64}, 2n reactions", "systems": args.nsys,
                   "rtol": RTOL, "atol": ATOL, "t": [0.0, TOUT]},
        "cpu_baseline": {"value": round(value, 2), "unit": "systems/s", "cores": cb["cores"],
                         "kind": "port", "sample": cb["sample"]},
        "e2e": {"value": round(value, 2), "unit": "systems/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--nsys", type=int, default=65536)
    ap.add_argument("--refine", type=int, default=1)
    ap.add_argument("--log2n", type=int, default=28)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-nvector", action="store_true")
    ap.add_argument("--no-spgmr", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--spgmr-only", action="store_true",
                    help="print only the SPGMR heat-2D measurement (no kinetics line)")
    ap.add_argument("--spgmr-solves", type=int, default=20)
    ap.add_argument("--nvector-only", action="store_true",
                    help="print only the N_Vector microbenchmark (no kinetics line)")
    args = ap.parse_args()
    if args.nvector_only:
        import torch
        torch.cuda.init()
        print(json.dumps(nvector_measure(args, 0, 0, steps=max(args.steps, 5), warmup=args.warmup)),
              flush=True)
        return
    if args.spgmr_only:
        print(json.dumps(spgmr_measure(solves=args.spgmr_solves, warmup=args.warmup)), flush=True)
        return
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_kinetics(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

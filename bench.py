#!/usr/bin/env python3
"""Benchmark of the GB300 SUNDIALS hot path.

Workload ``nvector`` (default; the N_Vector microbenchmark of the 2-D heat
configuration): FP64 vectors of length 2^28, values uniform[-1, 1], weights
1/(1e-6|y| + 1e-10).  One step = LinearSum + LinearCombination(5 vectors) +
DotProdMulti(5 vectors) + WrmsNorm through the N_Vector ops table, i.e.
(24 + 48 + 48 + 16) bytes per element of algorithmic HBM traffic.  Every
vector is 2 GiB, far above the 129 MB L2, so no L2 flush is needed between
steps.  The metric is HBM GB/s over the whole step.

``--impl reference`` times the reference's CPU algorithm for the same step on
the host cores (the oracle's restatement of NVECTOR_SERIAL arithmetic, split
across all threads like NVECTOR_OPENMP).

Output: ONE JSON line on rank 0.
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
NV_BYTES = {"LinearSum": 24, "LinearCombination5": 48, "DotProdMulti5": 48, "WrmsNorm": 16}


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
def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# --------------------------------------------------------- nvector workload
def gen_inputs(n, seed=1):
    rng = np.random.default_rng(seed)
    xs = [rng.uniform(-1.0, 1.0, n) for _ in range(6)]
    y = rng.uniform(-1.0, 1.0, n)
    w = 1.0 / (1e-6 * np.abs(y) + 1e-10)
    c5 = rng.uniform(-1.0, 1.0, 5)
    return xs, y, w, c5


def nvector_cpu_sample(n, threads_all: bool, target_s=10.0):
    """Time the step's four operations with the oracle's CPU code."""
    from oracle import port
    L = port.omp()
    xs, y, w, c5 = gen_inputs(n, seed=1)
    z = np.empty(n)
    z2 = np.empty(n)
    P = port.ptr
    d = (ct.c_double * 5)()
    if not threads_all:
        os.environ["OMP_NUM_THREADS"] = "1"

    def step():
        if threads_all:
            L.omp_linearsum(0.3, P(xs[0]), 0.7, P(y), P(z), n)
            L.omp_linearcombination(5, P(c5), port.ptrs(xs[:5]), P(z2), n)
            L.omp_dotprodmulti(5, P(xs[5]), port.ptrs(xs[:5]), d, n)
            L.omp_wrmsnorm(P(xs[0]), P(w), n)
        else:
            L.port_linearsum(0.3, P(xs[0]), 0.7, P(y), P(z), n)
            L.port_linearcombination(5, P(c5), port.ptrs(xs[:5]), P(z2), n)
            L.port_dotprodmulti(5, P(xs[5]), port.ptrs(xs[:5]), d, n)
            L.port_wrmsnorm(P(xs[0]), P(w), n)

    step()
    reps, t0 = 0, time.perf_counter()
    while True:
        step()
        reps += 1
        el = time.perf_counter() - t0
        if el >= target_s or reps >= 1000:
            break
    bytes_step = sum(NV_BYTES.values()) * n
    return bytes_step * reps / el / 1e9, reps, el, (L.omp_threads() if threads_all else 1)


def run_nvector(args, world, rank, local):
    import torch
    from sundials_gb300 import _lib
    from sundials_gb300.nvector import NVector

    lib = _lib.load()
    torch.cuda.set_device(local)
    n = 1 << args.log2n
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    xs, y, w, c5 = gen_inputs(n, seed=1 + rank)
    X = [NVector.from_numpy(a, stream=sp) for a in xs]
    Y = NVector.from_numpy(y, stream=sp)
    W = NVector.from_numpy(w, stream=sp)
    Z = NVector(n, stream=sp)
    Z2 = NVector(n, stream=sp)
    ops = Z.ops
    c5a = _lib.real_array(c5)
    arrX = _lib.nv_array([v.v for v in X[:5]])
    dots = (ct.c_double * 5)()

    evs = {k: [] for k in NV_BYTES}

    def step(timed):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(5)] if timed else None
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
            for k, name in enumerate(NV_BYTES):
                evs[name].append((e[k], e[k + 1]))

    for _ in range(args.warmup):
        step(False)
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler()
    if rank == 0:
        clocks.start()
    l0 = lib.SUNGB300_KernelLaunchCount()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        step(True)
    t1.record(stream)
    torch.cuda.synchronize()
    launches = lib.SUNGB300_KernelLaunchCount() - l0
    elapsed = t0.elapsed_time(t1) / 1e3
    barrier(world)
    ck = clocks.stop(local) if rank == 0 else None
    elapsed = max_over_ranks(world, elapsed)
    bytes_step = sum(NV_BYTES.values()) * n
    value = bytes_step * args.steps * world / elapsed / 1e9
    per_op = {}
    for name, lst in evs.items():
        ms = float(np.mean([a.elapsed_time(b) for a, b in lst]))
        per_op[name] = {"ms": ms, "GBs": NV_BYTES[name] * n / (ms / 1e3) / 1e9}

    # end to end through the C ABI with host buffers: H2D of every input of the
    # step, the four operations, D2H of both output vectors.
    h2d = (6 + 2) * 8 * n
    d2h = 2 * 8 * n
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    barrier(world)
    te = time.perf_counter()
    for _ in range(e2e_steps):
        for v in X + [Y, W]:
            lib.N_VCopyToDevice_GB300(v.v)
        step(False)
        lib.N_VCopyFromDevice_GB300(Z.v)
        lib.N_VCopyFromDevice_GB300(Z2.v)
    torch.cuda.synchronize()
    e2e_el = max_over_ranks(world, time.perf_counter() - te)
    e2e = bytes_step * e2e_steps * world / e2e_el / 1e9

    if rank != 0:
        return None
    hbm, src = peaks()
    dom = "LinearCombination5"
    achieved = per_op[dom]["GBs"]
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(elapsed / args.steps * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "nvector_microbench_2^%d" % args.log2n,
                   "ops": list(NV_BYTES), "vector_length": n,
                   "bytes_per_elem_step": sum(NV_BYTES.values()),
                   "l2": "inputs larger than L2 (2 GiB per vector), no flush",
                   "parallelism": "replicas" if world > 1 else "single"},
        "per_op": {k: {"ms": round(v["ms"], 4), "GBs": round(v["GBs"], 1)} for k, v in per_op.items()},
        "roofline": {"bound": "hbm", "kernel": "k_lincomb (LinearCombination, 5 vectors)",
                     "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "peak_source": src,
                     "traffic": None},
        "e2e": {"value": round(e2e, 2), "unit": "GB/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": ck,
    }
    if not args.no_cpu_baseline:
        ncpu = 1 << 24
        gbs, reps, el, cores = nvector_cpu_sample(ncpu, threads_all=False, target_s=args.cpu_seconds)
        out["cpu_baseline"] = {"value": round(gbs, 2), "unit": "GB/s", "cores": cores,
                               "kind": "port",
                               "sample": f"{reps} steps of the 4 ops at length 2^24 on 1 core "
                                         f"({el:.1f} s), oracle NVECTOR_SERIAL restatement"}
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return None
    n = 1 << min(args.log2n, 26)
    steps = []
    for _ in range(args.warmup):
        nvector_cpu_sample(n, threads_all=True, target_s=0.0)
    gbs_list = []
    cores = 1
    for _ in range(args.steps):
        gbs, reps, el, cores = nvector_cpu_sample(n, threads_all=True, target_s=0.0)
        gbs_list.append(gbs)
    value = float(np.median(gbs_list))
    ms = sum(NV_BYTES.values()) * n / (value * 1e9) * 1e3
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "nvector_microbench_2^%d" % args.log2n,
                   "ops": list(NV_BYTES), "vector_length_sampled": n},
        "cpu_baseline": {"value": round(value, 2), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": f"each step = the 4 ops once at length 2^{int(np.log2(n))} "
                                   "on all host threads (OpenMP)"},
        "e2e": {"value": round(value, 2), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--log2n", type=int, default=28)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_nvector(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

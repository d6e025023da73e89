"""The learned Newton predictor's pipeline: training data recorded by the plain
FP64 integrator on the training seeds, training by the library's own BF16
tensor-core kernels, and an A/B evaluation on held-out systems.

Training data: every converged Newton solve of the plain solver on
``generate(nsys, seed)`` for seeds 1001, 1002, ... (disjoint from the test
seed 1) gives one row -- the solve's features and its converged corrector in
error-weight units (include/sunbatchbdf_gb300.h, SetRecorder); the rows kept
and their order are fixed by their content, so training repeats bit for bit.  Targets are
clipped to +-TARGET_CLIP weighted-RMS units: a guess that far off is never
kept by the integrator's residual test anyway, and unclipped outliers would
dominate the squared loss."""
from __future__ import annotations

import time

import numpy as np

from . import kinetics as K
from .batch import BatchBDF
from .mlp import MLP, IN_PAD, OUT

TRAIN_SEED0 = 1001
TARGET_CLIP = 16.0


def _record_into(nsys, seeds, cap, rtol, atol, tout):
    import torch
    X = torch.zeros((cap, IN_PAD), dtype=torch.int16, device="cuda")
    T = torch.zeros((cap, OUT), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    for seed in seeds:
        B = BatchBDF(K.generate(nsys, seed=seed)).configure(rtol, atol, "fp64")
        B.set_recorder(X.data_ptr(), T.data_ptr(), cap, cnt.data_ptr())
        B.solve(tout)
        B.free()
    return X, T, int(cnt.item())


def _row_keys(X, T, chunk=1 << 20):
    """A 64-bit hash of every row's bits (in chunks, to bound the memory)."""
    import torch
    keys = torch.empty(X.shape[0], dtype=torch.int64, device="cuda")
    width = X.shape[1] // 2 + T.shape[1]
    mult = torch.arange(1, width + 1, device="cuda", dtype=torch.int64) * 2654435761
    for a in range(0, X.shape[0], chunk):
        b = min(a + chunk, X.shape[0])
        words = torch.cat([X[a:b].view(torch.int32), T[a:b].view(torch.int32)], dim=1)
        keys[a:b] = (words.to(torch.int64) * mult).sum(dim=1)
    return keys


def record(nsys: int, seeds, capacity: int, rtol=1e-6, atol=1e-12, tout=100.0):
    """(X, T) device tensors of at most `capacity` training rows (X: BF16 bits
    as int16), the same rows in the same order on every call.  The recorder
    appends rows in the order warps finish their solves and drops those past
    the buffer, so when the solves produce more rows than `capacity` they are
    recorded again into a buffer that holds them all; the rows are then put
    in the order of a hash of their bits and the first `capacity` kept -- a
    fixed pseudo-random subset, so that the shuffled mini-batches and the
    trained weights repeat."""
    import torch
    seeds = list(seeds)
    X, T, total = _record_into(nsys, seeds, capacity, rtol, atol, tout)
    if total > capacity:
        del X, T
        X, T, total = _record_into(nsys, seeds, total, rtol, atol, tout)
    X, T = X[:total], T[:total]
    order = torch.argsort(_row_keys(X, T), stable=True)[:capacity]
    return X[order].contiguous(), T[order].clamp_(-TARGET_CLIP, TARGET_CLIP)


def train(mlp: MLP, X, T, epochs=8, batch=4096, lr=2e-3, seed=0):
    """Adam over shuffled mini-batches (the last partial batch is dropped);
    returns the loss of the last batch of each epoch."""
    import torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    nb = X.shape[0] // batch
    assert nb >= 1, "fewer rows than one batch"
    losses = []
    for _ in range(epochs):
        perm = torch.randperm(X.shape[0], device="cuda", generator=gen)
        loss = None
        for b in range(nb):
            idx = perm[b * batch:(b + 1) * batch]
            xb = X.index_select(0, idx).contiguous()
            tb = T.index_select(0, idx).contiguous()
            loss = mlp.train_step(batch, xb.data_ptr(), tb.data_ptr(), lr, want_loss=(b == nb - 1))
        losses.append(loss)
    return losses


def evaluate(batch: K.KineticsBatch, mlp: MLP, rtol=1e-6, atol=1e-12, tout=100.0, mode="mixed",
             repeats=1):
    """Solve the same systems with and without the predictor: counters,
    kernel time, predictor usage and the final states."""
    out = {}
    for name, use in (("plain", False), ("learned", True)):
        B = BatchBDF(batch).configure(rtol, atol, mode)
        B.set_predictor(mlp if use else None)
        ms = []
        for _ in range(repeats):
            y, st = B.solve(tout)
            ms.append(B.last_kernel_ms)
        res = {"kernel_ms": float(np.min(ms)), "y": y, "stats": st,
               "nni": int(st["nni"].sum()), "nfe": int(st["nfe"].sum()),
               "nst": int(st["nst"].sum()), "nsetups": int(st["nsetups"].sum()),
               "ncfn": int(st["ncfn"].sum()), "failed": int(np.sum(st["flag"] != 0))}
        if use:
            res["calls"], res["kept"] = B.predictor_counts()
        B.free()
        out[name] = res
    return out


def pipeline(train_nsys=8192, seeds=4, capacity=1 << 20, epochs=8, mlp_seed=7):
    """Record, train, return (mlp, info)."""
    t0 = time.perf_counter()
    X, T = record(train_nsys, range(TRAIN_SEED0, TRAIN_SEED0 + seeds), capacity)
    t1 = time.perf_counter()
    mlp = MLP(seed=mlp_seed)
    losses = train(mlp, X, T, epochs=epochs)
    t2 = time.perf_counter()
    return mlp, {"rows": int(X.shape[0]), "record_s": t1 - t0, "train_s": t2 - t1,
                 "losses": losses, "target_var": float(T.var().item())}


def _main(argv=None):
    """Record and train (a profiling and smoke entry):
    python -m sundials_gb300.learned --nsys 2048 --seeds 1 --epochs 1"""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--nsys", type=int, default=2048)
    ap.add_argument("--seeds", type=int, default=1)
    ap.add_argument("--epochs", type=int, default=1)
    ap.add_argument("--capacity", type=int, default=1 << 19)
    args = ap.parse_args(argv)
    _, info = pipeline(args.nsys, args.seeds, args.capacity, args.epochs)
    print(json.dumps(info))


if __name__ == "__main__":
    _main()

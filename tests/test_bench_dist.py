"""CPU: bench.py's multi-process path on 2 gloo ranks (the GPU runs use one
process per GPU over NCCL with the same helpers): the barrier, the max / sum
over ranks, each rank's own batch seed, the whole-job throughput over the
slowest rank, and the reference arm, which only rank 0 runs."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import argparse

    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_setup(world, backend="gloo")
    bench.barrier(w)
    mx = bench.max_over_ranks(w, 1.5 + r)
    sm = bench.sum_over_ranks(w, 1.5 + r)
    # rank 1 is the slow one: the job's throughput is set by its time
    elapsed = bench.max_over_ranks(w, 2.0 if r == 1 else 1.0)
    value = bench.weak_value(1000, 3, w, elapsed)
    ref = bench.run_reference(argparse.Namespace(nsys=64, warmup=0, steps=1, ref_seconds=0.01),
                              w, r) if r != 0 else "rank0"
    Path(out_dir, f"r{r}.txt").write_text(
        f"{w} {r} {local} {mx} {sm} {value} {bench.rank_seed(r)} {ref is None}")
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    rows = [Path(tmp_path, f"r{r}.txt").read_text().split() for r in range(2)]
    for r, row in enumerate(rows):
        w, rank, local = int(row[0]), int(row[1]), int(row[2])
        assert (w, rank, local) == (2, r, r)
        assert float(row[3]) == 2.5 and float(row[4]) == 4.0
        assert float(row[5]) == 1000 * 3 * 2 / 2.0  # both ranks' work over the slower time
    assert int(rows[0][6]) == 1 and int(rows[1][6]) != 1  # rank 0 keeps the seed-1 batch
    assert rows[1][7] == "True"  # the reference arm does no work on rank 1


def test_single_process_helpers_are_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(1, 3.25) == 3.25 and bench.sum_over_ranks(1, 3.25) == 3.25
    assert bench.weak_value(65536, 5, 1, 10.0) == 65536 * 5 / 10.0
    assert len({bench.rank_seed(r) for r in range(8)}) == 8

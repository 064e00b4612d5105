"""Multi-GPU form of the benchmark on CPU ranks (gloo, world size 2).

The path shards by independent blob sets: every rank solves its own seeded
set with no data-path collective, the job time is the slowest rank's, and
the throughput is the sum over ranks.  These tests run the host-side parts
of that (per-rank workloads, the max-over-ranks reduction, the aggregate)
as two gloo processes; no GPU is involved.
"""
from __future__ import annotations

import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import argparse
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, _ = bench.dist_env()
    assert (r, w) == (rank, world)
    args = argparse.Namespace(workload="uniform", n=4000)
    b, name = bench.workload(args, rank)
    local_ms = 10.0 + 5.0 * rank  # rank 1 is the slow replica
    job_ms = bench.max_over_ranks(local_ms, world)
    value = bench.replica_throughput(b.n, 3, job_ms, world)
    np.savez(os.path.join(out_dir, f"r{rank}.npz"), xy=b.xy, job_ms=job_ms, value=value, name=name)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_on_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    r0 = np.load(tmp_path / "r0.npz")
    r1 = np.load(tmp_path / "r1.npz")
    # each replica solves its own set (distinct seeds), of the same size
    assert r0["xy"].shape == r1["xy"].shape and not np.array_equal(r0["xy"], r1["xy"])
    # the job time is the slowest rank's, the same on every rank
    assert float(r0["job_ms"]) == float(r1["job_ms"]) == 15.0
    # throughput sums the replicas: 2 x 4000 targets x 3 steps in 15 ms
    assert float(r0["value"]) == pytest.approx(2 * 4000 * 3 / 15e-3)
    assert str(r0["name"]) == "uniform_4000"

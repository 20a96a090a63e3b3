"""The multi-process path of bench.py on CPU (gloo, world size 2): one process per GPU in
production, each tracing its own rays (no data exchanged) -- the rank seeds differ, the
barrier and the max-over-ranks timing agree on every rank, and the whole-job rate is every
rank's rays over the slowest rank's time. The reference arm runs on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, root):
    import sys

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, root)
    import torch

    import bench

    dist, r, ws = bench._dist()
    assert (r, ws) == (rank, world) and dist.get_backend() == "gloo"
    bench._sync_all(dist, torch)
    assert bench._max_over_ranks(dist, torch, float(rank + 1)) == float(world)
    # rank k traces 100 (k + 1) rays in 0.5 (k + 1) s: 300 rays over the slowest rank's 1 s
    assert bench._job_rate(dist, torch, 100.0 * (rank + 1), 0.5 * (rank + 1)) == pytest.approx(300.0)
    seeds = [None] * world
    dist.all_gather_object(seeds, bench._rank_seed(bench.SEED, rank))
    assert len(set(seeds)) == world
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    mp.spawn(_worker, args=(2, _free_port(), root), nprocs=2, join=True)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.run_reference(None) is None  # returns at once, no work, no output

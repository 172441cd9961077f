"""Multi-GPU host logic (replicas only) on CPU: two gloo ranks."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    from vlapy_gb300 import replicas
    replicas.init(world, backend="gloo")
    replicas.barrier(world)
    # rank r took 10 + r ms for 100 (r + 1) units
    t_max, total, rate = replicas.aggregate(10.0 + rank, 100.0 * (rank + 1), world)
    out[rank] = (t_max, total, rate)
    dist.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    world, port = 2, _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        t_max, total, rate = out[r]
        assert t_max == 11.0 and total == 300.0
        assert rate == pytest.approx(300.0 / 0.011)


def test_shards_are_disjoint_and_complete():
    from vlapy_gb300.replicas import shard_runs, shard_seed
    from vlapy_gb300.sweep import sweep_config
    runs = list(range(4097))
    for world in (1, 2, 3, 8):
        parts = [shard_runs(runs, r, world) for r in range(world)]
        assert sum(parts, []) == runs
        assert max(map(len, parts)) - min(map(len, parts)) <= 1
    assert shard_seed(20261203, 0) == 20261203
    a = sweep_config(64, shard_seed(20261203, 0))
    b = sweep_config(64, shard_seed(20261203, 1))
    assert a != b and len(a) == len(b) == 64


def test_single_rank_needs_no_process_group():
    from vlapy_gb300 import replicas
    replicas.init(1)
    assert not dist.is_initialized()
    assert replicas.aggregate(20.0, 1000.0, 1) == (20.0, 1000.0, 1000.0 / 0.02)

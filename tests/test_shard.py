"""Batch sharding over ranks: LPT partition properties and the host-side
gather, run as world_size-2 gloo process groups on the CPU (no GPU)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from superfluid_dynamics_gb300 import shard, workloads


def test_lpt_partition_covers_and_balances():
    sizes = [s.n for s in workloads.helium_batch(512, seed=3)]
    for nr in (1, 2, 3, 4, 8):
        parts = shard.lpt_partition(sizes, nr)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = shard.rank_loads(sizes, parts)
        ideal = sum(loads) / nr
        biggest = max(shard.surface_cost(n) for n in sizes)
        # LPT bound: makespan <= ideal + the largest single job
        assert max(loads) <= ideal + biggest
        if nr > 1:
            assert max(loads) / min(loads) < 1.02


def test_lpt_is_deterministic():
    sizes = [128, 2048, 640, 2048, 96, 1024]
    assert shard.lpt_partition(sizes, 2) == shard.lpt_partition(list(sizes), 2)
    p = shard.lpt_partition(sizes, 2)
    assert {1, 3} & set(p[0]) and {1, 3} & set(p[1])  # the two largest go to different ranks


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        parts = shard.lpt_partition(sizes, world)
        local = {i: np.full(3 * sizes[i], float(i)) + np.arange(3 * sizes[i]) * 1e-3 for i in parts[rank]}
        res = shard.gather_states(local, len(sizes))
        if rank == 0:
            np.save(out_path, np.array([r.sum() for r in res]))
    finally:
        dist.destroy_process_group()


def test_gather_two_ranks_gloo(tmp_path):
    sizes = [s.n for s in workloads.helium_batch(24, seed=3)]
    out = str(tmp_path / "sums.npy")
    mp.start_processes(_worker, args=(2, _free_port(), sizes, out), nprocs=2, start_method="spawn")
    got = np.load(out)
    want = np.array([(np.full(3 * n, float(i)) + np.arange(3 * n) * 1e-3).sum() for i, n in enumerate(sizes)])
    assert np.allclose(got, want, rtol=0, atol=1e-9)

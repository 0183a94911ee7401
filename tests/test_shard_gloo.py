"""Multi-rank host logic on CPU: scene sharding and the gather of recorder
histories to rank 0, with two gloo ranks (world size 2).  No GPU."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from ard_gb300 import shard


def test_assign_is_a_balanced_partition():
    rng = np.random.default_rng(0)
    costs = [int(c) for c in rng.integers(1000, 100000, size=37)]
    for world in (1, 2, 3, 8):
        owned = shard.assign(costs, world)
        flat = sorted(i for o in owned for i in o)
        assert flat == list(range(len(costs)))            # every scene exactly once
        loads = [sum(costs[i] for i in o) for o in owned]
        assert max(loads) - min(loads) <= max(costs)      # LPT bound
    assert shard.local_scenes([5], 1, 4) == [0]           # one scene: replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, costs, out_path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    owned = shard.assign(costs, world)
    mine = owned[rank]
    # stand-in histories: scene s has (10 + s) steps and (s % 3) + 1 recorders
    local = [np.full((10 + s, s % 3 + 1), float(s)) + np.arange(10 + s)[:, None] for s in mine]
    got = shard.gather_histories(local, owned, len(costs), dist=dist)
    if rank == 0:
        np.save(out_path, np.array([g.sum() for g in got]))
        for s, g in enumerate(got):
            assert g.shape == (10 + s, s % 3 + 1)
    dist.barrier()
    dist.destroy_process_group()


def test_gather_histories_two_gloo_ranks(tmp_path):
    costs = [3, 9, 4, 4, 7, 1, 8]
    out = str(tmp_path / "sums.npy")
    mp.start_processes(_worker, args=(2, _free_port(), costs, out), nprocs=2, join=True, start_method="spawn")
    sums = np.load(out)
    want = [np.sum(np.full((10 + s, s % 3 + 1), float(s)) + np.arange(10 + s)[:, None]) for s in range(len(costs))]
    np.testing.assert_allclose(sums, want)

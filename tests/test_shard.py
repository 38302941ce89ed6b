"""Multi-GPU host logic on CPU: placing independent scenes on ranks and the
whole-job reduction, including a world-size-2 gloo run (127.0.0.1)."""
import os
import socket

import numpy as np
import pytest

from novaphy_gb300 import shard, workloads


def test_partition_is_complete_disjoint_and_balanced():
    counts = [w.n for w in workloads.batched_scenes(nscenes=64, seed=3)]
    for ws in (1, 2, 3, 8):
        parts = shard.partition_scenes(counts, ws)
        assert len(parts) == ws
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(counts)))
        loads = [sum(counts[i] for i in p) for p in parts]
        # LPT: every rank is within one scene of the lightest
        assert max(loads) - min(loads) <= max(counts)
        assert parts == shard.partition_scenes(counts, ws)  # deterministic


def test_partition_edge_cases():
    assert shard.partition_scenes([], 2) == [[], []]
    assert shard.partition_scenes([5], 3) == [[0], [], []]
    assert shard.partition_scenes([3, 3, 3, 3], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard.partition_scenes([1], 0)
    with pytest.raises(ValueError):
        shard.rank_scenes([1], 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world_size, port, counts, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    mine = shard.rank_scenes(counts, world_size, rank)
    units = float(sum(counts[i] for i in mine))
    seconds = 1.0 + rank  # the slowest rank decides the job time
    total, slowest = shard.job_throughput(units, seconds, dist)
    out[rank] = (mine, units, total, slowest)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_over_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    counts = [w.n for w in workloads.batched_scenes(nscenes=16, seed=5)]
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.spawn(_rank_main, args=(2, _free_port(), counts, out), nprocs=2, join=True)
    (m0, u0, t0, s0), (m1, u1, t1, s1) = out[0], out[1]
    assert sorted(m0 + m1) == list(range(len(counts))) and not set(m0) & set(m1)
    assert t0 == t1 == float(sum(counts)) == u0 + u1
    assert s0 == s1 == 2.0
    assert np.isclose(t0 / s0, sum(counts) / 2.0)

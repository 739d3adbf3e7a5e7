"""The N-GPU bench path on CPU: world shards per rank and the max-over-ranks reduction, run as
two gloo ranks (the GPU run uses the same functions over NCCL)."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world_size, port, out):
    sys.path.insert(0, str(ROOT))
    import bench  # noqa: PLC0415

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    seeds = bench.shard_seeds(rank, world_size, 8)
    ms = 10.0 + rank  # rank 1 is slower: the job time is its time
    ms_max, bodies = bench.reduce_over_ranks(ms, 100 * (rank + 1), "cpu")
    out[rank] = (seeds, ms_max, bodies)
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    s0, m0, b0 = out[0]
    s1, m1, b1 = out[1]
    assert set(s0).isdisjoint(s1) and sorted(s0 + s1) == list(range(16))
    assert m0 == m1 == 11.0
    assert b0 == b1 == 300.0

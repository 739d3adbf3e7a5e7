"""The N-GPU bench path on CPU: cost-balanced world shards per rank, each rank stepping its own
worlds, and the max/sum reductions over ranks, run as two gloo ranks (the GPU run uses the same
functions over NCCL). The worlds are stepped by the CPU oracle here (the engine needs a GPU);
the union of the shards' results must equal one rank stepping every world."""
import ctypes as C
import hashlib
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]
WORLDS_PER_RANK, STEPS = 12, 20


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _step_worlds(seeds):
    """Steps the batched workload's worlds `seeds` on the CPU oracle; returns ({seed: digest of
    its body states}, dynamic bodies, seconds)."""
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import bench  # noqa: PLC0415
    import oracle_bind as ob  # noqa: PLC0415

    orc = ob.Oracle()
    worlds, nb = bench.oracle_batch(orc, seeds)
    hs = (C.c_void_p * max(len(worlds), 1))(*[w.h for w in worlds])
    secs = orc.orc_worlds_step_parallel(hs, len(worlds), 1 / 60, 8, 3, STEPS, 2) if worlds else 0.0
    digests = {s: hashlib.sha256(b"".join(bytes(b)[:40] for b in w.bodies())).hexdigest() for s, w in zip(seeds, worlds)}
    return digests, nb, secs


def _worker(rank, world_size, port, out):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import bench  # noqa: PLC0415
    import oracle_bind as ob  # noqa: PLC0415

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    orc = ob.Oracle()
    seeds = bench.shard_seeds(rank, world_size, WORLDS_PER_RANK, cost=lambda s: orc.batch_world_params(s)[0])
    digests, nb, secs = _step_worlds(seeds)
    ms_max, bodies = bench.reduce_over_ranks(secs * 1e3 / STEPS, nb, "cpu")
    gathered = [None] * world_size
    dist.all_gather_object(gathered, digests)
    out[rank] = (seeds, nb, secs * 1e3 / STEPS, ms_max, bodies, gathered)
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_step_and_reduce():
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    s0, nb0, ms0, max0, bodies0, g0 = out[0]
    s1, nb1, ms1, max1, bodies1, g1 = out[1]
    total = 2 * WORLDS_PER_RANK
    # contiguous, disjoint, covering every world of the job
    assert s0 and s1 and s0 + s1 == list(range(total))
    # balanced by body count: neither shard holds much more than half of the bodies
    assert max(nb0, nb1) < 0.75 * (nb0 + nb1)
    # the reductions: job time = the slower rank's, bodies = the sum
    assert max0 == max1 == max(ms0, ms1)
    assert bodies0 == bodies1 == nb0 + nb1
    assert g0 == g1
    union = {**g0[0], **g0[1]}
    assert sorted(union) == list(range(total))
    # one rank stepping every world gets the same states
    alone, nb_all, _ = _step_worlds(list(range(total)))
    assert union == alone and nb_all == nb0 + nb1


def test_shards_are_contiguous_and_cost_balanced():
    sys.path.insert(0, str(ROOT))
    import bench  # noqa: PLC0415

    cost = lambda s: 1 + (s % 7) * 100  # noqa: E731
    for n in (1, 2, 3, 4, 8):
        shards = [bench.shard_seeds(r, n, 64, cost=cost) for r in range(n)]
        assert sum(shards, []) == list(range(64 * n))
        loads = [sum(cost(s) for s in sh) for sh in shards]
        assert max(loads) - min(loads) <= 2 * max(cost(s) for s in range(64 * n))
    assert bench.shard_seeds(1, 2, 5) == [5, 6, 7, 8, 9]  # equal counts without a cost

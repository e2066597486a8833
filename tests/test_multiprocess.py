"""Multi-rank path on CPU: world_size-2 gloo ranks each price a shard of one
seeded workload (with the oracle, since this runs without a GPU) and the
gathered prices equal a single-process run; the partition covers every
option exactly once with balanced work."""
import os
import socket

import numpy as np
import pytest

from fd_adi_gb300.shard import partition

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _work(n=8, seed=5):
    from fd_adi_gb300 import mesh
    rng = np.random.RandomState(seed)
    out = []
    for k in range(n):
        K = 100 * rng.uniform(0.8, 1.2)
        nS = int(rng.choice([16, 24, 32]))
        nv = int(rng.choice([8, 12]))
        S, v = mesh.heston_meshes(100., K, 0.04, nS, nv, 8 * K, 5.0)
        p = (0.05, rng.uniform(1, 3), 0.04, rng.uniform(0.2, 0.6), -0.5)
        out.append((K, S, v, p))
    return out


def _price_shard(work, idx):
    from oracle import oracle as O
    from fd_adi_gb300 import mesh
    res = {}
    for k in idx:
        K, S, v, p = work[k]
        V0 = np.maximum(S[:, None] - K, 0) * np.ones((1, v.size))
        V = O.heston_solve(S, v, *p, V0, [("implicit", 2, 0.025, 1.0), ("hv", 9, 0.05, 0.6)])
        res[k] = float(V[mesh.price_index(S, v, 100., 0.04)])
    return res


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    work = _work()
    costs = [w[1].size * w[2].size for w in work]
    mine = partition(costs, world)[rank]
    res = _price_shard(work, mine)
    gathered = [None] * world
    dist.all_gather_object(gathered, res)
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        merged = {}
        for g in gathered:
            merged.update(g)
        q.put(merged)


def test_partition_balanced_and_complete():
    rng = np.random.RandomState(0)
    costs = rng.randint(64, 512, 4096) * rng.randint(32, 256, 4096)
    parts = partition(costs, 8)
    allidx = sorted(i for p in parts for i in p)
    assert allidx == list(range(4096))
    loads = [costs[p].sum() for p in parts]
    assert max(loads) / min(loads) < 1.01


def test_gloo_two_ranks_match_single_process():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    work = _work()
    single = _price_shard(work, range(len(work)))
    assert sorted(merged) == sorted(single)
    for k in single:
        assert merged[k] == single[k]

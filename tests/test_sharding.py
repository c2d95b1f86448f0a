"""Multi-GPU host logic on CPU: facet sharding and the max-over-ranks step time, two gloo ranks."""
import os
import socket

import numpy as np
import pytest

from bullseye_gb300.sharding import facet_shard


@pytest.mark.parametrize("n,world", [(16, 1), (16, 2), (17, 4), (3, 8), (96, 8)])
def test_shards_cover_facets_once(n, world):
    seen = []
    sizes = []
    for r in range(world):
        rg = facet_shard(n, world, r)
        seen.extend(rg)
        sizes.append(len(rg))
    assert seen == list(range(n))
    assert max(sizes) - min(sizes) <= 1


def test_bad_rank():
    with pytest.raises(ValueError):
        facet_shard(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n_facets, q):
    import torch.distributed as dist
    from bullseye_gb300.sharding import facet_shard, max_over_ranks
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        mine = list(facet_shard(n_facets, world, rank))
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        t = max_over_ranks(10.0 + rank)
        q.put((rank, gathered, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world, n = 2, 16
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, t in out:
        assert sorted(f for part in gathered for f in part) == list(range(n))
        assert all(len(set(a) & set(b)) == 0 for i, a in enumerate(gathered) for b in gathered[i + 1:])
        assert t == 11.0  # max over ranks of 10 + rank


def test_shard_problem_cuts_facets_and_their_jones_terms():
    from bullseye_gb300 import synth
    from bullseye_gb300.sharding import shard_problem
    p = synth.small_problem("double", nx=48, n_ant=5, n_times=4, n_chan=2, n_facets=5, jones=True)
    seen = []
    for r in range(2):
        q, rg = shard_problem(p, 2, r)
        assert q.n_facets == len(rg) and q.rows == p.rows
        assert np.array_equal(q.facet_centres, p.facet_centres[rg.start:rg.stop])
        for i, f in enumerate(rg):  # [T][A][F][S][Ch][4]: facet i of the shard is facet f of the field
            assert np.array_equal(q.jones[:, :, i], p.jones[:, :, f])
        seen.extend(rg)
    assert seen == list(range(5))

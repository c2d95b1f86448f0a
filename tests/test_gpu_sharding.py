"""Facet sharding through the CUDA library: two ranks, each gridding its own facets.

Two processes (a gloo process group on 127.0.0.1, both on cuda:0) each take a disjoint facet range
of a four-facet field with Jones terms, grid it with the 64-bit library through the reference's
call sequence (the rows replicated, the Jones terms cut to the rank's facets), and gather their
grids on rank 0.  The gathered grids must equal a single-process run over the whole field to
1e-12, as the reference's OpenMP loop over facets (bullseye/mo/cpu_algorithm/templated_gridder.h:
29-30) would produce them.  The ranks' kernels wait on nothing: no data-path collective.
"""
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem():
    from bullseye_gb300 import synth
    return synth.small_problem("double", nx=64, n_ant=6, n_times=8, n_chan=2, n_facets=4, jones=True, s=4, os=9,
                               wplanes=4, min_support=5)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    from bullseye_gb300.imaging import run_imaging
    from bullseye_gb300.library import check, load_library
    from bullseye_gb300.sharding import shard_problem
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        sub, rg = shard_problem(_problem(), world, rank)
        lib = load_library("GPU", "double")
        res = run_imaging(lib, sub, "facet_4_cor_corrections", repack=True, keep_raw=True, uniform=True,
                          norm_bins=(2 * sub.conv_support + 1) ** 2)
        check(lib)
        parts = [None] * world
        dist.all_gather_object(parts, (list(rg), res.raw_grid, res.grid, res.normalization))
        if rank == 0:
            q.put(parts)
    except Exception as exc:  # reported to the test process
        q.put(repr(exc))
        raise
    finally:
        dist.destroy_process_group()


def test_two_ranks_grid_their_facets_like_one_process(gpu_required, built_libraries):
    import torch.multiprocessing as mp
    from bullseye_gb300.imaging import run_imaging
    from bullseye_gb300.library import check, load_library
    p = _problem()
    lib = load_library("GPU", "double")
    full = run_imaging(lib, p, "facet_4_cor_corrections", repack=True, keep_raw=True, uniform=True,
                       norm_bins=(2 * p.conv_support + 1) ** 2)
    check(lib)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port, world = _free_port(), 2
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for pr in procs:
        pr.start()
    parts = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    assert not isinstance(parts, str), parts
    facets = [f for rg, *_ in parts for f in rg]
    assert facets == [0, 1, 2, 3]
    raw = np.concatenate([x[1] for x in parts])
    grid = np.concatenate([x[2] for x in parts])
    norm = np.concatenate([x[3] for x in parts])
    s = np.max(np.abs(full.raw_grid))
    assert s > 0
    assert np.max(np.abs(raw - full.raw_grid)) / s <= 1e-12
    assert np.max(np.abs(norm - full.normalization)) / np.max(np.abs(full.normalization)) <= 1e-12
    assert np.max(np.abs(grid - full.grid)) / np.max(np.abs(full.grid)) <= 1e-10

"""Facet sharding across GPUs.

Facets are independent: every facet grids the whole visibility stream into its own grid, and the
reference parallelises exactly this way on the CPU (bullseye/mo/cpu_algorithm/templated_gridder.h:29,
an OpenMP loop over facets).  Ranks therefore take disjoint facet ranges with the visibilities
replicated, and nothing is exchanged on the data path; the only collective is the max over ranks of
a step time.
"""
from __future__ import annotations


def facet_shard(n_facets: int, world: int, rank: int) -> range:
    """Contiguous, balanced facet range of ``rank`` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(int(n_facets), world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of ``value`` over the ranks of the default process group (the value when none)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_problem(problem, world: int, rank: int):
    """The part of a faceted problem that ``rank`` grids: its facet range's centres and the Jones
    terms of those facets (the terms are laid out [time][antenna][facet][spw][channel][4], so the
    facet axis is cut), with every row replicated.  Returns (sub-problem, facet range)."""
    from dataclasses import replace
    if problem.facet_centres is None:
        raise ValueError("facet sharding needs a faceted problem")
    rg = facet_shard(problem.n_facets, world, rank)
    jones = None if problem.jones is None else problem.jones[:, :, rg.start:rg.stop].copy()
    return replace(problem, facet_centres=problem.facet_centres[rg.start:rg.stop].copy(), jones=jones), rg

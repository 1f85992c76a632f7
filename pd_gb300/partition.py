"""A batch of independent cloths split across ranks (one process per GPU).

The cloths of a batch never exchange data, so a batch shards with no collective on the data path:
each rank creates a simulator for its own part of the batch on its own GPU and steps it; the final
states come back to rank 0 in one gather at the end. The reference has no counterpart (it steps one
cloth on the host cores, core/math/Parallel.cpp).

The split is longest-processing-time first: cloths in decreasing order of estimated cost, each to
the rank with the least work so far (ties to the lower rank), then each rank's cloths in batch
order. It depends only on the cloths' sizes, so every rank computes the same split alone.
"""
from __future__ import annotations

import math

import numpy as np


def instance_cost(n_vertices: int, n_edges: int, n_bends: int, iterations: int) -> float:
    """Relative cost of one substep of a cloth: iterations × (the edge, bend and vertex work plus the
    solve, whose nested-dissection factor grows as n·log n)."""
    n = max(1, int(n_vertices))
    return float(max(1, iterations)) * (4.0 * n * math.log2(n + 1) + 8.0 * n_edges + 4.0 * n_bends + 4.0 * n)


def scene_costs(scenes, cfgs) -> list[float]:
    return [instance_cost(s.n, int(np.asarray(s.edges).reshape(-1, 2).shape[0]),
                          int(np.asarray(s.bends).reshape(-1, 3).shape[0]), c.max_iterations)
            for s, c in zip(scenes, cfgs)]


def partition(costs, world: int) -> list[list[int]]:
    """Indices of the cloths each of `world` ranks steps (longest processing time first)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]


def gather_states(parts, local_states, rank: int, world: int, group=None):
    """Rank 0 receives every rank's final (x, v) per cloth and returns them in batch order (a list of
    length sum(len(p) for p in parts)); the other ranks return None. `local_states` lists this rank's
    (x, v) in the order of parts[rank]. One gather of Python objects (torch.distributed)."""
    if len(local_states) != len(parts[rank]):
        raise ValueError("one (x, v) per cloth of this rank's part")
    if world == 1:
        return list(local_states)
    import torch.distributed as dist
    payload = [(np.asarray(x, np.float64), np.asarray(v, np.float64)) for x, v in local_states]
    got = [None] * world if rank == 0 else None
    dist.gather_object(payload, got, dst=0, group=group)
    if rank != 0:
        return None
    total = sum(len(p) for p in parts)
    out = [None] * total
    for r in range(world):
        if len(got[r]) != len(parts[r]):
            raise RuntimeError(f"rank {r} sent {len(got[r])} states for {len(parts[r])} cloths")
        for i, st in zip(parts[r], got[r]):
            out[i] = st
    return out

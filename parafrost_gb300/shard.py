"""Formula sharding over ranks (one process per GPU) for batched work.

Formulas are independent, so a batch splits across ranks with no exchange in the
data path: every rank runs one batched round over its share, and only the
per-formula results travel back to rank 0 (host side, after the rounds). Shares
are balanced by estimated device footprint with a greedy longest-first bin
packing, and every rank keeps its formulas in batch order.
"""
from __future__ import annotations

import heapq

from .serve import estimate_footprint


def shard_formulas(formulas: list, world: int) -> list:
    """Indices of the formulas each rank takes: a list of `world` ascending lists."""
    if world < 1:
        raise ValueError("world must be >= 1")
    cost = [estimate_footprint(nv, off.size - 1, lits.size) for nv, lits, off in formulas]
    order = sorted(range(len(formulas)), key=lambda i: (-cost[i], i))
    heap = [(0, r) for r in range(world)]
    heapq.heapify(heap)
    shares = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + cost[i], r))
    return [sorted(s) for s in shares]


def run_sharded(formulas: list, opts, rank: int, world: int, library: str | None = None, group=None) -> list | None:
    """Batched round over this rank's share; rank 0 returns every formula's
    (status, phases, Result) in batch order, other ranks return None. Needs an
    initialised torch.distributed process group when world > 1."""
    from .sigma import Simplifier

    mine = shard_formulas(formulas, world)[rank]
    out = []
    if mine:
        s = Simplifier(opts, library=library)
        s.awaken_batch([formulas[i] for i in mine])
        s.sigmify()
        out = list(zip(mine, s.batch_results()))
        s.close()
    if world == 1:
        return [r for _, r in sorted(out, key=lambda x: x[0])]
    import torch.distributed as dist
    parts = [None] * world if rank == 0 else None
    dist.gather_object(out, parts, dst=0, group=group)
    if rank != 0:
        return None
    merged = sorted((x for p in parts for x in p), key=lambda x: x[0])
    return [r for _, r in merged]

"""Column sharding across ranks, one GPU per rank.

Soil columns exchange nothing (no lateral flow: src/standalone/Soil/rre.jl:106,
src/standalone/Soil/energy_hydrology.jl:258), so a domain splits into
contiguous column ranges, one per rank, balanced by cell count (a step costs
in proportion to its layers). Each rank steps its range with its own handle;
the only collectives are reductions of per-column scalars (water and energy
totals, flagged columns, Newton iterations) and, on request, a gather of the
state. The rain-pulse forcing hashes global column indices
(clm_config.column_offset), so a sharded run reproduces the unsharded one
bit for bit.
"""
from __future__ import annotations

import numpy as np


def partition(nlayers, world: int) -> list[tuple[int, int]]:
    """Contiguous ranges [c0, c1) of columns, one per rank, with cell counts
    as equal as whole columns allow (no range is empty while there are at
    least `world` columns)."""
    nl = np.asarray(nlayers, dtype=np.int64)
    ncol = len(nl)
    if world < 1 or ncol < world:
        raise ValueError(f"{ncol} columns cannot be split over {world} ranks")
    cum = np.concatenate([[0], np.cumsum(nl)])
    bounds = [0]
    for r in range(1, world):
        c = int(np.searchsorted(cum, cum[-1] * r / world, side="left"))
        c = max(c, bounds[-1] + 1)          # at least one column per range
        c = min(c, ncol - (world - r))      # leave one for each later rank
        bounds.append(c)
    bounds.append(ncol)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def shard(w, rank: int, world: int):
    """This rank's part of workload `w` (a Workload over its column range)."""
    c0, c1 = partition(w.nlayers, world)[rank]
    return w.columns(c0, c1)


def _dist():
    import torch.distributed as dist
    return dist


def gather_state(w, state, rank: int, world: int, dst: int = 0):
    """Concatenate every rank's state (tuple of 5 arrays in the C ABI layout)
    on rank `dst`, in global column order; other ranks get None."""
    import torch
    dist = _dist()
    ranges = partition(w.nlayers, world)
    out = []
    for i, a in enumerate(state):
        if a is None:
            out.append(None)
            continue
        per_col = i >= 3  # intF_w, intF_e are per column; the rest per cell
        sizes = [(c1 - c0) if per_col else int(w.offsets[c1] - w.offsets[c0]) for c0, c1 in ranges]
        n = max(sizes)
        buf = torch.zeros(n, dtype=torch.float64)
        buf[: len(a)] = torch.from_numpy(np.ascontiguousarray(a))
        parts = [torch.zeros(n, dtype=torch.float64) for _ in range(world)] if rank == dst else None
        dist.gather(buf, parts, dst=dst)
        out.append(None if rank != dst else np.concatenate([p[:s].numpy() for p, s in zip(parts, sizes)]))
    return tuple(out) if rank == dst else None


def reduce_totals(values, op="sum"):
    """All-reduce a small vector of per-rank scalars (budget totals, counts)."""
    import torch
    dist = _dist()
    t = torch.tensor(np.asarray(values, dtype=np.float64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM if op == "sum" else dist.ReduceOp.MAX)
    return t.numpy()


class ShardedColumns:
    """One rank's handle over its column range of a workload (GPU), with the
    collectives of the sharded run."""

    def __init__(self, w, rank: int, world: int, **kw):
        from .device import SoilColumns
        self.w, self.rank, self.world = w, rank, world
        self.part = shard(w, rank, world)
        self.cols = SoilColumns(self.part, **kw)

    def step(self, t, dt, nsteps=1):
        self.cols.step(t, dt, nsteps)

    def totals(self):
        """Global water and energy totals and the number of flagged columns."""
        W, E = self.cols.budgets()
        flags, _ = self.cols.status()
        return reduce_totals([float(np.sum(W)), float(np.sum(E)), float(np.count_nonzero(flags))])

    def gather(self, dst=0):
        return gather_state(self.w, self.cols.get_state(), self.rank, self.world, dst)

    def close(self):
        self.cols.close()

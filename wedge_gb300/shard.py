"""Destination-range shards of one traversal, one shard per GPU.

The reference splits a graph across NUMA nodes by its destination-grouped
edge list (graphdata.c:1050-1065: the edge vectors divided as evenly as
possible; graphdata.c:656-689: each part's vertex range ends at its last
destination, rounded up to a 512-vertex boundary) and every node pulls its
part.  Here each shard holds the in-edges of one destination range on its own
GPU (wedge_cuda_load_shard), over every vertex as a source.  A traversal runs
the reference's driver loop (execution_bfs.c:139-353) on every shard in step:

    pull (every shard, its own destinations)
    exchange: properties by element-wise minimum, pulled frontier bitmaps by
              bitwise or (the shards' destinations are disjoint), changed mass
              by sum -- over the shards of this process and, through a
              torch.distributed process group, over the other processes
    import the combined state into every shard; the whole graph's decision
    Wedge build from the combined frontier (each shard's own CSRI), advance

BFS, CC and SSSP are supported: their properties only decrease, so the
element-wise minimum of the shards' arrays is every vertex's owner's value.
Results are read from any shard after the last exchange.

One difference from the reference, on purpose: a destination's in-edges all
go to one shard (the split falls between destinations), so no partial result
of a destination crosses shards.
"""
from __future__ import annotations

import numpy as np

from . import engine as W

ALIGN = 512  # vertex-range boundaries (graphdata.c:672)
U64_FLIP = np.uint64(1 << 63)


def partition(num_vertices: int, dst: np.ndarray, num_shards: int) -> list[tuple[int, int]]:
    """[(first, last)] destination ranges (inclusive, possibly empty: last < first) of
    num_shards shards of the edge list dst (ascending).  The edges are divided as evenly
    as possible; each range ends at the last destination of its share, rounded up to a
    multiple of 512 (graphdata.c:656-689), the last one at num_vertices - 1."""
    if num_shards < 1 or num_vertices < 1:
        raise ValueError("need at least one shard and one vertex")
    E = len(dst)
    per = E // num_shards
    out = []
    first = 0
    for i in range(num_shards):
        if i < num_shards - 1:
            last = int(dst[(i + 1) * per - 1]) if per else first - 1
            if last >= 0:
                last += ALIGN - 1 - (last & (ALIGN - 1))
            last = min(max(last, first - 1), num_vertices - 1)
        else:
            last = num_vertices - 1
        out.append((first, last))
        first = last + 1
    return out


def shard_edges(dst: np.ndarray, bounds: tuple[int, int]) -> slice:
    """the slice of the ascending edge list holding the in-edges of the range"""
    first, last = bounds
    lo = int(np.searchsorted(dst, first, side="left"))
    hi = int(np.searchsorted(dst, last, side="right")) if last >= first else lo
    return slice(lo, hi)


class Exchange:
    """Reduces the shards' state: over this process's shards, then over a
    torch.distributed process group (None: one process)."""

    def __init__(self, group=None):
        self.group = group

    def _allreduce(self, a: np.ndarray, op: str) -> np.ndarray:
        if self.group is None:
            return a
        import torch
        import torch.distributed as dist

        if a.dtype == np.uint64:  # order-preserving map into int64
            t = torch.from_numpy((a ^ U64_FLIP).view(np.int64).copy())
        else:
            t = torch.from_numpy(a.astype(np.int64))
        dist.all_reduce(t, op=dist.ReduceOp.MIN if op == "min" else dist.ReduceOp.SUM, group=self.group)
        r = t.numpy()
        if a.dtype == np.uint64:
            return r.view(np.uint64) ^ U64_FLIP
        return r.astype(a.dtype)

    def min(self, arrays: list[np.ndarray]) -> np.ndarray:
        return self._allreduce(np.minimum.reduce(arrays) if len(arrays) > 1 else arrays[0].copy(), "min")

    def bit_or(self, arrays: list[np.ndarray]) -> np.ndarray:
        # disjoint bits: the sum over processes is their or
        local = np.bitwise_or.reduce(arrays) if len(arrays) > 1 else arrays[0].copy()
        return self._allreduce(local, "sum")

    def sum(self, values: list[int]) -> int:
        return int(self._allreduce(np.array([sum(values)], np.uint64).astype(np.int64), "sum")[0])


def _prop_dtype(app: int):
    return np.uint64 if app == W.APP_SSSP else np.uint32


def run(shards, app: int, params: W.Params, exchange: Exchange, global_outdeg: np.ndarray,
        global_edges: int, max_iterations: int = 0) -> dict:
    """The reference's driver loop over this process's shards (Graph handles, or
    any object with their run_phase / shard_state / shard_decide methods).
    global_outdeg: the whole graph's out-degrees (the root's is the first mass).
    Returns {"iterations", "wedge_iterations"}; results are read from any shard."""
    if app not in (W.APP_BFS, W.APP_CC, W.APP_SSSP):
        raise ValueError("sharded traversals run BFS, CC and SSSP")
    V = len(global_outdeg)
    thr = global_edges * params.threshold_pct // 100  # execution_bfs.c:132
    root = params.root if params.root < V else 0  # main.c:81-85
    for g in shards:
        g.run_phase(app, W.PHASE_INIT, params)
    active = global_edges if app == W.APP_CC else int(global_outdeg[root])
    props = [np.empty(V, _prop_dtype(app)) for _ in shards]
    fronts = [np.empty((V + 31) // 32, np.uint32) for _ in shards]
    cap = max_iterations or V + 1
    it = wedge_its = 0
    while True:
        dense = (app == W.APP_CC and it == 0) or active > thr  # execution_bfs.c:141, execution_cc.c:103
        phase = W.PHASE_PULL_DENSE if dense else W.PHASE_PULL_WEDGE
        masses = [g.run_phase(app, phase, params) for g in shards]
        it += 1
        wedge_its += 0 if dense else 1
        for g, p, f in zip(shards, props, fronts):
            g.shard_state(W.SHARD_PROPS, p)
            g.shard_state(W.SHARD_FRONTIER, f)
        prop = exchange.min(props)
        front = exchange.bit_or(fronts)
        active = exchange.sum(masses)
        for g in shards:
            g.shard_state(W.SHARD_PROPS, prop, True)
            g.shard_state(W.SHARD_FRONTIER, front, True)
            g.shard_decide(active, params.threshold_pct)
        if active == 0 or it >= cap:
            break
        for g in shards:
            g.run_phase(app, W.PHASE_WEDGE_BUILD, params)  # no-op before a dense pull
        for g in shards:
            g.run_phase(app, W.PHASE_ADVANCE, params)
    return {"iterations": it, "wedge_iterations": wedge_its, "converged": active == 0}

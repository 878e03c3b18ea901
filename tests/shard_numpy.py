"""Test infrastructure: a numpy shard with the interface of a GPU shard handle
(run_phase / shard_state / shard_decide / read_results), pulling its own
destinations Jacobi-style (every pull reads the properties the last exchange
left).  It lets the sharded driver loop (wedge_gb300/shard.py) and its
exchange run as gloo ranks on hosts without a GPU.  Vertex numbering: the
caller's (the GPU shards use the engine's; both agree across shards)."""
from __future__ import annotations

import numpy as np

from wedge_gb300 import engine as W

NONE32 = np.uint32(0xFFFFFFFF)
NONE64 = np.uint64(0xFFFFFFFFFFFFFFFF)


class NumpyShard:
    def __init__(self, V, src, dst, global_outdeg, weights=None):
        self.V = V
        self.src = np.asarray(src, np.int64)
        self.dst = np.asarray(dst, np.int64)
        self.w = None if weights is None else np.asarray(weights, np.uint64)
        self.od = np.asarray(global_outdeg, np.uint64)
        self.app = None

    def run_phase(self, app, phase, params):
        V = self.V
        if phase == W.PHASE_INIT:
            self.app = app
            root = params.root if params.root < V else 0
            self.cur = np.zeros(V, bool)
            self.nxt = np.zeros(V, bool)
            if app == W.APP_BFS:
                self.prop = np.full(V, NONE32, np.uint32)
                self.visited = np.zeros(V, bool)
                self.visited[root] = True
                self.cur[root] = True
            elif app == W.APP_CC:
                self.prop = np.arange(V, dtype=np.uint32)
            else:
                self.prop = np.full(V, NONE64, np.uint64)
                self.prop[root] = 0
                self.cur[root] = True
            return 0
        if phase in (W.PHASE_PULL_DENSE, W.PHASE_PULL_WEDGE):
            return self._pull()
        if phase == W.PHASE_ADVANCE:
            self.nxt[:] = False
        return 0

    def _pull(self):
        s, d = self.src, self.dst
        old = self.prop.copy()
        if self.app == W.APP_BFS:
            m = self.cur[s] & ~self.visited[d]
            cand = np.full(self.V, np.iinfo(np.int64).max, np.int64)
            np.minimum.at(cand, d[m], s[m])
            hit = cand != np.iinfo(np.int64).max
            self.prop[hit] = cand[hit].astype(np.uint32)
            self.visited |= hit
            changed = hit
        elif self.app == W.APP_CC:
            new = old.copy()
            np.minimum.at(new, d, old[s])
            changed = new < old
            self.prop = new
        else:
            val = np.where(old[s] == NONE64, NONE64, old[s] + self.w)
            new = old.copy()
            np.minimum.at(new, d, val)
            changed = new < old
            self.prop = new
        self.nxt = changed
        return int(self.od[changed].sum())

    def shard_state(self, which, out, import_=False):
        if which == W.SHARD_PROPS:
            if import_:
                self.prop = out.astype(self.prop.dtype).copy()
            else:
                out[:] = self.prop
            return out
        if import_:
            self.cur = np.unpackbits(out.view(np.uint8), bitorder="little")[: self.V].astype(bool)
            self.nxt[:] = False
        else:
            words = np.packbits(self.nxt, bitorder="little")
            buf = np.zeros(len(out) * 4, np.uint8)
            buf[: len(words)] = words
            out[:] = buf.view(np.uint32)
        return out

    def shard_decide(self, global_mass, threshold_pct=20):
        pass

    def read_results(self):
        """graph_vertex_props in the reference's representation"""
        if self.app == W.APP_BFS:
            return np.where(self.prop == NONE32, NONE64, self.prop.astype(np.uint64))
        if self.app == W.APP_CC:
            return self.prop.astype(np.float64).view(np.uint64)
        return self.prop.copy()

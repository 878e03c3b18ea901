"""Shared checks for the parity tests (independent of both the oracle and the engine)."""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
UNREACHED = np.uint64(0xFFFFFFFFFFFFFFFF)


def golden():
    with open(os.path.join(HERE, "golden", "golden.json")) as f:
        meta = json.load(f)
    data = np.load(os.path.join(HERE, "golden", "golden.npz"))
    return meta, data


def out_csr(V, src, dst):
    """out-adjacency (CSR by source) of a dst-sorted edge list"""
    order = np.argsort(src, kind="stable")
    s = src[order].astype(np.int64)
    d = dst[order].astype(np.int64)
    off = np.zeros(V + 1, np.int64)
    np.add.at(off, s + 1, 1)
    return np.cumsum(off), d


def bfs_levels(V, src, dst, root):
    """textbook level-synchronous BFS along out-edges; -1 = unreached"""
    off, nbr = out_csr(V, src, dst)
    level = np.full(V, -1, np.int64)
    level[root] = 0
    frontier = np.array([root], np.int64)
    depth = 0
    while frontier.size:
        depth += 1
        starts = off[frontier]
        lens = off[frontier + 1] - starts
        total = int(lens.sum())
        if total == 0:
            break
        first = np.cumsum(lens) - lens
        idx = np.arange(total) + np.repeat(starts - first, lens)
        cand = np.unique(nbr[idx])
        cand = cand[level[cand] < 0]
        level[cand] = depth
        frontier = cand
    return level


def levels_from_parents(parents, root):
    """levels implied by a BFS parent array (reference representation); root is level 0"""
    V = len(parents)
    p = parents.astype(np.uint64)
    has = p != UNREACHED
    has[root] = False
    par = np.where(has, p, 0).astype(np.int64)
    level = np.full(V, -1, np.int64)
    level[root] = 0
    for _ in range(V + 1):
        upd = has & (level < 0) & (level[par] >= 0)
        if not upd.any():
            break
        level[upd] = level[par[upd]] + 1
    return level


def check_bfs(parents, V, src, dst, root, expect_levels=None):
    """BFS parents: every reached vertex other than the root has a parent that is an
    in-neighbour one level up; levels equal the textbook BFS.  Returns the levels."""
    expect = bfs_levels(V, src, dst, root) if expect_levels is None else expect_levels
    level = levels_from_parents(parents, root)
    reached = (parents != UNREACHED)
    reached[root] = True
    assert np.array_equal(reached, expect >= 0), "reached set differs from BFS"
    assert np.array_equal(level, expect), "BFS levels differ"
    v = np.nonzero((parents != UNREACHED) & (np.arange(V) != root))[0]
    p = parents[v].astype(np.int64)
    keys = np.sort(dst.astype(np.int64) << 32 | src.astype(np.int64))
    q = v.astype(np.int64) << 32 | p
    pos = np.searchsorted(keys, q)
    pos = np.minimum(pos, len(keys) - 1)
    assert np.all(keys[pos] == q), "a parent is not an in-neighbour"
    return level


def rel_l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def check_bfs_sorted(parents, V, src, dst, root, expect_levels):
    """check_bfs for large graphs whose edges are sorted by (dst, src): levels equal
    to expect_levels, every parent an in-neighbour, without sorting the edge list"""
    level = levels_from_parents(parents, root)
    assert np.array_equal(level, expect_levels), "BFS levels differ"
    v = np.nonzero((parents != UNREACHED) & (np.arange(V) != root))[0]
    q = (v.astype(np.uint64) << np.uint64(32)) | parents[v].astype(np.uint64)
    keys = (dst.astype(np.uint64) << np.uint64(32)) | src.astype(np.uint64)
    assert np.all(keys[1:] >= keys[:-1]), "edges are not sorted by (dst, src)"
    pos = np.minimum(np.searchsorted(keys, q), len(keys) - 1)
    assert np.all(keys[pos] == q), "a parent is not an in-neighbour"
    return level

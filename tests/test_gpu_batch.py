"""Batched queries in one persistent kernel (wedge_cuda_batch_*): every query's
result equals its own CPU run -- SSSP distances bit-exact, BFS levels exact
with every parent an in-neighbour one level up -- on a small mixed batch, on
the full 256 BFS + 256 SSSP over 64 graphs workload, with and without the
captured CUDA graph, under every tuning the autotuner may pick."""
import os

import numpy as np
import pytest

from helpers import check_bfs_sorted, levels_from_parents

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8


@pytest.fixture(scope="module")
def W(engine_lib):
    return engine_lib


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _expected(O, params, queries):
    """per query: ('sssp', distances) or ('bfs', levels), from the oracle run alone"""
    want = {}
    for gi, (scale, ef, seed, _h) in enumerate(params):
        mine = [(qi, app, root) for qi, (g, app, root) in enumerate(queries) if g == gi]
        if not mine:
            continue
        V, s, d = O.rmat(scale, ef, seed, threads=THREADS)
        s, d = O.sort_edges(V, s, d, threads=THREADS)
        w = O.weights(s, d)
        gb = O.Graph.from_edges(V, s, d, O.BFS, threads=THREADS)
        gs = O.Graph.from_edges(V, s, d, O.SSSP, w, threads=THREADS)
        for qi, app, root in mine:
            if app == 0:  # BFS
                p, _, _ = gb.run(root=root, threads=THREADS)
                want[qi] = ("bfs", levels_from_parents(p, root), V, s, d, root)
            else:
                want[qi] = ("sssp", gs.run(root=root, threads=THREADS)[0])
        gb.close()
        gs.close()
    return want


def _check(batch, want):
    for qi, exp in want.items():
        got = batch.read_result(qi)
        if exp[0] == "sssp":
            assert np.array_equal(got, exp[1]), f"query {qi}: SSSP distances differ"
        else:
            _, levels, V, s, d, root = exp
            check_bfs_sorted(got, V, s, d, root, levels)


def test_small_mixed_batch(W, O):
    from wedge_gb300 import batch as B

    params = B.graph_params(num_graphs=8, seed=9, scales=(8, 12), edge_factors=(4, 24))
    qs = B.queries(params, 3, 3)
    qs.append((0, W.APP_BFS, 10**9))  # out-of-range root selects vertex 0 (main.c:81-85)
    want = _expected(O, params, [(g, a, r if r < (1 << params[g][0]) else 0) for g, a, r in qs])
    graphs = B.load_graphs(params)
    with W.Batch(graphs, qs) as b:
        st = b.run()
        assert st["rounds"] >= 2 and st["chunks_pulled"] > 0 and st["captured"] == 0
        _check(b, want)
        it1 = b.iterations().copy()
        st2 = b.run(flags=W.FLAG_GRAPH)
        assert st2["captured"] == 1
        _check(b, want)
        b.run(flags=W.FLAG_GRAPH)  # replay of the captured graph
        _check(b, want)
        # BFS depth is a property of the graph; SSSP's iteration count depends on
        # the order of the asynchronous updates, its distances do not
        bfs = np.array([app == W.APP_BFS for _, app, _ in qs])
        assert np.array_equal(b.iterations()[bfs], it1[bfs])
    for g in graphs:
        g.close()


@pytest.mark.parametrize("tuning", [dict(), dict(threshold_pct=5, grab=1, blocks_per_sm=1, split=8),
                                    dict(threshold_pct=60, grab=32, blocks_per_sm=2, split=1024)])
def test_tunings_agree(W, O, tuning):
    from wedge_gb300 import batch as B

    params = B.graph_params(num_graphs=5, seed=11, scales=(9, 13), edge_factors=(8, 16))
    qs = B.queries(params, 2, 2)
    want = _expected(O, params, qs)
    graphs = B.load_graphs(params)
    with W.Batch(graphs, qs) as b:
        b.run(W.BatchTuning(**tuning) if tuning else None)
        _check(b, want)
    for g in graphs:
        g.close()


def test_full_workload_64_graphs(W, O):
    """256 BFS + 256 SSSP over 64 R-MAT graphs, scales 12-20, edge factors 8-32, seed 4"""
    from wedge_gb300 import autotune as A
    from wedge_gb300 import batch as B

    params = B.graph_params()
    qs = B.queries(params)
    assert len(params) == 64 and len(qs) == 512
    assert {p[0] for p in params} <= set(range(12, 21)) and {p[1] for p in params} <= set(range(8, 33))
    graphs = B.load_graphs(params)
    with W.Batch(graphs, qs) as b:
        st = b.run(A.load_tuning(), flags=W.FLAG_GRAPH)
        print("batch of 512 queries:", st)
        want = _expected(O, params, qs)
        _check(b, want)
    for g in graphs:
        g.close()

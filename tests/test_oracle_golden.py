"""The oracle (oracle/wedge_oracle.c) against the reference's own outputs.

tests/golden/golden.npz holds what the reference, compiled from its own sources,
produced on these graphs (tests/golden/make_golden.py).  Regenerating the
graph checks the generator; running the oracle on it checks the restatement:
CC labels and SSSP distances bit-exact, BFS reached set / levels exact and
parents valid, PageRank within 1e-12 relative L1 (the reference's AVX2 sum
order differs), with the same iteration counts where the algorithm is
deterministic.
"""
import numpy as np
import pytest

from helpers import UNREACHED, check_bfs, golden, levels_from_parents, rel_l1

META, DATA = golden()


def _graph(O, case):
    import hashlib

    p = case["params"]
    if case["kind"] == "rmat":
        V, s, d = O.rmat(p["scale"], p["edge_factor"], p["seed"])
    else:
        V, s, d = O.grid(p["side"], p["frac"], p["seed"])
    if case["variant"] == "symmetric":
        s, d = O.symmetrise(s, d)
    s, d = O.sort_edges(V, s, d)
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(s).tobytes())
    h.update(np.ascontiguousarray(d).tobytes())
    assert h.hexdigest()[:16] == case["edges_sha"], "generator output changed"
    return V, s, d


@pytest.mark.parametrize("case", META, ids=[c["key"] for c in META])
def test_oracle_matches_reference(oracle_lib, case):
    O = oracle_lib
    V, s, d = _graph(O, case)
    app = O.APP_NAMES[case["app"]]
    w = O.weights(s, d) if case["app"] == "sssp" else None
    ra = case["run"]
    g = O.Graph.from_edges(V, s, d, app, w)
    props, outdeg, st = g.run(root=ra.get("root", 0), threshold_pct=ra.get("threshold_pct", 20),
                              iterations=ra.get("iterations", 1), threads=1)
    ref = DATA[case["key"] + ".props"]
    if case["app"] in ("cc", "sssp"):
        assert np.array_equal(props, ref)
        assert st["iterations"] == case["stats"]["iterations"]
        assert st["wedge_iterations"] == case["stats"]["wedge_iterations"]
    elif case["app"] == "bfs":
        root = ra.get("root", 0)
        # single-threaded runs of the reference are deterministic: identical parents
        assert np.array_equal(props, ref)
        lv = check_bfs(props, V, s, d, root)
        ref_reached = ref != UNREACHED
        ref_reached[root] = True
        assert np.array_equal(lv >= 0, ref_reached)
        assert np.array_equal(levels_from_parents(ref, root), lv)
        assert st["iterations"] == case["stats"]["iterations"]
    else:
        assert rel_l1(props.view(np.float64), ref.view(np.float64)) < 1e-12
        assert np.array_equal(outdeg, DATA[case["key"] + ".outdeg"])


def test_pagerank_sum_is_one(oracle_lib):
    """the reference's built-in self-check (execution_pr.c:63-71)"""
    O = oracle_lib
    V, s, d = O.rmat(10, 16, 1)
    s, d = O.sort_edges(V, s, d)
    props, outdeg, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=16, threads=2)
    od = outdeg.view(np.float64)
    rank = props.view(np.float64) * np.where(od == 0, V, od)
    assert abs(rank.sum() - 1.0) < 1e-9


@pytest.mark.parametrize("app", ["cc", "sssp"])
def test_oracle_thread_count_invariance(oracle_lib, app):
    """CC labels and SSSP distances do not depend on the thread count"""
    O = oracle_lib
    V, s, d = O.rmat(12, 8, 2)
    if app == "cc":
        s, d = O.symmetrise(s, d)
    s, d = O.sort_edges(V, s, d)
    w = O.weights(s, d) if app == "sssp" else None
    g = O.Graph.from_edges(V, s, d, O.APP_NAMES[app], w)
    a, _, _ = g.run(threads=1)
    b, _, _ = g.run(threads=4)
    assert np.array_equal(a, b)

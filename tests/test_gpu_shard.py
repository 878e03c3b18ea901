"""Destination-range shards on the GPU (wedge_cuda_load_shard, _shard_state,
_shard_decide) driven by the sharded loop of wedge_gb300/shard.py.  This run
has one GPU, so the shards of a traversal are handles on that one GPU, stepped
by one process; their kernels never wait on each other (the exchange is on
the host between launches).  Results equal the oracle's whole-graph run: CC
labels and SSSP distances bit-exact, BFS levels exact with every parent an
in-neighbour one level up."""
import numpy as np
import pytest

from helpers import check_bfs, levels_from_parents

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nshards", [2, 3])
@pytest.mark.parametrize("app", ["bfs", "cc", "sssp"])
def test_gpu_shards_match_the_oracle(engine_lib, oracle_lib, app, nshards):
    W, O = engine_lib, oracle_lib
    from wedge_gb300 import shard as SH

    V, s, d = O.rmat(14, 16, 43)
    if app == "cc":
        s, d = O.symmetrise(s, d)
    s, d = O.sort_edges(V, s, d)
    w = O.weights(s, d) if app == "sssp" else None
    outdeg = np.bincount(s, minlength=V).astype(np.uint64)
    a = {"bfs": W.APP_BFS, "cc": W.APP_CC, "sssp": W.APP_SSSP}[app]
    shards = []
    for b in SH.partition(V, d, nshards):
        sl = SH.shard_edges(d, b)
        shards.append(W.Graph.shard(V, s[sl], d[sl], outdeg, len(s), None if w is None else w[sl]))
    if app == "sssp" and nshards == 3:
        for g in shards:  # the 512-edge pull (64-bit sums on shards) with its spanning-destination finish
            g.set_knob("sssp_tile", 512)
    try:
        info = SH.run(shards, a, W.Params(root=0), SH.Exchange(None), outdeg, len(s))
        assert info["converged"]
        got = shards[-1].read_results()
    finally:
        for g in shards:
            g.close()
    if app == "bfs":
        ref, _, _ = O.Graph.from_edges(V, s, d, O.BFS).run(root=0, threads=4)
        check_bfs(got, V, s, d, 0, levels_from_parents(ref, 0))
    elif app == "cc":
        ref, _, _ = O.Graph.from_edges(V, s, d, O.CC).run(threads=4)
        assert np.array_equal(got, ref)
    else:
        ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=0, threads=4)
        assert np.array_equal(got, ref)

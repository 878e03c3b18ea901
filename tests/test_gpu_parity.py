"""Parity of the CUDA engine (through the C ABI) with the oracle and the
reference's golden outputs.  Bars: CC labels and SSSP distances bit-exact;
BFS reached set and levels exact, every parent an in-neighbour one level up;
PageRank FP64 within 1e-12 relative L1; compensated FP32 PageRank within 1e-6
relative L1 of the FP64 oracle, and every vertex within 2e-5 relative of it."""
import os

import numpy as np
import pytest

from helpers import UNREACHED, bfs_levels, check_bfs, golden, rel_l1

pytestmark = pytest.mark.gpu

META, DATA = golden()
PR_TOL = 1e-12
PR32_TOL = 1e-6      # relative L1 of compensated FP32 against the FP64 oracle
PR32_MAXREL = 2e-5   # largest per-vertex relative difference


@pytest.fixture(scope="module")
def W(engine_lib):
    return engine_lib


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def graph_edges(O, kind, p, symmetric=False):
    if kind == "rmat":
        V, s, d = O.rmat(p["scale"], p["edge_factor"], p["seed"])
    else:
        V, s, d = O.grid(p["side"], p["frac"], p["seed"])
    if symmetric:
        s, d = O.symmetrise(s, d)
    s, d = O.sort_edges(V, s, d)
    return V, s, d


def run_engine(W, V, s, d, app, w=None, weight_kind=None, knobs=None, **params):
    wk = weight_kind if weight_kind is not None else W.WEIGHTS_U64
    with W.Graph.from_edges(V, s, d, w, wk if w is not None else W.WEIGHTS_NONE) as g:
        for k, v in (knobs or {}).items():
            g.set_knob(k, v)
        st = g.run(app, W.Params(**params))
        props = g.read_results()
        od = g.read_outdegrees()
    assert st["pull_launches"] > 0 or len(s) == 0
    return props, od, st


@pytest.mark.parametrize("case", META, ids=[c["key"] for c in META])
def test_engine_matches_reference_golden(W, O, case):
    V, s, d = graph_edges(O, case["kind"], case["params"], case["variant"] == "symmetric")
    app = {"bfs": W.APP_BFS, "cc": W.APP_CC, "pr": W.APP_PR, "sssp": W.APP_SSSP}[case["app"]]
    ra = case["run"]
    w = O.weights(s, d) if case["app"] == "sssp" else None
    props, od, st = run_engine(W, V, s, d, app, w, root=ra.get("root", 0), threshold_pct=ra.get("threshold_pct", 20),
                               num_iterations=ra.get("iterations", 1))
    ref = DATA[case["key"] + ".props"]
    if case["app"] in ("cc", "sssp"):
        assert np.array_equal(props, ref)
    elif case["app"] == "bfs":
        root = ra.get("root", 0)
        lv = check_bfs(props, V, s, d, root)
        reached = ref != UNREACHED
        reached[root] = True
        assert np.array_equal(lv >= 0, reached)
    else:
        assert rel_l1(props.view(np.float64), ref.view(np.float64)) < PR_TOL
        assert np.array_equal(od.astype(np.float64), DATA[case["key"] + ".outdeg"].view(np.float64))
        assert abs(st["pr_sum"] - 1.0) < 1e-9


SIZES = [(8, 4, 11), (11, 16, 12), (13, 8, 13), (14, 32, 14)]
SCHEDS = ["plain", "dense", "wedge"]


def sched_id(W, name):
    return {"plain": W.SCHED_PLAIN, "dense": W.SCHED_DENSE, "wedge": W.SCHED_WEDGE}[name]


@pytest.mark.parametrize("scale,ef,seed", SIZES)
@pytest.mark.parametrize("sched", SCHEDS)
def test_cc_bit_exact(W, O, scale, ef, seed, sched):
    for symmetric in (True, False):
        V, s, d = graph_edges(O, "rmat", dict(scale=scale, edge_factor=ef, seed=seed), symmetric)
        ref, _, _ = O.Graph.from_edges(V, s, d, O.CC).run(threads=4)
        got, _, st = run_engine(W, V, s, d, W.APP_CC, sched=sched_id(W, sched))
        assert np.array_equal(got, ref)
        if sched == "wedge":
            assert st["wedge_iterations"] >= 1 or st["iterations"] <= 2


@pytest.mark.parametrize("scale,ef,seed", SIZES)
@pytest.mark.parametrize("sched", SCHEDS)
@pytest.mark.parametrize("tile", [256, 512])
def test_sssp_bit_exact(W, O, scale, ef, seed, sched, tile):
    V, s, d = graph_edges(O, "rmat", dict(scale=scale, edge_factor=ef, seed=seed))
    w = O.weights(s, d)
    for root in (0, 3):
        ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=root, threads=4)
        got, _, _ = run_engine(W, V, s, d, W.APP_SSSP, w, knobs={"sssp_tile": tile}, root=root, sched=sched_id(W, sched))
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("scale,ef,seed", SIZES)
def test_sssp_fp64_weights_bit_exact(W, O, scale, ef, seed):
    V, s, d = graph_edges(O, "rmat", dict(scale=scale, edge_factor=ef, seed=seed))
    w = O.weights(s, d, O.WEIGHTS_F64)
    ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=0, threads=2, weight_kind=O.WEIGHTS_F64)
    got, _, _ = run_engine(W, V, s, d, W.APP_SSSP, w, weight_kind=W.WEIGHTS_F64, root=0)
    assert np.array_equal(got, ref)  # 0 ULP


def dijkstra_u64(V, s, d, w, root):
    """exact shortest distances (float64 holds these integer sums exactly) of the
    parallel-edge multigraph; UINT64_MAX where unreachable"""
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    order = np.lexsort((w, d, s))
    s, d, w = s[order], d[order], w[order]
    first = np.ones(len(s), bool)
    first[1:] = (s[1:] != s[:-1]) | (d[1:] != d[:-1])  # the least weight of each (s, d)
    m = sp.csr_matrix((w[first].astype(np.float64), (s[first], d[first])), shape=(V, V))
    dist = csgraph.dijkstra(m, directed=True, indices=root)
    out = np.full(V, np.iinfo(np.uint64).max, np.uint64)
    fin = np.isfinite(dist)
    out[fin] = dist[fin].astype(np.uint64)
    return out


@pytest.mark.parametrize("sched", SCHEDS)
@pytest.mark.parametrize("shift", [0, 25, 30])
def test_sssp_distances_beyond_32_bits(W, O, sched, shift):
    """the pulls gather a 32-bit copy of the distances while they fit: weights
    scaled by 2^shift push a fifth of the distances past 2^32 (shift 25) or
    nearly all (30), and the engine switches to the 64-bit distances; the results are
    exact shortest distances (the reference's 32-bit minimum, _mm_min_epu32,
    is not a 64-bit minimum there, so the check is Dijkstra's)"""
    V, s, d = graph_edges(O, "rmat", dict(scale=11, edge_factor=16, seed=12))
    w = O.weights(s, d).astype(np.uint64) << np.uint64(shift)
    for root in (0, 5):
        got, _, _ = run_engine(W, V, s, d, W.APP_SSSP, w, root=root, sched=sched_id(W, sched))
        ref = dijkstra_u64(V, s, d, w, root)
        assert np.array_equal(got, ref)
        if shift:
            assert got[got != np.iinfo(np.uint64).max].max() >= 2**32


def test_sssp_narrow_copy_off_matches(W, O, monkeypatch):
    """WEDGE_SSSP_NARROW=0 (64-bit gathers) gives the same distances"""
    V, s, d = graph_edges(O, "rmat", dict(scale=13, edge_factor=8, seed=13))
    w = O.weights(s, d)
    on, _, _ = run_engine(W, V, s, d, W.APP_SSSP, w, root=0)
    monkeypatch.setenv("WEDGE_SSSP_NARROW", "0")
    off, _, _ = run_engine(W, V, s, d, W.APP_SSSP, w, root=0)
    assert np.array_equal(on, off)


@pytest.mark.parametrize("scale,ef,seed", SIZES)
@pytest.mark.parametrize("sched", SCHEDS)
def test_bfs_levels_exact_parents_valid(W, O, scale, ef, seed, sched):
    V, s, d = graph_edges(O, "rmat", dict(scale=scale, edge_factor=ef, seed=seed))
    for root in (0, 1, V - 1):
        lv = bfs_levels(V, s, d, root)
        got, _, _ = run_engine(W, V, s, d, W.APP_BFS, root=root, sched=sched_id(W, sched))
        check_bfs(got, V, s, d, root, lv)
        ref, _, _ = O.Graph.from_edges(V, s, d, O.BFS).run(root=root, threads=4)
        check_bfs(ref, V, s, d, root, lv)


@pytest.mark.parametrize("scale,ef,seed", SIZES)
@pytest.mark.parametrize("damping", [0.875, 0.85])
def test_pagerank_fp64(W, O, scale, ef, seed, damping):
    V, s, d = graph_edges(O, "rmat", dict(scale=scale, edge_factor=ef, seed=seed))
    ref, _, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=16, damping=damping, threads=4)
    got, _, st = run_engine(W, V, s, d, W.APP_PR, num_iterations=16, damping=damping)
    assert rel_l1(got.view(np.float64), ref.view(np.float64)) < PR_TOL
    assert abs(st["pr_sum"] - 1.0) < 1e-9


def test_pagerank_graph_matches_stream(W, O):
    """the captured iteration loop gives the stream-launched ranks bit for bit, across
    iteration counts, damping factors and precisions (each change re-keys or rebuilds the capture)"""
    V, s, d = graph_edges(O, "rmat", dict(scale=12, edge_factor=16, seed=4))
    ref, _, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=7, damping=0.85, threads=4)
    with W.Graph.from_edges(V, s, d) as g:
        for iters, damping, prec in ((16, 0.875, W.PREC_FP64), (7, 0.85, W.PREC_FP64), (16, 0.875, W.PREC_FP64),
                                     (30, 0.875, W.PREC_FP32C), (1, 0.875, W.PREC_FP32C)):
            p = dict(num_iterations=iters, damping=damping, precision=prec)
            st0 = g.run(W.APP_PR, W.Params(**p))
            a = g.read_results()
            st1 = g.run(W.APP_PR, W.Params(flags=W.FLAG_GRAPH, **p))
            b = g.read_results()
            assert np.array_equal(a, b), (iters, damping, prec)
            assert st1["iterations"] == iters and st0["pr_sum"] == st1["pr_sum"]
            if (iters, damping) == (7, 0.85):
                assert rel_l1(b.view(np.float64), ref.view(np.float64)) < PR_TOL


def check_pr32(got, ref):
    """compensated FP32 against FP64: relative L1 and the largest per-vertex relative difference"""
    a, b = got.view(np.float64), ref.view(np.float64)
    err = rel_l1(a, b)
    maxrel = float(np.max(np.abs(a - b) / np.abs(b))) if len(b) else 0.0
    assert err < PR32_TOL and maxrel < PR32_MAXREL, (err, maxrel)
    return err, maxrel


@pytest.mark.parametrize("scale,ef,seed", SIZES)
def test_pagerank_fp32_compensated(W, O, scale, ef, seed):
    V, s, d = graph_edges(O, "rmat", dict(scale=scale, edge_factor=ef, seed=seed))
    ref, _, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=30, threads=4)
    got, _, st = run_engine(W, V, s, d, W.APP_PR, num_iterations=30, precision=W.PREC_FP32C)
    check_pr32(got, ref)
    assert abs(st["pr_sum"] - 1.0) < 1e-5


def test_pagerank_fp32_edge_structure(W, O):
    """hubs spanning many 512-edge tiles, destinations spanning one boundary,
    vertices with out-edges but no in-edges, vertices with no edges at all,
    dangling vertices and self-loops, under the compensated FP32 form"""
    rng = np.random.default_rng(5)
    V = 20000
    hub_src = rng.integers(0, V, 9000).astype(np.uint32)       # 9000 in-edges: 18 tiles
    small_d = rng.integers(10000, 12000, 30000).astype(np.uint32)
    small_s = rng.integers(0, 15000, 30000).astype(np.uint32)  # 15000..19999: no out-edges
    src = np.concatenate([hub_src, small_s, np.array([7, 7, 7], np.uint32)])
    dst = np.concatenate([np.full(9000, 3, np.uint32), small_d, np.array([7, 8, 9], np.uint32)])
    order = np.lexsort((src, dst))
    s, d = src[order], dst[order]
    for damping in (0.875, 0.85):
        ref, _, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=12, damping=damping, threads=2)
        got, _, st = run_engine(W, V, s, d, W.APP_PR, num_iterations=12, damping=damping, precision=W.PREC_FP32C)
        check_pr32(got, ref)
        assert abs(st["pr_sum"] - 1.0) < 1e-5
    # zero iterations leave the initial ranks 1/N / outdegree'
    with W.Graph.from_edges(V, s, d) as g:
        g.run(W.APP_PR, W.Params(num_iterations=0, precision=W.PREC_FP32C))
        got, od = g.read_results(), g.read_outdegrees()
    init = 1.0 / V / np.where(od == 0, V, od).astype(np.float64)
    assert np.allclose(got.view(np.float64), init, rtol=1e-6, atol=0)


def test_pagerank_fp32_phase_api(W, O):
    """init, pulls and the closing vertex phase through wedge_cuda_run_phase give run()'s ranks bit for bit"""
    V, s, d = graph_edges(O, "rmat", dict(scale=12, edge_factor=16, seed=9))
    p = W.Params(num_iterations=6, damping=0.85, precision=W.PREC_FP32C)
    with W.Graph.from_edges(V, s, d) as g:
        g.run(W.APP_PR, p)
        a = g.read_results()
        g.run_phase(W.APP_PR, W.PHASE_INIT, p)
        for _ in range(6):
            g.run_phase(W.APP_PR, W.PHASE_PULL_DENSE, p)
        g.run_phase(W.APP_PR, W.PHASE_VERTEX_PR, p)
        b = g.read_results()
    assert np.array_equal(a, b)


def test_async_runs_and_reads_match_sync(W, O):
    """wedge_cuda_run_async + wedge_cuda_read_results_async into page-locked memory
    give wedge_cuda_run's results; handles sharing a caller's stream run in
    order; a later run of a handle waits for its queued export"""
    torch = pytest.importorskip("torch")
    V, s, d = graph_edges(O, "rmat", dict(scale=13, edge_factor=16, seed=31))
    w = O.weights(s, d)
    p_pr = dict(num_iterations=5, damping=0.85, precision=W.PREC_FP32C)
    with W.Graph.from_edges(V, s, d, w, W.WEIGHTS_U64) as g1, W.Graph.from_edges(V, s, d) as g2:
        g1.run(W.APP_SSSP, W.Params(root=0))
        want0 = g1.read_results()
        g1.run(W.APP_SSSP, W.Params(root=3))
        want3 = g1.read_results()
        g2.run(W.APP_PR, W.Params(**p_pr))
        want_pr = g2.read_results()
        stream = torch.cuda.Stream()
        g1.set_stream(stream.cuda_stream)
        g2.set_stream(stream.cuda_stream)
        host = [torch.empty(V, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64) for _ in range(3)]
        g1.run_async(W.APP_SSSP, W.Params(root=0))
        g1.read_results_async(host[0])
        g2.run_async(W.APP_PR, W.Params(**p_pr))
        g2.read_results_async(host[1])
        g1.run_async(W.APP_SSSP, W.Params(root=3))  # overwrites the distances once host[0] is written
        g1.read_results_async(host[2])
        st1, st2 = g1.wait(), g2.wait()
        assert np.array_equal(host[0], want0)
        assert np.array_equal(host[1], want_pr)
        assert np.array_equal(host[2], want3)
        assert st1["iterations"] > 0 and st2["iterations"] == 5
        assert abs(st2["pr_sum"] - 1.0) < 1e-5
        # pipelined: each query's results are waited for after the next query is queued
        roots = [0, 3, 7, 0]
        wants = {0: want0, 3: want3}
        for i, r in enumerate(roots):
            if i:
                g1.wait_results()  # query i-1's results are in host[0]
                if roots[i - 1] in wants:
                    assert np.array_equal(host[0], wants[roots[i - 1]])
            g1.run_async(W.APP_SSSP, W.Params(root=r))
            g1.read_results_async(host[0])
        g1.wait()
        assert np.array_equal(host[0], want0)
        g1.wait_results()  # nothing pending: returns at once
        g1.set_stream(None)
        with pytest.raises(W.WedgeError):  # asynchronous reads need page-locked memory
            g1.read_results_async(np.empty(V, np.uint64))
        with pytest.raises(W.WedgeError):  # per-iteration timing needs the host between iterations
            g1.run_async(W.APP_SSSP, W.Params(root=0, flags=W.FLAG_TIMING))


def test_grid_sssp_and_bfs(W, O):
    V, s, d = graph_edges(O, "grid", dict(side=64, frac=0.01, seed=3))
    w = O.weights(s, d)
    ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=0, threads=4)
    got, _, st = run_engine(W, V, s, d, W.APP_SSSP, w, root=0)
    assert np.array_equal(got, ref)
    got, _, _ = run_engine(W, V, s, d, W.APP_BFS, root=17)
    check_bfs(got, V, s, d, 17)


# ---------------------------------------------------------------- edge cases
def test_hub_spanning_many_tiles(W, O):
    """one destination with 5000 in-edges (40 tiles), others tiny"""
    V = 6000
    src = np.concatenate([np.arange(5000, dtype=np.uint32), np.array([1, 2, 3], np.uint32)])
    dst = np.concatenate([np.full(5000, 5001, np.uint32), np.array([5002, 5002, 5003], np.uint32)])
    order = np.lexsort((src, dst))
    s, d = src[order], dst[order]
    ref, _, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=5, threads=2)
    got, _, _ = run_engine(W, V, s, d, W.APP_PR, num_iterations=5)
    assert rel_l1(got.view(np.float64), ref.view(np.float64)) < PR_TOL
    # CC: the hub takes the minimum source label
    got, _, _ = run_engine(W, V, s, d, W.APP_CC)
    assert got.view(np.float64)[5001] == 0.0
    got, _, _ = run_engine(W, V, s, d, W.APP_BFS, root=4999)
    assert got[5001] == 4999


def test_empty_and_tiny_graphs(W, O):
    s = np.zeros(0, np.uint32)
    d = np.zeros(0, np.uint32)
    got, _, _ = run_engine(W, 5, s, d, W.APP_BFS, root=2)
    assert np.all(got == UNREACHED)
    got, _, _ = run_engine(W, 5, s, d, W.APP_CC)
    assert got.view(np.float64).tolist() == [0.0, 1.0, 2.0, 3.0, 4.0]
    got, _, _ = run_engine(W, 1, np.array([0], np.uint32), np.array([0], np.uint32), W.APP_PR, num_iterations=3)
    assert abs(got.view(np.float64)[0] - 1.0) < 1e-15


@pytest.mark.parametrize("name", ["path", "star", "fanin"])
def test_known_answers(W, O, name):
    from test_oracle import KATS, _kat

    V, edges, levels = KATS[name]
    s, d = _kat(O, V, edges)
    got, _, _ = run_engine(W, V, s, d, W.APP_BFS, root=0)
    assert check_bfs(got, V, s, d, 0).tolist() == levels
    dist, _, _ = run_engine(W, V, s, d, W.APP_SSSP, np.ones(len(s), np.uint64), root=0)
    assert [(-1 if x == UNREACHED else int(x)) for x in dist] == levels


def test_root_out_of_range_uses_vertex_zero(W, O):
    V, s, d = graph_edges(O, "rmat", dict(scale=9, edge_factor=8, seed=1))
    a, _, _ = run_engine(W, V, s, d, W.APP_BFS, root=10**9)
    b, _, _ = run_engine(W, V, s, d, W.APP_BFS, root=0)
    check_bfs(a, V, s, d, 0)
    assert np.array_equal(a != UNREACHED, b != UNREACHED)


# ---------------------------------------------------------------- load paths
def test_load_paths_agree(W, O, tmp_path):
    V, s, d = graph_edges(O, "rmat", dict(scale=12, edge_factor=8, seed=21))
    w = O.weights(s, d)
    p2 = str(tmp_path / "g2.bin")
    p3 = str(tmp_path / "g3.bin")
    O.write_file(p2, V, s, d)
    O.write_file(p3, V, s, d, w)
    ref_pr, _, _ = run_engine(W, V, s, d, W.APP_PR, num_iterations=4)
    with W.Graph.load(p2, W.APP_PR) as g:
        g.run(W.APP_PR, W.Params(num_iterations=4))
        assert np.array_equal(g.read_results(), ref_pr)  # same CSC -> same summation order
    with W.Graph.load_image(open(p2, "rb").read(), W.APP_PR) as g:
        g.run(W.APP_PR, W.Params(num_iterations=4))
        assert np.array_equal(g.read_results(), ref_pr)
    vec = O.Graph.from_edges(V, s, d, O.PR).edge_vectors()
    with W.Graph.from_edge_vectors(V, vec, weighted=False) as g:
        g.run(W.APP_PR, W.Params(num_iterations=4))
        assert np.array_equal(g.read_results(), ref_pr)
    ref_ss, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=0, threads=2)
    with W.Graph.load(p3, W.APP_SSSP) as g:
        g.run(W.APP_SSSP, W.Params(root=0))
        assert np.array_equal(g.read_results(), ref_ss)
    vecw = O.Graph.from_edges(V, s, d, O.SSSP, w).edge_vectors()
    with W.Graph.from_edge_vectors(V, vecw, weighted=True) as g:
        g.run(W.APP_SSSP, W.Params(root=0))
        assert np.array_equal(g.read_results(), ref_ss)


@pytest.mark.parametrize("symmetrise", [False, True])
def test_device_generator_matches_cpu_generator(W, O, symmetrise):
    V, s, d = graph_edges(O, "rmat", dict(scale=13, edge_factor=8, seed=4), symmetrise)
    a, od_a, _ = run_engine(W, V, s, d, W.APP_PR, num_iterations=3)
    with W.Graph.rmat(13, 8, 4, symmetrise=symmetrise) as g:
        assert g.V == V and g.E == len(s)
        g.run(W.APP_PR, W.Params(num_iterations=3))
        assert np.array_equal(g.read_results(), a)
        assert np.array_equal(g.read_outdegrees(), od_a)


def test_device_grid_generator_matches_cpu(W, O):
    V, s, d = graph_edges(O, "grid", dict(side=48, frac=0.01, seed=3))
    w = O.weights(s, d)
    ref, _, _ = run_engine(W, V, s, d, W.APP_SSSP, w, root=5)
    with W.Graph.grid(48, 0.01, 3, W.WEIGHTS_U64) as g:
        assert g.V == V and g.E == len(s)
        g.run(W.APP_SSSP, W.Params(root=5))
        assert np.array_equal(g.read_results(), ref)


def test_bad_inputs(W, O, tmp_path):
    V, s, d = graph_edges(O, "rmat", dict(scale=8, edge_factor=4, seed=1))
    p = str(tmp_path / "g.bin")
    O.write_file(p, V, s, d)
    with pytest.raises(W.WedgeError) as e:
        W.Graph.load(p, W.APP_SSSP)  # 2-tuples where SSSP expects 3-tuples
    assert e.value.status == -2
    raw = open(p, "rb").read()
    with pytest.raises(W.WedgeError) as e:
        W.Graph.load_image(raw[:-8], W.APP_BFS)
    assert e.value.status == -2
    with pytest.raises(W.WedgeError) as e:
        W.Graph.from_edges(V, d[::-1].copy(), d[::-1].copy())  # descending destinations
    assert e.value.status == -2
    with pytest.raises(W.WedgeError) as e:
        W.Graph.from_edges(4, np.array([9], np.uint32), np.array([0], np.uint32))  # id out of range
    assert e.value.status == -2
    with W.Graph.from_edges(V, s, d) as g:
        with pytest.raises(W.WedgeError) as e:
            g.run(W.APP_SSSP)  # no weights loaded
        assert e.value.status == -6
        with pytest.raises(W.WedgeError) as e:
            g.run(W.APP_BFS, W.Params(threshold_pct=101))
        assert e.value.status == -6


# ---------------------------------------------------------------- execution modes
@pytest.mark.parametrize("app", ["bfs", "cc", "sssp"])
def test_cuda_graph_loop_matches_host_loop(W, O, app):
    V, s, d = graph_edges(O, "rmat", dict(scale=13, edge_factor=16, seed=5), app == "cc")
    w = O.weights(s, d) if app == "sssp" else None
    a = {"bfs": W.APP_BFS, "cc": W.APP_CC, "sssp": W.APP_SSSP}[app]
    host, _, st1 = run_engine(W, V, s, d, a, w, root=0)
    graph, _, st2 = run_engine(W, V, s, d, a, w, root=0, flags=W.FLAG_GRAPH)
    timed, _, st3 = run_engine(W, V, s, d, a, w, root=0, flags=W.FLAG_TIMING)
    if app == "bfs":
        check_bfs(graph, V, s, d, 0)
        check_bfs(timed, V, s, d, 0)
    else:
        assert np.array_equal(host, graph) and np.array_equal(host, timed)
    assert st3["pull_ms_dense"] + st3["pull_ms_wedge"] > 0


def test_phase_api_drives_the_reference_loop(W, O):
    """execution_impl_bfs's own loop (execution_bfs.c:139-353) over wedge_cuda_run_phase"""
    V, s, d = graph_edges(O, "rmat", dict(scale=12, edge_factor=16, seed=6))
    E = len(s)
    p = W.Params(root=0)
    with W.Graph.from_edges(V, s, d) as g:
        g.run_phase(W.APP_BFS, 0, p)
        od = g.read_outdegrees()
        active = int(od[0])
        threshold = E * 20 // 100
        iters = 0
        while True:
            iters += 1
            phase = 1 if active > threshold else 2
            active = g.run_phase(W.APP_BFS, phase, p)
            if active == 0:
                break
            g.run_phase(W.APP_BFS, 4, p)  # wedge build (no-op when the next pull is dense)
            g.run_phase(W.APP_BFS, 5, p)  # advance
            assert iters < 100
        check_bfs(g.read_results(), V, s, d, 0)


@pytest.mark.parametrize("tile", [256, 512])
def test_phase_api_drives_the_reference_sssp_loop(W, O, tile):
    """execution_impl_sssp's loop over wedge_cuda_run_phase, with either dense-pull
    tile (512: the 32-bit pull, its 64-bit twin and the spanning destinations'
    finish run inside each pull phase); distances bit-exact"""
    V, s, d = graph_edges(O, "rmat", dict(scale=12, edge_factor=16, seed=6))
    w = O.weights(s, d)
    E = len(s)
    p = W.Params(root=0)
    ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=0, threads=4)
    with W.Graph.from_edges(V, s, d, w, W.WEIGHTS_U64) as g:
        g.set_knob("sssp_tile", tile)
        g.run_phase(W.APP_SSSP, W.PHASE_INIT, p)
        active = int(g.read_outdegrees()[0])
        iters = 0
        while True:
            iters += 1
            phase = W.PHASE_PULL_DENSE if active > E * 20 // 100 else W.PHASE_PULL_WEDGE
            active = g.run_phase(W.APP_SSSP, phase, p)
            if active == 0:
                break
            g.run_phase(W.APP_SSSP, W.PHASE_WEDGE_BUILD, p)
            g.run_phase(W.APP_SSSP, W.PHASE_ADVANCE, p)
            assert iters < 100
        assert np.array_equal(g.read_results(), ref)


def test_phase_api_cc_symmetric_reads_mid_traversal(W, O):
    """CC over wedge_cuda_run_phase on a symmetric graph (engine-id labels): results read
    between pulls are caller ids no lower than the final labels, and reading them does not
    disturb the traversal, which ends on the reference's labels"""
    V, s, d = graph_edges(O, "rmat", dict(scale=12, edge_factor=8, seed=7), True)
    ref, _, _ = O.Graph.from_edges(V, s, d, O.CC).run(threads=4)
    final = ref.view(np.float64)
    p = W.Params()
    with W.Graph.from_edges(V, s, d) as g:
        g.run_phase(W.APP_CC, 0, p)
        iters = 0
        while True:
            iters += 1
            active = g.run_phase(W.APP_CC, 1, p)  # dense pull
            mid = g.read_results().view(np.float64)
            assert np.all(mid >= final) and np.all(mid < V) and np.all(mid == np.floor(mid))
            if active == 0:
                break
            g.run_phase(W.APP_CC, 4, p)
            g.run_phase(W.APP_CC, 5, p)
            assert iters < 100
        assert np.array_equal(g.read_results(), ref)


def test_cc_label_space_symmetry_check(W, O):
    """a symmetric graph propagates engine ids and converts them; one edge without its
    reverse keeps the caller's ids; isolated vertices (V > E) change nothing: all exact"""
    V, s, d = graph_edges(O, "rmat", dict(scale=11, edge_factor=8, seed=8), True)
    i = int(np.flatnonzero(s != d)[len(s) // 2])
    keep = ~((s == s[i]) & (d == d[i]))  # every copy of one edge, its reverse stays
    for VV, ss, dd in ((V, s[keep], d[keep]), (V * 40, s, d)):
        ref, _, _ = O.Graph.from_edges(VV, ss, dd, O.CC).run(threads=4)
        for flags in (0, W.FLAG_GRAPH):
            got, _, _ = run_engine(W, VV, ss, dd, W.APP_CC, flags=flags)
            assert np.array_equal(got, ref)


def test_read_results_into_page_locked_memory(W, O):
    """page-locked caller buffers receive the export directly from the device:
    the same words as a pageable buffer, for every application and for CC
    labels read between phase-driven pulls (converted at read time)"""
    torch = pytest.importorskip("torch")
    V, s, d = graph_edges(O, "rmat", dict(scale=12, edge_factor=8, seed=9), True)
    w = O.weights(s, d)
    pinned = torch.empty(V, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    with W.Graph.from_edges(V, s, d, w, W.WEIGHTS_U64) as g:
        for app in (W.APP_BFS, W.APP_CC, W.APP_SSSP, W.APP_PR):
            g.run(app, W.Params(root=3, num_iterations=5))
            a = g.read_results()
            pinned[:] = 0
            g.read_results(pinned)
            assert np.array_equal(a, pinned), app
        g.run_phase(W.APP_CC, 0, W.Params())
        g.run_phase(W.APP_CC, 1, W.Params())
        a = g.read_results()
        pinned[:] = 0
        g.read_results(pinned)
        assert np.array_equal(a, pinned)


def test_wedge_pulls_over_chunk_ids(W, O, monkeypatch):
    """the chunk form of the Wedge frontier (CSRI chunk ids, the encoding of graphs
    beyond 2^32 padded in-edges, selected here by WEDGE_CSRI_CHUNKS) gives the
    same results as the candidate form"""
    monkeypatch.setenv("WEDGE_CSRI_CHUNKS", "1")
    V, s, d = graph_edges(O, "rmat", dict(scale=13, edge_factor=16, seed=11))
    Vs, ss, ds = graph_edges(O, "rmat", dict(scale=13, edge_factor=16, seed=11), True)
    lv = bfs_levels(V, s, d, 0)
    cc_ref, _, _ = O.Graph.from_edges(Vs, ss, ds, O.CC).run(threads=4)
    for sched in (W.SCHED_PLAIN, W.SCHED_WEDGE):
        got, _, st = run_engine(W, V, s, d, W.APP_BFS, root=0, sched=sched)
        check_bfs(got, V, s, d, 0, lv)
        assert st["wedge_iterations"] >= 1
        got, _, _ = run_engine(W, Vs, ss, ds, W.APP_CC, sched=sched)
        assert np.array_equal(got, cc_ref)


# sssp_narrow above 1: a limit of the 32-bit distance copy low enough that the
# traversals cross it, switching to 64-bit distances mid-way (the 512-edge pull
# drops its 32-bit sums at the limit and redoes the pull in 64 bits)
KNOB_SETTINGS = [{"hub_bytes": 0}, {"hub_bytes": 98304}, {"probe_edges": 1}, {"probe_edges": 4096},
                 {"sssp_tile": 512}, {"sssp_narrow": 0}, {"sssp_tile": 256, "sssp_narrow": 0},
                 {"sssp_tile": 512, "sssp_narrow": 0, "hub_bytes": 16},
                 {"sssp_tile": 256, "sssp_narrow": 40}, {"sssp_tile": 512, "sssp_narrow": 40},
                 {"sssp_tile": 512, "sssp_narrow": 150}]


@pytest.mark.parametrize("knobs", KNOB_SETTINGS, ids=[",".join(f"{k}={v}" for k, v in x.items()) for x in KNOB_SETTINGS])
def test_knobs_keep_results(W, O, knobs):
    """every launch knob the autotuner may set gives the same results"""
    V, s, d = graph_edges(O, "rmat", dict(scale=12, edge_factor=16, seed=12))
    Vs, ss, ds = graph_edges(O, "rmat", dict(scale=12, edge_factor=16, seed=12), True)
    w = O.weights(s, d)
    sssp_ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=0, threads=4)
    cc_ref, _, _ = O.Graph.from_edges(Vs, ss, ds, O.CC).run(threads=4)
    pr_ref, _, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=8, damping=0.85, threads=4)
    lv = bfs_levels(V, s, d, 0)
    with W.Graph.from_edges(V, s, d, w, W.WEIGHTS_U64) as g, W.Graph.from_edges(Vs, ss, ds) as gs:
        for k, v in knobs.items():
            g.set_knob(k, v)
            gs.set_knob(k, v)
            assert g.knob(k) == v
        for sched in (W.SCHED_PLAIN, W.SCHED_DENSE, W.SCHED_WEDGE):
            g.run(W.APP_SSSP, W.Params(root=0, sched=sched))
            assert np.array_equal(g.read_results(), sssp_ref)
            g.run(W.APP_BFS, W.Params(root=0, sched=sched))
            check_bfs(g.read_results(), V, s, d, 0, lv)
            gs.run(W.APP_CC, W.Params(sched=sched))
            assert np.array_equal(gs.read_results(), cc_ref)
        g.run(W.APP_PR, W.Params(num_iterations=8, damping=0.85, precision=W.PREC_FP32C))
        check_pr32(g.read_results(), pr_ref)


def test_knob_values_are_checked(W, O):
    V, s, d = graph_edges(O, "rmat", dict(scale=8, edge_factor=4, seed=11))
    with W.Graph.from_edges(V, s, d) as g:
        for k, v in (("hub_bytes", 17), ("hub_bytes", 1 << 20), ("probe_edges", 0), ("probe_edges", 4097),
                     ("sssp_tile", 128), ("sssp_narrow", 2**32 - 1)):
            with pytest.raises(W.WedgeError) as e:
                g.set_knob(k, v)
            assert e.value.status == -6  # WEDGE_ERR_ARG
        assert g.knob("hub_bytes") == 65536 or os.environ.get("WEDGE_HUB_BYTES")
        g.set_knob("probe_edges", 8)
        assert g.knob("probe_edges") == 8
        g.set_knob("probe_edges", None)
        assert g.knob("probe_edges") == int(os.environ.get("WEDGE_PROBE_EDGES", "16"))


def test_iteration_cap_reports_not_converged(W, O):
    V, s, d = graph_edges(O, "grid", dict(side=32, frac=0.0, seed=3))
    with W.Graph.from_edges(V, s, d) as g:
        with pytest.raises(W.WedgeError) as e:
            g.run(W.APP_BFS, W.Params(root=0, max_iterations=3))
        assert e.value.status == -5
        st = g.run(W.APP_BFS, W.Params(root=0, max_iterations=3), allow_not_converged=True)
        assert st["iterations"] == 3

"""Parity at the sizes of the workload configurations (GPU through the C ABI
against the oracle on the same seeded inputs):

- PageRank, R-MAT scale 16 (65,536 vertices, 1,048,576 edges, seed 1),
  16 iterations, damping 0.85: FP64 within 1e-12 relative L1 of the oracle;
  compensated FP32 within 1e-6 relative L1 of the FP64 oracle.
- BFS from vertex 0 and CC, R-MAT scale 24 (16,777,216 vertices, 268,435,456
  edges, seed 2; CC symmetrised): CC labels bit-exact, BFS levels exact and
  every parent an in-neighbour one level up.
- SSSP from vertex 0 on the 4096 x 4096 grid with 1% long-range edges (seed
  3): uint64 weights bit-exact, FP64 weights 0 ULP.
- R-MAT scale 26 (67,108,864 vertices, 1,073,741,824 edges, seed 5): BFS,
  CC, SSSP bit-exact under the plain and the learned schedule, 30-iteration
  compensated FP32 PageRank (damping 0.85) within 1e-6 relative L1 of the
  FP64 oracle, every vertex within 2e-5 relative of it.

The GPU side generates each graph on the device; the device generators are
bit-identical to the oracle's (test_gpu_parity.py checks them edge for edge).
"""
import os

import numpy as np
import pytest

from helpers import check_bfs_sorted, levels_from_parents, rel_l1

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8
PR_TOL = 1e-12
PR32_TOL = 1e-6      # relative L1 of compensated FP32 against the FP64 oracle
PR32_MAXREL = 2e-5   # largest per-vertex relative difference


@pytest.fixture(scope="module")
def W(engine_lib):
    return engine_lib


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _rmat_cpu(O, scale, ef, seed, symmetric=False):
    V, s, d = O.rmat(scale, ef, seed, threads=THREADS)
    if symmetric:
        s, d = O.symmetrise(s, d)
    s, d = O.sort_edges(V, s, d, threads=THREADS)
    return V, s, d


def test_pagerank_rmat16(W, O):
    V, s, d = _rmat_cpu(O, 16, 16, 1)
    assert (V, len(s)) == (65536, 1048576)
    ref, _, _ = O.Graph.from_edges(V, s, d, O.PR, threads=THREADS).run(iterations=16, damping=0.85, threads=THREADS)
    with W.Graph.rmat(16, 16, 1) as g:
        st = g.run(W.APP_PR, W.Params(num_iterations=16, damping=0.85))
        got = g.read_results().view(np.float64)
        g.run(W.APP_PR, W.Params(num_iterations=16, damping=0.85, precision=W.PREC_FP32C))
        got32 = g.read_results().view(np.float64)
    assert rel_l1(got, ref.view(np.float64)) < PR_TOL
    assert abs(st["pr_sum"] - 1.0) < 1e-9
    _pr32_close(got32, ref.view(np.float64))


def _pr32_close(got32, ref64):
    err = rel_l1(got32, ref64)
    maxrel = float(np.max(np.abs(got32 - ref64) / np.abs(ref64)))
    assert err < PR32_TOL and maxrel < PR32_MAXREL, (err, maxrel)


def test_bfs_cc_rmat24(W, O):
    V, s, d = _rmat_cpu(O, 24, 16, 2)
    assert (V, len(s)) == (16777216, 268435456)
    bfs_ref, _, _ = O.Graph.from_edges(V, s, d, O.BFS, threads=THREADS).run(root=0, threads=THREADS)
    with W.Graph.rmat(24, 16, 2) as g:
        g.run(W.APP_BFS, W.Params(root=0, flags=W.FLAG_GRAPH))
        parents = g.read_results()
    check_bfs_sorted(parents, V, s, d, 0, levels_from_parents(bfs_ref, 0))
    del s, d
    Vs, ss, ds = _rmat_cpu(O, 24, 16, 2, symmetric=True)
    assert len(ss) == 536870912
    ref, _, _ = O.Graph.from_edges(Vs, ss, ds, O.CC, threads=THREADS).run(threads=THREADS)
    del ss, ds
    with W.Graph.rmat(24, 16, 2, symmetrise=True) as g:
        g.run(W.APP_CC, W.Params(flags=W.FLAG_GRAPH))
        assert np.array_equal(g.read_results(), ref)


@pytest.mark.parametrize("kind", ["u64", "f64"])
def test_sssp_grid4096(W, O, kind):
    V, s, d = O.grid(4096, 0.01, 3)
    s, d = O.sort_edges(V, s, d, threads=THREADS)
    assert V == 16777216 and len(s) == 67092480 + 670924
    wk_o = O.WEIGHTS_U64 if kind == "u64" else O.WEIGHTS_F64
    wk_g = W.WEIGHTS_U64 if kind == "u64" else W.WEIGHTS_F64
    w = O.weights(s, d, wk_o)
    ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w, threads=THREADS).run(root=0, threads=THREADS, weight_kind=wk_o)
    del s, d, w
    with W.Graph.grid(4096, 0.01, 3, wk_g) as g:
        g.run(W.APP_SSSP, W.Params(root=0, flags=W.FLAG_GRAPH))
        assert np.array_equal(g.read_results(), ref)  # 0 ULP for FP64 weights


def test_rmat26_all_apps(W, O):
    from wedge_gb300 import autotune as A
    from wedge_gb300 import scheduler as S

    blob = S.load()
    V, s, d = _rmat_cpu(O, 26, 16, 5)
    assert (V, len(s)) == (67108864, 1073741824)
    w = O.weights(s, d)
    sssp_ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w, threads=THREADS).run(root=0, threads=THREADS)
    del w
    bfs_ref, _, _ = O.Graph.from_edges(V, s, d, O.BFS, threads=THREADS).run(root=0, threads=THREADS)
    levels = levels_from_parents(bfs_ref, 0)
    with W.Graph.rmat(26, 16, 5, weight_kind=W.WEIGHTS_U64) as g:
        g.set_scheduler(blob)
        for sched in (W.SCHED_PLAIN, W.SCHED_LEARNED):
            g.run(W.APP_SSSP, W.Params(root=0, sched=sched, flags=W.FLAG_GRAPH))
            assert np.array_equal(g.read_results(), sssp_ref)
            g.run(W.APP_BFS, W.Params(root=0, sched=sched, flags=W.FLAG_GRAPH))
            check_bfs_sorted(g.read_results(), V, s, d, 0, levels)
        # the launch knobs the benchmark runs with (the engine autotuner's table)
        assert A.apply_engine_tuning(g, "sssp", 26, 16)
        g.run(W.APP_SSSP, W.Params(root=0, flags=W.FLAG_GRAPH))
        assert np.array_equal(g.read_results(), sssp_ref)
        A.apply_engine_tuning(g, "bfs", 26, 16)
        g.run(W.APP_BFS, W.Params(root=0, flags=W.FLAG_GRAPH))
        check_bfs_sorted(g.read_results(), V, s, d, 0, levels)
        A.apply_engine_tuning(g, "pr", 26, 16)
        g.run(W.APP_PR, W.Params(num_iterations=30, damping=0.85, precision=W.PREC_FP32C, flags=W.FLAG_GRAPH))
        pr32 = g.read_results().view(np.float64).copy()
    del sssp_ref
    pr_ref, _, _ = O.Graph.from_edges(V, s, d, O.PR, threads=THREADS).run(iterations=30, damping=0.85, threads=THREADS)
    _pr32_close(pr32, pr_ref.view(np.float64))
    del s, d, pr_ref
    Vs, ss, ds = _rmat_cpu(O, 26, 16, 5, symmetric=True)
    cc_ref, _, _ = O.Graph.from_edges(Vs, ss, ds, O.CC, threads=THREADS).run(threads=THREADS)
    del ss, ds
    with W.Graph.rmat(26, 16, 5, symmetrise=True) as g:
        g.set_scheduler(blob)
        for sched in (W.SCHED_PLAIN, W.SCHED_LEARNED):
            g.run(W.APP_CC, W.Params(sched=sched, flags=W.FLAG_GRAPH))
            assert np.array_equal(g.read_results(), cc_ref)
        A.apply_engine_tuning(g, "cc", 26, 16)
        g.run(W.APP_CC, W.Params(flags=W.FLAG_GRAPH))
        assert np.array_equal(g.read_results(), cc_ref)

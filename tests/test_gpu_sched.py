"""The scheduler network and the strategies it picks from, on the GPU.

- The engine's CUDA forward / loss / gradient kernels against the CPU
  restatement (oracle/mlp_oracle.py): FP32 against FP64, relative tolerances
  stated in each test.
- Training on the GPU lowers the loss.
- Every strategy and every schedule leaves the results bit-exact: the
  source-filtered sweep, forced strategies (WEDGE_SCHED_PROBE) and network-chosen
  ones (WEDGE_SCHED_LEARNED).
- The trained network (wedge_gb300/data/sched_net.f32) against the fixed rule
  on held-out graphs: measured per-iteration costs of every strategy, and the
  choices each schedule makes on them.
"""
import math
import os

import numpy as np
import pytest

from helpers import check_bfs

pytestmark = pytest.mark.gpu
FWD_RTOL = 1e-5
GRAD_RTOL = 2e-4


@pytest.fixture(scope="module")
def W(engine_lib):
    return engine_lib


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _blob(rng, M):
    b = rng.normal(0, 0.3, M.BLOB)
    b[0:16] = rng.normal(0, 1, 16)
    b[16:32] = rng.uniform(0.5, 2.0, 16)
    b[32:48] = -10.0
    b[48:64] = 10.0
    b[-1] = 0.1
    return b.astype(np.float32)


def test_forward_matches_oracle(W):
    from oracle import mlp_oracle as M

    rng = np.random.default_rng(11)
    blob = _blob(rng, M)
    X = rng.normal(0, 1, (333, 16)).astype(np.float32)
    got = W.mlp_forward(blob, X)
    want, _ = M.forward(blob, X)
    assert np.abs(got - want).max() <= FWD_RTOL * max(1.0, np.abs(want).max())


def test_loss_and_gradient_match_oracle(W):
    from oracle import mlp_oracle as M

    rng = np.random.default_rng(12)
    blob = _blob(rng, M)
    n = 257
    X = rng.normal(0, 1, (n, 16)).astype(np.float32)
    Y = rng.normal(0, 1, (n, 3)).astype(np.float32)
    Mk = (rng.uniform(size=(n, 3)) < 0.8).astype(np.float32)
    loss, g = W.mlp_loss_grad(blob, X, Y, Mk)
    want_loss, want_g = M.loss_grad(blob, X, Y, Mk)
    assert abs(loss - want_loss) <= GRAD_RTOL * abs(want_loss)
    assert np.abs(g - want_g).max() <= GRAD_RTOL * np.abs(want_g).max()
    # per-layer relative L2 as well (small gradients in one layer must not hide)
    o = 0
    for _, shape in M.SHAPES:
        k = int(np.prod(shape))
        a, b = g[o:o + k], want_g[o:o + k]
        assert np.linalg.norm(a - b) <= GRAD_RTOL * max(np.linalg.norm(b), 1e-12)
        o += k


def test_training_lowers_the_loss(W):
    from wedge_gb300 import scheduler as S

    rng = np.random.default_rng(13)
    n = 600
    X = rng.uniform(0, 1, (n, 16)).astype(np.float32)
    Y = np.stack([X[:, 0] * 4 + 1, X[:, 1] * 3 - X[:, 2], np.sin(3 * X[:, 3]) + X[:, 4]], 1).astype(np.float32)
    Mk = np.ones((n, 3), np.float32)
    blob0 = S.init_blob(X, seed=1)
    loss0, _ = W.mlp_loss_grad(blob0, X, Y, Mk)
    blob, loss = W.mlp_train(blob0, X, Y, Mk, epochs=300, batch=64, lr=3e-3, seed=2)
    assert loss < 0.05 * loss0, (loss0, loss)
    blob2, loss2 = W.mlp_train(blob0, X, Y, Mk, epochs=300, batch=64, lr=3e-3, seed=2)
    assert np.array_equal(blob, blob2) and loss == loss2  # deterministic for a given order


def _rmat(O, scale, seed, symmetric=False):
    V, s, d = O.rmat(scale, 16, seed)
    if symmetric:
        s, d = O.symmetrise(s, d)
    s, d = O.sort_edges(V, s, d)
    return V, s, d


@pytest.mark.parametrize("sched", ["filtered", "probe", "learned"])
def test_every_schedule_is_bit_exact(W, O, sched):
    V, s, d = _rmat(O, 13, 5)
    Vs, ss, ds = _rmat(O, 13, 5, symmetric=True)
    w = O.weights(s, d)
    cc_want = O.Graph.from_edges(Vs, ss, ds, O.CC).run()[0]
    sssp_want = O.Graph.from_edges(V, s, d, O.SSSP, w=w).run(root=0)[0]
    always_wedge = None
    if sched == "learned":  # a network that always predicts the Wedge pull cheapest, everywhere in range
        from oracle import mlp_oracle as M

        always_wedge = np.zeros(M.BLOB, np.float32)
        always_wedge[16:32] = 1.0
        always_wedge[32:48] = -1e9
        always_wedge[48:64] = 1e9
        always_wedge[M.PARAM_OFFSET + M.PARAMS - 3:M.PARAM_OFFSET + M.PARAMS] = [10.0, 0.0, 10.0]
    runs = []
    for it in range(3):
        if sched == "filtered":
            p = dict(sched=W.SCHED_FILTERED)
        elif sched == "probe":
            p = dict(sched=W.SCHED_PROBE, probe_iter=it + 1, probe_mode=[W.MODE_DENSE, W.MODE_WEDGE, W.MODE_FILTERED][it])
        else:
            p = dict(sched=W.SCHED_LEARNED)
        runs.append(p)
    for p in runs:
        with W.Graph.from_edges(Vs, ss, ds) as g:
            if always_wedge is not None:
                g.set_scheduler(always_wedge)
            g.run(W.APP_CC, W.Params(**p))
            assert np.array_equal(g.read_results(), cc_want)
            log = g.iteration_log()
            if p["sched"] == W.SCHED_PROBE and p["probe_iter"] < len(log):
                assert log[p["probe_iter"]]["mode"] == p["probe_mode"]
            if p["sched"] == W.SCHED_LEARNED:
                assert all(r["mode"] == W.MODE_WEDGE for r in log[1:])
                assert any(r["learned"] for r in log[1:]) or len(log) < 2
            if p["sched"] == W.SCHED_FILTERED:
                assert all(r["mode"] == W.MODE_FILTERED for r in log[1:])
        with W.Graph.from_edges(V, s, d, w) as g:
            if always_wedge is not None:
                g.set_scheduler(always_wedge)
            g.run(W.APP_SSSP, W.Params(root=0, **p))
            assert np.array_equal(g.read_results(), sssp_want)
        with W.Graph.from_edges(V, s, d) as g:
            if always_wedge is not None:
                g.set_scheduler(always_wedge)
            g.run(W.APP_BFS, W.Params(root=0, **p))
            check_bfs(g.read_results(), V, s, d, 0)


def test_features_are_recorded_and_bounded(W):
    with W.Graph.rmat(14, 16, 3, symmetrise=False) as g:
        g.run(W.APP_BFS, W.Params(root=0))
        log = g.iteration_log()
    assert len(log) >= 3
    assert all(f == 0.0 for f in log[0]["features"])  # chosen before any pull
    for r in log[1:]:
        f = np.array(r["features"])
        assert np.all(np.isfinite(f)) and f.min() >= 0.0 and f.max() <= 2.0
        assert f[12] == 1.0 and f[13] == 0.0 and f[14] == 0.0  # BFS one-hot
        assert abs(f[5] + f[6] + f[7] + f[8] - 1.0) < 1e-5 or f[2] == 0.0


def test_trained_network_against_the_fixed_rule(W):
    """Held-out graphs (seeds not in the training set): every strategy's cost is
    measured per iteration, and the total cost of the network's choices is
    compared with the fixed rule's (gain = plain / learned) and with the
    per-iteration best (bound = plain / best, the most any choice could gain).
    Both are scored on the same measured cost table, so the comparison carries
    no run-to-run noise: the network must recover at least half of the bound."""
    from wedge_gb300 import scheduler as S

    if not os.path.exists(S.DEFAULT_NET):
        pytest.skip("no trained network committed")
    blob = S.load()
    samples = []
    for app, sym, wk in ((W.APP_BFS, False, W.WEIGHTS_NONE), (W.APP_CC, True, W.WEIGHTS_NONE),
                         (W.APP_SSSP, False, W.WEIGHTS_U64)):
        with W.Graph.rmat(20, 16, 91, symmetrise=sym, weight_kind=wk) as g:
            samples += S.probe_costs(g, app, reps=3, tag="heldout")
    r = S.evaluate(blob, samples)
    b = S.bound(samples)
    print("held-out R-MAT scale 20:", r, "bound", b)
    assert r["iterations"] > 5
    assert r["gain"] - 1.0 >= 0.5 * (b - 1.0)
    assert r["learned_us"] >= r["best_us"] - 1e-9

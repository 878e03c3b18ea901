"""The CPU restatement of the scheduler network (oracle/mlp_oracle.py): its
gradient against central finite differences, and its blob layout against the
constants the C ABI and the Python front end declare.  No GPU."""
import os
import re

import numpy as np

from oracle import mlp_oracle as M


def _blob(rng):
    b = rng.normal(0, 0.3, M.BLOB)
    b[0:16] = rng.normal(0, 1, 16)          # mu
    b[16:32] = rng.uniform(0.5, 2.0, 16)    # sd
    b[32:48] = -10.0
    b[48:64] = 10.0
    return b


def test_layout_matches_header_and_front_end():
    from wedge_gb300 import engine as W

    text = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "wedge_cuda.h")).read()
    assert int(re.search(r"#define WEDGE_SCHED_PARAM_OFFSET (\d+)", text).group(1)) == M.PARAM_OFFSET
    assert W.SCHED_PARAMS == M.PARAMS and W.SCHED_BLOB == M.BLOB and W.SCHED_PARAM_OFFSET == M.PARAM_OFFSET
    assert M.BLOB == 64 + 1024 + 64 + 4096 + 64 + 192 + 3 + 1


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    blob = _blob(rng)
    n = 9
    X = rng.normal(0, 1, (n, 16))
    Y = rng.normal(0, 1, (n, 3))
    Mk = (rng.uniform(size=(n, 3)) < 0.7).astype(float)
    loss, g = M.loss_grad(blob, X, Y, Mk)
    idx = rng.choice(M.PARAMS, 60, replace=False)
    h = 1e-6
    for i in idx:
        bp, bm = blob.copy(), blob.copy()
        bp[M.PARAM_OFFSET + i] += h
        bm[M.PARAM_OFFSET + i] -= h
        fd = (M.loss_grad(bp, X, Y, Mk)[0] - M.loss_grad(bm, X, Y, Mk)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_unmeasured_targets_do_not_contribute():
    rng = np.random.default_rng(4)
    blob = _blob(rng)
    X = rng.normal(0, 1, (5, 16))
    Y = rng.normal(0, 1, (5, 3))
    zero = np.zeros((5, 3))
    loss, g = M.loss_grad(blob, X, Y, zero)
    assert loss == 0.0 and not g.any()


def test_committed_network_against_the_fixed_rule_on_recorded_timings():
    """The committed network (wedge_gb300/data/sched_net.f32) on the held-out
    timings recorded with it (wedge_gb300/data/sched_samples.json: per-iteration
    cost of every strategy on R-MAT and grid graphs whose seeds are not in the
    training set).  The decision rule is the engine's; the network outputs come
    from the float64 restatement here, so this runs without a GPU."""
    import json

    from wedge_gb300 import scheduler as S

    blob = np.fromfile(S.DEFAULT_NET, np.float32)
    samples = json.load(open(S.DEFAULT_SAMPLES))["eval"]
    X, _, _ = S.to_arrays(samples)
    pred, _ = M.forward(blob, X)
    r = S.evaluate(blob, samples, pred=pred)
    assert r["iterations"] >= 50
    assert r["learned_us"] <= r["plain_us"]          # never worse than the rule it falls back to
    # the fixed rule's excess over the per-iteration best (plain_regret_us) is
    # what a scheduler can win; the network must recover at least half of it
    # (measured: gain 1.030 of a possible 1.049, 62% of the excess recovered;
    # the network trained without the scale-26 graph recovered 90% here but
    # left the scale-26 choices to the fixed rule)
    assert r["plain_us"] - r["learned_us"] >= 0.5 * r["plain_regret_us"]
    assert r["gain"] > 1.0

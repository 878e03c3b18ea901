"""CPU restatement of the scheduler network -- test infrastructure only.

The network (16 features -> 64 -> 64 -> 3, ReLU, predicted log2 costs of the
dense, Wedge and source-filtered pulls) has no counterpart in the reference:
the reference decides with its fixed threshold (execution_bfs.c:132,141).  This
float64 restatement of the forward pass, the loss and its gradient is the
oracle the engine's CUDA kernels (wedge_gb300/csrc/sched.cu) are checked
against; only tests import it.

Blob layout (float32, as include/wedge_cuda.h documents it):
    mu[16] sd[16] lo[16] hi[16] | W1[64][16] b1[64] W2[64][64] b2[64] W3[3][64] b3[3] | margin
"""
from __future__ import annotations

import numpy as np

NF, NH, NO = 16, 64, 3
PARAM_OFFSET = 4 * NF
SHAPES = [("W1", (NH, NF)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NO, NH)), ("b3", (NO,))]
PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)
BLOB = PARAM_OFFSET + PARAMS + 1


def unpack(blob):
    b = np.asarray(blob, np.float64)
    assert b.shape == (BLOB,)
    out = {"mu": b[0:NF], "sd": b[NF:2 * NF], "lo": b[2 * NF:3 * NF], "hi": b[3 * NF:4 * NF]}
    o = PARAM_OFFSET
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = b[o:o + n].reshape(shape)
        o += n
    out["margin"] = b[o]
    return out


def forward(blob, X):
    """outputs [n][3] and the activations the gradient needs"""
    p = unpack(blob)
    xs = (np.asarray(X, np.float64) - p["mu"]) / p["sd"]
    a1 = xs @ p["W1"].T + p["b1"]
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ p["W2"].T + p["b2"]
    h2 = np.maximum(a2, 0.0)
    y = h2 @ p["W3"].T + p["b3"]
    return y, (p, xs, h1, h2)


def loss_grad(blob, X, Y, M):
    """sum over measured outputs of (y - target)^2 / n, and d loss / d params (flat, blob order)"""
    n = len(X)
    y, (p, xs, h1, h2) = forward(blob, X)
    e = np.where(np.asarray(M) != 0, y - np.asarray(Y, np.float64), 0.0)
    loss = float((e * e).sum() / n)
    dy = 2.0 * e / n
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    d2 = (dy @ p["W3"]) * (h2 > 0)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(0)
    d1 = (d2 @ p["W2"]) * (h1 > 0)
    g["W1"] = d1.T @ xs
    g["b1"] = d1.sum(0)
    return loss, np.concatenate([g[name].ravel() for name, _ in SHAPES])


def params_view(blob):
    """the trainable slice of a blob (a view)"""
    return blob[PARAM_OFFSET:PARAM_OFFSET + PARAMS]

"""Autotuner of the batched multi-query kernel.

The persistent kernel has four knobs (wedge_batch_tuning_t): the dense/Wedge
threshold of each query's next pull, how many 32-edge chunks a warp takes from
the work queue at a time, how many persistent blocks run per SM, and the
out-degree above which the Wedge build expands a vertex with a whole warp
instead of one lane.  The tuner times every combination of a small grid on the
workload (captured CUDA graph, CUDA events, median of repeats) and keeps the
fastest; the table goes to data/batch_tuning.json.

    python -m wedge_gb300.autotune --out DIR
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import time

import numpy as np

from . import batch as B
from . import engine as W

DEFAULT_TUNING = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "batch_tuning.json")
GRID = {"threshold_pct": (10, 20, 40), "grab": (2, 8, 32), "blocks_per_sm": (1, 2, 4), "split": (8, 32, 128)}


def load_tuning(path: str = DEFAULT_TUNING):
    """the tuned knobs as a BatchTuning, or None (the engine's defaults) if no table exists"""
    try:
        with open(path) as f:
            best = json.load(f)["best"]
    except (OSError, KeyError, ValueError):
        return None
    return W.BatchTuning(**{k: int(best[k]) for k in GRID})


def tune(batch: W.Batch, grid=GRID, reps: int = 3, log=print):
    results = []
    keys = list(grid)
    for values in itertools.product(*(grid[k] for k in keys)):
        cfg = dict(zip(keys, values))
        t = W.BatchTuning(**cfg)
        batch.run(t, flags=W.FLAG_GRAPH)  # capture + warm-up
        ms = [batch.run(t, flags=W.FLAG_GRAPH)["running_ms"] for _ in range(reps)]
        results.append({**cfg, "ms": float(np.median(ms))})
        log(f"{cfg}: {results[-1]['ms']:.3f} ms")
    best = min(results, key=lambda r: r["ms"])
    return best, results


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    t0 = time.time()
    params = B.graph_params()
    qs = B.queries(params)
    graphs = B.load_graphs(params)
    with W.Batch(graphs, qs) as b:
        default_ms = float(np.median([b.run(flags=W.FLAG_GRAPH)["running_ms"] for _ in range(a.reps + 1)][1:]))
        best, results = tune(b, reps=a.reps)
    os.makedirs(a.out, exist_ok=True)
    table = {"workload": "256 BFS + 256 SSSP over 64 R-MAT graphs (scales 12-20, edge factors 8-32, seed 4)",
             "default_ms": default_ms, "best": best, "speedup_vs_default": default_ms / best["ms"],
             "results": results, "seconds": time.time() - t0}
    with open(os.path.join(a.out, "batch_tuning.json"), "w") as f:
        json.dump(table, f, indent=1)
    print(json.dumps({k: table[k] for k in ("default_ms", "best", "speedup_vs_default")}, indent=1))
    for g in graphs:
        g.close()


if __name__ == "__main__":
    main()

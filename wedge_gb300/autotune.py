"""Autotuners: the batched multi-query kernel and the single-query engine.

Batched kernel.  The persistent kernel has four knobs (wedge_batch_tuning_t):
the dense/Wedge threshold of each query's next pull, how many 32-edge chunks a
warp takes from the work queue at a time, how many persistent blocks run per
SM, and the out-degree above which the Wedge build expands a vertex with a
whole warp instead of one lane.  The tuner times every combination of a small
grid on the workload (captured CUDA graph, CUDA events, median of repeats) and
keeps the fastest; the table goes to data/batch_tuning.json.

Single-query engine.  Each application's launches have the knobs of
wedge_cuda_set_knob: the shared-memory hub cache's bytes (what the pulls
gather from shared memory instead of L1/L2), the BFS/CC per-destination probe
window, and for SSSP the dense-pull tile (256 or 512 in-edges) and whether the
pulls gather a 32-bit copy of the distances.  The tuner times every
combination per application on a workload's graphs (the runs' own CUDA-event
Running Time, median of repeats) and stores the fastest per application in
data/engine_tuning.json, keyed by the workload's graph (scale, edge factor);
apply_engine_tuning() sets them on a handle when its graph matches.

    python -m wedge_gb300.autotune --out DIR                 # batched kernel
    python -m wedge_gb300.autotune --engine --out DIR        # engine, R-MAT scale 26
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
DEFAULT_ENGINE_TUNING = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "engine_tuning.json")
HUB_CHOICES = (0, 32768, 65536, 81920, 98304, 114688)
ENGINE_SPACE = {
    "bfs": {"hub_bytes": HUB_CHOICES, "probe_edges": (8, 16, 32)},
    "cc": {"hub_bytes": HUB_CHOICES, "probe_edges": (8, 16, 32)},
    "sssp": {"hub_bytes": HUB_CHOICES, "sssp_tile": (256, 512), "sssp_narrow": (0, 1)},
    "pr": {"hub_bytes": HUB_CHOICES},
}
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


def _median_ms(g: W.Graph, app: int, params: W.Params, reps: int) -> float:
    g.run(app, params)  # builds the state under the knobs, captures the loop
    return float(np.median([g.run(app, params)["running_ms"] for _ in range(reps)]))


def tune_engine(g: W.Graph, app: int, params: W.Params, space: dict, reps: int = 5, log=print):
    """every combination of the knobs in space on one handle; returns (default, best, results),
    each result {knob: value, ..., "ms": median Running Time}; the knobs go back to their
    defaults afterwards"""
    keys = list(space)
    for k in keys:
        g.set_knob(k, None)
    default = {**{k: g.knob(k) for k in keys}, "ms": _median_ms(g, app, params, reps)}
    results = []
    for values in itertools.product(*(space[k] for k in keys)):
        cfg = dict(zip(keys, values))
        for k, v in cfg.items():
            g.set_knob(k, v)
        results.append({**cfg, "ms": _median_ms(g, app, params, reps)})
        log(f"app {app} {cfg}: {results[-1]['ms']:.3f} ms")
    for k in keys:
        g.set_knob(k, None)
    best = min(results, key=lambda r: r["ms"])
    if best["ms"] >= default["ms"]:
        best = default  # the defaults are in the grid; keep them on a tie
    return default, best, results


def load_engine_tuning(path: str = DEFAULT_ENGINE_TUNING):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def apply_engine_tuning(g: W.Graph, app_name: str, scale: int, edge_factor: int, table=None) -> dict:
    """set the tuned knobs of app_name on g when the table was tuned on a graph of this
    scale and edge factor; returns the knobs set ({} when none apply)"""
    table = table if table is not None else load_engine_tuning()
    if not table or (table.get("scale"), table.get("edge_factor")) != (scale, edge_factor):
        return {}
    best = table.get("apps", {}).get(app_name, {}).get("best")
    if not best:
        return {}
    knobs = {k: int(v) for k, v in best.items() if k in W.KNOB_NAMES}
    for k, v in knobs.items():
        g.set_knob(k, v)
    return knobs


def engine_main(a):
    """tune the four applications on the R-MAT graphs of one scale and edge factor (seed 5,
    the benchmark's: BFS and SSSP from vertex 0, CC on the symmetrised graph, 30 PageRank
    iterations in compensated FP32, plain schedule, threshold 20%)"""
    t0 = time.time()
    scale, ef, seed = a.scale, a.edge_factor, 5
    apps = {
        "bfs": (W.Graph.rmat(scale, ef, seed), W.APP_BFS, W.Params(root=0, threshold_pct=20, flags=W.FLAG_GRAPH)),
        "cc": (W.Graph.rmat(scale, ef, seed, symmetrise=True), W.APP_CC, W.Params(threshold_pct=20, flags=W.FLAG_GRAPH)),
        "sssp": (W.Graph.rmat(scale, ef, seed, weight_kind=W.WEIGHTS_U64), W.APP_SSSP,
                 W.Params(root=0, threshold_pct=20, flags=W.FLAG_GRAPH)),
        "pr": (W.Graph.rmat(scale, ef, seed), W.APP_PR,
               W.Params(num_iterations=30, damping=0.85, precision=W.PREC_FP32C, flags=W.FLAG_GRAPH)),
    }
    table = {"workload": f"R-MAT scale {scale}, edge factor {ef}, seed {seed}: BFS, CC (symmetrised), SSSP, "
                         "30 PageRank iterations (compensated FP32)",
             "scale": scale, "edge_factor": ef, "reps": a.reps, "apps": {}}
    for name, (g, app, params) in apps.items():
        default, best, results = tune_engine(g, app, params, ENGINE_SPACE[name], a.reps)
        table["apps"][name] = {"default": default, "best": best, "speedup_vs_default": default["ms"] / best["ms"],
                               "results": results}
        g.close()
    table["seconds"] = time.time() - t0
    os.makedirs(a.out, exist_ok=True)
    with open(os.path.join(a.out, "engine_tuning.json"), "w") as f:
        json.dump(table, f, indent=1)
    print(json.dumps({n: {k: v for k, v in t.items() if k != "results"} for n, t in table["apps"].items()}, indent=1))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--engine", action="store_true", help="tune the single-query engine's knobs")
    ap.add_argument("--scale", type=int, default=26)
    ap.add_argument("--edge-factor", type=int, default=16)
    a = ap.parse_args()
    if a.engine:
        engine_main(a)
        return
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

"""The batched multi-query workload: 256 BFS + 256 SSSP queries over 64
independent R-MAT graphs of uneven size, run together by one persistent kernel
(wedge_cuda_batch_*).

Graph i (of 64) has scale 12 + h % 9 (12..20) and edge factor 8 + (h >> 8) % 25
(8..32), with h = mix64(mix64(seed) + i) and the workload seed 4; its R-MAT
seed is 4000 + i.  Each graph gets 4 BFS and 4 SSSP roots,
root j = mix64(h + 1 + j) mod V.  Weights are the multiplicative hash of
(src, dst) used by every weighted graph here (uint64 in [1, 255]).
"""
from __future__ import annotations

from . import engine as W

MASK = (1 << 64) - 1


def mix64(z: int) -> int:
    """splitmix64 finaliser (the generators' counter-based draw)"""
    z = (z + 0x9E3779B97F4A7C15) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


def graph_params(num_graphs: int = 64, seed: int = 4, scales=(12, 20), edge_factors=(8, 32)):
    """[(scale, edge_factor, rmat_seed, h)] of the workload's graphs"""
    out = []
    base = mix64(seed)
    ns, ne = scales[1] - scales[0] + 1, edge_factors[1] - edge_factors[0] + 1
    for i in range(num_graphs):
        h = mix64((base + i) & MASK)
        out.append((scales[0] + h % ns, edge_factors[0] + (h >> 8) % ne, seed * 1000 + i, h))
    return out


def queries(params, bfs_per_graph: int = 4, sssp_per_graph: int = 4):
    """[(graph index, app, root)] of the workload"""
    out = []
    for gi, (scale, _ef, _seed, h) in enumerate(params):
        V = 1 << scale
        for j in range(bfs_per_graph + sssp_per_graph):
            app = W.APP_BFS if j < bfs_per_graph else W.APP_SSSP
            out.append((gi, app, mix64((h + 1 + j) & MASK) % V))
    return out


def load_graphs(params):
    """the graphs on the device (weighted, so BFS and SSSP queries share one handle)"""
    return [W.Graph.rmat(scale, ef, seed, weight_kind=W.WEIGHTS_U64) for scale, ef, seed, _h in params]


def main():
    """Run the batched workload (or its first N graphs) and print the device time
    of each run: python -m wedge_gb300.batch [--graphs N] [--runs R] [--no-graph]"""
    import argparse
    import json
    import os

    from . import autotune as A

    ap = argparse.ArgumentParser(description="the batched multi-query workload in one persistent kernel")
    ap.add_argument("--graphs", type=int, default=64, help="the first N graphs of the workload (and their queries)")
    ap.add_argument("--runs", type=int, default=3)
    ap.add_argument("--no-graph", action="store_true", help="launch the kernel directly, not from a CUDA graph")
    a = ap.parse_args()
    params = graph_params()[:a.graphs]
    qs = queries(params)
    graphs = load_graphs(params)
    tuning = A.load_tuning() if os.path.exists(A.DEFAULT_TUNING) else None
    flags = 0 if a.no_graph else W.FLAG_GRAPH
    try:
        with W.Batch(graphs, qs) as b:
            ms = [b.run(tuning, flags)["running_ms"] for _ in range(a.runs)]
        print(json.dumps({"graphs": len(graphs), "queries": len(qs), "edges": sum(g.E for g in graphs),
                          "running_ms": [round(x, 3) for x in ms]}))
    finally:
        for g in graphs:
            g.close()


if __name__ == "__main__":
    main()

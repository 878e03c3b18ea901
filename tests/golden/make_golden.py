"""Generates tests/golden/golden.npz from the reference itself.

The reference is compiled from its own sources (oracle/Makefile `ref`, needs an
x86-64 AVX2 host and the reference tree) and run single-threaded on small
synthetic graphs written in its binary edge-list format.  The fixture stores,
per case, the generator parameters, a checksum of the edge list, and the raw
64-bit vertex properties (plus out-degrees for PageRank) that the reference
produced, so tests can regenerate the same graph and compare.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

# (name, kind, params, runs: None = every entry of RUNS, else the indices of RUNS)
GRAPHS = [
    ("rmat10", "rmat", dict(scale=10, edge_factor=16, seed=1), None),
    ("rmat12", "rmat", dict(scale=12, edge_factor=8, seed=2), None),
    ("grid32", "grid", dict(side=32, frac=0.01, seed=3), None),
    # the PageRank configuration's graph (65,536 vertices, 1,048,576 edges): hubs span many
    # tiles; one run per application keeps the fixture small
    ("rmat16", "rmat", dict(scale=16, edge_factor=16, seed=1), (0, 4, 6, 8)),
]
# (app, variant, extra run args)
RUNS = [
    ("bfs", "directed", dict(root=0)),
    ("bfs", "directed", dict(root=5)),
    ("bfs", "directed", dict(root=0, threshold_pct=100)),
    ("bfs", "directed", dict(root=0, threshold_pct=0)),
    ("cc", "symmetric", dict()),
    ("cc", "directed", dict()),
    ("sssp", "directed", dict(root=0)),
    ("sssp", "directed", dict(root=7, threshold_pct=100)),
    ("pr", "directed", dict(iterations=16)),
]


def make_graph(kind, p):
    if kind == "rmat":
        V, s, d = O.rmat(p["scale"], p["edge_factor"], p["seed"])
    else:
        V, s, d = O.grid(p["side"], p["frac"], p["seed"])
    return V, s, d


def graph_variant(V, s, d, variant):
    if variant == "symmetric":
        s, d = O.symmetrise(s, d)
    return O.sort_edges(V, s, d)


def checksum(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def main():
    O.build()
    if not O.build_ref():
        raise SystemExit("the reference could not be built here (needs its sources and an AVX2 host)")
    out, meta = {}, []
    with tempfile.TemporaryDirectory() as td:
        for gname, kind, gp, which in GRAPHS:
            V, s0, d0 = make_graph(kind, gp)
            for app, variant, ra in (RUNS if which is None else [RUNS[i] for i in which]):
                s, d = graph_variant(V, s0, d0, variant)
                w = O.weights(s, d) if app == "sssp" else None
                path = os.path.join(td, f"{gname}_{app}_{variant}.bin")
                O.write_file(path, V, s, d, w)
                props, outdeg, stats = O.run_reference(path, app, threads=1, iterations=ra.get("iterations", 1),
                                                       root=ra.get("root", 0),
                                                       threshold_pct=ra.get("threshold_pct", 20))
                key = f"{gname}.{app}.{variant}.r{ra.get('root', 0)}.t{ra.get('threshold_pct', 20)}"
                out[key + ".props"] = props
                if outdeg is not None:
                    out[key + ".outdeg"] = outdeg
                meta.append(dict(key=key, graph=gname, kind=kind, params=gp, app=app, variant=variant, run=ra,
                                 V=int(V), E=int(len(s)), edges_sha=checksum(s, d), stats=stats))
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(f"wrote {len(meta)} cases")


if __name__ == "__main__":
    main()

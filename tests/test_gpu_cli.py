"""The reference-facing programs end to end on the GPU: wedge-gen writes the
reference's binary edge-list format byte-identically to the oracle's writer;
the `wedge` CLI reads it, runs every application, writes the -o file (GPU
formatting for BFS/CC/SSSP) in the reference's line formats
(execution_*:get_vertex_prop_string), and prints the ITERATION_STATS CSV."""
import os
import subprocess

import numpy as np
import pytest

from helpers import check_bfs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W(engine_lib):
    return engine_lib


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _bin(name):
    from wedge_gb300 import build as B

    return os.path.join(B.OUT_BIN, name)


def _run(args, **kw):
    r = subprocess.run(args, capture_output=True, text=True, timeout=600, **kw)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


@pytest.mark.parametrize("kind,args,weights", [
    ("rmat", ["12", "16", "7"], None), ("rmat", ["11", "8", "3", "--sym"], None),
    ("rmat", ["12", "16", "7"], "u64"), ("rmat", ["10", "16", "5"], "f64"), ("grid", ["48", "0.01", "3"], "u64")])
def test_wedge_gen_matches_oracle_writer(O, tmp_path, kind, args, weights):
    out = tmp_path / "g.bin"
    cmd = [_bin("wedge-gen"), kind] + args[:3] + [a for a in args[3:]]
    if weights:
        cmd.append(f"--weights={weights}")
    _run(cmd + ["-o", str(out)])
    if kind == "rmat":
        V, s, d = O.rmat(int(args[0]), int(args[1]), int(args[2]))
        if "--sym" in args:
            s, d = O.symmetrise(s, d)
    else:
        V, s, d = O.grid(int(args[0]), float(args[1]), int(args[2]))
    s, d = O.sort_edges(V, s, d)
    w = None if weights is None else O.weights(s, d, O.WEIGHTS_U64 if weights == "u64" else O.WEIGHTS_F64)
    ref = tmp_path / "ref.bin"
    O.write_file(str(ref), V, s, d, w)
    assert out.read_bytes() == ref.read_bytes()


def _lines(path):
    out = {}
    for ln in open(path):
        v, x = ln.split()
        out[int(v)] = x
    return out


def test_cli_outputs_every_application(O, tmp_path):
    f = tmp_path / "g.bin"
    fw = tmp_path / "gw.bin"
    _run([_bin("wedge-gen"), "rmat", "12", "16", "9", "-o", str(f)])
    _run([_bin("wedge-gen"), "rmat", "12", "16", "9", "--weights=u64", "-o", str(fw)])
    V, s, d = O.rmat(12, 16, 9)
    s, d = O.sort_edges(V, s, d)
    w = O.weights(s, d)
    # CC
    o = tmp_path / "cc.txt"
    r = _run([_bin("wedge"), "-i", str(f), "-a", "cc", "-o", str(o), "--graph"])
    assert "on the GPU" in r.stdout
    ref, _, _ = O.Graph.from_edges(V, s, d, O.CC).run()
    got = _lines(o)
    assert len(got) == V and all(got[v] == "%.0f" % ref.view(np.float64)[v] for v in range(V))
    # SSSP (uint64 weights)
    o = tmp_path / "sssp.txt"
    _run([_bin("wedge"), "-i", str(fw), "-a", "sssp", "-r", "3", "-o", str(o)])
    ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=3)
    got = _lines(o)
    assert all(got[v] == "%d" % ref.view(np.int64)[v] for v in range(V))
    # BFS: the parents printed are valid ones (levels and in-edges)
    o = tmp_path / "bfs.txt"
    r = _run([_bin("wedge"), "-i", str(f), "-a", "bfs", "-r", "5", "-o", str(o), "--iteration-stats"])
    got = _lines(o)
    par = np.array([int(got[v]) for v in range(V)], np.int64).view(np.uint64)
    check_bfs(par, V, s, d, 5)
    rows = [ln.split(",") for ln in r.stderr.strip().splitlines()]
    it = int([ln for ln in r.stdout.splitlines() if ln.startswith("Total Iterations")][0].split("=")[1])
    assert len(rows) == it and all(len(x) == 4 and x[1] in ("true", "false") for x in rows)
    assert all(float(x[2]) > 0.0 and float(x[3]) >= 0.0 for x in rows)
    # PageRank (host formatting of %.4le)
    o = tmp_path / "pr.txt"
    r = _run([_bin("wedge"), "-i", str(f), "-a", "pr", "-N", "4", "-o", str(o)])
    assert "on the host" in r.stdout
    ref, od, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=4)
    od = od.view(np.float64)  # PageRank keeps out-degrees as doubles (graph_vertex_outdegrees)
    got = _lines(o)
    want = ref.view(np.float64) * np.where(od == 0, V, od)
    # the reference's %.4le strings: the FP64 ranks agree with the oracle's to
    # about 1e-12, so a line may differ only where a value lies that close to a
    # rounding boundary of its fifth digit
    differ = [v for v in range(V) if got[v] != "%.4e" % want[v]]
    assert len(differ) <= 2, differ[:10]
    assert all(abs(float(got[v]) - want[v]) <= 1e-4 * abs(want[v]) for v in differ)


def test_gpu_formatting_equals_host_formatting(W, O, tmp_path):
    """the GPU writer's lines equal the reference formats applied to the results"""
    with W.Graph.rmat(13, 8, 4, weight_kind=W.WEIGHTS_U64) as g:
        for app, root in ((W.APP_BFS, 2), (W.APP_CC, 0), (W.APP_SSSP, 7)):
            g.run(app, W.Params(root=root))
            props = g.read_results()
            od = g.read_outdegrees()
            p = tmp_path / f"o{app}.txt"
            on_gpu, ms = g.write_output(str(p))
            assert on_gpu
            want = "".join("%d %s\n" % (v, W.prop_string(app, int(props[v]), int(od[v]), g.V))
                           for v in range(g.V))
            assert p.read_text() == want

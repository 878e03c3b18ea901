"""Benchmark of the edge-pull engine: GTEPS of BFS + CC on R-MAT scale 24.

Workload (one "step"): BFS from vertex 0 on the directed R-MAT graph (scale 24,
edge factor 16, a/b/c/d = 0.57/0.19/0.19/0.05, seed 2: 16,777,216 vertices,
268,435,456 edges) and Connected Components on its symmetrised copy
(536,870,912 edges), plain fixed-threshold scheduling (t = 20%).  Synthetic
graphs are generated on the device with the same counter-based generator the
CPU side uses.  GTEPS counts every input edge once per traversal:
    value = steps * (|E_bfs| + |E_cc|) / time.

Arms
  (default)          the CUDA engine through its C ABI; graphs resident in HBM
  --impl reference   the reference's algorithm on the host cores: the oracle's
                     portable-C restatement (the AVX2 reference cannot be
                     compiled on the Arm host), all host threads

Multi-GPU: every rank runs an independent replica of the workload (the
traversal itself is not sharded); value = all ranks' edges / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RMAT_ABC = (0.57, 0.19, 0.19)
WORKLOAD = dict(workload="rmat24_bfs_cc", scale=24, edge_factor=16, seed=2, bfs_root=0, threshold_pct=20)


def workload_name(scale: int, ef: int) -> str:
    """the workload as run: the default is rmat24_bfs_cc (R-MAT scale 24, edge factor 16)"""
    if (scale, ef) == (WORKLOAD["scale"], WORKLOAD["edge_factor"]):
        return WORKLOAD["workload"]
    return f"rmat{scale}_ef{ef}_bfs_cc"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=WORKLOAD["scale"])
    ap.add_argument("--edge-factor", type=int, default=WORKLOAD["edge_factor"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="graph", choices=["graph", "host"], help="traversal loop: CUDA graph or host")
    return ap.parse_args()


# ---------------------------------------------------------------- distributed helpers
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None

    def init(self, backend):
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def done(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region"""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.out.flush()
        self.out.seek(0)
        rows = [r.split(",") for r in self.out.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.out.name)
        sm = sorted(float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit())
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4) if r[5 + j].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].strip().replace(".", "").isdigit()),
                                   default=None)}


def visible_index(local_rank: int) -> int:
    cvd = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [x for x in cvd.split(",") if x.strip()]
    if ids and ids[0].strip().isdigit():
        return int(ids[0])
    return local_rank


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------- algorithmic bytes per pull launch
def pull_bytes(app: str, rec: dict, V: int, Vne: int) -> float:
    """Compulsory bytes of one pull launch, counting each touched array once:
    sources 4*E_s, destination offsets 8*V_s (+ ids 4*V_s), the property array
    read once, the frontier bitmaps, and the writes of changed properties."""
    Es, Vs, act = rec["edges_scanned"], rec["dsts_scanned"], rec["vertices_activated"]
    bitmap = V / 8.0
    if app == "bfs":
        # sources, offsets+ids, current frontier + next frontier + visited bits, parent writes
        return 4.0 * Es + 12.0 * Vs + 2 * bitmap + Vne / 8.0 + 4.0 * act
    if app == "cc":
        # sources, offsets+ids, labels read once, label writes, changed bitmap
        return 4.0 * Es + 12.0 * Vs + 4.0 * V + 4.0 * act + bitmap
    raise ValueError(app)


# ---------------------------------------------------------------- our arm
def run_ours(args, dist: Dist):
    if dist.world > 1:
        # one GPU per process, chosen before any CUDA call: the engine binds to the current device
        ids = [x for x in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if x.strip()]
        os.environ["CUDA_VISIBLE_DEVICES"] = ids[dist.local] if len(ids) > dist.local else str(dist.local)
    import ctypes
    import numpy as np
    import torch

    dist.init("nccl")
    torch.cuda.set_device(0)
    import wedge_gb300 as W

    steps, warmup = args.steps, max(3, args.warmup)
    scale, ef = args.scale, args.edge_factor
    gb = W.Graph.rmat(scale, ef, WORKLOAD["seed"], symmetrise=False)
    gc = W.Graph.rmat(scale, ef, WORKLOAD["seed"], symmetrise=True)
    V, E_bfs, E_cc = gb.V, gb.E, gc.E
    flags = W.FLAG_GRAPH if args.mode == "graph" else 0
    p_bfs = W.Params(root=WORKLOAD["bfs_root"], threshold_pct=WORKLOAD["threshold_pct"], flags=flags)
    p_cc = W.Params(threshold_pct=WORKLOAD["threshold_pct"], flags=flags)
    try:  # events on the engine's own streams; each run returns after its stream drained
        s_bfs = torch.cuda.ExternalStream(gb.stream)
        s_cc = torch.cuda.ExternalStream(gc.stream)
    except Exception:
        s_bfs = s_cc = torch.cuda.current_stream()

    def step(counts):
        a = gb.run(W.APP_BFS, p_bfs)
        b = gc.run(W.APP_CC, p_cc)
        counts["launches"] += a["kernel_launches"] + b["kernel_launches"]
        counts["iters_bfs"] = a["iterations"]
        counts["iters_cc"] = b["iterations"]
        counts["wedge_bfs"] = a["wedge_iterations"]
        counts["wedge_cc"] = b["wedge_iterations"]

    counts = {"launches": 0}
    for _ in range(warmup):
        step(counts)
    torch.cuda.synchronize()

    # ---- device-timed region: inputs resident in HBM
    sampler = ClockSampler(visible_index(dist.local))
    sampler.start()
    counts = {"launches": 0}
    dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s_bfs)
    t0 = time.perf_counter()
    for _ in range(steps):
        step(counts)
    e1.record(s_cc)
    e1.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    dist.barrier()
    clocks = sampler.stop()
    dev_ms = e0.elapsed_time(e1)
    t_max = dist.max(dev_ms / 1e3)
    edges_step = E_bfs + E_cc
    value = dist.world * steps * edges_step / t_max / 1e9

    # ---- the same steps under the learned scheduler (on-device network, plain-rule fallback)
    learned = _learned_arm(W, gb, gc, p_bfs, p_cc, steps, warmup, s_bfs, s_cc, edges_step, dist, value)

    # ---- end to end through the C ABI with host buffers: query parameters in,
    # full property arrays (8 bytes per vertex, graph_vertex_props) out, every step
    host_bfs = torch.empty(V, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    host_cc = torch.empty(V, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    e2e_steps = max(3, min(steps, 20))
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        gb.run(W.APP_BFS, p_bfs)
        gb.read_results(host_bfs)
        gc.run(W.APP_CC, p_cc)
        gc.read_results(host_cc)
    e2e_wall = dist.max(time.perf_counter() - t0)
    e2e_value = dist.world * e2e_steps * edges_step / e2e_wall / 1e9
    params_bytes = 2 * ctypes.sizeof(W.Params)  # each query's wedge_params_t, carried to the device in kernel arguments

    # ---- roofline of the dominant kernel (the edge pull), per launch, timed with CUDA events
    rec_b = _timed_records(W, gb, W.APP_BFS, p_bfs)
    rec_c = _timed_records(W, gc, W.APP_CC, p_cc)
    peak, peak_kind = measured_peaks()
    Vne_b = Vne_c = V  # visited-bitmap term bounded by |V|/8
    pull_ms = sum(r["pull_ms"] for r in rec_b + rec_c)
    pull_bytes_tot = sum(pull_bytes("bfs", r, V, Vne_b) for r in rec_b) + \
        sum(pull_bytes("cc", r, V, Vne_c) for r in rec_c)
    n_launch = len(rec_b) + len(rec_c)
    achieved = pull_bytes_tot / (pull_ms / 1e3) / 1e9 if pull_ms > 0 else 0.0
    dense = [r for r in rec_b + rec_c if not r["used_wedge"]]
    dense_ms = sum(r["pull_ms"] for r in dense)
    dense_bytes = sum(pull_bytes("bfs", r, V, Vne_b) for r in rec_b if not r["used_wedge"]) + \
        sum(pull_bytes("cc", r, V, Vne_c) for r in rec_c if not r["used_wedge"])
    traffic = _ncu_traffic()

    line = {
        "metric": "GTEPS per app at 1 GB300 (BFS + CC, plain fixed-threshold schedule)",
        "value": round(value, 4),
        "unit": "GTEPS",
        "n_gpus": dist.world,
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": round(t_max * 1e3 / steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (device R-MAT, counter-based generator; no dataset)",
        "config": {"workload": workload_name(scale, ef), "scale": scale, "edge_factor": ef, "seed": WORKLOAD["seed"],
                   "vertices": V, "edges_bfs": E_bfs, "edges_cc": E_cc, "bfs_root": WORKLOAD["bfs_root"],
                   "threshold_pct": WORKLOAD["threshold_pct"], "loop": args.mode,
                   "l2": "inputs larger than L2 (sources 1 GiB / 2 GiB vs 126 MB L2); no flush",
                   "parallelism": "replicas" if dist.world > 1 else "single GPU"},
        "per_app": {
            "bfs": {"iterations": counts.get("iters_bfs"), "wedge_iterations": counts.get("wedge_bfs")},
            "cc": {"iterations": counts.get("iters_cc"), "wedge_iterations": counts.get("wedge_cc")},
        },
        "e2e": {"value": round(e2e_value, 4), "unit": "GTEPS", "h2d_bytes_per_step": params_bytes,
                "d2h_bytes_per_step": 2 * 8 * V, "steps": e2e_steps,
                "what": "wedge_cuda_run + wedge_cuda_read_results per app into pinned host memory; "
                        "graph resident (loaded once, as the reference excludes load from Running Time)"},
        "roofline": {"bound": "hbm", "kernel": "edge pull: dst_kernel + pull_kernel (BFS + CC, all iterations)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "traffic": traffic,
                     "traffic_scope": "achieved, algorithmic_bytes and traffic are per step: all pull launches of "
                                      "one BFS + one CC traversal (traffic: ncu DRAM bytes, profiles/)",
                     "pull_iterations": n_launch,
                     "algorithmic_bytes": int(pull_bytes_tot), "pull_ms": round(pull_ms, 4),
                     "dense_only": {"achieved": round(dense_bytes / (dense_ms / 1e3) / 1e9, 1) if dense_ms else None,
                                    "frac": round(dense_bytes / (dense_ms / 1e3) / 1e9 / peak, 4) if dense_ms else None,
                                    "pull_iterations": len(dense)}},
        "learned": learned,
        "clocks": clocks,
        "gpu_launches": int(counts["launches"]),
        "wall_s_timed": round(wall, 4),
    }
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(scale, ef)
    gb.close()
    gc.close()
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.done()


def _learned_arm(W, gb, gc, p_bfs, p_cc, steps, warmup, s_bfs, s_cc, edges_step, dist, plain_value):
    """GTEPS of the same workload with WEDGE_SCHED_LEARNED and the committed network"""
    import torch
    from wedge_gb300 import scheduler as S

    try:
        blob = S.load()
    except Exception as e:  # no trained network: report it, do not guess
        return {"unavailable": f"no scheduler network: {e}"}
    gb.set_scheduler(blob)
    gc.set_scheduler(blob)
    lb = W.Params(root=p_bfs.root, threshold_pct=p_bfs.threshold_pct, flags=p_bfs.flags, sched=W.SCHED_LEARNED)
    lc = W.Params(threshold_pct=p_cc.threshold_pct, flags=p_cc.flags, sched=W.SCHED_LEARNED)
    for _ in range(warmup):
        gb.run(W.APP_BFS, lb)
        gc.run(W.APP_CC, lc)
    dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s_bfs)
    for _ in range(steps):
        gb.run(W.APP_BFS, lb)
        gc.run(W.APP_CC, lc)
    e1.record(s_cc)
    e1.synchronize()
    t = dist.max(e0.elapsed_time(e1) / 1e3)
    # which iterations the network changed (one timed-free run per app)
    changed = {}
    for name, g, app, p in (("bfs", gb, W.APP_BFS, lb), ("cc", gc, W.APP_CC, lc)):
        g.run(app, p)
        log = g.iteration_log()
        changed[name] = {"iterations": len(log), "chosen_by_network": sum(r["learned"] for r in log),
                         "modes": [r["mode"] for r in log]}
    value = dist.world * steps * edges_step / t / 1e9
    return {"value": round(value, 4), "unit": "GTEPS", "ms_per_step": round(t * 1e3 / steps, 4),
            "ratio_vs_plain": round(value / plain_value, 4), "network": "wedge_gb300/data/sched_net.f32",
            "per_app": changed}


def _timed_records(W, g, app, p):
    q = W.Params(root=p.root, threshold_pct=p.threshold_pct, flags=W.FLAG_TIMING)
    g.run(app, q)
    return g.iteration_log()


def _ncu_traffic():
    """DRAM bytes of one step's pull launches (ncu, full-size workload, one pass), if the
    committed profile summary holds them"""
    path = os.path.join(ROOT, "profiles", "pull_kernel_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get("traffic_bytes_per_step")
    except Exception:
        return None


# ---------------------------------------------------------------- CPU legs (oracle)
def _cpu_graphs(scale, ef, threads):
    from oracle import oracle as O

    V, s, d = O.rmat(scale, ef, WORKLOAD["seed"], threads=threads)
    sb, db = O.sort_edges(V, s, d, threads=threads)
    ss, ds = O.sort_edges(V, *O.symmetrise(s, d), threads=threads)
    del s, d
    gb = O.Graph.from_edges(V, sb, db, O.BFS)
    E_b = len(sb)
    del sb, db
    gc = O.Graph.from_edges(V, ss, ds, O.CC)
    E_c = len(ss)
    return O, gb, gc, V, E_b, E_c


def cpu_baseline(scale, ef):
    """the oracle's restatement of the reference on this host's cores: one BFS + one CC"""
    from oracle import oracle as O

    O.build()
    threads = O.lib().orc_online_cores()
    O, gb, gc, V, E_b, E_c = _cpu_graphs(scale, ef, threads)
    _, _, sb = gb.run(root=WORKLOAD["bfs_root"], threshold_pct=WORKLOAD["threshold_pct"], threads=threads)
    _, _, sc = gc.run(threshold_pct=WORKLOAD["threshold_pct"], threads=threads)
    secs = (sb["running_ms"] + sc["running_ms"]) / 1e3
    return {"value": round((E_b + E_c) / secs / 1e9, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"one BFS (root 0) + one CC traversal of the same R-MAT scale-{scale} graphs; "
                      f"timed as the reference's Running Time (pull + Wedge phases, load excluded)",
            "bfs_ms": round(sb["running_ms"], 3), "cc_ms": round(sc["running_ms"], 3),
            "bfs_iterations": sb["iterations"], "cc_iterations": sc["iterations"]}


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    from oracle import oracle as O

    O.build()
    threads = O.lib().orc_online_cores()
    scale, ef = args.scale, args.edge_factor
    O, gb, gc, V, E_b, E_c = _cpu_graphs(scale, ef, threads)
    warmup = max(3, args.warmup)
    steps = args.steps
    # each step is one BFS + one CC traversal; the step count is capped so the run stays within minutes
    steps = min(steps, 10)
    warmup = min(warmup, 3)

    def step():
        _, _, sb = gb.run(root=WORKLOAD["bfs_root"], threshold_pct=WORKLOAD["threshold_pct"], threads=threads)
        _, _, sc = gc.run(threshold_pct=WORKLOAD["threshold_pct"], threads=threads)
        return (sb["running_ms"] + sc["running_ms"]) / 1e3

    for _ in range(warmup):
        step()
    t = sum(step() for _ in range(steps))
    value = steps * (E_b + E_c) / t / 1e9
    line = {
        "impl": "reference",
        "metric": "GTEPS per app at 1 GB300 (BFS + CC, plain fixed-threshold schedule)",
        "value": round(value, 4), "unit": "GTEPS", "n_gpus": args.gpus, "steps": steps, "warmup": warmup,
        "ms_per_step": round(t * 1e3 / steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (CPU R-MAT, same generator as the GPU arm)",
        "config": {"workload": workload_name(scale, ef), "scale": scale, "edge_factor": ef, "seed": WORKLOAD["seed"],
                   "vertices": V, "edges_bfs": E_b, "edges_cc": E_c, "threads": threads},
        "cpu_baseline": {"value": round(value, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": f"{steps} steps of one BFS + one CC on the full scale-{scale} graphs "
                                   f"(the AVX2 reference does not compile on this Arm host)"},
        "e2e": {"value": round(value, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist = Dist()
    if args.impl == "reference":
        if dist.world > 1:
            dist.init("gloo")
        run_reference(args, dist)
        dist.done()
        return
    run_ours(args, dist)


if __name__ == "__main__":
    main()

"""Benchmark of the edge-pull engine: GTEPS per application on R-MAT scale 26.

Workload (one "step", the configuration the metric is quoted on): on the R-MAT
graph of scale 26 (edge factor 16, a/b/c/d = 0.57/0.19/0.19/0.05, seed 5:
67,108,864 vertices, 1,073,741,824 edges), BFS from vertex 0, SSSP from vertex
0 (uint64 hash weights in [1, 255]) and 30 iterations of compensated-FP32
PageRank (damping 0.85) on the directed graph, and Connected Components on its
symmetrised copy (2,147,483,648 edges); plain fixed-threshold scheduling (t =
20%).  Synthetic graphs are generated on the device with the same
counter-based generator the CPU side uses.  GTEPS counts every input edge once
per traversal (BFS, CC, SSSP) and once per iteration (PageRank):
    value = steps * (|E| + |E_sym| + |E| + 30 |E|) / time.
The same steps under the learned scheduler, per application, and sub-records
for the other configurations (PageRank R-MAT 16 FP64; BFS + CC R-MAT 24; SSSP
on the 4096^2 grid, uint64 and FP64 weights; 256 BFS + 256 SSSP queries over
64 graphs in one persistent kernel) follow in the same JSON line.

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
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RMAT_ABC = (0.57, 0.19, 0.19)
WORKLOAD = dict(workload="rmat26_bfs_cc_sssp_pr", scale=26, edge_factor=16, seed=5, root=0, threshold_pct=20,
                pr_iterations=30, damping=0.85)
APPS = ("bfs", "cc", "sssp", "pr")


def workload_name(scale: int, ef: int) -> str:
    """the workload as run: the default is rmat26_bfs_cc_sssp_pr (R-MAT scale 26, edge factor 16)"""
    if (scale, ef) == (WORKLOAD["scale"], WORKLOAD["edge_factor"]):
        return WORKLOAD["workload"]
    return f"rmat{scale}_ef{ef}_bfs_cc_sssp_pr"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=WORKLOAD["scale"])
    ap.add_argument("--edge-factor", type=int, default=WORKLOAD["edge_factor"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sub", action="store_true", help="skip the other configurations' sub-records")
    ap.add_argument("--mode", default="graph", choices=["graph", "host"], help="traversal loop: CUDA graph or host")
    ap.add_argument("--profile-steps", action="store_true",
                    help="only the warm-up and timed plain steps, no JSON line (for profiler launch lists)")
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


# ---------------------------------------------------------------- algorithmic bytes per pull
def pull_bytes(app: str, rec: dict, V: int, wbytes: int = 1) -> float:
    """Compulsory bytes of one iteration's pull, each touched array counted once
    (E_s = in-edges read, V_s = destinations examined, act = vertices activated):
      BFS   4 E_s + 12 V_s + 3 V/8 + 4 act  (sources, offsets + ids, frontier / next / visited bits, parents)
      CC    4 E_s + 12 V_s + 4 V + 4 act + V/8  (labels read once, changed labels, changed bitmap)
      SSSP  (4 + w) E_s + 12 V_s + 8 V + 8 act + 2 V/8  (w = stored weight bytes per in-edge)"""
    Es, Vs, act = rec["edges_scanned"], rec["dsts_scanned"], rec["vertices_activated"]
    bitmap = V / 8.0
    if app == "bfs":
        return 4.0 * Es + 12.0 * Vs + 3 * bitmap + 4.0 * act
    if app == "cc":
        return 4.0 * Es + 12.0 * Vs + 4.0 * V + 4.0 * act + bitmap
    if app == "sssp":
        return (4.0 + wbytes) * Es + 12.0 * Vs + 8.0 * V + 8.0 * act + 2 * bitmap
    raise ValueError(app)


def pr_iteration_bytes(V: int, E: int) -> float:
    """compensated-FP32 PageRank, one iteration: 4 E (sources) + 20 V (destination
    offsets 8, rank read 4, 1/outdegree' 4, rank write 4)"""
    return 4.0 * E + 20.0 * V


# ---------------------------------------------------------------- our arm
class Suite:
    """the four applications on the scale-26 graphs, one handle per application"""

    def __init__(self, W, scale, ef, seed, mode):
        self.W = W
        flags = W.FLAG_GRAPH if mode == "graph" else 0
        self.g = {
            "bfs": W.Graph.rmat(scale, ef, seed),
            "cc": W.Graph.rmat(scale, ef, seed, symmetrise=True),
            "sssp": W.Graph.rmat(scale, ef, seed, weight_kind=W.WEIGHTS_U64),
            "pr": W.Graph.rmat(scale, ef, seed),
        }
        # launch knobs from the engine autotuner's table where it was tuned on graphs of this size
        from wedge_gb300 import autotune as A

        self.knobs = {a: A.apply_engine_tuning(self.g[a], a, scale, ef) for a in APPS}
        self.V = self.g["bfs"].V
        self.E = {a: self.g[a].E for a in APPS}
        self.app = {"bfs": W.APP_BFS, "cc": W.APP_CC, "sssp": W.APP_SSSP, "pr": W.APP_PR}
        t = WORKLOAD["threshold_pct"]
        self.params = {}
        for sched_name, sched in (("plain", W.SCHED_PLAIN), ("learned", W.SCHED_LEARNED)):
            self.params[sched_name] = {
                "bfs": W.Params(root=WORKLOAD["root"], threshold_pct=t, flags=flags, sched=sched),
                "cc": W.Params(threshold_pct=t, flags=flags, sched=sched),
                "sssp": W.Params(root=WORKLOAD["root"], threshold_pct=t, flags=flags, sched=sched),
                "pr": W.Params(num_iterations=WORKLOAD["pr_iterations"], damping=WORKLOAD["damping"],
                               precision=W.PREC_FP32C, flags=flags),
            }

    def edges(self, a):
        """edges one run of application a processes (PageRank: per iteration)"""
        return self.E[a] * (WORKLOAD["pr_iterations"] if a == "pr" else 1)

    def step_edges(self):
        return sum(self.edges(a) for a in APPS)

    def run(self, a, sched="plain"):
        return self.g[a].run(self.app[a], self.params[sched][a])

    def close(self):
        for g in self.g.values():
            g.close()


def _timed_steps(W, suite, sched, steps, warmup, dist):
    """device time of `steps` four-application steps (CUDA events on the first and
    last handles' streams; each run returns after its stream drained) and the
    per-application device times from the runs' own events"""
    import torch

    for _ in range(warmup):
        for a in APPS:
            suite.run(a, sched)
    torch.cuda.synchronize()
    streams = {a: torch.cuda.ExternalStream(suite.g[a].stream) for a in APPS}
    per_app = {a: 0.0 for a in APPS}
    info = {a: {} for a in APPS}
    launches = 0
    dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(streams[APPS[0]])
    t0 = time.perf_counter()
    for _ in range(steps):
        for a in APPS:
            st = suite.run(a, sched)
            per_app[a] += st["running_ms"]
            launches += st["kernel_launches"]
            info[a] = {"iterations": st["iterations"], "wedge_iterations": st["wedge_iterations"]}
    e1.record(streams[APPS[-1]])
    e1.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    dist.barrier()
    return e0.elapsed_time(e1), per_app, info, launches, wall


def _timed_records(W, suite, a):
    """the per-iteration records of one run with per-pull CUDA events (WEDGE_FLAG_TIMING)"""
    p = suite.params["plain"][a]
    q = W.Params(root=p.root, threshold_pct=p.threshold_pct, num_iterations=p.num_iterations, damping=p.damping,
                 precision=p.precision, flags=W.FLAG_TIMING)
    st = suite.g[a].run(suite.app[a], q)
    return st, suite.g[a].iteration_log()


def _roofline(W, suite, peak):
    """per application: algorithmic bytes of its pulls over their CUDA-event time"""
    out = {}
    V = suite.V
    for a in APPS:
        st, log = _timed_records(W, suite, a)
        if a == "pr":
            n = len(log)
            ms = sum(r["pull_ms"] for r in log)
            byts = pr_iteration_bytes(V, suite.E[a]) * n
            out[a] = {"kernel": "pr32_pull_kernel (the pull with the fused vertex phase), per iteration",
                      "iterations": n, "pull_ms": round(ms, 4), "vertex_ms": round(st["vertex_ms"], 4),
                      "algorithmic_bytes": int(byts)}
        else:
            ms = sum(r["pull_ms"] for r in log)
            byts = sum(pull_bytes(a, r, V) for r in log)
            out[a] = {"kernel": "dst_kernel + pull_kernel" if a in ("bfs", "cc") else "pull_kernel",
                      "iterations": len(log), "pull_ms": round(ms, 4), "algorithmic_bytes": int(byts),
                      "modes": [r["mode"] for r in log], "edges_scanned": int(sum(r["edges_scanned"] for r in log))}
        ach = byts / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        out[a].update({"achieved": round(ach, 1), "frac": round(ach / peak, 4)})
    return out


def _ncu_traffic(default_workload: bool):
    """DRAM bytes per launch of the PageRank pull at this workload, from the committed
    one-pass ncu capture of one launch (profiles/), or None elsewhere"""
    if not default_workload:
        return None
    try:
        with open(os.path.join(ROOT, "profiles", "pr32_pull_traffic.json")) as f:
            return json.load(f).get("traffic_bytes_per_launch_rmat26")
    except Exception:
        return None


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
    from wedge_gb300 import scheduler as S

    steps, warmup = args.steps, max(3, args.warmup)
    scale, ef = args.scale, args.edge_factor
    default_workload = (scale, ef) == (WORKLOAD["scale"], WORKLOAD["edge_factor"])
    suite = Suite(W, scale, ef, WORKLOAD["seed"], args.mode)
    V = suite.V
    try:
        blob = S.load()
        for a in ("bfs", "cc", "sssp"):
            suite.g[a].set_scheduler(blob)
    except Exception as e:  # no trained network: the learned arm reports it
        blob = None
        blob_err = str(e)

    if args.profile_steps:
        for _ in range(args.warmup + args.steps):
            for a in APPS:
                suite.run(a)
        torch.cuda.synchronize()
        suite.close()
        dist.done()
        return

    # ---- device-timed region: graphs resident in HBM
    sampler = ClockSampler(visible_index(dist.local))
    sampler.start()
    dev_ms, per_app_ms, info, launches, wall = _timed_steps(W, suite, "plain", steps, warmup, dist)
    clocks = sampler.stop()
    t_max = dist.max(dev_ms / 1e3)
    value = dist.world * steps * suite.step_edges() / t_max / 1e9
    per_app = {}
    for a in APPS:
        gteps = steps * suite.edges(a) / (per_app_ms[a] / 1e3) / 1e9 if per_app_ms[a] > 0 else None
        per_app[a] = {"gteps": round(gteps, 2), "ms_per_run": round(per_app_ms[a] / steps, 4),
                      "edges": suite.E[a], **info[a]}
    per_app["pr"].update({"precision": "fp32 compensated (two-sum), fp64 total rank",
                          "iterations": WORKLOAD["pr_iterations"], "damping": WORKLOAD["damping"]})

    # ---- the same steps under the learned scheduler (on-device network, plain-rule fallback)
    if blob is not None:
        l_ms, l_app_ms, l_info, _, _ = _timed_steps(W, suite, "learned", steps, warmup, dist)
        l_value = dist.world * steps * suite.step_edges() / dist.max(l_ms / 1e3) / 1e9
        learned = {"value": round(l_value, 4), "unit": "GTEPS", "ms_per_step": round(l_ms / steps, 4),
                   "ratio_vs_plain": round(l_value / value, 4), "network": "wedge_gb300/data/sched_net.f32",
                   "per_app": {}}
        for a in APPS:
            lg = steps * suite.edges(a) / (l_app_ms[a] / 1e3) / 1e9
            learned["per_app"][a] = {"gteps": round(lg, 2), "ratio_vs_plain": round(lg / per_app[a]["gteps"], 4),
                                     **l_info[a]}
        learned["per_app"]["pr"]["note"] = "no schedule choice: every PageRank iteration is a dense pull"
    else:
        learned = {"unavailable": f"no scheduler network: {blob_err}"}

    # ---- end to end through the C ABI with host buffers: query parameters in,
    # full property arrays (8 bytes per vertex, graph_vertex_props) out, every
    # step.  The four handles share one stream, so their traversals run one
    # after another as in the device-timed region; each export to page-locked
    # host memory runs on its handle's second stream, under the next traversal.
    host = {a: torch.empty(V, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64) for a in APPS}
    shared = torch.cuda.Stream()
    for a in APPS:
        suite.g[a].set_stream(shared.cuda_stream)
    e2e_steps = max(3, min(steps, 10))
    checks = {a: 0 for a in APPS}

    def consume(a):
        checks[a] ^= int(host[a][V // 2])  # the host touches every step's results

    def e2e_step(pipelined):
        for a in APPS:
            if pipelined:
                suite.g[a].wait_results()  # the previous step's results of a, while this step runs
                consume(a)
            suite.g[a].run_async(suite.app[a], suite.params["plain"][a])
            suite.g[a].read_results_async(host[a])
        if not pipelined:
            for a in APPS:
                suite.g[a].wait()
                consume(a)

    def e2e_run(pipelined):
        e2e_step(False)
        dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step(pipelined)
        if pipelined:
            for a in APPS:
                suite.g[a].wait()
                consume(a)
        return dist.max(time.perf_counter() - t0)

    e2e_wall = e2e_run(True)
    e2e_value = dist.world * e2e_steps * suite.step_edges() / e2e_wall / 1e9
    e2e_step_wait = dist.world * e2e_steps * suite.step_edges() / e2e_run(False) / 1e9
    # the same with the blocking calls (run, then read into the same page-locked memory)
    for a in APPS:
        suite.g[a].set_stream(None)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for a in APPS:
            suite.run(a)
            suite.g[a].read_results(host[a])
    e2e_sync = dist.world * e2e_steps * suite.step_edges() / dist.max(time.perf_counter() - t0) / 1e9
    params_bytes = len(APPS) * ctypes.sizeof(W.Params)  # each query's wedge_params_t, in kernel arguments

    # ---- roofline of the dominant kernel (the PageRank pull) and of every application's pulls
    peak, peak_kind = measured_peaks()
    roof = _roofline(W, suite, peak)
    pr_roof = roof["pr"]
    line = {
        "metric": "GTEPS per app at 1 GB300 (BFS + CC + SSSP + 30-iteration PageRank, plain fixed-threshold "
                  "schedule; learned-scheduled beside it)",
        "value": round(value, 4),
        "unit": "GTEPS",
        "n_gpus": dist.world,
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": round(t_max * 1e3 / steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32/u64 (BFS, CC, SSSP), fp32 compensated (PageRank)",
        "data": "synthetic (device R-MAT, counter-based generator; no dataset)",
        "config": {"workload": workload_name(scale, ef), "scale": scale, "edge_factor": ef, "seed": WORKLOAD["seed"],
                   "vertices": V, "edges": suite.E["bfs"], "edges_sym": suite.E["cc"], "root": WORKLOAD["root"],
                   "threshold_pct": WORKLOAD["threshold_pct"], "pr_iterations": WORKLOAD["pr_iterations"],
                   "damping": WORKLOAD["damping"], "loop": args.mode,
                   "knobs": {a: {k: suite.g[a].knob(k) for k in W.KNOB_NAMES} for a in APPS},
                   "knobs_from": "wedge_gb300/data/engine_tuning.json" if any(suite.knobs.values()) else "defaults",
                   "l2": f"inputs larger than L2 (in-edge sources {4 * suite.E['bfs'] / 2**30:.1f} GiB / "
                         f"{4 * suite.E['cc'] / 2**30:.1f} GiB vs 126 MB L2); no flush",
                   "parallelism": "replicas" if dist.world > 1 else "single GPU"},
        "per_app": per_app,
        "e2e": {"value": round(e2e_value, 4), "unit": "GTEPS", "h2d_bytes_per_step": params_bytes,
                "d2h_bytes_per_step": len(APPS) * 8 * V, "steps": e2e_steps,
                "what": "per application and step wedge_cuda_run_async + wedge_cuda_read_results_async into "
                        "page-locked host memory; the four handles share one stream (traversals in sequence, each "
                        "export under the next traversal); before queueing an application's next query the host "
                        "waits for its previous results (wedge_cuda_wait_results) and reads them, so the last "
                        "export of a step runs under the next step; every step's results reach the host inside "
                        "the timed region (the last step's by wedge_cuda_wait); graphs resident (loaded once, as "
                        "the reference excludes load from Running Time)",
                "per_step_wait": {"value": round(e2e_step_wait, 4),
                                  "what": "the same calls with wedge_cuda_wait on every handle at the end of each step"},
                "blocking_calls": {"value": round(e2e_sync, 4),
                                   "what": "wedge_cuda_run + wedge_cuda_read_results, one after another"}},
        "roofline": {"bound": "hbm", "kernel": pr_roof["kernel"], "achieved": pr_roof["achieved"], "peak": peak,
                     "unit": "GB/s", "frac": pr_roof["frac"], "peak_source": peak_kind,
                     "traffic": _ncu_traffic(default_workload),
                     "traffic_scope": "per launch (one PageRank iteration's pull): ncu DRAM read + write bytes of "
                                      "one launch at this workload (profiles/pr32_pull_traffic.json)",
                     "algorithmic_bytes_per_launch": int(pr_roof["algorithmic_bytes"] / max(1, pr_roof["iterations"])),
                     "launch_ms": round(pr_roof["pull_ms"] / max(1, pr_roof["iterations"]), 4),
                     "per_app": roof},
        "learned": learned,
        "clocks": clocks,
        "gpu_launches": int(launches),
        "wall_s_timed": round(wall, 4),
    }
    suite.close()
    if not args.no_sub and dist.world == 1:
        line["sub"] = sub_records(W, S, blob, args, peak)
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(scale, ef, pr32=host["pr"].view(np.float64))
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.done()


# ---------------------------------------------------------------- sub-records (other configurations)
def _event_ms(g, fn, reps):
    """median of the runs' own device times (Running Time, CUDA events)"""
    import numpy as np

    fn()
    ts = [fn()["running_ms"] for _ in range(reps)]
    return float(np.median(ts))


def sub_records(W, S, blob, args, peak):
    import numpy as np

    out = {}
    reps = 5
    # C2: BFS + CC on R-MAT scale 24 (seed 2), plain and learned
    gb = W.Graph.rmat(24, 16, 2)
    gc = W.Graph.rmat(24, 16, 2, symmetrise=True)
    rec = {"workload": "rmat24_bfs_cc", "vertices": gb.V, "edges_bfs": gb.E, "edges_cc": gc.E}
    for name, sched in (("plain", W.SCHED_PLAIN), ("learned", W.SCHED_LEARNED)):
        if sched == W.SCHED_LEARNED:
            if blob is None:
                continue
            gb.set_scheduler(blob)
            gc.set_scheduler(blob)
        tb = _event_ms(gb, lambda: gb.run(W.APP_BFS, W.Params(root=0, sched=sched, flags=W.FLAG_GRAPH)), reps)
        tc = _event_ms(gc, lambda: gc.run(W.APP_CC, W.Params(sched=sched, flags=W.FLAG_GRAPH)), reps)
        rec[name] = {"gteps": round((gb.E + gc.E) / ((tb + tc) / 1e3) / 1e9, 2), "bfs_ms": round(tb, 4),
                     "cc_ms": round(tc, 4)}
    if "learned" in rec:
        rec["learned"]["ratio_vs_plain"] = round(rec["learned"]["gteps"] / rec["plain"]["gteps"], 4)
    gb.close()
    gc.close()
    out["C2"] = rec
    # C1: PageRank FP64, R-MAT scale 16 (seed 1), 16 iterations, damping 0.85
    g = W.Graph.rmat(16, 16, 1)
    t = _event_ms(g, lambda: g.run(W.APP_PR, W.Params(num_iterations=16, damping=0.85, flags=W.FLAG_GRAPH)), reps)
    out["C1"] = {"workload": "rmat16_pr_fp64", "vertices": g.V, "edges": g.E, "iterations": 16, "ms": round(t, 4),
                 "gteps": round(16 * g.E / (t / 1e3) / 1e9, 2),
                 "note": "the 4 MB graph stays in L2; launch-bound"}
    g.close()
    # C3: SSSP from vertex 0 on the 4096^2 grid with 1% long-range edges (seed 3), uint64 and FP64 weights
    for kind, wk in (("u64", W.WEIGHTS_U64), ("f64", W.WEIGHTS_F64)):
        g = W.Graph.grid(4096, 0.01, 3, wk)
        t = _event_ms(g, lambda: g.run(W.APP_SSSP, W.Params(root=0, flags=W.FLAG_GRAPH)), 3)
        st = g.run(W.APP_SSSP, W.Params(root=0, flags=W.FLAG_TIMING))
        log = g.iteration_log()
        ms = sum(r["pull_ms"] for r in log)
        byts = sum(pull_bytes("sssp", r, g.V, 1 if kind == "u64" else 8) for r in log)
        out[f"C3_{kind}"] = {"workload": f"grid4096_sssp_{kind}", "vertices": g.V, "edges": g.E, "ms": round(t, 4),
                             "gteps": round(g.E / (t / 1e3) / 1e9, 2), "iterations": st["iterations"],
                             "wedge_iterations": st["wedge_iterations"],
                             "roofline": {"pull_ms": round(ms, 4), "algorithmic_bytes": int(byts),
                                          "frac": round(byts / (ms / 1e3) / 1e9 / peak, 4) if ms > 0 else None}}
        g.close()
    # C4: 256 BFS + 256 SSSP over 64 graphs in one persistent kernel, against one query at a time
    out["C4"] = _batch_record(W)
    return out


def _batch_record(W):
    import json as _json

    import numpy as np
    from wedge_gb300 import batch as B

    params = B.graph_params()
    queries = B.queries(params)
    graphs = B.load_graphs(params)
    tuning = None
    try:
        with open(os.path.join(ROOT, "wedge_gb300", "data", "batch_tuning.json")) as f:
            best = _json.load(f)["best"]
        tuning = W.BatchTuning(best["threshold_pct"], best["grab"], best["blocks_per_sm"], best["split"])
    except Exception:
        pass
    with W.Batch(graphs, queries) as b:
        b.run(tuning, W.FLAG_GRAPH)
        ts = [b.run(tuning, W.FLAG_GRAPH)["running_ms"] for _ in range(3)]
        t0 = time.perf_counter()
        b.run(tuning, W.FLAG_GRAPH)
        bwall = (time.perf_counter() - t0) * 1e3
    # one query at a time through wedge_cuda_run's graph loop (BFS queries of a graph, then its SSSP queries)
    seq_dev = 0.0
    t0 = time.perf_counter()
    for gi, g in enumerate(graphs):
        for app in (W.APP_BFS, W.APP_SSSP):
            for (qg, qa, root) in queries:
                if qg == gi and qa == app:
                    seq_dev += g.run(app, W.Params(root=root, flags=W.FLAG_GRAPH))["running_ms"]
    seq_wall = (time.perf_counter() - t0) * 1e3
    edges = sum(g.E for g in graphs)
    qedges = sum(graphs[qg].E for (qg, _a, _r) in queries)
    for g in graphs:
        g.close()
    dev = float(np.median(ts))
    return {"workload": "batch64_bfs256_sssp256", "graphs": len(graphs), "queries": len(queries),
            "edges_resident": edges, "batch_ms": round(dev, 3), "batch_wall_ms": round(bwall, 3),
            "sequential_ms": round(seq_dev, 3), "sequential_wall_ms": round(seq_wall, 3),
            "speedup_device": round(seq_dev / dev, 3), "speedup_wall": round(seq_wall / bwall, 3),
            "gteps": round(qedges / (dev / 1e3) / 1e9, 2)}


# ---------------------------------------------------------------- CPU legs (oracle)
def _cpu_suite(scale, ef, threads):
    """the oracle's graphs for the four applications (the same generator as the device's)"""
    from oracle import oracle as O

    V, s, d = O.rmat(scale, ef, WORKLOAD["seed"], threads=threads)
    sd, dd = O.sort_edges(V, s, d, threads=threads)
    ss, ds = O.sort_edges(V, *O.symmetrise(s, d), threads=threads)
    del s, d
    w = O.weights(sd, dd)
    g = {"bfs": O.Graph.from_edges(V, sd, dd, O.BFS, threads=threads),
         "sssp": O.Graph.from_edges(V, sd, dd, O.SSSP, w, threads=threads),
         "pr": O.Graph.from_edges(V, sd, dd, O.PR, threads=threads)}
    E = {"bfs": len(sd), "sssp": len(sd), "pr": len(sd)}
    del sd, dd, w
    g["cc"] = O.Graph.from_edges(V, ss, ds, O.CC, threads=threads)
    E["cc"] = len(ss)
    return O, g, V, E


def _cpu_run(g, a, threads, pr_iterations):
    if a == "bfs":
        return g.run(root=WORKLOAD["root"], threshold_pct=WORKLOAD["threshold_pct"], threads=threads)
    if a == "cc":
        return g.run(threshold_pct=WORKLOAD["threshold_pct"], threads=threads)
    if a == "sssp":
        return g.run(root=WORKLOAD["root"], threshold_pct=WORKLOAD["threshold_pct"], threads=threads)
    return g.run(iterations=pr_iterations, damping=WORKLOAD["damping"], threads=threads)


def cpu_baseline(scale, ef, pr32=None):
    """the oracle's restatement of the reference on this host's cores: one run of
    each application on the same graphs (PageRank all 30 iterations); the FP64
    PageRank ranks also give the error of the GPU's compensated-FP32 ranks"""
    import numpy as np
    from oracle import oracle as O

    O.build()
    threads = O.lib().orc_online_cores()
    O, g, V, E = _cpu_suite(scale, ef, threads)
    ms = {}
    pr_err = None
    for a in APPS:
        props, _, st = _cpu_run(g[a], a, threads, WORKLOAD["pr_iterations"])
        ms[a] = st["running_ms"]
        if a == "pr" and pr32 is not None and len(pr32) == V:
            ref = props.view(np.float64)
            pr_err = {"rel_l1": float(np.abs(pr32 - ref).sum() / np.abs(ref).sum()),
                      "max_rel": float(np.max(np.abs(pr32 - ref) / np.abs(ref))),
                      "what": "GPU compensated-FP32 ranks (the e2e arm's last read) against the oracle's FP64 ranks"}
        g[a].close()
    edges = sum(E[a] * (WORKLOAD["pr_iterations"] if a == "pr" else 1) for a in APPS)
    secs = sum(ms.values()) / 1e3
    return {"value": round(edges / secs / 1e9, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"one run of each application on the same R-MAT scale-{scale} graphs (PageRank 30 iterations, "
                      f"FP64); timed as the reference's Running Time (pull, vertex and Wedge phases, load excluded)",
            "ms": {a: round(ms[a], 3) for a in APPS},
            "per_app_gteps": {a: round(E[a] * (WORKLOAD["pr_iterations"] if a == "pr" else 1) / (ms[a] / 1e3) / 1e9, 4)
                              for a in APPS},
            "pr_error_vs_fp64_oracle": pr_err}


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    from oracle import oracle as O

    O.build()
    threads = O.lib().orc_online_cores()
    scale, ef = args.scale, args.edge_factor
    O, g, V, E = _cpu_suite(scale, ef, threads)
    warmup = max(3, args.warmup)
    steps = args.steps
    # Each step is one BFS, CC and SSSP traversal and a bounded sample of the
    # PageRank run: PR_SAMPLE of its 30 iterations, whose time is scaled to 30
    # (every iteration is the same dense pull and vertex phase).
    pr_sample = 2
    scale_pr = WORKLOAD["pr_iterations"] / pr_sample

    def step():
        t = {}
        for a in APPS:
            _, _, st = _cpu_run(g[a], a, threads, pr_sample)
            t[a] = st["running_ms"] / 1e3 * (scale_pr if a == "pr" else 1.0)
        return t

    for _ in range(warmup):
        step()
    tot = {a: 0.0 for a in APPS}
    for _ in range(steps):
        for a, x in step().items():
            tot[a] += x
    t = sum(tot.values())
    edges = sum(E[a] * (WORKLOAD["pr_iterations"] if a == "pr" else 1) for a in APPS)
    value = steps * edges / t / 1e9
    line = {
        "impl": "reference",
        "metric": "GTEPS per app at 1 GB300 (BFS + CC + SSSP + 30-iteration PageRank, plain fixed-threshold "
                  "schedule; learned-scheduled beside it)",
        "value": round(value, 4), "unit": "GTEPS", "n_gpus": args.gpus, "steps": steps, "warmup": warmup,
        "ms_per_step": round(t * 1e3 / steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 (BFS, SSSP), fp64 (CC labels, PageRank)",
        "data": "synthetic (CPU R-MAT, same generator as the GPU arm)",
        "config": {"workload": workload_name(scale, ef), "scale": scale, "edge_factor": ef, "seed": WORKLOAD["seed"],
                   "vertices": V, "edges": E["bfs"], "edges_sym": E["cc"], "root": WORKLOAD["root"],
                   "threshold_pct": WORKLOAD["threshold_pct"], "pr_iterations": WORKLOAD["pr_iterations"],
                   "damping": WORKLOAD["damping"], "threads": threads},
        "per_app": {a: {"gteps": round(steps * E[a] * (WORKLOAD["pr_iterations"] if a == "pr" else 1) / tot[a] / 1e9, 4),
                        "ms_per_run": round(tot[a] * 1e3 / steps, 3)} for a in APPS},
        "cpu_baseline": {"value": round(value, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": f"{steps} steps of one BFS, CC and SSSP traversal and {pr_sample} PageRank "
                                   f"iterations (time scaled to 30) on the full scale-{scale} graphs (the AVX2 "
                                   f"reference does not compile on this Arm host)"},
        "e2e": {"value": round(value, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    for x in g.values():
        x.close()
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

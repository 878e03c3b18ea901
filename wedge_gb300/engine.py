"""ctypes binding of ``libwedge_cuda.so`` (the C ABI declared in include/wedge_cuda.h).

The Python side mirrors the reference's host flow for the edge-pull path
(source/main.c:33-110):

    app = application_select("bfs")                      # application.c:197-205
    g = Graph.load("graph.bin", app)                     # graphdata.c:946 + :648
    stats = g.run(app, Params(root=0))                   # execution_impl_* (execution.h:107-129)
    props = g.read_results()                             # graph_vertex_props

There is no CPU fallback: if the library cannot be loaded, importing this
module raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libwedge_cuda.so")

APP_BFS, APP_CC, APP_PR, APP_SSSP = 0, 1, 2, 3
WEIGHTS_NONE, WEIGHTS_U64, WEIGHTS_F64 = 0, 1, 2
PREC_FP64, PREC_FP32C = 0, 1
SCHED_PLAIN, SCHED_DENSE, SCHED_WEDGE, SCHED_FILTERED, SCHED_LEARNED, SCHED_PROBE = 0, 1, 2, 3, 4, 5
MODE_DENSE, MODE_WEDGE, MODE_FILTERED = 0, 1, 2
SCHED_FEATURES, SCHED_HIDDEN, SCHED_OUTPUTS = 16, 64, 3
SCHED_PARAM_OFFSET = 64
SCHED_PARAMS = 64 * 16 + 64 + 64 * 64 + 64 + 3 * 64 + 3
SCHED_BLOB = SCHED_PARAM_OFFSET + SCHED_PARAMS + 1
PHASE_INIT, PHASE_PULL_DENSE, PHASE_PULL_WEDGE, PHASE_VERTEX_PR, PHASE_WEDGE_BUILD, PHASE_ADVANCE = range(6)
FLAG_GRAPH, FLAG_TIMING = 1, 2
SHARD_PROPS, SHARD_FRONTIER = 0, 1
# launch knobs (enum wedge_knob); KNOB_DEFAULT: the environment variable, else the built-in default
KNOB_HUB_BYTES, KNOB_PROBE_EDGES, KNOB_SSSP_TILE, KNOB_SSSP_NARROW = 0, 1, 2, 3
KNOB_NAMES = {"hub_bytes": KNOB_HUB_BYTES, "probe_edges": KNOB_PROBE_EDGES, "sssp_tile": KNOB_SSSP_TILE,
              "sssp_narrow": KNOB_SSSP_NARROW}
KNOB_DEFAULT = (1 << 64) - 1

OK = 0
ERR_IO, ERR_FORMAT, ERR_OOM, ERR_CUDA, ERR_NOT_CONVERGED, ERR_ARG, ERR_UNSUPPORTED = -1, -2, -3, -4, -5, -6, -7

# names accepted by application_select (source/application.c:49-59)
_APP_NAMES = {
    APP_BFS: ("bfs", "breadth_first_search", "breadthfirstsearch"),
    APP_CC: ("cc", "connected_components", "connectedcomponents"),
    APP_PR: ("pr", "pagerank"),
    APP_SSSP: ("sssp", "single_source_shortest_path", "singlesourceshortestpath"),
}
APP_CANONICAL = {APP_BFS: "Breadth-First Search", APP_CC: "Connected Components", APP_PR: "PageRank",
                 APP_SSSP: "Single-Source Shortest Path"}


def application_select(name: str) -> int:
    """Application id for a name, as application_select (application.c:197-205); raises ValueError."""
    n = name.lower()
    for app, names in _APP_NAMES.items():
        if n in names:
            return app
    raise ValueError(f'Application: ERROR: unable to run "{name}"')


class Params(C.Structure):
    _fields_ = [("root", C.c_uint64), ("threshold_pct", C.c_uint32), ("num_iterations", C.c_uint32),
                ("damping", C.c_double), ("precision", C.c_int32), ("sched", C.c_int32),
                ("max_iterations", C.c_uint32), ("flags", C.c_uint32), ("probe_iter", C.c_uint32),
                ("probe_mode", C.c_int32)]

    def __init__(self, root=0, threshold_pct=20, num_iterations=1, damping=0.0, precision=PREC_FP64,
                 sched=SCHED_PLAIN, max_iterations=0, flags=0, probe_iter=0xFFFFFFFF, probe_mode=MODE_DENSE):
        super().__init__(root, threshold_pct, num_iterations, damping, precision, sched, max_iterations, flags,
                         probe_iter, probe_mode)


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_uint64), ("wedge_iterations", C.c_uint64), ("running_ms", C.c_double),
                ("pull_ms_dense", C.c_double), ("pull_ms_wedge", C.c_double), ("wedge_ms", C.c_double),
                ("vertex_ms", C.c_double), ("edges_scanned", C.c_uint64), ("tiles_scanned", C.c_uint64),
                ("dsts_scanned", C.c_uint64), ("vertices_activated", C.c_uint64),
                ("pull_launches", C.c_uint64), ("kernel_launches", C.c_uint64), ("pr_sum", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class IterationRecord(C.Structure):
    _fields_ = [("active_edges", C.c_uint64), ("used_wedge", C.c_uint32), ("iteration", C.c_uint32),
                ("pull_ms", C.c_double), ("wedge_ms", C.c_double), ("changed_mass", C.c_uint64),
                ("edges_scanned", C.c_uint64), ("tiles_scanned", C.c_uint64), ("dsts_scanned", C.c_uint64),
                ("vertices_activated", C.c_uint64), ("mode", C.c_uint32), ("learned", C.c_uint32),
                ("features", C.c_float * SCHED_FEATURES)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["features"] = list(self.features)
        return d


class Query(C.Structure):
    _fields_ = [("graph", C.c_uint32), ("app", C.c_int32), ("root", C.c_uint64)]


class BatchTuning(C.Structure):
    _fields_ = [("threshold_pct", C.c_uint32), ("grab", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("split", C.c_uint32)]


class BatchStats(C.Structure):
    _fields_ = [("running_ms", C.c_double), ("rounds", C.c_uint64), ("chunks_pulled", C.c_uint64),
                ("iterations", C.c_uint64), ("captured", C.c_uint32), ("blocks", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class WedgeError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {status_string(status)} ({status})")
        self.status = status


_lib = None

# every symbol include/wedge_cuda.h declares, with its ctypes signature
_SIGNATURES = {
    "wedge_cuda_load_graph": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    "wedge_cuda_load_graph_ex": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "wedge_cuda_load_graph_image": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "wedge_cuda_load_edges": (C.c_int, [C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                        C.POINTER(C.c_void_p)]),
    "wedge_cuda_load_edge_vectors": (C.c_int, [C.c_uint64, C.c_void_p, C.c_uint64, C.c_int, C.c_int,
                                               C.POINTER(C.c_void_p)]),
    "wedge_cuda_generate_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                           C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "wedge_cuda_generate_grid": (C.c_int, [C.c_uint32, C.c_double, C.c_uint64, C.c_int, C.POINTER(C.c_void_p)]),
    "wedge_cuda_run": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Params), C.POINTER(Stats)]),
    "wedge_cuda_run_phase": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(Params), C.POINTER(C.c_uint64)]),
    "wedge_cuda_read_results": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "wedge_cuda_run_async": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Params)]),
    "wedge_cuda_read_results_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "wedge_cuda_wait": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "wedge_cuda_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wedge_cuda_wait_results": (C.c_int, [C.c_void_p]),
    "wedge_cuda_set_knob": (C.c_int, [C.c_void_p, C.c_int, C.c_uint64]),
    "wedge_cuda_get_knob": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint64)]),
    "wedge_cuda_load_shard": (C.c_int, [C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                        C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "wedge_cuda_shard_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_uint64, C.c_int]),
    "wedge_cuda_shard_decide": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64]),
    "wedge_cuda_iteration_log": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "wedge_cuda_read_outdegrees": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "wedge_cuda_set_scheduler": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "wedge_cuda_write_output": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "wedge_cuda_rmat_edge_list": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                            C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_void_p,
                                            C.c_void_p, C.c_uint64]),
    "wedge_cuda_grid_edge_list": (C.c_int, [C.c_uint32, C.c_double, C.c_uint64, C.POINTER(C.c_uint64),
                                            C.POINTER(C.c_uint64), C.c_void_p, C.c_void_p, C.c_uint64]),
    "wedge_cuda_batch_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p)]),
    "wedge_cuda_batch_run": (C.c_int, [C.c_void_p, C.POINTER(BatchTuning), C.c_uint32, C.POINTER(BatchStats)]),
    "wedge_cuda_batch_read_result": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64]),
    "wedge_cuda_batch_iterations": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "wedge_cuda_batch_free": (None, [C.c_void_p]),
    "wedge_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "wedge_mlp_loss_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                      C.POINTER(C.c_double), C.c_void_p]),
    "wedge_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32,
                                  C.c_uint32, C.c_float, C.c_uint64, C.POINTER(C.c_double)]),
    "wedge_cuda_pr_iteration_noalloc": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                                  C.c_void_p]),
    "wedge_cuda_num_vertices": (C.c_uint64, [C.c_void_p]),
    "wedge_cuda_num_edges": (C.c_uint64, [C.c_void_p]),
    "wedge_cuda_stream": (C.c_void_p, [C.c_void_p]),
    "wedge_cuda_free": (None, [C.c_void_p]),
    "wedge_cuda_status_string": (C.c_char_p, [C.c_int]),
    "wedge_cuda_abi_version": (C.c_int, []),
}


def lib():
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def status_string(status: int) -> str:
    return lib().wedge_cuda_status_string(status).decode()


def _check(rc: int, what: str):
    if rc != OK:
        raise WedgeError(rc, what)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Graph:
    """A graph resident on the GPU (the handle of wedge_cuda.h)."""

    def __init__(self, handle: C.c_void_p, weight_kind: int = WEIGHTS_NONE):
        self._h = handle
        self.weight_kind = weight_kind
        self.last_app = None

    # ---------------------------------------------------------------- loading
    @classmethod
    def load(cls, path: str, app: int, weight_kind: int = WEIGHTS_U64) -> "Graph":
        h = C.c_void_p()
        _check(lib().wedge_cuda_load_graph_ex(path.encode(), app, weight_kind, C.byref(h)), "wedge_cuda_load_graph_ex")
        return cls(h, weight_kind if app == APP_SSSP else WEIGHTS_NONE)

    @classmethod
    def load_image(cls, image: bytes | np.ndarray, app: int, weight_kind: int = WEIGHTS_U64) -> "Graph":
        buf = np.frombuffer(image, np.uint8) if isinstance(image, (bytes, bytearray)) else np.ascontiguousarray(image)
        h = C.c_void_p()
        _check(lib().wedge_cuda_load_graph_image(_ptr(buf), buf.nbytes, app, weight_kind, C.byref(h)),
               "wedge_cuda_load_graph_image")
        return cls(h, weight_kind if app == APP_SSSP else WEIGHTS_NONE)

    @classmethod
    def from_edges(cls, V: int, src, dst, weights=None, weight_kind: int = WEIGHTS_U64) -> "Graph":
        s = np.ascontiguousarray(src, np.uint32)
        d = np.ascontiguousarray(dst, np.uint32)
        w = None if weights is None else np.ascontiguousarray(weights, np.uint64)
        h = C.c_void_p()
        _check(lib().wedge_cuda_load_edges(V, len(s), _ptr(s), _ptr(d), None if w is None else _ptr(w),
                                           weight_kind if w is not None else WEIGHTS_NONE, C.byref(h)),
               "wedge_cuda_load_edges")
        return cls(h, weight_kind if w is not None else WEIGHTS_NONE)

    @classmethod
    def shard(cls, V: int, src, dst, global_outdeg, global_edges: int, weights=None,
              weight_kind: int = WEIGHTS_U64) -> "Graph":
        """one destination-range shard: the in-edges of its destinations, the whole graph's out-degrees"""
        s = np.ascontiguousarray(src, np.uint32)
        d = np.ascontiguousarray(dst, np.uint32)
        od = np.ascontiguousarray(global_outdeg, np.uint64)
        w = None if weights is None else np.ascontiguousarray(weights, np.uint64)
        h = C.c_void_p()
        _check(lib().wedge_cuda_load_shard(V, len(s), _ptr(s), _ptr(d), None if w is None else _ptr(w),
                                           weight_kind if w is not None else WEIGHTS_NONE, _ptr(od), global_edges,
                                           C.byref(h)), "wedge_cuda_load_shard")
        return cls(h, weight_kind if w is not None else WEIGHTS_NONE)

    @classmethod
    def from_edge_vectors(cls, V: int, vectors: np.ndarray, weighted: bool, weight_kind: int = WEIGHTS_U64) -> "Graph":
        v = np.ascontiguousarray(vectors, np.uint64)
        words = 8 if weighted else 4
        h = C.c_void_p()
        _check(lib().wedge_cuda_load_edge_vectors(V, _ptr(v), v.size // words, int(weighted), weight_kind, C.byref(h)),
               "wedge_cuda_load_edge_vectors")
        return cls(h, weight_kind if weighted else WEIGHTS_NONE)

    @classmethod
    def rmat(cls, scale: int, edge_factor: int, seed: int, symmetrise: bool = False, weight_kind: int = WEIGHTS_NONE,
             abc=(0.57, 0.19, 0.19)) -> "Graph":
        h = C.c_void_p()
        _check(lib().wedge_cuda_generate_rmat(scale, edge_factor, abc[0], abc[1], abc[2], seed, int(symmetrise),
                                              weight_kind, C.byref(h)), "wedge_cuda_generate_rmat")
        return cls(h, weight_kind)

    @classmethod
    def grid(cls, side: int, long_range_frac: float, seed: int, weight_kind: int = WEIGHTS_U64) -> "Graph":
        h = C.c_void_p()
        _check(lib().wedge_cuda_generate_grid(side, long_range_frac, seed, weight_kind, C.byref(h)),
               "wedge_cuda_generate_grid")
        return cls(h, weight_kind)

    # ---------------------------------------------------------------- running
    @property
    def V(self) -> int:
        return lib().wedge_cuda_num_vertices(self._h)

    @property
    def E(self) -> int:
        return lib().wedge_cuda_num_edges(self._h)

    @property
    def stream(self) -> int:
        return lib().wedge_cuda_stream(self._h) or 0

    def run(self, app: int, params: Params | None = None, allow_not_converged: bool = False) -> dict:
        p = params or Params()
        st = Stats()
        rc = lib().wedge_cuda_run(self._h, app, C.byref(p), C.byref(st))
        if not (rc == OK or (allow_not_converged and rc == ERR_NOT_CONVERGED)):
            raise WedgeError(rc, "wedge_cuda_run")
        self.last_app = app
        d = st.as_dict()
        d["status"] = rc
        return d

    def run_async(self, app: int, params: Params | None = None):
        """queue the whole traversal (device-side loop) without waiting; see wait()"""
        self._async_params = params or Params()  # kept alive until the call returns
        _check(lib().wedge_cuda_run_async(self._h, app, C.byref(self._async_params)), "wedge_cuda_run_async")
        self.last_app = app

    def read_results_async(self, out: np.ndarray):
        """queue the export of the last run's results into page-locked host memory (out)"""
        _check(lib().wedge_cuda_read_results_async(self._h, _ptr(out), out.nbytes), "wedge_cuda_read_results_async")

    def wait(self, allow_not_converged: bool = False) -> dict:
        """wait for the queued run and reads; the queued run's statistics"""
        st = Stats()
        rc = lib().wedge_cuda_wait(self._h, C.byref(st))
        if not (rc == OK or (allow_not_converged and rc == ERR_NOT_CONVERGED)):
            raise WedgeError(rc, "wedge_cuda_wait")
        d = st.as_dict()
        d["status"] = rc
        return d

    def wait_results(self):
        """wait only for the last asynchronous read (work queued after it keeps running)"""
        _check(lib().wedge_cuda_wait_results(self._h), "wedge_cuda_wait_results")

    def set_stream(self, stream: int | None):
        """queue this handle's work on a caller's CUDA stream (its handle as an int; None: its own)"""
        _check(lib().wedge_cuda_set_stream(self._h, C.c_void_p(stream) if stream else None), "wedge_cuda_set_stream")

    def set_knob(self, knob: int | str, value: int | None):
        """set a launch knob (KNOB_* or its name in KNOB_NAMES); None: back to the default.
        The handle's traversal state is released and rebuilt by the next run."""
        k = KNOB_NAMES[knob] if isinstance(knob, str) else knob
        _check(lib().wedge_cuda_set_knob(self._h, k, KNOB_DEFAULT if value is None else int(value)),
               "wedge_cuda_set_knob")

    def knob(self, knob: int | str) -> int:
        """the value of a launch knob the next state build uses"""
        k = KNOB_NAMES[knob] if isinstance(knob, str) else knob
        v = C.c_uint64()
        _check(lib().wedge_cuda_get_knob(self._h, k, C.byref(v)), "wedge_cuda_get_knob")
        return int(v.value)

    def shard_state(self, which: int, out: np.ndarray, import_: bool = False):
        """a shard's properties or pulled frontier, to (import_ False) or from host memory"""
        _check(lib().wedge_cuda_shard_state(self._h, which, _ptr(out), out.nbytes, int(import_)),
               "wedge_cuda_shard_state")
        return out

    def shard_decide(self, global_mass: int, threshold_pct: int = 20):
        _check(lib().wedge_cuda_shard_decide(self._h, global_mass, threshold_pct), "wedge_cuda_shard_decide")

    def run_phase(self, app: int, phase: int, params: Params | None = None) -> int:
        p = params or Params()
        mass = C.c_uint64()
        _check(lib().wedge_cuda_run_phase(self._h, app, phase, C.byref(p), C.byref(mass)), "wedge_cuda_run_phase")
        self.last_app = app
        return mass.value

    def read_results(self, out: np.ndarray | None = None) -> np.ndarray:
        V = self.V
        if out is None:
            out = np.empty(V, np.uint64)
        _check(lib().wedge_cuda_read_results(self._h, _ptr(out), out.nbytes), "wedge_cuda_read_results")
        return out

    def iteration_log(self) -> list[dict]:
        """per-iteration records of the last run (the reference's ITERATION_STATS rows)"""
        n = C.c_uint64()
        _check(lib().wedge_cuda_iteration_log(self._h, None, 0, C.byref(n)), "wedge_cuda_iteration_log")
        recs = (IterationRecord * max(1, n.value))()
        _check(lib().wedge_cuda_iteration_log(self._h, C.cast(recs, C.c_void_p), n.value, C.byref(n)),
               "wedge_cuda_iteration_log")
        return [recs[i].as_dict() for i in range(n.value)]

    def set_scheduler(self, blob: np.ndarray):
        """load a scheduler network (SCHED_BLOB float32) for SCHED_LEARNED runs"""
        b = np.ascontiguousarray(blob, np.float32)
        _check(lib().wedge_cuda_set_scheduler(self._h, _ptr(b), b.size), "wedge_cuda_set_scheduler")

    def write_output(self, path: str):
        """the -o file of the last run; returns (formatted on the GPU, formatting ms)"""
        on_gpu, ms = C.c_int(), C.c_double()
        _check(lib().wedge_cuda_write_output(self._h, path.encode(), C.byref(on_gpu), C.byref(ms)),
               "wedge_cuda_write_output")
        return bool(on_gpu.value), ms.value

    def read_outdegrees(self) -> np.ndarray:
        out = np.empty(self.V, np.uint64)
        _check(lib().wedge_cuda_read_outdegrees(self._h, _ptr(out), out.nbytes), "wedge_cuda_read_outdegrees")
        return out

    def close(self):
        if self._h:
            lib().wedge_cuda_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prop_string(app: int, prop: int, outdeg: int, num_vertices: int, sssp_f64: bool = False) -> str:
    """One -o output value, formatted as execution_get_vertex_prop_string_* does."""
    if app == APP_BFS:  # execution_bfs.c:69-73
        return "%d" % np.int64(np.uint64(prop).view(np.int64))
    d = float(np.uint64(prop).view(np.float64))
    if app == APP_CC:  # execution_cc.c:47-51
        return "%.0f" % d
    if app == APP_PR:  # execution_pr.c:31-35
        return "%.4e" % (d * (num_vertices if outdeg == 0 else outdeg))
    if sssp_f64:
        return "%.17g" % d
    return "%d" % np.int64(np.uint64(prop).view(np.int64))  # execution_sssp.c:48-52


# ---------------------------------------------------------------- scheduler network (CUDA kernels)
def _f32(a, shape):
    a = np.ascontiguousarray(a, np.float32)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


def mlp_forward(blob: np.ndarray, X: np.ndarray) -> np.ndarray:
    """network outputs [n][3] for features X [n][16], computed by the engine's CUDA kernel"""
    b = _f32(blob, (SCHED_BLOB,))
    X = _f32(X, (len(X), SCHED_FEATURES))
    out = np.empty((len(X), SCHED_OUTPUTS), np.float32)
    _check(lib().wedge_mlp_forward(_ptr(b), _ptr(X), len(X), _ptr(out)), "wedge_mlp_forward")
    return out


def mlp_loss_grad(blob: np.ndarray, X: np.ndarray, Y: np.ndarray, M: np.ndarray):
    """(loss, gradient over the trainable parameters) from the engine's CUDA kernels"""
    n = len(X)
    b = _f32(blob, (SCHED_BLOB,))
    X, Y, M = _f32(X, (n, SCHED_FEATURES)), _f32(Y, (n, SCHED_OUTPUTS)), _f32(M, (n, SCHED_OUTPUTS))
    g = np.empty(SCHED_PARAMS, np.float32)
    loss = C.c_double()
    _check(lib().wedge_mlp_loss_grad(_ptr(b), _ptr(X), _ptr(Y), _ptr(M), n, C.byref(loss), _ptr(g)),
           "wedge_mlp_loss_grad")
    return loss.value, g


def mlp_train(blob: np.ndarray, X: np.ndarray, Y: np.ndarray, M: np.ndarray, epochs: int, batch: int = 256,
              lr: float = 1e-3, seed: int = 1):
    """Adam training on the GPU; returns (trained blob, final loss)"""
    n = len(X)
    b = np.array(_f32(blob, (SCHED_BLOB,)))
    X, Y, M = _f32(X, (n, SCHED_FEATURES)), _f32(Y, (n, SCHED_OUTPUTS)), _f32(M, (n, SCHED_OUTPUTS))
    loss = C.c_double()
    _check(lib().wedge_mlp_train(_ptr(b), _ptr(X), _ptr(Y), _ptr(M), n, epochs, batch, C.c_float(lr), seed,
                                 C.byref(loss)), "wedge_mlp_train")
    return b, loss.value


# ---------------------------------------------------------------- batched queries
class Batch:
    """Many BFS / SSSP queries over many resident graphs, run together in one
    persistent kernel (wedge_cuda_batch_*).  queries: (graph index, app, root)."""

    def __init__(self, graphs, queries):
        self._graphs = list(graphs)  # kept alive: the batch uses their device arrays
        hs = (C.c_void_p * len(self._graphs))(*[g._h.value if isinstance(g._h, C.c_void_p) else g._h
                                                for g in self._graphs])
        qs = (Query * len(queries))(*[Query(int(gi), int(app), int(root)) for gi, app, root in queries])
        self.queries = list(queries)
        self._h = C.c_void_p()
        _check(lib().wedge_cuda_batch_create(C.cast(hs, C.c_void_p), len(self._graphs), C.cast(qs, C.c_void_p),
                                             len(queries), C.byref(self._h)), "wedge_cuda_batch_create")

    def run(self, tuning: BatchTuning | None = None, flags: int = 0) -> dict:
        st = BatchStats()
        _check(lib().wedge_cuda_batch_run(self._h, C.byref(tuning) if tuning is not None else None, flags,
                                          C.byref(st)), "wedge_cuda_batch_run")
        return st.as_dict()

    def read_result(self, q: int) -> np.ndarray:
        out = np.empty(self._graphs[self.queries[q][0]].V, np.uint64)
        _check(lib().wedge_cuda_batch_read_result(self._h, q, _ptr(out), out.nbytes), "wedge_cuda_batch_read_result")
        return out

    def iterations(self) -> np.ndarray:
        out = np.empty(len(self.queries), np.uint32)
        _check(lib().wedge_cuda_batch_iterations(self._h, _ptr(out), len(out)), "wedge_cuda_batch_iterations")
        return out

    def close(self):
        if self._h:
            lib().wedge_cuda_batch_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

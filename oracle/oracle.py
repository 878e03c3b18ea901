"""ORACLE -- test infrastructure, not product code.

ctypes front end for ``liboracle.so`` (the portable-C restatement of the
reference's pull-only edge-pull engine in ``wedge_oracle.c``) and for the
reference binary built here from its own sources (``_ref/wedge_ref``).
Only tests/, the smoke check and bench.py's CPU-baseline legs import this.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "wedge_ref")

BFS, CC, PR, SSSP = 0, 1, 2, 3
APP_NAMES = {"bfs": BFS, "cc": CC, "pr": PR, "sssp": SSSP}
WEIGHTS_U64, WEIGHTS_F64 = 0, 1
# rmat quadrant probabilities used by every configuration of the benchmark
RMAT_ABC = (0.57, 0.19, 0.19)


class Params(C.Structure):
    _fields_ = [("root", C.c_uint64), ("threshold_pct", C.c_uint64), ("iterations", C.c_uint64),
                ("damping", C.c_double), ("threads", C.c_int32), ("weight_kind", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_uint64), ("wedge_iterations", C.c_uint64), ("running_ms", C.c_double),
                ("pull_ms_nowedge", C.c_double), ("pull_ms_wedge", C.c_double), ("wedge_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build(quiet: bool = True) -> None:
    """Compile liboracle.so (portable C; both x86-64 and aarch64)."""
    subprocess.run(["make", "-C", HERE, "liboracle.so"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def build_ref(quiet: bool = True) -> bool:
    """Compile the reference from its own sources (x86-64 + AVX2 hosts only)."""
    # WEDGE_REFERENCE_DIR, else the reference checkout beside this repository
    ref = os.environ.get("WEDGE_REFERENCE_DIR", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
    if not os.path.isdir(os.path.join(ref, "source")):
        return False
    r = subprocess.run(["make", "-C", HERE, "ref", f"REF={ref}"],
                       stdout=subprocess.DEVNULL if quiet else None, stderr=subprocess.DEVNULL if quiet else None)
    return r.returncode == 0 and os.path.exists(REF_BIN)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
        L.orc_mix64.restype = C.c_uint64
        L.orc_mix64.argtypes = [C.c_uint64]
        L.orc_draw.restype = C.c_uint64
        L.orc_draw.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.orc_rmat.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_uint64,
                               C.c_uint64, u32p, u32p, C.c_int]
        L.orc_grid_edge_count.restype = C.c_uint64
        L.orc_grid_edge_count.argtypes = [C.c_uint64, C.c_double]
        L.orc_grid.argtypes = [C.c_uint64, C.c_double, C.c_uint64, u32p, u32p]
        L.orc_weight_u64.restype = C.c_uint64
        L.orc_weight_u64.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_weight_f64.restype = C.c_double
        L.orc_weight_f64.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_weights.argtypes = [C.c_uint64, u32p, u32p, C.c_int, u64p]
        L.orc_sort_edges.argtypes = [C.c_uint64, C.c_uint64, u32p, u32p, C.c_int]
        L.orc_write_file.argtypes = [C.c_char_p, C.c_uint64, C.c_uint64, u32p, u32p, C.c_void_p]
        L.orc_load_file.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.orc_build.argtypes = [C.c_uint64, C.c_uint64, u32p, u32p, C.c_void_p, C.c_int, C.c_int,
                                C.POINTER(C.c_void_p)]
        L.orc_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(Params), C.POINTER(Stats)]
        for f in ("orc_num_vertices", "orc_num_edges", "orc_num_edge_vectors"):
            getattr(L, f).restype = C.c_uint64
            getattr(L, f).argtypes = [C.c_void_p]
        L.orc_props.restype = C.POINTER(C.c_uint64)
        L.orc_props.argtypes = [C.c_void_p]
        L.orc_outdegrees.restype = C.POINTER(C.c_uint64)
        L.orc_outdegrees.argtypes = [C.c_void_p]
        L.orc_edge_vectors.restype = C.POINTER(C.c_uint64)
        L.orc_edge_vectors.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_online_cores.restype = C.c_int
        _lib = L
    return _lib


# ---------------------------------------------------------------- generators
def rmat(scale: int, edge_factor: int, seed: int, abc=RMAT_ABC, threads: int = 0):
    E = edge_factor << scale
    src = np.empty(E, np.uint32)
    dst = np.empty(E, np.uint32)
    lib().orc_rmat(scale, abc[0], abc[1], abc[2], seed, 0, E, src, dst, threads)
    return 1 << scale, src, dst


def grid(side: int, long_range_frac: float, seed: int):
    E = lib().orc_grid_edge_count(side, long_range_frac)
    src = np.empty(E, np.uint32)
    dst = np.empty(E, np.uint32)
    lib().orc_grid(side, long_range_frac, seed, src, dst)
    return side * side, src, dst


def weights(src, dst, kind=WEIGHTS_U64):
    out = np.empty(len(src), np.uint64)
    lib().orc_weights(len(src), np.ascontiguousarray(src), np.ascontiguousarray(dst), kind, out)
    return out


def sort_edges(V, src, dst, threads: int = 0):
    src = np.ascontiguousarray(src, np.uint32).copy()
    dst = np.ascontiguousarray(dst, np.uint32).copy()
    if lib().orc_sort_edges(V, len(src), src, dst, threads) != 0:
        raise MemoryError("orc_sort_edges")
    return src, dst


def symmetrise(src, dst):
    return np.concatenate([src, dst]), np.concatenate([dst, src])


def write_file(path, V, src, dst, w=None):
    wp = None if w is None else np.ascontiguousarray(w, np.uint64)
    rc = lib().orc_write_file(path.encode(), V, len(src), np.ascontiguousarray(src, np.uint32),
                              np.ascontiguousarray(dst, np.uint32),
                              None if wp is None else wp.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise OSError(f"orc_write_file rc={rc}")


# ---------------------------------------------------------------- engine
class OracleError(RuntimeError):
    def __init__(self, rc, what):
        super().__init__(f"{what}: oracle error {rc}")
        self.rc = rc


class Graph:
    """A graph held in the reference's edge-vector layout by the oracle."""

    def __init__(self, handle, app):
        self._h = handle
        self.app = app

    @classmethod
    def from_edges(cls, V, src, dst, app, w=None, threads: int = 0):
        h = C.c_void_p()
        wp = None
        if w is not None:
            wp = np.ascontiguousarray(w, np.uint64)
        rc = lib().orc_build(V, len(src), np.ascontiguousarray(src, np.uint32), np.ascontiguousarray(dst, np.uint32),
                             None if wp is None else wp.ctypes.data_as(C.c_void_p), app, threads, C.byref(h))
        if rc != 0:
            raise OracleError(rc, "orc_build")
        return cls(h, app)

    @classmethod
    def from_file(cls, path, app, threads: int = 0):
        h = C.c_void_p()
        rc = lib().orc_load_file(path.encode(), app, threads, C.byref(h))
        if rc != 0:
            raise OracleError(rc, "orc_load_file")
        return cls(h, app)

    @property
    def V(self):
        return lib().orc_num_vertices(self._h)

    @property
    def E(self):
        return lib().orc_num_edges(self._h)

    @property
    def num_edge_vectors(self):
        return lib().orc_num_edge_vectors(self._h)

    def edge_vectors(self):
        n = C.c_uint64()
        p = lib().orc_edge_vectors(self._h, C.byref(n))
        return np.ctypeslib.as_array(p, shape=(n.value,)).copy()

    def run(self, root=0, threshold_pct=20, iterations=1, damping=0.875, threads=1, weight_kind=WEIGHTS_U64):
        p = Params(root, threshold_pct, iterations, damping, threads, weight_kind)
        s = Stats()
        rc = lib().orc_run(self._h, self.app, C.byref(p), C.byref(s))
        if rc != 0:
            raise OracleError(rc, "orc_run")
        V = self.V
        props = np.ctypeslib.as_array(lib().orc_props(self._h), shape=(V,)).copy()
        outdeg = np.ctypeslib.as_array(lib().orc_outdegrees(self._h), shape=(V,)).copy()
        return props, outdeg, s.as_dict()

    def close(self):
        if self._h:
            lib().orc_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_reference(path, app_name, threads=1, iterations=1, root=0, threshold_pct=20):
    """Run the reference binary built from its own sources; returns (props, outdeg_or_None, stats)."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "props.bin")
        r = subprocess.run([REF_BIN, path, app_name, str(threads), str(iterations), str(root), str(threshold_pct), out],
                           capture_output=True, text=True, check=True)
        stats = json.loads(r.stdout.strip().splitlines()[-1])
        raw = np.fromfile(out, np.uint64)
    V = int(raw[0])
    props = raw[1:1 + V].copy()
    outdeg = raw[1 + V:1 + 2 * V].copy() if len(raw) >= 1 + 2 * V else None
    return props, outdeg, stats

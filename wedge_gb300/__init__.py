"""GB300 (sm_103a) edge-pull engine with Wedge's application and phase interface.

The compute path is ``lib/libwedge_cuda.so`` (hand-written CUDA behind the C
ABI of ``include/wedge_cuda.h``); this package is its ctypes front end.
Build with ``wedge_gb300.build.build_all()``.
"""
from .engine import (APP_BFS, APP_CC, APP_PR, APP_SSSP, FLAG_GRAPH, FLAG_TIMING, PREC_FP32C, PREC_FP64,  # noqa: F401
                     SCHED_DENSE, SCHED_PLAIN, SCHED_WEDGE, WEIGHTS_F64, WEIGHTS_NONE, WEIGHTS_U64, Graph, Params,
                     WedgeError, application_select, lib, prop_string, status_string)

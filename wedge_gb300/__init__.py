"""GB300 (sm_103a) edge-pull engine with Wedge's application and phase interface.

The compute path is ``lib/libwedge_cuda.so`` (hand-written CUDA behind the C
ABI of ``include/wedge_cuda.h``); this package is its ctypes front end.
Build with ``wedge_gb300.build.build_all()``.
"""
from .engine import (APP_BFS, APP_CC, APP_PR, APP_SSSP, ERR_ARG, FLAG_GRAPH, FLAG_TIMING, KNOB_DEFAULT,  # noqa: F401
                     KNOB_HUB_BYTES, KNOB_NAMES, KNOB_PROBE_EDGES, KNOB_SSSP_NARROW, KNOB_SSSP_TILE, MODE_DENSE,
                     MODE_FILTERED, MODE_WEDGE, PHASE_ADVANCE, PHASE_INIT, PHASE_PULL_DENSE, PHASE_PULL_WEDGE,
                     PHASE_VERTEX_PR, PHASE_WEDGE_BUILD, PREC_FP32C, PREC_FP64, SCHED_BLOB, SCHED_DENSE, SCHED_FEATURES,
                     SCHED_FILTERED, SCHED_LEARNED, SCHED_PARAMS, SCHED_PLAIN, SCHED_PROBE, SCHED_WEDGE, WEIGHTS_F64,
                     WEIGHTS_NONE, WEIGHTS_U64, Batch, BatchTuning, Graph, Params, Query, WedgeError, application_select, lib, mlp_forward,
                     mlp_loss_grad, mlp_train, prop_string, status_string)

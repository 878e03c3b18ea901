"""The C ABI boundary: the library loads on any host, exports every function
include/wedge_cuda.h declares, and the ctypes mirror matches the C layout.
No CUDA work is done here."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "wedge_cuda.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wedge_(?:cuda|mlp)_\w+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("wedge_cuda_load_graph", "wedge_cuda_run", "wedge_cuda_run_phase", "wedge_cuda_read_results",
                     "wedge_cuda_free"):
        assert required in names


def test_library_exports_every_declared_symbol(engine_lib):
    L = engine_lib.lib()
    for name in declared_functions():
        assert hasattr(L, name), f"{name} is declared but not exported"


def test_ctypes_binding_covers_header(engine_lib):
    from wedge_gb300 import engine

    assert set(engine._SIGNATURES) == set(declared_functions())


def test_status_strings_and_version(engine_lib):
    W = engine_lib
    assert W.status_string(0) == "ok"
    assert "format" in W.status_string(-2) or "malformed" in W.status_string(-2)
    assert W.lib().wedge_cuda_abi_version() == 2


def test_null_handles_are_rejected(engine_lib):
    L = engine_lib.lib()
    from wedge_gb300.engine import Params, Stats

    assert L.wedge_cuda_run(None, 0, C.byref(Params()), C.byref(Stats())) == -6
    assert L.wedge_cuda_read_results(None, None, 0) == -6
    assert L.wedge_cuda_run_async(None, 0, C.byref(Params())) == -6
    assert L.wedge_cuda_read_results_async(None, None, 0) == -6
    assert L.wedge_cuda_wait(None, None) == -6
    assert L.wedge_cuda_set_stream(None, None) == -6
    assert L.wedge_cuda_wait_results(None) == -6
    assert L.wedge_cuda_set_knob(None, 0, 65536) == -6
    v = C.c_uint64()
    assert L.wedge_cuda_get_knob(None, 0, C.byref(v)) == -6
    assert L.wedge_cuda_num_vertices(None) == 0
    L.wedge_cuda_free(None)


def test_struct_layout_matches_c(engine_lib, tmp_path):
    from wedge_gb300.engine import BatchStats, BatchTuning, IterationRecord, Params, Query, Stats

    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "wedge_cuda.h"', "int main(void){"]
    want = []
    for cls, cname in ((Params, "wedge_params_t"), (Stats, "wedge_stats_t"),
                       (IterationRecord, "wedge_iteration_record_t"), (Query, "wedge_query_t"),
                       (BatchTuning, "wedge_batch_tuning_t"), (BatchStats, "wedge_batch_stats_t")):
        fields = [f for f, _ in cls._fields_]
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        lines += [f'printf("%zu\\n", offsetof({cname}, {f}));' for f in fields]
        want += [C.sizeof(cls)] + [getattr(cls, f).offset for f in fields]
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out == want


def test_missing_file_is_an_io_error_before_any_device_work(engine_lib):
    W = engine_lib
    with pytest.raises(W.WedgeError) as e:
        W.Graph.load("/nonexistent/graph.bin", W.APP_BFS)
    assert e.value.status == -1


def test_application_select_matches_reference_names(engine_lib):
    W = engine_lib
    assert W.application_select("BFS") == W.APP_BFS
    assert W.application_select("Breadth_First_Search") == W.APP_BFS
    assert W.application_select("connectedcomponents") == W.APP_CC
    assert W.application_select("PageRank") == W.APP_PR
    assert W.application_select("single_source_shortest_path") == W.APP_SSSP
    with pytest.raises(ValueError):
        W.application_select("bfsx")


def test_prop_strings(engine_lib):
    import numpy as np

    W = engine_lib
    assert W.prop_string(W.APP_BFS, 2**64 - 1, 0, 10) == "-1"
    assert W.prop_string(W.APP_BFS, 7, 0, 10) == "7"
    assert W.prop_string(W.APP_CC, int(np.float64(3.0).view(np.uint64)), 0, 10) == "3"
    r = int(np.float64(0.05).view(np.uint64))
    assert W.prop_string(W.APP_PR, r, 2, 10) == "1.0000e-01"
    assert W.prop_string(W.APP_PR, r, 0, 10) == "5.0000e-01"
    assert W.prop_string(W.APP_SSSP, 2**64 - 1, 0, 10) == "-1"


@pytest.mark.parametrize("args,code", [
    (["-x"], 1),                       # unknown option (cmdline.c:128-135)
    (["-a", "bfs", "-t", "abc", "-i", "g"], 2),  # invalid value
    (["-a"], 3),                       # missing value
    (["-i", "g"], 5),                  # missing required -a
    (["-a", "bfs"], 5),                # missing required -i
    (["-h"], 0),
])
def test_cli_exit_codes(engine_lib, args, code):
    from wedge_gb300 import build as B

    exe = os.path.join(B.OUT_BIN, "wedge")
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=60)
    assert r.returncode == code, r.stdout


def test_cli_rejects_unknown_application(engine_lib):
    from wedge_gb300 import build as B

    r = subprocess.run([os.path.join(B.OUT_BIN, "wedge"), "-a", "foo", "-i", "g"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode != 0 and 'unable to run "foo"' in r.stdout

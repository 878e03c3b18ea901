"""The allocation-free PageRank iteration (wedge_cuda_pr_iteration_noalloc).

It serves callers that cannot allocate device memory themselves -- a host
framework that hands the library only buffers from its own pool -- so here the
test, playing that caller, owns every device buffer (allocated through torch)
and the entry point must produce, call after call, the same ranks as the
regular entry point (wedge_cuda_run), within the PageRank FP64 tolerance of the
other parity tests (1e-12 relative L1).  Kept in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PR_TOL = 1e-12


def _csc(O, scale, edge_factor, seed):
    V, s, d = O.rmat(scale, edge_factor, seed)
    s, d = O.sort_edges(V, s, d)
    E = len(s)
    heads = np.r_[True, d[1:] != d[:-1]]
    dst_id = d[heads].astype(np.uint32)
    dst_off = np.r_[np.nonzero(heads)[0], E].astype(np.uint64)
    Epad = (E + 127) // 128 * 128
    src = np.full(Epad, 0xFFFFFFFF, np.uint32)
    src[:E] = s
    outdeg = np.bincount(s, minlength=V).astype(np.uint32)
    return V, s, d, dst_id, dst_off, src, outdeg


def _dev(torch, a):
    """a device copy owned by the caller (torch's allocator, not the library)"""
    view = {np.uint64: np.int64, np.uint32: np.int32, np.float64: np.float64}[a.dtype.type]
    return torch.from_numpy(np.ascontiguousarray(a).view(view)).cuda()


def _rel_l1(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())


@pytest.mark.parametrize("scale,edge_factor,seed", [(12, 16, 7), (14, 8, 8)])
def test_noalloc_iteration_matches_engine(engine_lib, oracle_lib, scale, edge_factor, seed):
    torch = pytest.importorskip("torch")
    W, O = engine_lib, oracle_lib
    L = W.lib()
    V, s, d, dst_id, dst_off, src, outdeg = _csc(O, scale, edge_factor, seed)
    E = len(s)

    # the regular entry point: one and two iterations from the reference's initial ranks
    with W.Graph.from_edges(V, s, d) as g:
        g.run(W.APP_PR, W.Params(num_iterations=1))
        want1 = g.read_results().view(np.float64).copy()
        g.run(W.APP_PR, W.Params(num_iterations=2))
        want2 = g.read_results().view(np.float64).copy()

    od = np.where(outdeg == 0, V, outdeg).astype(np.float64)
    rank0 = (1.0 / V) / od  # execution_initialize_pr (execution_pr.c:380-392)
    t_off, t_id, t_src, t_od = (_dev(torch, x) for x in (dst_off, dst_id, src, outdeg))
    r0 = _dev(torch, rank0)
    r1 = torch.empty(V, dtype=torch.float64, device="cuda")
    r2 = torch.empty(V, dtype=torch.float64, device="cuda")

    def call(rin, rout):
        torch.cuda.synchronize()
        rc = L.wedge_cuda_pr_iteration_noalloc(V, len(dst_id), E, t_off.data_ptr(), t_id.data_ptr(),
                                                t_src.data_ptr(), t_od.data_ptr(), rin.data_ptr(), rout.data_ptr(),
                                                0.0, None)
        assert rc == 0, W.status_string(rc)
        torch.cuda.synchronize()
        return rout.cpu().numpy()

    got1 = call(r0, r1)  # first call on this device also sets up the scratch address
    assert _rel_l1(got1, want1) < PR_TOL
    got2 = call(r1, r2)  # second call in a row: the shared scratch is reused
    assert _rel_l1(got2, want2) < PR_TOL
    # and against the oracle's restatement of the reference
    ref, _, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=2, threads=4)
    assert _rel_l1(got2, ref.view(np.float64)) < PR_TOL


def test_noalloc_reuse_across_graphs_on_a_stream(engine_lib, oracle_lib):
    """One caller-created stream; a graph at the scratch's limit (R-MAT scale 20,
    edge factor 16: exactly 2^24 in-edges) and then a smaller one reuse the shared
    scratch, which must hold nothing over from the larger call."""
    torch = pytest.importorskip("torch")
    W, O = engine_lib, oracle_lib
    L = W.lib()
    stream = torch.cuda.Stream()
    for scale, edge_factor, seed in ((20, 16, 21), (12, 8, 22)):
        V, s, d, dst_id, dst_off, src, outdeg = _csc(O, scale, edge_factor, seed)
        E = len(s)
        assert E <= 1 << 24
        with W.Graph.from_edges(V, s, d) as g:
            g.run(W.APP_PR, W.Params(num_iterations=1, damping=0.85))
            want = g.read_results().view(np.float64).copy()
        ref, _, _ = O.Graph.from_edges(V, s, d, O.PR).run(iterations=1, damping=0.85, threads=4)
        od = np.where(outdeg == 0, V, outdeg).astype(np.float64)
        with torch.cuda.stream(stream):
            t_off, t_id, t_src, t_od = (_dev(torch, x) for x in (dst_off, dst_id, src, outdeg))
            r0 = _dev(torch, (1.0 / V) / od)
            r1 = torch.empty(V, dtype=torch.float64, device="cuda")
        stream.synchronize()
        rc = L.wedge_cuda_pr_iteration_noalloc(V, len(dst_id), E, t_off.data_ptr(), t_id.data_ptr(), t_src.data_ptr(),
                                                t_od.data_ptr(), r0.data_ptr(), r1.data_ptr(), 0.85,
                                                C.c_void_p(stream.cuda_stream))
        assert rc == 0, W.status_string(rc)
        stream.synchronize()
        got = r1.cpu().numpy()
        assert _rel_l1(got, want) < PR_TOL, scale
        assert _rel_l1(got, ref.view(np.float64)) < PR_TOL, scale


def test_noalloc_rejects_sizes_beyond_its_scratch(engine_lib):
    W = engine_lib
    L = W.lib()
    limit = 1 << 24  # WEDGE_NOALLOC_MAX_EDGES
    p = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.wedge_cuda_pr_iteration_noalloc(1 << 20, 1 << 20, limit + 1, p, p, p, p, p, p, 0.0, None)
    assert rc == W.engine.ERR_ARG

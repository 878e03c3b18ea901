"""The destination-range split (wedge_gb300/shard.py) on CPU: the partition
rule of the reference's NUMA split, and the sharded driver loop with its
exchange run as world-size-2 gloo ranks, each rank one numpy shard
(tests/shard_numpy.py) -- results equal to the oracle's whole-graph run: CC
labels and SSSP distances bit-exact, BFS levels exact with every parent an
in-neighbour one level up."""
import os
import socket

import numpy as np
import pytest

from helpers import check_bfs, levels_from_parents
from wedge_gb300 import engine as W
from wedge_gb300 import shard as SH


def test_partition_follows_the_reference_rule():
    rng = np.random.default_rng(3)
    V = 10000
    dst = np.sort(rng.integers(0, V, 50000))
    for n in (1, 2, 3, 5):
        b = SH.partition(V, dst, n)
        assert len(b) == n and b[0][0] == 0 and b[-1][1] == V - 1
        for (f0, l0), (f1, l1) in zip(b, b[1:]):
            assert f1 == l0 + 1 and (l0 + 1) % 512 == 0  # ranges end on 512-vertex boundaries
        # every edge in exactly one shard, in order
        parts = [SH.shard_edges(dst, x) for x in b]
        assert sum(p.stop - p.start for p in parts) == len(dst)
        assert all(np.all((dst[p] >= f) & (dst[p] <= l)) for p, (f, l) in zip(parts, b))
    # more shards than 512-vertex blocks: trailing shards are empty ranges
    b = SH.partition(600, np.sort(rng.integers(0, 600, 1000)), 4)
    assert b[-1][1] == 599 and sum(max(0, l - f + 1) for f, l in b) == 600


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, V, src, dst, w, outdeg, app, root, out_path):
    import torch.distributed as dist

    from shard_numpy import NumpyShard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bounds = SH.partition(V, dst, world)[rank]
    sl = SH.shard_edges(dst, bounds)
    shard = NumpyShard(V, src[sl], dst[sl], outdeg, None if w is None else w[sl])
    info = SH.run([shard], app, W.Params(root=root), SH.Exchange(dist.group.WORLD), outdeg, len(src))
    if rank == 0:
        np.save(out_path, shard.read_results())
        np.save(out_path + ".iters.npy", np.array([info["iterations"]]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("app", ["bfs", "cc", "sssp"])
def test_two_gloo_ranks_match_the_oracle(oracle_lib, tmp_path, app):
    import torch.multiprocessing as mp

    O = oracle_lib
    V, s, d = O.rmat(11, 16, 41)
    if app == "cc":
        s, d = O.symmetrise(s, d)
    s, d = O.sort_edges(V, s, d)
    w = O.weights(s, d) if app == "sssp" else None
    outdeg = np.bincount(s, minlength=V).astype(np.uint64)
    a = {"bfs": W.APP_BFS, "cc": W.APP_CC, "sssp": W.APP_SSSP}[app]
    out = str(tmp_path / "props.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), V, s, d, w, outdeg, a, 0, out), nprocs=2, join=True)
    got = np.load(out)
    if app == "bfs":
        ref, _, _ = O.Graph.from_edges(V, s, d, O.BFS).run(root=0, threads=2)
        check_bfs(got, V, s, d, 0, levels_from_parents(ref, 0))
    elif app == "cc":
        ref, _, _ = O.Graph.from_edges(V, s, d, O.CC).run(threads=2)
        assert np.array_equal(got, ref)
    else:
        ref, _, _ = O.Graph.from_edges(V, s, d, O.SSSP, w).run(root=0, threads=2)
        assert np.array_equal(got, ref)

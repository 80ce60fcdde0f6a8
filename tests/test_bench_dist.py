"""The multi-process plumbing of bench.py on CPU: two gloo ranks, as `torchrun --nproc-per-node 2`
launches them.  Replicas only (no data-path collective): the ranks meet at a barrier around the timed
region, the device time is the maximum over ranks, and the reference arm runs on rank 0 alone while the
other ranks return without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "EP_BENCH_GLOO": "1"})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, w = bench.dist_init()
    bench.barrier(w)
    mx = bench.allmax(float(10 * r + 1), w)
    # the reference arm: only rank 0 works; the others must return at once
    skipped = bench.run_reference(None, r, w) is None if r != 0 else True
    bench.barrier(w)
    out.put((r, w, mx, skipped))
    dist.destroy_process_group()


def test_two_gloo_ranks_replicas():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert all(g[2] == 11.0 for g in got)          # the maximum over ranks reaches every rank
    assert all(g[3] for g in got)

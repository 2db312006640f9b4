"""bench.py's replica plumbing on CPU: two gloo ranks run dist_init, the
barrier and the max over ranks, and the whole-job rate counts every rank's
units against the slowest rank's time."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "TCFFT_DIST_BACKEND": "gloo"})
    sys.path.insert(0, REPO)
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_init()
    bench.barrier(w)
    ms = bench.max_over_ranks(w, 10.0 + 5.0 * r)  # rank 1 is the slow one
    out.put((r, w, ms, bench.whole_job_rate(100.0, w, ms)))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1]
    for _, w, ms, rate in res:
        assert w == 2 and ms == 15.0
        assert rate == pytest.approx(100.0 * 2 / 15e-3)


def test_single_rank_defaults(monkeypatch):
    sys.path.insert(0, REPO)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_init() == (1, 0, 0)
    assert bench.max_over_ranks(1, 3.5) == 3.5

"""bench.py's multi-rank plumbing on CPU: two `gloo` ranks (127.0.0.1) time different
step lists; the whole-job figure is all ranks' frames over the slowest rank's total."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, steps, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "AXR_DIST_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    try:
        d.barrier()
        value, ms = bench.aggregate(steps, d)
        out.put((rank, value, ms, d.max(float(rank))))
    finally:
        d.close()


@pytest.mark.timeout(120)
def test_two_rank_aggregate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    steps = {0: [1.0, 2.0], 1: [3.0, 4.0]}
    procs = [ctx.Process(target=_rank, args=(r, 2, port, steps[r], q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank, value, ms, mx in res:
        # 2 ranks x 2 steps = 4 frames over the slowest rank's 7 ms
        assert value == pytest.approx(4 / 7e-3)
        assert ms == pytest.approx(3.5)
        assert mx == 1.0


def test_single_rank_aggregate():
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    value, ms = bench.aggregate([2.0, 2.0], d)
    assert value == pytest.approx(2 / 4e-3) and ms == pytest.approx(2.0)

"""bench.py under torchrun: every rank runs its own replica (the path has no
exchange step); the timing is maxed over ranks and the work summed.  Checked
here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_setup()
    bench.dist_barrier(w)
    mx = bench.dist_max(w, 10.0 + r)       # this rank's time
    sm = bench.dist_sum(w, 1000.0 * (r + 1))  # this rank's site-updates
    q.put((r, w, local, mx, sm))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_ranks_max_time_and_sum_work():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[:3] for g in got] == [(0, 2, 0), (1, 2, 1)]
    assert all(g[3] == 11.0 for g in got)       # the slower rank's time
    assert all(g[4] == 3000.0 for g in got)     # both ranks' work


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (1, 0, 0)
    assert bench.dist_max(w, 3.5) == 3.5 and bench.dist_sum(w, 2.0) == 2.0

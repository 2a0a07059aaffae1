"""The replica path of bench.py on the host: world size 2 over gloo (no GPU).  Every rank gets the
slowest rank's time, and the whole-job rate counts the units of all ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    r, w = bench.dist_init('gloo')
    bench.barrier(w)
    seconds = 0.5 + rank          # rank 1 is the slow one
    slowest = bench.max_over_ranks(seconds, w)
    rate = bench.replica_rate(10, seconds, w)
    bench.barrier(w)
    dist.destroy_process_group()
    q.put((r, w, slowest, rate))


def test_two_gloo_replicas_share_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[2] == pytest.approx(1.5) for o in out)
    assert all(o[3] == pytest.approx(2 * 10 / 1.5) for o in out)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.25, 1) == 0.25
    assert bench.replica_rate(10, 0.5, 1) == pytest.approx(20.0)

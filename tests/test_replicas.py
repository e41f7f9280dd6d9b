"""bench.py's replica plumbing on two gloo ranks (CPU): each GPU runs an
independent replica; the ranks only meet for the barrier around the timed
region and for the whole-job reductions (max of times, sum of work)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist(world)
    d.barrier()
    out.put((rank, d.world, d.local, d.max(float(rank) * 10.0), d.sum(float(rank + 1))))
    d.barrier()
    d.pg.destroy_process_group()


def test_two_gloo_ranks_reduce_like_one_job():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for rank, world, local, mx, sm in res:
        assert world == 2 and local == rank
        assert mx == 10.0  # slowest rank's time
        assert sm == 3.0   # work of both ranks

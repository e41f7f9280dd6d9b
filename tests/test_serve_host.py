"""The query server's host logic without a GPU: the seeded stream, its split
across replicas, and the merge of two gloo ranks' answers into one summary
(subway_gb300/serve.py).  A stand-in batch object answers each batch after a
short sleep, as sgw_batch_run would on a GPU."""
import os
import socket
import sys
import time
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


class _G:
    def __init__(self, n):
        self.n = n


class _FakeBatch:
    def __init__(self, n, log=None):
        self.graph = _G(n)
        self.log = log if log is not None else []

    def run(self, algo, sources, view=False, answers="u32"):
        self.log.append(np.asarray(sources).copy())
        time.sleep(0.0005)


def test_stream_is_seeded_and_shards_cover_it_once():
    from subway_gb300 import serve
    a = serve.make_stream([100, 1000], queries=500, rate=1000.0, seed=3)
    b = serve.make_stream([100, 1000], queries=500, rate=1000.0, seed=3)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    arr, tgt, src = a
    assert np.all(np.diff(arr) > 0) and np.all(src < np.where(tgt == 0, 100, 1000))
    parts = [serve.shard(a, 3, r) for r in range(3)]
    assert sum(len(p[0]) for p in parts) == 500
    merged = np.sort(np.concatenate([p[0] for p in parts]))
    assert np.array_equal(merged, arr)


def test_single_replica_serves_every_query():
    from subway_gb300 import serve
    log = []
    batches = [_FakeBatch(50, log), _FakeBatch(80, log)]
    res = serve.serve(batches, "bfs", queries=300, rate=3000.0, seed=1, lanes=8)
    assert res["queries"] == 300 and res["max_batch"] <= 8
    assert sum(len(x) for x in log) == 300 and res["batches"] == len(log)
    assert 0 < res["p50_ms"] <= res["p99_ms"] and res["qps"] > 0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, out):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as td
    from subway_gb300 import serve
    td.init_process_group("gloo")
    log = []
    res = serve.serve_replicas([_FakeBatch(60, log), _FakeBatch(90, log)], td, "sssp", queries=240,
                               rate=2000.0, seed=7, lanes=4)
    out.put((rank, res, sorted(int(s) for x in log for s in x)))
    td.destroy_process_group()


def test_two_replicas_merge_into_one_summary():
    torch = pytest.importorskip("torch")
    from subway_gb300 import serve
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_replica, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted((q.get(timeout=120) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, res0, src0), (_, res1, src1) = got
    assert res1 is None
    assert res0["replicas"] == 2 and res0["queries"] == 240
    assert res0["queries_per_replica"] == [120, 120]
    _, _, sources = serve.make_stream([60, 90], queries=240, rate=2000.0, seed=7)
    assert sorted(src0 + src1) == sorted(int(s) for s in sources)  # each query served once
    assert res0["max_batch"] <= 4 and 0 < res0["p50_ms"] <= res0["p99_ms"]

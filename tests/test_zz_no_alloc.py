"""sgw_generate_noalloc: the allocation-free form of the engine's compaction.

Callers that cannot allocate device memory (a host framework that owns every
device byte through its own pool, or a latency-critical loop where cudaMalloc
would synchronise the device) pass in their own arrays; the scan state lives
in a static device array inside the library.  Its output must equal the
engine's own generate step (sgw_state_init + sgw_read_active) exactly, on two
calls in a row that reuse the shared static array.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a: np.ndarray):
    return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()


def _noalloc(native, torch, g, label2, consume=1, label1=None):
    n = g.n
    l1 = _dev(torch, np.zeros(n, np.uint8) if label1 is None else label1.astype(np.uint8))
    l2 = _dev(torch, label2.astype(np.uint8))
    off = _dev(torch, np.ascontiguousarray(g.node_pointer))
    queue = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    ptr = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
    cnt, edges = C.c_uint32(), C.c_uint64()
    torch.cuda.synchronize()
    st = native.lib().sgw_generate_noalloc(l1.data_ptr(), l2.data_ptr(), off.data_ptr(), n, consume,
                                           queue.data_ptr(), ptr.data_ptr(),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                           C.byref(cnt), C.byref(edges))
    native.check(st, "sgw_generate_noalloc")
    c = cnt.value
    q = queue[:c].cpu().numpy().view(np.uint32)
    p = ptr[: c + 1].cpu().numpy().view(np.uint32)
    if label1 is not None:
        return q, p, edges.value, l1.cpu().numpy(), l2.cpu().numpy()
    return q, p, edges.value, l2.cpu().numpy()


def test_noalloc_matches_engine_generate_twice(gpu):
    torch = pytest.importorskip("torch")
    native = gpu
    g = native.Graph.rmat(16, 16, seed=21)
    src = int(g.pick_sources(1, seed=4)[0])
    eng = native.Engine(g)
    # existing entry point, call 1: every vertex active (cc-sync start)
    eng.state_init("cc", "sync")
    q_ref1, p_ref1 = eng.read_active()
    # existing entry point, call 2: only the source active (bfs-sync start)
    eng.state_init("bfs", "sync", src)
    q_ref2, p_ref2 = eng.read_active()
    eng.close()

    q1, p1, e1, l2_after = _noalloc(native, torch, g, np.ones(g.n, np.uint8))
    assert np.array_equal(q1, q_ref1) and np.array_equal(p1, p_ref1)
    assert e1 == int(p_ref1[-1])
    assert not l2_after.any(), "consume=1 clears the labels it queued"

    one = np.zeros(g.n, np.uint8)
    one[src] = 1
    q2, p2, e2, _ = _noalloc(native, torch, g, one)
    assert np.array_equal(q2, q_ref2) and np.array_equal(p2, p_ref2)
    assert q2.tolist() == [src] and e2 == int(g.out_degree()[src])


def test_noalloc_ragged_tiles_both_forms_three_calls(gpu, orc):
    """40 full 4096-vertex tiles and a partial 41st (so every tile's
    look-back passes more than 32 predecessors), random labels in both
    arrays, consume = 0, 1, 0 on three calls in a row through the shared
    static array: each call's queue and pointers equal the oracle's
    compaction of the vertices with out-edges, and the labels afterwards are
    what the form promises (consume clears queued vertices; active vertices
    without out-edges are always cleared; the rest are left alone)."""
    torch = pytest.importorskip("torch")
    native = gpu
    n = 40 * 4096 + 123
    g = native.Graph.er(n, 6 * n, seed=29)
    deg = g.out_degree()
    assert (deg == 0).any()
    rng = np.random.default_rng(31)
    for consume in (0, 1, 0):
        l1 = (rng.random(n) < 0.15).astype(np.uint8)
        l2 = (rng.random(n) < 0.25).astype(np.uint8)
        q_all, p_all = orc.generate(l1, l2, deg)
        keep = deg[q_all] > 0
        q, p, e, l1a, l2a = _noalloc(native, torch, g, l2, consume=consume, label1=l1)
        assert np.array_equal(q, q_all[keep]), consume
        assert np.array_equal(p[:-1], p_all[:-1][keep]) and p[-1] == p_all[-1] == e, consume
        active = (l1 | l2) != 0
        cleared = active & ((deg == 0) | bool(consume))
        assert not (l1a[cleared] | l2a[cleared]).any(), consume
        assert np.array_equal(l1a[~cleared], l1[~cleared]) and np.array_equal(l2a[~cleared], l2[~cleared]), consume


def test_noalloc_rejects_oversize(gpu):
    torch = pytest.importorskip("torch")
    native = gpu
    x = torch.zeros(16, dtype=torch.int32, device="cuda")
    cnt, edges = C.c_uint32(), C.c_uint64()
    limit = 67108864
    st = native.lib().sgw_generate_noalloc(x.data_ptr(), x.data_ptr(), x.data_ptr(), limit + 1, 1,
                                           x.data_ptr(), x.data_ptr(), None, C.byref(cnt), C.byref(edges))
    assert st == -9  # SGW_ERANGE, before any device work
    assert b"static scratch limit" in native.lib().sgw_last_error()

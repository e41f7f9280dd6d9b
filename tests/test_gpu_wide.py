"""Graphs with u64 node pointers and the per-generate edge limit, on the GPU,
against the oracle.  The reference reads u32 counts and offsets
(shared/graph.cu:43-51), so it has no counterpart past 2^32 edges; the last
test runs such a graph (R-MAT scale 28, edge factor 17: about 4.5 G edges,
18 GB of records) end to end."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALGS = ["bfs", "sssp", "sswp", "cc"]
MODES = ["sync", "async"]


def _wide(gpu, g):
    """The same graph over a caller's u64 node pointers."""
    return gpu.Graph.from_csr(g.node_pointer.astype(np.uint64), np.array(g.edges), g.weighted)


def _oracle(orc, g, algo, src):
    e = g.edges
    if algo in ("bfs", "cc") and g.weighted:
        e = np.ascontiguousarray(e[:, 0])
    return orc.run(algo, g.node_pointer, e, src)


@pytest.mark.parametrize("flags", ["", "NO_PACK", "SPLIT_WEIGHTS", "SCALAR_GATHER"])
def test_u64_node_pointers_bit_exact(gpu, orc, flags):
    """Engines on u64 node pointers use the wide gather kernels (host
    positions from the low words plus a base per 1024 vertices) in every
    transfer form, with the transfer copy in 16 KiB chunks and the plain and
    learned schedules; the answers are the oracle's."""
    fl = 0
    for f in filter(None, flags.split("|")):
        fl |= getattr(gpu, "OPT_" + f)
    g = _wide(gpu, gpu.Graph.rmat(14, 16, seed=12, weighted=True, wmax=64))
    assert g.node_pointer.dtype == np.uint64
    budget = 18 * g.n + 128 * 1024 + (g.m // 6) * 8 * 3
    plain = gpu.Engine(g, budget_bytes=budget, flags=fl, transfer_chunk_log2=14)
    learned = gpu.Engine(g, budget_bytes=budget, flags=fl, transfer_chunk_log2=14, num_buffers=3)
    learned.set_policy("learned")
    assert plain.max_partition_size() < g.m
    src = int(g.pick_sources(1, seed=3)[0])
    for algo in ALGS:
        ref = _oracle(orc, g, algo, src)
        for mode in MODES:
            for eng in (plain, learned):
                vals, _ = eng.run(algo, mode, src)
                assert np.array_equal(vals, ref), (algo, mode, flags)
    plain.close()
    learned.close()


def test_u64_hub_and_batch(gpu, orc):
    """A vertex above the edge buffer, streamed in pieces from u64
    positions, and a multi-source batch on a device-resident u64 graph."""
    n = 3000
    rng = np.random.default_rng(5)
    src = np.concatenate([np.zeros(2500, np.int64), rng.integers(0, n, 4000)])
    dst = np.concatenate([np.arange(1, 2501), rng.integers(0, n, 4000)])
    keep = (src != dst) & (src != n - 2)
    pairs = np.unique(np.stack([src[keep], dst[keep]], 1), axis=0)
    npt = np.zeros(n + 1, np.uint64)
    np.add.at(npt, pairs[:, 0] + 1, 1)
    npt = np.cumsum(npt).astype(np.uint64)
    w = (1 + (pairs[:, 0] * 7 + pairs[:, 1] * 13) % 50).astype(np.uint32)
    g = gpu.Graph.from_csr(npt, np.stack([pairs[:, 1].astype(np.uint32), w], 1), True)
    eng = gpu.Engine(g, budget_bytes=18 * n + 15 * 1024 + 1000 * 16)
    assert eng.max_partition_size() < 2500
    for algo in ALGS:
        for mode in MODES:
            vals, _ = eng.run(algo, mode, 0)
            assert np.array_equal(vals, _oracle(orc, g, algo, 0)), (algo, mode)
    eng.close()
    big = _wide(gpu, gpu.Graph.rmat(13, 16, seed=21, weighted=True, wmax=64))
    sources = [int(s) for s in big.pick_sources(8, seed=2)]
    b = gpu.Batch(big, lanes=32)
    for algo in ("bfs", "sssp"):
        got, _ = b.run(algo, sources)
        for k, s in enumerate(sources):
            assert np.array_equal(got[k], _oracle(orc, big, algo, s)), (algo, s)
    b.close()


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("policy", ["plain", "learned"])
def test_generate_edge_limit(gpu, orc, wide, policy):
    """A generate limited to a prefix of whole 4096-vertex tiles (the first
    tile with edges always) leaves the later tiles' vertices active for the
    next iteration: the answers stay the oracle's and the runs take more
    global iterations.  Limit 1 takes one tile per generate."""
    g = gpu.Graph.rmat(15, 8, seed=4, weighted=True, wmax=64)
    if wide:
        g = _wide(gpu, g)
    budget = 18 * g.n + 128 * 1024 + (g.m // 3) * 8 * 3
    engines = {}
    for lim in (0, 1, g.m // 5):
        e = gpu.Engine(g, budget_bytes=budget, generate_edge_limit=lim, num_buffers=3)
        if policy == "learned":
            e.set_policy("learned")
        engines[lim] = e
    src = int(g.pick_sources(1, seed=6)[0])
    for algo in ALGS:
        ref = _oracle(orc, g, algo, src)
        for mode in MODES:
            iters = {}
            for lim, e in engines.items():
                vals, st = e.run(algo, mode, src)
                assert np.array_equal(vals, ref), (algo, mode, lim)
                iters[lim] = st["global_iterations"]
            assert iters[1] > iters[0], (algo, mode, iters)
    for e in engines.values():
        e.close()


@pytest.mark.parametrize("wide", [False, True])
def test_pagerank_generate_edge_limit(gpu, orc, wide):
    """PageRank's generate under an edge limit: tiles past the limit keep
    their residuals for the next round.  Ranks stay within the residual bound
    of the FP64 oracle (twice acc / init, both being within acc / init of the
    fixpoint), and without a limit within 2.5e-7 (the same bulk-synchronous
    rounds)."""
    g = gpu.Graph.rmat(14, 16, seed=32)
    if wide:
        g = _wide(gpu, g)
    init, acc, damp = (float(np.float32(x)) for x in (0.15, 1e-3, 0.85))
    ref, _ = orc.pagerank(g.node_pointer, g.ends, init=init, acc=acc, damping=damp)
    budget = 36 * g.n + 128 * 1024 + (g.m // 3) * 4 * 2
    for lim, bound in ((0, 2.5e-7), (1, 2 * acc / init), (g.m // 4, 2 * acc / init)):
        e = gpu.Engine(g, budget_bytes=budget, generate_edge_limit=lim)
        for mode in MODES:
            vals, st = e.run("pr", mode, pr_acc=acc)
            rel = np.max(np.abs(vals.astype(np.float64) - ref) / ref)
            assert rel < (bound if mode == "sync" else 2 * acc / init), (lim, mode, rel)
        e.close()


def test_graph_past_2pow32_edges(gpu, orc):
    """R-MAT scale 28, edge factor 17, unweighted: more than 2^32 edges, so
    the library keeps u64 node pointers, the engine gathers from host
    positions above 2^32 and limits each generate to 2^31 edges.  BFS (both
    modes, plain and learned schedules, 8 GB budget) equals the OpenMP
    oracle; a u32 file refuses the graph."""
    g = gpu.Graph.rmat(28, 17, seed=28)
    assert g.m >= 2 ** 32
    npt = g.node_pointer
    assert npt.dtype == np.uint64 and int(npt[-1]) == g.m
    with pytest.raises(gpu.SgwError):
        g.save("/nonexistent-dir/never-written.bcsr")  # u32 header refused before any file is made
    ref = orc.run("bfs", npt, g.ends, 0, parallel=True)
    assert int((ref != 4294967294).sum()) > g.n // 4  # R-MAT leaves many vertices unreached
    eng = gpu.Engine(g, budget_bytes=int(8e9))
    for mode in MODES:
        vals, st = eng.run("bfs", mode, 0)
        assert np.array_equal(vals, ref), (mode, int(np.count_nonzero(vals != ref)))
        assert st["reached_edges"] > 2 ** 32
    eng.set_policy("learned")
    vals, _ = eng.run("bfs", "async", 0)
    assert np.array_equal(vals, ref)
    eng.close()
    g.close()

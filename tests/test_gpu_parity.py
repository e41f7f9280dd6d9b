"""Parity of the CUDA engine against the CPU oracle (bit-exact for the
integer algorithms), through the C ABI, on seeded graphs small enough for the
serial oracle, across budgets that force one or hundreds of partitions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALGS = ["bfs", "sssp", "sswp", "cc"]
MODES = ["sync", "async"]


def _graph(native, scale, weighted, seed=11, ef=16):
    return native.Graph.rmat(scale, ef, seed=seed, weighted=weighted, wmax=64)


def _oracle(orc, g, algo, src):
    e = g.edges
    if algo in ("bfs", "cc") and g.weighted:
        e = np.ascontiguousarray(e[:, 0])
    return orc.run(algo, g.node_pointer, e, src)


@pytest.fixture(scope="module")
def g12w(gpu):
    return _graph(gpu, 12, True)


@pytest.fixture(scope="module")
def g12u(gpu):
    return _graph(gpu, 12, False)


@pytest.mark.parametrize("algo", ALGS)
@pytest.mark.parametrize("mode", MODES)
def test_in_memory_small(gpu, orc, g12w, g12u, algo, mode):
    g = g12w if algo in ("sssp", "sswp") else g12u
    eng = gpu.Engine(g)
    src = 0
    vals, st = eng.run(algo, mode, src)
    ref = _oracle(orc, g, algo, src)
    assert np.array_equal(vals, ref), f"{algo}-{mode}: {np.count_nonzero(vals != ref)} mismatches"
    assert st["global_iterations"] >= 1


@pytest.mark.parametrize("algo", ALGS)
@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("budget_edges", [64, 1000, 20000])
def test_out_of_budget(gpu, orc, g12w, algo, mode, budget_edges):
    """Budgets far below the graph: many partitions, hubs split over pieces."""
    g = g12w
    fixed = 18 * g.n + 72 * 1024
    eng = gpu.Engine(g, budget_bytes=fixed + budget_edges * 2 * 8 + 4096)
    cap = eng.max_partition_size()
    assert cap < g.m
    src = int(g.pick_sources(1, seed=3)[0])
    vals, st = eng.run(algo, mode, src)
    ref = _oracle(orc, g, algo, src)
    assert np.array_equal(vals, ref), f"{algo}-{mode} cap={cap}: {np.count_nonzero(vals != ref)} mismatches"
    assert eng.device_bytes() <= fixed + budget_edges * 2 * 8 + 4096
    assert st["partitions"] >= st["global_iterations"]


@pytest.mark.parametrize("mode", MODES)
def test_config1_rmat16(gpu, orc, mode):
    """RMAT 2^16, edge factor 16, source 0, BFS and SSSP (w in [1,64])."""
    gw = _graph(gpu, 16, True, seed=1)
    gu = _graph(gpu, 16, False, seed=1)
    for algo, g in (("bfs", gu), ("sssp", gw)):
        eng = gpu.Engine(g)
        vals, _ = eng.run(algo, mode, 0)
        assert np.array_equal(vals, _oracle(orc, g, algo, 0)), f"{algo}-{mode}"


@pytest.mark.parametrize("algo", ["bfs", "sssp"])
def test_many_sources_er(gpu, orc, algo):
    g = gpu.Graph.er(5000, 60000, seed=9, weighted=(algo == "sssp"))
    eng = gpu.Engine(g, budget_bytes=18 * g.n + 72 * 1024 + 3000 * 16)
    for src in g.pick_sources(4, seed=2):
        for mode in MODES:
            vals, _ = eng.run(algo, mode, int(src))
            assert np.array_equal(vals, _oracle(orc, g, algo, int(src))), (algo, mode, src)


def test_generate_matches_reference_compaction(gpu, orc, g12u):
    """The first sync generate from a CC start (all vertices active) equals
    the reference's compaction restricted to vertices with out-edges."""
    g = g12u
    eng = gpu.Engine(g)
    eng.state_init("cc", "sync")
    nodes, ptr = eng.read_active()
    deg = g.out_degree()
    q, p = orc.generate(np.zeros(g.n, np.uint8), np.ones(g.n, np.uint8), deg)
    keep = deg[q] > 0
    assert np.array_equal(nodes, q[keep])
    assert np.array_equal(ptr[:-1], p[:-1][keep])
    assert ptr[-1] == p[-1]


def test_generate_many_tiles_ragged(gpu, orc):
    """Over a thousand 4096-vertex tiles (each thread of the tile scan takes
    several) and a partial last tile: the compaction of an all-active start
    equals the reference's, and BFS/SSSP equal the oracle under a budget that
    forces many partitions."""
    g = gpu.Graph.er(5_000_011, 20_000_000, seed=17, weighted=True, wmax=64)
    eng = gpu.Engine(g, budget_bytes=18 * g.n + 4 * 1024 * 1024 + (1 << 22) * 4)
    eng.state_init("cc", "sync")
    nodes, ptr = eng.read_active()
    deg = g.out_degree()
    q, p = orc.generate(np.zeros(g.n, np.uint8), np.ones(g.n, np.uint8), deg)
    keep = deg[q] > 0
    assert np.array_equal(nodes, q[keep])
    assert np.array_equal(ptr[:-1], p[:-1][keep])
    assert ptr[-1] == p[-1]
    src = int(g.pick_sources(1, seed=4)[0])
    for algo in ("bfs", "sssp"):
        e = g.edges if algo == "sssp" else np.ascontiguousarray(g.edges[:, 0])
        ref = orc.run(algo, g.node_pointer, e, src, parallel=True)
        for mode in MODES:
            vals, st = eng.run(algo, mode, src)
            assert np.array_equal(vals, ref), (algo, mode)
            assert st["partitions"] > st["global_iterations"]
    eng.close()


def test_engine_on_mapped_graph(gpu, orc, tmp_path):
    """A .bwcsr / .bcsr file mapped in place (edges in the page cache) runs
    like a loaded one."""
    for weighted in (True, False):
        g = _graph(gpu, 14, weighted, seed=23)
        p = tmp_path / ("g.bwcsr" if weighted else "g.bcsr")
        g.save(p)
        h = gpu.Graph.map(p)
        eng = gpu.Engine(h, budget_bytes=18 * h.n + 96 * 1024 + 20000 * 8)
        src = int(g.pick_sources(1, seed=2)[0])
        for algo in ("bfs", "sssp") if weighted else ("bfs", "cc"):
            for mode in MODES:
                vals, _ = eng.run(algo, mode, src)
                assert np.array_equal(vals, _oracle(orc, g, algo, src)), (weighted, algo, mode)
        eng.close()
        h.close()


def test_step_api_loop(gpu, orc, g12w):
    """The reference's app loop written against the step API."""
    g = g12w
    eng = gpu.Engine(g, budget_bytes=18 * g.n + 72 * 1024 + 5000 * 16)
    eng.state_init("sssp", "async", 0)
    iters = 0
    while True:
        parts = eng.partition()
        if not parts:
            break
        iters += 1
        for i in range(len(parts)):
            assert eng.process_partition(i) >= 1
        a, _ = eng.generate()
        if a == 0:
            break
    vals = eng.read_values()
    assert np.array_equal(vals, _oracle(orc, g, "sssp", 0))
    assert iters >= 1


def test_hub_larger_than_budget(gpu, orc):
    """A vertex whose out-degree exceeds the edge buffer (the reference's
    partitioner never terminates here) is streamed in pieces."""
    n = 3000
    rng = np.random.default_rng(5)
    src = np.concatenate([np.zeros(2500, np.int64), rng.integers(0, n, 4000)])
    dst = np.concatenate([np.arange(1, 2501), rng.integers(0, n, 4000)])
    keep = (src != dst) & (src != n - 2)
    src, dst = src[keep], dst[keep]
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    pairs = np.unique(np.stack([src, dst], 1), axis=0)
    src, dst = pairs[:, 0], pairs[:, 1]
    npt = np.zeros(n + 1, np.uint32)
    np.add.at(npt, src + 1, 1)
    npt = np.cumsum(npt).astype(np.uint32)
    w = (1 + (src * 7 + dst * 13) % 50).astype(np.uint32)
    edges = np.stack([dst.astype(np.uint32), w], 1)
    g = gpu.Graph.from_csr(npt, edges, True)
    eng = gpu.Engine(g, budget_bytes=18 * n + 15 * 1024 + 1000 * 16)
    assert eng.max_partition_size() < 2500
    for algo in ("bfs", "sssp", "sswp", "cc"):
        for mode in MODES:
            vals, _ = eng.run(algo, mode, 0)
            ref = _oracle(orc, g, algo, 0)
            assert np.array_equal(vals, ref), (algo, mode)


@pytest.mark.parametrize("flags", ["", "NO_PACK", "SPLIT_WEIGHTS", "SCALAR_GATHER", "NO_PACK|SCALAR_GATHER",
                                   "PAGEABLE_COPY", "SPLIT_WEIGHTS|PAGEABLE_COPY", "NO_PACK|PAGEABLE_COPY"])
def test_transfer_copy_in_small_chunks(gpu, orc, flags):
    """The host transfer copy cut into dozens of 16 KiB chunks (4 KiB for the
    hub graph), pinned or (PAGEABLE_COPY) ordinary pages: rows and 16-byte
    words of the gather, whole-range copies of the learned schedule and the
    pieces of a vertex larger than the edge buffer (copy kernel from
    pageable pages, at 4-byte and byte offsets) all cross chunk boundaries,
    in every transfer form, and give the oracle's answers."""
    fl = 0
    for f in filter(None, flags.split("|")):
        fl |= getattr(gpu, "OPT_" + f)
    g = gpu.Graph.rmat(14, 16, seed=12, weighted=True, wmax=64)
    budget = 18 * g.n + 128 * 1024 + (g.m // 6) * 8 * 3
    plain = gpu.Engine(g, budget_bytes=budget, flags=fl, transfer_chunk_log2=14)
    learned = gpu.Engine(g, budget_bytes=budget, flags=fl, transfer_chunk_log2=14, num_buffers=3)
    learned.set_policy("learned")
    assert plain.max_partition_size() < g.m
    src = int(g.pick_sources(1, seed=3)[0])
    for algo in ("bfs", "sssp"):
        ref = _oracle(orc, g, algo, src)
        for mode in MODES:
            for eng in (plain, learned):
                vals, _ = eng.run(algo, mode, src)
                assert np.array_equal(vals, ref), (algo, mode)
    # a hub above the buffer, streamed in pieces that cross 4 KiB chunks
    n = 3000
    rng = np.random.default_rng(7)
    hs = np.concatenate([np.zeros(2500, np.int64), rng.integers(0, n, 4000)])
    hd = np.concatenate([np.arange(1, 2501), rng.integers(0, n, 4000)])
    keep = (hs != hd) & (hs != n - 2)
    pairs = np.unique(np.stack([hs[keep], hd[keep]], 1), axis=0)
    npt = np.zeros(n + 1, np.uint32)
    np.add.at(npt, pairs[:, 0] + 1, 1)
    npt = np.cumsum(npt).astype(np.uint32)
    w = (1 + (pairs[:, 0] * 7 + pairs[:, 1] * 13) % 50).astype(np.uint32)
    hg = gpu.Graph.from_csr(npt, np.stack([pairs[:, 1].astype(np.uint32), w], 1), True)
    heng = None
    for extra in range(0, 64 * 1024, 1024):  # the smallest budget this transfer form fits
        try:
            heng = gpu.Engine(hg, budget_bytes=18 * n + 13 * 1024 + 1000 * 16 + extra, flags=fl,
                              transfer_chunk_log2=12)
            break
        except gpu.SgwError:
            continue
    assert heng is not None and heng.max_partition_size() < 2500
    for algo in ("bfs", "sssp"):
        vals, _ = heng.run(algo, "async", 0)
        assert np.array_equal(vals, _oracle(orc, hg, algo, 0)), algo


# ---- PageRank ------------------------------------------------------------------
PR_INIT, PR_ACC, PR_DAMP = (float(np.float32(x)) for x in (0.15, 0.01, 0.85))


def _pr_engine_values(gpu, eng):
    import ctypes as C
    out = np.empty(eng.graph.n, np.float64)
    gpu.check(gpu.lib().sgw_read_values_f64(eng.h, out.ctypes.data), "sgw_read_values_f64")
    return out


@pytest.mark.parametrize("budget_edges", [None, 300, 5000])
def test_pagerank_sync_matches_bsp_oracle(gpu, orc, g12u, budget_edges):
    """Sync PR is the bulk-synchronous delta schedule: FP64 ranks agree with
    the FP64 oracle to 1e-9 (max-abs); the FP32 output is their cast."""
    g = g12u
    kw = {} if budget_edges is None else {"budget_bytes": 36 * g.n + 96 * 1024 + budget_edges * 8}
    eng = gpu.Engine(g, **kw)
    vals, st = eng.run("pr", "sync")
    ref, rounds = orc.pagerank(g.node_pointer, g.edges, init=PR_INIT, acc=PR_ACC, damping=PR_DAMP)
    f64 = _pr_engine_values(gpu, eng)
    assert np.max(np.abs(f64 - ref)) <= 1e-9
    assert np.array_equal(vals, ref.astype(np.float32)) or np.max(np.abs(vals - ref) / np.maximum(ref, 1e-30)) < 2.5e-7
    assert st["global_iterations"] == rounds


@pytest.mark.parametrize("budget_edges", [None, 2000])
def test_pagerank_async_within_residual_bound(gpu, orc, g12u, budget_edges):
    """Async PR stops with every residual <= acc, so each rank is within
    (acc / init) x its exact value of the fixpoint."""
    g = g12u
    kw = {} if budget_edges is None else {"budget_bytes": 36 * g.n + 96 * 1024 + budget_edges * 8}
    eng = gpu.Engine(g, **kw)
    eng.run("pr", "async")
    f64 = _pr_engine_values(gpu, eng)
    exact, _ = orc.pagerank(g.node_pointer, g.edges, init=PR_INIT, acc=1e-14, damping=PR_DAMP)
    assert np.all(np.abs(f64 - exact) <= (PR_ACC / PR_INIT) * exact + 1e-9)
    assert np.all(f64 <= exact + 1e-9), "delta-PR only adds mass: ranks approach the fixpoint from below"


def test_pagerank_tight_tolerance(gpu, orc):
    """With acc = 1e-6 the FP64 ranks are within 1e-6 (max-abs) of the FP64
    oracle's exact fixpoint on an ER graph."""
    g = gpu.Graph.er(3000, 30000, seed=4)
    eng = gpu.Engine(g)
    acc = float(np.float32(1e-6))
    eng.run("pr", "sync", pr_acc=acc)
    f64 = _pr_engine_values(gpu, eng)
    ref, _ = orc.pagerank(g.node_pointer, g.edges, init=PR_INIT, acc=acc, damping=PR_DAMP)
    assert np.max(np.abs(f64 - ref)) <= 1e-9
    exact, _ = orc.pagerank(g.node_pointer, g.edges, init=PR_INIT, acc=1e-15, damping=PR_DAMP)
    assert np.max(np.abs(f64 - exact)) <= 1e-4


def test_engine_matches_reference_golden(gpu):
    """The engine against the reference build's own outputs (tests/golden)."""
    from pathlib import Path
    d = np.load(Path(__file__).resolve().parent / "golden" / "ref_rmat13.npz")
    scale, ef, seed, wmax = (int(x) for x in d["params"][:4])
    gu = gpu.Graph.rmat(scale, ef, seed=seed)
    gw = gpu.Graph.rmat(scale, ef, seed=seed, weighted=True, wmax=wmax)
    engines = {False: gpu.Engine(gu, budget_bytes=36 * gu.n + 96 * 1024 + 20000 * 8),
               True: gpu.Engine(gw, budget_bytes=36 * gw.n + 96 * 1024 + 20000 * 16)}
    for k in d.keys():
        if not k.startswith("fixed/"):
            continue
        _, app, *s = k.split("/")
        algo, mode = app.split("-")
        eng = engines[algo in ("sssp", "sswp")]
        src = int(s[0][1:]) if s else 0
        vals, _ = eng.run(algo, mode, src)
        if algo == "pr":
            ref = d[k].astype(np.float64)
            if mode == "sync":
                assert np.max(np.abs(vals - ref) / ref) < 1e-5, k
            else:
                assert np.max(np.abs(vals - ref) / ref) < PR_ACC / PR_INIT, k
        else:
            assert np.array_equal(vals, d[k]), k


def test_engine_matches_reference_rmat16(gpu):
    """BFS-sync and SSSP-sync from source 0 on R-MAT scale 16, whole graph on
    the device: bit-exact against the fixed reference build's outputs."""
    from pathlib import Path
    d = np.load(Path(__file__).resolve().parent / "golden" / "ref_rmat16.npz")
    scale, ef, seed, wmax = (int(x) for x in d["params"][:4])
    gu = gpu.Graph.rmat(scale, ef, seed=seed)
    gw = gpu.Graph.rmat(scale, ef, seed=seed, weighted=True, wmax=wmax)
    for algo, g in (("bfs", gu), ("sssp", gw)):
        vals, _ = gpu.Engine(g).run(algo, "sync", 0)
        assert np.array_equal(vals, d[f"fixed/{algo}-sync/s0"]), algo


@pytest.mark.parametrize("policy", ["plain", "learned"])
def test_engine_matches_reference_rmat24_digests(gpu, policy):
    """SSSP-async on R-MAT scale 24 under a 1 GB budget (the smaller benchmark
    workload), 8 sources: each distance array hashes to the fixed reference
    build's digest."""
    import hashlib
    import json
    from pathlib import Path
    rep = json.loads((Path(__file__).resolve().parent / "golden" / "ref_rmat24_sssp_async_1gb.json").read_text())
    g = gpu.Graph.rmat(24, 16, seed=24, weighted=True, wmax=64)
    assert g.pick_sources(8, seed=24).tolist() == rep["sources"]
    nb = gpu.sched_buffers(g, 1e9) if policy == "learned" else 0
    eng = gpu.Engine(g, budget_bytes=1_000_000_000, num_buffers=nb)
    if policy == "learned":
        from subway_gb300 import scheduler
        eng.set_policy("learned", scheduler.load_default(0))
    for s in rep["sources"]:
        vals, _ = eng.run("sssp", "async", s)
        assert hashlib.sha256(vals.tobytes()).hexdigest() == rep["runs"][f"fixed/sssp-async/s{s}"]["sha256"], s


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("flags", ["NO_PACK", "SCALAR_GATHER", "NO_PACK|SCALAR_GATHER", "CTA_TILES",
                                   "NO_PACK|CTA_TILES", "SPLIT_WEIGHTS", "SPLIT_WEIGHTS|CTA_TILES"])
def test_transfer_forms(gpu, orc, g12w, mode, flags):
    """8-byte records (SGW_OPT_NO_PACK), the one-record-per-thread gather
    (SGW_OPT_SCALAR_GATHER) and CTA-tile expansion (SGW_OPT_CTA_TILES) give
    the same answers as the defaults."""
    g = g12w
    f = 0
    for name in flags.split("|"):
        f |= getattr(gpu, "OPT_" + name)
    eng = gpu.Engine(g, budget_bytes=18 * g.n + 72 * 1024 + 3000 * 16, flags=f)
    src = int(g.pick_sources(1, seed=9)[0])
    for algo in ALGS:
        vals, _ = eng.run(algo, mode, src)
        assert np.array_equal(vals, _oracle(orc, g, algo, src)), (algo, mode)


def test_async_inner_cap(gpu, orc, g12w):
    """Async runs with the inner iterations of each partition visit capped
    (the labels left over go to the next generate) give the oracle's answers."""
    g = g12w
    eng = gpu.Engine(g, budget_bytes=18 * g.n + 72 * 1024 + 3000 * 16)
    src = int(g.pick_sources(1, seed=21)[0])
    for algo in ALGS:
        for mi in (1, 3):
            vals, st = eng.run(algo, "async", src, max_inner=mi)
            assert np.array_equal(vals, _oracle(orc, g, algo, src)), (algo, mi)
            assert st["partitions"] >= st["global_iterations"] > 0
            assert st["inner_iterations"] <= mi * st["partitions"], (algo, mi)


@pytest.mark.parametrize("mode", MODES)
def test_split_weights_bytes_and_answers(gpu, orc, g12w, mode):
    """The split form moves 4 bytes per edge for BFS/CC and 5 for SSSP/SSWP
    (destination word + weight byte), under plain and learned schedules,
    with hub vertices streamed in pieces, and answers like the oracle."""
    g = g12w
    budget = 18 * g.n + 72 * 1024 + 1500 * 20
    for policy in ("plain", "learned"):
        eng = gpu.Engine(g, budget_bytes=budget, flags=gpu.OPT_SPLIT_WEIGHTS,
                         num_buffers=3 if policy == "learned" else 0)
        if policy == "learned":
            eng.set_policy("learned")
        src = int(g.pick_sources(1, seed=4)[0])
        for algo in ALGS:
            vals, st = eng.run(algo, mode, src)
            assert np.array_equal(vals, _oracle(orc, g, algo, src)), (algo, mode, policy)
            per_edge = 5 if algo in ("sssp", "sswp") else 4
            assert st["h2d_bytes"] % per_edge == 0, (algo, st["h2d_bytes"])


def test_wide_weights_fall_back_to_full_records(gpu, orc):
    """Weights that do not fit beside the vertex id keep 8-byte records."""
    g0 = gpu.Graph.rmat(12, 8, seed=13, weighted=True)
    e = np.array(g0.edges)
    e[:, 1] = (e[:, 1].astype(np.uint64) * 40503 % (1 << 22) + 1).astype(np.uint32)  # 22-bit weights
    g = gpu.Graph.from_csr(np.array(g0.node_pointer), e, True)
    eng = gpu.Engine(g, budget_bytes=18 * g.n + 72 * 1024 + 2000 * 16)
    for algo in ("sssp", "sswp"):
        for mode in MODES:
            vals, st = eng.run(algo, mode, 0)
            assert np.array_equal(vals, _oracle(orc, g, algo, 0)), (algo, mode)
    assert st["h2d_bytes"] % 8 == 0


@pytest.mark.parametrize("n", [1, 5, 17, 4097, 8191])
def test_odd_vertex_counts(gpu, orc, n):
    """Vertex counts that are not multiples of 16 or of the 4096-vertex scan
    tile (partial lane groups and tiles in the generate step), a single
    vertex, and a vertex count below one lane's 16: every algorithm, both
    modes, plain and learned schedules, bit-exact."""
    rng = np.random.default_rng(n)
    m0 = 6 * n
    src = rng.integers(0, n, m0)
    dst = rng.integers(0, n, m0)
    keep = src != dst
    pairs = np.unique(np.stack([src[keep], dst[keep]], 1), axis=0) if keep.any() else np.zeros((0, 2), np.int64)
    npt = np.zeros(n + 1, np.uint32)
    np.add.at(npt, pairs[:, 0] + 1, 1)
    npt = np.cumsum(npt).astype(np.uint32)
    w = (1 + (pairs[:, 0] * 5 + pairs[:, 1] * 3) % 60).astype(np.uint32)
    edges = np.stack([pairs[:, 1].astype(np.uint32), w], 1)
    g = gpu.Graph.from_csr(npt, edges, True)
    budget = 18 * n + 96 * 1024 + max(64, g.m // 3) * 8 * 3
    s0 = int(np.argmax(np.diff(npt))) if g.m else 0
    for policy in ("plain", "learned"):
        eng = gpu.Engine(g, budget_bytes=budget, num_buffers=3 if policy == "learned" else 0)
        if policy == "learned":
            eng.set_policy("learned")
        for algo in ALGS:
            for mode in MODES:
                vals, _ = eng.run(algo, mode, s0)
                assert np.array_equal(vals, _oracle(orc, g, algo, s0)), (n, policy, algo, mode)


@pytest.mark.parametrize("weighted", [False, True])
def test_graph_read_in_place(gpu, orc, tmp_path, weighted):
    """SGW_OPT_GRAPH_IN_PLACE: on records the library holds (generated or
    loaded) the engine makes no transfer copy and gathers, streams and
    copies hub pieces from the records themselves through the host page
    tables; a caller's arrays still get a (pageable) copy.  Every answer is
    the oracle's, plain and learned, with hubs larger than the buffer."""
    fl = gpu.OPT_GRAPH_IN_PLACE | gpu.OPT_PAGEABLE_COPY
    g = gpu.Graph.rmat(14, 16, seed=12, weighted=weighted, wmax=64)
    ext = "bwcsr" if weighted else "bcsr"
    g.save(tmp_path / f"g.{ext}")
    loaded = gpu.Graph.load(tmp_path / f"g.{ext}")
    budget = 18 * g.n + 128 * 1024 + (g.m // 6) * 8 * 3
    src = int(g.pick_sources(1, seed=3)[0])
    algos = ("bfs", "sssp", "sswp", "cc") if weighted else ("bfs", "cc")
    for graph in (g, loaded):
        plain = gpu.Engine(graph, budget_bytes=budget, flags=fl)
        learned = gpu.Engine(graph, budget_bytes=budget, flags=fl, num_buffers=3)
        learned.set_policy("learned")
        assert plain.host_copy_bytes() == 0 and learned.host_copy_bytes() == 0
        assert plain.max_partition_size() < graph.m
        for algo in algos:
            ref = _oracle(orc, graph, algo, src)
            for mode in MODES:
                for eng in (plain, learned):
                    vals, _ = eng.run(algo, mode, src)
                    assert np.array_equal(vals, ref), (algo, mode)
        plain.close()
        learned.close()
    caller = gpu.Graph.from_csr(np.array(g.node_pointer), np.array(g.edges), weighted)
    e = gpu.Engine(caller, budget_bytes=budget, flags=fl)
    assert e.host_copy_bytes() > 0
    vals, _ = e.run("bfs", "async", src)
    assert np.array_equal(vals, _oracle(orc, caller, "bfs", src))
    e.close()
    # a vertex above the edge buffer, streamed in pieces from the records
    n = 3000
    rng = np.random.default_rng(9)
    hs = np.concatenate([np.zeros(2500, np.int64), rng.integers(0, n, 4000)])
    hd = np.concatenate([np.arange(1, 2501), rng.integers(0, n, 4000)])
    keep = (hs != hd) & (hs != n - 2)
    pairs = np.unique(np.stack([hs[keep], hd[keep]], 1), axis=0)
    npt = np.zeros(n + 1, np.uint32)
    np.add.at(npt, pairs[:, 0] + 1, 1)
    npt = np.cumsum(npt).astype(np.uint32)
    w = (1 + (pairs[:, 0] * 7 + pairs[:, 1] * 13) % 50).astype(np.uint32)
    hub = gpu.Graph.from_csr(npt, np.stack([pairs[:, 1].astype(np.uint32), w], 1), True)
    hub.save(tmp_path / "hub.bwcsr")
    hub = gpu.Graph.load(tmp_path / "hub.bwcsr")
    heng = None
    for extra in range(0, 64 * 1024, 1024):  # the smallest budget the 8-byte records fit
        try:
            heng = gpu.Engine(hub, budget_bytes=18 * n + 13 * 1024 + 1000 * 16 + extra, flags=fl)
            break
        except gpu.SgwError:
            continue
    assert heng is not None and heng.host_copy_bytes() == 0 and heng.max_partition_size() < 2500
    for algo in ("bfs", "sssp", "sswp", "cc"):
        for mode in MODES:
            vals, _ = heng.run(algo, mode, 0)
            assert np.array_equal(vals, _oracle(orc, hub, algo, 0)), (algo, mode)
    heng.close()

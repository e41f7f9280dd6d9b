"""The CPU oracle: known answers, agreement of its serial and parallel
forms, and its restatement of the reference's generate/partition steps."""
import numpy as np
import pytest

INF = 4294967294

# README.md example graph (0 1 26, 0 3 33, 2 3 40, 1 2 10) as CSR
R_NP = np.array([0, 2, 3, 4, 4], np.uint32)
R_ED = np.array([[1, 26], [3, 33], [2, 10], [3, 40]], np.uint32)


def test_readme_known_answers(orc):
    assert orc.run("bfs", R_NP, R_ED[:, 0].copy(), 0).tolist() == [0, 1, 2, 1]
    assert orc.run("sssp", R_NP, R_ED, 0).tolist() == [0, 26, 36, 33]
    assert orc.run("sswp", R_NP, R_ED, 0).tolist() == [INF, 26, 10, 33]
    assert orc.run("cc", R_NP, R_ED, 0).tolist() == [0, 0, 0, 0]
    assert orc.run("bfs", R_NP, R_ED, 2).tolist() == [INF, INF, 0, 1]
    assert orc.run("sswp", R_NP, R_ED, 3).tolist() == [0, 0, 0, INF]
    assert orc.run("cc", R_NP, R_ED, 0).tolist() == orc.run("cc", R_NP, R_ED, 0, parallel=True).tolist()


def test_chain_and_isolated(orc):
    n = 50
    npt = np.concatenate([np.arange(n, dtype=np.uint32), [n - 1]]).astype(np.uint32)  # i -> i+1
    ed = np.stack([np.arange(1, n, dtype=np.uint32), np.full(n - 1, 3, np.uint32)], 1)
    assert orc.run("bfs", npt, ed, 0).tolist() == list(range(n))
    assert orc.run("sssp", npt, ed, 0).tolist() == [3 * i for i in range(n)]
    assert orc.run("sswp", npt, ed, 0).tolist() == [INF] + [3] * (n - 1)
    assert orc.run("bfs", npt, ed, n - 1).tolist() == [INF] * (n - 1) + [0]
    # CC along out-edges only: every vertex is reached by 0
    assert orc.run("cc", npt, ed, 0).tolist() == [0] * n


@pytest.mark.parametrize("algo", ["bfs", "sssp", "sswp", "cc"])
def test_serial_equals_parallel(native, orc, algo):
    g = native.Graph.rmat(14, 16, seed=8, weighted=True)
    for src in g.pick_sources(3, seed=2):
        a = orc.run(algo, g.node_pointer, g.edges, int(src))
        b = orc.run(algo, g.node_pointer, g.edges, int(src), parallel=True)
        assert np.array_equal(a, b)


def test_certificates(native, orc):
    """Exact answers satisfy the optimality certificates used at full size."""
    g = native.Graph.rmat(13, 16, seed=3, weighted=True)
    npt, e = g.node_pointer, g.edges
    src = np.repeat(np.arange(g.n, dtype=np.int64), np.diff(npt))
    d = orc.run("sssp", npt, e, 0).astype(np.int64)
    ok = d[src] != INF
    assert np.all(d[e[ok, 0]] <= d[src[ok]] + e[ok, 1])
    tight = np.zeros(g.n, bool)
    tight[e[ok, 0][d[e[ok, 0]] == d[src[ok]] + e[ok, 1]]] = True
    reached = (d != INF)
    reached[0] = False
    assert np.all(tight[reached])


def test_pagerank_against_linear_solve(orc):
    rng = np.random.default_rng(1)
    n = 60
    src = rng.integers(0, n, 300)
    dst = rng.integers(0, n, 300)
    keep = src != dst
    pairs = np.unique(np.stack([src[keep], dst[keep]], 1), axis=0)
    npt = np.zeros(n + 1, np.int64)
    np.add.at(npt, pairs[:, 0] + 1, 1)
    npt = np.cumsum(npt).astype(np.uint32)
    ed = pairs[:, 1].astype(np.uint32)
    val, rounds = orc.pagerank(npt, ed, acc=1e-13)
    # fixpoint: x = 0.15 + 0.85 * A^T D^-1 x (dangling mass dropped)
    deg = np.diff(npt.astype(np.int64))
    M = np.zeros((n, n))
    for u, v in pairs:
        M[v, u] += 0.85 / deg[u]
    x = np.linalg.solve(np.eye(n) - M, np.full(n, 0.15))
    assert rounds > 10
    assert np.max(np.abs(val - x)) < 1e-10
    v2, _ = orc.pagerank(npt, ed, acc=1e-13, parallel=True)
    assert np.max(np.abs(v2 - x)) < 1e-10


def test_generate_restatement(orc):
    rng = np.random.default_rng(2)
    n = 1000
    l1 = (rng.random(n) < 0.1).astype(np.uint8)
    l2 = (rng.random(n) < 0.1).astype(np.uint8)
    deg = rng.integers(0, 20, n).astype(np.uint32)
    q, p = orc.generate(l1, l2, deg)
    act = np.flatnonzero(l1 | l2)
    assert np.array_equal(q, act)
    assert np.array_equal(p[:-1], np.concatenate([[0], np.cumsum(deg[act])[:-1]]))
    assert p[-1] == deg[act].sum()


def test_partition_restatement(orc):
    ptr = np.array([0, 5, 10, 12, 30, 31], np.uint32)
    fr, sz = orc.partition(ptr, 18)
    assert fr.tolist() == [0, 3, 4] and sz.tolist() == [3, 1, 1]
    assert orc.partition(ptr, 12) is None  # vertex 3 has 18 > 10 edges: the reference never ends
    fr, sz = orc.partition(ptr, 100)
    assert fr.tolist() == [0] and sz.tolist() == [5]


@pytest.mark.parametrize("scale,weighted,seed", [(10, True, 3), (13, False, 5), (15, True, 24)])
def test_rmat_writer_matches_engine_generator(native, orc, tmp_path, scale, weighted, seed):
    """The oracle's R-MAT file (the reference arm's input, made without the
    engine library) has the same bytes as the engine generator's saved graph,
    and its source choice is the same."""
    ext = "bwcsr" if weighted else "bcsr"
    g = native.Graph.rmat(scale, 16, seed=seed, weighted=weighted, wmax=64)
    g.save(tmp_path / f"eng.{ext}")
    m = orc.rmat_write(tmp_path / f"orc.{ext}", scale, 16, seed=seed, weighted=weighted, wmax=64)
    assert m == g.m
    assert (tmp_path / f"eng.{ext}").read_bytes() == (tmp_path / f"orc.{ext}").read_bytes()
    npt, ed = orc.read_csr(tmp_path / f"orc.{ext}")
    assert np.array_equal(npt, g.node_pointer)
    src = orc.pick_sources(npt, ed, 16, seed=seed)
    assert src.tolist() == g.pick_sources(16, seed=seed).tolist()


def test_delta_stepping_equals_dijkstra_and_frontier(native, orc):
    """omp_sssp (delta-stepping) against serial Dijkstra and the bucket-free
    frontier method, on R-MAT and on a graph with heavy weights."""
    for g in (native.Graph.rmat(15, 16, seed=11, weighted=True, wmax=64),
              native.Graph.er(20000, 200000, seed=3, weighted=True, wmax=100000)):
        for s in g.pick_sources(4, seed=9):
            ref = orc.run("sssp", g.node_pointer, g.edges, int(s))
            assert np.array_equal(orc.run("sssp", g.node_pointer, g.edges, int(s), parallel=True), ref)
            assert np.array_equal(orc.sssp_frontier(g.node_pointer, g.edges, int(s)), ref)


def test_reached_edges_multi_source(native, orc):
    """The bit-parallel reachability count equals one BFS per source (70
    sources: two calls of 64 and 6), including repeated sources."""
    g = native.Graph.rmat(13, 8, seed=4, weighted=False)
    src = np.concatenate([g.pick_sources(68, seed=1), [0, 0]]).astype(np.uint32)
    deg = g.out_degree().astype(np.uint64)
    want = [int(deg[orc.run("bfs", g.node_pointer, g.ends, int(s)) != INF].sum()) for s in src]
    assert orc.reached_edges(g.node_pointer, g.ends, src).tolist() == want
    gw = native.Graph.rmat(12, 16, seed=4, weighted=True)
    s2 = gw.pick_sources(5, seed=3)
    want2 = [int(gw.out_degree()[orc.run("bfs", gw.node_pointer, gw.edges, int(s)) != INF].astype(np.uint64).sum())
             for s in s2]
    assert orc.reached_edges(gw.node_pointer, gw.edges, s2).tolist() == want2

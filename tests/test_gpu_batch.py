"""Batched multi-source queries: every lane's answer equals the single-source
answer (oracle and engine), for 1..64 lanes, BFS and SSSP."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gw(gpu):
    return gpu.Graph.rmat(13, 16, seed=41, weighted=True)


@pytest.mark.parametrize("lanes", [32, 64])
@pytest.mark.parametrize("algo", ["bfs", "sssp"])
def test_batch_matches_oracle(gpu, orc, gw, lanes, algo):
    b = gpu.Batch(gw, lanes=lanes)
    rng = np.random.default_rng(lanes)
    for nsrc in (1, 7, lanes):
        src = rng.integers(0, gw.n, nsrc).astype(np.uint32)
        out, st = b.run(algo, src)
        e = gw.edges if algo == "sssp" else gw.ends
        for i, s in enumerate(src):
            assert np.array_equal(out[i], orc.run(algo, gw.node_pointer, e, int(s))), (algo, nsrc, i)
        assert st["queries"] == nsrc and st["iterations"] >= 1


def test_batch_matches_engine_and_repeats(gpu, gw):
    b = gpu.Batch(gw, lanes=64, chunk_edges=64)
    eng = gpu.Engine(gw)
    src = gw.pick_sources(64, seed=3)
    out1, _ = b.run("sssp", src)
    out2, _ = b.run("sssp", src[::-1].copy())
    for i in (0, 17, 63):
        v, _ = eng.run("sssp", "async", int(src[i]))
        assert np.array_equal(out1[i], v)
        assert np.array_equal(out2[63 - i], v)


def test_batch_admission_and_arguments(gpu, gw):
    with pytest.raises(gpu.SgwError) as e:
        gpu.Batch(gw, lanes=64, budget_bytes=1 << 20)
    assert e.value.status == -5  # SGW_EBUDGET
    b = gpu.Batch(gw, lanes=32)
    with pytest.raises(gpu.SgwError):
        b.run("bfs", np.arange(33, dtype=np.uint32))
    with pytest.raises(gpu.SgwError):
        b.run("cc", np.arange(3, dtype=np.uint32))
    gu = gpu.Graph.rmat(10, 8, seed=2)
    with pytest.raises(gpu.SgwError):
        gpu.Batch(gu, lanes=32).run("sssp", np.arange(3, dtype=np.uint32))


def test_batch_pinned_results_view(gpu, orc, gw):
    b = gpu.Batch(gw, lanes=32)
    src = np.array([3, 5, 8], np.uint32)
    view, _ = b.run("bfs", src, view=True)
    assert not view.flags.writeable and view.shape == (3, gw.n)
    for i, s in enumerate(src):
        assert np.array_equal(view[i], orc.run("bfs", gw.node_pointer, gw.ends, int(s)))


@pytest.mark.parametrize("lanes", [32, 64])
@pytest.mark.parametrize("algo", ["bfs", "sssp"])
def test_persistent_batch_matches_graph_loop(gpu, orc, gw, lanes, algo):
    """The persistent form (one cooperative launch, grid barriers) gives every
    lane the oracle's answer and runs as many iterations as the graph loop."""
    pb = gpu.Batch(gw, lanes=lanes, flags=gpu.OPT_BATCH_PERSISTENT)
    gb = gpu.Batch(gw, lanes=lanes, flags=gpu.OPT_BATCH_GRAPH)
    rng = np.random.default_rng(lanes + 7)
    e = gw.edges if algo == "sssp" else gw.ends
    for nsrc in (1, 5, lanes):
        src = rng.integers(0, gw.n, nsrc).astype(np.uint32)
        out, st = pb.run(algo, src)
        ref, st_g = gb.run(algo, src)
        assert np.array_equal(out, ref), (algo, nsrc)
        assert st["iterations"] == st_g["iterations"]
        for i, s in enumerate(src[:3]):
            assert np.array_equal(out[i], orc.run(algo, gw.node_pointer, e, int(s))), (algo, nsrc, i)


def test_persistent_batch_wait_runs_out(gpu, orc, gw):
    """A grid barrier that cannot fill (it waits for one block more than the
    launch has) gives up after its limit: the run returns SGW_ETIMEOUT, the
    device stays usable and the next batch is exact."""
    b = gpu.Batch(gw, lanes=64, flags=gpu.OPT_BATCH_PERSISTENT)
    assert b.check_wait_timeout(2_000_000) == -7  # SGW_ETIMEOUT
    assert b"grid barrier" in gpu.lib().sgw_last_error()
    src = np.array([3, 11], np.uint32)
    out, _ = b.run("sssp", src)
    for i, s in enumerate(src):
        assert np.array_equal(out[i], orc.run("sssp", gw.node_pointer, gw.edges, int(s)))


@pytest.mark.parametrize("persistent", [False, True])
def test_batch_u16_answers(gpu, gw, persistent):
    """16-bit answers equal the 32-bit ones (unreached as 0xffff), copied out
    or left in the pinned buffer; a distance that does not fit is refused."""
    fl = gpu.OPT_BATCH_PERSISTENT if persistent else gpu.OPT_BATCH_GRAPH
    b = gpu.Batch(gw, lanes=64, flags=fl)
    src = np.random.default_rng(5).integers(0, gw.n, 40).astype(np.uint32)
    for algo in ("bfs", "sssp"):
        ref, _ = b.run(algo, src)
        want = np.where(ref == 4294967294, 0xFFFF, ref).astype(np.uint16)
        got, st = b.run(algo, src, answers="u16")
        assert np.array_equal(got, want) and st["d2h_bytes"] == 2 * gw.n * len(src)
        view, _ = b.run(algo, src, answers="u16", view=True)
        assert np.array_equal(view, want)
    # weights that push distances past 16 bits
    big = gpu.Graph.from_csr(np.array([0, 1, 2, 2], np.uint32),
                             np.array([[1, 40000], [2, 40000]], np.uint32), weighted=True)
    bb = gpu.Batch(big, lanes=32, flags=fl)
    with pytest.raises(gpu.SgwError):
        bb.run("sssp", np.array([0], np.uint32), answers="u16")
    ok, _ = bb.run("sssp", np.array([1], np.uint32), answers="u16")
    assert ok[0].tolist() == [0xFFFF, 0, 40000]

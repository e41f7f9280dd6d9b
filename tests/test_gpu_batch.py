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

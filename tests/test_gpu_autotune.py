"""The autotuner: a short greedy search on a small out-of-budget workload
returns settings from its search space, and the engine and batch objects
built with them give the oracle's answers bit-exact (the knobs shape the
kernels, never the results)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_engine_returns_exact_settings(gpu, orc):
    from subway_gb300 import autotune
    g = gpu.Graph.rmat(14, 16, seed=3, weighted=True, wmax=64)
    budget = 18 * g.n + 128 * 1024 + (g.m // 3) * 4  # vertex state, tables, two buffers of ~m/6 edges
    src = g.pick_sources(2, seed=5)
    best, best_ms, trials = autotune.tune_engine(g, budget, "sssp", "async", sources=src)
    space = autotune.ENGINE_SPACE
    assert all(best[k] in v for k, v in space.items())
    # one trial per candidate other than the current best (which may move)
    assert 1 + sum(len(v) - 1 for v in space.values()) <= len(trials) <= 1 + sum(len(v) for v in space.values())
    assert best_ms > 0 and best_ms <= min(ms for _, ms in trials) / 0.98 + 1e-9
    eng = gpu.Engine(g, budget_bytes=budget, **autotune.engine_opts(best))
    assert eng.max_partition_size() < g.m
    for s in src:
        vals, _ = eng.run("sssp", "async", int(s))
        assert np.array_equal(vals, orc.run("sssp", g.node_pointer, g.edges, int(s)))


def test_tune_batch_returns_exact_setting(gpu, orc):
    from subway_gb300 import autotune
    g = gpu.Graph.rmat(14, 16, seed=4)
    best, res = autotune.tune_batch(g, "bfs", lanes=64, candidates=(64, 256, 1024))
    assert best in (64, 256, 1024) and len(res) == 3
    b = gpu.Batch(g, lanes=64, chunk_edges=best)
    src = g.pick_sources(5, seed=6)
    out, _ = b.run("bfs", src)
    for i, s in enumerate(src):
        assert np.array_equal(out[i], orc.run("bfs", g.node_pointer, g.ends, int(s)))

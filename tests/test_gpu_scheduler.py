"""The learned scheduler: its network's kernels against an FP64 CPU
restatement, and the policy's results against the oracle (the schedule may
change, the answers may not)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PR_INIT, PR_ACC, PR_DAMP = (float(np.float32(x)) for x in (0.15, 0.01, 0.85))


def _unpack(p):
    p = p.astype(np.float64)
    return (p[0:320].reshape(64, 5), p[320:384], p[384:4480].reshape(64, 64), p[4480:4544],
            p[4544:4608], p[4608])


def _ref_forward_grad(p, x, t):
    """FP64 forward pass, binary cross-entropy and its gradient."""
    W1, b1, W2, b2, W3, b3 = _unpack(p)
    x = x.astype(np.float64)
    t = t.astype(np.float64)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    y = 1 / (1 + np.exp(-(h2 @ W3 + b3)))
    n = len(x)
    yc = np.clip(y, 1e-7, 1 - 1e-7)
    loss = -np.mean(t * np.log(yc) + (1 - t) * np.log(1 - yc))
    d3 = (y - t) / n
    d2 = d3[:, None] * W3[None, :] * (z2 > 0)
    d1 = (d2 @ W2) * (z1 > 0)
    g = np.concatenate([(d1.T @ x).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), h2.T @ d3, [d3.sum()]])
    return y, g, loss


def test_mlp_forward_and_gradient_match_fp64(gpu):
    m = gpu.Mlp.create(0, seed=3)
    rng = np.random.default_rng(0)
    p = m.params()
    assert p.shape == (4609,)
    x = rng.random((256, 5), dtype=np.float32)
    t = rng.random(256, dtype=np.float32)
    y_ref, g_ref, loss_ref = _ref_forward_grad(p, x, t)
    y = m.forward(x)
    assert np.max(np.abs(y - y_ref)) < 1e-4
    g, loss = m.gradient(x, t)
    assert abs(loss - loss_ref) < 1e-4 * max(1.0, abs(loss_ref))
    assert np.max(np.abs(g - g_ref)) <= 2e-3 * np.max(np.abs(g_ref))
    # the weights the kernels use are BF16 values
    assert np.array_equal(p, p.astype(np.float32).view(np.uint32).__and__(0xFFFF0000).view(np.float32))


def test_mlp_training_fits_and_round_trips(gpu, tmp_path):
    rng = np.random.default_rng(1)
    x = rng.random((4000, 5), dtype=np.float32)
    t = (1 / (1 + np.exp(-(3 * x[:, 1] - 2 * x[:, 3] + 0.5)))).astype(np.float32)
    m = gpu.Mlp.create(0, seed=5)
    loss0 = m.gradient(x, t)[1]
    loss = m.train(x, t, steps=400, lr=3e-3)
    assert loss < loss0
    assert np.mean(np.abs(m.forward(x) - t)) < 0.03
    m.save(tmp_path / "m.bin")
    m2 = gpu.Mlp.load(tmp_path / "m.bin")
    assert np.array_equal(m.params(), m2.params())
    assert np.array_equal(m.forward(x[:64]), m2.forward(x[:64]))


def _oracle(orc, g, algo, src):
    e = g.edges if algo in ("sssp", "sswp") else g.ends
    return orc.run(algo, g.node_pointer, e, src)


@pytest.mark.parametrize("model_kind", ["persistence", "random"])
@pytest.mark.parametrize("num_buffers,defer", [(2, 0), (3, 0), (3, 30), (4, 200)])
def test_learned_policy_bit_exact(gpu, orc, model_kind, num_buffers, defer):
    """Any network, buffer count and frontier deferral target: the answers
    are the oracle's."""
    g = gpu.Graph.rmat(12, 16, seed=31, weighted=True)
    model = gpu.Mlp.create(0, seed=9) if model_kind == "random" else None
    for edges_budget in (400, 6000, 60000):
        eng = gpu.Engine(g, budget_bytes=18 * g.n + 96 * 1024 + edges_budget * 4 * num_buffers,
                         num_buffers=num_buffers, sched_defer_permille=defer)
        eng.set_policy("learned", model)
        src = int(g.pick_sources(1, seed=edges_budget)[0])
        for algo in ("bfs", "sssp", "sswp", "cc"):
            for mode in ("sync", "async"):
                vals, st = eng.run(algo, mode, src)
                assert np.array_equal(vals, _oracle(orc, g, algo, src)), (algo, mode, edges_budget)
        eng.close()


def test_learned_policy_pagerank(gpu, orc):
    g = gpu.Graph.rmat(12, 16, seed=32)
    eng = gpu.Engine(g, budget_bytes=36 * g.n + 96 * 1024 + 8000 * 8)
    eng.set_policy("learned")
    vals, _ = eng.run("pr", "sync")
    ref, _ = orc.pagerank(g.node_pointer, g.edges, init=PR_INIT, acc=PR_ACC, damping=PR_DAMP)
    assert np.max(np.abs(vals.astype(np.float64) - ref) / ref) < 2.5e-7


def test_learned_policy_uses_residency(gpu):
    """With most of the graph fitting in the buffers, later iterations find
    ranges resident and move fewer bytes than the plain policy (inner cap
    off); with the inner cap on, kept ranges stop early and the answers stay
    bit-exact."""
    g = gpu.Graph.rmat(14, 16, seed=33, weighted=True)
    budget = 18 * g.n + 96 * 1024 + int(0.4 * g.m) * 4 * 2
    plain = gpu.Engine(g, budget_bytes=budget)
    learned = gpu.Engine(g, budget_bytes=budget, sched_active_permille=2000, num_buffers=3)
    learned.set_policy("learned")
    learned.trace_enable(True)
    src = int(g.pick_sources(1, seed=1)[0])
    v1, s1 = plain.run("sssp", "async", src)
    v2, s2 = learned.run("sssp", "async", src)
    assert np.array_equal(v1, v2)
    rec = learned.range_trace()
    assert (rec["action"] == gpu.ACT_RESIDENT).any()
    assert s2["h2d_bytes"] <= s1["h2d_bytes"]
    capped = gpu.Engine(g, budget_bytes=budget, sched_active_permille=1, sched_inner=1, num_buffers=3)
    capped.set_policy("learned")
    capped.trace_enable(True)
    v3, s3 = capped.run("sssp", "async", src)
    assert np.array_equal(v1, v3)
    rec = capped.range_trace()
    kept = np.isin(rec["action"], [gpu.ACT_RESIDENT, gpu.ACT_STREAM]) & (rec["active_nodes"] > 0)
    kept &= rec["predicted"] >= 0.001
    assert kept.any() and (rec["inner_iterations"][kept] <= 1).all()


def test_trained_network_gains(gpu):
    """What the trained network adds, on a graph it was not trained on
    (R-MAT scale 20, seed 777; training used scales 22-25), measured against
    the same schedule with the persistence predictor ("the active fraction
    stays the same") in place of the network: the network predicts the next
    iteration's range activity better, the answers are identical, and the
    schedule's cost (H2D bytes, relaxed edges) stays within 10% of the
    persistence predictor's.  On these workloads the schedule's decisions
    are not sensitive to the prediction error, so the network buys no
    measurable time or bytes (the design notes give the measurements); both
    learned schedules still relax far fewer edges than the plain one."""
    from subway_gb300 import scheduler
    model = scheduler.load_default(0)
    assert model is not None, "trained scheduler model missing"
    g = gpu.Graph.rmat(20, 16, seed=777, weighted=True, wmax=64)
    x, y = scheduler.collect(g, algos=("sssp",), sources=2, budget_fraction=0.4, seed=5)
    assert len(x) > 20
    mae_net = float(np.mean(np.abs(model.forward(x) - y)))
    mae_same = float(np.mean(np.abs(x[:, 1] - y)))
    assert mae_net < 0.75 * mae_same, (mae_net, mae_same)

    budget = int(scheduler.fixed_state_bytes(g.n) + 0.4 * g.m * 4)
    plain = gpu.Engine(g, budget_bytes=budget)
    net = gpu.Engine(g, budget_bytes=budget, num_buffers=3)
    net.set_policy("learned", model)
    same = gpu.Engine(g, budget_bytes=budget, num_buffers=3)
    same.set_policy("learned", None)
    tot = {k: [0, 0] for k in ("plain", "net", "same")}
    for s in g.pick_sources(3, seed=9):
        ref = None
        for k, eng in (("plain", plain), ("net", net), ("same", same)):
            v, st = eng.run("sssp", "async", int(s))
            ref = v if ref is None else ref
            assert np.array_equal(v, ref), k
            tot[k][0] += st["h2d_bytes"]
            tot[k][1] += st["relaxed_edges"]
    assert tot["net"][0] <= 1.1 * tot["same"][0] and tot["net"][1] <= 1.1 * tot["same"][1], tot
    assert tot["net"][0] <= tot["plain"][0], tot
    assert tot["net"][1] < 0.9 * tot["plain"][1], tot

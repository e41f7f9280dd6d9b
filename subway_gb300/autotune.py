"""Autotuner for the relaxation thresholds, tile sizes and gather grid.

Times candidate settings of the engine options that shape the kernels
(tile_degree_max: sources above it leave the CTA tile for the chunk list;
chunk_edges: edges per chunk-list item; gather_ctas: gather grid) on a short
sample of the actual workload, greedily one option at a time, and returns the
fastest.  For batched queries it tunes the edges per work item.  Nothing here
changes results: every candidate computes the same fixpoint.
"""
from __future__ import annotations

import numpy as np

from . import native as N

ENGINE_SPACE = {
    "tile_degree_max": (64, 128, 256, 512, 1024),
    "chunk_edges": (256, 512, 1024, 2048),
    "gather_ctas_per_sm": (1, 2, 3, 4),
}


def _time_engine(g, budget, opts, algo, mode, sources, policy, model, device, reps=1):
    kw = dict(opts)
    gps = kw.pop("gather_ctas_per_sm", 2)
    eng = N.Engine(g, budget_bytes=budget, device=device, gather_ctas=gps * _sm_count(device), **kw)
    if policy != "plain":
        eng.set_policy(policy, model)
    eng.run(algo, mode, int(sources[0]))  # warm
    ms = 0.0
    for _ in range(reps):
        for s in sources:
            _, st = eng.run(algo, mode, int(s))
            ms += st["ms_device"]
    eng.close()
    return ms


def _sm_count(device):
    return N.device_info(device)["sm_count"]


def tune_engine(g, budget, algo="sssp", mode="async", sources=None, policy="plain", model=None,
                device=0, num_buffers=0):
    """Greedy coordinate search; returns (best option dict, trials)."""
    if sources is None:
        sources = g.pick_sources(2, seed=11)
    best = {"tile_degree_max": 256, "chunk_edges": 1024, "gather_ctas_per_sm": 2}
    if num_buffers:
        best["num_buffers"] = num_buffers
    trials = []
    best_ms = _time_engine(g, budget, best, algo, mode, sources, policy, model, device)
    trials.append((dict(best), best_ms))
    for key, cands in ENGINE_SPACE.items():
        for c in cands:
            if c == best[key]:
                continue
            cand = dict(best)
            cand[key] = c
            ms = _time_engine(g, budget, cand, algo, mode, sources, policy, model, device)
            trials.append((cand, ms))
            if ms < best_ms * 0.98:  # keep a change only for a clear gain
                best, best_ms = cand, ms
    return best, best_ms, trials


def engine_opts(best: dict, device=0) -> dict:
    """Engine keyword arguments for a tuned setting."""
    o = {k: v for k, v in best.items() if k != "gather_ctas_per_sm"}
    o["gather_ctas"] = best.get("gather_ctas_per_sm", 2) * _sm_count(device)
    return o


def tune_batch(g, algo="bfs", lanes=64, device=0, candidates=(64, 128, 256, 512, 1024), seed=3):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, g.n, lanes).astype(np.uint32)
    res = []
    for c in candidates:
        b = N.Batch(g, lanes=lanes, device=device, chunk_edges=c)
        b.run(algo, src[:2])
        _, st = b.run(algo, src)
        res.append((c, st["ms_device"]))
        b.close()
    best = min(res, key=lambda x: x[1])[0]
    return best, res

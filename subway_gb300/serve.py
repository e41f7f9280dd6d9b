"""Batched query serving: Poisson arrivals over graphs resident in HBM.

Queries (BFS or SSSP from uniformly random sources) arrive as a seeded
Poisson process and queue per graph; the server repeatedly takes the graph
whose oldest query has waited longest and runs up to `lanes` of its queued
queries as one batch (sgw_batch_run), so batch sizes follow the load.  Graphs
are admitted under one device-memory budget: each one's batch object must
fit in what the graphs admitted before it left.

    python -m subway_gb300.serve --scales 22 24 26 --queries 4096 --rate 2000
prints one JSON line with p50/p99 latency and queries per second.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import native as N


def admit(graphs, lanes, budget_bytes, device=0, chunk_edges=0):
    """Batch objects for the graphs that fit the remaining budget, in order.
    chunk_edges: one value for all graphs or one per graph (0 = default)."""
    left = budget_bytes
    admitted, rejected = [], []
    chunks = chunk_edges if isinstance(chunk_edges, (list, tuple)) else [chunk_edges] * len(graphs)
    for g, ch in zip(graphs, chunks):
        try:
            b = N.Batch(g, lanes=lanes, budget_bytes=left, device=device, chunk_edges=ch)
        except N.SgwError as e:
            if e.status != -5:  # only a budget refusal means "not admitted"
                raise
            rejected.append(g)
            continue
        left -= b.device_bytes()
        admitted.append(b)
    return admitted, rejected


def serve(batches, algo="bfs", queries=4096, rate=2000.0, seed=5, lanes=64):
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, queries))
    target = rng.integers(0, len(batches), queries)
    sources = np.array([rng.integers(0, batches[t].graph.n) for t in target], np.uint32)
    done = np.zeros(queries)
    pending = [[] for _ in batches]  # query ids per graph, in arrival order
    sizes = []
    nxt = 0
    served = 0
    t0 = time.perf_counter()
    while served < queries:
        now = time.perf_counter() - t0
        while nxt < queries and arrivals[nxt] <= now:
            pending[target[nxt]].append(nxt)
            nxt += 1
        if not any(pending):
            wait = arrivals[nxt] - now
            if wait > 0.0005:
                time.sleep(wait - 0.0002)
            continue
        k = min((i for i in range(len(batches)) if pending[i]), key=lambda i: arrivals[pending[i][0]])
        ids = pending[k][:lanes]
        pending[k] = pending[k][lanes:]
        batches[k].run(algo, sources[ids], view=True)  # answers land in pinned memory
        t = time.perf_counter() - t0
        done[ids] = t
        served += len(ids)
        sizes.append(len(ids))
    lat_ms = (done - arrivals) * 1e3
    span = done.max() - arrivals[0]
    return {"queries": queries, "rate_per_s": rate, "algo": algo, "p50_ms": float(np.percentile(lat_ms, 50)),
            "p99_ms": float(np.percentile(lat_ms, 99)), "mean_ms": float(lat_ms.mean()),
            "qps": queries / span, "batches": len(sizes), "mean_batch": float(np.mean(sizes)),
            "max_batch": int(max(sizes))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scales", type=int, nargs="+", default=[22, 24, 26])
    ap.add_argument("--queries", type=int, default=4096)
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--algo", default="bfs", choices=["bfs", "sssp"])
    ap.add_argument("--lanes", type=int, default=64)
    ap.add_argument("--budget", type=float, default=200e9)
    ap.add_argument("--chunk-edges", type=int, default=0)
    ap.add_argument("--autotune", action="store_true", help="pick each graph's edges per work item by timing")
    a = ap.parse_args()
    t = time.time()
    graphs = [N.Graph.rmat(s, 16, seed=5000 + s, weighted=True, wmax=64) for s in a.scales]
    t_gen = time.time() - t
    chunks = a.chunk_edges
    tuned = None
    if a.autotune:
        from .autotune import tune_batch
        tuned = [tune_batch(g, a.algo, a.lanes) for g in graphs]
        chunks = [best for best, _ in tuned]
    admitted, rejected = admit(graphs, a.lanes, int(a.budget), chunk_edges=chunks)
    # warm the graphs up once
    for b in admitted:
        b.run(a.algo, np.zeros(1, np.uint32))
    res = serve(admitted, a.algo, a.queries, a.rate, lanes=a.lanes)
    if tuned:
        res["autotune"] = [{"scale": s, "chunk_edges": best, "trials_ms": [(c, round(ms, 2)) for c, ms in trials]}
                           for s, (best, trials) in zip(a.scales, tuned)]
    res.update({"scales_admitted": [s for s, g in zip(a.scales, graphs) if g not in rejected],
                "device_bytes": sum(b.device_bytes() for b in admitted), "generate_s": round(t_gen, 1)})
    print(json.dumps(res))


if __name__ == "__main__":
    main()

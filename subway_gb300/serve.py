"""Batched query serving: Poisson arrivals over graphs resident in HBM.

Queries (BFS or SSSP from uniformly random sources) arrive as a seeded
Poisson process and queue per graph; the server repeatedly takes the graph
whose oldest query has waited longest and runs up to `lanes` of its queued
queries as one batch (sgw_batch_run), so batch sizes follow the load.  Graphs
are admitted under one device-memory budget: each one's batch object must
fit in what the graphs admitted before it left.

    python -m subway_gb300.serve --scales 22 24 26 --queries 4096 --rate 2000
prints one JSON line with p50/p99 latency and queries per second.

Replicas: launched under torchrun (one process per GPU, RANK / WORLD_SIZE /
LOCAL_RANK from the environment), every rank draws the same seeded query
stream, serves the queries whose index is congruent to its rank on its own
GPU with its own copy of the graphs, and rank 0 merges the latencies into one
line; QPS is all queries over the span from the first arrival to the last
answer on any rank.  The ranks meet only for a barrier before the clocks
start and for the final gather.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import native as N


def admit(graphs, lanes, budget_bytes, device=0, chunk_edges=0, flags=0):
    """Batch objects for the graphs that fit the remaining budget, in order.
    chunk_edges: one value for all graphs or one per graph (0 = default)."""
    left = budget_bytes
    admitted, rejected = [], []
    chunks = chunk_edges if isinstance(chunk_edges, (list, tuple)) else [chunk_edges] * len(graphs)
    for g, ch in zip(graphs, chunks):
        try:
            b = N.Batch(g, lanes=lanes, budget_bytes=left, device=device, chunk_edges=ch, flags=flags)
        except N.SgwError as e:
            if e.status != -5:  # only a budget refusal means "not admitted"
                raise
            rejected.append(g)
            continue
        left -= b.device_bytes()
        admitted.append(b)
    return admitted, rejected


def make_stream(graph_sizes, queries=4096, rate=2000.0, seed=5):
    """Seeded Poisson arrivals (s), target graph and source vertex per query."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, queries))
    target = rng.integers(0, len(graph_sizes), queries)
    sources = np.array([rng.integers(0, graph_sizes[t]) for t in target], np.uint32)
    return arrivals, target, sources


def shard(stream, world=1, rank=0):
    """The queries of one replica: every world-th query, starting at rank."""
    return tuple(x[rank::world] for x in stream)


def serve_stream(batches, arrivals, target, sources, algo="bfs", lanes=64, answers="u32"):
    """Serves one stream in real time; returns answer times (s from the
    start of the clock) and the batch sizes."""
    queries = len(arrivals)
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
        batches[k].run(algo, sources[ids], view=True, answers=answers)  # answers land in pinned memory
        t = time.perf_counter() - t0
        done[ids] = t
        served += len(ids)
        sizes.append(len(ids))
    return done, sizes


def summarize(arrivals, done, sizes, rate, algo):
    lat_ms = (done - arrivals) * 1e3
    span = done.max() - arrivals.min()
    return {"queries": int(len(arrivals)), "rate_per_s": rate, "algo": algo,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "mean_ms": float(lat_ms.mean()), "qps": len(arrivals) / span, "batches": len(sizes),
            "mean_batch": float(np.mean(sizes)), "max_batch": int(max(sizes))}


def serve(batches, algo="bfs", queries=4096, rate=2000.0, seed=5, lanes=64, answers="u32"):
    arrivals, target, sources = make_stream([b.graph.n for b in batches], queries, rate, seed)
    done, sizes = serve_stream(batches, arrivals, target, sources, algo, lanes, answers)
    return summarize(arrivals, done, sizes, rate, algo)


def serve_replicas(batches, pg, algo="bfs", queries=4096, rate=2000.0, seed=5, lanes=64, answers="u32"):
    """One replica's share of the stream; rank 0 returns the merged summary,
    the other ranks None.  pg: torch.distributed, initialised."""
    world, rank = pg.get_world_size(), pg.get_rank()
    arrivals, target, sources = shard(make_stream([b.graph.n for b in batches], queries, rate, seed), world, rank)
    pg.barrier()
    done, sizes = serve_stream(batches, arrivals, target, sources, algo, lanes, answers)
    parts = [None] * world
    pg.all_gather_object(parts, (arrivals, done, sizes))
    if rank != 0:
        return None
    res = summarize(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]),
                    [x for p in parts for x in p[2]], rate, algo)
    res["replicas"] = world
    res["queries_per_replica"] = [int(len(p[0])) for p in parts]
    return res


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
    ap.add_argument("--answers", default="u32", choices=["u32", "u16"],
                    help="u16: 16-bit answers (unreached = 0xffff), half the bytes copied out")
    ap.add_argument("--form", default="auto", choices=["auto", "persistent", "graph"],
                    help="batch form: auto (persistent for SSSP, graph loop for BFS), or one for both")
    a = ap.parse_args()
    import os
    world = int(os.environ.get("WORLD_SIZE", "1"))
    device = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as pg
        pg.init_process_group("gloo")
    t = time.time()
    graphs = [N.Graph.rmat(s, 16, seed=5000 + s, weighted=True, wmax=64) for s in a.scales]
    t_gen = time.time() - t
    chunks = a.chunk_edges
    tuned = None
    if a.autotune:
        from .autotune import tune_batch
        tuned = [tune_batch(g, a.algo, a.lanes, device=device) for g in graphs]
        chunks = [best for best, _ in tuned]
    admitted, rejected = admit(graphs, a.lanes, int(a.budget), device=device, chunk_edges=chunks,
                               flags={"auto": 0, "persistent": N.OPT_BATCH_PERSISTENT,
                                      "graph": N.OPT_BATCH_GRAPH}[a.form])
    # warm the graphs up once
    for b in admitted:
        b.run(a.algo, np.zeros(1, np.uint32))
    if pg:
        res = serve_replicas(admitted, pg, a.algo, a.queries, a.rate, lanes=a.lanes, answers=a.answers)
        if res is None:
            pg.destroy_process_group()
            return
    else:
        res = serve(admitted, a.algo, a.queries, a.rate, lanes=a.lanes, answers=a.answers)
    if tuned:
        res["autotune"] = [{"scale": s, "chunk_edges": best, "trials_ms": [(c, round(ms, 2)) for c, ms in trials]}
                           for s, (best, trials) in zip(a.scales, tuned)]
    res.update({"answers": a.answers, "form": a.form, "scales_admitted": [s for s, g in zip(a.scales, graphs) if g not in rejected],
                "device_bytes": sum(b.device_bytes() for b in admitted), "generate_s": round(t_gen, 1)})
    print(json.dumps(res))
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()

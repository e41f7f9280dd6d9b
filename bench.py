"""Benchmark: out-of-HBM-budget SSSP-async on weighted R-MAT scale 28.

Workload (default; one "step" = one SSSP-async run from one source, cycling
over the sources): R-MAT(0.57, 0.19, 0.19, 0.05), 2^28 vertices, edge factor
16 (4.26 G edges after removing self-loops and duplicates), uint32 weights
uniform in [1, 64], 16 seeded sources from the largest weakly connected
component, device-memory budget 8 GB (the edges take 21 GB in the engine's
transfer form, 34 GB as the reference's 8-byte records).  `--scale 24
--budget 1e9 --sources 8` is the smaller RMAT-24 / 1 GB workload.

Metric: GTEPS = reached edges (Graph500 m_reached) / time, plus the bytes the
device read from host memory per run.  Three schedules are timed on the same
graph: the plain one (the reference's: every active edge compacted and sent
each iteration, async partitions relaxed to convergence), the learned one
with its trained network (the headline), and the learned one with the
network replaced by the persistence predictor ("activity stays the same"),
which isolates what the network adds to the schedule's rules.
  value     device-timed processing loop of the learned schedule (CUDA events
            on the engine's compute stream, from after the first generate to
            the end of the loop: the reference's t_processing convention)
  e2e       one query as a process runs it, measured like the reference arm:
            engine creation (device arena, transfer copy of the host edges),
            sgw_run through the C ABI with host buffers (state init, every
            host->device edge transfer, the distance read-back) and engine
            destruction; the graph load is excluded on both arms.  The engine
            is made as the drop-in apps make it: no transfer copy, the
            gather reads the graph's 8-byte records in place through the host
            page tables (SGW_OPT_GRAPH_IN_PLACE); e2e_pinned is the same with
            the library default, the packed pinned transfer copy
  e2e_warm  sgw_run alone on a live engine (a resident query service)
After the timed loops every distinct source's distances from every schedule
are compared with the OpenMP oracle; the line carries the mismatch count and
the process exits non-zero if it is not 0.

--impl reference runs the reference's own sssp-async build (oracle/_ref,
compiled from the upstream sources for sm_103a) on the same graph, written by
the oracle's generator (the engine library is not loaded), with the same
device budget, and reports per process: the wall time after its CUDA context
is up minus its own "Graph Reading finished" time (its e2e) and its
"Processing finished" time.  Under torchrun every rank runs an independent
replica (the path does not shard); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GTEPS & H2D bytes per run, out-of-HBM-budget RMAT SSSP/BFS: learned vs plain"
SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
INF = 4294967294


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=28)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--budget", type=float, default=8e9)
    ap.add_argument("--algo", default="sssp", choices=["bfs", "sssp", "sswp"])
    ap.add_argument("--mode", default="async", choices=["sync", "async"])
    ap.add_argument("--sources", type=int, default=16)
    ap.add_argument("--seed", type=int, default=24)
    ap.add_argument("--check", default="all", choices=["all", "none"],
                    help="compare every distinct source's answer with the OpenMP oracle")
    ap.add_argument("--no-pack", action="store_true", help="move the reference's 8-byte records")
    ap.add_argument("--gather-ctas", type=int, default=0)
    ap.add_argument("--tile-degree-max", type=int, default=0)
    ap.add_argument("--chunk-edges", type=int, default=0)
    ap.add_argument("--inner-batch", type=int, default=0)
    ap.add_argument("--policy", default="all", choices=["plain", "learned", "all"],
                    help="all: plain, learned with the persistence predictor, learned (headline)")
    ap.add_argument("--model", default="", help="scheduler model file (default: the committed one)")
    ap.add_argument("--num-buffers", type=int, default=0,
                    help="edge buffers of the learned policy (0 = sgw_sched_buffers' choice)")
    ap.add_argument("--sched-inner", type=int, default=0)
    ap.add_argument("--sched-defer", type=int, default=0)
    ap.add_argument("--sched-permille", type=int, default=0)
    ap.add_argument("--suite", default="", choices=["", "scale27"],
                    help="scale27: BFS, CC, SSWP (and PR with --suite-pr) sync and async on R-MAT scale 27 "
                         "under a 4 GB budget plus an Erdos-Renyi control, each checked against the oracle")
    ap.add_argument("--suite-pr", action="store_true", help="add PageRank (6 GB budget) to the suite")
    ap.add_argument("--profile-engine", choices=["service", "one-query"], default="service",
                    help="with --profile-run: the long-lived engine (pinned packed copy, the value's) or the "
                         "one-query engine of the drop-in apps and of e2e (records read in place)")
    ap.add_argument("--profile-run", action="store_true",
                    help="one warm-up run and one measured run of --policy (plain or learned) from the first "
                         "two sources; prints each run's launches per kernel class (for ncu -s / -c) and the "
                         "measured run's algorithmic bytes")
    ap.add_argument("--ref-time-limit", type=float, default=900.0,
                    help="reference arm: stop starting processes after this many seconds (>= 2 timed)")
    return ap.parse_args(argv)


# ---- distributed plumbing (replicas) ------------------------------------------
class Dist:
    def __init__(self, n):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())


# ---- clocks during the timed region --------------------------------------------
class ClockSampler:
    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={SMI_FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def weighted_algo(algo):
    return algo in ("sssp", "sswp")


def transfer_record_bytes(n, weighted, no_pack, wmax=64):
    """Host bytes per edge in the engine's transfer form: the destination
    word (weighted: with the weight packed above a 32-bit destination of
    bits(n) bits when w < 2^(32 - bits), else a separate weight byte), or the
    reference's 8-byte record with --no-pack."""
    if not weighted:
        return 4
    if no_pack:
        return 8
    nb = 1
    while nb < 32 and (1 << nb) < n:
        nb += 1
    return 4 if nb < 31 and wmax < (1 << (32 - nb)) else 5


def workload_config(a):
    """The workload, identical for both arms."""
    w = "-w64" if weighted_algo(a.algo) else ""
    return {"workload": f"rmat{a.scale}-ef{a.edge_factor}{w} {a.algo}-{a.mode}, device budget "
                        f"{a.budget / 1e9:g} GB, {a.sources} sources from the largest WCC",
            "graph": f"R-MAT(0.57,0.19,0.19,0.05) scale {a.scale}, edge factor {a.edge_factor}, "
                     "dedup, no self-loops" + (", u32 weights in [1,64]" if w else ""),
            "budget_bytes": int(a.budget), "sources": a.sources, "seed": a.seed,
            "l2": "inputs larger than L2: the edges stay in host memory",
            "parallelism": "replicas"}


# ---- our engine ------------------------------------------------------------------
def probe_link(N, dev):
    import ctypes as C
    h, d = C.c_double(), C.c_double()
    N.check(N.lib().sgw_probe_link(dev, 1 << 30, 5, C.byref(h), C.byref(d)), "sgw_probe_link")
    return h.value, d.value


# DRAM bytes (read + write) per algorithmic byte of each kernel class, from
# one-kernel-class ncu captures over one measured RMAT-24 / 1 GB run
# (profiles/dram_per_class_rmat24_sssp_async_1gb.md; ncu empties the caches
# before each launch, so these are cold-cache figures).  A full-size launch's
# traffic is the ratio times its algorithmic bytes: an estimate, not a count.
DRAM_PER_ALGO_BYTE = {"gather": 0.73, "relax": 1.06, "generate": 2.23}
# Host-link bytes (L2 sectors filled from host memory) per algorithmic byte of
# the gather, from a one-kernel capture over every gather of one measured
# RMAT-24 / 1 GB run (profiles/k_gather_v_rmat24_sssp_async_1gb.md).
LINK_PER_ALGO_BYTE = {"gather": 1.063}


def run_ours(a, dist):
    import numpy as np

    from subway_gb300 import native as N
    from subway_gb300 import scheduler

    dev = dist.local
    t0 = time.time()
    weighted = weighted_algo(a.algo)
    g = N.Graph.rmat(a.scale, a.edge_factor, seed=a.seed, weighted=weighted, wmax=64)
    sources = [int(s) for s in g.pick_sources(a.sources, seed=a.seed)]
    t_gen = time.time() - t0
    flags = N.OPT_PROFILE | (N.OPT_NO_PACK if a.no_pack else 0)
    h2d_peak, _ = probe_link(N, dev)
    out = np.empty(g.n, np.uint32)  # host result buffer
    nb_learned = a.num_buffers or N.sched_buffers(g, a.budget)

    def make_engine(arm, extra_flags=0):
        nb = 0 if arm == "plain" else nb_learned
        e = N.Engine(g, budget_bytes=int(a.budget), device=dev, flags=flags | extra_flags, gather_ctas=a.gather_ctas,
                     tile_degree_max=a.tile_degree_max, chunk_edges=a.chunk_edges,
                     inner_batch=a.inner_batch, num_buffers=nb, sched_inner=a.sched_inner,
                     sched_active_permille=a.sched_permille, sched_defer_permille=a.sched_defer)
        if arm != "plain":
            model = None
            if arm == "learned":
                model = N.Mlp.load(a.model, dev) if a.model else scheduler.load_default(dev)
            e.set_policy("learned", model)
            e._model = model
        return e

    arms = {"plain": ["plain"], "learned": ["learned"], "all": ["plain", "rules", "learned"]}[a.policy]

    # the oracle's answers first (the CPU baseline, timed with the GPU idle);
    # every schedule is checked against them right after its timed loop, so
    # one engine at a time holds its pinned transfer copy
    check = {"checked_sources": 0, "mismatches": 0, "reached_mismatches": 0}
    cpu, refs = None, {}
    if a.check == "all":
        from oracle import oracle
        e = g.edges if weighted else g.ends
        deg = g.out_degree()
        npt = np.ascontiguousarray(g.node_pointer, dtype=np.uint64)  # the oracle's width, once
        secs, reached_cpu = 0.0, 0
        for s in dict.fromkeys(sources):
            t = time.perf_counter()
            ref = oracle.run(a.algo, npt, e, s, parallel=True)
            secs += time.perf_counter() - t
            want = int(deg[ref != (0 if a.algo == "sswp" else INF)].astype(np.uint64).sum())
            reached_cpu += want
            refs[s] = (ref, want)
        check["checked_sources"] = len(refs)
        cpu = {"value": round(reached_cpu / secs / 1e9, 4), "unit": "GTEPS", "cores": oracle.num_threads(),
               "kind": "port",
               "sample": f"{len(refs)} full {a.algo} runs of the OpenMP oracle "
                         f"({'delta-stepping' if a.algo == 'sssp' else 'frontier label-correcting'}) on the "
                         "same graph, the runs that check the engine's answers",
               "seconds": round(secs, 2)}

    def check_engine(arm, eng):
        for s, (ref, want) in refs.items():
            _, st = eng.run(a.algo, a.mode, s, out=out)
            check["mismatches"] += int(np.count_nonzero(out != ref))
            check["reached_mismatches"] += int(st["reached_edges"] != want)
        # where tests/golden holds the reference build's own digests for this
        # workload, the learned schedule's distances are compared with them too
        import hashlib
        gold = ROOT / "tests" / "golden" / f"ref_rmat{a.scale}_{a.algo}_{a.mode}_{int(a.budget / 1e9)}gb.json"
        if arm == "learned" and a.check == "all" and gold.exists() and a.edge_factor == 16:
            rep = json.loads(gold.read_text())
            if f"seed {a.seed}," in rep["graph"] and rep["budget_bytes"] == int(a.budget):
                hits = 0
                for s in rep["sources"]:
                    eng.run(a.algo, a.mode, s, out=out)
                    key = next(k for k in rep["runs"] if k.startswith("fixed/") and k.endswith(f"/s{s}"))
                    hits += hashlib.sha256(out.tobytes()).hexdigest() == rep["runs"][key]["sha256"]
                check["reference_digests"] = {"checked": len(rep["sources"]), "equal": hits,
                                              "fixture": gold.name}
                check["mismatches"] += len(rep["sources"]) - hits

    res = {}
    for arm in arms:
        t = time.perf_counter()
        eng = make_engine(arm)
        create_s = time.perf_counter() - t
        for k in range(a.warmup):
            eng.run(a.algo, a.mode, sources[k % len(sources)], out=out)
        steps = []
        dist.barrier()
        with ClockSampler(dev) as clk:
            t_start = time.perf_counter()
            for k in range(a.steps):
                t = time.perf_counter()
                _, st = eng.run(a.algo, a.mode, sources[k % len(sources)], out=out)
                st["wall_ms"] = (time.perf_counter() - t) * 1e3
                steps.append(st)
            t_total = time.perf_counter() - t_start
        dist.barrier()
        res[arm] = {"steps": steps, "clk": clk, "t_total": t_total, "create_s": create_s}
        if arm == "learned":
            # one more run, untimed, with the range trace on: how often the
            # predictions behind its transfer decisions were wrong
            eng.trace_enable(True)
            eng.run(a.algo, a.mode, sources[0], out=out)
            res[arm]["mispredicted"] = scheduler.mispredictions(eng.range_trace())
            eng.trace_enable(False)
        check_engine(arm, eng)
        eng.close()
        del eng

    # one query as a process runs it: create, run with host buffers, destroy;
    # the engine made as the drop-in apps make it (the graph's records read in
    # place, no transfer copy), and for the learned schedule also with the
    # library's default pinned copy
    one_query = N.OPT_GRAPH_IN_PLACE | N.OPT_PAGEABLE_COPY
    e2e_loops = [(arm, "e2e", one_query) for arm in ("plain", "learned") if arm in arms]
    e2e_loops += [("learned", "e2e_pinned", 0)] if "learned" in arms else []
    for arm, key, xf in e2e_loops:
        walls, st_all, phases = [], [], []
        for k in range(a.warmup + a.steps):
            t = time.perf_counter()
            eng = make_engine(arm, xf)
            t1 = time.perf_counter()
            _, st = eng.run(a.algo, a.mode, sources[k % len(sources)], out=out)
            t2 = time.perf_counter()
            eng.close()
            t3 = time.perf_counter()
            if k >= a.warmup:
                walls.append(t3 - t)
                st_all.append(st)
                phases.append((t1 - t, t2 - t1, t3 - t2))
        res[arm][key + "_walls"] = walls
        res[arm][key + "_phases_ms"] = {name: round(1e3 * sum(p[i] for p in phases) / len(phases), 2)
                                        for i, name in enumerate(("create", "run", "destroy"))}
        res[arm][key + "_reached"] = sum(s["reached_edges"] for s in st_all)
        res[arm][key + "_h2d"] = sum(s["h2d_bytes"] for s in st_all) / len(st_all)
    refs.clear()

    hbm_peak, hbm_src = measured_peaks()

    def summary(arm):
        r = res[arm]
        steps = r["steps"]
        K = len(steps)
        reached = dist.sum(sum(s["reached_edges"] for s in steps))
        dev_ms = dist.max(sum(s["ms_device"] for s in steps))
        warm_ms = dist.max(sum(s["wall_ms"] for s in steps))
        d = {"value": round(reached / (dev_ms * 1e6), 4),
             "e2e_warm": round(reached / (warm_ms * 1e6), 4),
             "h2d_bytes_per_run": int(sum(s["h2d_bytes"] for s in steps) / K),
             "ms_per_step": round(dev_ms / K, 4),
             "iterations_per_step": round(sum(s["global_iterations"] for s in steps) / K, 2),
             "engine_create_s": round(r["create_s"], 3)}
        for key in ("e2e", "e2e_pinned"):
            if key + "_walls" in r:
                d[key] = round(dist.sum(r[key + "_reached"]) / (dist.max(sum(r[key + "_walls"])) * 1e9), 4)
                d[key + "_ms_per_step"] = round(1e3 * sum(r[key + "_walls"]) / len(r[key + "_walls"]), 2)
        return d

    head = "learned" if "learned" in arms else "plain"
    sums = {arm: summary(arm) for arm in arms}
    steps = res[head]["steps"]
    K = a.steps
    hs = sums[head]

    # kernel classes: the gather kernel, the whole-range DMA copies, the
    # relaxation and the generate step (algorithmic bytes per launch)
    esz = transfer_record_bytes(g.n, weighted, a.no_pack)
    gbytes = sum(s["gather_bytes"] for s in steps)
    sbytes = sum(s["h2d_bytes"] - s["gather_bytes"] for s in steps)
    relax_bytes = sum(s["relaxed_sources"] * 17 + s["relaxed_edges"] * (esz + 4) for s in steps)
    gen_bytes = sum(s["generate_launches"] * 2 * g.n + s["active_vertices"] * 16 for s in steps)
    classes = {
        "gather": ("host_link", gbytes, sum(s["ms_gather"] for s in steps), sum(s["gather_launches"] for s in steps),
                   h2d_peak, "measured pinned cudaMemcpyAsync H2D on this GPU (bench)"),
        "relax": ("hbm", relax_bytes, sum(s["ms_relax"] for s in steps), sum(s["relax_launches"] for s in steps),
                  hbm_peak, f"MEASURED_PEAKS.json hbm_gbs ({hbm_src})"),
        "generate": ("hbm", gen_bytes, sum(s["ms_generate"] for s in steps),
                     sum(s["generate_launches"] for s in steps), hbm_peak,
                     f"MEASURED_PEAKS.json hbm_gbs ({hbm_src})"),
    }
    roof = {}
    for name, (bound, byts, ms, launches, peak, src) in classes.items():
        ach = byts / (ms * 1e6) if ms > 0 else 0.0
        bpl = byts / max(launches, 1)
        roof[name] = {"bound": bound, "achieved": round(ach, 2), "peak": round(peak, 1), "unit": "GB/s",
                      "frac": round(ach / peak, 4) if peak else None,
                      "traffic": int(DRAM_PER_ALGO_BYTE[name] * bpl), "launches": launches,
                      "link_traffic": int(LINK_PER_ALGO_BYTE[name] * bpl) if name in LINK_PER_ALGO_BYTE else None,
                      "ms_per_launch": round(ms / max(launches, 1), 4), "bytes_per_launch": round(bpl),
                      "peak_source": src}
    stream_ms = sum(s["ms_stream"] for s in steps)
    dma = {"bytes_per_step": int(sbytes / K), "ms_per_step": round(stream_ms / K, 4),
           "achieved": round(sbytes / (stream_ms * 1e6), 2) if stream_ms > 0 else 0.0, "unit": "GB/s",
           "peak": round(h2d_peak, 1)}
    dom = max(roof, key=lambda k: classes[k][2])
    e2e_walls = res[head].get("e2e_walls", [])
    e2e_reached = res[head].get("e2e_reached", 0)
    # per e2e step: the node pointers uploaded at engine creation, the edges
    # moved by the run, the distance array read back
    h2d_e2e = 4 * (g.n + 1) + res[head].get("e2e_h2d", hs["h2d_bytes_per_run"])
    d2h_e2e = int(sum(s["d2h_bytes"] for s in steps) / K)
    line = {
        "metric": METRIC, "value": hs["value"], "unit": "GTEPS", "n_gpus": dist.world, "steps": K,
        "warmup": a.warmup, "ms_per_step": hs["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(a),
        "schedule": {"policy": head, "scheduler_model": (Path(a.model).name if a.model else
                                                         scheduler.DEFAULT_MODEL.name) if head == "learned" else None,
                     "edge_buffers": nb_learned if head == "learned" else 2,
                     "transfer_record_bytes": esz},
        "e2e": {"value": hs.get("e2e"), "unit": "GTEPS", "h2d_bytes_per_step": int(h2d_e2e),
                "d2h_bytes_per_step": d2h_e2e, "ms_per_step": hs.get("e2e_ms_per_step"),
                "includes": "engine creation (arena, transfer copy), sgw_run with host buffers, engine destruction",
                "transfer_copy": "none: the records read in place, as the drop-in apps do "
                                 "(SGW_OPT_GRAPH_IN_PLACE)",
                "phases_ms": res[head].get("e2e_phases_ms")},
        "e2e_pinned": {"value": hs.get("e2e_pinned"), "unit": "GTEPS", "ms_per_step": hs.get("e2e_pinned_ms_per_step"),
                       "phases_ms": res[head].get("e2e_pinned_phases_ms"),
                       "transfer_copy": "pinned (cudaHostAlloc), the library default"},
        "e2e_warm": {"value": hs["e2e_warm"], "unit": "GTEPS", "ms_per_step":
                     round(dist.max(sum(s["wall_ms"] for s in steps)) / K, 4)},
        "mismatches": check["mismatches"] if a.check == "all" else None,
        "parity": dict(check, against="OpenMP oracle (oracle/sgw_oracle.c), every distinct source, every schedule"),
        "h2d_bytes_per_run": hs["h2d_bytes_per_run"],
        "gpu_launches": int(sum(s["launches"] for s in steps)),
        "roofline": dict(roof[dom], kernel=dom),
        "roofline_kernels": roof,
        "stream_dma": dma,
        "clocks": res[head]["clk"].summary(),
        "breakdown_ms_per_step": {"gather_kernel": round(classes["gather"][2] / K, 4),
                                  "stream_dma": round(stream_ms / K, 4),
                                  "relax": round(classes["relax"][2] / K, 4),
                                  "generate": round(classes["generate"][2] / K, 4)},
        "schedules": sums,
        "setup_s": {"generate_graph": round(t_gen, 2)},
        "timed_region_s": round(res[head]["t_total"], 3),
    }
    if "plain" in sums and head == "learned":
        p, l = sums["plain"], sums["learned"]
        line["learned_over_plain"] = {"speedup": round(l["value"] / p["value"], 3),
                                      "e2e_speedup": round(l["e2e"] / p["e2e"], 3),
                                      "e2e_warm_speedup": round(l["e2e_warm"] / p["e2e_warm"], 3),
                                      "h2d_bytes_ratio": round(l["h2d_bytes_per_run"] / max(p["h2d_bytes_per_run"], 1), 3),
                                      "mispredictions": res["learned"].get("mispredicted")}
    if "rules" in sums and head == "learned":
        r, l = sums["rules"], sums["learned"]
        line["learned_over_rules"] = {"speedup": round(l["value"] / r["value"], 3),
                                      "h2d_bytes_ratio": round(l["h2d_bytes_per_run"] / max(r["h2d_bytes_per_run"], 1), 3),
                                      "rules": "same schedule with the persistence predictor in place of the network"}
    if dist.rank == 0 and cpu:
        line["cpu_baseline"] = cpu
    return line


# ---- one run for a profiler ------------------------------------------------------------
def run_profile(a, dist):
    """What an ncu capture of one run needs: the launch counts of the warm-up
    run (ncu -s) and of the measured run (ncu -c) per kernel class, and the
    measured run's algorithmic bytes to compare with the captured DRAM bytes.
    Per generate step the integer family launches k_generate_count, _scan and
    _write; per relaxation pass k_relax_warp and k_relax_chunks."""
    import numpy as np

    from subway_gb300 import native as N
    from subway_gb300 import scheduler

    policy = "plain" if a.policy == "plain" else "learned"
    weighted = weighted_algo(a.algo)
    g = N.Graph.rmat(a.scale, a.edge_factor, seed=a.seed, weighted=weighted, wmax=64)
    src = [int(s) for s in g.pick_sources(2, seed=a.seed)]
    nb = (a.num_buffers or N.sched_buffers(g, a.budget)) if policy == "learned" else 0
    fl = N.OPT_PROFILE | ((N.OPT_GRAPH_IN_PLACE | N.OPT_PAGEABLE_COPY) if a.profile_engine == "one-query" else 0)
    e = N.Engine(g, budget_bytes=int(a.budget), device=dist.local, flags=fl, num_buffers=nb,
                 gather_ctas=a.gather_ctas, tile_degree_max=a.tile_degree_max, chunk_edges=a.chunk_edges)
    if policy == "learned":
        e.set_policy("learned", scheduler.load_default(dist.local))
    out = np.empty(g.n, np.uint32)
    _, w = e.run(a.algo, a.mode, src[1], out=out)
    _, st = e.run(a.algo, a.mode, src[0], out=out)
    in_place = e.host_copy_bytes() == 0
    esz = (8 if weighted else 4) if in_place else transfer_record_bytes(g.n, weighted, a.no_pack)
    keys = ("gather_launches", "relax_launches", "generate_launches", "launches")
    return {"profile_run": policy, "engine": a.profile_engine, "records_in_place": in_place,
            "workload": workload_config(a)["workload"],
            "warm": {k: w[k] for k in keys},
            "run": {k: st[k] for k in keys + ("ms_gather", "ms_relax", "ms_generate", "ms_device", "relaxed_edges",
                                              "relaxed_sources", "active_vertices", "gather_bytes", "h2d_bytes")},
            "algorithmic_bytes": {"gather": st["gather_bytes"],
                                  "relax": st["relaxed_sources"] * 17 + st["relaxed_edges"] * (esz + 4),
                                  "generate": st["generate_launches"] * 2 * g.n + st["active_vertices"] * 16},
            "record_bytes": esz}


# ---- the scale-27 suite --------------------------------------------------------------
def run_suite(a, dist):
    """The full algorithm suite at R-MAT scale 27 (2^27 vertices, edge factor
    16) under a 4 GB device budget: BFS, CC on the symmetrised graph, SSWP
    with weights in [1, 1024] (8-byte records), an Erdos-Renyi graph of the
    same size as a low-skew control, and optionally delta-PageRank; sync and
    async; one source from the largest WCC.  Every integer result is compared
    with the OpenMP oracle; PageRank with the FP64 bulk-synchronous oracle."""
    import numpy as np

    from oracle import oracle
    from subway_gb300 import native as N

    dev = dist.local
    scale, seed = 27, 27
    cases = []

    def run_cases(g, label, algo, budget, ref_fn):
        src = int(g.pick_sources(1, seed=seed)[0]) if algo not in ("cc", "pr") else 0
        t = time.perf_counter()
        eng = N.Engine(g, budget_bytes=int(budget), device=dev, flags=N.OPT_PROFILE)
        create_s = time.perf_counter() - t
        t = time.perf_counter()
        ref = ref_fn(src)
        oracle_s = time.perf_counter() - t
        for mode in ("sync", "async"):
            t = time.perf_counter()
            kw = {"pr_acc": 1e-6} if algo == "pr" else {}
            vals, st = eng.run(algo, mode, src, **kw)
            wall = time.perf_counter() - t
            c = {"graph": label, "algo": algo, "mode": mode, "budget_bytes": int(budget), "source": src,
                 "edges": g.m, "ms_device": round(st["ms_device"], 1), "ms_run_wall": round(wall * 1e3, 1),
                 "engine_create_s": round(create_s, 2), "h2d_bytes": st["h2d_bytes"],
                 "global_iterations": st["global_iterations"], "oracle_s": round(oracle_s, 1)}
            if algo == "pr":
                c["max_abs"] = float(np.max(np.abs(vals.astype(np.float64) - ref)))
                c["max_rel"] = float(np.max(np.abs(vals.astype(np.float64) - ref) / np.maximum(ref, 1e-30)))
            else:
                c["mismatches"] = int(np.count_nonzero(vals != ref))
                c["gteps"] = round(st["reached_edges"] / (st["ms_device"] * 1e6), 3)
            cases.append(c)
            print(json.dumps(c), file=sys.stderr, flush=True)
        eng.close()

    g = N.Graph.rmat(scale, 16, seed=seed)
    run_cases(g, f"rmat{scale}", "bfs", 4e9, lambda s: oracle.run("bfs", g.node_pointer, g.ends, s, parallel=True))
    if a.suite_pr:
        run_cases(g, f"rmat{scale}", "pr", 6e9,
                  lambda s: oracle.pagerank(g.node_pointer, g.ends, init=float(np.float32(0.15)),
                                            acc=float(np.float32(1e-6)), damping=float(np.float32(0.85)),
                                            parallel=True)[0])
    gs = g.symmetrize()
    g.close()
    run_cases(gs, f"rmat{scale}-symmetrised", "cc", 4e9,
              lambda s: oracle.run("cc", gs.node_pointer, gs.ends, 0, parallel=True))
    gs.close()
    gw = N.Graph.rmat(scale, 16, seed=seed, weighted=True, wmax=1024)
    run_cases(gw, f"rmat{scale}-w1024", "sswp", 4e9,
              lambda s: oracle.run("sswp", gw.node_pointer, gw.edges, s, parallel=True))
    gw.close()
    ge = N.Graph.er(1 << scale, 1 << 31, seed=seed)
    run_cases(ge, f"er{scale}", "bfs", 4e9, lambda s: oracle.run("bfs", ge.node_pointer, ge.ends, s, parallel=True))
    ge.close()
    bad = sum(c.get("mismatches", 0) for c in cases)
    return {"suite": "scale27", "metric": "GTEPS per run (device time) with the oracle's verdict",
            "cases": cases, "mismatches": bad, "n_gpus": dist.world, "data": "synthetic",
            "pr_run": bool(a.suite_pr)}


# ---- the reference build ------------------------------------------------------------
def run_reference_process(exe, path, source, env, timeout):
    """One reference process; (wall after its CUDA context is up, its read time, its processing time)."""
    t0 = time.perf_counter()
    p = subprocess.Popen([str(exe), "--input", str(path), "--source", str(source)], stdout=subprocess.PIPE,
                         stderr=subprocess.PIPE, text=True, env=env)
    first = [None]
    lines = []

    def reader():
        for ln in p.stdout:
            if first[0] is None:
                first[0] = time.perf_counter()  # "Reading the input graph ..." (flushed by endl)
            lines.append(ln)

    th = threading.Thread(target=reader, daemon=True)
    th.start()
    try:
        p.wait(timeout=timeout)
    except subprocess.TimeoutExpired:
        p.kill()
        p.wait()
        return None, "timeout"
    th.join(timeout=10)
    t_end = time.perf_counter()
    text = "".join(lines)
    rd = re.search(r"Graph Reading finished in ([0-9.eE+-]+) \(s\)", text)
    pf = re.search(r"Processing finished in ([0-9.eE+-]+) \((m?s)\)", text)
    if p.returncode != 0 or not rd or not pf or first[0] is None:
        return None, f"rc={p.returncode}: {p.stderr.read().strip()[-200:]}"
    proc_s = float(pf.group(1)) / (1000.0 if pf.group(2) == "ms" else 1.0)
    return {"wall_s": t_end - t0, "after_context_s": t_end - first[0], "read_s": float(rd.group(1)),
            "processing_s": proc_s}, None


def run_reference(a, dist):
    """The reference's own build on the same graph and budget.  Only the
    oracle is imported here: the graph file, the sources and the reached-edge
    counts come from oracle/sgw_oracle.c, never from the engine library."""
    from oracle import build_ref, oracle

    exe = build_ref.binary(f"{a.algo}-{a.mode}")
    line = {"impl": "reference", "metric": METRIC, "unit": "GTEPS", "n_gpus": dist.world,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": workload_config(a)}
    if not exe.exists():
        try:
            build_ref.build_ref()
        except Exception as exc:  # noqa: BLE001
            line["unavailable"] = f"reference build failed: {str(exc).splitlines()[0][:200]}"
            return line
    if not exe.exists():
        line["unavailable"] = "reference sources not staged under oracle/_ref"
        return line
    weighted = weighted_algo(a.algo)
    tmp = Path(tempfile.mkdtemp(prefix="sgw_ref_"))
    path = tmp / ("g.bwcsr" if weighted else "g.bcsr")
    t = time.time()
    oracle.rmat_write(path, a.scale, a.edge_factor, seed=a.seed, weighted=weighted, wmax=64)
    npt, ed = oracle.read_csr(path)
    sources = [int(s) for s in oracle.pick_sources(npt, ed, a.sources, seed=a.seed)]
    reached = dict(zip(sources, (int(x) for x in oracle.reached_edges(npt, ed, sources))))
    del npt, ed
    t_setup = time.time() - t
    env = dict(os.environ, SUBWAY_BUDGET_BYTES=str(int(a.budget)), MALLOC_MMAP_THRESHOLD_="4096",
               GLIBC_TUNABLES="glibc.malloc.mmap_threshold=4096")
    # Every process is a cold start of the reference (it reads the graph, pins
    # its two edge arrays, generates and runs once); one warm-up process fills
    # the page cache with the graph file.
    warm = min(a.warmup, 1)
    runs = []
    t_arm = time.time()
    k = 0
    err = None
    while len(runs) < a.steps:
        if k >= warm and len(runs) >= 2 and time.time() - t_arm > a.ref_time_limit:
            break
        s = sources[k % len(sources)]
        r, err = run_reference_process(exe, path, s, env, timeout=1800)
        if r is None:
            break
        if k >= warm:
            r["source"] = s
            runs.append(r)
        k += 1
    try:
        path.unlink()
        tmp.rmdir()
    except OSError:
        pass
    if not runs:
        line["unavailable"] = f"reference run failed {err}"
        return line
    tot_reached = sum(reached[r["source"]] for r in runs)
    e2e_s = sum(r["after_context_s"] - r["read_s"] for r in runs)
    proc_s = sum(r["processing_s"] for r in runs)
    value = tot_reached / e2e_s / 1e9
    n_runs = len(runs)
    line.update({
        "value": round(value, 4), "steps": n_runs, "warmup": warm, "steps_requested": a.steps,
        "ms_per_step": round(e2e_s / n_runs * 1e3, 2),
        "e2e": {"value": round(value, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "processing": {"value": round(tot_reached / proc_s / 1e9, 4), "unit": "GTEPS",
                       "ms_per_step": round(proc_s / n_runs * 1e3, 2),
                       "what": "the reference's own 'Processing finished' timer (subway/sssp-async.cu:69,124)"},
        "cpu_baseline": {"value": round(value, 4), "unit": "GTEPS", "cores": os.cpu_count(), "kind": "reference",
                         "sample": f"{n_runs} runs of the reference {a.algo}-{a.mode} build (its GPU kernels and "
                                   f"{min(64, os.cpu_count() or 1)}-thread host gather): process wall time after "
                                   "its CUDA context is up, minus its own 'Graph Reading finished' time; "
                                   "m_reached from the oracle"},
        "per_process_s": {"wall": round(sum(r["wall_s"] for r in runs) / n_runs, 3),
                          "read": round(sum(r["read_s"] for r in runs) / n_runs, 3),
                          "processing": round(proc_s / n_runs, 3)},
        "setup_s": {"write_graph_and_sources": round(t_setup, 1)},
    })
    return line


def main():
    a = parse_args()
    dist = Dist(a.gpus)
    if a.profile_run:
        line = run_profile(a, dist)
    elif a.suite:
        line = run_suite(a, dist)
    elif a.impl == "reference":
        if dist.rank != 0:
            return 0
        line = run_reference(a, dist)
    else:
        line = run_ours(a, dist)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    if (a.impl == "ours" or a.suite) and line.get("mismatches"):
        print(f"bench: {line['mismatches']} values differ from the oracle", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())

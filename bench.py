"""Benchmark: out-of-HBM-budget SSSP-async on weighted R-MAT scale 24.

Workload (one "step" = one SSSP-async run from one source, cycling over the
sources): R-MAT(0.57, 0.19, 0.19, 0.05), 2^24 vertices, edge factor 16,
self-loops and duplicates removed, uint32 weights uniform in [1, 64], 8
seeded sources from the largest weakly connected component, device-memory
budget 1 GB (about 0.46 of the 2.1 GB of edge records stays resident).

Metric: GTEPS = reached edges (Graph500 m_reached) / processing time, plus
the bytes the device read from host memory per run.  Both schedules are
timed, the plain one (the reference's: every active edge compacted and sent
each iteration, async partitions relaxed to convergence) first; the learned
one is the headline line and `plain_policy` / `learned_over_plain` carry the
comparison (speed-up, H2D bytes ratio, mispredictions of one traced run).
  value  device-timed processing loop (CUDA events on the engine's compute
         stream, from after the first generate to the end of the loop, the
         reference's t_processing convention)
  e2e    the whole sgw_run() call through the C ABI with host buffers: state
         init, every host->device edge transfer, and the device->host copy of
         the distances.

--impl reference runs the reference's own sssp-async build (oracle/_ref,
compiled from the upstream sources for sm_103a) on the same graph file with
the same device budget, and reports its own "Processing finished" time.
Under torchrun every rank runs an independent replica (the path does not
shard); rank 0 prints the JSON line.
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


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=24)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--budget", type=float, default=1e9)
    ap.add_argument("--algo", default="sssp")
    ap.add_argument("--mode", default="async")
    ap.add_argument("--sources", type=int, default=8)
    ap.add_argument("--seed", type=int, default=24)
    ap.add_argument("--cpu-sample", type=int, default=8, help="sources timed for the CPU baseline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-pack", action="store_true", help="move the reference's 8-byte records")
    ap.add_argument("--gather-ctas", type=int, default=0)
    ap.add_argument("--tile-degree-max", type=int, default=0)
    ap.add_argument("--chunk-edges", type=int, default=0)
    ap.add_argument("--inner-batch", type=int, default=0)
    ap.add_argument("--policy", default="both", choices=["plain", "learned", "both"],
                    help="both: time the plain (reference) schedule, then the learned one (headline)")
    ap.add_argument("--model", default="", help="scheduler model file; 'none' = persistence predictor")
    ap.add_argument("--num-buffers", type=int, default=0,
                    help="edge buffers of the learned policy (0 = sgw_sched_buffers' choice)")
    ap.add_argument("--sched-inner", type=int, default=0,
                    help="learned policy: inner-iteration cap of kept ranges predicted active (0 = library default)")
    ap.add_argument("--sched-defer", type=int, default=0,
                    help="learned policy: frontier per global iteration in 1/1000 of the edges (0 = whole)")
    ap.add_argument("--sched-permille", type=int, default=0,
                    help="learned policy: predicted active fraction (1/1000) that caps a kept range (0 = default)")
    return ap.parse_args()


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


def workload_config(a, extra=None):
    c = {"workload": f"rmat{a.scale}-ef{a.edge_factor}-w64 {a.algo}-{a.mode}, device budget "
                     f"{a.budget / 1e9:g} GB, {a.sources} sources from the largest WCC",
         "graph": f"R-MAT(0.57,0.19,0.19,0.05) scale {a.scale}, edge factor {a.edge_factor}, "
                  "dedup, no self-loops, u32 weights in [1,64]",
         "budget_bytes": int(a.budget), "sources": a.sources, "seed": a.seed,
         "l2": f"inputs larger than L2: edges stay in host memory, vertex state "
               f"~{18 * (1 << a.scale) / 1e6:.0f} MB in HBM",
         "parallelism": "replicas"}
    if extra:
        c.update(extra)
    return c


def cpu_baseline(g, sources, algo, count):
    """OpenMP CPU implementation (oracle/sgw_oracle.c omp_*) on this host."""
    from oracle import oracle
    e = g.edges if algo in ("sssp", "sswp") else g.ends
    npt = g.node_pointer
    reached, secs = 0, 0.0
    deg = g.out_degree()
    for s in list(sources)[:count]:
        t = time.perf_counter()
        v = oracle.run(algo, npt, e, int(s), parallel=True)
        secs += time.perf_counter() - t
        reached += int(deg[v != 4294967294].sum())
    return {"value": reached / secs / 1e9, "unit": "GTEPS", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{count} full {algo} runs (OpenMP frontier label-correcting) on the same graph",
            "seconds": round(secs, 3)}


def run_ours(a, dist):
    from subway_gb300 import native as N

    dev = dist.local
    t0 = time.time()
    weighted = a.algo in ("sssp", "sswp")
    g = N.Graph.rmat(a.scale, a.edge_factor, seed=a.seed, weighted=weighted, wmax=64)
    sources = g.pick_sources(a.sources, seed=a.seed)
    t_gen = time.time() - t0
    flags = N.OPT_PROFILE | (N.OPT_NO_PACK if a.no_pack else 0)
    h2d_peak, d2h_peak = probe_link(N, dev)
    import numpy as np
    out = np.empty(g.n, np.float32 if a.algo == "pr" else np.uint32)  # host result buffer

    def engine(policy):
        nb = (a.num_buffers or N.sched_buffers(g, a.budget)) if policy == "learned" else 0
        e = N.Engine(g, budget_bytes=int(a.budget), device=dev, flags=flags, gather_ctas=a.gather_ctas,
                     tile_degree_max=a.tile_degree_max, chunk_edges=a.chunk_edges,
                     inner_batch=a.inner_batch, num_buffers=nb, sched_inner=a.sched_inner,
                     sched_active_permille=a.sched_permille, sched_defer_permille=a.sched_defer)
        if policy == "learned":
            from subway_gb300 import scheduler
            model = None if a.model == "none" else (N.Mlp.load(a.model, dev) if a.model else
                                                     scheduler.load_default(dev))
            e.set_policy("learned", model)
            e.model_name = "persistence" if model is None else Path(a.model or scheduler.DEFAULT_MODEL).name
        e.edge_buffers = nb or 2
        e.dma_gbs = round(e.dma_rate(), 1)
        return e

    def measure(eng):
        for k in range(a.warmup):
            eng.run(a.algo, a.mode, int(sources[k % len(sources)]), out=out)
        steps = []
        dist.barrier()
        with ClockSampler(dev) as clk:
            t_start = time.perf_counter()
            for k in range(a.steps):
                t = time.perf_counter()
                _, st = eng.run(a.algo, a.mode, int(sources[k % len(sources)]), out=out)
                st["wall_ms"] = (time.perf_counter() - t) * 1e3
                steps.append(st)
            t_total = time.perf_counter() - t_start
        dist.barrier()
        return steps, clk, t_total

    plain_summary = None
    if a.policy in ("plain", "both"):
        eng = engine("plain")
        steps, clk, t_total = measure(eng)
        if a.policy == "both":
            r = dist.sum(sum(s["reached_edges"] for s in steps))
            plain_summary = {"value": round(r / (dist.max(sum(s["ms_device"] for s in steps)) * 1e6), 4),
                             "e2e": round(r / (dist.max(sum(s["wall_ms"] for s in steps)) * 1e6), 4),
                             "h2d_bytes_per_run": int(sum(s["h2d_bytes"] for s in steps) / a.steps),
                             "ms_per_step": round(sum(s["ms_device"] for s in steps) / a.steps, 4),
                             "iterations_per_step": round(sum(s["global_iterations"] for s in steps) / a.steps, 2)}
            eng.close()
    mispredicted = None
    if a.policy in ("learned", "both"):
        eng = engine("learned")
        steps, clk, t_total = measure(eng)
        # one more run, untimed, with the range trace on: how often the
        # predictions behind its transfer decisions were wrong
        from subway_gb300 import scheduler
        eng.trace_enable(True)
        eng.run(a.algo, a.mode, int(sources[0]), out=out)
        mispredicted = scheduler.mispredictions(eng.range_trace())
        eng.trace_enable(False)
    reached = sum(s["reached_edges"] for s in steps)
    dev_ms = sum(s["ms_device"] for s in steps)
    wall_ms = sum(s["wall_ms"] for s in steps)
    # whole job: all ranks' reached edges over the slowest rank's time
    tot_reached = dist.sum(reached)
    dev_ms_max = dist.max(dev_ms)
    wall_ms_max = dist.max(wall_ms)
    K = a.steps
    value = tot_reached / (dev_ms_max * 1e6)
    e2e = tot_reached / (wall_ms_max * 1e6)
    h2d = sum(s["h2d_bytes"] for s in steps) / K
    d2h = sum(s["d2h_bytes"] for s in steps) / K
    # dominant kernel class by device time
    cls = {"gather": sum(s["ms_gather"] for s in steps), "relax": sum(s["ms_relax"] for s in steps),
           "generate": sum(s["ms_generate"] for s in steps)}
    launches = {"gather": sum(s["gather_launches"] for s in steps),
                "relax": sum(s["relax_launches"] for s in steps),
                "generate": sum(s["generate_launches"] for s in steps)}
    esz = 8 if weighted and a.no_pack else 4  # device edge record (packed when weighted)
    relax_bytes = sum(s["relaxed_sources"] * 17 + s["relaxed_edges"] * (esz + 4) for s in steps)
    gen_bytes = sum(s["generate_launches"] * 2 * g.n + s["active_vertices"] * 16 for s in steps)
    hbm_peak, hbm_src = measured_peaks()
    kernels = {
        "gather": {"bound": "host_link", "bytes": h2d * K, "ms": cls["gather"], "peak": h2d_peak,
                   "peak_src": "measured pinned cudaMemcpyAsync H2D on this GPU (bench)"},
        "relax": {"bound": "hbm", "bytes": relax_bytes, "ms": cls["relax"], "peak": hbm_peak,
                  "peak_src": f"MEASURED_PEAKS.json hbm_gbs ({hbm_src})"},
        "generate": {"bound": "hbm", "bytes": gen_bytes, "ms": cls["generate"], "peak": hbm_peak,
                     "peak_src": f"MEASURED_PEAKS.json hbm_gbs ({hbm_src})"},
    }
    dom = max(cls, key=cls.get)
    roof = {}
    for name, kv in kernels.items():
        ach = kv["bytes"] / (kv["ms"] * 1e6) if kv["ms"] > 0 else 0.0
        roof[name] = {"bound": kv["bound"], "achieved": round(ach, 2), "peak": round(kv["peak"], 1),
                      "unit": "GB/s", "frac": round(ach / kv["peak"], 4) if kv["peak"] else None,
                      "traffic": None, "launches": launches[name],
                      "ms_per_launch": round(kv["ms"] / max(launches[name], 1), 4),
                      "bytes_per_launch": round(kv["bytes"] / max(launches[name], 1)),
                      "peak_source": kv["peak_src"]}
    for name in roof:
        roof[name]["traffic"] = traffic_per_launch(name, roof[name]["bytes_per_launch"])
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "GTEPS", "n_gpus": dist.world, "steps": K,
        "warmup": a.warmup, "ms_per_step": round(dev_ms_max / K, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(a, {"policy": "plain" if a.policy == "plain" else "learned",
                                      "scheduler_model": getattr(eng, "model_name", None),
                                      "edge_buffers": getattr(eng, "edge_buffers", 2),
                                      "transfer_copy_dma_gbs": getattr(eng, "dma_gbs", None),
                                      "transfer_record_bytes": 4 if (weighted and not a.no_pack) or not weighted else 8}),
        "plain_policy": plain_summary,
        "learned_over_plain": (None if not plain_summary else
                               {"speedup": round(value / plain_summary["value"], 3),
                                "e2e_speedup": round(e2e / plain_summary["e2e"], 3),
                                "h2d_bytes_ratio": round(h2d / max(plain_summary["h2d_bytes_per_run"], 1), 3),
                                "mispredictions": mispredicted}),
        "e2e": {"value": round(e2e, 4), "unit": "GTEPS", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(wall_ms_max / K, 4)},
        "h2d_bytes_per_run": int(h2d),
        "gpu_launches": int(sum(s["launches"] for s in steps)),
        "roofline": dict(roof[dom], kernel=dom),
        "roofline_kernels": roof,
        "clocks": clk.summary(),
        "breakdown_ms_per_step": {k: round(v / K, 4) for k, v in cls.items()},
        "iterations_per_step": round(sum(s["global_iterations"] for s in steps) / K, 2),
        "setup_s": {"generate_graph": round(t_gen, 2)},
        "timed_region_s": round(t_total, 3),
    }
    if dist.rank == 0 and not a.no_cpu:
        line["cpu_baseline"] = cpu_baseline(g, sources, a.algo, a.cpu_sample)
    return line


def probe_link(N, dev):
    import ctypes as C
    h, d = C.c_double(), C.c_double()
    N.check(N.lib().sgw_probe_link(dev, 1 << 30, 5, C.byref(h), C.byref(d)), "sgw_probe_link")
    return h.value, d.value


# DRAM bytes (read + write) per algorithmic byte, from ncu captures on small
# cases: gather from profiles/k_gather_v_rmat21.md (launch 3); relax and
# generate from every launch of one RMAT-22 SSSP-async run under a 300 MB
# budget (profiles/dram_traffic_rmat22_sssp_async.md; ncu empties the caches
# before each launch, so these are cold-cache figures).  A full-size launch's
# traffic is this ratio times its algorithmic bytes.
DRAM_PER_ALGO_BYTE = {"gather": 1.21, "relax": 0.93, "generate": 2.36}


def traffic_per_launch(name, bytes_per_launch):
    r = DRAM_PER_ALGO_BYTE.get(name)
    return None if r is None else int(r * bytes_per_launch)


def run_reference(a, dist):
    """The reference's sssp-async build on the same graph and budget."""
    from oracle import build_ref, oracle
    from subway_gb300 import native as N

    exe = build_ref.binary(f"{a.algo}-{a.mode}")
    line = {"impl": "reference", "metric": METRIC, "unit": "GTEPS", "n_gpus": dist.world, "steps": a.steps,
            "warmup": a.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32", "data": "synthetic", "config": workload_config(a)}
    if not exe.exists():
        try:
            build_ref.build_ref()
        except Exception as exc:  # noqa: BLE001
            line["unavailable"] = f"reference build failed: {str(exc).splitlines()[0][:200]}"
            return line
    if not exe.exists():
        line["unavailable"] = "reference sources not staged under oracle/_ref"
        return line
    weighted = a.algo in ("sssp", "sswp")
    g = N.Graph.rmat(a.scale, a.edge_factor, seed=a.seed, weighted=weighted, wmax=64)
    sources = g.pick_sources(a.sources, seed=a.seed)
    deg = g.out_degree()
    e = g.edges if weighted else g.ends
    reached = {}
    for s in sources:
        v = oracle.run(a.algo, g.node_pointer, e, int(s), parallel=True)
        reached[int(s)] = int(deg[v != 4294967294].sum())
    tmp = Path(tempfile.mkdtemp(prefix="sgw_ref_"))
    path = tmp / ("g.bwcsr" if weighted else "g.bcsr")
    g.save(path)
    del g
    env = dict(os.environ, SUBWAY_BUDGET_BYTES=str(int(a.budget)), MALLOC_MMAP_THRESHOLD_="4096",
               GLIBC_TUNABLES="glibc.malloc.mmap_threshold=4096")
    times, walls = [], []
    for k in range(a.warmup + a.steps):
        s = int(sources[k % len(sources)])
        t = time.perf_counter()
        p = subprocess.run([str(exe), "--input", str(path), "--source", str(s)], capture_output=True,
                           text=True, env=env, timeout=900)
        w = time.perf_counter() - t
        m = re.search(r"Processing finished in ([0-9.eE+-]+) \((m?s)\)", p.stdout)
        if p.returncode != 0 or not m:
            line["unavailable"] = f"reference run failed rc={p.returncode}: {p.stderr.strip()[-200:]}"
            return line
        secs = float(m.group(1)) / (1000.0 if m.group(2) == "ms" else 1.0)
        if k >= a.warmup:
            times.append((s, secs))
            walls.append(w)
    try:
        path.unlink()
        tmp.rmdir()
    except OSError:
        pass
    tot_reached = sum(reached[s] for s, _ in times)
    tot_s = sum(t for _, t in times)
    value = tot_reached / tot_s / 1e9
    line.update({
        "value": round(value, 4), "ms_per_step": round(tot_s / len(times) * 1e3, 3),
        "e2e": {"value": round(value, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_baseline": {"value": round(value, 4), "unit": "GTEPS", "cores": os.cpu_count(), "kind": "reference",
                         "sample": f"{len(times)} runs of the reference {a.algo}-{a.mode} build (its GPU kernels "
                                   f"and {min(64, os.cpu_count() or 1)}-thread host gather), 'Processing finished' "
                                   "time; m_reached from the oracle"},
        "process_wall_s_per_step": round(sum(walls) / len(walls), 3),
    })
    return line


def main():
    a = parse_args()
    dist = Dist(a.gpus)
    if a.impl == "reference":
        if dist.rank != 0:
            return
        line = run_reference(a, dist)
    else:
        line = run_ours(a, dist)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

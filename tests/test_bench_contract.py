"""The engine arm's JSON line (CPU only): bench.run_ours driven end to end
with a stand-in engine whose answers come from the oracle, so that the line
the benchmark prints keeps its contract (keys, units, e2e copies, roofline,
CPU baseline, launches, parity) whatever changes in how it is assembled.
The real engine's numbers are measured on a GPU."""
import json

import numpy as np

INF = 4294967294


def test_engine_arm_line_contract(native, orc, monkeypatch):
    import bench
    from subway_gb300 import scheduler

    N = native
    made = []

    class StandInEngine:
        def __init__(self, g, budget_bytes=0, device=0, flags=0, **kw):
            self.g, self.flags = g, flags
            made.append(flags)

        def set_policy(self, policy, model=None):
            self.policy = policy

        def trace_enable(self, on=True):
            pass

        def range_trace(self):
            return np.zeros(0, N.RANGE_REC)

        def host_copy_bytes(self):
            return 0 if self.flags & N.OPT_GRAPH_IN_PLACE else 5 * self.g.m

        def close(self):
            pass

        def run(self, algo, mode, source=0, out=None, **kw):
            e = self.g.edges if self.g.weighted else self.g.ends
            vals = orc.run(algo, self.g.node_pointer, e, source)
            reached = int(self.g.out_degree()[vals != INF].astype(np.uint64).sum())
            if out is not None:
                out[:] = vals
            st = {k: 0 for k, _ in N.RunStats._fields_}
            st.update(global_iterations=5, partitions=7, reached_edges=reached, ms_device=2.0, ms_gather=1.2,
                      ms_relax=0.9, ms_generate=0.2, launches=40, gather_launches=7, relax_launches=25,
                      generate_launches=5, relaxed_edges=reached, relaxed_sources=100, gather_bytes=5 * reached,
                      h2d_bytes=5 * reached, d2h_bytes=4 * self.g.n, active_vertices=100, active_edges=reached)
            return vals, st

    monkeypatch.setattr(N, "Engine", StandInEngine)
    monkeypatch.setattr(bench, "probe_link", lambda _N, _dev: (211.6, 200.0))
    monkeypatch.setattr(scheduler, "load_default", lambda dev=0: None)
    a = bench.parse_args(["--scale", "10", "--budget", "1e6", "--sources", "3", "--steps", "3", "--warmup", "3"])
    line = json.loads(json.dumps(bench.run_ours(a, bench.Dist(1))))

    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "clocks",
              "gpu_launches", "mismatches", "parity"):
        assert k in line, k
    assert line["unit"] == "GTEPS" and line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["steps"] == 3 and line["warmup"] == 3 and line["mismatches"] == 0
    assert line["config"] == bench.workload_config(a)
    assert line["value"] > 0 and line["gpu_launches"] == 3 * 40
    e2e = line["e2e"]
    assert e2e["value"] > 0 and e2e["unit"] == "GTEPS"
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] == 4 * 1024
    assert set(e2e["phases_ms"]) == {"create", "run", "destroy"}
    assert line["e2e_pinned"]["value"] > 0
    r = line["roofline"]
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= set(r)
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-3 * max(1.0, r["frac"])
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] > 0 and cpu["unit"] == "GTEPS"
    assert line["parity"]["checked_sources"] == 3 and line["parity"]["mismatches"] == 0
    # the one-query e2e engines were made as the drop-in apps make them
    one_query = N.OPT_GRAPH_IN_PLACE | N.OPT_PAGEABLE_COPY
    assert any(f & one_query == one_query for f in made) and any(not f & one_query for f in made)

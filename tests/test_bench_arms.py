"""bench.py's reference arm on CPU with a stand-in for the reference binary:
it must produce its JSON line from the oracle alone, without loading the
engine library (the driver checks which native libraries each arm maps)."""
import json
import os
import subprocess
import sys
import textwrap
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

FAKE = """#!/bin/bash
echo "Reading the input graph from the following file:"
echo ">> $2"
echo "Graph Reading finished in 0.05 (s)."
sleep 0.05
echo "1 Inner Iteration in Global Iteration 1, Partition 0"
echo "Processing finished in 0.02 (s)."
echo "Results of first 30 nodes:"
"""


def test_reference_arm_loads_no_engine_library(tmp_path):
    exe = tmp_path / "sssp-async"
    exe.write_text(FAKE)
    exe.chmod(0o755)
    code = textwrap.dedent(f"""
        import json, sys
        sys.path.insert(0, {str(ROOT)!r})
        import bench
        from oracle import build_ref
        build_ref.binary = lambda app, fixed=False: __import__("pathlib").Path({str(exe)!r})
        a = bench.parse_args(["--impl", "reference", "--scale", "11", "--sources", "3", "--steps", "3",
                              "--warmup", "2"])
        line = bench.run_reference(a, bench.Dist(1))
        maps = open("/proc/self/maps").read()
        print(json.dumps({{"line": line, "engine_module": "subway_gb300" in sys.modules,
                          "engine_lib": "libsubwaygb" in maps}}))
    """)
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert p.returncode == 0, p.stderr
    r = json.loads(p.stdout.strip().splitlines()[-1])
    assert not r["engine_module"] and not r["engine_lib"]
    line = r["line"]
    assert "unavailable" not in line, line
    assert line["impl"] == "reference" and line["steps"] == 3 and line["warmup"] == 1
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["per_process_s"]["read"] == 0.05
    # same workload description as the engine's arm
    a = __import__("bench").parse_args(["--scale", "11", "--sources", "3"])
    assert line["config"] == __import__("bench").workload_config(a)

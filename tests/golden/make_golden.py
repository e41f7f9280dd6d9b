"""Generates the golden fixtures: outputs of the Subway reference build itself.

Runs on a machine with a GPU, after `__graft_entry__.build()` has compiled the
reference apps into oracle/_ref (bin/ as shipped, bin_fixed/ with the
host-gather chunk rounded up).  For a seeded R-MAT graph it runs every app
of both builds with --output and stores the values, with a digest of the
graph so the CPU tests can regenerate the same graph and check the oracle
against the reference's answers.

    python tests/golden/make_golden.py OUT_DIR
writes OUT_DIR/ref_rmat13.npz (copied into tests/golden/ and committed).
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

SCALE, EF, SEED, WMAX = 13, 16, 1301, 64
APPS = [f"{a}-{m}" for a in ("bfs", "cc", "sssp", "sswp", "pr") for m in ("sync", "async")]


def digest(g) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(g.node_pointer).tobytes())
    h.update(np.ascontiguousarray(g.edges).tobytes())
    return h.hexdigest()


def graphs():
    from subway_gb300 import native as N
    gu = N.Graph.rmat(SCALE, EF, seed=SEED, weighted=False)
    gw = N.Graph.rmat(SCALE, EF, seed=SEED, weighted=True, wmax=WMAX)
    return gu, gw


def run_app(exe: Path, graph_path: Path, source, out_path: Path) -> list[str]:
    env = dict(os.environ, MALLOC_MMAP_THRESHOLD_="4096", GLIBC_TUNABLES="glibc.malloc.mmap_threshold=4096")
    cmd = [str(exe), "--input", str(graph_path), "--output", str(out_path)]
    if source is not None:
        cmd += ["--source", str(source)]
    p = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=300)
    if p.returncode != 0:
        raise RuntimeError(f"{exe.name} failed ({p.returncode}): {p.stderr[-300:]}")
    return p.stdout.splitlines()


def main(out_dir: Path):
    from oracle import build_ref
    gu, gw = graphs()
    src = int(gw.pick_sources(1, seed=SEED)[0])
    tmp = Path(tempfile.mkdtemp(prefix="sgw_golden_"))
    pu, pw = tmp / "g.bcsr", tmp / "g.bwcsr"
    gu.save(pu)
    gw.save(pw)
    arrays = {"digest_unweighted": np.array(digest(gu)), "digest_weighted": np.array(digest(gw)),
              "params": np.array([SCALE, EF, SEED, WMAX, src], np.int64)}
    for variant in ("shipped", "fixed"):
        for app in APPS:
            algo = app.split("-")[0]
            path = pw if algo in ("sssp", "sswp") else pu
            sources = [None] if algo in ("cc", "pr") else [0, src]
            for s in sources:
                out = tmp / "out.txt"
                log = run_app(build_ref.binary(app, fixed=(variant == "fixed")), path, s, out)
                vals = np.loadtxt(out, dtype=np.float64 if algo == "pr" else np.uint64)[:, 1]
                key = f"{variant}/{app}" + ("" if s is None else f"/s{s}")
                arrays[key] = vals.astype(np.float32 if algo == "pr" else np.uint32)
                it = [ln for ln in log if ln.startswith("Number of iterations")]
                print(key, len(vals), it[0] if it else "", flush=True)
    out_dir.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(out_dir / f"ref_rmat{SCALE}.npz", **arrays)
    print("wrote", out_dir / f"ref_rmat{SCALE}.npz")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent)

"""Generates the golden fixtures: outputs of the Subway reference build itself.

Runs on a machine with a GPU, after `__graft_entry__.build()` has compiled the
reference apps into oracle/_ref (bin/ as shipped, bin_fixed/ with the
host-gather chunk rounded up, shared/subgraph_generator.cu:75).  Each set runs
reference apps with --output on a seeded R-MAT graph written by the oracle's
generator (byte-identical to the engine's) and stores either the values
(small graphs) or, per source, a SHA-256 digest of the values and how many
vertices differ from the OpenMP oracle (large graphs, whose arrays are too
big to commit).

    python tests/golden/make_golden.py rmat13 [OUT_DIR]  # every app, sources 0 and one
                                                         # picked, both builds -> ref_rmat13.npz
    python tests/golden/make_golden.py rmat16 [OUT_DIR]  # bfs-sync and sssp-sync from source 0,
                                                         # no budget, both builds -> ref_rmat16.npz
    python tests/golden/make_golden.py rmat24 [OUT_DIR]  # sssp-async under a 1 GB budget, 8
                                                         # sources, both builds -> ref_rmat24_sssp_async_1gb.json
    python tests/golden/make_golden.py rmat28 [OUT_DIR]  # sssp-async under an 8 GB budget, 2 of
                                                         # the 16 sources, fixed build -> ref_rmat28_sssp_async_8gb.json
OUT_DIR defaults to tests/golden/.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

APPS = [f"{a}-{m}" for a in ("bfs", "cc", "sssp", "sswp", "pr") for m in ("sync", "async")]
INF = 4294967294
# name: scale, edge factor, seed, weight max, apps, device budget (0: the
# reference's own rule), sources (None: 0 and one picked; int: that many picked)
SETS = {
    "rmat13": (13, 16, 1301, 64, APPS, 0, None),
    "rmat16": (16, 16, 16, 64, ["bfs-sync", "sssp-sync"], 0, [0]),
    "rmat24": (24, 16, 24, 64, ["sssp-async"], 1_000_000_000, 8),
    "rmat28": (28, 16, 24, 64, ["sssp-async"], 8_000_000_000, 2),
}


def file_digest(path: Path) -> str:
    """SHA-256 of the CSR in memory order: node pointers (n + 1) then the edges."""
    from oracle import oracle
    npt, ed = oracle.read_csr(path)
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(npt).tobytes())
    for k in range(0, len(ed), 1 << 26):
        h.update(np.ascontiguousarray(ed[k:k + (1 << 26)]).tobytes())
    return h.hexdigest()


def values_digest(v: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(v, dtype=np.uint32).tobytes()).hexdigest()


def read_output(path: Path, algo: str) -> np.ndarray:
    """The reference's --output file: 'i value' per line (shared/subway_utilities.cpp:40-61)."""
    flat = np.fromfile(path, sep=" ", dtype=np.float64 if algo == "pr" else np.uint64)
    vals = flat.reshape(-1, 2)[:, 1]
    return vals.astype(np.float32 if algo == "pr" else np.uint32)


def run_app(exe: Path, graph_path: Path, source, out_path: Path, budget: int) -> list[str]:
    env = dict(os.environ, MALLOC_MMAP_THRESHOLD_="4096", GLIBC_TUNABLES="glibc.malloc.mmap_threshold=4096")
    if budget:
        env["SUBWAY_BUDGET_BYTES"] = str(budget)
    cmd = [str(exe), "--input", str(graph_path), "--output", str(out_path)]
    if source is not None:
        cmd += ["--source", str(source)]
    p = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=3600)
    if p.returncode != 0:
        raise RuntimeError(f"{exe.name} failed ({p.returncode}): {p.stderr[-300:]}")
    return p.stdout.splitlines()


def main(name: str, out_dir: Path):
    from oracle import build_ref, oracle
    scale, ef, seed, wmax, apps, budget, nsrc = SETS[name]
    tmp = Path(tempfile.mkdtemp(prefix="sgw_golden_"))
    pu, pw = tmp / "g.bcsr", tmp / "g.bwcsr"
    need_u = any(a.split("-")[0] in ("bfs", "cc", "pr") for a in apps)
    need_w = any(a.split("-")[0] in ("sssp", "sswp") for a in apps)
    if need_u:
        oracle.rmat_write(pu, scale, ef, seed=seed, weighted=False)
    oracle.rmat_write(pw, scale, ef, seed=seed, weighted=True, wmax=wmax)
    npw, edw = oracle.read_csr(pw)
    if nsrc is None:
        sources = [0, int(oracle.pick_sources(npw, edw, 1, seed=seed)[0])]
    elif isinstance(nsrc, list):
        sources = nsrc
    else:
        sources = [int(s) for s in oracle.pick_sources(npw, edw, nsrc if name != "rmat28" else 16, seed=seed)]
        sources = sources[:nsrc]
    big = name in ("rmat24", "rmat28")
    variants = ("fixed",) if name == "rmat28" else ("shipped", "fixed")
    arrays = {"params": np.array([scale, ef, seed, wmax] + sources, np.int64)}
    if need_u:
        arrays["digest_unweighted"] = np.array(file_digest(pu))
    if need_w:
        arrays["digest_weighted"] = np.array(file_digest(pw))
    report = {"graph": f"R-MAT(0.57,0.19,0.19,0.05) scale {scale}, edge factor {ef}, seed {seed}, w in [1,{wmax}]",
              "budget_bytes": budget, "sources": sources, "digest_weighted": str(arrays["digest_weighted"]),
              "runs": {}}
    refs = {}
    for variant in variants:
        for app in apps:
            algo = app.split("-")[0]
            weighted = algo in ("sssp", "sswp")
            path = pw if weighted else pu
            for s in ([None] if algo in ("cc", "pr") else sources):
                out = tmp / "out.txt"
                t = time.time()
                log = run_app(build_ref.binary(app, fixed=(variant == "fixed")), path, s, out, budget)
                vals = read_output(out, algo)
                out.unlink()
                key = f"{variant}/{app}" + ("" if s is None else f"/s{s}")
                it = [ln for ln in log if ln.startswith("Number of iterations")]
                if big:
                    if s not in refs:
                        npt, ed = (npw, edw) if weighted else oracle.read_csr(path)
                        refs[s] = oracle.run(algo, npt, ed, s, parallel=True)
                    report["runs"][key] = {"sha256": values_digest(vals),
                                           "mismatches_vs_oracle": int(np.count_nonzero(vals != refs[s])),
                                           "oracle_sha256": values_digest(refs[s])}
                else:
                    arrays[key] = vals
                    if algo != "pr":  # B2 shows up as differences of the shipped build
                        npt, ed = oracle.read_csr(path)
                        ref = oracle.run(algo, npt, ed, 0 if s is None else s)
                        arrays["mismatches/" + key] = np.array(int(np.count_nonzero(vals != ref)), np.int64)
                print(key, len(vals), it[0] if it else "", f"{time.time() - t:.1f}s", flush=True)
    out_dir.mkdir(parents=True, exist_ok=True)
    if big:
        app = apps[0]
        target = out_dir / f"ref_{name}_{app.replace('-', '_')}_{budget // 1_000_000_000}gb.json"
        target.write_text(json.dumps(report, indent=1) + "\n")
    else:
        target = out_dir / f"ref_{name}.npz"
        np.savez_compressed(target, **arrays)
    for f in (pu, pw):
        if f.exists():
            f.unlink()
    tmp.rmdir()
    print("wrote", target)


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "rmat13"
    main(which, Path(sys.argv[2]) if len(sys.argv) > 2 else Path(__file__).resolve().parent)

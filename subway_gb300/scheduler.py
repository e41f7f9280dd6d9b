"""The learned scheduler's data and training (host orchestration only).

The engine logs, for every static vertex range and global iteration of a
SGW_POLICY_LEARNED run, the five features its range-statistics kernel fed to
the network and what the range did.  A training sample is the features of
range s at iteration t with, as target, the active edge fraction of the same
range at iteration t + 1 (0 once the run has converged).  Training runs the
library's own kernels (sgw_mlp_train: forward, backward, Adam).

    python -m subway_gb300.scheduler --out subway_gb300/models/sched_mlp.bin
trains on 32 seeded R-MAT graphs (scales 22-25, edge factor 16) with
SSSP-async and BFS-async runs under budgets that keep 1/4 to 2/3 of the
edges resident, and writes the model and a JSON report beside it.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import native as N

MODEL_DIR = Path(__file__).resolve().parent / "models"
DEFAULT_MODEL = MODEL_DIR / "sched_mlp.bin"


def samples_from_trace(rec: np.ndarray):
    """(features, targets) from one run's range trace."""
    if len(rec) == 0:
        return np.zeros((0, N.MLP_INPUTS), np.float32), np.zeros(0, np.float32)
    last = int(rec["global_iteration"].max())
    nxt = {(int(r["global_iteration"]), int(r["range"])): r for r in rec}
    xs, ys = [], []
    for r in rec:
        t, s = int(r["global_iteration"]), int(r["range"])
        n = nxt.get((t + 1, s))
        if n is not None:
            y = float(n["features"][1])
        elif t >= last:
            y = 0.0  # converged: nothing is active afterwards
        else:
            continue
        xs.append(r["features"])
        ys.append(y)
    return np.asarray(xs, np.float32).reshape(-1, N.MLP_INPUTS), np.asarray(ys, np.float32)


def fixed_state_bytes(n: int) -> int:
    return 18 * n + 4 * 1024 * 1024


def collect(g, algos=("sssp", "bfs"), mode="async", sources=2, budget_fraction=0.5, seed=1,
            model=None, device=0, num_buffers=2):
    """Runs the learned policy (model or persistence predictor) and returns samples."""
    esz = 4  # packed or unweighted transfer records
    budget = int(fixed_state_bytes(g.n) + budget_fraction * g.m * esz)
    eng = N.Engine(g, budget_bytes=budget, device=device, num_buffers=num_buffers)
    eng.set_policy("learned", model)
    eng.trace_enable(True)
    xs, ys = [], []
    for algo in algos:
        if algo in ("sssp", "sswp") and not g.weighted:
            continue
        for s in g.pick_sources(sources, seed=seed):
            eng.run(algo, mode, int(s))
            x, y = samples_from_trace(eng.range_trace())
            xs.append(x)
            ys.append(y)
    eng.close()
    return np.concatenate(xs), np.concatenate(ys)


def train(x, y, steps=600, lr=3e-3, seed=7, device=0):
    m = N.Mlp.create(device, seed)
    loss0 = float(m.gradient(x, y)[1])
    loss = m.train(x, y, steps=steps, lr=lr)
    return m, loss0, loss


def load_default(device=0):
    return N.Mlp.load(DEFAULT_MODEL, device) if DEFAULT_MODEL.exists() else None


def mispredictions(rec: np.ndarray) -> dict:
    """How often the predictions behind one run's decisions were wrong.

    A transfer decision for range s at iteration t (stream the whole range and
    keep it, or send only its active edges) compares the prediction p with
    the break-even fraction 1 - A/E: streaming pays E - A extra bytes now and
    saves the next iteration's transfer, worth y * E, where y is the range's
    actual active edge fraction at t + 1 (0 if it is not active again).  The
    decision was mispredicted when p and y fall on different sides of the
    break-even point."""
    if len(rec) == 0:
        return {"transfer_decisions": 0, "transfer_mispredicted": 0, "prediction_mae": None}
    nxt = {(int(r["global_iteration"]), int(r["range"])): r for r in rec}
    dec = bad = 0
    err = []
    for r in rec:
        if int(r["action"]) not in (N.ACT_STREAM, N.ACT_COMPACT):
            continue
        n = nxt.get((int(r["global_iteration"]) + 1, int(r["range"])))
        y = float(n["active_edges"]) / max(1, int(n["range_edges"])) if n is not None else 0.0
        p = float(r["predicted"])
        even = 1.0 - float(r["active_edges"]) / max(1, int(r["range_edges"]))
        dec += 1
        bad += int((p >= even) != (y >= even))
        err.append(abs(p - y))
    return {"transfer_decisions": dec, "transfer_mispredicted": bad,
            "prediction_mae": round(float(np.mean(err)), 4) if err else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(DEFAULT_MODEL))
    ap.add_argument("--graphs", type=int, default=32)
    ap.add_argument("--min-scale", type=int, default=22)
    ap.add_argument("--max-scale", type=int, default=25)
    ap.add_argument("--steps", type=int, default=800)
    ap.add_argument("--lr", type=float, default=3e-3)
    a = ap.parse_args()
    t0 = time.time()
    xs, ys, meta = [], [], []
    rng = np.random.default_rng(2024)
    for k in range(a.graphs):
        scale = int(a.min_scale + k % (a.max_scale - a.min_scale + 1))
        frac = float(rng.uniform(0.25, 0.67))
        g = N.Graph.rmat(scale, 16, seed=1000 + k, weighted=True, wmax=64)
        x, y = collect(g, budget_fraction=frac, seed=1000 + k)
        xs.append(x)
        ys.append(y)
        meta.append({"scale": scale, "seed": 1000 + k, "budget_fraction": round(frac, 3), "samples": len(x)})
        del g
    x = np.concatenate(xs)
    y = np.concatenate(ys)
    m, loss0, loss = train(x, y, steps=a.steps, lr=a.lr)
    out = Path(a.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    m.save(out)
    pred = m.forward(x)
    report = {"samples": int(len(x)), "graphs": meta, "loss_initial": loss0, "loss_final": loss,
              "mae": float(np.mean(np.abs(pred - y))),
              "mae_persistence": float(np.mean(np.abs(x[:, 1] - y))),
              "steps": a.steps, "lr": a.lr, "seconds": round(time.time() - t0, 1)}
    out.with_suffix(".json").write_text(json.dumps(report, indent=1))
    print(json.dumps({k: v for k, v in report.items() if k != "graphs"}))


if __name__ == "__main__":
    main()

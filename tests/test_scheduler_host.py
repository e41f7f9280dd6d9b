"""Host-side logic of the learned scheduler: training samples and the
misprediction count built from a range trace (no GPU)."""
import numpy as np

from subway_gb300 import native as N
from subway_gb300 import scheduler


def _rec(rows):
    rec = np.zeros(len(rows), N.RANGE_REC)
    for i, (t, s, act, ae, re, pred) in enumerate(rows):
        rec[i]["global_iteration"] = t
        rec[i]["range"] = s
        rec[i]["action"] = act
        rec[i]["active_edges"] = ae
        rec[i]["range_edges"] = re
        rec[i]["predicted"] = pred
        rec[i]["features"][1] = ae / re
    return rec


def test_samples_target_next_iteration_fraction():
    rec = _rec([(1, 0, N.ACT_COMPACT, 50, 100, 0.2), (2, 0, N.ACT_STREAM, 80, 100, 0.9),
                (1, 1, N.ACT_COMPACT, 10, 100, 0.0), (3, 0, N.ACT_RESIDENT, 5, 100, 0.1)])
    x, y = scheduler.samples_from_trace(rec)
    # range 0: t1 -> 0.8, t2 -> 0.05, t3 is the last iteration -> 0; range 1 at
    # t1 has no t2 record and t1 is not the last iteration: no sample
    assert len(x) == 3
    assert np.allclose(sorted(y), [0.0, 0.05, 0.8])


def test_mispredictions_against_break_even():
    rec = _rec([
        (1, 0, N.ACT_STREAM, 60, 100, 0.5),   # even 0.4: p >= even, next 0.7 -> right
        (2, 0, N.ACT_RESIDENT, 70, 100, 0.5),
        (1, 1, N.ACT_STREAM, 90, 100, 0.2),   # even 0.1: p >= even, never active again -> wrong
        (1, 2, N.ACT_COMPACT, 10, 100, 0.3),  # even 0.9: p < even, next 0.95 -> wrong
        (2, 2, N.ACT_COMPACT, 95, 100, 0.0),  # even 0.05: p < even, inactive after -> right
    ])
    m = scheduler.mispredictions(rec)
    assert m["transfer_decisions"] == 4
    assert m["transfer_mispredicted"] == 2
    assert abs(m["prediction_mae"] - np.mean([0.2, 0.2, 0.65, 0.0])) < 1e-4
    assert scheduler.mispredictions(rec[:0])["transfer_decisions"] == 0


def test_sched_buffers_rule():
    """3 edge buffers when a third of the space left after the 18 B/vertex
    state holds at least 15% of the edges at the transfer record size (4 B
    packed or unweighted, 8 B for weights that neither pack beside the ids nor
    fit a byte), else 2."""
    g = N.Graph.rmat(12, 16, seed=3, weighted=True, wmax=64)  # packs: 4 B records
    state = 18 * g.n
    edge = int(np.ceil(0.15 * g.m)) * 4 * 3
    assert N.sched_buffers(g, state + edge) == 3
    assert N.sched_buffers(g, state + edge - 16) == 2
    assert N.sched_buffers(g, state) == 2
    assert N.sched_buffers(g, 0) == 2
    u = N.Graph.rmat(12, 16, seed=3)
    assert N.sched_buffers(u, 18 * u.n + int(np.ceil(0.15 * u.m)) * 12) == 3
    # weights of 2^24 leave no room beside 12-bit ids: 8-byte records
    e = g.edges.copy()
    e[:, 1] = 1 << 24
    w = N.Graph.from_csr(g.node_pointer, e, True)
    need8 = int(np.ceil(0.15 * w.m)) * 8 * 3
    assert N.sched_buffers(w, 18 * w.n + need8) == 3
    assert N.sched_buffers(w, 18 * w.n + need8 // 2) == 2

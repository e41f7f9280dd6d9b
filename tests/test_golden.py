"""The oracle against the Subway reference's own outputs.

tests/golden/ref_rmat13.npz holds every app's output from the reference build
(as shipped and with the host-gather chunk fix), run on a GB300 by
tests/golden/make_golden.py on a seeded R-MAT scale-13 graph; the graph is
regenerated here and checked against the stored digest first."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "ref_rmat13.npz"
PR_INIT, PR_ACC, PR_DAMP = (float(np.float32(x)) for x in (0.15, 0.01, 0.85))


def _digest(g):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(g.node_pointer).tobytes())
    h.update(np.ascontiguousarray(g.edges).tobytes())
    return h.hexdigest()


@pytest.fixture(scope="module")
def gold(native):
    d = np.load(GOLD)
    scale, ef, seed, wmax, src = (int(x) for x in d["params"])
    gu = native.Graph.rmat(scale, ef, seed=seed)
    gw = native.Graph.rmat(scale, ef, seed=seed, weighted=True, wmax=wmax)
    assert _digest(gu) == str(d["digest_unweighted"])
    assert _digest(gw) == str(d["digest_weighted"])
    return d, gu, gw


def _cases(d):
    for k in d.keys():
        if "/" in k:
            yield k


def test_integer_apps_bit_exact(orc, gold):
    d, gu, gw = gold
    n = 0
    for k in _cases(d):
        variant, app, *s = k.split("/")
        algo = app.split("-")[0]
        if algo == "pr":
            continue
        g = gw if algo in ("sssp", "sswp") else gu
        e = g.edges if algo in ("sssp", "sswp") else g.ends
        src = int(s[0][1:]) if s else 0
        assert np.array_equal(orc.run(algo, g.node_pointer, e, src), d[k]), k
        n += 1
    assert n == 28  # 7 integer apps x sources x {shipped, fixed}


def test_pagerank_close_to_reference(orc, gold):
    """The reference prints ranks with 6 significant digits; its (non
    bulk-synchronous, float) schedule lands within 1e-5 relative of the FP64
    bulk-synchronous oracle."""
    d, gu, _ = gold
    bsp, _ = orc.pagerank(gu.node_pointer, gu.ends, init=PR_INIT, acc=PR_ACC, damping=PR_DAMP)
    for k in _cases(d):
        if "/pr-" in k:
            ref = d[k].astype(np.float64)
            assert np.max(np.abs(ref - bsp) / bsp) < 1e-5, k

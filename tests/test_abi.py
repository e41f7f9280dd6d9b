"""The C-ABI library: loads, exports every declared symbol, reports errors
as status codes, and plans partitions like the reference (CPU only)."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w]+[\s\*]+\**(sgw_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_loads_and_exports_header(native):
    L = native.lib()
    declared = _declared()
    assert len(declared) >= 30
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_binding_covers_header(native):
    assert _declared() <= set(native.exported_symbols())


def test_strerror(native):
    L = native.lib()
    assert L.sgw_strerror(0) == b"ok"
    for code in range(-1, -10, -1):
        assert L.sgw_strerror(code) != b"unknown status"


def test_engine_without_gpu_is_an_error_not_exit(native):
    if native.device_count() > 0:
        pytest.skip("a GPU is visible")
    g = native.Graph.rmat(8, 4, seed=1)
    with pytest.raises(native.SgwError) as ei:
        native.Engine(g)
    assert ei.value.status == -6  # SGW_ECUDA


def test_from_csr_validation(native):
    npt = np.array([0, 1, 2], np.uint32)
    with pytest.raises(native.SgwError):
        native.Graph.from_csr(npt, np.array([1, 5], np.uint32), False)  # endpoint >= n
    with pytest.raises(native.SgwError):
        native.Graph.from_csr(np.array([0, 2, 1], np.uint32), np.array([1], np.uint32), False)
    g = native.Graph.from_csr(npt, np.array([1, 0], np.uint32), False)
    assert (g.n, g.m) == (2, 2)


def _random_ptr(rng, count, maxdeg):
    deg = rng.integers(1, maxdeg, count).astype(np.uint64)
    if count > 3:
        deg[rng.integers(0, count)] = maxdeg * 50  # one hub
    ptr = np.zeros(count + 1, np.uint64)
    ptr[1:] = np.cumsum(deg)
    return ptr.astype(np.uint32)


@pytest.mark.parametrize("seed", range(6))
def test_plan_partitions_properties(native, orc, seed):
    rng = np.random.default_rng(seed)
    ptr = _random_ptr(rng, int(rng.integers(1, 3000)), 40)
    cap = int(rng.integers(20, 3000))
    fr, sz = native.plan_partitions(ptr, cap)
    # contiguous cover of the queue
    assert fr[0] == 0 and np.all(fr[1:] == fr[:-1] + sz[:-1]) and fr[-1] + sz[-1] == len(ptr) - 1
    edges = ptr[fr + sz].astype(np.int64) - ptr[fr]
    single = sz == 1
    assert np.all((edges <= cap) | single), "a multi-vertex partition exceeds the cap"
    # greedy maximality: the next vertex would not have fit
    nxt = fr + sz
    has_next = nxt < len(ptr) - 1
    grown = ptr[np.minimum(nxt + 1, len(ptr) - 1)].astype(np.int64) - ptr[fr]
    assert np.all(~has_next | (grown > cap))
    ref = orc.partition(ptr, cap)
    if ref is None:
        assert np.any(edges > cap), "the reference only fails with a vertex above the cap"
    else:
        assert len(fr) <= len(ref[0])


def test_plan_partitions_matches_reference_when_exact(native, orc):
    """When every partition boundary is exact, the reference's bisection
    finds the same greedy split."""
    ptr = np.arange(0, 1001, 1, dtype=np.uint32)  # 1000 unit-degree vertices
    for cap in (1, 7, 64, 999, 1000, 5000):
        fr, sz = native.plan_partitions(ptr, cap)
        ref = orc.partition(ptr, cap)
        assert ref is not None
        assert np.array_equal(fr, ref[0]) and np.array_equal(sz, ref[1]), cap

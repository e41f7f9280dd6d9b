"""Host-side helpers of the C ABI (CPU only): removing a vertex's out-edges
(the apps' --subway-compat, which reproduces the reference ignoring vertex
n-2's out-edges, shared/graph.cu:179-181) and the trace's CSV writer."""
import numpy as np
import pytest


def _graph_with_edges_at(native, n, seed):
    """A small CSR whose every vertex, n - 2 included, has out-edges."""
    rng = np.random.default_rng(seed)
    deg = rng.integers(1, 6, n)
    npt = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint32)
    dst = rng.integers(0, n, int(npt[-1])).astype(np.uint32)
    w = rng.integers(1, 65, int(npt[-1])).astype(np.uint32)
    return npt, np.stack([dst, w], 1)


@pytest.mark.parametrize("which", ["middle", "n-2", "last", "first"])
def test_clear_out_edges(native, tmp_path, which):
    n = 500
    npt, edges = _graph_with_edges_at(native, n, 3)
    native.Graph.from_csr(npt, edges, True).save(tmp_path / "g.bwcsr")
    g = native.Graph.load(tmp_path / "g.bwcsr")
    v = {"middle": 123, "n-2": n - 2, "last": n - 1, "first": 0}[which]
    keep = np.ones(len(edges), bool)
    keep[npt[v]:npt[v + 1]] = False
    deg = np.diff(npt.astype(np.int64))
    deg[v] = 0
    want_np = np.concatenate([[0], np.cumsum(deg)])
    g.clear_out_edges(v)
    assert g.m == int(keep.sum())
    assert np.array_equal(g.node_pointer.astype(np.int64), want_np)
    assert np.array_equal(g.edges, edges[keep])
    g.save(tmp_path / "h.bwcsr")  # still a valid graph
    h = native.Graph.load(tmp_path / "h.bwcsr")
    assert np.array_equal(h.edges, edges[keep])
    g.clear_out_edges(v)  # nothing left to remove
    assert g.m == int(keep.sum())


def test_clear_out_edges_refuses_borrowed_arrays(native, tmp_path):
    npt, edges = _graph_with_edges_at(native, 50, 4)
    caller = native.Graph.from_csr(npt, edges, True)
    with pytest.raises(native.SgwError):
        caller.clear_out_edges(3)
    caller.save(tmp_path / "g.bwcsr")
    mapped = native.Graph.map(tmp_path / "g.bwcsr")
    with pytest.raises(native.SgwError):
        mapped.clear_out_edges(3)
    with pytest.raises(native.SgwError):
        native.Graph.load(tmp_path / "g.bwcsr").clear_out_edges(50)  # v >= n


def test_trace_csv(native, tmp_path):
    rng = np.random.default_rng(7)
    recs = np.zeros(17, native.TRACE_REC)
    for f in native.TRACE_REC.names:
        if f != "reserved":
            hi = 2 ** 40 if native.TRACE_REC[f] == np.dtype("<u8") else 2 ** 31
            recs[f] = rng.integers(0, hi, len(recs))
    native.write_trace_csv(recs, tmp_path / "t.csv")
    lines = (tmp_path / "t.csv").read_text().splitlines()
    fields = [f for f in native.TRACE_REC.names if f != "reserved"]
    assert lines[0].split(",") == fields
    got = np.array([[int(x) for x in line.split(",")] for line in lines[1:]], dtype=np.uint64)
    assert got.shape == (len(recs), len(fields))
    for k, f in enumerate(fields):
        assert np.array_equal(got[:, k], recs[f].astype(np.uint64)), f
    native.write_trace_csv(recs[:0], tmp_path / "empty.csv")
    assert (tmp_path / "empty.csv").read_text().splitlines() == [lines[0]]

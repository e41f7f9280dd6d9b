"""Graphs with u64 node pointers and the .bcsr64 / .bwcsr64 files (CPU only).

The reference's binary header holds u32 counts (shared/graph.cu:43-44), so it
cannot describe a graph of 2^32 edges or more; these files and entry points
carry such graphs.  Graphs that large do not fit a CPU test, so the tests
here pin the format, the conversions between the two widths and the checks on
small graphs; the GPU tests run a graph past 2^32 edges."""
import numpy as np
import pytest


def _same(a, b):
    assert (a.n, a.m, a.weighted) == (b.n, b.m, b.weighted)
    assert np.array_equal(a.node_pointer.astype(np.uint64), b.node_pointer.astype(np.uint64))
    assert np.array_equal(a.edges, b.edges)


@pytest.mark.parametrize("weighted", [False, True])
@pytest.mark.parametrize("scale", [9, 10])  # n - 2 keeps no edges: n odd / even offsets both occur below
def test_bcsr64_layout_and_round_trip(native, tmp_path, weighted, scale):
    g = native.Graph.rmat(scale, 8, seed=5, weighted=weighted, wmax=64)
    ext = "bwcsr64" if weighted else "bcsr64"
    p = tmp_path / f"g.{ext}"
    g.save(p)
    raw = p.read_bytes()
    esz = 8 if weighted else 4
    assert len(raw) == 16 + 8 * g.n + esz * g.m
    hdr = np.frombuffer(raw[:16], np.uint64)
    assert hdr.tolist() == [g.n, g.m]
    assert np.array_equal(np.frombuffer(raw[16:16 + 8 * g.n], np.uint64), g.node_pointer[:-1].astype(np.uint64))
    assert raw[16 + 8 * g.n:] == np.ascontiguousarray(g.edges).tobytes()
    for h in (native.Graph.load(p), native.Graph.map(p)):
        _same(g, h)
        assert h.node_pointer.dtype == np.uint32  # below 2^32 edges the library keeps u32 pointers


@pytest.mark.parametrize("weighted", [False, True])
def test_from_csr64_equals_u32_graph(native, tmp_path, weighted):
    """A caller's u64 node pointers: same graph, u64 view, same files."""
    g = native.Graph.rmat(11, 8, seed=7, weighted=weighted, wmax=64)
    np64 = g.node_pointer.astype(np.uint64)
    w = native.Graph.from_csr(np64, np.array(g.edges), weighted)
    assert w.node_pointer.dtype == np.uint64 and np.array_equal(w.node_pointer, np64)
    _same(g, w)
    assert np.array_equal(w.out_degree(), g.out_degree())
    assert w.pick_sources(8, seed=3).tolist() == g.pick_sources(8, seed=3).tolist()
    assert w.largest_wcc() == g.largest_wcc()
    for ext in (("bwcsr", "bwcsr64", "wel") if weighted else ("bcsr", "bcsr64", "el")):
        g.save(tmp_path / f"a.{ext}")
        w.save(tmp_path / f"b.{ext}")
        assert (tmp_path / f"a.{ext}").read_bytes() == (tmp_path / f"b.{ext}").read_bytes(), ext
    if not weighted:
        s1, s2 = g.symmetrize(), w.symmetrize()
        _same(s1, s2)


def test_text_to_bcsr64_and_back(native, tmp_path):
    (tmp_path / "g.wel").write_text("0 1 26\n0 3 33\n2 3 40\n1 2 10\n")
    g = native.Graph.load(tmp_path / "g.wel")
    g.save(tmp_path / "g.bwcsr64")
    h = native.Graph.load(tmp_path / "g.bwcsr64")
    _same(g, h)
    h.save(tmp_path / "h.wel")
    assert (tmp_path / "h.wel").read_text() == "0 1 26\n0 3 33\n1 2 10\n2 3 40\n"


def test_from_csr64_checks(native):
    e = np.array([1, 0], np.uint32)
    with pytest.raises(native.SgwError):
        native.Graph.from_csr(np.array([0, 2, 1], np.uint64), np.array([1], np.uint32), False)  # not monotone
    with pytest.raises(native.SgwError):
        native.Graph.from_csr(np.array([0, 1, 2], np.uint64), np.array([1, 5], np.uint32), False)  # endpoint >= n
    g = native.Graph.from_csr(np.array([0, 1, 2], np.uint64), e, False)
    assert (g.n, g.m) == (2, 2)


def test_bcsr64_format_errors(native, tmp_path):
    g = native.Graph.rmat(8, 4, seed=2)
    g.save(tmp_path / "g.bcsr64")
    raw = bytearray((tmp_path / "g.bcsr64").read_bytes())
    (tmp_path / "short.bcsr64").write_bytes(bytes(raw[:-4]))
    bad = bytearray(raw)
    bad[24:32] = np.array([1 << 40], np.uint64).tobytes()  # node_pointer[1] > node_pointer[2]
    (tmp_path / "mono.bcsr64").write_bytes(bytes(bad))
    big = bytearray(raw)
    big[0:8] = np.array([1 << 32], np.uint64).tobytes()  # n beyond u32 vertex ids
    (tmp_path / "bign.bcsr64").write_bytes(bytes(big))
    for name in ("short", "mono", "bign"):
        for fn in (native.Graph.load, native.Graph.map):
            with pytest.raises(native.SgwError):
                fn(tmp_path / f"{name}.bcsr64")


def test_oracle_reads_bcsr64(native, orc, tmp_path):
    g = native.Graph.rmat(10, 8, seed=9, weighted=True, wmax=64)
    g.save(tmp_path / "g.bwcsr")
    g.save(tmp_path / "g.bwcsr64")
    n32, e32 = orc.read_csr(tmp_path / "g.bwcsr")
    n64, e64 = orc.read_csr(tmp_path / "g.bwcsr64")
    assert n32.dtype == np.uint32 and n64.dtype == np.uint64
    assert np.array_equal(n32.astype(np.uint64), n64) and np.array_equal(e32, e64)
    s = int(g.pick_sources(1, seed=1)[0])
    assert np.array_equal(orc.run("sssp", n32, e32, s), orc.run("sssp", n64, e64, s, parallel=True))

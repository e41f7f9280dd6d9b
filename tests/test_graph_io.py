"""Graph formats and the seeded generators (CPU only)."""
import hashlib
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
README_EL = "0 1\n0 3\n2 3\n1 2\n"            # the example graph of the reference README
README_WEL = "0 1 26\n0 3 33\n2 3 40\n1 2 10\n"


def _digest(g):
    h = hashlib.sha256()
    h.update(g.node_pointer.tobytes())
    h.update(np.ascontiguousarray(g.edges).tobytes())
    return h.hexdigest()


def test_rmat_deterministic(native):
    a = native.Graph.rmat(12, 8, seed=3, weighted=True)
    b = native.Graph.rmat(12, 8, seed=3, weighted=True)
    c = native.Graph.rmat(12, 8, seed=4, weighted=True)
    assert _digest(a) == _digest(b) != _digest(c)


def test_rmat_independent_of_thread_count(native):
    code = ("import sys; sys.path.insert(0, %r); from subway_gb300 import native as N; "
            "import hashlib, numpy as np; g=N.Graph.rmat(13, 8, seed=9, weighted=True); "
            "h=hashlib.sha256(); h.update(g.node_pointer.tobytes()); "
            "h.update(np.ascontiguousarray(g.edges).tobytes()); print(h.hexdigest())" % str(ROOT))
    outs = []
    for t in ("1", "3"):
        env = dict(os.environ, OMP_NUM_THREADS=t)
        outs.append(subprocess.run([sys.executable, "-c", code], env=env, capture_output=True,
                                   text=True, check=True).stdout.strip())
    assert outs[0] == outs[1]


@pytest.mark.parametrize("kind", ["rmat", "er"])
def test_generator_invariants(native, kind):
    g = (native.Graph.rmat(12, 16, seed=2, weighted=True, wmax=64) if kind == "rmat"
         else native.Graph.er(4096, 60000, seed=2, weighted=True, wmax=64))
    npt, e = g.node_pointer, g.edges
    assert npt[0] == 0 and npt[-1] == g.m and np.all(np.diff(npt.astype(np.int64)) >= 0)
    src = np.repeat(np.arange(g.n, dtype=np.uint32), np.diff(npt))
    assert np.all(src != e[:, 0]), "self-loop"
    key = src.astype(np.uint64) << np.uint64(32) | e[:, 0].astype(np.uint64)
    assert np.all(np.diff(key.astype(np.int64)) > 0), "rows unsorted or duplicated"
    assert e[:, 1].min() >= 1 and e[:, 1].max() <= 64
    assert npt[g.n - 1] == npt[g.n - 2], "vertex n-2 must have no out-edges"


def test_rmat_skew(native):
    g = native.Graph.rmat(14, 16, seed=1)
    deg = g.out_degree()
    assert deg[0] == deg.max(), "vertex 0 is the top hub (no permutation)"
    assert g.m > 0.7 * 16 * g.n


@pytest.mark.parametrize("ext", ["bcsr", "bwcsr", "el", "wel"])
def test_save_load_round_trip(native, tmp_path, ext):
    g = native.Graph.rmat(10, 8, seed=5, weighted=ext in ("bwcsr", "wel"))
    p = tmp_path / f"g.{ext}"
    g.save(p)
    h = native.Graph.load(p)
    assert h.weighted == g.weighted
    if ext in ("el", "wel"):
        # text drops trailing isolated vertices: n = max id + 1 (graph.cu:85)
        assert h.m == g.m and h.n <= g.n
        assert np.array_equal(h.node_pointer, g.node_pointer[: h.n + 1])
    else:
        assert (h.n, h.m) == (g.n, g.m)
        assert np.array_equal(h.node_pointer, g.node_pointer)
    assert np.array_equal(h.edges, g.edges)


def test_readme_example(native, tmp_path):
    (tmp_path / "Graph.el").write_text(README_EL)
    (tmp_path / "Graph.wel").write_text(README_WEL)
    g = native.Graph.load(tmp_path / "Graph.el")
    assert (g.n, g.m) == (4, 4)
    assert g.node_pointer.tolist() == [0, 2, 3, 4, 4]
    assert g.ends.tolist() == [1, 3, 2, 3]
    w = native.Graph.load(tmp_path / "Graph.wel")
    assert w.edges.tolist() == [[1, 26], [3, 33], [2, 10], [3, 40]]
    # the converter's binary output, written by this library, reads back
    w.save(tmp_path / "Graph.bwcsr")
    raw = (tmp_path / "Graph.bwcsr").read_bytes()
    assert np.frombuffer(raw[:8], np.uint32).tolist() == [4, 4]
    assert len(raw) == 8 + 4 * 4 + 4 * 8


def test_format_errors(native, tmp_path):
    with pytest.raises(native.SgwError) as e:
        native.Graph.load(tmp_path / "missing.bcsr")
    assert e.value.status == -2
    (tmp_path / "g.txt").write_text(README_EL)
    with pytest.raises(native.SgwError) as e:
        native.Graph.load(tmp_path / "g.txt")
    assert e.value.status == -3
    g = native.Graph.rmat(8, 4, seed=1)
    g.save(tmp_path / "t.bcsr")
    raw = (tmp_path / "t.bcsr").read_bytes()
    (tmp_path / "trunc.bcsr").write_bytes(raw[:-4])
    with pytest.raises(native.SgwError) as e:
        native.Graph.load(tmp_path / "trunc.bcsr")
    assert e.value.status == -3
    bad = bytearray(raw)
    bad[-4:] = np.uint32(10**6).tobytes()  # endpoint out of range
    (tmp_path / "bad.bcsr").write_bytes(bytes(bad))
    with pytest.raises(native.SgwError):
        native.Graph.load(tmp_path / "bad.bcsr")
    (tmp_path / "w.wel").write_text("0 1\n")
    with pytest.raises(native.SgwError):
        native.Graph.load(tmp_path / "w.wel")


def test_symmetrize(native):
    g = native.Graph.rmat(11, 8, seed=4)
    s = g.symmetrize()
    npt, e = s.node_pointer, s.ends
    src = np.repeat(np.arange(s.n), np.diff(npt))
    fwd = set(zip(src.tolist(), e.tolist()))
    for u, v in list(fwd)[:5000]:
        assert (v, u) in fwd or v == s.n - 2
    assert np.all(np.diff(npt)[s.n - 2] == 0)


def test_pick_sources(native):
    g = native.Graph.rmat(12, 16, seed=6)
    a = g.pick_sources(8, seed=1)
    b = g.pick_sources(8, seed=1)
    assert np.array_equal(a, b) and len(set(a.tolist())) == 8
    assert np.all(g.out_degree()[a] > 0)
    nv, ne = g.largest_wcc()
    assert nv > g.n // 4 and ne > g.m // 2


def _reference_text_csr(text, weighted):
    """The reference's text reader restated (graph.cu:65-113): n = max id + 1,
    a counting sort by source that keeps file order within a row.  Blank and
    comment lines are skipped, as this library documents."""
    rows = []
    for line in text.splitlines():
        t = line.strip(" \t\r")
        if not t or t[0] in "#%":
            continue
        f = t.split()
        rows.append(tuple(int(x) for x in f[: 3 if weighted else 2]))
    n = max(max(r[0], r[1]) for r in rows) + 1
    order = sorted(range(len(rows)), key=lambda i: rows[i][0])  # stable
    npt = np.zeros(n + 1, np.uint32)
    np.add.at(npt, np.array([r[0] for r in rows]) + 1, 1)
    npt = np.cumsum(npt).astype(np.uint32)
    edges = np.array([rows[i][1:] for i in order], np.uint32)
    return n, npt, edges if weighted else edges[:, 0]


def _messy_text(rng, m, n, weighted):
    lines = ["# comment", "% another comment"]
    for k in range(m):
        s, d = int(rng.integers(n)), int(rng.integers(n))
        sep = "\t" if k % 7 == 0 else " "
        line = f"{s}{sep}{d}" + (f" {int(rng.integers(1, 2**32))}" if weighted else "")
        if k % 11 == 0:
            line = "  " + line + " trailing"
        if k % 13 == 0:
            line += "\r"
        lines.append(line)
        if k % 97 == 0:
            lines.append("")
    return "\n".join(lines)  # no newline after the last line


@pytest.mark.parametrize("weighted", [False, True])
def test_text_load_matches_reference_reader(native, tmp_path, weighted):
    """Several pieces per file (> 1 MiB), duplicates, unsorted rows, tabs,
    CRLF, comments, blank lines and a missing final newline."""
    rng = np.random.default_rng(11 + weighted)
    text = _messy_text(rng, 150_000, 5000, weighted)
    assert len(text) > (1 << 20)
    p = tmp_path / ("g.wel" if weighted else "g.el")
    p.write_text(text)
    n, npt, edges = _reference_text_csr(text, weighted)
    g = native.Graph.load(p)
    assert (g.n, g.m) == (n, len(edges))
    assert np.array_equal(g.node_pointer, npt)
    assert np.array_equal(g.edges if weighted else g.ends, edges)


def test_text_io_independent_of_thread_count(tmp_path):
    rng = np.random.default_rng(5)
    (tmp_path / "g.wel").write_text(_messy_text(rng, 200_000, 30_000, True))
    code = ("import sys, hashlib; sys.path.insert(0, %r); from subway_gb300 import native as N; "
            "g=N.Graph.load(sys.argv[1]); g.save(sys.argv[2]); h=hashlib.sha256(); "
            "h.update(g.node_pointer.tobytes()); h.update(g.edges.tobytes()); "
            "h.update(open(sys.argv[2], 'rb').read()); print(h.hexdigest())" % str(ROOT))
    outs = []
    for t in ("1", "3", "8"):
        env = dict(os.environ, OMP_NUM_THREADS=t)
        outs.append(subprocess.run([sys.executable, "-c", code, str(tmp_path / "g.wel"),
                                    str(tmp_path / f"out{t}.wel")], env=env, capture_output=True,
                                   text=True, check=True).stdout.strip())
    assert outs[0] == outs[1] == outs[2]


def test_text_errors_name_the_first_bad_line(native, tmp_path):
    good = "".join(f"{i} {i + 1}\n" for i in range(120_000))
    (tmp_path / "bad.el").write_text(good + "7 x\n" + good + "1 2 3\nq\n")
    with pytest.raises(native.SgwError) as e:
        native.Graph.load(tmp_path / "bad.el")
    assert e.value.status == -3 and "'7 x'" in str(e.value)
    (tmp_path / "big.el").write_text(good + "4294967295 1\n")
    with pytest.raises(native.SgwError) as e:
        native.Graph.load(tmp_path / "big.el")
    assert e.value.status == -9  # SGW_ERANGE: ids must stay below 2^32 - 1
    (tmp_path / "empty.el").write_text("# only a comment\n\n")
    with pytest.raises(native.SgwError):
        native.Graph.load(tmp_path / "empty.el")


@pytest.mark.parametrize("ext,n_odd", [("bcsr", False), ("bwcsr", False), ("bcsr", True), ("bwcsr", True)])
def test_mapped_binary_equals_loaded(native, tmp_path, ext, n_odd):
    weighted = ext == "bwcsr"
    if n_odd:
        g = native.Graph.er(4099, 40000, seed=8, weighted=weighted)
    else:
        g = native.Graph.rmat(12, 8, seed=8, weighted=weighted)
    p = tmp_path / f"g.{ext}"
    g.save(p)
    a = native.Graph.load(p)
    b = native.Graph.map(p)
    assert (b.n, b.m, b.weighted) == (a.n, a.m, a.weighted)
    assert np.array_equal(b.node_pointer, a.node_pointer)
    assert np.array_equal(b.edges, a.edges)
    if weighted:
        assert native.lib().sgw_graph_edges(b.h) % 8 == 0
    del b  # releases the mapping
    assert np.array_equal(native.Graph.map(p).out_degree(), g.out_degree())


def test_mapped_binary_errors(native, tmp_path):
    g = native.Graph.rmat(8, 4, seed=1)
    g.save(tmp_path / "t.bcsr")
    raw = (tmp_path / "t.bcsr").read_bytes()
    (tmp_path / "trunc.bcsr").write_bytes(raw[:-4])
    bad = bytearray(raw)
    bad[-4:] = np.uint32(10**6).tobytes()
    (tmp_path / "bad.bcsr").write_bytes(bytes(bad))
    (tmp_path / "g.el").write_text("0 1\n")
    for name, status in (("missing.bcsr", -2), ("trunc.bcsr", -3), ("bad.bcsr", -3), ("g.el", -3)):
        with pytest.raises(native.SgwError) as e:
            native.Graph.map(tmp_path / name)
        assert e.value.status == status, name


def test_text_reader_survives_random_bytes(native, tmp_path):
    """Random bytes, digits and separators (including lines cut anywhere and
    pieces of more than 1 MiB): the reader returns a graph or an error status,
    and whatever it accepts round-trips through the binary format."""
    rng = np.random.default_rng(99)
    alphabet = np.frombuffer(b"0123456789 \t\r\n#%-x", np.uint8)
    accepted = 0
    for k in range(18):
        size = int(rng.choice([1, 7, 100, 5000, 1_500_000]))
        if k % 3 == 0:
            data = rng.integers(0, 256, size, dtype=np.uint8).tobytes()
        elif k % 3 == 1:
            data = alphabet[rng.integers(0, len(alphabet), size)].tobytes()
        else:  # whole "src dst w" lines with random blanks, comments and CRs
            lines = []
            for _ in range(size // 12 + 1):
                a, b, w = (int(x) for x in rng.integers(0, 5000, 3))
                sep = str(rng.choice([" ", "\t", "  "]))
                lines.append(f"{a}{sep}{b}{sep}{w}" + str(rng.choice(["", "\r", " #x"])))
                if rng.random() < 0.05:
                    lines.append(str(rng.choice(["", "# c", "%"])))
            data = "\n".join(lines).encode()
        for ext in ("el", "wel"):
            p = tmp_path / f"f{k}.{ext}"
            p.write_bytes(data)
            try:
                g = native.Graph.load(p)
            except native.SgwError as e:
                assert e.status in (-3, -4, -9)
                continue
            accepted += 1
            q = tmp_path / f"f{k}.{'bwcsr' if ext == 'wel' else 'bcsr'}"
            g.save(q)
            h = native.Graph.load(q)
            assert np.array_equal(h.node_pointer, g.node_pointer) and np.array_equal(h.edges, g.edges)
    assert accepted > 0

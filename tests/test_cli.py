"""The ten drop-in apps: Subway's command line (shared/argument_parsing.cu:
25-119), its stdout lines and its --output format
(shared/subway_utilities.cpp:4-61).  Argument handling runs without a GPU;
the runs are marked gpu."""
import re
import subprocess

import numpy as np
import pytest

APPS = [f"{a}-{m}" for a in ("bfs", "cc", "sssp", "sswp", "pr") for m in ("sync", "async")]


@pytest.fixture(scope="session")
def bindir(native):
    from subway_gb300 import build
    return build.build_apps()


def _run(bindir, app, *args, timeout=120):
    return subprocess.run([str(bindir / app), *map(str, args)], capture_output=True, text=True, timeout=timeout)


@pytest.mark.parametrize("app", APPS)
def test_help_and_argument_errors_exit_zero(bindir, app):
    p = _run(bindir, app)
    assert p.returncode == 0 and "Required arguments:" in p.stdout and "[--input]" in p.stdout
    p = _run(bindir, app, "--input")  # odd number of arguments
    assert p.returncode == 0 and "There was an error parsing command line arguments" in p.stdout
    p = _run(bindir, app, "--output", "x.txt")
    assert p.returncode == 0 and "Input graph file argument is required." in p.stdout
    p = _run(bindir, app, "--input", "g.bcsr", "--bogus", "1")
    assert p.returncode == 0 and "error parsing command line argument <--bogus>" in p.stdout


def test_extra_flags_in_help_and_parsed(bindir):
    """--trace and --subway-compat are listed and parsed (a missing input file
    then fails at the read, after parsing, with exit status 1)."""
    p = _run(bindir, "bfs-async")
    assert "[--trace]" in p.stdout and "[--subway-compat]" in p.stdout
    p = _run(bindir, "bfs-async", "--input", "/nonexistent/g.bcsr", "--trace", "t.csv", "--subway-compat", "1")
    assert "error parsing" not in p.stdout and p.returncode == 1 and "ReadGraph" in p.stderr


def test_cc_sync_rejects_source(bindir):
    """cc-sync has no --source (subway/cc-sync.cu:17); cc-async accepts it."""
    p = _run(bindir, "cc-sync", "--input", "g.bcsr", "--source", "3")
    assert p.returncode == 0 and "error parsing command line argument <--source>" in p.stdout
    assert "[--source]" not in p.stdout


def test_missing_file_fails_without_a_gpu_call(bindir, tmp_path):
    p = _run(bindir, "bfs-sync", "--input", tmp_path / "none.bcsr")
    assert p.returncode != 0 and "cannot open" in p.stderr


README_EL = "0 1\n0 3\n2 3\n1 2\n"  # the reference README's example graph
README_WEL = "0 1 26\n0 3 33\n2 3 40\n1 2 10\n"


def test_converter_writes_the_reference_binary_layout(bindir, tmp_path):
    """tools/converter.cpp:20-172: g.el -> g.bcsr, g.wel -> g.bwcsr, laid out
    [n][m][nodePointer x n][edges x m] with rows in file order."""
    (tmp_path / "Graph.el").write_text(README_EL)
    (tmp_path / "Graph.wel").write_text(README_WEL)
    for name in ("Graph.el", "Graph.wel"):
        p = _run(bindir, "converter", tmp_path / name)
        assert p.returncode == 0, p.stderr
    raw = np.frombuffer((tmp_path / "Graph.bcsr").read_bytes(), np.uint32)
    assert raw.tolist() == [4, 4, 0, 2, 3, 4, 1, 3, 2, 3]
    raw = np.frombuffer((tmp_path / "Graph.bwcsr").read_bytes(), np.uint32)
    assert raw.tolist() == [4, 4, 0, 2, 3, 4, 1, 26, 3, 33, 2, 10, 3, 40]


def test_converter_argument_errors_exit_zero(bindir, tmp_path):
    p = _run(bindir, "converter")
    assert p.returncode == 0 and "There was an error parsing command line arguments" in p.stdout
    p = _run(bindir, "converter", tmp_path / "a.el", tmp_path / "b.el")
    assert p.returncode == 0 and "There was an error parsing command line arguments" in p.stdout
    (tmp_path / "g.txt").write_text(README_EL)
    p = _run(bindir, "converter", tmp_path / "g.txt")
    assert p.returncode == 0 and "Input file format is not supported." in p.stdout
    p = _run(bindir, "converter", tmp_path / "missing.el")
    assert p.returncode != 0 and "cannot open" in p.stderr


def test_converter_large_file_round_trip(native, bindir, tmp_path):
    g = native.Graph.rmat(14, 16, seed=21, weighted=True, wmax=64)
    g.save(tmp_path / "r.wel")
    p = _run(bindir, "converter", tmp_path / "r.wel")
    assert p.returncode == 0, p.stderr
    h = native.Graph.load(tmp_path / "r.bwcsr")
    assert h.m == g.m and np.array_equal(h.edges, g.edges)
    assert np.array_equal(h.node_pointer, g.node_pointer[: h.n + 1])


def _write(gpu, tmp_path, weighted):
    g = gpu.Graph.rmat(12, 8, seed=77, weighted=weighted, wmax=64)
    path = tmp_path / ("g.bwcsr" if weighted else "g.bcsr")
    g.save(path)
    return g, path


@pytest.mark.gpu
@pytest.mark.parametrize("app", APPS)
def test_app_output_matches_oracle(gpu, orc, bindir, tmp_path, app):
    algo = app.split("-")[0]
    weighted = algo in ("sssp", "sswp")
    g, path = _write(gpu, tmp_path, weighted)
    src = int(g.pick_sources(1, seed=5)[0])
    out = tmp_path / "out.txt"
    state = 36 * g.n if algo == "pr" else 18 * g.n  # PR keeps f64 ranks and residuals
    args = ["--input", path, "--output", out, "--budget", state + 64 * 1024 + 4000 * 8]
    if app != "cc-sync":
        args += ["--source", src]
    p = _run(bindir, app, *args)
    assert p.returncode == 0, p.stderr
    assert f"Number of nodes = {g.n}" in p.stdout and f"Number of edges = {g.m}" in p.stdout
    unit = "ms" if app == "sssp-sync" else "s"
    assert re.search(rf"Processing finished in [0-9.e+-]+ \({unit}\)", p.stdout)
    first = re.search(r"Results of first 30 nodes:\n\[(.*)\]", p.stdout).group(1).split(" ")
    assert len(first) == 30 and first[0].startswith("0:")
    rows = np.loadtxt(out)
    assert rows.shape == (g.n, 2) and np.array_equal(rows[:, 0], np.arange(g.n))
    e = g.edges if weighted else g.ends
    if algo == "pr":
        ref, _ = orc.pagerank(g.node_pointer, e)
        # the file carries 6 significant digits (%g), as the reference writes
        # it; async follows another schedule, bounded by acc / init
        bound = 1e-4 if app.endswith("sync") and not app.endswith("async") else 0.01 / 0.15
        assert np.max(np.abs(rows[:, 1] - ref) / ref) < bound
    else:
        ref = orc.run(algo, g.node_pointer, e, 0 if app == "cc-sync" else src)
        assert np.array_equal(rows[:, 1].astype(np.uint64), ref.astype(np.uint64))


@pytest.mark.gpu
def test_app_learned_scheduler_same_answers(gpu, orc, bindir, tmp_path):
    from subway_gb300 import scheduler
    g, path = _write(gpu, tmp_path, True)
    out = tmp_path / "out.txt"
    p = _run(bindir, "sssp-async", "--input", path, "--output", out, "--source", 1,
             "--budget", 18 * g.n + 96 * 1024 + 4000 * 12, "--scheduler", scheduler.DEFAULT_MODEL)
    assert p.returncode == 0, p.stderr
    assert re.search(r"Inner Iterations? in Global Iteration \d+, Range \d+", p.stdout)
    rows = np.loadtxt(out)
    assert np.array_equal(rows[:, 1].astype(np.uint64), orc.run("sssp", g.node_pointer, g.edges, 1).astype(np.uint64))


@pytest.mark.gpu
def test_pr_output_precision(gpu, orc, bindir, tmp_path):
    """--precision 9 writes every PageRank value so that it reads back as the
    same float32; the default keeps the reference's 6 digits."""
    g, path = _write(gpu, tmp_path, False)
    budget = 36 * g.n + 64 * 1024 + 4000 * 8
    for digits in (6, 9):
        out = tmp_path / f"pr{digits}.txt"
        args = ["--input", path, "--output", out, "--budget", budget]
        if digits != 6:
            args += ["--precision", digits]
        p = _run(bindir, "pr-sync", *args)
        assert p.returncode == 0, p.stderr
        vals = [ln.split()[1] for ln in out.read_text().splitlines()]
        sig = max(len(v.split("e")[0].replace(".", "").lstrip("0")) for v in vals)
        assert sig == digits
        x = np.array(vals, np.float64).astype(np.float32)
        if digits == 9:
            assert all(f"{float(v):.9g}" == s for v, s in zip(x, vals))
        ref, _ = orc.pagerank(g.node_pointer, g.ends)
        assert np.max(np.abs(x - ref) / ref) < 1e-4


@pytest.mark.gpu
def test_app_subway_compat_and_trace(gpu, orc, bindir, tmp_path):
    """--subway-compat 1 ignores vertex n-2's out-edges as the reference does
    (it never writes that out-degree, shared/graph.cu:179-181); without it
    they count.  --trace writes one CSV line per processed partition."""
    n = 3000
    rng = np.random.default_rng(11)
    deg = rng.integers(1, 8, n)
    deg[n - 2] = 60  # vertex n - 2 reaches much of the graph
    npt = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint32)
    dst = rng.integers(0, n, int(npt[-1])).astype(np.uint32)
    path = tmp_path / "g.bcsr"
    gpu.Graph.from_csr(npt, dst, False).save(path)
    cut = np.concatenate([dst[:npt[n - 2]], dst[npt[n - 1]:]])
    npc = npt.astype(np.int64).copy()
    npc[n - 1:] -= deg[n - 2]
    src = n - 2
    for compat, (p_, e_) in ((0, (npt, dst)), (1, (npc.astype(np.uint32), cut))):
        out, trace = tmp_path / f"out{compat}.txt", tmp_path / f"trace{compat}.csv"
        p = _run(bindir, "bfs-async", "--input", path, "--output", out, "--source", src, "--trace", trace,
                 "--subway-compat", compat, "--budget", 18 * n + 64 * 1024 + 2000 * 8)
        assert p.returncode == 0, p.stderr
        rows = np.loadtxt(out)
        assert np.array_equal(rows[:, 1].astype(np.uint64), orc.run("bfs", p_, e_, src).astype(np.uint64)), compat
        lines = trace.read_text().splitlines()
        assert lines[0].startswith("global_iteration,partition,") and len(lines) >= 2
        assert all(len(x.split(",")) == 11 for x in lines[1:])

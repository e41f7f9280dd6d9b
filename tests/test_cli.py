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


def test_cc_sync_rejects_source(bindir):
    """cc-sync has no --source (subway/cc-sync.cu:17); cc-async accepts it."""
    p = _run(bindir, "cc-sync", "--input", "g.bcsr", "--source", "3")
    assert p.returncode == 0 and "error parsing command line argument <--source>" in p.stdout
    assert "[--source]" not in p.stdout


def test_missing_file_fails_without_a_gpu_call(bindir, tmp_path):
    p = _run(bindir, "bfs-sync", "--input", tmp_path / "none.bcsr")
    assert p.returncode != 0 and "cannot open" in p.stderr


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

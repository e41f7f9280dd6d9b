"""The C++ role classes (include/subway_gb300.hpp): a program written like a
reference app's driver loop (subway/sssp-async.cu:77-122: generate,
partition, process each partition) compiles against the header and the
library (no GPU needed) and, on a GPU, gives the oracle's distances."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent

APP = r'''
#include <cstdio>
#include <vector>
#include "subway_gb300.hpp"
using namespace subway;

int main(int argc, char **argv) {
  if (argc != 5) return 2;
  try {
    Graph<OutEdgeWeighted> graph(argv[1], true);
    graph.ReadGraph();
    Subgraph<OutEdgeWeighted> subgraph(graph, std::stoull(argv[2]));
    SubgraphGenerator<OutEdgeWeighted> subgen(graph);
    subgraph.Init(SGW_SSSP, SGW_ASYNC, (uint)std::stoul(argv[3]));
    Partitioner<OutEdgeWeighted> partitioner;
    unsigned iterations = 0, partitions = 0;
    while (subgraph.numActiveNodes > 0) {
      partitioner.partition(subgraph, subgraph.numActiveNodes);
      for (uint i = 0; i < partitioner.numPartitions; i++) partitioner.process(subgraph, i);
      partitions += partitioner.numPartitions;
      subgen.generate(graph, subgraph);
      ++iterations;
    }
    std::vector<uint> value;
    subgraph.ReadValues(value);
    FILE *f = std::fopen(argv[4], "wb");
    std::fwrite(value.data(), sizeof(uint), value.size(), f);
    std::fclose(f);
    std::printf("iterations %u partitions %u\n", iterations, partitions);
  } catch (const Error &e) {
    std::fprintf(stderr, "%s (%d)\n", e.what(), e.status);
    return 1;
  }
  return 0;
}
'''


APP_PR = r'''
#include <cstdio>
#include <vector>
#include "subway_gb300.hpp"
using namespace subway;

// subway/pr-sync.cu's loop: GraphPR, generate with acc, partition, process
int main(int argc, char **argv) {
  if (argc != 4) return 2;
  try {
    GraphPR<OutEdge> graph(argv[1], false);
    graph.ReadGraph();
    Subgraph<OutEdge> subgraph(graph, std::stoull(argv[2]));
    SubgraphGenerator<OutEdge> subgen(graph);
    const float acc = 0.01f;
    subgraph.InitPR(SGW_SYNC, 0.15f, acc, 0.85f);
    Partitioner<OutEdge> partitioner;
    unsigned rounds = 0;
    while (subgraph.numActiveNodes > 0) {
      partitioner.partition(subgraph, subgraph.numActiveNodes);
      for (uint i = 0; i < partitioner.numPartitions; i++) partitioner.process(subgraph, i);
      subgen.generate(graph, subgraph, acc);
      ++rounds;
    }
    std::vector<float> value;
    subgraph.ReadValues(value);
    FILE *f = std::fopen(argv[3], "wb");
    std::fwrite(value.data(), sizeof(float), value.size(), f);
    std::fclose(f);
    std::printf("rounds %u\n", rounds);
  } catch (const Error &e) {
    std::fprintf(stderr, "%s (%d)\n", e.what(), e.status);
    return 1;
  }
  return 0;
}
'''


def _compile(src_text, d, name):
    from subway_gb300 import build
    src = d / f"{name}.cpp"
    src.write_text(src_text)
    exe = d / name
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe),
                    f"-L{build.LIBDIR}", "-lsubwaygb", f"-Wl,-rpath,{build.LIBDIR}"], check=True)
    return exe


@pytest.fixture(scope="module")
def role_app_pr(native, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    return _compile(APP_PR, tmp_path_factory.mktemp("roles_pr"), "roles_pr")


def test_pagerank_role_classes_compile(role_app_pr):
    assert role_app_pr.exists()


@pytest.mark.gpu
def test_pagerank_role_class_loop_matches_oracle(gpu, orc, role_app_pr, tmp_path):
    """GraphPR and the acc overload of generate, in subway/pr-sync.cu's loop
    under a budget that forces several partitions: the bulk-synchronous
    rounds of the FP64 oracle, cast to float."""
    g = gpu.Graph.rmat(12, 16, seed=92)
    path = tmp_path / "g.bcsr"
    g.save(path)
    out = tmp_path / "pr.bin"
    budget = 36 * g.n + 96 * 1024 + 4000 * 8
    p = subprocess.run([str(role_app_pr), str(path), str(budget), str(out)], capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 0, p.stderr
    ranks = np.fromfile(out, dtype=np.float32).astype(np.float64)
    init, acc, damp = (float(np.float32(x)) for x in (0.15, 0.01, 0.85))
    ref, _ = orc.pagerank(g.node_pointer, g.ends, init=init, acc=acc, damping=damp)
    assert np.max(np.abs(ranks - ref) / ref) < 1e-6


@pytest.fixture(scope="module")
def role_app(native, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    from subway_gb300 import build
    d = tmp_path_factory.mktemp("roles")
    src = d / "roles.cpp"
    src.write_text(APP)
    exe = d / "roles"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe),
                    f"-L{build.LIBDIR}", "-lsubwaygb", f"-Wl,-rpath,{build.LIBDIR}"], check=True)
    return exe


def test_role_classes_compile(role_app):
    assert role_app.exists()


@pytest.mark.gpu
def test_role_class_loop_matches_oracle(gpu, orc, role_app, tmp_path):
    g = gpu.Graph.rmat(12, 16, seed=91, weighted=True, wmax=64)
    path = tmp_path / "g.bwcsr"
    g.save(path)
    src = int(g.pick_sources(1, seed=3)[0])
    out = tmp_path / "d.bin"
    budget = 18 * g.n + 96 * 1024 + 4000 * 8
    p = subprocess.run([str(role_app), str(path), str(budget), str(src), str(out)], capture_output=True,
                       text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    parts = int(p.stdout.split()[3])
    assert parts > int(p.stdout.split()[1])  # the budget forces several partitions per iteration
    dist = np.fromfile(out, dtype=np.uint32)
    assert np.array_equal(dist, orc.run("sssp", g.node_pointer, g.edges, src))

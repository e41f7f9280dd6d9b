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

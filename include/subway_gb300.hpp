// subway_gb300.hpp — C++ role classes over the C ABI, shaped like the
// reference's Graph / GraphPR / Subgraph / SubgraphGenerator / Partitioner
// (shared/graph.cuh:7-59, shared/subgraph.cuh:8-29,
// shared/subgraph_generator.cuh:12-30, shared/partitioner.cuh:8-22).
//
// Differences a caller of the reference will notice:
//  - errors throw subway::Error (status code + message) instead of exit();
//  - Subgraph is built from the Graph and a device budget in bytes (the
//    reference derives its budget from totalGlobalMem, shared/subgraph.cu:24);
//  - vertex state lives on the device; read it with Subgraph::ReadValues.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "subway_gb300.h"

namespace subway {

typedef unsigned int uint;
typedef unsigned long long ull;

struct OutEdge { uint end; };                     // shared/globals.hpp:33-35
struct OutEdgeWeighted { uint end; uint w8; };    // shared/globals.hpp:37-40

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &what)
      : std::runtime_error(what + ": " + sgw_strerror(status) + " (" + sgw_last_error() + ")"),
        status(status) {}
  int status;
};

inline void check(int status, const char *what) {
  if (status != SGW_OK) throw Error(status, what);
}

template <class E>
class Graph {
 public:
  std::string graphFilePath;
  bool isWeighted;
  uint num_nodes = 0;
  uint num_edges = 0;
  const uint *nodePointer = nullptr;
  const E *edgeList = nullptr;
  std::vector<uint> outDegree;
  sgw_graph *handle = nullptr;

  Graph(std::string path, bool weighted) : graphFilePath(std::move(path)), isWeighted(weighted) {}
  Graph(const Graph &) = delete;
  Graph &operator=(const Graph &) = delete;
  ~Graph() { sgw_graph_free(handle); }

  // Graph<E>::ReadGraph (shared/graph.cu:32-197)
  void ReadGraph() {
    check(sgw_graph_load(graphFilePath.c_str(), &handle), "ReadGraph");
    int w = 0;
    check(sgw_graph_info(handle, &num_nodes, &num_edges, &w), "ReadGraph");
    if ((sizeof(E) == sizeof(OutEdgeWeighted)) && !w)
      throw Error(SGW_EFORMAT, "weighted application needs a .bwcsr/.wel input");
    nodePointer = sgw_graph_node_pointer(handle);
    edgeList = static_cast<const E *>(sgw_graph_edges(handle));
    outDegree.resize(num_nodes);
    check(sgw_graph_out_degree(handle, outDegree.data()), "ReadGraph");
  }
};

// GraphPR<E> (shared/graph.cuh:36-59): the same graph for PageRank.  Its
// ranks and residuals live on the device (FP64; Subgraph::InitPR sets
// value = 0 and delta = init, as subway/pr-sync.cu:33-40 does on the host)
// and are read as float with Subgraph::ReadValues.
template <class E>
class GraphPR : public Graph<E> {
 public:
  GraphPR(std::string path, bool weighted) : Graph<E>(std::move(path), weighted) {}
};

template <class E>
class Subgraph {
 public:
  uint num_nodes = 0;
  uint num_edges = 0;
  uint numActiveNodes = 0;
  ull numActiveEdges = 0;
  ull max_partition_size = 0;
  sgw_engine *engine = nullptr;

  explicit Subgraph(Graph<E> &g, ull budget_bytes = 0, int device = 0, uint flags = 0) {
    sgw_engine_opts o;
    sgw_engine_opts_default(&o);
    o.budget_bytes = budget_bytes;
    o.device = device;
    o.flags = flags;
    check(sgw_engine_create(g.handle, &o, &engine), "Subgraph");
    num_nodes = g.num_nodes;
    num_edges = g.num_edges;
    uint64_t cap = 0;
    check(sgw_engine_max_partition_size(engine, &cap), "Subgraph");
    max_partition_size = cap;
  }
  Subgraph(const Subgraph &) = delete;
  Subgraph &operator=(const Subgraph &) = delete;
  ~Subgraph() { sgw_engine_destroy(engine); }

  // Initial values/labels of an application plus its first generate.
  void Init(int algo, int mode, uint source) {
    sgw_run_params p;
    sgw_run_params_default(&p, algo, mode, source);
    check(sgw_state_init(engine, &p), "Init");
    uint64_t e = 0;
    sgw_run_stats st;
    check(sgw_get_stats(engine, &st), "Init");
    uint32_t cnt = 0;
    check(sgw_read_active(engine, nullptr, nullptr, 0xffffffffu, &cnt), "Init");
    numActiveNodes = cnt;
    (void)e;
  }

  // PageRank's initial state (value = 0, delta = init) and first generate,
  // with the activation threshold acc and the damping factor
  // (subway/pr-sync.cu:33-34, shared/gpu_kernels.cu:239).
  void InitPR(int mode, float init = 0.15f, float acc = 0.01f, float damping = 0.85f) {
    sgw_run_params p;
    sgw_run_params_default(&p, SGW_PR, mode, 0);
    p.pr_init = init;
    p.pr_acc = acc;
    p.pr_damping = damping;
    check(sgw_state_init(engine, &p), "InitPR");
    uint32_t cnt = 0;
    check(sgw_read_active(engine, nullptr, nullptr, 0xffffffffu, &cnt), "InitPR");
    numActiveNodes = cnt;
    pr_acc = acc;
  }
  float pr_acc = 0.01f;  // the threshold InitPR set

  template <class T>
  void ReadValues(std::vector<T> &out) {
    out.resize(num_nodes);
    check(sgw_read_values(engine, out.data()), "ReadValues");
  }
};

template <class E>
class SubgraphGenerator {
 public:
  explicit SubgraphGenerator(Graph<E> &) {}
  // SubgraphGenerator<E>::generate (shared/subgraph_generator.cu:128-204)
  void generate(Graph<E> &, Subgraph<E> &s) {
    uint32_t a = 0;
    uint64_t e = 0;
    check(sgw_generate(s.engine, &a, &e), "generate");
    s.numActiveNodes = a;
    s.numActiveEdges = e;
  }
  // The PageRank overload (shared/subgraph_generator.cu:128-204 with
  // prePrefix's PR form, :24-41): acc is the threshold of the run, fixed by
  // Subgraph::InitPR.
  void generate(GraphPR<E> &g, Subgraph<E> &s, float acc) {
    if (acc != s.pr_acc) throw Error(SGW_EINVAL, "generate: acc differs from the one InitPR set");
    generate(static_cast<Graph<E> &>(g), s);
  }
};

template <class E>
class Partitioner {
 public:
  uint numPartitions = 0;
  std::vector<uint> fromNode, fromEdge, partitionNodeSize;
  std::vector<ull> partitionEdgeSize;

  // Partitioner<E>::partition (shared/partitioner.cu:12-91)
  void partition(Subgraph<E> &s, uint /*numActiveNodes*/) {
    reset();
    uint32_t p = 0;
    check(sgw_partition(s.engine, &p), "partition");
    numPartitions = p;
    for (uint32_t i = 0; i < p; ++i) {
      uint32_t fn, fe, ns;
      uint64_t es;
      check(sgw_partition_info(s.engine, i, &fn, &fe, &ns, &es), "partition");
      fromNode.push_back(fn);
      fromEdge.push_back(fe);
      partitionNodeSize.push_back(ns);
      partitionEdgeSize.push_back(es);
    }
  }
  // The transfer and relaxation of partition i (subway/*-async.cu:85-117).
  uint process(Subgraph<E> &s, uint i) {
    uint32_t it = 0;
    check(sgw_process_partition(s.engine, i, &it), "process");
    return it;
  }
  void reset() {
    numPartitions = 0;
    fromNode.clear();
    fromEdge.clear();
    partitionNodeSize.clear();
    partitionEdgeSize.clear();
  }
};

}  // namespace subway

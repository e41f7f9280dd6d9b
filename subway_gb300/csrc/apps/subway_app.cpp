// The ten Subway applications as one binary: bfs|cc|sssp|sswp|pr - sync|async,
// chosen by the name it is invoked under (bin/<app> links to this program).
//
// Command line and output follow the reference apps:
//   flags as --flag value pairs (shared/argument_parsing.cu:25-119): --input
//   (required), --source (rejected by cc-sync), --output, --device; help and
//   argument errors print the help text and exit 0;
//   stdout lines of subway/<app>.cu and utilities::PrintResults /
//   SaveResults (shared/subway_utilities.cpp:4-72).
// Extra flags: --budget BYTES (device-memory budget), --inner N (async inner
// iterations per partition visit, 0 = until converged), --stats FILE (JSON),
// --scheduler MODEL (learned scheduling policy with this network file; the
// answers are the same, the schedule and the bytes moved change), --precision
// DIGITS (significant digits of PageRank values in the --output file; the
// reference writes 6, 9 round-trips every float exactly), --trace FILE (the
// per-partition trace as CSV), --subway-compat 1 (vertex n-2's out-edges
// ignored, as the reference ignores them: it never writes that vertex's
// out-degree, shared/graph.cu:179-181).
//
// Invoked as `converter`, it is the reference's tools/converter: one argument,
// a .el or .wel file, written beside it as .bcsr or .bwcsr (.bcsr64 / .bwcsr64
// at 2^32 edges or more)
// (tools/converter.cpp:20-172), through the library's parallel text reader.

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <algorithm>
#include <string>
#include <vector>

#include "subway_gb300.h"

namespace {

struct Args {
  std::string input, output, stats, scheduler, trace;
  bool compat = false;
  unsigned source = 0;
  int device = 0;
  unsigned long long budget = 0;
  unsigned inner = 0;
  int precision = 6;
  bool has_output = false;
};

std::string help(bool can_source) {
  std::string s = "\nRequired arguments:";
  s += "\n    [--input]: Input graph file. E.g., --input FacebookGraph.txt";
  s += "\nOptional arguments";
  if (can_source) s += "\n    [--source]:  Begins from the source (Default: 0). E.g., --source 10";
  s += "\n    [--output]: Output file for results. E.g., --output results.txt";
  s += "\n    [--device]: Select GPU device (default: 0). E.g., --device 1";
  s += "\n    [--budget]: Device-memory budget in bytes (default: Subway's rule). E.g., --budget 1000000000";
  s += "\n    [--inner]: Async inner iterations per partition visit (default: 0 = until converged)";
  s += "\n    [--stats]: Write run statistics as JSON to this file";
  s += "\n    [--scheduler]: Learned scheduling with this model file (e.g. subway_gb300/models/sched_mlp.bin)";
  s += "\n    [--precision]: Significant digits of float results in the output file (default: 6)";
  s += "\n    [--trace]: Write the per-partition trace as CSV to this file";
  s += "\n    [--subway-compat]: 1 = ignore vertex n-2's out-edges, as the reference does";
  s += "\n\n";
  return s;
}

[[noreturn]] void usage_exit(bool can_source, const char *msg) {
  if (msg) printf("%s", msg);
  printf("%s", help(can_source).c_str());
  exit(0);
}

Args parse(int argc, char **argv, bool can_source) {
  Args a;
  if (argc == 1) usage_exit(can_source, nullptr);
  if (argc == 2 && (!strcmp(argv[1], "--help") || !strcmp(argv[1], "-help") ||
                    !strcmp(argv[1], "--h") || !strcmp(argv[1], "-h")))
    usage_exit(can_source, nullptr);
  if (argc % 2 == 0) usage_exit(can_source, "\nThere was an error parsing command line arguments\n");
  bool has_input = false;
  for (int i = 1; i < argc - 1; i += 2) {
    const char *k = argv[i], *v = argv[i + 1];
    if (!strcmp(k, "--input")) { a.input = v; has_input = true; }
    else if (!strcmp(k, "--output")) { a.output = v; a.has_output = true; }
    else if (!strcmp(k, "--source") && can_source) a.source = (unsigned)atoi(v);
    else if (!strcmp(k, "--device")) a.device = atoi(v);
    else if (!strcmp(k, "--budget")) a.budget = strtoull(v, nullptr, 10);
    else if (!strcmp(k, "--inner")) a.inner = (unsigned)strtoul(v, nullptr, 10);
    else if (!strcmp(k, "--stats")) a.stats = v;
    else if (!strcmp(k, "--scheduler")) a.scheduler = v;
    else if (!strcmp(k, "--precision")) a.precision = std::max(1, std::min(17, atoi(v)));
    else if (!strcmp(k, "--trace")) a.trace = v;
    else if (!strcmp(k, "--subway-compat")) a.compat = atoi(v) != 0;
    else {
      std::string m = std::string("\nThere was an error parsing command line argument <") + k + ">\n";
      usage_exit(can_source, m.c_str());
    }
  }
  if (!has_input) usage_exit(can_source, "\nInput graph file argument is required.\n");
  return a;
}

double now_ms() {
  timeval t;
  gettimeofday(&t, nullptr);
  return t.tv_sec * 1000.0 + t.tv_usec / 1000.0;
}

void die(int st, const char *what) {
  fprintf(stderr, "%s: %s (%s)\n", what, sgw_strerror(st), sgw_last_error());
  exit(1);
}

template <class T>
void print_results(const std::vector<T> &v, unsigned n) {
  printf("Results of first %u nodes:\n[", n);
  for (unsigned i = 0; i < n; ++i) {
    if (i) printf(" ");
    if (sizeof(T) == 4 && T(0.5) == T(0)) printf("%u:%u", i, (unsigned)v[i]);
    else printf("%u:%g", i, (double)v[i]);
  }
  printf("]\n");
}

void save_u32(const std::string &path, const std::vector<unsigned> &v) {
  printf("Saving the results into the following file:\n>> %s\n", path.c_str());
  FILE *f = fopen(path.c_str(), "w");
  if (!f) die(SGW_EIO, "SaveResults");
  std::vector<char> buf(1 << 22);
  setvbuf(f, buf.data(), _IOFBF, buf.size());
  for (size_t i = 0; i < v.size(); ++i) fprintf(f, "%zu %u\n", i, v[i]);
  fclose(f);
  printf("Done saving.\n");
}

void save_f32(const std::string &path, const std::vector<float> &v, int digits) {
  printf("Saving the results into %s ...... ", path.c_str());
  fflush(stdout);
  FILE *f = fopen(path.c_str(), "w");
  if (!f) die(SGW_EIO, "SaveResults");
  std::vector<char> buf(1 << 22);
  setvbuf(f, buf.data(), _IOFBF, buf.size());
  for (size_t i = 0; i < v.size(); ++i) fprintf(f, "%zu %.*g\n", i, digits, (double)v[i]);
  fclose(f);
  printf(" Completed.\n");
}

// tools/converter: messages and exit codes as tools/converter.cpp:22-25,167-170.
int convert(int argc, char **argv) {
  if (argc != 2) {
    printf("\nThere was an error parsing command line arguments\n");
    return 0;
  }
  std::string in = argv[1];
  size_t dot = in.find_last_of('.');
  std::string ext = dot == std::string::npos ? "" : in.substr(dot + 1);
  if (ext != "el" && ext != "wel") {
    printf("\nInput file format is not supported.\n");
    return 0;
  }
  sgw_graph *g = nullptr;
  int st = sgw_graph_load(in.c_str(), &g);
  if (st != SGW_OK) die(st, "converter");
  // 2^32 edges or more do not fit the u32 header: the 64-bit form instead
  uint32_t n = 0;
  uint64_t m = 0;
  sgw_graph_info64(g, &n, &m, nullptr);
  std::string outp = in.substr(0, dot + 1) + (ext == "el" ? "bcsr" : "bwcsr") +
                     (m >= (uint64_t(1) << 32) ? "64" : "");
  if (m >= (uint64_t(1) << 32)) printf("%llu edges: writing %s\n", (unsigned long long)m, outp.c_str());
  st = sgw_graph_save(g, outp.c_str());
  sgw_graph_free(g);
  if (st != SGW_OK) die(st, "converter");
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  std::string name = argv[0];
  size_t slash = name.find_last_of('/');
  if (slash != std::string::npos) name = name.substr(slash + 1);
  if (name == "converter") return convert(argc, argv);
  size_t dash = name.find('-');
  std::string algo_s = name.substr(0, dash), mode_s = dash == std::string::npos ? "" : name.substr(dash + 1);
  int algo = algo_s == "bfs" ? SGW_BFS : algo_s == "sssp" ? SGW_SSSP : algo_s == "sswp" ? SGW_SSWP
           : algo_s == "cc" ? SGW_CC : algo_s == "pr" ? SGW_PR : -1;
  int mode = mode_s == "sync" ? SGW_SYNC : mode_s == "async" ? SGW_ASYNC : -1;
  if (algo < 0 || mode < 0) {
    fprintf(stderr, "invoke as one of bfs|cc|sssp|sswp|pr-sync|async (got %s)\n", name.c_str());
    return 2;
  }
  const bool can_source = !(algo == SGW_CC && mode == SGW_SYNC);  // cc-sync.cu:17
  Args a = parse(argc, argv, can_source);

  double t0 = now_ms();
  printf("Reading the input graph from the following file:\n>> %s\n", a.input.c_str());
  sgw_graph *g = nullptr;
  // every format is read into the library's memory (binary files with
  // parallel reads, as the reference reads the whole file, text parsed), so
  // that the engine can gather from the records in place
  int st = sgw_graph_load(a.input.c_str(), &g);
  if (st != SGW_OK) die(st, "ReadGraph");
  if (a.compat) {
    uint32_t nn = 0;
    sgw_graph_info64(g, &nn, nullptr, nullptr);
    if (nn >= 2 && (st = sgw_graph_clear_out_edges(g, nn - 2)) != SGW_OK) die(st, "subway-compat");
  }
  uint32_t n = 0;
  uint64_t m = 0;
  int weighted = 0;
  sgw_graph_info64(g, &n, &m, &weighted);
  printf("Done reading.\nNumber of nodes = %u\nNumber of edges = %llu\n", n, (unsigned long long)m);
  printf("Graph Reading finished in %g (s).\n", (now_ms() - t0) / 1000.0);

  sgw_engine_opts o;
  sgw_engine_opts_default(&o);
  o.budget_bytes = a.budget;
  o.device = a.device;
  // one query per process: no transfer copy where the GPU reads the records
  // in place, else the copy that is cheaper to set up
  o.flags |= SGW_OPT_GRAPH_IN_PLACE | SGW_OPT_PAGEABLE_COPY;
  if (!a.scheduler.empty() && a.budget) sgw_sched_buffers(g, a.budget, &o.num_buffers);
  sgw_engine *e = nullptr;
  st = sgw_engine_create(g, &o, &e);
  if (st != SGW_OK) die(st, "engine");
  sgw_mlp *model = nullptr;
  if (!a.scheduler.empty()) {
    st = sgw_mlp_load(a.device, a.scheduler.c_str(), &model);
    if (st != SGW_OK) die(st, "scheduler model");
    st = sgw_set_policy(e, SGW_POLICY_LEARNED, model);
    if (st != SGW_OK) die(st, "scheduler policy");
  }
  sgw_trace_enable(e, 1);
  sgw_run_params p;
  sgw_run_params_default(&p, algo, mode, a.source);
  p.max_inner = a.inner;
  std::vector<unsigned> vu;
  std::vector<float> vf;
  void *out = nullptr;
  if (algo == SGW_PR) { vf.resize(n); out = vf.data(); }
  else { vu.resize(n); out = vu.data(); }
  sgw_run_stats s;
  st = sgw_run(e, &p, out, &s);
  if (st != SGW_OK) die(st, "run");

  if (mode == SGW_ASYNC && model) {  // one line per processed vertex range
    uint64_t cnt = 0;
    sgw_range_trace_count(e, &cnt);
    std::vector<sgw_range_rec> tr(cnt);
    sgw_range_trace_read(e, tr.data(), cnt, &cnt);
    for (const auto &r : tr)
      if (r.active_nodes)
        printf("%u %s in Global Iteration %u, Range %u\n", r.inner_iterations,
               r.inner_iterations > 1 ? "Inner Iterations" : "Inner Iteration", r.global_iteration, r.range);
  } else if (mode == SGW_ASYNC) {  // per-partition log lines (subway/sssp-async.cu:117)
    uint64_t cnt = 0;
    sgw_trace_count(e, &cnt);
    std::vector<sgw_trace_rec> tr(cnt);
    sgw_trace_read(e, tr.data(), cnt, &cnt);
    for (const auto &r : tr) {
      if (algo == SGW_SSWP)
        for (uint32_t k = 1; k <= r.inner_iterations; ++k) printf("\t\tIteration %u\n", k);
      printf("%u %s in Global Iteration %u, Partition %u\n", r.inner_iterations,
             r.inner_iterations > 1 ? "Inner Iterations" : "Inner Iteration", r.global_iteration,
             r.partition);
    }
  }
  if (algo == SGW_SSSP && mode == SGW_SYNC)
    printf("Processing finished in %g (ms).\n", s.ms_device);  // sssp-sync.cu:92
  else
    printf("Processing finished in %g (s).\n", s.ms_device / 1000.0);
  if (mode == SGW_SYNC || algo == SGW_PR) printf("Number of iterations = %u\n", s.global_iterations);
  const unsigned shown = n < 30 ? n : 30;
  if (algo == SGW_PR) print_results(vf, shown);
  else print_results(vu, shown);
  if (a.has_output) {
    if (algo == SGW_PR) save_f32(a.output, vf, a.precision);
    else save_u32(a.output, vu);
  }
  if (!a.trace.empty() && (st = sgw_trace_save(e, a.trace.c_str())) != SGW_OK) die(st, "trace");
  if (!a.stats.empty()) {
    FILE *f = fopen(a.stats.c_str(), "w");
    if (f) {
      fprintf(f,
              "{\"global_iterations\": %u, \"partitions\": %u, \"inner_iterations\": %llu, "
              "\"h2d_bytes\": %llu, \"d2h_bytes\": %llu, \"reached_edges\": %llu, \"ms_device\": %.4f}\n",
              s.global_iterations, s.partitions, (unsigned long long)s.inner_iterations,
              (unsigned long long)s.h2d_bytes, (unsigned long long)s.d2h_bytes,
              (unsigned long long)s.reached_edges, s.ms_device);
      fclose(f);
    }
  }
  sgw_engine_destroy(e);
  if (model) sgw_mlp_destroy(model);
  sgw_graph_free(g);
  return 0;
}

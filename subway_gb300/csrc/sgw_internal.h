// Internal definitions shared by the host (g++) and device (nvcc) halves of
// libsubwaygb.  Not part of the public ABI.
#pragma once

#include <atomic>
#include <stddef.h>
#include <stdint.h>

#include "subway_gb300.h"

struct sgw_graph {
  uint32_t n = 0;
  uint64_t m = 0;
  int weighted = 0;
  uint32_t esz = 4;               // bytes per edge record (4 or 8)
  // n + 1 node pointers, [n] == m: u32 (node_pointer) for graphs of fewer
  // than 2^32 edges, which every reader and generator produces; u64
  // (node_pointer64) at 2^32 edges and above, and for a caller's u64 arrays
  // (sgw_graph_from_csr64).  Exactly one of the two is set.
  uint32_t *node_pointer = nullptr;
  uint64_t *node_pointer64 = nullptr;
  void *edges = nullptr;          // m * esz bytes, page aligned when owned
  bool owns = false;              // arrays allocated (and freed) by the library
  size_t edges_bytes_alloc = 0;   // rounded allocation size of edges
  void *map_base = nullptr;       // sgw_graph_map: the file mapping holding edges
  size_t map_len = 0;
  // Largest edge weight, found by the first engine created on a graph whose
  // records the library owns or maps read-only (-1: not known yet).  A
  // caller's arrays (sgw_graph_from_csr) may change between engines, so for
  // those it is found again every time.
  mutable std::atomic<int64_t> wmax_cache{-1};
};

namespace sgw {

// Node pointer v of either width.
inline uint64_t np_at(const sgw_graph *g, uint64_t v) {
  return g->node_pointer64 ? g->node_pointer64[v] : (uint64_t)g->node_pointer[v];
}
// Out-degree of v (below 2^32: degrees are checked when a graph is made).
inline uint32_t deg_at(const sgw_graph *g, uint64_t v) { return (uint32_t)(np_at(g, v + 1) - np_at(g, v)); }

// Node pointers on the device: the low 32 bits of every one (degrees are
// their differences) and, for graphs with u64 node pointers, the full pointer
// of every 2^kOffGroupLog2-th vertex (obase, n / 2^kOffGroupLog2 + 2 entries).
// No group of that many vertices spans 2^32 edges (checked when a graph is
// given to an engine or a batch), so the low bits and the group's base give
// the rest.
constexpr uint32_t kOffGroupLog2 = 10;
#ifdef __CUDACC__
__device__ __forceinline__ unsigned long long off_at(const uint32_t *off, const unsigned long long *obase,
                                                     uint32_t v) {
  const uint32_t o = off[v];
  if (!obase) return o;
  const unsigned long long b = obase[v >> kOffGroupLog2];
  return b + (uint32_t)(o - (uint32_t)b);
}
#endif
// The device form of a graph's node pointers: lo[v] = low 32 bits of
// np[v] (n + 1 entries) and, for u64 node pointers, base[k] = np[min(n, k <<
// kOffGroupLog2)].  Returns false (filling nothing) when some group spans
// 2^32 edges or more.
bool device_offsets(const sgw_graph *g, uint32_t *lo, unsigned long long *base);

// Records a status with a message for sgw_last_error() and returns it.
int fail(int status, const char *fmt, ...);
void clear_error();

// Page-aligned host allocation (64 KiB granularity, the page size of Arm GB300 hosts),
// suitable for cudaHostRegister.  Returns nullptr on failure.
void *host_alloc(size_t bytes, size_t *rounded);
void host_free(void *p);

// Creates a graph object owning freshly allocated arrays.
int graph_alloc(uint32_t n, uint64_t m, int weighted, sgw_graph **out);

// Transfer format for weighted graphs: one u32 per edge, (w << nbits) | dst,
// with nbits = bits of the largest vertex id.  Returns false, allocating
// nothing, when some weight does not fit in the remaining 32 - nbits bits.
bool pack_weighted(const sgw_graph *g, uint32_t **out, size_t *alloc_bytes, uint32_t *nbits);
// The same decision and fill into a caller-provided array of m words.
bool pack_bits(const sgw_graph *g, uint32_t *nbits);
// The same test given the largest weight (from max_weight).
bool pack_bits_for(const sgw_graph *g, uint32_t wmax, uint32_t *nbits);
// Edges [e0, e1) of the packed / split / record forms, written from out[0].
void pack_range(const sgw_graph *g, uint32_t nbits, uint32_t *out, uint64_t e0, uint64_t e1);
void split_ends_range(const sgw_graph *g, uint32_t *ends, uint64_t e0, uint64_t e1);
void split_weights_range(const sgw_graph *g, uint8_t *w8, uint64_t e0, uint64_t e1);
void copy_records_range(const sgw_graph *g, void *out, uint64_t e0, uint64_t e1);
// Parallel memcpy in 64 MiB pieces.
void copy_bytes(void *dst, const void *src, size_t bytes);
void pack_into(const sgw_graph *g, uint32_t nbits, uint32_t *out);
// Largest edge weight (0 for an unweighted graph).
uint32_t max_weight(const sgw_graph *g);

// Device address of a scheduler model's BF16 weights, and its device.
const void *mlp_device_weights(const sgw_mlp *m);
int mlp_device(const sgw_mlp *m);

// Greedy partition planner shared by the host entry point and the device
// planner: largest prefix of the queue starting at `from` whose edge count
// is <= cap, at least one vertex.
inline uint32_t plan_next(const uint32_t *ptr, uint32_t from, uint32_t count,
                          uint64_t cap) {
  // upper_bound over ptr[from+1 .. count] for ptr[from] + cap
  uint64_t limit = (uint64_t)ptr[from] + cap;
  uint32_t lo = from + 1, hi = count + 1;  // search in [lo, hi)
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo) / 2;
    if ((uint64_t)ptr[mid] <= limit) lo = mid + 1; else hi = mid;
  }
  uint32_t to = lo - 1;          // last index with ptr[to] - ptr[from] <= cap
  if (to <= from) to = from + 1; // one vertex larger than cap: its own run
  return to;
}

}  // namespace sgw

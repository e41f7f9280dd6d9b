// Batched multi-source BFS / SSSP over a graph resident in HBM: up to 64
// queries share one traversal, one lane (bit / distance column) per query.
// No counterpart in the reference, which answers one source per process.
//
// Device state: the CSR (packed 4-byte records when weights fit, as in the
// engine), dist[v][lane] (vertex-major, so a warp touches one 128-byte line
// per edge), and per-vertex 64-bit lane masks for the current and next
// frontier.  One iteration:
//   k_b_frontier  vertices with a next-mask move it to the current mask and
//                 append (vertex, edge chunk) work items
//   k_b_relax     one warp per work item: the 32 (or 2 x 32) lanes relax the
//                 item's edges for their own query; improvements are
//                 balloted into one atomicOr on the destination's next mask
//   k_b_cond      sets the conditional handle: loop while the frontier was
//                 non-empty (bounded by an iteration limit)
// The iteration is the body of a CUDA-graph conditional WHILE node, so a
// whole batch is one graph launch with no host round trip per iteration.

#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "sgw_internal.h"

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t _e = (call);                                                           \
    if (_e != cudaSuccess)                                                             \
      return sgw::fail(SGW_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), \
                       __FILE__, __LINE__);                                            \
  } while (0)

namespace {

constexpr uint32_t kBInf = 4294967294u;
constexpr int kBThreads = 256;
constexpr uint32_t kBUnroll = 4;

struct BItem {
  uint32_t u;    // source vertex
  uint32_t e0;   // first edge: low 32 bits
  uint32_t cnt;  // edges in this item
  uint32_t e0hi; //   and high 32 bits
};

// counters: [0] work items, [1] frontier vertices, [2] iterations run,
// [3] error (1 = item list overflow, 2 = iteration limit)
__global__ void k_b_fill(uint32_t *dist, size_t count, unsigned long long *next, unsigned long long *seen,
                         uint32_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    dist[i] = kBInf;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    next[v] = 0ull;
    seen[v] = 0ull;
  }
}

template <int L>
__global__ void k_b_seed(const uint32_t *src, uint32_t nsrc, uint32_t *dist, unsigned long long *next,
                         unsigned long long *seen, uint32_t *ctr) {
  const uint32_t l = threadIdx.x;
  if (l < nsrc) {
    const uint32_t s = src[l];
    dist[(size_t)s * L + l] = 0;
    atomicOr(&next[s], 1ull << l);
    atomicOr(&seen[s], 1ull << l);
  }
  if (l < 16) ctr[l] = 0;
}

__global__ void k_b_reset(uint32_t *ctr) {
  ctr[0] = 0;
  ctr[1] = 0;
}

// Loads that follow writes made earlier in the same launch (the persistent
// form runs every phase in one kernel) go through L2 (__ldcg): L1 and the
// read-only path are not kept coherent within a kernel.
__device__ __forceinline__ BItem b_item(const BItem *items, uint32_t i) {
  const uint4 v = __ldcg(reinterpret_cast<const uint4 *>(items) + i);
  BItem it;
  it.u = v.x;
  it.e0 = v.y;
  it.cnt = v.z;
  it.e0hi = v.w;
  return it;
}

// Frontier phase.  ctr[0]: work items appended, ctr[1]: frontier vertices;
// err: set to 1 when the item list overflows.
__device__ __forceinline__ size_t b_first_edge(const BItem &it) { return ((size_t)it.e0hi << 32) | it.e0; }

__device__ __forceinline__ void b_frontier(uint32_t n, const uint32_t *__restrict__ off,
                                           const unsigned long long *__restrict__ obase, unsigned long long *cur,
                                           unsigned long long *next, BItem *items, uint32_t cap, uint32_t *ctr,
                                           uint32_t chunk, uint32_t *err) {
  const int lane = threadIdx.x & 31;
  const uint32_t stride = gridDim.x * blockDim.x;
  // loop bound rounded up to whole warps so every lane reaches the shuffles
  const uint32_t limit = (n + 31) & ~31u;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < limit; v += stride) {
    uint32_t nch = 0, deg = 0;
    unsigned long long e0 = 0;
    bool act = false;
    if (v < n) {
      const unsigned long long m = __ldcg(&next[v]);
      if (m) {
        act = true;
        cur[v] = m;
        next[v] = 0ull;
        e0 = sgw::off_at(off, obase, v);
        deg = off[v + 1] - off[v];
        nch = (deg + chunk - 1) / chunk;
      }
    }
    const uint32_t nact = __popc(__ballot_sync(0xffffffffu, act));
    if (lane == 0 && nact) atomicAdd(&ctr[1], nact);
    // warp-aggregated reservation of item slots
    uint32_t incl = nch;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && tot) base = atomicAdd(&ctr[0], tot);
    base = __shfl_sync(0xffffffffu, base, 31) + incl - nch;
    for (uint32_t c = 0; c < nch; ++c) {
      if (base + c < cap) {
        BItem it;
        it.u = v;
        const unsigned long long f = e0 + (unsigned long long)c * chunk;
        it.e0 = (uint32_t)f;
        it.cnt = min(chunk, deg - c * chunk);
        it.e0hi = (uint32_t)(f >> 32);
        items[base + c] = it;
      } else {
        atomicExch(err, 1u);
      }
    }
  }
}

__global__ void __launch_bounds__(kBThreads) k_b_frontier(uint32_t n, const uint32_t *__restrict__ off,
                                                          const unsigned long long *__restrict__ obase,
                                                          unsigned long long *cur, unsigned long long *next,
                                                          BItem *items, uint32_t cap, uint32_t *ctr,
                                                          uint32_t chunk) {
  b_frontier(n, off, obase, cur, next, items, cap, ctr, chunk, &ctr[3]);
}

// Distance-lane relaxation phase over the nitems work items.
template <bool SSSP, int W, int L>
__device__ __forceinline__ void b_relax(const BItem *items, uint32_t nitems,
                                        const uint32_t *__restrict__ edges, uint32_t pbits, uint32_t *dist,
                                        const unsigned long long *cur, unsigned long long *next) {
  const int lane = threadIdx.x & 31;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  const uint32_t dmask = pbits ? ((1u << pbits) - 1u) : 0xffffffffu;
  for (uint32_t i = gw; i < nitems; i += nw) {
    const BItem it = b_item(items, i);
    const unsigned long long mask = __ldcg(&cur[it.u]);
#pragma unroll
    for (int h = 0; h < L / 32; ++h) {
      const uint32_t bits = (uint32_t)(mask >> (32 * h));
      if (bits == 0) continue;
      const bool active = (bits >> lane) & 1u;
      const uint32_t du = active ? __ldcg(&dist[(size_t)it.u * L + 32 * h + lane]) : kBInf;
      for (uint32_t c = 0; c < it.cnt; c += 32) {
        // lane k loads edge c + k; the warp then walks them together
        uint32_t rd = 0, rw = 0;
        if (c + lane < it.cnt) {
          const size_t e = b_first_edge(it) + c + lane;
          if (W == 1) {
            const uint32_t r = edges[e];
            rd = r & dmask;
            rw = pbits ? (r >> pbits) : 0u;
          } else {
            rd = edges[2 * e];
            rw = edges[2 * e + 1];
          }
        }
        const uint32_t cnt = min(32u, it.cnt - c);
        // kBUnroll destination lines in flight per warp before the compares
        for (uint32_t k0 = 0; k0 < cnt; k0 += kBUnroll) {
          uint32_t dst[kBUnroll], w[kBUnroll], seen[kBUnroll];
#pragma unroll
          for (int q = 0; q < kBUnroll; ++q) {
            dst[q] = __shfl_sync(0xffffffffu, rd, (k0 + q) & 31u);
            w[q] = __shfl_sync(0xffffffffu, rw, (k0 + q) & 31u);
          }
#pragma unroll
          for (int q = 0; q < kBUnroll; ++q)
            seen[q] = (active && k0 + q < cnt) ? __ldcg(&dist[(size_t)dst[q] * L + 32 * h + lane]) : 0u;
#pragma unroll
          for (int q = 0; q < kBUnroll; ++q) {
            if (k0 + q >= cnt) break;  // uniform across the warp
            // a candidate below the value read improves the destination in
            // this iteration (by this lane or by whichever wins), so the
            // non-returning atomic suffices and the lane bit is right
            bool improved = false;
            if (active) {
              const uint32_t cand = du + (SSSP ? w[q] : 1u);
              if (cand < seen[q]) {
                atomicMin(&dist[(size_t)dst[q] * L + 32 * h + lane], cand);
                improved = true;
              }
            }
            const uint32_t imp = __ballot_sync(0xffffffffu, improved);
            if (imp && lane == 0) atomicOr(&next[dst[q]], (unsigned long long)imp << (32 * h));
          }
        }
      }
    }
  }
}

template <bool SSSP, int W, int L>
__global__ void __launch_bounds__(kBThreads) k_b_relax(const BItem *__restrict__ items, const uint32_t *ctr,
                                                       uint32_t cap, const uint32_t *__restrict__ edges,
                                                       uint32_t pbits, uint32_t *dist,
                                                       const unsigned long long *__restrict__ cur,
                                                       unsigned long long *next) {
  b_relax<SSSP, W, L>(items, min(ctr[0], cap), edges, pbits, dist, cur, next);
}

// BFS, bit-parallel over the lanes (multi-source BFS): a vertex's 64-bit
// `seen` mask holds the queries that have reached it.  Lane k of the warp
// takes edge c + k of the item; one atomicOr claims, for every query whose
// frontier holds the item's vertex, the destination's still-unseen lanes;
// those get level = iteration + 1 and join the next frontier.  Each (vertex,
// query) bit is claimed exactly once, so the levels are the BFS levels.
template <int W, int L>
__device__ __forceinline__ void b_bfs_relax(const BItem *items, uint32_t nitems, uint32_t level,
                                            const uint32_t *__restrict__ edges, uint32_t pbits, uint32_t *dist,
                                            const unsigned long long *cur, unsigned long long *next,
                                            unsigned long long *seen) {
  const int lane = threadIdx.x & 31;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  const uint32_t dmask = pbits ? ((1u << pbits) - 1u) : 0xffffffffu;
  for (uint32_t i = gw; i < nitems; i += nw) {
    const BItem it = b_item(items, i);
    const unsigned long long f = __ldcg(&cur[it.u]);
    if (f == 0ull) continue;
    for (uint32_t c = lane; c < it.cnt; c += 32) {
      const size_t e = b_first_edge(it) + c;
      const uint32_t dst = W == 1 ? (edges[e] & dmask) : edges[2 * e];
      if ((__ldcg(&seen[dst]) & f) == f) continue;  // every query here has been there (a stale read only costs the atomic)
      const unsigned long long fresh = f & ~atomicOr(&seen[dst], f);
      if (fresh == 0ull) continue;
      atomicOr(&next[dst], fresh);
      for (unsigned long long m = fresh; m; m &= m - 1) dist[(size_t)dst * L + (__ffsll((long long)m) - 1)] = level;
    }
  }
}

template <int W, int L>
__global__ void __launch_bounds__(kBThreads) k_b_bfs_relax(const BItem *__restrict__ items, const uint32_t *ctr,
                                                           uint32_t cap, const uint32_t *__restrict__ edges,
                                                           uint32_t pbits, uint32_t *dist,
                                                           const unsigned long long *__restrict__ cur,
                                                           unsigned long long *next, unsigned long long *seen) {
  b_bfs_relax<W, L>(items, min(ctr[0], cap), ctr[2] + 1, edges, pbits, dist, cur, next, seen);
}

// ---- persistent form -----------------------------------------------------------
// One cooperative launch runs every iteration of a batch: frontier phase,
// grid barrier, relaxation phase, grid barrier, and the loop test, all on the
// device.  Counter words (ctr): [0..3] as in the graph loop (items, frontier,
// iterations, error), [4..7] the items / frontier counts of even and odd
// iterations (the next iteration's pair is cleared during the relaxation
// phase), [8] barrier arrivals, [9] barrier generation.  A barrier waits at
// most wait_ns (GPU global timer); a block that gives up records error 4 and
// returns, and every other block then gives up at its next barrier, so a lost
// block ends the kernel with an error instead of a hang.
struct BPersist {
  uint32_t n, cap, chunk, pbits, max_iters, expect_blocks;
  unsigned long long wait_ns;
  const uint32_t *off, *edges;
  const unsigned long long *obase;
  uint32_t *dist, *ctr;
  unsigned long long *cur, *next, *seen;
  BItem *items;
};

__device__ __forceinline__ unsigned long long b_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid barrier with a bounded wait; false once any block has given up.
__device__ bool b_grid_sync(const BPersist &a) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t *gen = a.ctr + 9;
    const uint32_t g = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(a.ctr + 8, 1u) == a.expect_blocks - 1) {
      a.ctr[8] = 0;
      __threadfence();
      atomicAdd(a.ctr + 9, 1u);
    } else {
      const unsigned long long t0 = b_now();
      while (*gen == g) {
        if (b_now() - t0 > a.wait_ns) {
          atomicExch(a.ctr + 3, 4u);
          ok = 0;
          break;
        }
        __nanosleep(200);
      }
    }
    __threadfence();
    if (*(volatile uint32_t *)(a.ctr + 3) == 4u) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <bool SSSP, int W, int L>
__global__ void __launch_bounds__(kBThreads) k_b_persist(BPersist a) {
  for (uint32_t it = 0;; ++it) {
    uint32_t *c = a.ctr + 4 + 2 * (it & 1u);
    b_frontier(a.n, a.off, a.obase, a.cur, a.next, a.items, a.cap, c, a.chunk, a.ctr + 3);
    if (!b_grid_sync(a)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      uint32_t *cn = a.ctr + 4 + 2 * ((it + 1) & 1u);
      cn[0] = 0;
      cn[1] = 0;
    }
    const uint32_t nitems = min(*(volatile uint32_t *)c, a.cap);
    if (SSSP) b_relax<true, W, L>(a.items, nitems, a.edges, a.pbits, a.dist, a.cur, a.next);
    else b_bfs_relax<W, L>(a.items, nitems, it + 1, a.edges, a.pbits, a.dist, a.cur, a.next, a.seen);
    if (!b_grid_sync(a)) return;
    const uint32_t frontier = *(volatile uint32_t *)(c + 1);
    const uint32_t err = *(volatile uint32_t *)(a.ctr + 3);
    const bool more = frontier > 0 && err == 0;
    if (!more || it + 1 >= a.max_iters) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ctr[2] = it + 1;
        if (more) a.ctr[3] = 2;  // iteration limit
      }
      return;
    }
  }
}

__global__ void k_b_cond(cudaGraphConditionalHandle handle, uint32_t *ctr, uint32_t max_iters) {
  const uint32_t it = ++ctr[2];
  uint32_t go = ctr[1] > 0 ? 1u : 0u;
  if (ctr[3]) go = 0;
  if (go && it >= max_iters) { ctr[3] = 2; go = 0; }
  cudaGraphSetConditional(handle, go);
}

// out[l * n + v - v0] = dist[v * L + l] for v in [v0, v0 + len), l < nsrc.
template <int L>
__global__ void k_b_transpose(const uint32_t *dist, uint32_t v0, uint32_t len, uint32_t nsrc, uint32_t *out,
                              uint32_t *) {
  __shared__ uint32_t tile[32][L + 1];
  const uint32_t vb = blockIdx.x * 32;
  for (uint32_t i = threadIdx.x; i < 32 * L; i += blockDim.x) {
    const uint32_t r = i / L, l = i % L;
    tile[r][l] = (vb + r < len) ? dist[(size_t)(v0 + vb + r) * L + l] : 0;
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < 32 * L; i += blockDim.x) {
    const uint32_t l = i / 32, r = i % 32;
    if (l < nsrc && vb + r < len) out[(size_t)l * len + vb + r] = tile[r][l];
  }
}

// 16-bit answers: unreached (kBInf) becomes 0xffff; a reached distance that
// does not fit below 0xffff sets *overflow (the run then reports SGW_ERANGE).
template <int L>
__global__ void k_b_transpose16(const uint32_t *dist, uint32_t v0, uint32_t len, uint32_t nsrc, uint16_t *out,
                                uint32_t *overflow) {
  __shared__ uint32_t tile[32][L + 1];
  const uint32_t vb = blockIdx.x * 32;
  for (uint32_t i = threadIdx.x; i < 32 * L; i += blockDim.x) {
    const uint32_t r = i / L, l = i % L;
    tile[r][l] = (vb + r < len) ? dist[(size_t)(v0 + vb + r) * L + l] : 0;
  }
  __syncthreads();
  bool over = false;
  for (uint32_t i = threadIdx.x; i < 32 * L; i += blockDim.x) {
    const uint32_t l = i / 32, r = i % 32;
    if (l < nsrc && vb + r < len) {
      uint32_t v = tile[r][l];
      if (v == kBInf) v = 0xffffu;
      else if (v >= 0xffffu) { over = true; v = 0xfffeu; }
      out[(size_t)l * len + vb + r] = (uint16_t)v;
    }
  }
  if (over) atomicExch(overflow, 1u);
}

}  // namespace

struct sgw_batch {
  const sgw_graph *g = nullptr;
  int device = 0;
  int num_sms = 0;
  uint32_t n = 0, W = 1, pbits = 0;
  uint64_t m = 0;
  uint32_t lanes = 64;            // 32 or 64 distance columns
  uint32_t chunk = 256;           // edges per work item
  uint32_t items_cap = 0;
  char *d_arena = nullptr;
  size_t arena_bytes = 0;
  uint32_t *d_off = nullptr, *d_edges = nullptr, *d_dist = nullptr, *d_stage = nullptr;
  unsigned long long *d_obase = nullptr;  // u64 node pointers: full pointer of every 1024th vertex
  unsigned long long *d_cur = nullptr, *d_next = nullptr, *d_seen = nullptr;
  BItem *d_items = nullptr;
  uint32_t *d_ctr = nullptr, *d_src = nullptr;
  uint32_t stage_vertices = 0;
  uint32_t *h_ctr = nullptr;      // pinned
  uint32_t *h_out = nullptr;      // pinned results, lanes x n (lane-major)
  cudaStream_t s = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaGraph_t graph[2] = {nullptr, nullptr};        // BFS, SSSP
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  uint32_t max_iters = 0;
  int form = 0;                   // 0: by algorithm, 1: persistent, 2: graph loop
};

namespace {

size_t al(size_t x) { return (x + 255) / 256 * 256; }

template <bool SSSP, int W, int L>
int capture_body(sgw_batch *b, cudaGraph_t body, cudaGraphConditionalHandle h) {
  CK(cudaStreamBeginCaptureToGraph(b->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  k_b_reset<<<1, 1, 0, b->s>>>(b->d_ctr);
  const uint32_t grid = (uint32_t)b->num_sms * 8;
  k_b_frontier<<<grid, kBThreads, 0, b->s>>>(b->n, b->d_off, b->d_obase, b->d_cur, b->d_next, b->d_items, b->items_cap,
                                             b->d_ctr, b->chunk);
  if (SSSP)
    k_b_relax<SSSP, W, L><<<grid, kBThreads, 0, b->s>>>(b->d_items, b->d_ctr, b->items_cap, b->d_edges, b->pbits,
                                                        b->d_dist, b->d_cur, b->d_next);
  else
    k_b_bfs_relax<W, L><<<grid, kBThreads, 0, b->s>>>(b->d_items, b->d_ctr, b->items_cap, b->d_edges, b->pbits,
                                                      b->d_dist, b->d_cur, b->d_next, b->d_seen);
  k_b_cond<<<1, 1, 0, b->s>>>(h, b->d_ctr, b->max_iters);
  cudaGraph_t out = nullptr;
  CK(cudaStreamEndCapture(b->s, &out));
  return SGW_OK;
}

template <bool SSSP>
int build_graph(sgw_batch *b) {
  const int k = SSSP ? 1 : 0;
  CK(cudaGraphCreate(&b->graph[k], 0));
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, b->graph[k], 1, cudaGraphCondAssignDefault));
  // the parameter union has no default constructor: build it in zeroed storage
  alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
  memset(raw, 0, sizeof(raw));
  cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(raw);
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, b->graph[k], nullptr, nullptr, 0, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  int st;
  if (b->lanes == 64)
    st = b->W == 1 ? capture_body<SSSP, 1, 64>(b, body, h) : capture_body<SSSP, 2, 64>(b, body, h);
  else
    st = b->W == 1 ? capture_body<SSSP, 1, 32>(b, body, h) : capture_body<SSSP, 2, 32>(b, body, h);
  if (st != SGW_OK) return st;
  CK(cudaGraphInstantiate(&b->exec[k], b->graph[k], 0));
  return SGW_OK;
}

// Launches the persistent kernel with as many blocks as fit on the device at
// once (the cooperative launch refuses more), so every block reaches the
// grid barriers.  extra_blocks > 0 makes each barrier wait for blocks that
// do not exist (the wait-limit check).
template <bool SSSP, int W, int L>
int launch_persist_t(sgw_batch *b, uint32_t extra_blocks, unsigned long long wait_ns) {
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_b_persist<SSSP, W, L>, kBThreads, 0));
  if (per_sm < 1) return sgw::fail(SGW_ECUDA, "persistent batch kernel does not fit on an SM");
  const uint32_t grid = (uint32_t)b->num_sms * (uint32_t)std::min(per_sm, 8);
  BPersist a;
  a.n = b->n;
  a.cap = b->items_cap;
  a.chunk = b->chunk;
  a.pbits = b->pbits;
  a.max_iters = b->max_iters;
  a.expect_blocks = grid + extra_blocks;
  a.wait_ns = wait_ns;
  a.off = b->d_off;
  a.obase = b->d_obase;
  a.edges = b->d_edges;
  a.dist = b->d_dist;
  a.ctr = b->d_ctr;
  a.cur = b->d_cur;
  a.next = b->d_next;
  a.seen = b->d_seen;
  a.items = b->d_items;
  void *args[] = {&a};
  CK(cudaLaunchCooperativeKernel((const void *)k_b_persist<SSSP, W, L>, dim3(grid), dim3(kBThreads), args, 0,
                                 b->s));
  return SGW_OK;
}

int launch_persist(sgw_batch *b, bool sssp, uint32_t extra_blocks, unsigned long long wait_ns) {
  if (b->lanes == 64) {
    if (b->W == 1) return sssp ? launch_persist_t<true, 1, 64>(b, extra_blocks, wait_ns)
                               : launch_persist_t<false, 1, 64>(b, extra_blocks, wait_ns);
    return sssp ? launch_persist_t<true, 2, 64>(b, extra_blocks, wait_ns)
                : launch_persist_t<false, 2, 64>(b, extra_blocks, wait_ns);
  }
  if (b->W == 1) return sssp ? launch_persist_t<true, 1, 32>(b, extra_blocks, wait_ns)
                             : launch_persist_t<false, 1, 32>(b, extra_blocks, wait_ns);
  return sssp ? launch_persist_t<true, 2, 32>(b, extra_blocks, wait_ns)
              : launch_persist_t<false, 2, 32>(b, extra_blocks, wait_ns);
}

// A grid barrier waits at most this long before the kernel gives up; a
// barrier of a healthy run waits for the slowest block of one phase (well
// under 100 ms on the largest graphs measured).
constexpr unsigned long long kBarrierWaitNs = 2000000000ull;

int batch_run(sgw_batch *b, int algo, const uint32_t *sources, uint32_t nsrc, void *out, uint32_t answer_bytes,
              sgw_batch_stats *stats, bool persistent, uint32_t extra_blocks, unsigned long long wait_ns);

// Default form per algorithm, measured on R-MAT 22-26 with 64 queries: the
// persistent kernel runs SSSP batches 2-9% faster than the graph loop and BFS
// batches within 4% either way, so SSSP takes it and BFS keeps the graph.
bool use_persistent(const sgw_batch *b, int algo) {
  return b->form == 1 || (b->form == 0 && algo == SGW_SSSP);
}

}  // namespace

extern "C" {

int sgw_batch_create(const sgw_graph *g, const sgw_engine_opts *opts, uint32_t lanes, sgw_batch **out) {
  sgw::clear_error();
  if (!g || !out) return sgw::fail(SGW_EINVAL, "null argument");
  *out = nullptr;
  if (lanes != 32 && lanes != 64) return sgw::fail(SGW_EINVAL, "lanes must be 32 or 64");
  sgw_engine_opts o;
  sgw_engine_opts_default(&o);
  if (opts) o = *opts;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return sgw::fail(SGW_ECUDA, "no CUDA device");
  }
  CK(cudaSetDevice(o.device));
  sgw_batch *b = new (std::nothrow) sgw_batch();
  if (!b) return sgw::fail(SGW_ENOMEM, "batch object");
  b->g = g;
  b->device = o.device;
  b->n = g->n;
  b->m = g->m;
  b->lanes = lanes;
  b->chunk = o.chunk_edges ? o.chunk_edges : 256;
  if ((o.flags & SGW_OPT_BATCH_PERSISTENT) && (o.flags & SGW_OPT_BATCH_GRAPH)) {
    delete b;
    return sgw::fail(SGW_EINVAL, "SGW_OPT_BATCH_PERSISTENT and SGW_OPT_BATCH_GRAPH exclude each other");
  }
  b->form = (o.flags & SGW_OPT_BATCH_PERSISTENT) ? 1 : (o.flags & SGW_OPT_BATCH_GRAPH) ? 2 : 0;
  {
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, o.device) != cudaSuccess || !coop) {
      cudaGetLastError();
      if (b->form == 1) {
        delete b;
        return sgw::fail(SGW_EINVAL, "device %d has no cooperative launch", o.device);
      }
      b->form = 2;
    }
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, o.device) != cudaSuccess) { delete b; return sgw::fail(SGW_ECUDA, "props"); }
  b->num_sms = prop.multiProcessorCount;
  // resident edge records: packed when the weights fit beside the ids
  uint32_t *packed = nullptr;
  size_t packed_bytes = 0;
  const void *src_edges = g->edges;
  b->W = g->weighted ? 2 : 1;
  if (g->weighted && !(o.flags & SGW_OPT_NO_PACK) && sgw::pack_weighted(g, &packed, &packed_bytes, &b->pbits)) {
    b->W = 1;
    src_edges = packed;
  }
  b->items_cap = (uint32_t)std::min<uint64_t>((uint64_t)g->m / b->chunk + g->n + 64, 0xffffffffull);
  b->stage_vertices = std::min<uint32_t>(g->n, 1u << 22);
  const bool wide = g->node_pointer64 != nullptr;
  const size_t nbase = (g->n >> sgw::kOffGroupLog2) + 2;
  const size_t need = al(4ull * (g->n + 1)) + (wide ? al(8 * nbase) : 0) + al((size_t)g->m * 4 * b->W) + al((size_t)g->n * lanes * 4) +
                      3 * al(8ull * g->n) + al(sizeof(BItem) * (size_t)b->items_cap) + al(64) + al(256) +
                      al((size_t)b->stage_vertices * lanes * 4);
  if (o.budget_bytes && need > o.budget_bytes) {
    sgw::host_free(packed);
    delete b;
    return sgw::fail(SGW_EBUDGET, "graph and %u query lanes need %zu B > budget %llu B", lanes, need,
                     (unsigned long long)o.budget_bytes);
  }
  auto cleanup = [&](int st) { sgw::host_free(packed); sgw_batch_destroy(b); return st; };
  if (cudaMalloc(&b->d_arena, need) != cudaSuccess) { cudaGetLastError(); return cleanup(sgw::fail(SGW_ECUDA, "cudaMalloc(%zu)", need)); }
  b->arena_bytes = need;
  char *p = b->d_arena;
  auto take = [&](size_t bytes) { char *r = p; p += al(bytes); return r; };
  b->d_off = (uint32_t *)take(4ull * (g->n + 1));
  if (wide) b->d_obase = (unsigned long long *)take(8 * nbase);
  b->d_edges = (uint32_t *)take((size_t)g->m * 4 * b->W);
  b->d_dist = (uint32_t *)take((size_t)g->n * lanes * 4);
  b->d_cur = (unsigned long long *)take(8ull * g->n);
  b->d_next = (unsigned long long *)take(8ull * g->n);
  b->d_seen = (unsigned long long *)take(8ull * g->n);
  b->d_items = (BItem *)take(sizeof(BItem) * (size_t)b->items_cap);
  b->d_ctr = (uint32_t *)take(64);
  b->d_src = (uint32_t *)take(256);
  b->d_stage = (uint32_t *)take((size_t)b->stage_vertices * lanes * 4);
  b->max_iters = 4u * g->n + 64u;  // label-correcting rounds never exceed this
  if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess ||
      cudaMallocHost(&b->h_ctr, 64) != cudaSuccess ||
      cudaHostAlloc((void **)&b->h_out, (size_t)g->n * lanes * 4, cudaHostAllocPortable) != cudaSuccess)
    return cleanup(sgw::fail(SGW_ECUDA, "stream/event/pinned setup"));
  cudaError_t ce;
  if (!wide) {
    ce = cudaMemcpyAsync(b->d_off, g->node_pointer, 4ull * (g->n + 1), cudaMemcpyHostToDevice, b->s);
  } else {
    std::vector<uint32_t> lo((size_t)g->n + 1);
    std::vector<unsigned long long> base(nbase);
    if (!sgw::device_offsets(g, lo.data(), base.data()))
      return cleanup(sgw::fail(SGW_ERANGE, "1024 consecutive vertices hold 2^32 edges or more"));
    ce = cudaMemcpy(b->d_off, lo.data(), 4 * lo.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(b->d_obase, base.data(), 8 * base.size(), cudaMemcpyHostToDevice);
  }
  if (ce == cudaSuccess && g->m)
    ce = cudaMemcpyAsync(b->d_edges, src_edges, (size_t)g->m * 4 * b->W, cudaMemcpyHostToDevice, b->s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->s);
  sgw::host_free(packed);
  packed = nullptr;
  if (ce != cudaSuccess) return cleanup(sgw::fail(SGW_ECUDA, "graph upload: %s", cudaGetErrorString(ce)));
  int st = build_graph<false>(b);
  if (st == SGW_OK && g->weighted) st = build_graph<true>(b);
  if (st != SGW_OK) { sgw_batch_destroy(b); return st; }
  *out = b;
  return SGW_OK;
}

int sgw_batch_destroy(sgw_batch *b) {
  if (!b) return SGW_OK;
  cudaSetDevice(b->device);
  if (b->s) cudaStreamSynchronize(b->s);
  for (int k = 0; k < 2; ++k) {
    if (b->exec[k]) cudaGraphExecDestroy(b->exec[k]);
    if (b->graph[k]) cudaGraphDestroy(b->graph[k]);
  }
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  if (b->s) cudaStreamDestroy(b->s);
  if (b->h_ctr) cudaFreeHost(b->h_ctr);
  if (b->h_out) cudaFreeHost(b->h_out);
  if (b->d_arena) cudaFree(b->d_arena);
  cudaGetLastError();
  delete b;
  return SGW_OK;
}

int sgw_batch_results(const sgw_batch *b, const uint32_t **results) {
  if (!b || !results) return sgw::fail(SGW_EINVAL, "null argument");
  *results = b->h_out;
  return SGW_OK;
}

int sgw_batch_device_bytes(const sgw_batch *b, uint64_t *bytes) {
  if (!b || !bytes) return sgw::fail(SGW_EINVAL, "null argument");
  *bytes = b->arena_bytes;
  return SGW_OK;
}

int sgw_batch_run(sgw_batch *b, int algo, const uint32_t *sources, uint32_t nsrc, uint32_t *out,
                  sgw_batch_stats *stats) {
  sgw::clear_error();
  if (!b) return sgw::fail(SGW_EINVAL, "null argument");
  return batch_run(b, algo, sources, nsrc, out, 4, stats, use_persistent(b, algo), 0, kBarrierWaitNs);
}

int sgw_batch_run_u16(sgw_batch *b, int algo, const uint32_t *sources, uint32_t nsrc, uint16_t *out,
                      sgw_batch_stats *stats) {
  sgw::clear_error();
  if (!b) return sgw::fail(SGW_EINVAL, "null argument");
  return batch_run(b, algo, sources, nsrc, out, 2, stats, use_persistent(b, algo), 0, kBarrierWaitNs);
}

int sgw_batch_check_wait_timeout(sgw_batch *b, uint64_t wait_ns) {
  sgw::clear_error();
  if (!b) return sgw::fail(SGW_EINVAL, "null argument");
  if (wait_ns == 0 || wait_ns > 1000000000ull) return sgw::fail(SGW_EINVAL, "wait_ns outside 1..1e9");
  const uint32_t src = 0;
  return batch_run(b, SGW_BFS, &src, 1, nullptr, 4, nullptr, true, 1, wait_ns);
}

}  // extern "C"

namespace {

int batch_run(sgw_batch *b, int algo, const uint32_t *sources, uint32_t nsrc, void *out, uint32_t answer_bytes,
              sgw_batch_stats *stats, bool persistent, uint32_t extra_blocks, unsigned long long wait_ns) {
  if (!b || !sources) return sgw::fail(SGW_EINVAL, "null argument");
  if (!out) out = b->h_out;  // results stay in the batch's pinned buffer
  if (nsrc == 0 || nsrc > b->lanes) return sgw::fail(SGW_ERANGE, "1..%u sources per batch", b->lanes);
  if (algo != SGW_BFS && algo != SGW_SSSP) return sgw::fail(SGW_EINVAL, "batches run BFS or SSSP");
  if (algo == SGW_SSSP && !b->g->weighted) return sgw::fail(SGW_EINVAL, "SSSP needs a weighted graph");
  for (uint32_t i = 0; i < nsrc; ++i)
    if (sources[i] >= b->n) return sgw::fail(SGW_EINVAL, "source %u out of range", sources[i]);
  CK(cudaSetDevice(b->device));
  const auto w0 = std::chrono::steady_clock::now();
  CK(cudaMemcpyAsync(b->d_src, sources, 4ull * nsrc, cudaMemcpyHostToDevice, b->s));
  CK(cudaEventRecord(b->t0, b->s));
  const size_t cells = (size_t)b->n * b->lanes;
  k_b_fill<<<b->num_sms * 8, 256, 0, b->s>>>(b->d_dist, cells, b->d_next, b->d_seen, b->n);
  if (b->lanes == 64) k_b_seed<64><<<1, 64, 0, b->s>>>(b->d_src, nsrc, b->d_dist, b->d_next, b->d_seen, b->d_ctr);
  else k_b_seed<32><<<1, 64, 0, b->s>>>(b->d_src, nsrc, b->d_dist, b->d_next, b->d_seen, b->d_ctr);
  CK(cudaGetLastError());
  if (persistent) {
    const int st = launch_persist(b, algo == SGW_SSSP, extra_blocks, wait_ns);
    if (st != SGW_OK) return st;
  } else {
    CK(cudaGraphLaunch(b->exec[algo == SGW_SSSP ? 1 : 0], b->s));
  }
  CK(cudaEventRecord(b->t1, b->s));
  // lane-major results, staged through a transposed device tile
  const size_t ab = answer_bytes;
  char *outb = static_cast<char *>(out);
  for (uint32_t v0 = 0; v0 < b->n; v0 += b->stage_vertices) {
    const uint32_t len = std::min(b->stage_vertices, b->n - v0);
    const uint32_t blocks = (len + 31) / 32;
    uint16_t *st16 = reinterpret_cast<uint16_t *>(b->d_stage);
    if (ab == 2) {
      if (b->lanes == 64) k_b_transpose16<64><<<blocks, 256, 0, b->s>>>(b->d_dist, v0, len, nsrc, st16, b->d_ctr + 10);
      else k_b_transpose16<32><<<blocks, 256, 0, b->s>>>(b->d_dist, v0, len, nsrc, st16, b->d_ctr + 10);
    } else {
      if (b->lanes == 64) k_b_transpose<64><<<blocks, 256, 0, b->s>>>(b->d_dist, v0, len, nsrc, b->d_stage, nullptr);
      else k_b_transpose<32><<<blocks, 256, 0, b->s>>>(b->d_dist, v0, len, nsrc, b->d_stage, nullptr);
    }
    CK(cudaGetLastError());
    CK(cudaMemcpy2DAsync(outb + ab * v0, ab * b->n, b->d_stage, ab * len, ab * len, nsrc,
                         cudaMemcpyDeviceToHost, b->s));
  }
  CK(cudaMemcpyAsync(b->h_ctr, b->d_ctr, 64, cudaMemcpyDeviceToHost, b->s));
  CK(cudaStreamSynchronize(b->s));
  if (b->h_ctr[3] == 1) return sgw::fail(SGW_ERANGE, "work item list overflow");
  if (b->h_ctr[3] == 2) return sgw::fail(SGW_ETIMEOUT, "iteration limit reached");
  if (b->h_ctr[3] == 4) return sgw::fail(SGW_ETIMEOUT, "grid barrier wait timed out");
  if (b->h_ctr[10]) return sgw::fail(SGW_ERANGE, "a distance does not fit 16 bits: use sgw_batch_run");
  if (stats) {
    float ms = 0;
    cudaEventElapsedTime(&ms, b->t0, b->t1);
    stats->iterations = b->h_ctr[2];
    stats->queries = nsrc;
    stats->ms_device = ms;
    stats->ms_wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    stats->d2h_bytes = ab * b->n * nsrc;
  }
  return SGW_OK;
}

}  // namespace


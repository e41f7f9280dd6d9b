// Device kernels of the engine (sm_103a).
//
// Hot path per global iteration (reference: shared/subgraph_generator.cu:
// 128-204 and subway/*-{sync,async}.cu):
//   k_generate_count / _scan / _write (BFS, SSSP, SSWP, CC) and k_generate
//                (PageRank; single-pass decoupled-lookback scan): activeness,
//                scan and compaction into the active queue (replaces
//                prePrefix, thrust::reduce, two thrust::exclusive_scan,
//                makeQueue, makeActiveNodesPointer)
//   k_plan       greedy partition boundaries on the device (Partitioner)
//   k_gather_v   active-edge gather from the engine's mapped pinned transfer
//                copy of the edges into an HBM edge buffer, 16-byte reads
//                (replaces the host std::thread copy dynamic<E>); k_gather
//                is the one-record-per-thread form
//   k_relax_warp warp-cooperative expansion of 32 frontier sources at a time
//                (bfs/sssp/sswp/cc kernels, sync and async forms); k_relax_tile
//                the CTA-tile form staged in shared memory
//   k_relax_chunks warp-per-chunk expansion of high-degree sources
// Learned policy only (no reference counterpart):
//   k_select_*   value range, degree histogram and cut of the frontier when
//                far vertices are deferred
//   k_range_stats per-range features and the scheduler network's forward pass
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "sgw_internal.h"
#include "sgw_mlp.cuh"

namespace sgw {

constexpr uint32_t kInf = 4294967294u;  // DIST_INFINITY (shared/globals.hpp:27)

// ---- device control block -------------------------------------------------
struct Ctl {
  uint32_t tile_ticket;      // dynamic tile index of the running scan
  uint32_t tile_done;        // finished tiles of the running scan
  uint32_t error;            // nonzero: a bounded wait gave up
  uint32_t num_active;       // queued vertices (degree > 0) of the last generate
  unsigned long long num_active_edges;
  uint32_t num_parts;        // partitions of the last plan
  uint32_t num_seen;         // vertices found active (any degree)
  uint32_t upd[4];           // async inner iteration k: relaxations that improved
  uint32_t wl_count[4];      // chunk-list items of inner iteration k
  uint32_t iters_run;        // inner iterations that did work
  uint32_t hub_active;       // single-vertex partition: the source was dirty
  uint32_t hub_value;        // single-vertex partition: its value
  uint32_t sel_bin;          // deferral: the last value bin selected this iteration
  uint32_t iters_total;      // inner iterations that did work, whole run
  unsigned long long reached_edges;
  unsigned long long relaxed_edges;
  unsigned long long relaxed_sources;
  double hub_push;           // single-vertex PR partition: its push value
};

struct Part {                // one partition of the active queue
  uint32_t from;             // first queue index
  uint32_t size;             // queue entries
  uint32_t edge_from;        // ptr[from]
  uint32_t first_vertex;     // queue[from]
  unsigned long long edge_count;
};

struct WorkItem {            // a chunk of one high-degree source's edges
  uint32_t boff;             // first edge in the device edge buffer
  uint32_t count;            // edges in this chunk
  uint32_t value;            // source value snapshot
  uint32_t vertex;
};

// ---- small PTX helpers ----------------------------------------------------
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// First index in a[0, n) whose value is >= x (a sorted ascending).
__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *a, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Warp-inclusive scan of a u32.
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  return x;
}

// Bounded wait on a scan tile flag; returns the flag, or 0 after the limit
// (and records the error).  Flags are (epoch << 2) | status, status 1 =
// aggregate available, 2 = inclusive prefix available.
constexpr uint32_t kSpinLimit = 1u << 22;
__device__ __forceinline__ uint32_t wait_tile_flag(const uint32_t *flag, uint32_t epoch, Ctl *ctl) {
  for (uint32_t spin = 0; spin < kSpinLimit; ++spin) {
    uint32_t f = ld_acquire_u32(flag);
    if ((f >> 2) == epoch && (f & 3u) != 0) return f;
    __nanosleep(spin < 64 ? 32 : 256);
  }
  atomicExch(&ctl->error, 1u);
  return 0;
}

// Decoupled look-back for tile `tile` with aggregate `agg`, run by a whole
// warp.  Values are packed (count << 32) | edges; both sums stay below 2^32
// so the packed add never carries.  Lane k examines predecessors
// tile - 1 - (kLookPer k + q) - 32 kLookPer r, q < kLookPer, so one round
// covers 32 kLookPer predecessors; the sum stops at the nearest predecessor
// whose inclusive prefix is published.  One per lane measured best: with 4
// per lane (128 per round) a tile waits on more unpublished neighbours and
// the scan ran 30-40% longer.  Called by all lanes of one warp; returns the
// exclusive prefix on every lane.
constexpr int kLookPer = 1;
__device__ __forceinline__ unsigned long long lookback_warp(
    uint32_t tile, unsigned long long agg, uint32_t *tflag, unsigned long long *tagg,
    unsigned long long *tincl, uint32_t epoch, Ctl *ctl, int lane) {
  if (tile == 0) {
    if (lane == 0) {
      st_relaxed_u64(&tincl[0], agg);
      st_release_u32(&tflag[0], (epoch << 2) | 2u);
    }
    return 0ull;
  }
  if (lane == 0) {
    st_relaxed_u64(&tagg[tile], agg);
    st_release_u32(&tflag[tile], (epoch << 2) | 1u);
  }
  unsigned long long excl = 0;
  for (int32_t base = (int32_t)tile - 1;; base -= 32 * kLookPer) {
    unsigned long long v[kLookPer];
    uint32_t f[kLookPer];
    int stop_q = kLookPer;  // nearest of this lane's predecessors that ends the walk
    // the lane's 4 flags are read together; only a flag not yet published
    // for this epoch is waited on (bounded)
#pragma unroll
    for (int q = 0; q < kLookPer; ++q) {
      const int32_t j = base - (lane * kLookPer + q);
      f[q] = j >= 0 ? ld_acquire_u32(&tflag[j]) : 0u;
    }
#pragma unroll
    for (int q = 0; q < kLookPer; ++q) {
      const int32_t j = base - (lane * kLookPer + q);
      if (j >= 0 && !((f[q] >> 2) == epoch && (f[q] & 3u) != 0)) f[q] = wait_tile_flag(&tflag[j], epoch, ctl);
    }
#pragma unroll
    for (int q = 0; q < kLookPer; ++q) {
      const int32_t j = base - (lane * kLookPer + q);
      v[q] = 0;
      if (j < 0 || f[q] == 0) {  // before tile 0 (an inclusive 0), or timed out (error recorded)
        if (stop_q == kLookPer) stop_q = q;
      } else if ((f[q] & 3u) == 2u) {
        v[q] = ld_relaxed_u64(&tincl[j]);
        if (stop_q == kLookPer) stop_q = q;
      } else {
        v[q] = ld_relaxed_u64(&tagg[j]);
      }
    }
    // the walk ends at the nearest (lowest lane, then lowest q) stopping predecessor
    const uint32_t stop = __ballot_sync(0xffffffffu, stop_q < kLookPer);
    const int first = stop ? __ffs(stop) - 1 : 32;
    const int first_q = __shfl_sync(0xffffffffu, stop_q, first < 32 ? first : 0);
    unsigned long long s = 0;
#pragma unroll
    for (int q = 0; q < kLookPer; ++q)
      if (lane < first || (lane == first && q <= first_q)) s += v[q];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    excl += s;
    if (stop) break;
  }
  if (lane == 0) {
    st_relaxed_u64(&tincl[tile], excl + agg);
    st_release_u32(&tflag[tile], (epoch << 2) | 2u);
  }
  return excl;
}

// ---- generate: activeness -> scan -> compaction --------------------------
constexpr int kGenThreads = 256;
constexpr int kGenRounds = 16;
constexpr uint32_t kGenTile = kGenThreads * kGenRounds;  // 4096 vertices

struct GenArgs {
  uint32_t n;
  uint8_t *l1;
  uint8_t *l2;
  const uint32_t *off;       // n + 1 node pointers (device copy)
  uint32_t *queue;           // activeNodes
  uint32_t *ptr;             // activeNodesPointer (count + 1)
  uint32_t *tflag;
  unsigned long long *tagg;
  unsigned long long *tincl;
  Ctl *ctl;
  uint32_t *gmask;           // count/write form: per 16-vertex group, keep bits | clear bits << 16
  uint32_t epoch;
  uint32_t num_tiles;
  int consume;               // sync: labels of queued vertices are cleared
  // Count/write form: most edges one generate queues (0: no limit).  Only
  // whole tiles are queued, in order, up to the limit (the first tile with
  // edges always); the later tiles keep their labels, and the count pass
  // leaves label clearing to the write pass of the tiles that are queued.
  uint32_t edge_limit = 0;
  // PageRank form (activeness delta > acc instead of labels)
  double *delta;             // pending residual per vertex
  double *pval;              // accumulated rank per vertex
  double *qpush;             // per queued vertex: damping * delta / outdeg
  double acc;
  double damping;
  // Value-aware selection (integer algorithms, learned policy), bit flags:
  // 1: active vertices that cannot push (BFS/SSSP value INF, SSWP value 0)
  //    are dropped like degree-0 ones, since relaxing them changes nothing;
  // 2: active vertices whose value lies beyond the bin chosen by
  //    k_select_pick are deferred (labels kept, not queued).
  int sel_mode = 0;
  int algo = 0;
  const uint32_t *value = nullptr;
};

// Whether a vertex with this value produces candidates when relaxed.
__device__ __forceinline__ bool pushable(int algo, uint32_t v) {
  if (algo == SGW_BFS || algo == SGW_SSSP) return v != kInf;
  if (algo == SGW_SSWP) return v != 0;
  return true;
}

// Deferral bins: fixed and monotone in the value, so one pass builds the
// histogram: values below 64 get a bin each, larger ones 32 bins per power of
// two (bin < 896 of kSelBins).  Min-algorithms take the lowest bins first,
// SSWP (max) the highest.
constexpr uint32_t kSelBins = 1024;
__device__ __forceinline__ uint32_t sel_bin_of(uint32_t v) {
  if (v < 64u) return v;
  const uint32_t e = 31u - (uint32_t)__clz((int)v);
  return 64u + (e - 6u) * 32u + ((v >> (e - 5u)) & 31u);
}
__device__ __forceinline__ bool selected(int algo, uint32_t v, uint32_t bin) {
  const uint32_t b = sel_bin_of(v);
  return algo == SGW_SSWP ? b >= bin : b <= bin;
}

// One CTA per 4096-vertex tile.  Each warp owns 512 consecutive vertices,
// 32 per round: a lane reads label1|label2 of its vertex, the warp ballots the
// activeness, and only active lanes read their node pointers to get degrees.
// Active vertices of degree 0 have nothing to relax: their labels are
// cleared here and they are not queued.  Integer algorithms; the engine uses
// the count / scan / write form, this single-pass form serves the
// allocation-free entry point.
__global__ void __launch_bounds__(kGenThreads) k_generate(GenArgs a) {
  __shared__ uint32_t s_tile;
  __shared__ unsigned long long s_warp[kGenThreads / 32];
  __shared__ unsigned long long s_prefix;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(&a.ctl->tile_ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  if (tile >= a.num_tiles) {  // stale ticket counter: refuse to index past the tiles
    if (tid == 0) atomicExch(&a.ctl->error, 4u);
    return;
  }
  const uint32_t wbase = tile * kGenTile + warp * (32 * kGenRounds);

  uint32_t deg[kGenRounds];
  uint32_t keepmask[kGenRounds];
  uint32_t wcount = 0, wedges = 0, seen = 0;
  uint32_t sel_bin = 0;
  if (a.sel_mode & 2) sel_bin = a.ctl->sel_bin;
#pragma unroll
  for (int r = 0; r < kGenRounds; ++r) {
    const uint32_t v = wbase + r * 32 + lane;
    bool act = false, defer = false;
    uint32_t d = 0;
    if (v < a.n) {
      act = (a.l1[v] | a.l2[v]) != 0;
      if (act) {
        d = __ldg(&a.off[v + 1]) - __ldg(&a.off[v]);
        bool drop = d == 0;
        if (a.sel_mode && !drop) {
          const uint32_t val = a.value[v];
          if (!pushable(a.algo, val)) drop = (a.sel_mode & 1) != 0;
          else if ((a.sel_mode & 2) && !selected(a.algo, val, sel_bin)) defer = true;
        }
        if (!defer && (a.consume || drop)) { a.l1[v] = 0; a.l2[v] = 0; }
        if (drop) d = 0;
      }
    }
    seen += __popc(__ballot_sync(0xffffffffu, act));
    const bool keep = act && d > 0 && !defer;
    keepmask[r] = __ballot_sync(0xffffffffu, keep);
    deg[r] = keep ? d : 0;
    wcount += __popc(keepmask[r]);
    wedges += __reduce_add_sync(0xffffffffu, deg[r]);
  }
  if (lane == 0) {
    s_warp[warp] = ((unsigned long long)wcount << 32) | wedges;
    if (seen) atomicAdd(&a.ctl->num_seen, seen);
  }
  __syncthreads();
  if (warp == 0) {
    unsigned long long acc = 0;
    if (lane == 0) {
#pragma unroll
      for (int w = 0; w < kGenThreads / 32; ++w) {
        unsigned long long x = s_warp[w];
        s_warp[w] = acc;
        acc += x;
      }
    }
    acc = __shfl_sync(0xffffffffu, acc, 0);
    const unsigned long long excl = lookback_warp(tile, acc, a.tflag, a.tagg, a.tincl, a.epoch, a.ctl, lane);
    if (lane == 0) {
      s_prefix = excl;
      if (tile == a.num_tiles - 1) {
        const unsigned long long tot = excl + acc;
        const uint32_t cnt = (uint32_t)(tot >> 32);
        a.ctl->num_active = cnt;
        a.ctl->num_active_edges = tot & 0xffffffffull;
        a.ptr[cnt] = (uint32_t)(tot & 0xffffffffull);  // sentinel (subgraph_generator.cu:160)
      }
    }
  }
  __syncthreads();
  unsigned long long run = s_prefix + s_warp[warp];
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int r = 0; r < kGenRounds; ++r) {
    const uint32_t incl = warp_incl_scan(deg[r], lane);
    const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
    if (keepmask[r] & (1u << lane)) {
      const uint32_t pos = (uint32_t)(run >> 32) + __popc(keepmask[r] & lt);
      a.queue[pos] = wbase + r * 32 + lane;
      a.ptr[pos] = (uint32_t)(run & 0xffffffffull) + (incl - deg[r]);
    }
    run += ((unsigned long long)__popc(keepmask[r]) << 32) | tot;
  }
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&a.ctl->tile_done, 1u) == a.num_tiles - 1) {
      a.ctl->tile_ticket = 0;
      a.ctl->tile_done = 0;
    }
  }
}

// Integer-family generate with 16 consecutive vertices per lane, in three
// launches with no chain between CTAs: k_generate_count, k_generate_scan,
// k_generate_write.  A lane reads its vertices' labels as two 16-byte words
// and, only if one of them is active, their 17 node pointers (and values, for
// the learned policy's selection) as 16-byte words.  The count pass stores
// each 4096-vertex tile's (queued vertices, edges) total; one CTA turns the
// totals into exclusive tile prefixes; the write pass recomputes the same
// selection from the same labels and values, scans within the tile, writes
// the queue and pointers in order and clears the consumed labels.  Labels
// and values do not change between the passes (nothing else runs on the
// stream in between), so both passes select the same vertices.  Same results
// as k_generate<false>; the label, pointer and value arrays must be 16-byte
// aligned (the engine's arena is).
//
// The single-pass form with a decoupled look-back (k_generate, kept for
// PageRank and the allocation-free entry point) took 1.7-2x as long on
// RMAT-24: with hundreds of tiles in flight the prefixes travel 32 tiles per
// look-back step and every CTA of a wave waits for them, while the second
// pass's labels and pointers come mostly from L2.
constexpr uint32_t kGenVPerLane = 16;

struct GenLane {
  uint32_t keepmask = 0, clearmask = 0, cnt = 0, edges = 0, seen = 0;
  uint32_t l1w[4] = {0, 0, 0, 0}, l2w[4] = {0, 0, 0, 0};
  uint32_t o[kGenVPerLane + 1];  // node pointers; a queued vertex's degree is o[k + 1] - o[k]
};

// Selection for the lane's 16 vertices starting at v0.
__device__ __forceinline__ void gen_lane(const GenArgs &a, uint32_t v0, bool full, GenLane &L) {
  uint32_t sel_bin = 0;
  if (a.sel_mode & 2) sel_bin = a.ctl->sel_bin;
  if (full) {
    const uint4 x = *reinterpret_cast<const uint4 *>(a.l1 + v0);
    const uint4 y = *reinterpret_cast<const uint4 *>(a.l2 + v0);
    L.l1w[0] = x.x; L.l1w[1] = x.y; L.l1w[2] = x.z; L.l1w[3] = x.w;
    L.l2w[0] = y.x; L.l2w[1] = y.y; L.l2w[2] = y.z; L.l2w[3] = y.w;
  } else {
    for (uint32_t k = 0; k < kGenVPerLane; ++k)
      if (v0 + k < a.n) {
        L.l1w[k / 4] |= (uint32_t)a.l1[v0 + k] << (8 * (k % 4));
        L.l2w[k / 4] |= (uint32_t)a.l2[v0 + k] << (8 * (k % 4));
      }
  }
  uint32_t actmask = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t lw = L.l1w[q] | L.l2w[q];
#pragma unroll
    for (int b = 0; b < 4; ++b)
      if ((lw >> (8 * b)) & 0xffu) actmask |= 1u << (4 * q + b);
  }
  L.seen = (uint32_t)__popc(actmask);
  if (!actmask) return;
  uint32_t val[kGenVPerLane];
  if (full) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint4 p = __ldg(reinterpret_cast<const uint4 *>(a.off + v0) + q);
      L.o[4 * q] = p.x; L.o[4 * q + 1] = p.y; L.o[4 * q + 2] = p.z; L.o[4 * q + 3] = p.w;
    }
    L.o[kGenVPerLane] = __ldg(&a.off[v0 + kGenVPerLane]);
    if (a.sel_mode) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint4 p = reinterpret_cast<const uint4 *>(a.value + v0)[q];
        val[4 * q] = p.x; val[4 * q + 1] = p.y; val[4 * q + 2] = p.z; val[4 * q + 3] = p.w;
      }
    }
  } else {
#pragma unroll
    for (uint32_t k = 0; k <= kGenVPerLane; ++k) L.o[k] = (v0 + k <= a.n) ? __ldg(&a.off[v0 + k]) : 0u;
#pragma unroll
    for (uint32_t k = 0; k < kGenVPerLane; ++k) val[k] = (a.sel_mode && v0 + k < a.n) ? a.value[v0 + k] : 0u;
  }
#pragma unroll
  for (uint32_t k = 0; k < kGenVPerLane; ++k) {
    if (!((actmask >> k) & 1u)) continue;
    uint32_t d = L.o[k + 1] - L.o[k];
    bool drop = d == 0, defer = false;
    if (a.sel_mode && !drop) {
      if (!pushable(a.algo, val[k])) drop = (a.sel_mode & 1) != 0;
      else if ((a.sel_mode & 2) && !selected(a.algo, val[k], sel_bin)) defer = true;
    }
    if (!defer && (a.consume || drop)) L.clearmask |= 1u << k;
    if (!drop && !defer) {
      L.keepmask |= 1u << k;
      ++L.cnt;
      L.edges += d;
    }
  }
}

// PageRank selection for the lane's 16 vertices (prePrefix PR overload,
// shared/subgraph_generator.cu:24-41): active = delta > acc.  keepmask: the
// active vertices with out-edges (queued); clearmask: every active vertex,
// whose residual the write pass moves into its rank.  Reads only.
__device__ __forceinline__ void gen_lane_pr(const GenArgs &a, uint32_t v0, bool full, GenLane &L) {
  double dl[kGenVPerLane];
  if (full) {
#pragma unroll
    for (int q = 0; q < kGenVPerLane / 2; ++q) {
      const double2 p = reinterpret_cast<const double2 *>(a.delta + v0)[q];
      dl[2 * q] = p.x;
      dl[2 * q + 1] = p.y;
    }
  } else {
#pragma unroll
    for (uint32_t k = 0; k < kGenVPerLane; ++k) dl[k] = v0 + k < a.n ? a.delta[v0 + k] : 0.0;
  }
  uint32_t actmask = 0;
#pragma unroll
  for (uint32_t k = 0; k < kGenVPerLane; ++k)
    if (dl[k] > a.acc) actmask |= 1u << k;
  L.seen = (uint32_t)__popc(actmask);
  L.clearmask = actmask;
  if (!actmask) return;
  if (full) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint4 p = __ldg(reinterpret_cast<const uint4 *>(a.off + v0) + q);
      L.o[4 * q] = p.x; L.o[4 * q + 1] = p.y; L.o[4 * q + 2] = p.z; L.o[4 * q + 3] = p.w;
    }
    L.o[kGenVPerLane] = __ldg(&a.off[v0 + kGenVPerLane]);
  } else {
#pragma unroll
    for (uint32_t k = 0; k <= kGenVPerLane; ++k) L.o[k] = (v0 + k <= a.n) ? __ldg(&a.off[v0 + k]) : 0u;
  }
#pragma unroll
  for (uint32_t k = 0; k < kGenVPerLane; ++k) {
    const uint32_t d = L.o[k + 1] - L.o[k];
    if (((actmask >> k) & 1u) && d) {
      L.keepmask |= 1u << k;
      ++L.cnt;
      L.edges += d;
    }
  }
}

// Clears the labels of the lane's vertices in L.clearmask (16-byte stores of
// the words read by gen_lane when the group is whole).
__device__ __forceinline__ void gen_clear(const GenArgs &a, uint32_t v0, bool full, const GenLane &L) {
  if (!L.clearmask) return;
  uint32_t cw[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    cw[q] = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b)
      if ((L.clearmask >> (4 * q + b)) & 1u) cw[q] |= 0xffu << (8 * b);
  }
  if (full) {
    *reinterpret_cast<uint4 *>(a.l1 + v0) =
        make_uint4(L.l1w[0] & ~cw[0], L.l1w[1] & ~cw[1], L.l1w[2] & ~cw[2], L.l1w[3] & ~cw[3]);
    *reinterpret_cast<uint4 *>(a.l2 + v0) =
        make_uint4(L.l2w[0] & ~cw[0], L.l2w[1] & ~cw[1], L.l2w[2] & ~cw[2], L.l2w[3] & ~cw[3]);
  } else {
    for (uint32_t k = 0; k < kGenVPerLane; ++k)
      if ((L.clearmask >> k) & 1u) { a.l1[v0 + k] = 0; a.l2[v0 + k] = 0; }
  }
}

// Count pass: the selection of every lane's 16 vertices, whose keep and
// clear bits it records per group (so the write pass reads 4 bytes per 16
// vertices instead of the labels and values again), the label clearing, and
// the tile's (count, edges) total.
template <bool PR>
__global__ void __launch_bounds__(kGenThreads) k_generate_count(GenArgs a) {
  __shared__ unsigned long long s_warp[kGenThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t tile = blockIdx.x;
  const uint32_t v0 = tile * kGenTile + warp * (32 * kGenRounds) + lane * kGenVPerLane;
  const bool full = v0 + kGenVPerLane <= a.n;
  GenLane L;
  if (v0 < a.n) {
    if (PR) {
      gen_lane_pr(a, v0, full, L);  // residuals move in the write pass
    } else {
      gen_lane(a, v0, full, L);
      if (!a.edge_limit) gen_clear(a, v0, full, L);
    }
    a.gmask[v0 / kGenVPerLane] = L.keepmask | (L.clearmask << 16);
  }
  const uint32_t seen = __reduce_add_sync(0xffffffffu, L.seen);
  const uint32_t c = __reduce_add_sync(0xffffffffu, L.cnt);
  const uint32_t e = __reduce_add_sync(0xffffffffu, L.edges);
  if (lane == 0) {
    s_warp[warp] = ((unsigned long long)c << 32) | e;
    if (seen) atomicAdd(&a.ctl->num_seen, seen);
  }
  __syncthreads();
  if (tid == 0) {
    unsigned long long acc = 0;
#pragma unroll
    for (int w = 0; w < kGenThreads / 32; ++w) acc += s_warp[w];
    a.tagg[tile] = acc;
  }
}

// One CTA: exclusive prefixes of the tile totals (count << 32 | edges) into
// tincl, the totals into the control block and the pointer sentinel
// (subgraph_generator.cu:160).
constexpr int kGenScanThreads = 1024;

// Exclusive prefix of x over the CTA's threads (kGenScanThreads), in thread order.
__device__ __forceinline__ unsigned long long gen_block_excl(unsigned long long x, unsigned long long *s_warp) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  unsigned long long incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  __syncthreads();  // s_warp may still be read by a previous call
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long w = s_warp[lane];
    unsigned long long wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += y;
    }
    s_warp[lane] = wi - w;
  }
  __syncthreads();
  return s_warp[warp] + incl - x;
}

// The scan under an edge limit: tile t is queued when the edges of the tiles
// before it plus its own stay within the limit, or when no tile before it has
// edges.  The queued tiles are a prefix (the edge prefix only grows); each
// gets its (count, edges) prefix in tincl, the others ~0, and the last
// queued tile writes the totals and the sentinel.
__device__ __forceinline__ void gen_scan_limited(const GenArgs &a, uint32_t lo, uint32_t hi,
                                                 unsigned long long *s_warp) {
  unsigned long long sc = 0, se = 0;
  for (uint32_t t = lo; t < hi; ++t) {
    const unsigned long long x = a.tagg[t];
    sc += x >> 32;
    se += x & 0xffffffffull;
  }
  unsigned long long rc = gen_block_excl(sc, s_warp);
  unsigned long long re = gen_block_excl(se, s_warp);
  const unsigned long long lim = a.edge_limit;
  for (uint32_t t = lo; t < hi; ++t) {
    const unsigned long long x = a.tagg[t];
    const unsigned long long ct = x >> 32, et = x & 0xffffffffull;
    const bool in = re + et <= lim || re == 0;
    a.tincl[t] = in ? ((rc << 32) | re) : ~0ull;
    if (in) {
      bool next_in = false;
      if (t + 1 < a.num_tiles) {
        const unsigned long long ne = re + et, en = a.tagg[t + 1] & 0xffffffffull;
        next_in = ne + en <= lim || ne == 0;
      }
      if (!next_in) {
        const uint32_t c = (uint32_t)(rc + ct);
        a.ctl->num_active = c;
        a.ctl->num_active_edges = re + et;
        a.ptr[c] = (uint32_t)(re + et);
      }
    }
    rc += ct;
    re += et;
  }
}

__global__ void __launch_bounds__(kGenScanThreads) k_generate_scan(GenArgs a) {
  __shared__ unsigned long long s_warp[kGenScanThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t per = (a.num_tiles + kGenScanThreads - 1) / kGenScanThreads;
  const uint32_t lo = min(a.num_tiles, tid * per), hi = min(a.num_tiles, lo + per);
  if (a.edge_limit) {
    gen_scan_limited(a, lo, hi, s_warp);
    return;
  }
  unsigned long long sum = 0;
  for (uint32_t t = lo; t < hi; ++t) sum += a.tagg[t];
  unsigned long long incl = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = s_warp[lane];
    unsigned long long wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += y;
    }
    s_warp[lane] = wi - w;
    if (lane == 31) {
      const uint32_t c = (uint32_t)(wi >> 32);
      a.ctl->num_active = c;
      a.ctl->num_active_edges = wi & 0xffffffffull;
      a.ptr[c] = (uint32_t)(wi & 0xffffffffull);
    }
  }
  __syncthreads();
  unsigned long long run = s_warp[warp] + incl - sum;
  for (uint32_t t = lo; t < hi; ++t) {
    const unsigned long long x = a.tagg[t];
    a.tincl[t] = run;
    run += x;
  }
}

// Write pass: the group's keep bits from the count pass, the node pointers
// of groups that queue a vertex, and the queue / pointer entries.  PR: every
// active vertex's residual moves into its rank (value += delta, delta = 0,
// the first half of pr_kernel, shared/gpu_kernels.cu:234-250) and its queue
// entry carries the push damping * delta / outdeg, so each round is a
// bulk-synchronous snapshot.
template <bool PR>
__global__ void __launch_bounds__(kGenThreads) k_generate_write(GenArgs a) {
  __shared__ unsigned long long s_warp[kGenThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t tile = blockIdx.x;
  const uint32_t v0 = tile * kGenTile + warp * (32 * kGenRounds) + lane * kGenVPerLane;
  const bool full = v0 + kGenVPerLane <= a.n;
  if (a.edge_limit && a.tincl[tile] == ~0ull) return;  // beyond the limit: labels kept for later
  GenLane L;
  if (v0 < a.n) {
    const uint32_t gm = a.gmask[v0 / kGenVPerLane];
    L.keepmask = gm & 0xffffu;
    if (!PR && a.edge_limit && (gm >> 16)) {  // the clearing the count pass left to this tile
      L.clearmask = gm >> 16;
      if (full) {
        const uint4 x = *reinterpret_cast<const uint4 *>(a.l1 + v0);
        const uint4 y = *reinterpret_cast<const uint4 *>(a.l2 + v0);
        L.l1w[0] = x.x; L.l1w[1] = x.y; L.l1w[2] = x.z; L.l1w[3] = x.w;
        L.l2w[0] = y.x; L.l2w[1] = y.y; L.l2w[2] = y.z; L.l2w[3] = y.w;
      }
      gen_clear(a, v0, full, L);
    }
    if (L.keepmask) {
      if (full) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint4 p = __ldg(reinterpret_cast<const uint4 *>(a.off + v0) + q);
          L.o[4 * q] = p.x; L.o[4 * q + 1] = p.y; L.o[4 * q + 2] = p.z; L.o[4 * q + 3] = p.w;
        }
        L.o[kGenVPerLane] = __ldg(&a.off[v0 + kGenVPerLane]);
      } else {
#pragma unroll
        for (uint32_t k = 0; k <= kGenVPerLane; ++k) L.o[k] = (v0 + k <= a.n) ? __ldg(&a.off[v0 + k]) : 0u;
      }
      L.cnt = (uint32_t)__popc(L.keepmask);
#pragma unroll
      for (uint32_t k = 0; k < kGenVPerLane; ++k)
        if ((L.keepmask >> k) & 1u) L.edges += L.o[k + 1] - L.o[k];
    }
  }
  const uint32_t incl_c = warp_incl_scan(L.cnt, lane);
  const uint32_t incl_e = warp_incl_scan(L.edges, lane);
  if (lane == 31) s_warp[warp] = ((unsigned long long)incl_c << 32) | incl_e;
  __syncthreads();
  if (tid == 0) {
    unsigned long long acc = a.tincl[tile];
#pragma unroll
    for (int w = 0; w < kGenThreads / 32; ++w) {
      const unsigned long long x = s_warp[w];
      s_warp[w] = acc;
      acc += x;
    }
  }
  __syncthreads();
  if (L.keepmask) {
    const unsigned long long run = s_warp[warp] + (((unsigned long long)(incl_c - L.cnt) << 32) | (incl_e - L.edges));
    uint32_t pos = (uint32_t)(run >> 32), ep = (uint32_t)(run & 0xffffffffull);
#pragma unroll
    for (uint32_t k = 0; k < kGenVPerLane; ++k) {
      if ((L.keepmask >> k) & 1u) {
        const uint32_t d = L.o[k + 1] - L.o[k];
        a.queue[pos] = v0 + k;
        a.ptr[pos] = ep;
        if (PR) a.qpush[pos] = a.damping * a.delta[v0 + k] / (double)d;
        ++pos;
        ep += d;
      }
    }
  }
  if (PR && v0 < a.n) {  // residuals of every active vertex (queued or of degree 0) into the ranks
    const uint32_t cm = a.gmask[v0 / kGenVPerLane] >> 16;
#pragma unroll
    for (uint32_t k = 0; k < kGenVPerLane; ++k)
      if ((cm >> k) & 1u) {
        a.pval[v0 + k] += a.delta[v0 + k];
        a.delta[v0 + k] = 0.0;
      }
  }
}

// ---- frontier deferral (learned policy) --------------------------------------
// Before a generate, two small passes pick how much of the frontier to take:
// a histogram of the pushable active vertices' out-degrees over the fixed
// value bins, and the bin at which the cumulative degree reaches the target
// (lowest values first; highest for SSWP).  The
// generate then queues only the selected vertices; the rest keep their labels
// for a later iteration.  Relaxing far vertices first wastes their edges'
// transfer when they improve again later; this is the delta-stepping idea
// applied to out-of-memory partitions.
// Visits the pushable active vertices of degree > 0: each thread reads the
// two label arrays 16 bytes at a time (label arrays are 256-byte aligned),
// so a pass over n vertices keeps enough loads in flight to run at memory
// speed; only active vertices read their pointers and value.
template <class F>
__device__ __forceinline__ void for_sel_candidates(uint32_t n, int algo, const uint8_t *l1, const uint8_t *l2,
                                                   const uint32_t *off, const uint32_t *value, F f) {
  const uint32_t nvec = n / 16u;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  auto visit = [&](uint32_t v) {
    const uint32_t deg = __ldg(&off[v + 1]) - __ldg(&off[v]);
    if (deg == 0) return;
    const uint32_t val = value[v];
    if (pushable(algo, val)) f(val, deg);
  };
  for (uint32_t i = tid; i < nvec; i += nth) {
    const uint4 a = reinterpret_cast<const uint4 *>(l1)[i];
    const uint4 b = reinterpret_cast<const uint4 *>(l2)[i];
    const uint32_t w[4] = {a.x | b.x, a.y | b.y, a.z | b.z, a.w | b.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (w[q] == 0) continue;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if ((w[q] >> (8 * k)) & 0xffu) visit(16u * i + 4u * q + k);
    }
  }
  for (uint32_t v = 16u * nvec + tid; v < n; v += nth)
    if ((l1[v] | l2[v]) != 0) visit(v);
}

// Per-CTA bins in shared memory (per-CTA sums stay below m < 2^32), added
// into 64-bit global bins at the end.
__global__ void __launch_bounds__(256) k_select_hist(uint32_t n, int algo, const uint8_t *l1, const uint8_t *l2,
                                                     const uint32_t *off, const uint32_t *value, const Ctl *ctl,
                                                     unsigned long long *hist) {
  __shared__ uint32_t s_hist[kSelBins];
  for (uint32_t i = threadIdx.x; i < kSelBins; i += blockDim.x) s_hist[i] = 0u;
  __syncthreads();
  for_sel_candidates(n, algo, l1, l2, off, value,
                     [&](uint32_t val, uint32_t deg) { atomicAdd(&s_hist[sel_bin_of(val)], deg); });
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < kSelBins; i += blockDim.x)
    if (s_hist[i]) atomicAdd(&hist[i], (unsigned long long)s_hist[i]);
}

// One CTA of kSelBins / 4 threads: cumulative degree over the bins in
// selection order; sel_bin = first bin at which it reaches `target`.
__global__ void __launch_bounds__(kSelBins / 4) k_select_pick(int algo, const unsigned long long *hist,
                                                              unsigned long long target, Ctl *ctl) {
  __shared__ unsigned long long s_part[kSelBins / 4 / 32];
  __shared__ uint32_t s_k;  // first position (selection order) reaching the target
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool rev = algo == SGW_SSWP;
  if (tid == 0) s_k = kSelBins - 1u;  // target never reached: take everything
  // thread t owns 4 consecutive bins in selection order
  unsigned long long h[4], mine = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t k = 4u * tid + q;
    h[q] = hist[rev ? kSelBins - 1u - k : k];
    mine += h[q];
  }
  unsigned long long incl = mine;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_part[warp] = incl;
  __syncthreads();
  if (tid == 0) {
    unsigned long long acc = 0;
    for (int w = 0; w < (int)(kSelBins / 4 / 32); ++w) {
      const unsigned long long x = s_part[w];
      s_part[w] = acc;
      acc += x;
    }
  }
  __syncthreads();
  unsigned long long run = s_part[warp] + incl - mine;
  uint32_t first = 0xffffffffu;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    run += h[q];
    if (first == 0xffffffffu && h[q] && run >= target) first = 4u * tid + q;
  }
  if (first != 0xffffffffu) atomicMin(&s_k, first);
  __syncthreads();
  if (tid == 0) ctl->sel_bin = rev ? kSelBins - 1u - s_k : s_k;
}

// ---- partition planner ------------------------------------------------------
// One warp.  For each partition: the largest run of queue entries starting at
// `from` whose edges fit `cap`, found by a 32-way search (each step probes 32
// evenly spaced entries and keeps the bracket of the last one that fits).
__global__ void k_plan(const uint32_t *ptr, const uint32_t *queue, Ctl *ctl,
                       Part *parts, uint32_t max_parts, unsigned long long cap) {
  const int lane = threadIdx.x & 31;
  const uint32_t count = ctl->num_active;
  uint32_t from = 0, p = 0;
  while (from < count) {
    const unsigned long long limit = (unsigned long long)ptr[from] + cap;
    // answer t in [from, count]: largest index with ptr[t] <= limit
    uint32_t lo = from + 1, hi = count;  // candidates above `from`
    uint32_t best = from;
    while (lo <= hi) {
      const uint32_t span = hi - lo + 1;
      const uint32_t step = (span + 31) / 32;
      const uint32_t idx = lo + (uint32_t)lane * step;
      const bool ok = idx <= hi && (unsigned long long)ptr[idx] <= limit;
      const uint32_t bal = __ballot_sync(0xffffffffu, ok);
      const int k = __popc(bal);  // ok is a prefix of the lanes
      if (k == 0) break;
      const uint32_t last_ok = lo + (uint32_t)(k - 1) * step;
      best = last_ok;
      if (step == 1) break;
      lo = last_ok + 1;
      const uint32_t next_bad = lo - 1 + step;  // first probe that failed
      if (k < 32 && next_bad - 1 < hi) hi = next_bad - 1;
    }
    uint32_t to = best > from ? best : from + 1;  // a vertex beyond cap runs alone
    if (lane == 0 && p < max_parts) {
      Part q;
      q.from = from;
      q.size = to - from;
      q.edge_from = ptr[from];
      q.first_vertex = queue[from];
      q.edge_count = (unsigned long long)ptr[to] - ptr[from];
      parts[p] = q;
    }
    ++p;
    from = to;
  }
  if (lane == 0) {
    ctl->num_parts = p;
    if (p > max_parts) atomicExch(&ctl->error, 2u);
  }
}

// ---- gather: host CSR -> device edge buffer -------------------------------
// The engine's host transfer copy is a series of pinned chunks of 2^shift
// bytes (allocated by two host threads at once, which halves the set-up of
// a 21 GB copy); base is a device table of their device addresses.  A
// 16-byte word or a record never straddles two chunks.
struct HostChunks {
  const unsigned long long *base;
  uint32_t shift;
};

__device__ __forceinline__ const char *hc_at(const HostChunks &h, size_t byte) {
  const char *c = reinterpret_cast<const char *>(__ldg(h.base + (byte >> h.shift)));
  return c + (byte & ((size_t(1) << h.shift) - 1));
}

// Copies bytes [off, off + bytes) of a host stream to dst, for streams in
// pageable memory (read through the host page tables), where a DMA copy would
// be staged by the host thread.  Each thread reads one aligned 16-byte word of
// the stream (words never straddle chunks) and stores the part in range as
// one 16-byte word, four 4-byte words or single bytes, whichever the two
// addresses' alignment allows.  Chunks are padded to 16 bytes, so the words at
// either end stay inside their chunk.
__global__ void __launch_bounds__(256) k_copy_host(HostChunks src, unsigned long long off,
                                                   unsigned long long bytes, uint8_t *__restrict__ dst) {
  const unsigned long long w0 = off >> 4, w1 = (off + bytes + 15) >> 4, end = off + bytes;
  const unsigned long long skew = (reinterpret_cast<uintptr_t>(dst) - off) & 15;
  for (unsigned long long w = w0 + blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; w < w1;
       w += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long s = w << 4;
    const uint4 v = *reinterpret_cast<const uint4 *>(hc_at(src, s));
    if (skew == 0 && s >= off && s + 16 <= end) {
      *reinterpret_cast<uint4 *>(dst + (s - off)) = v;
      continue;
    }
    const uint32_t q[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const unsigned long long a = s + 4 * k;
      if ((skew & 3) == 0 && a >= off && a + 4 <= end) {
        *reinterpret_cast<uint32_t *>(dst + (a - off)) = q[k];
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (a + i >= off && a + i < end) dst[a + i - off] = (uint8_t)(q[k] >> (8 * i));
      }
    }
  }
}

constexpr int kGatherThreads = 256;
// Output edges per CTA tile of the vectorised gather (its shared memory is
// dynamic: 16 bytes per tile edge plus the weight bytes); the scalar gather
// keeps 2048.
#ifndef SGW_GATHER_TILE
#define SGW_GATHER_TILE 2048
#endif
constexpr uint32_t kGatherTile = SGW_GATHER_TILE;
constexpr uint32_t kScalarGatherTile = 2048;

// Index of the last element <= x in a[0..len) (a non-decreasing, a[0] <= x).
__device__ __forceinline__ uint32_t last_le(const uint32_t *a, uint32_t len, uint32_t x) {
  uint32_t lo = 0, hi = len;  // first index with a[i] > x in [lo, hi)
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1; else hi = mid;
  }
  return lo - 1;
}

// Last queue index i in [lo, hi) with ptr[i] - edge_from <= target, found by
// one warp in 32-way steps (about five dependent loads for 2^24 entries
// instead of one per halving).  ptr is non-decreasing and
// ptr[lo] - edge_from <= target.  Every lane returns the answer.
__device__ __forceinline__ uint32_t warp_last_le(const uint32_t *__restrict__ ptr, uint32_t lo, uint32_t hi,
                                                 uint32_t edge_from, uint32_t target, int lane) {
  while (hi - lo > 32u) {
    const uint32_t step = (hi - lo + 31u) / 32u;
    const uint32_t idx = lo + (uint32_t)lane * step;
    const bool le = idx < hi && ptr[idx] - edge_from <= target;
    const uint32_t m = __ballot_sync(0xffffffffu, le);  // a prefix of lanes; lane 0 always
    const uint32_t k = 31u - (uint32_t)__clz((int)m);
    lo += k * step;
    hi = min(hi, lo + step);
  }
  const uint32_t idx = lo + (uint32_t)lane;
  const bool le = idx < hi && ptr[idx] - edge_from <= target;
  const uint32_t m = __ballot_sync(0xffffffffu, le);
  return lo + 31u - (uint32_t)__clz((int)m);
}

// Copies the edges of queue entries [from, from+size) from the mapped host
// CSR to buf[0 .. edge_count).  Output positions are balanced per CTA; each
// CTA stages the (buffer offset, host offset) of the sources its tile covers
// in shared memory and every thread copies edges by binary search in it.
// Consecutive threads read consecutive host edges of one source, so host
// reads are coalesced; E is the edge record (one or two u32 words).
template <int W, bool WIDE>
__global__ void __launch_bounds__(kGatherThreads) k_gather(
    const uint32_t *__restrict__ queue, const uint32_t *__restrict__ ptr,
    const uint32_t *__restrict__ off, const unsigned long long *__restrict__ obase, HostChunks host_edges,
    uint32_t *__restrict__ buf, uint32_t from, uint32_t size, uint32_t edge_from,
    uint32_t edge_count) {
  using HP = typename std::conditional<WIDE, unsigned long long, uint32_t>::type;
  __shared__ uint32_t s_bpos[kScalarGatherTile + 1];
  __shared__ HP s_hpos[kScalarGatherTile + 1];
  __shared__ uint32_t s_first, s_last;
  const uint32_t ntiles = (edge_count + kScalarGatherTile - 1) / kScalarGatherTile;
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint32_t j0 = t * kScalarGatherTile;
    const uint32_t j1 = min(edge_count, j0 + kScalarGatherTile);
    // sources covering [j0, j1): warp 0 finds the first, warp 1 the last
    if (threadIdx.x < 64) {
      const int lane = threadIdx.x & 31;
      const uint32_t r = warp_last_le(ptr, from, from + size, edge_from, threadIdx.x < 32 ? j0 : j1 - 1, lane);
      if (lane == 0) (threadIdx.x < 32 ? s_first : s_last) = r;
    }
    __syncthreads();
    const uint32_t first = s_first, nsrc = s_last - s_first + 1;
    for (uint32_t k = threadIdx.x; k < nsrc; k += blockDim.x) {
      const uint32_t i = first + k;
      s_bpos[k] = ptr[i] - edge_from;
      s_hpos[k] = WIDE ? (HP)off_at(off, obase, queue[i]) : (HP)off[queue[i]];
    }
    __syncthreads();
    // four independent host loads in flight per thread before any store
    constexpr int U = 4;
    for (uint32_t jb = j0 + threadIdx.x; jb < j1; jb += U * blockDim.x) {
      uint2 e[U];
      uint32_t jj[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t j = jb + u * blockDim.x;
        jj[u] = j;
        if (j < j1) {
          const uint32_t k = last_le(s_bpos, nsrc, j);
          const size_t h = (size_t)s_hpos[k] + (j - s_bpos[k]);
          if (W == 1) e[u].x = *reinterpret_cast<const uint32_t *>(hc_at(host_edges, h * 4));
          else e[u] = *reinterpret_cast<const uint2 *>(hc_at(host_edges, h * 8));
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (jj[u] < j1) {
          if (W == 1) buf[jj[u]] = e[u].x;
          else reinterpret_cast<uint2 *>(buf)[jj[u]] = e[u];
        }
      }
    }
    __syncthreads();
  }
}

// Same tiling as k_gather, but host memory is read as aligned 16-byte words:
// each source's clipped host range is covered by ceil-aligned chunks of
// R = 16 / RB records of RB bytes, the CTA scans the chunk counts of its
// tile's sources, and every thread loads whole chunks (4 in flight) and
// scatters the records that belong to the source into the device buffer.
// RB = 4 (one word per edge) or 8 (the reference's {end, w8}).  With WS the
// split form's weight bytes of the same edges follow in the same tile (same
// source ranges, chunks of 16 weights), put together in shared memory and
// stored as 16-byte words.  Needs 16-byte aligned host arrays (the engine's
// own allocations are 64 KiB aligned).
constexpr uint32_t kGatherPer = (kGatherTile + kGatherThreads - 1) / kGatherThreads;

// Exclusive scan of the tile's per-source chunk counts (R records per
// chunk) into s_cs; returns the tile's chunk total.
template <uint32_t R>
__device__ __forceinline__ uint32_t gather_scan(uint32_t nsrc, const uint32_t *s_hlo, const uint32_t *s_len,
                                                uint32_t *s_cs, uint32_t *s_part) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  auto chunks = [&](uint32_t k) {  // depends on the source's record mod R only
    return (s_hlo[k] % R + s_len[k] + R - 1) / R;
  };
  uint32_t part = 0;
  for (uint32_t q = 0; q < kGatherPer; ++q) {
    const uint32_t k = tid * kGatherPer + q;
    if (k < nsrc) part += chunks(k);
  }
  const uint32_t incl = warp_incl_scan(part, lane);
  if (lane == 31) s_part[warp] = incl;
  __syncthreads();
  if (tid == 0) {
    uint32_t acc = 0;
    for (int w = 0; w < kGatherThreads / 32; ++w) { uint32_t x = s_part[w]; s_part[w] = acc; acc += x; }
    s_part[kGatherThreads] = acc;
  }
  __syncthreads();
  uint32_t run = s_part[warp] + incl - part;
  for (uint32_t q = 0; q < kGatherPer; ++q) {
    const uint32_t k = tid * kGatherPer + q;
    if (k < nsrc) { s_cs[k] = run; run += chunks(k); }
  }
  __syncthreads();
  return s_part[kGatherThreads];
}

// Copies the tile's chunks of RB-byte records: RB 4 / 8 straight into buf,
// RB 1 into the shared byte tile at position - j0.  A source's first record
// is (s_hhi:s_hlo), s_hhi only with WIDE; a chunk's records are matched to
// the source by their distance from it, which fits 32 bits.
template <int RB, bool WIDE>
__device__ __forceinline__ void gather_copy(uint32_t total, uint32_t nsrc, uint32_t j0, const uint32_t *s_cs,
                                            const uint32_t *s_hlo, const uint32_t *s_hhi, const uint32_t *s_len,
                                            const uint32_t *s_bpos, const HostChunks &host16,
                                            void *__restrict__ buf, uint8_t *s_bytes) {
  using CT = typename std::conditional<WIDE, unsigned long long, uint32_t>::type;
  constexpr uint32_t R = 16 / RB;
  constexpr int U = 4;
  for (uint32_t jb = threadIdx.x; jb < total; jb += U * blockDim.x) {
    uint4 v[U];
    uint32_t kk[U];
    CT cc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t j = jb + u * blockDim.x;
      kk[u] = 0xffffffffu;
      if (j < total) {
        const uint32_t k = last_le(s_cs, nsrc, j);
        CT h = s_hlo[k];
        if (WIDE) h |= (CT)s_hhi[k] << (WIDE ? 32 : 0);
        const CT c = h / R + (j - s_cs[k]);
        kk[u] = k;
        cc[u] = c;
        v[u] = *reinterpret_cast<const uint4 *>(hc_at(host16, (size_t)c << 4));
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (kk[u] == 0xffffffffu) continue;
      const uint32_t k = kk[u];
      const uint32_t len = s_len[k], bpos = s_bpos[k];
      // distance of the chunk's first record from the source's first (mod 2^32)
      const uint32_t d0 = (uint32_t)cc[u] * R - s_hlo[k];
      const uint32_t w[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
      for (uint32_t r = 0; r < R; ++r) {
        const uint32_t d = d0 + r;
        if (d < len) {
          const uint32_t o = bpos + d;
          if (RB == 4) reinterpret_cast<uint32_t *>(buf)[o] = w[r];
          else if (RB == 8) reinterpret_cast<uint2 *>(buf)[o] = make_uint2(w[2 * r], w[2 * r + 1]);
          else s_bytes[o - j0] = (uint8_t)(w[r / 4] >> (8 * (r % 4)));
        }
      }
    }
  }
}

// Dynamic shared memory of k_gather_v: four u32 arrays of kGatherTile + 1
// entries, the scan partials, then (16-byte aligned) the tile's weight bytes;
// the WIDE form adds the high words of the sources' host positions.
constexpr size_t kGatherBytesOff = ((4 * (kGatherTile + 1) + kGatherThreads + 1) * 4 + 15) / 16 * 16;
constexpr size_t kGatherSmemBytes = kGatherBytesOff + kGatherTile;
constexpr size_t kGatherSmemBytesWide = kGatherSmemBytes + ((kGatherTile + 1) * 4 + 15) / 16 * 16;

template <int RB, bool WS, bool WIDE>
__global__ void __launch_bounds__(kGatherThreads) k_gather_v(
    const uint32_t *__restrict__ queue, const uint32_t *__restrict__ ptr,
    const uint32_t *__restrict__ off, const unsigned long long *__restrict__ obase, HostChunks host16,
    void *__restrict__ buf, HostChunks host_w16, uint8_t *__restrict__ wbuf,
    uint32_t from, uint32_t size, uint32_t edge_from, uint32_t edge_count) {
  extern __shared__ __align__(16) unsigned char g_gather_smem[];
  uint32_t *const s_bpos = reinterpret_cast<uint32_t *>(g_gather_smem);
  uint32_t *const s_hlo = s_bpos + (kGatherTile + 1);
  uint32_t *const s_len = s_hlo + (kGatherTile + 1);
  uint32_t *const s_cs = s_len + (kGatherTile + 1);
  uint32_t *const s_part = s_cs + (kGatherTile + 1);
  uint8_t *const s_bytes = g_gather_smem + kGatherBytesOff;
  uint32_t *const s_hhi = WIDE ? reinterpret_cast<uint32_t *>(g_gather_smem + kGatherSmemBytes) : nullptr;
  __shared__ uint32_t s_first, s_last;
  const uint32_t ntiles = (edge_count + kGatherTile - 1) / kGatherTile;
  const int tid = threadIdx.x;
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint32_t j0 = t * kGatherTile;
    const uint32_t j1 = min(edge_count, j0 + kGatherTile);
    // sources covering [j0, j1): warp 0 finds the first, warp 1 the last
    if (tid < 64) {
      const int lane = tid & 31;
      const uint32_t r = warp_last_le(ptr, from, from + size, edge_from, tid < 32 ? j0 : j1 - 1, lane);
      if (lane == 0) (tid < 32 ? s_first : s_last) = r;
    }
    __syncthreads();
    const uint32_t first = s_first, nsrc = s_last - s_first + 1;
    // per-source clipped ranges (buffer position, host record, length)
#pragma unroll
    for (uint32_t q = 0; q < kGatherPer; ++q) {
      const uint32_t k = tid * kGatherPer + q;
      if (k < nsrc) {
        const uint32_t i = first + k;
        const uint32_t bp = ptr[i] - edge_from, be = ptr[i + 1] - edge_from;
        const uint32_t lo = max(bp, j0), hi = min(be, j1);
        s_bpos[k] = lo;
        if (WIDE) {
          const unsigned long long h = off_at(off, obase, queue[i]) + (lo - bp);
          s_hlo[k] = (uint32_t)h;
          s_hhi[k] = (uint32_t)(h >> 32);
        } else {
          s_hlo[k] = off[queue[i]] + (lo - bp);
        }
        s_len[k] = hi - lo;
      }
    }
    __syncthreads();
    uint32_t total = gather_scan<16 / RB>(nsrc, s_hlo, s_len, s_cs, s_part);
    gather_copy<RB, WIDE>(total, nsrc, j0, s_cs, s_hlo, s_hhi, s_len, s_bpos, host16, buf, s_bytes);
    if (WS) {
      __syncthreads();  // s_cs is reused
      total = gather_scan<16>(nsrc, s_hlo, s_len, s_cs, s_part);
      gather_copy<1, WIDE>(total, nsrc, j0, s_cs, s_hlo, s_hhi, s_len, s_bpos, host_w16, nullptr, s_bytes);
      __syncthreads();
      uint8_t *dst = wbuf + j0;
      const uint32_t len = j1 - j0;
      if (((uintptr_t)dst & 15u) == 0) {  // j0 is a multiple of the tile; wbuf is 16-byte aligned
        for (uint32_t i = tid; i < len / 16u; i += blockDim.x)
          reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(s_bytes)[i];
        for (uint32_t i = (len & ~15u) + tid; i < len; i += blockDim.x) dst[i] = s_bytes[i];
      } else {
        for (uint32_t i = tid; i < len; i += blockDim.x) dst[i] = s_bytes[i];
      }
    }
    __syncthreads();
  }
}

// ---- relaxation ----------------------------------------------------------------
// Per-algorithm semiring (shared/gpu_kernels.cu): candidate value from the
// source value and the edge, and whether it improves the destination.
template <int ALGO> struct Op;
template <> struct Op<SGW_BFS> {   // bfs_kernel: value+1, atomicMin (:45-46)
  static constexpr bool kMax = false;
  __device__ static uint32_t cand(uint32_t v, uint32_t) { return v + 1; }
};
template <> struct Op<SGW_SSSP> {  // sssp_kernel: value+w8, atomicMin (:146-149)
  static constexpr bool kMax = false;
  __device__ static uint32_t cand(uint32_t v, uint32_t w) { return v + w; }
};
template <> struct Op<SGW_SSWP> {  // sswp_kernel: min(value,w8), atomicMax (:196-199)
  static constexpr bool kMax = true;
  __device__ static uint32_t cand(uint32_t v, uint32_t w) { return min(v, w); }
};
template <> struct Op<SGW_CC> {    // cc_kernel: value, atomicMin (:96-98)
  static constexpr bool kMax = false;
  __device__ static uint32_t cand(uint32_t v, uint32_t) { return v; }
};

// Relaxes one edge given the destination's value as read beforehand: when
// the candidate beats it, a non-returning atomicMin/atomicMax (a reduction,
// no round trip for the thread) lowers the value and the destination's label
// is set.  The label is right even when another thread's candidate won: the
// read value is at most as good as the value when this kernel started (values
// move one way), so the candidate beat that value and the destination did
// improve in this kernel, by this thread or by the winner.  Returns whether
// the candidate beat the read value.
template <int ALGO>
__device__ __forceinline__ bool relax_edge_seen(uint32_t sval, uint32_t dst, uint32_t w, uint32_t cur,
                                                uint32_t *value, uint8_t *nxt) {
  const uint32_t c = Op<ALGO>::cand(sval, w);
  if (Op<ALGO>::kMax ? (c > cur) : (c < cur)) {
    if (Op<ALGO>::kMax) atomicMax(&value[dst], c);
    else atomicMin(&value[dst], c);
    nxt[dst] = 1;
    return true;
  }
  return false;
}

template <int ALGO>
__device__ __forceinline__ bool relax_edge(uint32_t sval, uint32_t dst, uint32_t w,
                                           uint32_t *value, uint8_t *nxt) {
  return relax_edge_seen<ALGO>(sval, dst, w, value[dst], value, nxt);
}

// Edges each thread keeps in flight in the expansion loops: the record and
// destination-value loads of kRelaxUnroll edges are issued before any of
// their compares and atomics, so a warp waits on one memory round trip per
// kRelaxUnroll edges instead of per edge.
constexpr int kRelaxUnroll = 4;

// Whether a source with this value may push (guards u32 overflow of INF+w;
// the reference relies on INF vertices never carrying a label).
template <int ALGO>
__device__ __forceinline__ bool can_push(uint32_t v) {
  if (ALGO == SGW_BFS || ALGO == SGW_SSSP) return v != kInf;
  if (ALGO == SGW_SSWP) return v != 0;
  return true;
}

// Reads edge record e of a device edge buffer: W = 2 words {end, w8};
// W = 1 either {end} (pbits = 0; its weight, if any, in the byte stream wbuf
// of the split form) or the packed transfer form (w8 << pbits) | end.
template <int W>
__device__ __forceinline__ void load_edge(const uint32_t *buf, uint32_t e, uint32_t pbits,
                                          uint32_t &dst, uint32_t &w, const uint8_t *wbuf = nullptr) {
  if (W == 1) {
    const uint32_t r = buf[e];
    if (pbits) { dst = r & ((1u << pbits) - 1u); w = r >> pbits; }
    else { dst = r; w = wbuf ? (uint32_t)wbuf[e] : 0u; }
  } else {
    const uint2 ed = reinterpret_cast<const uint2 *>(buf)[e];
    dst = ed.x;
    w = ed.y;
  }
}

struct RelaxArgs {
  const uint32_t *queue;
  const uint32_t *ptr;
  const uint32_t *buf;       // device edge buffer (W words per edge)
  uint32_t *value;
  uint8_t *cur;              // async: label of this inner iteration (cleared)
  uint8_t *nxt;              // label set on improvement
  Ctl *ctl;
  WorkItem *wl;
  uint32_t wl_cap;
  uint32_t from, size, edge_from;
  uint32_t iter;             // inner iteration number (1-based)
  uint32_t tile_degree_max;  // sources above this go to the chunk list
  uint32_t chunk_edges;
  uint32_t pbits;            // packed records: bits of the destination
  // streamed partition: the buffer holds a whole vertex range starting at
  // edge stream_base, so a source's edges sit at off[u] - stream_base
  uint32_t streamed;
  uint32_t stream_base;
  const uint32_t *off;
  const uint8_t *wbuf;       // split form: the buffer's weight bytes (else null)
};

constexpr int kRelaxThreads = 256;

// Tile of kRelaxThreads partition sources per CTA (grid-stride).  Each thread
// claims one source (async: only if its label is set, clearing it), the CTA
// scans the degrees in shared memory and all threads expand the tile's edges
// together: edge j of the tile belongs to the source found by binary search
// in the scanned degrees.  Sources above tile_degree_max are cut into chunks
// and appended to the chunk list instead.
struct TileSmem {
  uint32_t scan[kRelaxThreads + 1];
  uint32_t boff[kRelaxThreads];
  uint32_t val[kRelaxThreads];
  uint32_t hub[kRelaxThreads];
  uint32_t wsum[kRelaxThreads / 32];
  uint32_t nhub, wbase;
  int skip;
};

template <int ALGO, bool ASYNC, int W>
__device__ __forceinline__ void relax_tile_phase(const RelaxArgs &a, TileSmem &sm) {
  uint32_t *const s_scan = sm.scan;
  uint32_t *const s_boff = sm.boff;
  uint32_t *const s_val = sm.val;
  uint32_t *const s_hub = sm.hub;
  uint32_t &s_nhub = sm.nhub;
  uint32_t &s_wbase = sm.wbase;
  int &s_skip = sm.skip;
  const int tid = threadIdx.x;
  const uint32_t slot = a.iter & 3u;
  if (tid == 0) {
    int skip = 0;
    if (ASYNC && a.iter > 1 && ld_acquire_u32(&a.ctl->upd[(a.iter - 1) & 3u]) == 0) skip = 1;
    s_skip = skip;
    if (blockIdx.x == 0) {
      a.ctl->upd[(a.iter + 1) & 3u] = 0;
      a.ctl->wl_count[(a.iter + 1) & 3u] = 0;
      if (!skip) {
        atomicAdd(&a.ctl->iters_run, 1u);
        atomicAdd(&a.ctl->iters_total, 1u);
      }
    }
  }
  __syncthreads();
  if (s_skip) return;
  bool any_update = false;
  const uint32_t ntiles = (a.size + kRelaxThreads - 1) / kRelaxThreads;
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    if (tid == 0) s_nhub = 0;
    __syncthreads();
    const uint32_t idx = t * kRelaxThreads + tid;
    uint32_t d = 0, boff = 0, val = 0, u = 0;
    if (idx < a.size) {
      const uint32_t i = a.from + idx;
      u = a.queue[i];
      bool act = true;
      if (ASYNC) {
        act = a.cur[u] != 0;
        if (act) a.cur[u] = 0;
      }
      if (act) {
        val = a.value[u];
        if (can_push<ALGO>(val)) {
          const uint32_t p0 = a.ptr[i];
          d = a.ptr[i + 1] - p0;
          boff = a.streamed ? a.off[u] - a.stream_base : p0 - a.edge_from;
          if (d > a.tile_degree_max) {
            s_hub[atomicAdd(&s_nhub, 1u)] = tid;
            atomicAdd(&a.ctl->relaxed_edges, (unsigned long long)d);
          }
        }
      }
    }
    s_boff[tid] = boff;
    s_val[tid] = val;
    {
      const int nsrc = __syncthreads_count(d > 0);
      if (tid == 0 && nsrc) atomicAdd(&a.ctl->relaxed_sources, (unsigned long long)nsrc);
    }
    // chunk out high-degree sources (whole CTA writes the items)
    const uint32_t nhub = s_nhub;
    for (uint32_t h = 0; h < nhub; ++h) {
      const uint32_t ht = s_hub[h];
      if (tid == ht) {
        const uint32_t nch = (d + a.chunk_edges - 1) / a.chunk_edges;
        s_wbase = atomicAdd(&a.ctl->wl_count[slot], nch);
        s_scan[kRelaxThreads] = d;  // temporary: degree of this hub
      }
      __syncthreads();
      const uint32_t hd = s_scan[kRelaxThreads];
      const uint32_t nch = (hd + a.chunk_edges - 1) / a.chunk_edges;
      const uint32_t wb = s_wbase;
      for (uint32_t c = tid; c < nch; c += blockDim.x) {
        if (wb + c < a.wl_cap) {
          WorkItem it;
          it.boff = s_boff[ht] + c * a.chunk_edges;
          it.count = min(a.chunk_edges, hd - c * a.chunk_edges);
          it.value = s_val[ht];
          it.vertex = 0;
          a.wl[wb + c] = it;
        } else {
          atomicExch(&a.ctl->error, 3u);
        }
      }
      __syncthreads();
    }
    if (d > a.tile_degree_max) d = 0;
    // block exclusive scan of d
    {
      const int lane = tid & 31, warp = tid >> 5;
      const uint32_t incl = warp_incl_scan(d, lane);
      uint32_t *const s_wsum = sm.wsum;
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      if (tid == 0) {
        uint32_t acc = 0;
        for (int w = 0; w < kRelaxThreads / 32; ++w) { uint32_t x = s_wsum[w]; s_wsum[w] = acc; acc += x; }
        s_scan[kRelaxThreads] = acc;
      }
      __syncthreads();
      s_scan[tid] = s_wsum[warp] + incl - d;
      __syncthreads();
    }
    const uint32_t total = s_scan[kRelaxThreads];
    if (tid == 0 && total) atomicAdd(&a.ctl->relaxed_edges, (unsigned long long)total);
    for (uint32_t j0 = tid; j0 < total; j0 += kRelaxUnroll * kRelaxThreads) {
      uint32_t dst[kRelaxUnroll], w[kRelaxUnroll], sv[kRelaxUnroll], cur[kRelaxUnroll];
      bool ok[kRelaxUnroll];
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q) {
        const uint32_t j = j0 + q * kRelaxThreads;
        ok[q] = j < total;
        if (ok[q]) {
          // last source k with s_scan[k] <= j (sources with d == 0 share
          // offsets; the last one with that offset is the one that owns edge j)
          uint32_t lo = 0, hi = kRelaxThreads;
          while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (s_scan[mid] <= j) lo = mid + 1; else hi = mid;
          }
          const uint32_t k = lo - 1;
          load_edge<W>(a.buf, s_boff[k] + (j - s_scan[k]), a.pbits, dst[q], w[q], a.wbuf);
          sv[q] = s_val[k];
        }
      }
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q)
        if (ok[q]) cur[q] = a.value[dst[q]];
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q)
        if (ok[q]) any_update |= relax_edge_seen<ALGO>(sv[q], dst[q], w[q], cur[q], a.value, a.nxt);
    }
    __syncthreads();
  }
  if (__syncthreads_or(any_update) && tid == 0) atomicAdd(&a.ctl->upd[slot], 1u);
}

template <int ALGO, bool ASYNC, int W>
__global__ void __launch_bounds__(kRelaxThreads) k_relax_tile(RelaxArgs a) {
  __shared__ TileSmem sm;
  relax_tile_phase<ALGO, ASYNC, W>(a, sm);
}

// Warp-tile form of k_relax_tile: each warp takes 32 partition sources at a
// time and expands their edges on its own (warp scan of the degrees, each
// edge's owner found with warp votes and shuffles, no shared memory), so
// warps never wait on each other: a warp that runs out of tiles adds its counters
// to the CTA's in shared memory and leaves, and the last warp of the CTA to
// leave publishes them.  Sources above tile_degree_max go to the chunk list
// as in the CTA form.
constexpr int kWarpsPerCta = kRelaxThreads / 32;
// Resident CTAs per SM the warp relaxation is compiled for (registers are
// capped to fit them); 4 keeps it free of spills.
#ifndef SGW_RELAX_MIN_BLOCKS
#define SGW_RELAX_MIN_BLOCKS 4
#endif
template <int ALGO, bool ASYNC, int W>
__global__ void __launch_bounds__(kRelaxThreads, SGW_RELAX_MIN_BLOCKS) k_relax_warp(RelaxArgs a) {
  __shared__ int s_skip;
  __shared__ unsigned long long s_edges, s_srcs;
  __shared__ uint32_t s_any, s_done;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint32_t slot = a.iter & 3u;
  if (tid == 0) {
    int skip = 0;
    if (ASYNC && a.iter > 1 && ld_acquire_u32(&a.ctl->upd[(a.iter - 1) & 3u]) == 0) skip = 1;
    s_skip = skip;
    s_edges = 0;
    s_srcs = 0;
    s_any = 0;
    s_done = 0;
    if (blockIdx.x == 0) {
      a.ctl->upd[(a.iter + 1) & 3u] = 0;
      a.ctl->wl_count[(a.iter + 1) & 3u] = 0;
      if (!skip) {
        atomicAdd(&a.ctl->iters_run, 1u);
        atomicAdd(&a.ctl->iters_total, 1u);
      }
    }
  }
  __syncthreads();
  if (s_skip) return;
  bool any_update = false;
  unsigned long long my_edges = 0, my_srcs = 0;
  const uint32_t ntiles = (a.size + 31u) / 32u;
  const uint32_t gw = blockIdx.x * kWarpsPerCta + wid, nw = gridDim.x * kWarpsPerCta;
  for (uint32_t t = gw; t < ntiles; t += nw) {
    const uint32_t idx = t * 32u + lane;
    uint32_t d = 0, boff = 0, val = 0;
    if (idx < a.size) {
      const uint32_t i = a.from + idx;
      const uint32_t u = a.queue[i];
      bool act = true;
      if (ASYNC) {
        act = a.cur[u] != 0;
        if (act) a.cur[u] = 0;
      }
      if (act) {
        val = a.value[u];
        if (can_push<ALGO>(val)) {
          const uint32_t p0 = a.ptr[i];
          d = a.ptr[i + 1] - p0;
          boff = a.streamed ? a.off[u] - a.stream_base : p0 - a.edge_from;
        }
      }
    }
    my_srcs += __popc(__ballot_sync(0xffffffffu, d > 0));
    // high-degree sources: the warp writes their chunk items together
    unsigned hubs = __ballot_sync(0xffffffffu, d > a.tile_degree_max);
    while (hubs) {
      const int h = __ffs(hubs) - 1;
      hubs &= hubs - 1;
      const uint32_t hd = __shfl_sync(0xffffffffu, d, h);
      const uint32_t hb = __shfl_sync(0xffffffffu, boff, h);
      const uint32_t hv = __shfl_sync(0xffffffffu, val, h);
      const uint32_t nch = (hd + a.chunk_edges - 1) / a.chunk_edges;
      uint32_t wb = 0;
      if (lane == 0) wb = atomicAdd(&a.ctl->wl_count[slot], nch);
      wb = __shfl_sync(0xffffffffu, wb, 0);
      for (uint32_t c = lane; c < nch; c += 32) {
        if (wb + c < a.wl_cap) {
          WorkItem it;
          it.boff = hb + c * a.chunk_edges;
          it.count = min(a.chunk_edges, hd - c * a.chunk_edges);
          it.value = hv;
          it.vertex = 0;
          a.wl[wb + c] = it;
        } else {
          atomicExch(&a.ctl->error, 3u);
        }
      }
      my_edges += hd;
    }
    if (d > a.tile_degree_max) d = 0;
    const uint32_t incl = warp_incl_scan(d, lane);
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    const uint32_t excl = incl - d;
    const uint32_t owners = __ballot_sync(0xffffffffu, d > 0);  // lanes owning edges, in edge order
    my_edges += total;
    for (uint32_t w0 = 0; w0 < total; w0 += 32u * kRelaxUnroll) {
      uint32_t dst[kRelaxUnroll], w[kRelaxUnroll], sv[kRelaxUnroll], cur[kRelaxUnroll];
      bool ok[kRelaxUnroll];
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q) {
        // window of 32 edges [wb, wb + 32), lane i takes edge wb + i; its
        // owner is found with votes instead of a search: the owners whose
        // range starts at or before wb, plus those starting inside the
        // window up to edge wb + i, count the owner's rank among `owners`
        const uint32_t wb = w0 + 32u * q;
        const uint32_t j = wb + lane;
        ok[q] = j < total;
        const bool own = d > 0;
        const uint32_t starts =
            __reduce_or_sync(0xffffffffu, (own && excl > wb && excl < wb + 32u) ? (1u << (excl - wb)) : 0u);
        const uint32_t before = __popc(__ballot_sync(0xffffffffu, own && excl <= wb));
        const uint32_t rank = before + __popc(starts & ((2u << lane) - 1u)) - 1u;
        const int k = __fns(owners, 0, (int)rank + 1);
        const uint32_t kb = __shfl_sync(0xffffffffu, boff, k & 31);
        const uint32_t ke = __shfl_sync(0xffffffffu, excl, k & 31);
        const uint32_t kv = __shfl_sync(0xffffffffu, val, k & 31);
        if (ok[q]) {
          load_edge<W>(a.buf, kb + (j - ke), a.pbits, dst[q], w[q], a.wbuf);
          sv[q] = kv;
        }
      }
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q)
        if (ok[q]) cur[q] = a.value[dst[q]];
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q)
        if (ok[q]) any_update |= relax_edge_seen<ALGO>(sv[q], dst[q], w[q], cur[q], a.value, a.nxt);
    }
  }
  const bool warp_any = __any_sync(0xffffffffu, any_update);
  if (lane == 0) {
    if (my_edges) atomicAdd(&s_edges, my_edges);
    if (my_srcs) atomicAdd(&s_srcs, my_srcs);
    if (warp_any) atomicOr(&s_any, 1u);
    __threadfence_block();
    if (atomicAdd(&s_done, 1u) == kWarpsPerCta - 1) {  // the CTA's last warp publishes
      __threadfence_block();
      if (s_any) atomicAdd(&a.ctl->upd[slot], 1u);
      if (s_edges) atomicAdd(&a.ctl->relaxed_edges, s_edges);
      if (s_srcs) atomicAdd(&a.ctl->relaxed_sources, s_srcs);
    }
  }
}

// Chunk list of inner iteration `iter`: one warp per item.
template <int ALGO, bool ASYNC, int W>
__device__ __forceinline__ void relax_chunks_phase(const RelaxArgs &a) {
  const uint32_t slot = a.iter & 3u;
  if (ASYNC && a.iter > 1 && ld_acquire_u32(&a.ctl->upd[(a.iter - 1) & 3u]) == 0) return;
  const uint32_t items = min(ld_acquire_u32(&a.ctl->wl_count[slot]), a.wl_cap);
  const int lane = threadIdx.x & 31;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  bool any_update = false;
  for (uint32_t it = gw; it < items; it += nw) {
    const WorkItem wi = a.wl[it];
    for (uint32_t j0 = lane; j0 < wi.count; j0 += 32 * kRelaxUnroll) {
      uint32_t dst[kRelaxUnroll], w[kRelaxUnroll], cur[kRelaxUnroll];
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q)
        if (j0 + 32 * q < wi.count) load_edge<W>(a.buf, wi.boff + j0 + 32 * q, a.pbits, dst[q], w[q], a.wbuf);
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q)
        if (j0 + 32 * q < wi.count) cur[q] = a.value[dst[q]];
#pragma unroll
      for (int q = 0; q < kRelaxUnroll; ++q)
        if (j0 + 32 * q < wi.count)
          any_update |= relax_edge_seen<ALGO>(wi.value, dst[q], w[q], cur[q], a.value, a.nxt);
    }
  }
  if (__syncthreads_or(any_update) && threadIdx.x == 0) atomicAdd(&a.ctl->upd[slot], 1u);
}

template <int ALGO, bool ASYNC, int W>
__global__ void __launch_bounds__(kRelaxThreads) k_relax_chunks(RelaxArgs a) {
  relax_chunks_phase<ALGO, ASYNC, W>(a);
}

// Single-vertex partition (degree above the edge buffer): claim the source
// once, then relax its edges piece by piece.
template <bool ASYNC>
__global__ void k_hub_claim(uint32_t u, const uint32_t *value, uint8_t *l1, uint8_t *l2, Ctl *ctl) {
  uint32_t act = 1;
  if (ASYNC) {
    act = (l1[u] | l2[u]) != 0;
    l1[u] = 0;
    l2[u] = 0;
  }
  ctl->hub_active = act;
  ctl->hub_value = value[u];
  ctl->upd[1] = 0;
}

template <int ALGO, int W>
__global__ void k_relax_flat(const uint32_t *buf, const uint8_t *wbuf, uint32_t count, uint32_t pbits,
                             uint32_t *value, uint8_t *nxt, Ctl *ctl) {
  if (!ctl->hub_active) return;
  const uint32_t sval = ctl->hub_value;
  if (!can_push<ALGO>(sval)) return;
  bool any = false;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
    uint32_t dst, w;
    load_edge<W>(buf, j, pbits, dst, w, wbuf);
    any |= relax_edge<ALGO>(sval, dst, w, value, nxt);
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicAdd(&ctl->upd[1], 1u);
}

// ---- label hand-off (shared/gpu_kernels.cu:515-534) ------------------------
// mixLabels: label1 |= label2; label2 = 0 for the partition's sources.
__global__ void k_mix(const uint32_t *queue, uint32_t from, uint32_t size, uint8_t *l1, uint8_t *l2) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < size; i += gridDim.x * blockDim.x) {
    const uint32_t u = queue[from + i];
    if (l2[u]) { l1[u] = 1; l2[u] = 0; }
  }
}

// ---- state init and summaries ------------------------------------------------
// Initial values and labels of subway/<algo>-<mode>.cu.
__global__ void k_init(uint32_t n, int algo, int mode, uint32_t source, uint32_t *value,
                       uint8_t *l1, uint8_t *l2) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    uint32_t val;
    switch (algo) {
      case SGW_BFS:
      case SGW_SSSP: val = (v == source) ? 0u : kInf; break;
      case SGW_SSWP: val = (v == source) ? kInf : 0u; break;
      default: val = v; break;  // CC
    }
    value[v] = val;
    uint8_t a1, a2;
    if (mode == SGW_ASYNC) { a1 = 1; a2 = 0; }            // all active for the first generate
    else if (algo == SGW_CC) { a1 = 0; a2 = 1; }           // cc-sync.cu:31-33
    else { a1 = 0; a2 = (v == source) ? 1 : 0; }           // bfs-sync.cu:30-36
    l1[v] = a1;
    l2[v] = a2;
  }
}

// After the first async generate, label1 = {source} (subway/sssp-async.cu:59-63);
// cc-async keeps every vertex active.
__global__ void k_async_reset(uint32_t n, uint32_t source, uint8_t *l1) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    l1[v] = (v == source) ? 1 : 0;
}

// Graph500 m_reached: edges whose source left its initial value.
__global__ void k_reached(uint32_t n, int algo, uint32_t source, const uint32_t *value,
                          const uint32_t *off, Ctl *ctl) {
  unsigned long long acc = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const uint32_t x = value[v];
    bool reached;
    switch (algo) {
      case SGW_BFS:
      case SGW_SSSP: reached = x != kInf; break;
      case SGW_SSWP: reached = x != 0 || v == source; break;
      default: reached = true; break;
    }
    if (reached) acc += off[v + 1] - off[v];
  }
  acc = __reduce_add_sync(0xffffffffu, (uint32_t)acc) ; // per-warp (degree sums fit u32 per warp)
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&ctl->reached_edges, acc);
}

// ---- PageRank (pr_kernel / pr_async, shared/gpu_kernels.cu:211-254, :459-502) --
// Ranks and residuals are kept in double precision on the device; the
// reference's float results are the final cast.
struct PrItem {              // a chunk of one high-degree source's pushes
  uint32_t boff;
  uint32_t count;
  double push;
};

struct PrArgs {
  const uint32_t *queue;
  const uint32_t *ptr;
  const uint32_t *buf;       // device edge buffer (W words per edge)
  double *pval;
  double *delta;
  const double *qpush;       // pushes snapshotted by the generate step
  Ctl *ctl;
  PrItem *wl;
  uint32_t wl_cap;
  uint32_t from, size, edge_from;
  uint32_t iter;
  uint32_t tile_degree_max;
  uint32_t chunk_edges;
  uint32_t pbits;
  uint32_t streamed;
  uint32_t stream_base;
  const uint32_t *off;
  double acc;
  double damping;
};

__device__ __forceinline__ double ld_relaxed_f64(const double *p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}

// Same tiling as k_relax_tile.  Inner iteration 1 pushes the snapshot taken
// by the generate step (every queued source is active); async iterations > 1
// re-activate partition sources whose residual grew above acc
// (value += delta; delta -= delta, atomically against concurrent pushes).
template <bool ASYNC, int W>
__global__ void __launch_bounds__(kRelaxThreads) k_pr_tile(PrArgs a) {
  __shared__ uint32_t s_scan[kRelaxThreads + 1];
  __shared__ uint32_t s_boff[kRelaxThreads];
  __shared__ double s_push[kRelaxThreads];
  __shared__ uint32_t s_hub[kRelaxThreads];
  __shared__ uint32_t s_wsum[kRelaxThreads / 32];
  __shared__ uint32_t s_nhub, s_wbase;
  __shared__ int s_skip;
  const int tid = threadIdx.x;
  const uint32_t slot = a.iter & 3u;
  if (tid == 0) {
    int skip = 0;
    if (ASYNC && a.iter > 1 && ld_acquire_u32(&a.ctl->upd[(a.iter - 1) & 3u]) == 0) skip = 1;
    s_skip = skip;
    if (blockIdx.x == 0) {
      a.ctl->upd[(a.iter + 1) & 3u] = 0;
      a.ctl->wl_count[(a.iter + 1) & 3u] = 0;
      if (!skip) {
        atomicAdd(&a.ctl->iters_run, 1u);
        atomicAdd(&a.ctl->iters_total, 1u);
      }
    }
  }
  __syncthreads();
  if (s_skip) return;
  bool any_push = false;
  const uint32_t ntiles = (a.size + kRelaxThreads - 1) / kRelaxThreads;
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    if (tid == 0) s_nhub = 0;
    __syncthreads();
    const uint32_t i = a.from + t * kRelaxThreads + tid;
    uint32_t d = 0, boff = 0;
    double push = 0.0;
    if (i < a.from + a.size) {
      const uint32_t p0 = a.ptr[i];
      const uint32_t deg = a.ptr[i + 1] - p0;
      bool act;
      if (!ASYNC || a.iter == 1) {
        push = a.qpush[i];
        act = true;
      } else {
        const uint32_t u = a.queue[i];
        const double res = ld_relaxed_f64(&a.delta[u]);
        act = res > a.acc;
        if (act) {
          a.pval[u] += res;
          atomicAdd(&a.delta[u], -res);
          push = a.damping * res / (double)deg;
        }
      }
      if (act) {
        any_push = true;
        d = deg;
        boff = a.streamed ? a.off[a.queue[i]] - a.stream_base : p0 - a.edge_from;
        if (d > a.tile_degree_max) {
          s_hub[atomicAdd(&s_nhub, 1u)] = tid;
          atomicAdd(&a.ctl->relaxed_edges, (unsigned long long)d);
        }
      }
    }
    s_boff[tid] = boff;
    s_push[tid] = push;
    {
      const int nsrc = __syncthreads_count(d > 0);
      if (tid == 0 && nsrc) atomicAdd(&a.ctl->relaxed_sources, (unsigned long long)nsrc);
    }
    const uint32_t nhub = s_nhub;
    for (uint32_t h = 0; h < nhub; ++h) {
      const uint32_t ht = s_hub[h];
      if (tid == ht) {
        s_wbase = atomicAdd(&a.ctl->wl_count[slot], (d + a.chunk_edges - 1) / a.chunk_edges);
        s_scan[kRelaxThreads] = d;
      }
      __syncthreads();
      const uint32_t hd = s_scan[kRelaxThreads];
      const uint32_t nch = (hd + a.chunk_edges - 1) / a.chunk_edges;
      const uint32_t wb = s_wbase;
      for (uint32_t c = tid; c < nch; c += blockDim.x) {
        if (wb + c < a.wl_cap) {
          PrItem it;
          it.boff = s_boff[ht] + c * a.chunk_edges;
          it.count = min(a.chunk_edges, hd - c * a.chunk_edges);
          it.push = s_push[ht];
          a.wl[wb + c] = it;
        } else {
          atomicExch(&a.ctl->error, 3u);
        }
      }
      __syncthreads();
    }
    if (d > a.tile_degree_max) d = 0;
    {
      const int lane = tid & 31, warp = tid >> 5;
      const uint32_t incl = warp_incl_scan(d, lane);
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      if (tid == 0) {
        uint32_t acc = 0;
        for (int w = 0; w < kRelaxThreads / 32; ++w) { uint32_t x = s_wsum[w]; s_wsum[w] = acc; acc += x; }
        s_scan[kRelaxThreads] = acc;
      }
      __syncthreads();
      s_scan[tid] = s_wsum[warp] + incl - d;
      __syncthreads();
    }
    const uint32_t total = s_scan[kRelaxThreads];
    if (tid == 0 && total) atomicAdd(&a.ctl->relaxed_edges, (unsigned long long)total);
    for (uint32_t j = tid; j < total; j += blockDim.x) {
      uint32_t lo = 0, hi = kRelaxThreads;
      while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (s_scan[mid] <= j) lo = mid + 1; else hi = mid;
      }
      const uint32_t k = lo - 1;
      uint32_t dst, w;
      load_edge<W>(a.buf, s_boff[k] + (j - s_scan[k]), a.pbits, dst, w);
      atomicAdd(&a.delta[dst], s_push[k]);
    }
    __syncthreads();
  }
  if (__syncthreads_or(any_push) && tid == 0) atomicAdd(&a.ctl->upd[slot], 1u);
}

template <bool ASYNC, int W>
__global__ void __launch_bounds__(kRelaxThreads) k_pr_chunks(PrArgs a) {
  const uint32_t slot = a.iter & 3u;
  if (ASYNC && a.iter > 1 && ld_acquire_u32(&a.ctl->upd[(a.iter - 1) & 3u]) == 0) return;
  const uint32_t items = min(ld_acquire_u32(&a.ctl->wl_count[slot]), a.wl_cap);
  const int lane = threadIdx.x & 31;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t it = gw; it < items; it += nw) {
    const PrItem wi = a.wl[it];
    for (uint32_t j = lane; j < wi.count; j += 32) {
      uint32_t dst, w;
      load_edge<W>(a.buf, wi.boff + j, a.pbits, dst, w);
      atomicAdd(&a.delta[dst], wi.push);
    }
  }
}

// Single-vertex PR partition: the generate snapshot of its push.
__global__ void k_pr_hub_claim(uint32_t from, const double *qpush, Ctl *ctl) {
  ctl->hub_push = qpush[from];
}

template <int W>
__global__ void k_pr_flat(const uint32_t *buf, uint32_t count, uint32_t pbits, double *delta,
                          const Ctl *ctl) {
  const double push = ctl->hub_push;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
    uint32_t dst, w;
    load_edge<W>(buf, j, pbits, dst, w);
    atomicAdd(&delta[dst], push);
  }
}

// delta = init, value = 0 (subway/pr-sync.cu:36-40).
__global__ void k_pr_init(uint32_t n, double init, double *pval, double *delta) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    pval[v] = 0.0;
    delta[v] = init;
  }
}

// ---- learned scheduler: per-range statistics and prediction -------------------
struct RangeInfo {           // a static vertex range [v0, v1) with edges [e0, e1)
  uint32_t v0, v1;
  unsigned long long e0, e1;
};

struct RangeStat {           // one global iteration of one range
  uint32_t qa, qb;           // its segment of the active queue
  uint32_t edge_from;        // ptr[qa]
  uint32_t act_edges;        // ptr[qb] - ptr[qa]
  uint32_t prev_edges;       // act_edges of the previous global iteration
  uint32_t first_vertex;     // queue[qa]
  float pred;                // predicted active edge fraction next iteration
  float feat[kMlpIn];
  uint32_t pad;
};

// One warp per range: locate the range's queue segment, form the five
// features, evaluate the network (or, with no weights, predict that the
// current active edge fraction persists).
__global__ void k_range_stats(const RangeInfo *__restrict__ ranges, uint32_t num_ranges,
                              const uint32_t *__restrict__ queue, const uint32_t *__restrict__ ptr,
                              const Ctl *__restrict__ ctl, RangeStat *st,
                              const __nv_bfloat16 *__restrict__ w, uint32_t iter, uint32_t cap) {
  const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= num_ranges) return;
  const RangeInfo r = ranges[s];
  const uint32_t count = ctl->num_active;
  uint32_t qa = 0, qb = 0;
  if (lane == 0) {
    qa = lower_bound_u32(queue, count, r.v0);
    qb = qa + lower_bound_u32(queue + qa, count - qa, r.v1);
  }
  qa = __shfl_sync(0xffffffffu, qa, 0);
  qb = __shfl_sync(0xffffffffu, qb, 0);
  const uint32_t efrom = ptr[qa];
  const uint32_t act = ptr[qb] - efrom;
  const uint32_t prev = st[s].prev_edges;
  const float redges = (float)(r.e1 - r.e0);
  float x[kMlpIn];
  x[0] = (r.v1 > r.v0) ? (float)(qb - qa) / (float)(r.v1 - r.v0) : 0.0f;
  x[1] = redges > 0.0f ? (float)act / redges : 0.0f;
  x[2] = fminf(fmaxf(__log2f(((float)act + 1.0f) / ((float)prev + 1.0f)) / 16.0f, -1.0f), 1.0f);
  x[3] = fminf((float)iter, 64.0f) / 64.0f;
  x[4] = cap ? fminf(redges / (float)cap, 1.0f) : 0.0f;
  const float pred = w ? mlp_forward_warp(w, x, lane) : x[1];
  if (lane == 0) {
    RangeStat o;
    o.qa = qa;
    o.qb = qb;
    o.edge_from = efrom;
    o.act_edges = act;
    o.prev_edges = act;  // becomes "previous" for the next iteration
    o.first_vertex = qb > qa ? queue[qa] : r.v0;
    o.pred = pred;
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) o.feat[k] = x[k];
    o.pad = prev;        // the previous count, reported with this iteration
    st[s] = o;
  }
}

__global__ void k_pr_to_f32(uint32_t n, const double *pval, float *out) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    out[v] = (float)pval[v];
}

}  // namespace sgw

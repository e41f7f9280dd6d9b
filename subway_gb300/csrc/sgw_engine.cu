// Device half of libsubwaygb: the engine object, its budgeted device arena,
// the global-iteration / partition / inner-iteration loops and the C ABI.
//
// Reference control flow: subway/sssp-async.cu:53-127 (async) and
// subway/bfs-sync.cu:44-98 (sync); roles shared/subgraph.cu,
// shared/subgraph_generator.cu, shared/partitioner.cu.

#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <sys/mman.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <thread>
#include <vector>

#include "sgw_internal.h"
#include "sgw_kernels.cuh"

using namespace sgw;

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess)                                                        \
      return fail(SGW_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), \
                  __FILE__, __LINE__);                                            \
  } while (0)

#define TRY(call)                \
  do {                           \
    int _s = (call);             \
    if (_s != SGW_OK) return _s; \
  } while (0)

namespace {

enum KClass { K_GENERATE = 0, K_PLAN, K_GATHER, K_RELAX, K_STREAM, K_NCLASS };

struct ProfEvent {
  int cls;
  cudaEvent_t a, b;
};

constexpr int kMaxBuf = 8;  // edge buffers an engine can hold
constexpr int kMaxHostChunks = 64;  // pieces of one host transfer stream

// One stream of the host transfer copy (edge words, or the split form's
// weight bytes) in pinned, mapped chunks of 2^shift bytes; 16 zero bytes
// follow the data in the last chunk for the gather's vector reads.
struct HostStream {
  std::vector<char *> h;               // host addresses of the chunks
  std::vector<size_t> size;            // allocated bytes of each chunk
  std::vector<unsigned long long> d;   // device addresses of the chunks
  uint32_t shift = 30;
  size_t bytes = 0;                    // data bytes
  bool pageable = false;               // chunks are ordinary pages, read through the host page tables
  bool borrowed = false;               // the graph's own records (not allocated, not freed here)
  const unsigned long long *dtab = nullptr;  // the chunk table on the device
};

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

struct sgw_engine {
  const sgw_graph *g = nullptr;
  int device = 0;
  int num_sms = 0;
  sgw_engine_opts opts{};
  uint64_t budget = 0;
  uint32_t n = 0, W = 1;  // W: u32 words per edge record
  uint64_t m = 0;

  // device arena
  char *d_arena = nullptr;
  size_t arena_bytes = 0;
  uint32_t *d_off = nullptr;               // node pointers (their low 32 bits when wide)
  unsigned long long *d_obase = nullptr;   // wide: node pointer of every 1024th vertex
  bool wide = false;                       // u64 node pointers on the host
  uint32_t edge_limit = 0;                 // most edges one generate queues (0: no limit)
  uint32_t *d_value = nullptr;
  uint8_t *d_l1 = nullptr, *d_l2 = nullptr;
  uint32_t range_inner_cap = 0;  // learned policy: inner-iteration cap of the running range
  uint64_t hub_iters = 0;        // single-vertex partitions relaxed (counted on the host)
  uint32_t *d_queue = nullptr, *d_ptr = nullptr;
  uint32_t *d_tflag = nullptr;
  uint32_t *d_gmask = nullptr;             // generate: keep | clear bits per 16-vertex group
  unsigned long long *d_tagg = nullptr, *d_tincl = nullptr;
  Ctl *d_ctl = nullptr;
  Part *d_parts = nullptr;
  WorkItem *d_wl = nullptr;
  uint32_t *d_buf[kMaxBuf] = {};
  double *d_pval = nullptr, *d_delta = nullptr, *d_qpush = nullptr;  // PR family
  __nv_bfloat16 *d_mlp = nullptr;          // scheduler weights (learned policy)
  unsigned long long *d_sel_hist = nullptr; // frontier deferral histogram (learned policy)
  RangeInfo *d_ranges = nullptr;           // static vertex ranges of this family
  RangeStat *d_rstat = nullptr;            // per-range statistics, one iteration
  int fam = 0;
  uint64_t cap_fam[2] = {0, 0};  // edge-buffer capacity of each family in this arena
  uint64_t cap = 0;  // edges per buffer
  uint32_t nbuf = 2;
  uint32_t max_parts = 0, wl_cap = 0, num_tiles = 0;

  // host side
  Ctl *h_ctl = nullptr;
  Part *h_parts = nullptr;
  HostStream hs_ends;                      // transfer records (destination words)
  HostStream hs_w;                         // split form: weight bytes
  unsigned long long *d_hct = nullptr;     // device chunk tables: ends, then weights
  // Split form: weights below 256 that do not pack beside the vertex id
  // travel as a separate byte stream (5 bytes per edge instead of 8).
  double dma_gbs = -1.0;                   // measured DMA rate from the transfer copy (-1: not timed)
  uint64_t stream_bytes = 0;               // whole-range copies timed so far (profiling)
  double stream_ms = 0.0;
  bool split = false;
  bool use_w = false;                      // this run reads the weight stream
  uint8_t *d_wbuf[kMaxBuf] = {};           // weight bytes of each edge buffer
  uint32_t rec_bytes = 4;                  // device bytes per edge in a buffer
  size_t packed_bytes = 0;                 // bytes of the whole transfer copy

  bool vec_gather = false;                 // host records readable as aligned 16-B words
  bool in_place = false;                   // the gather reads the graph's own records (no transfer copy)
  uint32_t cur_streamed = 0;               // partition being relaxed: whole-range buffer
  uint64_t cur_stream_base = 0;            //   and the first edge of that range
  uint32_t pbits = 0;                      // packed: bits of the destination id
  cudaStream_t s_comp = nullptr, s_copy = nullptr;
  cudaEvent_t ev_ready[kMaxBuf] = {}, ev_free[kMaxBuf] = {};
  cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
  std::vector<ProfEvent> prof;
  size_t prof_used = 0;
  uint32_t epoch = 0;

  // run state
  sgw_run_params params{};
  bool initialized = false;
  uint32_t num_active = 0;
  uint64_t num_active_edges = 0;
  uint32_t num_parts = 0;
  bool parts_valid = false;
  uint32_t gitr = 0;  // current global iteration (1-based once processing)
  sgw_run_stats stats{};
  bool trace_on = false;
  std::vector<sgw_trace_rec> trace;

  // learned policy
  int policy = SGW_POLICY_PLAIN;
  bool have_model = false;                 // d_mlp holds trained weights
  std::vector<RangeInfo> ranges;           // host copy of the static ranges
  RangeStat *h_rstat = nullptr;            // pinned, max_parts entries
  int buf_range[kMaxBuf];                  // range a buffer holds whole, or -1
  std::vector<sgw_range_rec> rtrace;
};

namespace {

// ---- timing helpers -----------------------------------------------------------
int prof_begin(sgw_engine *e, int cls, cudaStream_t s, size_t *slot) {
  if (!(e->opts.flags & SGW_OPT_PROFILE)) return SGW_OK;
  if (e->prof_used == e->prof.size()) {
    ProfEvent pe;
    pe.cls = cls;
    CK(cudaEventCreate(&pe.a));
    CK(cudaEventCreate(&pe.b));
    e->prof.push_back(pe);
  }
  *slot = e->prof_used++;
  e->prof[*slot].cls = cls;
  CK(cudaEventRecord(e->prof[*slot].a, s));
  return SGW_OK;
}

int prof_end(sgw_engine *e, cudaStream_t s, size_t slot) {
  if (!(e->opts.flags & SGW_OPT_PROFILE)) return SGW_OK;
  CK(cudaEventRecord(e->prof[slot].b, s));
  return SGW_OK;
}

// Whole-range DMA rate below which the learned policy stops streaming.
constexpr double kMinStreamGBs = 120.0;

int prof_collect(sgw_engine *e) {
  double ms[K_NCLASS] = {0, 0, 0, 0, 0};
  for (size_t i = 0; i < e->prof_used; ++i) {
    float t = 0;
    CK(cudaEventElapsedTime(&t, e->prof[i].a, e->prof[i].b));
    ms[e->prof[i].cls] += t;
  }
  e->prof_used = 0;
  e->stats.ms_generate += ms[K_GENERATE];
  e->stats.ms_partition += ms[K_PLAN];
  e->stats.ms_gather += ms[K_GATHER];
  e->stats.ms_stream += ms[K_STREAM];
  e->stats.ms_relax += ms[K_RELAX];
  // the whole-range copies' own rate: if it falls below what the policy
  // assumes, later runs send compacted edges only
  e->stream_ms += ms[K_STREAM];
  if (e->stream_bytes >= (uint64_t(256) << 20) && e->stream_ms > 0) {
    const double rate = (double)e->stream_bytes / (e->stream_ms * 1e6);
    if (rate < kMinStreamGBs) e->dma_gbs = rate;
  }
  return SGW_OK;
}

int check_ctl_error(sgw_engine *e) {
  uint32_t err = e->h_ctl->error;
  if (err == 0) return SGW_OK;
  if (err == 1) return fail(SGW_ETIMEOUT, "scan look-back wait timed out");
  if (err == 2) return fail(SGW_ERANGE, "partition table overflow");
  if (err == 3) return fail(SGW_ERANGE, "chunk list overflow");
  if (err == 4) return fail(SGW_ESTATE, "scan ticket counter out of step");
  return fail(SGW_ECUDA, "device error code %u", err);
}

// Copy of bytes [off, off + bytes) of a host stream: one DMA cudaMemcpyAsync
// per chunk it touches, or for pageable chunks one k_copy_host launch (a DMA
// copy from pageable memory is staged through the calling thread, which would
// stall the pipeline).
int copy_from_host(const HostStream &hs, void *dst, size_t off, size_t bytes, cudaStream_t st) {
  if (hs.pageable) {
    if (!bytes) return SGW_OK;
    const unsigned long long words = ((off + bytes + 15) >> 4) - (off >> 4);
    const uint32_t grid = (uint32_t)std::min<unsigned long long>((words + 255) / 256, 1216);
    k_copy_host<<<grid, 256, 0, st>>>(HostChunks{hs.dtab, hs.shift}, off, bytes, static_cast<uint8_t *>(dst));
    CK(cudaGetLastError());
    return SGW_OK;
  }
  char *d = static_cast<char *>(dst);
  const size_t cb = size_t(1) << hs.shift;
  while (bytes) {
    const size_t k = off >> hs.shift, o = off & (cb - 1);
    const size_t n = std::min(bytes, cb - o);
    CK(cudaMemcpyAsync(d, hs.h[k] + o, n, cudaMemcpyHostToDevice, st));
    d += n;
    off += n;
    bytes -= n;
  }
  return SGW_OK;
}

// Chunk sizes of a stream of `bytes` data bytes: chunks of 2^log2_chunk bytes
// (1 GiB by default, at least 4 KiB; larger powers of two when more than
// kMaxHostChunks would be needed), the last one cut to what remains plus 16
// zero bytes, all multiples of 16.
void plan_stream(HostStream &hs, size_t bytes, uint32_t log2_chunk) {
  hs.bytes = bytes;
  hs.shift = log2_chunk ? std::max<uint32_t>(log2_chunk, 12u) : 30u;
  const size_t total = bytes + 16;
  while (((total + (size_t(1) << hs.shift) - 1) >> hs.shift) > (size_t)kMaxHostChunks) ++hs.shift;
  const size_t cb = size_t(1) << hs.shift, k = (total + cb - 1) / cb;
  hs.h.assign(k, nullptr);
  hs.d.assign(k, 0);
  hs.size.assign(k, cb);
  hs.size[k - 1] = (total - (k - 1) * cb + 15) / 16 * 16;
}

// Allocates the chunks of both streams with two host threads while the
// calling thread fills each chunk as soon as it exists (fill(stream, k)):
// pinned allocation is mostly the driver zeroing and locking pages, and two
// calls in flight at once take about 0.6 of the time one call takes for the
// same bytes (21 GiB on a GB300 host: 0.78 s against 1.27 s; more threads
// did not help), while filling a chunk takes all host cores for a fraction
// of its allocation time.
#ifndef SGW_ALLOC_THREADS
#define SGW_ALLOC_THREADS 2
#endif
constexpr int kAllocThreads = SGW_ALLOC_THREADS;

template <class Fill>
cudaError_t alloc_and_fill(HostStream &a, HostStream &b, Fill fill) {
  std::vector<std::pair<HostStream *, size_t>> items;
  for (size_t i = 0; i < a.h.size(); ++i) items.push_back({&a, i});
  for (size_t i = 0; i < b.h.size(); ++i) items.push_back({&b, i});
  std::unique_ptr<std::atomic<int>[]> state(new std::atomic<int>[items.size()]);  // 0 pending, 1 ready, 2 failed
  for (size_t i = 0; i < items.size(); ++i) state[i].store(0);
  std::atomic<int> stop{0};
  cudaError_t err[kAllocThreads];
  for (int t = 0; t < kAllocThreads; ++t) err[t] = cudaSuccess;
  auto work = [&](int t) {
    for (size_t i = (size_t)t; i < items.size(); i += kAllocThreads) {
      if (stop.load()) { state[i].store(2); continue; }
      HostStream &hs = *items[i].first;
      const size_t k = items[i].second;
      void *p = nullptr;
      cudaError_t ce = cudaSuccess;
      if (hs.pageable) {  // ordinary pages, first touched (zeroed) by the filling threads
        p = mmap(nullptr, hs.size[k], PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
        if (p == MAP_FAILED) { p = nullptr; ce = cudaErrorMemoryAllocation; }
        else madvise(p, hs.size[k], MADV_NOHUGEPAGE);
      } else {
        ce = cudaHostAlloc(&p, hs.size[k], cudaHostAllocMapped | cudaHostAllocPortable);
      }
      if (ce != cudaSuccess) {
        err[t] = ce;
        stop.store(1);
        state[i].store(2);
        continue;
      }
      hs.h[k] = static_cast<char *>(p);
      state[i].store(1);
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < kAllocThreads; ++t) th.emplace_back(work, t);
  for (size_t i = 0; i < items.size(); ++i) {
    int st;
    while ((st = state[i].load()) == 0) std::this_thread::yield();
    if (st != 1) break;
    fill(*items[i].first, items[i].second);
  }
  for (auto &t : th) t.join();
  for (int t = 0; t < kAllocThreads; ++t)
    if (err[t] != cudaSuccess) return err[t];
  return cudaSuccess;
}

// Frees both streams' chunks, two at a time (as they were allocated).
void free_streams(HostStream &a, HostStream &b) {
  std::vector<std::pair<char *, size_t>> all;  // (chunk, bytes if pageable else 0)
  for (HostStream *hs : {&a, &b})
    for (size_t k = 0; k < hs->h.size() && !hs->borrowed; ++k)
      if (hs->h[k]) all.push_back({hs->h[k], hs->pageable ? hs->size[k] : 0});
  auto work = [&](size_t t) {
    for (size_t i = t; i < all.size(); i += 2) {
      if (all[i].second) munmap(all[i].first, all[i].second);
      else cudaFreeHost(all[i].first);
    }
  };
  if (all.size() > 1) {
    std::thread other(work, 1);
    work(0);
    other.join();
  } else {
    work(0);
    work(1);
  }
  for (HostStream *hs : {&a, &b}) {
    hs->h.clear();
    hs->d.clear();
    hs->size.clear();
  }
}

// Whole-range streaming moves records by DMA from the transfer copy.  On
// some GB300 machines the learned policy's transfers ran at half their
// usual rate while the plain policy's gathers did not, so the engine times a
// few DMA copies at creation (and, when profiling, the streamed copies of
// every run, in prof_collect); the learned policy streams whole ranges only
// while the rate is at least kMinStreamGBs.  Copies below 64 MB are too short
// to time: the rate is then taken as good.
int probe_stream_dma(sgw_engine *e) {
  e->dma_gbs = -1.0;
  if (e->hs_ends.h.empty()) return SGW_OK;
  const size_t bytes = std::min<size_t>(std::min<size_t>(e->hs_ends.size[0], (size_t)e->cap * 4 * e->W),
                                        size_t(256) << 20) & ~size_t(15);
  if (bytes < (size_t(64) << 20)) return SGW_OK;
  cudaEvent_t a = nullptr, b = nullptr;
  CK(cudaEventCreate(&a));
  if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return fail(SGW_ECUDA, "event creation"); }
  double best = 0.0;
  int st = SGW_OK;
  for (int i = 0; i < 4 && st == SGW_OK; ++i) {  // the first copy warms up
    cudaEventRecord(a, e->s_copy);
    st = copy_from_host(e->hs_ends, e->d_buf[0], 0, bytes, e->s_copy);
    cudaEventRecord(b, e->s_copy);
    if (cudaEventSynchronize(b) != cudaSuccess) { st = fail(SGW_ECUDA, "transfer-copy DMA probe"); break; }
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (i > 0 && ms > 0) best = std::max(best, (double)bytes / (ms * 1e6));
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (st == SGW_OK) e->dma_gbs = best;
  return st;
}

int read_ctl(sgw_engine *e) {
  CK(cudaMemcpyAsync(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->s_comp));
  e->stats.d2h_bytes += sizeof(Ctl);
  CK(cudaStreamSynchronize(e->s_comp));
  e->stats.inner_iterations = (uint64_t)e->h_ctl->iters_total + e->hub_iters;
  return check_ctl_error(e);
}

// ---- arena layout ------------------------------------------------------------------
// One cudaMalloc holds everything.  The node pointers, scan tile state and
// control block sit at the front for the engine's lifetime; the rest is carved
// per run for the algorithm family:
//   integer (BFS/SSSP/SSWP/CC): value u32, label1/label2 u8, queue, ptr
//   PR: rank f64, residual f64, queue, ptr, per-queue-entry push f64
// followed by the partition table, the chunk list and the edge buffers.
enum Family { FAM_INT = 0, FAM_PR = 1 };

struct Layout {
  size_t off, obase, tflag, tagg, tincl, ctl, mlp, sel, gmask, hct;  // common
  size_t value, l1, l2, queue, ptr, delta, qpush;     // family
  size_t parts, ranges, rstat, wl, buf[kMaxBuf], total;
  uint64_t cap;
  uint32_t max_parts, wl_cap;
};

Layout make_layout(int fam, uint32_t n, uint64_t m, uint32_t esz, uint32_t nbuf,
                   uint32_t num_tiles, uint64_t cap, uint32_t chunk, uint32_t tdm, bool wide) {
  Layout L{};
  size_t p = 0;
  auto take = [&](size_t bytes) { size_t at = p; p += align_up(bytes, 256); return at; };
  L.off = take(4ull * (n + 1));
  L.obase = take(wide ? 8ull * ((n >> kOffGroupLog2) + 2) : 0);
  L.tflag = take(4ull * num_tiles);
  L.tagg = take(8ull * num_tiles);
  L.tincl = take(8ull * num_tiles);
  L.ctl = take(sizeof(Ctl));
  L.mlp = take(sizeof(__nv_bfloat16) * kMlpParams);
  L.sel = take(sizeof(unsigned long long) * kSelBins);
  L.gmask = take(4ull * ((n + kGenVPerLane - 1) / kGenVPerLane));
  L.hct = take(2ull * kMaxHostChunks * sizeof(unsigned long long));
  if (fam == FAM_INT) {
    L.value = take(4ull * n);
    L.l1 = take(n);
    L.l2 = take(n);
  } else {
    L.value = take(8ull * n);
    L.delta = take(8ull * n);
  }
  L.queue = take(4ull * n);
  L.ptr = take(4ull * (n + 1));
  if (fam == FAM_PR) L.qpush = take(8ull * n);
  L.cap = cap;
  L.max_parts = (uint32_t)std::min<uint64_t>(2ull * ((uint64_t)m / std::max<uint64_t>(cap, 1) + 1) + 2,
                                             0x7fffffffull);
  L.wl_cap = (uint32_t)std::min<uint64_t>(cap / chunk + cap / std::max<uint32_t>(tdm, 1) + 64, 0x7fffffffull);
  L.parts = take(sizeof(Part) * (size_t)L.max_parts);
  L.ranges = take(sizeof(RangeInfo) * (size_t)L.max_parts);
  L.rstat = take(sizeof(RangeStat) * (size_t)L.max_parts);
  L.wl = take(16ull * (size_t)L.wl_cap);  // WorkItem and PrItem are 16 B
  for (uint32_t b = 0; b < kMaxBuf; ++b) L.buf[b] = b < nbuf ? take(cap * esz) : L.buf[0];
  L.total = p;
  return L;
}

// Largest edge-buffer capacity whose layout fits `bytes` (0 if none does).
uint64_t fit_cap(int fam, const sgw_engine_opts &o, uint32_t n, uint64_t m, uint32_t esz,
                 uint32_t nbuf, uint32_t num_tiles, uint64_t bytes, bool wide) {
  auto total = [&](uint64_t cap) {
    return (uint64_t)make_layout(fam, n, m, esz, nbuf, num_tiles, cap, o.chunk_edges, o.tile_degree_max, wide).total;
  };
  // max_partition_size <= DIST_INFINITY, and no larger than the whole graph
  const uint64_t hi_cap = std::min<uint64_t>(std::max<uint64_t>(m, 64), 4294967294ull);
  // The layout is convex in cap: the partition/range tables shrink as 1/cap,
  // the buffers grow as cap.  Below the minimum nothing fits; above it the
  // size grows monotonically, so bisect for the largest cap that fits.
  const double table = 2.0 * m * (sizeof(Part) + sizeof(RangeInfo) + sizeof(RangeStat));
  const double per_edge = (double)nbuf * esz + 16.0 / o.chunk_edges + 16.0 / o.tile_degree_max;
  uint64_t lo = std::max<uint64_t>(64, (uint64_t)std::sqrt(table / per_edge));
  lo = std::min(lo, hi_cap);
  if (total(lo) > bytes) return 0;
  if (total(hi_cap) <= bytes) return hi_cap;
  uint64_t a = lo, b = hi_cap;  // total(a) fits, total(b) does not
  while (b - a > 1) {
    const uint64_t mid = a + (b - a) / 2;
    if (total(mid) <= bytes) a = mid; else b = mid;
  }
  return a;
}

int carve(sgw_engine *e, int fam, uint64_t cap) {
  const Layout L = make_layout(fam, e->n, e->m, e->rec_bytes, e->nbuf, e->num_tiles, cap,
                               e->opts.chunk_edges, e->opts.tile_degree_max, e->wide);
  if (L.total > e->arena_bytes) return fail(SGW_EBUDGET, "layout exceeds the arena");
  char *b = e->d_arena;
  e->d_off = (uint32_t *)(b + L.off);
  e->d_obase = (unsigned long long *)(b + L.obase);
  e->d_tflag = (uint32_t *)(b + L.tflag);
  e->d_tagg = (unsigned long long *)(b + L.tagg);
  e->d_tincl = (unsigned long long *)(b + L.tincl);
  e->d_ctl = (Ctl *)(b + L.ctl);
  e->d_gmask = (uint32_t *)(b + L.gmask);
  e->d_hct = (unsigned long long *)(b + L.hct);
  e->d_value = (uint32_t *)(b + L.value);
  e->d_l1 = fam == FAM_INT ? (uint8_t *)(b + L.l1) : nullptr;
  e->d_l2 = fam == FAM_INT ? (uint8_t *)(b + L.l2) : nullptr;
  e->d_pval = fam == FAM_PR ? (double *)(b + L.value) : nullptr;
  e->d_delta = fam == FAM_PR ? (double *)(b + L.delta) : nullptr;
  e->d_qpush = fam == FAM_PR ? (double *)(b + L.qpush) : nullptr;
  e->d_queue = (uint32_t *)(b + L.queue);
  e->d_ptr = (uint32_t *)(b + L.ptr);
  e->d_parts = (Part *)(b + L.parts);
  e->d_ranges = (RangeInfo *)(b + L.ranges);
  e->d_rstat = (RangeStat *)(b + L.rstat);
  e->d_mlp = (__nv_bfloat16 *)(b + L.mlp);
  e->d_sel_hist = (unsigned long long *)(b + L.sel);
  e->d_wl = (WorkItem *)(b + L.wl);
  for (int i = 0; i < kMaxBuf; ++i) {
    e->d_buf[i] = (uint32_t *)(b + L.buf[i]);
    // split form: the buffer's cap weight bytes follow its cap end words
    e->d_wbuf[i] = e->split ? (uint8_t *)(b + L.buf[i]) + 4ull * L.cap : nullptr;
  }
  e->cap = L.cap;
  e->max_parts = L.max_parts;
  e->wl_cap = L.wl_cap;
  e->fam = fam;
  // static vertex ranges: greedy runs of whole vertices whose edges fit one
  // buffer; a vertex above the buffer is a range of its own
  e->ranges.clear();
  const sgw_graph *g = e->g;
  for (uint32_t v = 0; v < e->n;) {
    const uint64_t limit = np_at(g, v) + e->cap;
    uint32_t lo = v + 1, hi = e->n + 1;  // first index in (v, n] with np > limit
    while (lo < hi) {
      const uint32_t mid = lo + (hi - lo) / 2;
      if (np_at(g, mid) <= limit) lo = mid + 1; else hi = mid;
    }
    uint32_t v1 = lo - 1;
    if (v1 <= v) v1 = v + 1;
    e->ranges.push_back(RangeInfo{v, v1, np_at(g, v), np_at(g, v1)});
    v = v1;
  }
  if (e->ranges.size() > e->max_parts) return fail(SGW_ERANGE, "too many vertex ranges");
  for (int i = 0; i < kMaxBuf; ++i) e->buf_range[i] = -1;
  return SGW_OK;
}

int generate_and_stats(sgw_engine *e, int consume);

// Copies the range table to the device (after carving, on the compute stream).
int upload_ranges(sgw_engine *e) {
  if (!e->ranges.empty())
    CK(cudaMemcpyAsync(e->d_ranges, e->ranges.data(), sizeof(RangeInfo) * e->ranges.size(),
                       cudaMemcpyHostToDevice, e->s_comp));
  CK(cudaMemsetAsync(e->d_rstat, 0, sizeof(RangeStat) * e->max_parts, e->s_comp));
  return SGW_OK;
}

// ---- launch helpers ---------------------------------------------------------------
uint32_t grid_for(const sgw_engine *e, uint64_t items, uint32_t per_cta) {
  uint64_t g = (items + per_cta - 1) / per_cta;
  uint64_t mx = (uint64_t)e->num_sms * 8;
  return (uint32_t)std::max<uint64_t>(1, std::min(g, mx));
}

// Deferral target in 1/1000 of the edges (0 = whole frontier).  Automatic:
// defer when the edges are far larger than what the buffers hold, where each
// avoided re-transfer is worth more than the selection passes cost.
uint32_t defer_permille(const sgw_engine *e) {
  const uint32_t o = e->opts.sched_defer_permille;
  if (o > 1000) return 0;
  if (o) return o;
  const double edges = (double)e->m * e->rec_bytes;
  const double space = (double)e->nbuf * (double)e->cap * e->rec_bytes;
  return edges > 4.0 * space ? 250u : 0u;
}

// Frontier deferral: value range, degree histogram and the selected bin of
// the pushable active vertices, all on the device (the generate reads the
// result from the control block).
int launch_select(sgw_engine *e) {
  const int algo = e->params.algo;
  size_t slot = 0;
  TRY(prof_begin(e, K_GENERATE, e->s_comp, &slot));
  CK(cudaMemsetAsync(e->d_sel_hist, 0, sizeof(unsigned long long) * kSelBins, e->s_comp));
  const uint32_t grid = grid_for(e, (e->n + 15) / 16, 256);
  k_select_hist<<<grid, 256, 0, e->s_comp>>>(e->n, algo, e->d_l1, e->d_l2, e->d_off, e->d_value, e->d_ctl,
                                             e->d_sel_hist);
  CK(cudaGetLastError());
  const unsigned long long target = (unsigned long long)((double)e->m * (double)defer_permille(e) / 1000.0);
  k_select_pick<<<1, kSelBins / 4, 0, e->s_comp>>>(algo, e->d_sel_hist, target, e->d_ctl);
  CK(cudaGetLastError());
  TRY(prof_end(e, e->s_comp, slot));
  e->stats.launches += 2;
  return SGW_OK;
}

int launch_generate(sgw_engine *e, int consume) {
  GenArgs a;
  a.n = e->n;
  a.l1 = e->d_l1;
  a.l2 = e->d_l2;
  a.off = e->d_off;
  a.queue = e->d_queue;
  a.ptr = e->d_ptr;
  a.tflag = e->d_tflag;
  a.tagg = e->d_tagg;
  a.tincl = e->d_tincl;
  a.ctl = e->d_ctl;
  a.gmask = e->d_gmask;
  e->epoch = (e->epoch + 1) & 0x3fffffffu;
  if (e->epoch == 0) e->epoch = 1;
  a.epoch = e->epoch;
  a.num_tiles = e->num_tiles;
  a.consume = consume;
  a.edge_limit = e->edge_limit;
  a.delta = e->d_delta;
  a.pval = e->d_pval;
  a.qpush = e->d_qpush;
  a.acc = (double)e->params.pr_acc;
  a.damping = (double)e->params.pr_damping;
  if (e->policy == SGW_POLICY_LEARNED && e->fam == FAM_INT) {
    // learned policy: never queue vertices that cannot push, and with a
    // deferral target take the frontier lowest values first (highest: SSWP)
    a.sel_mode = (e->opts.sched_flags & SGW_SCHED_KEEP_IDLE) ? 0 : 1;
    a.algo = e->params.algo;
    a.value = e->d_value;
    // sync BFS queues one level at a time: nothing to order, so no passes
    const bool level_sync = e->params.algo == SGW_BFS && e->params.mode == SGW_SYNC;
    if (defer_permille(e) && !level_sync) {
      a.sel_mode |= 2;
      TRY(launch_select(e));
    }
  }
  CK(cudaMemsetAsync(&e->d_ctl->num_seen, 0, sizeof(uint32_t), e->s_comp));
  size_t slot = 0;
  TRY(prof_begin(e, K_GENERATE, e->s_comp, &slot));
  if (e->fam == FAM_PR) k_generate_count<true><<<e->num_tiles, kGenThreads, 0, e->s_comp>>>(a);
  else k_generate_count<false><<<e->num_tiles, kGenThreads, 0, e->s_comp>>>(a);
  CK(cudaGetLastError());
  k_generate_scan<<<1, kGenScanThreads, 0, e->s_comp>>>(a);
  CK(cudaGetLastError());
  if (e->fam == FAM_PR) k_generate_write<true><<<e->num_tiles, kGenThreads, 0, e->s_comp>>>(a);
  else k_generate_write<false><<<e->num_tiles, kGenThreads, 0, e->s_comp>>>(a);
  e->stats.launches += 3;
  CK(cudaGetLastError());
  TRY(prof_end(e, e->s_comp, slot));
  e->stats.generate_launches += 1;
  e->parts_valid = false;
  return SGW_OK;
}

int launch_plan(sgw_engine *e) {
  size_t slot = 0;
  TRY(prof_begin(e, K_PLAN, e->s_comp, &slot));
  k_plan<<<1, 32, 0, e->s_comp>>>(e->d_ptr, e->d_queue, e->d_ctl, e->d_parts, e->max_parts,
                                   (unsigned long long)e->cap);
  CK(cudaGetLastError());
  TRY(prof_end(e, e->s_comp, slot));
  e->stats.launches += 1;
  return SGW_OK;
}

// generate + plan + one read-back: the per-global-iteration host sync.
int generate_and_plan(sgw_engine *e, int consume) {
  TRY(launch_generate(e, consume));
  TRY(launch_plan(e));
  CK(cudaMemcpyAsync(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->s_comp));
  CK(cudaStreamSynchronize(e->s_comp));
  TRY(check_ctl_error(e));
  e->num_active = e->h_ctl->num_active;
  e->num_active_edges = e->h_ctl->num_active_edges;
  e->num_parts = e->h_ctl->num_parts;
  if (e->num_parts > 0) {
    CK(cudaMemcpyAsync(e->h_parts, e->d_parts, sizeof(Part) * e->num_parts,
                       cudaMemcpyDeviceToHost, e->s_comp));
    CK(cudaStreamSynchronize(e->s_comp));
  }
  e->stats.d2h_bytes += sizeof(Ctl) + sizeof(Part) * e->num_parts;
  e->parts_valid = true;
  return SGW_OK;
}

bool is_hub(const sgw_engine *e, const Part &p) { return p.edge_count > e->cap; }

void trace_partition(sgw_engine *e, uint32_t p, uint32_t inner) {
  if (!e->trace_on) return;
  const Part &q = e->h_parts[p];
  sgw_trace_rec r;
  memset(&r, 0, sizeof(r));
  r.global_iteration = e->gitr;
  r.partition = p;
  r.num_partitions = e->num_parts;
  r.inner_iterations = inner;
  r.active_nodes = q.size;
  r.first_vertex = q.first_vertex;
  r.active_edges = q.edge_count;
  r.iteration_active_nodes = e->num_active;
  r.iteration_active_edges = e->num_active_edges;
  r.bytes_h2d = q.edge_count * (4ull * e->W + (e->use_w ? 1 : 0));
  r.transfer = is_hub(e, q) ? 2 : 0;
  e->trace.push_back(r);
}

int gather_into(sgw_engine *e, const Part &q, uint32_t b, cudaStream_t s);

int enqueue_gather(sgw_engine *e, uint32_t p, cudaStream_t s) {
  const Part &q = e->h_parts[p];
  if (is_hub(e, q) || q.edge_count == 0) return SGW_OK;
  return gather_into(e, q, p % e->nbuf, s);
}

// Opts the vectorised gather kernels into more than 48 KB of dynamic shared
// memory where their tile needs it.
template <bool WIDE>
bool allow_gather_smem(size_t bytes) {
  if (bytes <= 48 * 1024) return true;
  const auto A = cudaFuncAttributeMaxDynamicSharedMemorySize;
  return cudaFuncSetAttribute(k_gather_v<4, true, WIDE>, A, (int)bytes) == cudaSuccess &&
         cudaFuncSetAttribute(k_gather_v<4, false, WIDE>, A, (int)bytes) == cudaSuccess &&
         cudaFuncSetAttribute(k_gather_v<8, false, WIDE>, A, (int)bytes) == cudaSuccess;
}

// The gather kernel for the engine's transfer form; WIDE: host positions
// of 2^32 records or more (u64 node pointers).
template <bool WIDE>
void launch_gather(sgw_engine *e, const Part &q, uint32_t b, cudaStream_t s, uint32_t grid,
                   const HostChunks &h16, const HostChunks &hw16) {
  const unsigned long long *ob = WIDE ? e->d_obase : nullptr;
  const size_t smem = WIDE ? kGatherSmemBytesWide : kGatherSmemBytes;
  const uint32_t cnt = (uint32_t)q.edge_count;
  if (e->vec_gather && e->W == 1 && e->use_w)  // split form: destination words and weight bytes
    k_gather_v<4, true, WIDE><<<grid, kGatherThreads, smem, s>>>(e->d_queue, e->d_ptr, e->d_off, ob, h16,
                                                                 e->d_buf[b], hw16, e->d_wbuf[b], q.from, q.size,
                                                                 q.edge_from, cnt);
  else if (e->vec_gather && e->W == 1)
    k_gather_v<4, false, WIDE><<<grid, kGatherThreads, smem, s>>>(e->d_queue, e->d_ptr, e->d_off, ob, h16,
                                                                  e->d_buf[b], hw16, nullptr, q.from, q.size,
                                                                  q.edge_from, cnt);
  else if (e->vec_gather)
    k_gather_v<8, false, WIDE><<<grid, kGatherThreads, smem, s>>>(e->d_queue, e->d_ptr, e->d_off, ob, h16,
                                                                  e->d_buf[b], hw16, nullptr, q.from, q.size,
                                                                  q.edge_from, cnt);
  else if (e->W == 1)
    k_gather<1, WIDE><<<grid, kGatherThreads, 0, s>>>(e->d_queue, e->d_ptr, e->d_off, ob, h16, e->d_buf[b],
                                                      q.from, q.size, q.edge_from, cnt);
  else
    k_gather<2, WIDE><<<grid, kGatherThreads, 0, s>>>(e->d_queue, e->d_ptr, e->d_off, ob, h16, e->d_buf[b],
                                                      q.from, q.size, q.edge_from, cnt);
}

// Gathers partition q's active edges into buffer b on stream s, after the
// buffer's last reader, and records ev_ready[b].
int gather_into(sgw_engine *e, const Part &q, uint32_t b, cudaStream_t s) {
  CK(cudaStreamWaitEvent(s, e->ev_free[b], 0));
  size_t slot = 0;
  TRY(prof_begin(e, K_GATHER, s, &slot));
  // default grid: 2 CTAs per SM (measured on RMAT-28 / 8 GB, learned
  // schedule, one process, alternating order: 163.9 ms per run against 167.6
  // with 1.5 per SM and 166.3 with 3; within 1.5% at RMAT-24 / 1 GB).  Fewer
  // gather CTAs leave the concurrent relaxation more of each SM (72 against
  // 116 ms of relaxation per run at 1.5 and 3 per SM); with one per SM the
  // gather no longer keeps up with the host link.
  const uint32_t gmax = e->opts.gather_ctas ? e->opts.gather_ctas : 2u * e->num_sms;
  const uint32_t grid = std::min<uint32_t>(grid_for(e, q.edge_count, kGatherTile), gmax);
  const HostChunks h16{e->d_hct, e->hs_ends.shift};
  const HostChunks hw16{e->d_hct + kMaxHostChunks, e->hs_w.shift};
  if (e->wide) launch_gather<true>(e, q, b, s, grid, h16, hw16);
  else launch_gather<false>(e, q, b, s, grid, h16, hw16);
  CK(cudaGetLastError());
  e->stats.h2d_bytes += q.edge_count * (4ull * e->W + (e->use_w ? 1 : 0));
  e->stats.gather_bytes += q.edge_count * (4ull * e->W + (e->use_w ? 1 : 0));
  TRY(prof_end(e, s, slot));
  CK(cudaEventRecord(e->ev_ready[b], s));
  e->stats.launches += 1;
  e->stats.gather_launches += 1;
  return SGW_OK;
}

template <int ALGO, bool ASYNC, int W>
int launch_relax_pair(sgw_engine *e, const Part &q, uint32_t b, uint32_t iter, uint8_t *cur,
                      uint8_t *nxt) {
  RelaxArgs a;
  a.queue = e->d_queue;
  a.ptr = e->d_ptr;
  a.buf = e->d_buf[b];
  a.value = e->d_value;
  a.cur = cur;
  a.nxt = nxt;
  a.ctl = e->d_ctl;
  a.wl = e->d_wl;
  a.wl_cap = e->wl_cap;
  a.from = q.from;
  a.size = q.size;
  a.edge_from = q.edge_from;
  a.iter = iter;
  a.tile_degree_max = e->opts.tile_degree_max;
  a.chunk_edges = e->opts.chunk_edges;
  a.pbits = e->pbits;
  a.streamed = e->cur_streamed;
  a.stream_base = (uint32_t)e->cur_stream_base;  // with the low words of off: offsets mod 2^32
  a.off = e->d_off;
  a.wbuf = e->use_w ? e->d_wbuf[b] : nullptr;
  const uint32_t g1 = grid_for(e, q.size, kRelaxThreads);
  if (e->opts.flags & SGW_OPT_CTA_TILES) k_relax_tile<ALGO, ASYNC, W><<<g1, kRelaxThreads, 0, e->s_comp>>>(a);
  else k_relax_warp<ALGO, ASYNC, W><<<g1, kRelaxThreads, 0, e->s_comp>>>(a);
  CK(cudaGetLastError());
  k_relax_chunks<ALGO, ASYNC, W><<<e->num_sms * 4, kRelaxThreads, 0, e->s_comp>>>(a);
  CK(cudaGetLastError());
  e->stats.launches += 2;
  e->stats.relax_launches += 2;
  return SGW_OK;
}

template <int ALGO, int W>
int relax_dispatch_w(sgw_engine *e, const Part &q, uint32_t b, uint32_t iter, bool async,
                     uint8_t *cur, uint8_t *nxt) {
  if (async) return launch_relax_pair<ALGO, true, W>(e, q, b, iter, cur, nxt);
  return launch_relax_pair<ALGO, false, W>(e, q, b, iter, cur, nxt);
}

template <int ALGO>
int relax_dispatch(sgw_engine *e, const Part &q, uint32_t b, uint32_t iter, bool async,
                   uint8_t *cur, uint8_t *nxt) {
  if (e->W == 1) return relax_dispatch_w<ALGO, 1>(e, q, b, iter, async, cur, nxt);
  return relax_dispatch_w<ALGO, 2>(e, q, b, iter, async, cur, nxt);
}

template <bool ASYNC, int W>
int launch_pr_pair(sgw_engine *e, const Part &q, uint32_t b, uint32_t iter) {
  PrArgs a;
  a.queue = e->d_queue;
  a.ptr = e->d_ptr;
  a.buf = e->d_buf[b];
  a.pval = e->d_pval;
  a.delta = e->d_delta;
  a.qpush = e->d_qpush;
  a.ctl = e->d_ctl;
  a.wl = reinterpret_cast<PrItem *>(e->d_wl);
  a.wl_cap = e->wl_cap;
  a.from = q.from;
  a.size = q.size;
  a.edge_from = q.edge_from;
  a.iter = iter;
  a.tile_degree_max = e->opts.tile_degree_max;
  a.chunk_edges = e->opts.chunk_edges;
  a.pbits = e->pbits;
  a.streamed = e->cur_streamed;
  a.stream_base = (uint32_t)e->cur_stream_base;  // with the low words of off: offsets mod 2^32
  a.off = e->d_off;
  a.acc = (double)e->params.pr_acc;
  a.damping = (double)e->params.pr_damping;
  k_pr_tile<ASYNC, W><<<grid_for(e, q.size, kRelaxThreads), kRelaxThreads, 0, e->s_comp>>>(a);
  CK(cudaGetLastError());
  k_pr_chunks<ASYNC, W><<<e->num_sms * 4, kRelaxThreads, 0, e->s_comp>>>(a);
  CK(cudaGetLastError());
  e->stats.launches += 2;
  e->stats.relax_launches += 2;
  return SGW_OK;
}

int launch_relax(sgw_engine *e, const Part &q, uint32_t b, uint32_t iter, bool async) {
  if (e->params.algo == SGW_PR) {
    if (e->W == 1) return async ? launch_pr_pair<true, 1>(e, q, b, iter) : launch_pr_pair<false, 1>(e, q, b, iter);
    return async ? launch_pr_pair<true, 2>(e, q, b, iter) : launch_pr_pair<false, 2>(e, q, b, iter);
  }
  uint8_t *cur = e->d_l1, *nxt = e->d_l2;
  if (async && (iter % 2 == 0)) std::swap(cur, nxt);  // ping-pong (sssp-async.cu:108-109)
  switch (e->params.algo) {
    case SGW_BFS: return relax_dispatch<SGW_BFS>(e, q, b, iter, async, cur, nxt);
    case SGW_SSSP: return relax_dispatch<SGW_SSSP>(e, q, b, iter, async, cur, nxt);
    case SGW_SSWP: return relax_dispatch<SGW_SSWP>(e, q, b, iter, async, cur, nxt);
    case SGW_CC: return relax_dispatch<SGW_CC>(e, q, b, iter, async, cur, nxt);
    default: return fail(SGW_EINVAL, "algorithm %d not supported", e->params.algo);
  }
}

template <int ALGO, int W>
int launch_flat_w(sgw_engine *e, uint32_t b, uint32_t count) {
  k_relax_flat<ALGO, W><<<grid_for(e, count, 256), 256, 0, e->s_comp>>>(
      e->d_buf[b], e->use_w ? e->d_wbuf[b] : nullptr, count, e->pbits, e->d_value, e->d_l2, e->d_ctl);
  CK(cudaGetLastError());
  return SGW_OK;
}
template <int ALGO>
int launch_flat(sgw_engine *e, uint32_t b, uint32_t count) {
  return e->W == 1 ? launch_flat_w<ALGO, 1>(e, b, count) : launch_flat_w<ALGO, 2>(e, b, count);
}

// A single vertex whose edges exceed one buffer: claim it once, then stream
// and relax its edges piece by piece (one inner iteration).
int process_hub(sgw_engine *e, const Part &q, uint32_t b) {
  const bool async = e->params.mode == SGW_ASYNC;
  const bool pr = e->params.algo == SGW_PR;
  const uint32_t u = q.first_vertex;
  if (pr) k_pr_hub_claim<<<1, 1, 0, e->s_comp>>>(q.from, e->d_qpush, e->d_ctl);
  else if (async) k_hub_claim<true><<<1, 1, 0, e->s_comp>>>(u, e->d_value, e->d_l1, e->d_l2, e->d_ctl);
  else k_hub_claim<false><<<1, 1, 0, e->s_comp>>>(u, e->d_value, e->d_l1, e->d_l2, e->d_ctl);
  CK(cudaGetLastError());
  const uint64_t deg = q.edge_count;
  const uint64_t hoff = np_at(e->g, u);
  const size_t esz = 4ull * e->W;
  for (uint64_t s = 0; s < deg; s += e->cap) {
    const uint32_t cnt = (uint32_t)std::min<uint64_t>(e->cap, deg - s);
    size_t slot = 0;
    TRY(prof_begin(e, K_STREAM, e->s_comp, &slot));
    TRY(copy_from_host(e->hs_ends, e->d_buf[b], (hoff + s) * esz, cnt * esz, e->s_comp));
    e->stats.h2d_bytes += cnt * esz;
    e->stream_bytes += cnt * esz + (e->use_w ? cnt : 0);
    if (e->use_w) {
      TRY(copy_from_host(e->hs_w, e->d_wbuf[b], hoff + s, cnt, e->s_comp));
      e->stats.h2d_bytes += cnt;
    }
    TRY(prof_end(e, e->s_comp, slot));
    TRY(prof_begin(e, K_RELAX, e->s_comp, &slot));
    int st = SGW_OK;
    switch (e->params.algo) {
      case SGW_PR:
        if (e->W == 1) k_pr_flat<1><<<grid_for(e, cnt, 256), 256, 0, e->s_comp>>>(e->d_buf[b], cnt, e->pbits, e->d_delta, e->d_ctl);
        else k_pr_flat<2><<<grid_for(e, cnt, 256), 256, 0, e->s_comp>>>(e->d_buf[b], cnt, e->pbits, e->d_delta, e->d_ctl);
        if (cudaGetLastError() != cudaSuccess) st = fail(SGW_ECUDA, "k_pr_flat launch");
        break;
      case SGW_BFS: st = launch_flat<SGW_BFS>(e, b, cnt); break;
      case SGW_SSSP: st = launch_flat<SGW_SSSP>(e, b, cnt); break;
      case SGW_SSWP: st = launch_flat<SGW_SSWP>(e, b, cnt); break;
      default: st = launch_flat<SGW_CC>(e, b, cnt); break;
    }
    TRY(st);
    TRY(prof_end(e, e->s_comp, slot));
    e->stats.launches += 1;
    e->stats.relax_launches += 1;
  }
  e->hub_iters += 1;
  e->stats.inner_iterations += 1;
  return SGW_OK;
}

// Relaxation of one resident partition: sync = one pass; async = mixLabels
// then inner iterations until no relaxation improves (or max_inner).
// Inner iterations are counted on the device (Ctl::iters_total, refreshed
// into the statistics by every control-block read).  With sync_always false
// a partition whose inner cap is reached returns without waiting for it
// (*iters_out is then 0: unknown until the next read).  The learned policy
// keeps the wait: letting the host run ahead put more gathers beside each
// relaxation and made both slower (RMAT-24 SSSP-async: 12.2 against 17.0
// GTEPS).
int process_resident(sgw_engine *e, const Part &q, uint32_t b, uint32_t *iters_out, bool sync_always = true) {
  const bool async = e->params.mode == SGW_ASYNC;
  // upd, wl_count, iters_run
  CK(cudaMemsetAsync(&e->d_ctl->upd[0], 0, sizeof(uint32_t) * 9, e->s_comp));
  if (!async) {
    size_t slot = 0;
    TRY(prof_begin(e, K_RELAX, e->s_comp, &slot));
    TRY(launch_relax(e, q, b, 1, false));
    TRY(prof_end(e, e->s_comp, slot));
    if (iters_out) *iters_out = 1;
    return SGW_OK;
  }
  if (e->params.algo != SGW_PR) {  // PR carries no labels
    k_mix<<<grid_for(e, q.size, 256), 256, 0, e->s_comp>>>(e->d_queue, q.from, q.size, e->d_l1, e->d_l2);
    CK(cudaGetLastError());
    e->stats.launches += 1;
  }
  uint32_t max_inner = e->params.max_inner ? e->params.max_inner : 0xffffffffu;
  if (e->range_inner_cap) max_inner = std::min(max_inner, e->range_inner_cap);
  uint32_t iter = 1;
  const uint32_t batch = std::max<uint32_t>(1, e->opts.inner_batch);
  while (true) {
    const uint32_t nb = std::min<uint32_t>(batch, max_inner - (iter - 1));
    size_t slot = 0;
    TRY(prof_begin(e, K_RELAX, e->s_comp, &slot));
    for (uint32_t k = 0; k < nb; ++k, ++iter) TRY(launch_relax(e, q, b, iter, true));
    TRY(prof_end(e, e->s_comp, slot));
    const uint32_t last = iter - 1;
    if (!sync_always && last >= max_inner) {  // capped: nothing to decide on the host
      if (iters_out) *iters_out = 0;
      return SGW_OK;
    }
    TRY(read_ctl(e));
    if (e->h_ctl->upd[last & 3u] == 0) break;  // converged
    if (last >= max_inner) break;             // leftover labels go to the next generate
  }
  if (iters_out) *iters_out = e->h_ctl->iters_run;
  return SGW_OK;
}

int validate_params(const sgw_engine *e, const sgw_run_params *p) {
  if (!p) return fail(SGW_EINVAL, "null params");
  if (p->algo < SGW_BFS || p->algo > SGW_PR) return fail(SGW_EINVAL, "bad algorithm %d", p->algo);
  if (p->mode != SGW_SYNC && p->mode != SGW_ASYNC) return fail(SGW_EINVAL, "bad mode %d", p->mode);
  if (p->algo == SGW_PR && e->cap_fam[FAM_PR] == 0)
    return fail(SGW_EBUDGET, "budget too small for the PageRank vertex state (f64 ranks and residuals)");
  if (p->algo == SGW_PR && !(p->pr_acc > 0.0f) )
    return fail(SGW_EINVAL, "pr_acc must be positive");
  if ((p->algo == SGW_SSSP || p->algo == SGW_SSWP) && !e->g->weighted)
    return fail(SGW_EINVAL, "SSSP/SSWP need a weighted graph (.bwcsr/.wel)");
  if (p->algo != SGW_CC && p->algo != SGW_PR && p->source >= e->n)
    return fail(SGW_EINVAL, "source %u out of range (n=%u)", p->source, e->n);
  return SGW_OK;
}

int state_init(sgw_engine *e, const sgw_run_params *p) {
  TRY(validate_params(e, p));
  CK(cudaSetDevice(e->device));
  e->params = *p;
  e->use_w = e->split && (p->algo == SGW_SSSP || p->algo == SGW_SSWP);
  e->stats = sgw_run_stats{};
  e->hub_iters = 0;
  e->prof_used = 0;
  e->initialized = false;
  e->gitr = 0;
  e->trace.clear();
  e->rtrace.clear();
  const int fam = p->algo == SGW_PR ? FAM_PR : FAM_INT;
  if (fam != e->fam) TRY(carve(e, fam, e->cap_fam[fam]));
  // every run starts with empty edge buffers (nothing carried between runs)
  for (int i = 0; i < kMaxBuf; ++i) e->buf_range[i] = -1;
  if (e->policy == SGW_POLICY_LEARNED) TRY(upload_ranges(e));
  const uint32_t src = (p->algo == SGW_CC || p->algo == SGW_PR) ? 0xffffffffu : p->source;
  if (fam == FAM_PR)
    k_pr_init<<<grid_for(e, e->n, 256), 256, 0, e->s_comp>>>(e->n, (double)p->pr_init, e->d_pval, e->d_delta);
  else
    k_init<<<grid_for(e, e->n, 256), 256, 0, e->s_comp>>>(e->n, p->algo, p->mode, src, e->d_value,
                                                          e->d_l1, e->d_l2);
  CK(cudaGetLastError());
  CK(cudaMemsetAsync(e->d_ctl, 0, sizeof(Ctl), e->s_comp));
  e->stats.launches += 1;
  const bool async = p->mode == SGW_ASYNC;
  if (e->policy == SGW_POLICY_LEARNED) TRY(generate_and_stats(e, async ? 0 : 1));
  else TRY(generate_and_plan(e, async ? 0 : 1));
  if (async && p->algo != SGW_CC && p->algo != SGW_PR) {
    k_async_reset<<<grid_for(e, e->n, 256), 256, 0, e->s_comp>>>(e->n, p->source, e->d_l1);
    CK(cudaGetLastError());
    e->stats.launches += 1;
  }
  e->initialized = true;
  return SGW_OK;
}

// All partitions of one global iteration, gathers double-buffered on the
// copy stream against relaxation on the compute stream.
int process_iteration(sgw_engine *e) {
  const uint32_t P = e->num_parts;
  if (P == 0) return SGW_OK;
  TRY(enqueue_gather(e, 0, e->s_copy));
  for (uint32_t p = 0; p < P; ++p) {
    const Part &q = e->h_parts[p];
    const uint32_t b = p % e->nbuf;
    if (e->nbuf > 1 && p + 1 < P) TRY(enqueue_gather(e, p + 1, e->s_copy));
    uint32_t inner = 1;
    if (is_hub(e, q)) {
      TRY(process_hub(e, q, b));
    } else {
      CK(cudaStreamWaitEvent(e->s_comp, e->ev_ready[b], 0));
      TRY(process_resident(e, q, b, &inner));
    }
    CK(cudaEventRecord(e->ev_free[b], e->s_comp));
    trace_partition(e, p, inner);
    if (e->nbuf == 1 && p + 1 < P) TRY(enqueue_gather(e, p + 1, e->s_copy));
    e->stats.partitions += 1;
  }
  return SGW_OK;
}

// ---- learned policy ------------------------------------------------------------
// generate + per-range statistics and predictions + one read-back.
int generate_and_stats(sgw_engine *e, int consume) {
  TRY(launch_generate(e, consume));
  const uint32_t S = (uint32_t)e->ranges.size();
  const __nv_bfloat16 *w = e->have_model ? e->d_mlp : nullptr;
  size_t slot = 0;
  TRY(prof_begin(e, K_PLAN, e->s_comp, &slot));
  k_range_stats<<<(S * 32 + 255) / 256, 256, 0, e->s_comp>>>(
      e->d_ranges, S, e->d_queue, e->d_ptr, e->d_ctl, e->d_rstat, w, e->gitr + 1,
      (uint32_t)std::min<uint64_t>(e->cap, 0xffffffffull));
  CK(cudaGetLastError());
  TRY(prof_end(e, e->s_comp, slot));
  e->stats.launches += 1;
  CK(cudaMemcpyAsync(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->s_comp));
  CK(cudaMemcpyAsync(e->h_rstat, e->d_rstat, sizeof(RangeStat) * S, cudaMemcpyDeviceToHost, e->s_comp));
  CK(cudaStreamSynchronize(e->s_comp));
  TRY(check_ctl_error(e));
  e->num_active = e->h_ctl->num_active;
  e->num_active_edges = e->h_ctl->num_active_edges;
  e->stats.d2h_bytes += sizeof(Ctl) + sizeof(RangeStat) * S;
  e->parts_valid = false;
  return SGW_OK;
}

struct Job {
  uint32_t s;       // first range
  uint32_t s_end;   // one past the last range (consecutive compacted ranges merge)
  uint32_t action;  // SGW_ACT_*
  Part part;        // the queue segment relaxed
  int buf = -1;     // buffer it is processed from
  bool ready = false;
};

Part range_part(const RangeStat &st) {
  Part q;
  q.from = st.qa;
  q.size = st.qb - st.qa;
  q.edge_from = st.edge_from;
  q.first_vertex = st.first_vertex;
  q.edge_count = st.act_edges;
  return q;
}

// Enqueues job j's transfer into buffer b on the copy stream.
int range_transfer(sgw_engine *e, Job &j, int b) {
  const RangeInfo &r = e->ranges[j.s];
  if (j.action == SGW_ACT_STREAM) {
    const size_t esz = 4ull * e->W;
    const size_t bytes = (size_t)(r.e1 - r.e0) * esz;
    CK(cudaStreamWaitEvent(e->s_copy, e->ev_free[b], 0));
    size_t slot = 0;
    TRY(prof_begin(e, K_STREAM, e->s_copy, &slot));
    e->stream_bytes += bytes + (e->use_w ? (size_t)(r.e1 - r.e0) : 0);
    // a whole range is contiguous: one DMA copy, no SM time taken from the
    // relaxation running on the compute stream
    TRY(copy_from_host(e->hs_ends, e->d_buf[b], (size_t)r.e0 * esz, bytes, e->s_copy));
    if (e->use_w) {
      TRY(copy_from_host(e->hs_w, e->d_wbuf[b], r.e0, (size_t)(r.e1 - r.e0), e->s_copy));
      e->stats.h2d_bytes += (size_t)(r.e1 - r.e0);
    }
    TRY(prof_end(e, e->s_copy, slot));
    CK(cudaEventRecord(e->ev_ready[b], e->s_copy));
    e->stats.h2d_bytes += bytes;
    e->buf_range[b] = (int)j.s;
  } else {
    TRY(gather_into(e, j.part, (uint32_t)b, e->s_copy));
    e->buf_range[b] = -1;
  }
  j.buf = b;
  j.ready = true;
  return SGW_OK;
}

// All active ranges of one global iteration under the learned policy.
int process_iteration_ranges(sgw_engine *e) {
  const uint32_t S = (uint32_t)e->ranges.size();
  const uint32_t esz = 4 * e->W + (e->use_w ? 1 : 0);  // bytes moved per edge
  std::vector<int> held(S, -1);
  for (uint32_t b = 0; b < e->nbuf; ++b)
    if (e->buf_range[b] >= 0) held[e->buf_range[b]] = (int)b;
  std::vector<Job> jobs;
  std::vector<uint32_t> act(S, SGW_ACT_SKIP);
  for (uint32_t s = 0; s < S; ++s) {  // resident ranges first: no transfer to wait for
    const RangeStat &st = e->h_rstat[s];
    if (st.qb > st.qa && held[s] >= 0) {
      Job j;
      j.s = s;
      j.s_end = s + 1;
      j.action = act[s] = SGW_ACT_RESIDENT;
      j.part = range_part(st);
      j.buf = held[s];
      j.ready = true;
      jobs.push_back(j);
    }
  }
  // Streaming a whole range pays E - A extra bytes now and saves the next
  // iteration's transfer (predicted p * E) only if the range then is still
  // in a buffer.  Two buffers keep the transfer/relax pipeline going, so at
  // most num_buffers - 2 ranges can stay: stream the ranges with the largest
  // predicted net saving, up to that many; send the others compacted.
  std::vector<std::pair<double, uint32_t>> stream_cand;
  for (uint32_t s = 0; s < S; ++s) {
    const RangeStat &st = e->h_rstat[s];
    if (st.qb <= st.qa || held[s] >= 0) continue;
    const RangeInfo &r = e->ranges[s];
    const double E = (double)(r.e1 - r.e0), A = (double)st.act_edges;
    if (E > (double)e->cap) act[s] = SGW_ACT_SPLIT;
    else if (E - A <= (double)st.pred * E) {
      act[s] = SGW_ACT_STREAM;
      stream_cand.push_back({(double)st.pred * E - (E - A), s});
    } else {
      act[s] = SGW_ACT_COMPACT;
    }
  }
  const bool dma_ok = e->dma_gbs < 0.0 || e->dma_gbs >= kMinStreamGBs;
  const size_t keep_slots = (e->nbuf > 2 && dma_ok) ? e->nbuf - 2 : 0;
  if (stream_cand.size() > keep_slots) {
    std::sort(stream_cand.begin(), stream_cand.end(),
              [](const std::pair<double, uint32_t> &x, const std::pair<double, uint32_t> &y) {
                return x.first > y.first || (x.first == y.first && x.second < y.second);
              });
    for (size_t k = keep_slots; k < stream_cand.size(); ++k) act[stream_cand[k].second] = SGW_ACT_COMPACT;
  }
  long open_compact = -1;  // job that the next compacted range may join
  for (uint32_t s = 0; s < S; ++s) {
    const RangeStat &st = e->h_rstat[s];
    if (st.qb <= st.qa || held[s] >= 0) continue;
    const uint32_t action = act[s];
    if (action == SGW_ACT_COMPACT && open_compact >= 0) {
      // compacted ranges whose queue segments touch share one gather and
      // one relaxation, up to a buffer of active edges (as plain partitions)
      Part &q = jobs[(size_t)open_compact].part;
      if (q.from + q.size == st.qa && q.edge_count + st.act_edges <= e->cap) {
        q.size = st.qb - q.from;
        q.edge_count += st.act_edges;
        jobs[(size_t)open_compact].s_end = s + 1;
        continue;
      }
    }
    Job j;
    j.s = s;
    j.s_end = s + 1;
    j.action = action;
    j.part = range_part(st);
    jobs.push_back(j);
    open_compact = action == SGW_ACT_COMPACT ? (long)jobs.size() - 1 : -1;
  }
  // keep value of a buffer: predicted bytes it saves next iteration
  auto value = [&](uint32_t b) -> double {
    const int r = e->buf_range[b];
    if (r < 0) return -1.0;
    return (double)e->h_rstat[r].pred * (double)(e->ranges[r].e1 - e->ranges[r].e0);
  };
  // a victim is not used by any job not yet enqueued and is not `exclude`
  auto victim = [&](size_t from_job, int exclude) -> int {
    int best = -1;
    for (uint32_t b = 0; b < e->nbuf; ++b) {
      if ((int)b == exclude) continue;
      bool used = false;
      for (size_t k = from_job; k < jobs.size() && !used; ++k) used = jobs[k].buf == (int)b;
      if (used) continue;
      if (best < 0 || value(b) < value((uint32_t)best)) best = (int)b;
    }
    return best;
  };
  std::vector<uint32_t> inner_of(S, 0);
  for (size_t k = 0; k < jobs.size(); ++k) {
    Job &j = jobs[k];
    if (!j.ready && j.action != SGW_ACT_SPLIT) {
      const int b = victim(k, -1);
      if (b < 0) return fail(SGW_ESTATE, "no edge buffer free");
      TRY(range_transfer(e, j, b));
    }
    if (k + 1 < jobs.size()) {  // prefetch the next transfer behind this relaxation
      Job &nx = jobs[k + 1];
      if (!nx.ready && nx.action != SGW_ACT_SPLIT) {
        const int b = victim(k + 1, j.buf);
        if (b >= 0) TRY(range_transfer(e, nx, b));
      }
    }
    const RangeInfo &r = e->ranges[j.s];
    const Part q = j.part;
    uint32_t inner = 1;
    if (j.action == SGW_ACT_SPLIT) {
      const int b = victim(k, -1);
      if (b < 0) return fail(SGW_ESTATE, "no edge buffer free");
      j.buf = b;
      e->buf_range[b] = -1;
      CK(cudaStreamWaitEvent(e->s_comp, e->ev_free[b], 0));
      TRY(process_hub(e, q, (uint32_t)b));
    } else {
      CK(cudaStreamWaitEvent(e->s_comp, e->ev_ready[j.buf], 0));
      e->cur_streamed = (j.action == SGW_ACT_RESIDENT || j.action == SGW_ACT_STREAM) ? 1u : 0u;
      e->cur_stream_base = r.e0;
      // a range that stays in its buffer and is predicted to be active again
      // next iteration stops early: what further inner passes would settle
      // is likely to be redone then, and its leftover sources cost no bytes
      const double thr = (e->opts.sched_active_permille ? e->opts.sched_active_permille : 1u) / 1000.0;
      const bool kept = j.action == SGW_ACT_RESIDENT || j.action == SGW_ACT_STREAM;
      float pred = 0.0f;
      for (uint32_t s = j.s; s < j.s_end; ++s) pred = std::max(pred, e->h_rstat[s].pred);
      const bool cappable = kept || (e->opts.sched_flags & SGW_SCHED_CAP_COMPACT);
      e->range_inner_cap = cappable && (double)pred >= thr ? (e->opts.sched_inner ? e->opts.sched_inner : 3u) : 0u;
      const int st = process_resident(e, q, (uint32_t)j.buf, &inner);
      e->cur_streamed = 0;
      e->range_inner_cap = 0;
      TRY(st);
    }
    CK(cudaEventRecord(e->ev_free[j.buf], e->s_comp));
    for (uint32_t s = j.s; s < j.s_end; ++s) inner_of[s] = inner;
    e->stats.partitions += 1;
  }
  if (e->trace_on) {
    for (uint32_t s = 0; s < S; ++s) {
      const RangeStat &st = e->h_rstat[s];
      const RangeInfo &r = e->ranges[s];
      sgw_range_rec rec;
      memset(&rec, 0, sizeof(rec));
      rec.global_iteration = e->gitr;
      rec.range = s;
      rec.active_nodes = st.qb - st.qa;
      rec.range_nodes = r.v1 - r.v0;
      rec.active_edges = st.act_edges;
      rec.range_edges = r.e1 - r.e0;
      rec.action = act[s];
      rec.inner_iterations = inner_of[s];
      for (int f = 0; f < 5; ++f) rec.features[f] = st.feat[f];
      rec.predicted = st.pred;
      rec.bytes_h2d = act[s] == SGW_ACT_STREAM ? (uint64_t)(r.e1 - r.e0) * esz
                      : act[s] == SGW_ACT_COMPACT || act[s] == SGW_ACT_SPLIT ? (uint64_t)st.act_edges * esz : 0;
      e->rtrace.push_back(rec);
    }
  }
  return SGW_OK;
}

}  // namespace

extern "C" {

void sgw_engine_opts_default(sgw_engine_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->budget_bytes = 0;
  o->device = 0;
  o->flags = 0;
  o->inner_batch = 8;
  o->tile_degree_max = 256;
  o->chunk_edges = 1024;
  o->sched_inner = 3;
  o->sched_active_permille = 1;
  o->sched_flags = SGW_SCHED_CAP_COMPACT;
}

void sgw_run_params_default(sgw_run_params *p, int algo, int mode, uint32_t source) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->algo = algo;
  p->mode = mode;
  p->source = source;
  p->pr_init = 0.15f;
  p->pr_acc = 0.01f;
  p->pr_damping = 0.85f;
  p->max_inner = 0;
}

int sgw_device_info(int device, uint32_t *sm_count, uint64_t *total_bytes) {
  clear_error();
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  if (sm_count) *sm_count = (uint32_t)prop.multiProcessorCount;
  if (total_bytes) *total_bytes = (uint64_t)prop.totalGlobalMem;
  return SGW_OK;
}

int sgw_device_count(int *count) {
  if (!count) return fail(SGW_EINVAL, "null argument");
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess) c = 0;
  cudaGetLastError();
  *count = c;
  return SGW_OK;
}

int sgw_probe_link(int device, uint64_t bytes, int iters, double *h2d_gbs, double *d2h_gbs) {
  clear_error();
  if (bytes == 0 || iters <= 0) return fail(SGW_EINVAL, "bad probe size");
  CK(cudaSetDevice(device));
  void *h = nullptr, *d = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  int st = SGW_OK;
  double best_h2d = 0, best_d2h = 0;
  if (cudaMallocHost(&h, bytes) != cudaSuccess || cudaMalloc(&d, bytes) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    st = fail(SGW_ECUDA, "probe allocation");
  } else {
    memset(h, 1, bytes);
    for (int dir = 0; dir < 2 && st == SGW_OK; ++dir) {
      for (int i = 0; i <= iters; ++i) {  // first copy warms up
        cudaEventRecord(a, s);
        if (dir == 0) cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s);
        else cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s);
        cudaEventRecord(b, s);
        if (cudaEventSynchronize(b) != cudaSuccess) { st = fail(SGW_ECUDA, "probe copy"); break; }
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        double gbs = (double)bytes / (ms * 1e6);
        if (i > 0) {
          if (dir == 0) best_h2d = std::max(best_h2d, gbs);
          else best_d2h = std::max(best_d2h, gbs);
        }
      }
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (s) cudaStreamDestroy(s);
  if (d) cudaFree(d);
  if (h) cudaFreeHost(h);
  cudaGetLastError();
  if (h2d_gbs) *h2d_gbs = best_h2d;
  if (d2h_gbs) *d2h_gbs = best_d2h;
  return st;
}

int sgw_engine_create(const sgw_graph *g, const sgw_engine_opts *opts_in, sgw_engine **out) {
  clear_error();
  if (!g || !out) return fail(SGW_EINVAL, "null argument");
  *out = nullptr;
  sgw_engine_opts o;
  sgw_engine_opts_default(&o);
  if (opts_in) o = *opts_in;
  if (o.inner_batch == 0) o.inner_batch = 8;
  if (o.tile_degree_max == 0) o.tile_degree_max = 256;
  if (o.chunk_edges == 0) o.chunk_edges = 1024;
  if (o.chunk_edges % 32) return fail(SGW_EINVAL, "chunk_edges must be a multiple of 32");
  if (g->weighted && (((uintptr_t)g->edges) & 7u)) return fail(SGW_EINVAL, "edges must be 8-byte aligned");
  if (g->n >= 0x80000000u) return fail(SGW_ERANGE, "vertex count %u above 2^31", g->n);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(SGW_ECUDA, "no CUDA device");
  }
  if (o.device < 0 || o.device >= ndev) return fail(SGW_EINVAL, "device %d out of range", o.device);
  CK(cudaSetDevice(o.device));

  sgw_engine *e = new (std::nothrow) sgw_engine();
  if (!e) return fail(SGW_ENOMEM, "engine object");
  e->g = g;
  e->device = o.device;
  e->opts = o;
  e->n = g->n;
  e->m = g->m;
  e->W = g->weighted ? 2 : 1;
  e->wide = g->node_pointer64 != nullptr;
  {
    // queue positions are u32: at 2^32 edges and more a generate queues at
    // most 2^31 edges, whole tiles of fewer than 2^31 edges each
    const bool big = g->m >= (uint64_t(1) << 32);
    uint64_t lim = o.generate_edge_limit ? o.generate_edge_limit : (big ? uint64_t(1) << 31 : 0);
    if (big) lim = std::min<uint64_t>(lim, uint64_t(1) << 31);
    e->edge_limit = (uint32_t)lim;
    const uint32_t n = g->n;
    int over = 0;
    if (big) {
#pragma omp parallel for reduction(| : over)
      for (int64_t t = 0; t < (int64_t)((n + kGenTile - 1) / kGenTile); ++t) {
        const uint64_t v0 = (uint64_t)t * kGenTile, v1 = std::min<uint64_t>(n, v0 + kGenTile);
        if (np_at(g, v1) - np_at(g, v0) >= (uint64_t(1) << 31)) over |= 1;
      }
    }
    if (over) {
      delete e;
      return fail(SGW_ERANGE, "a 4096-vertex tile holds 2^31 edges or more");
    }
  }
  // whether the device reads pageable memory through the host page tables
  bool pageable_ok = false;
  if (o.flags & (SGW_OPT_PAGEABLE_COPY | SGW_OPT_GRAPH_IN_PLACE)) {
    int pma = 0, hpt = 0;
    pageable_ok = cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, o.device) == cudaSuccess &&
                  cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, o.device) ==
                      cudaSuccess && pma && hpt;
    cudaGetLastError();
  }
  // In place: records the library itself holds in anonymous memory (loaded
  // or generated; 64 KiB aligned and rounded up, so the 16-byte words the
  // gather reads past the last record stay inside the allocation).  File
  // mappings and caller arrays get a transfer copy.
  {
    const size_t rec_bytes = size_t(g->m) * g->esz;
    e->in_place = (o.flags & SGW_OPT_GRAPH_IN_PLACE) && pageable_ok && g->owns && !g->map_base && g->m > 0 &&
                  ((uintptr_t)g->edges & 15u) == 0 && g->edges_bytes_alloc >= rec_bytes + 16;
  }
  // weighted records travel as one packed word when (w << bits(n)) | dst fits
  const uint32_t wmax = max_weight(g);  // one pass over the records
  bool pack = !e->in_place && g->weighted && !(o.flags & (SGW_OPT_NO_PACK | SGW_OPT_SPLIT_WEIGHTS)) &&
              pack_bits_for(g, wmax, &e->pbits);
  if (pack) e->W = 1;
  else e->pbits = 0;
  // otherwise weights below 256 travel as their own byte stream
  e->split = !e->in_place && g->weighted && !pack && !(o.flags & (SGW_OPT_NO_PACK | SGW_OPT_SCALAR_GATHER)) &&
             wmax < 256;
  if (e->split) e->W = 1;
  e->rec_bytes = 4 * e->W + (e->split ? 1 : 0);
  e->nbuf = (o.flags & SGW_OPT_NO_OVERLAP) ? 1 : 2;
  if (o.num_buffers) {
    if (o.num_buffers > (uint32_t)kMaxBuf) { delete e; return fail(SGW_EINVAL, "num_buffers above %d", kMaxBuf); }
    e->nbuf = o.num_buffers;
  }
  e->num_tiles = (uint32_t)((g->n + kGenTile - 1) / kGenTile);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, o.device) != cudaSuccess) { delete e; return fail(SGW_ECUDA, "device properties"); }
  e->num_sms = prop.multiProcessorCount;

  const uint32_t esz = e->rec_bytes;
  // The arena never exceeds what holds the whole graph in both buffers.
  const uint64_t mfull = std::max<uint64_t>(e->m, 64);
  size_t need = 0;
  for (int fam = 0; fam < 2; ++fam)
    need = std::max(need, make_layout(fam, e->n, e->m, esz, e->nbuf, e->num_tiles, mfull,
                                      o.chunk_edges, o.tile_degree_max, e->wide).total);
  uint64_t budget = o.budget_bytes;
  if (budget == 0) {
    // Subway's rule: 0.9 * (totalGlobalMem - 32 n) bytes of edges
    // (shared/subgraph.cu:24), here on top of the engine's own vertex state.
    const Layout L0 = make_layout(FAM_PR, e->n, e->m, esz, e->nbuf, e->num_tiles, mfull,
                                  o.chunk_edges, o.tile_degree_max, e->wide);
    const double state = (double)L0.total - (double)e->nbuf * mfull * esz;  // all but the buffers
    double edges_bytes = 0.9 * ((double)prop.totalGlobalMem - 32.0 * e->n);
    budget = (uint64_t)(state + std::max(0.0, edges_bytes));
  }
  const size_t arena = (size_t)std::min<uint64_t>(budget, need);
  for (int fam = 0; fam < 2; ++fam) {
    e->cap_fam[fam] = fit_cap(fam, o, e->n, e->m, esz, e->nbuf, e->num_tiles, arena, e->wide);
    // split form: the weight bytes start at 4 * cap past a 256-byte aligned
    // buffer; a multiple of 4 keeps them 16-byte aligned for vector stores
    if (e->split && e->cap_fam[fam] > 16) e->cap_fam[fam] &= ~3ull;
  }
  if (e->cap_fam[FAM_INT] == 0) {
    const Layout L0 = make_layout(FAM_INT, e->n, e->m, esz, e->nbuf, e->num_tiles, 4096,
                                  o.chunk_edges, o.tile_degree_max, e->wide);
    delete e;
    return fail(SGW_EBUDGET, "budget %llu B < vertex state and minimum edge buffers (about %zu B)",
                (unsigned long long)budget, L0.total);
  }
  e->budget = budget;
  cudaError_t ce = cudaMalloc(&e->d_arena, arena);
  if (ce != cudaSuccess) {
    delete e;
    return fail(SGW_ECUDA, "cudaMalloc(%zu): %s", arena, cudaGetErrorString(ce));
  }
  e->arena_bytes = arena;
  carve(e, FAM_INT, e->cap_fam[FAM_INT]);
  uint32_t parts_host = 0;
  for (int fam = 0; fam < 2; ++fam)
    if (e->cap_fam[fam])
      parts_host = std::max(parts_host, make_layout(fam, e->n, e->m, esz, e->nbuf, e->num_tiles,
                                                    e->cap_fam[fam], o.chunk_edges, o.tile_degree_max, e->wide).max_parts);

  int st = SGW_OK;
  auto cleanup = [&](int s) { sgw_engine_destroy(e); return s; };
  // The transfer copy: the edge records (packed when they fit) in pinned,
  // mapped host memory from cudaHostAlloc, read in place by the gather
  // kernels and by DMA copies, in chunks (HostStream) so that two host
  // threads can allocate it at once; with SGW_OPT_PAGEABLE_COPY (where the
  // device reads pageable memory through the host page tables) in ordinary
  // pages instead, which the filling threads touch first and the kernels read
  // at their host addresses.  On a GB300 host the 21 GB copy of RMAT-28 took
  // 1.0-1.08 s to create pinned and 0.47-0.58 s pageable; the plain
  // schedule's runs took the same time from either (271 ms), the learned
  // schedule's 4% longer from pageable pages (166 against 160 ms).
  if (g->m > 0 && e->in_place) {  // one borrowed chunk: the graph's records
    HostStream &hs = e->hs_ends;
    hs.bytes = (size_t)e->m * g->esz;
    hs.shift = 62;
    hs.h.assign(1, static_cast<char *>(g->edges));
    hs.d.assign(1, 0);
    hs.size.assign(1, g->edges_bytes_alloc);
    hs.pageable = hs.borrowed = true;
    e->packed_bytes = 0;
  } else if (g->m > 0) {
    const size_t rec = 4ull * e->W;  // bytes per record in the ends stream
    if (o.transfer_chunk_log2 > 40) return cleanup(fail(SGW_EINVAL, "transfer_chunk_log2 above 40"));
    plan_stream(e->hs_ends, (size_t)e->m * rec, o.transfer_chunk_log2);
    if (e->split) plan_stream(e->hs_w, (size_t)e->m, o.transfer_chunk_log2);
    e->hs_ends.pageable = e->hs_w.pageable = (o.flags & SGW_OPT_PAGEABLE_COPY) && pageable_ok;
    e->packed_bytes = e->hs_ends.bytes + e->hs_w.bytes;
    HostStream *ends = &e->hs_ends;
    ce = alloc_and_fill(e->hs_ends, e->hs_w, [&](HostStream &hs, size_t k) {
      const size_t cb = size_t(1) << hs.shift;
      if (&hs == ends) {  // edge words (packed, split-form destinations or records)
        const uint64_t e0 = std::min<uint64_t>(e->m, (uint64_t)(k * cb / rec));
        const uint64_t e1 = std::min<uint64_t>(e->m, (uint64_t)((k + 1) * cb / rec));
        char *dst = hs.h[k];
        if (pack) pack_range(g, e->pbits, (uint32_t *)dst, e0, e1);
        else if (e->split) split_ends_range(g, (uint32_t *)dst, e0, e1);
        else copy_records_range(g, dst, e0, e1);
        const size_t used = (size_t)(e1 - e0) * rec;
        memset(dst + used, 0, hs.size[k] - used);
      } else {  // split form: weight bytes
        const uint64_t e0 = std::min<uint64_t>(e->m, (uint64_t)(k * cb));
        const uint64_t e1 = std::min<uint64_t>(e->m, (uint64_t)((k + 1) * cb));
        split_weights_range(g, (uint8_t *)hs.h[k], e0, e1);
        memset(hs.h[k] + (e1 - e0), 0, hs.size[k] - (size_t)(e1 - e0));
      }
    });
    if (ce != cudaSuccess) {
      cudaGetLastError();
      return cleanup(fail(SGW_ECUDA, "cudaHostAlloc of the %zu-byte transfer copy: %s", e->packed_bytes,
                          cudaGetErrorString(ce)));
    }
  }
  if (g->m > 0) {  // chunk tables: device addresses (pageable and borrowed chunks: the host address)
    unsigned long long table[2 * kMaxHostChunks] = {};
    HostStream *streams[2] = {&e->hs_ends, &e->hs_w};
    for (int t = 0; t < 2; ++t)
      for (size_t k = 0; k < streams[t]->h.size(); ++k) {
        void *dp = streams[t]->h[k];  // pageable: the device uses the host address
        if (!streams[t]->pageable) ce = cudaHostGetDevicePointer(&dp, streams[t]->h[k], 0);
        if (ce != cudaSuccess) {
          cudaGetLastError();
          return cleanup(fail(SGW_ECUDA, "cudaHostGetDevicePointer: %s", cudaGetErrorString(ce)));
        }
        streams[t]->d[k] = (unsigned long long)(uintptr_t)dp;
        table[t * kMaxHostChunks + k] = streams[t]->d[k];
      }
    ce = cudaMemcpy(e->d_hct, table, sizeof(table), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) return cleanup(fail(SGW_ECUDA, "chunk table upload: %s", cudaGetErrorString(ce)));
    e->hs_ends.dtab = e->d_hct;
    e->hs_w.dtab = e->d_hct + kMaxHostChunks;
  }
  e->vec_gather = !(o.flags & SGW_OPT_SCALAR_GATHER) && !e->hs_ends.h.empty();
  if (!allow_gather_smem<false>(kGatherSmemBytes) || !allow_gather_smem<true>(kGatherSmemBytesWide)) {
    cudaGetLastError();
    return cleanup(fail(SGW_ECUDA, "gather shared memory of %zu bytes refused", kGatherSmemBytesWide));
  }
  if (cudaStreamCreateWithFlags(&e->s_comp, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e->s_copy, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup(fail(SGW_ECUDA, "stream creation"));
  for (int i = 0; i < kMaxBuf; ++i) {
    if (cudaEventCreateWithFlags(&e->ev_ready[i], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->ev_free[i], cudaEventDisableTiming) != cudaSuccess)
      return cleanup(fail(SGW_ECUDA, "event creation"));
  }
  if (cudaEventCreate(&e->ev_t0) != cudaSuccess || cudaEventCreate(&e->ev_t1) != cudaSuccess)
    return cleanup(fail(SGW_ECUDA, "event creation"));
  if (cudaMallocHost(&e->h_ctl, sizeof(Ctl)) != cudaSuccess ||
      cudaMallocHost(&e->h_parts, sizeof(Part) * (size_t)parts_host) != cudaSuccess ||
      cudaMallocHost(&e->h_rstat, sizeof(RangeStat) * (size_t)parts_host) != cudaSuccess)
    return cleanup(fail(SGW_ECUDA, "pinned control block"));
  memset(e->h_ctl, 0, sizeof(Ctl));
  if (!e->wide) {
    ce = cudaMemcpyAsync(e->d_off, g->node_pointer, 4ull * (e->n + 1), cudaMemcpyHostToDevice, e->s_comp);
  } else {  // low words of every node pointer, full pointers of every group start
    std::vector<uint32_t> lo((size_t)e->n + 1);
    std::vector<unsigned long long> base((e->n >> kOffGroupLog2) + 2);
    if (!device_offsets(g, lo.data(), base.data()))
      return cleanup(fail(SGW_ERANGE, "1024 consecutive vertices hold 2^32 edges or more"));
    ce = cudaMemcpy(e->d_off, lo.data(), 4 * lo.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(e->d_obase, base.data(), 8 * base.size(), cudaMemcpyHostToDevice);
  }
  if (ce == cudaSuccess) ce = cudaMemsetAsync(e->d_ctl, 0, sizeof(Ctl), e->s_comp);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(e->d_tflag, 0, 4ull * e->num_tiles, e->s_comp);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->s_comp);
  if (ce != cudaSuccess) return cleanup(fail(SGW_ECUDA, "engine setup copies: %s", cudaGetErrorString(ce)));
  st = probe_stream_dma(e);
  if (st != SGW_OK) return cleanup(st);
  *out = e;
  return SGW_OK;
}

int sgw_engine_destroy(sgw_engine *e) {
  if (!e) return SGW_OK;
  cudaSetDevice(e->device);
  if (e->s_comp) cudaStreamSynchronize(e->s_comp);
  if (e->s_copy) cudaStreamSynchronize(e->s_copy);
  for (auto &pe : e->prof) { cudaEventDestroy(pe.a); cudaEventDestroy(pe.b); }
  for (int i = 0; i < kMaxBuf; ++i) {
    if (e->ev_ready[i]) cudaEventDestroy(e->ev_ready[i]);
    if (e->ev_free[i]) cudaEventDestroy(e->ev_free[i]);
  }
  if (e->h_rstat) cudaFreeHost(e->h_rstat);
  if (e->ev_t0) cudaEventDestroy(e->ev_t0);
  if (e->ev_t1) cudaEventDestroy(e->ev_t1);
  if (e->s_comp) cudaStreamDestroy(e->s_comp);
  if (e->s_copy) cudaStreamDestroy(e->s_copy);
  if (e->h_ctl) cudaFreeHost(e->h_ctl);
  if (e->h_parts) cudaFreeHost(e->h_parts);
  free_streams(e->hs_ends, e->hs_w);
  if (e->d_arena) cudaFree(e->d_arena);
  cudaGetLastError();
  delete e;
  return SGW_OK;
}

int sgw_engine_max_partition_size(const sgw_engine *e, uint64_t *edges) {
  if (!e || !edges) return fail(SGW_EINVAL, "null argument");
  *edges = e->cap;
  return SGW_OK;
}

int sgw_engine_host_copy_bytes(const sgw_engine *e, uint64_t *bytes) {
  if (!e || !bytes) return fail(SGW_EINVAL, "null argument");
  *bytes = e->packed_bytes;
  return SGW_OK;
}

int sgw_engine_device_bytes(const sgw_engine *e, uint64_t *bytes) {
  if (!e || !bytes) return fail(SGW_EINVAL, "null argument");
  *bytes = e->arena_bytes;
  return SGW_OK;
}

int sgw_state_init(sgw_engine *e, const sgw_run_params *p) {
  clear_error();
  if (!e) return fail(SGW_EINVAL, "null engine");
  return state_init(e, p);
}

int sgw_generate(sgw_engine *e, uint32_t *num_active_nodes, uint64_t *num_active_edges) {
  clear_error();
  if (!e || !e->initialized) return fail(SGW_ESTATE, "engine not initialised");
  CK(cudaSetDevice(e->device));
  TRY(launch_generate(e, e->params.mode == SGW_SYNC ? 1 : 0));
  TRY(read_ctl(e));
  e->num_active = e->h_ctl->num_active;
  e->num_active_edges = e->h_ctl->num_active_edges;
  if (num_active_nodes) *num_active_nodes = e->num_active;
  if (num_active_edges) *num_active_edges = e->num_active_edges;
  return SGW_OK;
}

int sgw_partition(sgw_engine *e, uint32_t *num_partitions) {
  clear_error();
  if (!e || !e->initialized) return fail(SGW_ESTATE, "engine not initialised");
  CK(cudaSetDevice(e->device));
  TRY(launch_plan(e));
  TRY(read_ctl(e));
  e->num_parts = e->h_ctl->num_parts;
  if (e->num_parts) {
    CK(cudaMemcpyAsync(e->h_parts, e->d_parts, sizeof(Part) * e->num_parts, cudaMemcpyDeviceToHost, e->s_comp));
    CK(cudaStreamSynchronize(e->s_comp));
  }
  e->parts_valid = true;
  if (num_partitions) *num_partitions = e->num_parts;
  return SGW_OK;
}

int sgw_partition_info(const sgw_engine *e, uint32_t i, uint32_t *from_node, uint32_t *from_edge,
                       uint32_t *node_size, uint64_t *edge_size) {
  if (!e || !e->parts_valid) return fail(SGW_ESTATE, "no partition table");
  if (i >= e->num_parts) return fail(SGW_EINVAL, "partition %u out of range", i);
  const Part &q = e->h_parts[i];
  if (from_node) *from_node = q.from;
  if (from_edge) *from_edge = q.edge_from;
  if (node_size) *node_size = q.size;
  if (edge_size) *edge_size = q.edge_count;
  return SGW_OK;
}

int sgw_process_partition(sgw_engine *e, uint32_t i, uint32_t *inner_iterations) {
  clear_error();
  if (!e || !e->initialized || !e->parts_valid) return fail(SGW_ESTATE, "no partition table");
  if (i >= e->num_parts) return fail(SGW_EINVAL, "partition %u out of range", i);
  CK(cudaSetDevice(e->device));
  const Part &q = e->h_parts[i];
  uint32_t iters = 1;
  if (is_hub(e, q)) {
    TRY(process_hub(e, q, 0));
  } else {
    TRY(enqueue_gather(e, i, e->s_comp));
    TRY(process_resident(e, q, i % e->nbuf, &iters));
  }
  CK(cudaStreamSynchronize(e->s_comp));
  TRY(read_ctl(e));
  e->stats.partitions += 1;
  if (i == 0) e->gitr += 1;
  trace_partition(e, i, iters);
  if (inner_iterations) *inner_iterations = iters;
  return SGW_OK;
}

int sgw_engine_dma_rate(const sgw_engine *e, double *gbs) {
  if (!e || !gbs) return fail(SGW_EINVAL, "null argument");
  *gbs = e->dma_gbs;
  return SGW_OK;
}

int sgw_sched_buffers(const sgw_graph *g, uint64_t budget_bytes, uint32_t *num_buffers) {
  clear_error();
  if (!g || !num_buffers) return fail(SGW_EINVAL, "null argument");
  uint32_t bits = 0;
  const double rec = !g->weighted || pack_bits(g, &bits) ? 4.0 : (max_weight(g) < 256 ? 5.0 : 8.0);
  const double space = (double)budget_bytes - 18.0 * (double)g->n;  // integer vertex state
  const double third = space > 0 ? space / 3.0 / rec : 0.0;
  *num_buffers = (g->m > 0 && third >= 0.15 * (double)g->m) ? 3u : 2u;
  return SGW_OK;
}

int sgw_set_policy(sgw_engine *e, int policy, const sgw_mlp *model) {
  clear_error();
  if (!e) return fail(SGW_EINVAL, "null engine");
  if (policy != SGW_POLICY_PLAIN && policy != SGW_POLICY_LEARNED)
    return fail(SGW_EINVAL, "unknown policy %d", policy);
  CK(cudaSetDevice(e->device));
  if (model) {
    if (mlp_device(model) != e->device) return fail(SGW_EINVAL, "model lives on another device");
    CK(cudaMemcpy(e->d_mlp, mlp_device_weights(model), sizeof(__nv_bfloat16) * kMlpParams,
                  cudaMemcpyDeviceToDevice));
  }
  e->have_model = model != nullptr;
  e->policy = policy;
  e->initialized = false;  // the step API restarts from sgw_state_init
  return SGW_OK;
}

int sgw_range_trace_count(const sgw_engine *e, uint64_t *count) {
  if (!e || !count) return fail(SGW_EINVAL, "null argument");
  *count = e->rtrace.size();
  return SGW_OK;
}

int sgw_range_trace_read(const sgw_engine *e, sgw_range_rec *out, uint64_t capacity, uint64_t *count) {
  if (!e || !count) return fail(SGW_EINVAL, "null argument");
  const uint64_t k = std::min<uint64_t>(capacity, e->rtrace.size());
  if (out && k) memcpy(out, e->rtrace.data(), k * sizeof(sgw_range_rec));
  *count = k;
  return SGW_OK;
}

int sgw_trace_enable(sgw_engine *e, int on) {
  if (!e) return fail(SGW_EINVAL, "null engine");
  e->trace_on = on != 0;
  return SGW_OK;
}

int sgw_trace_count(const sgw_engine *e, uint64_t *count) {
  if (!e || !count) return fail(SGW_EINVAL, "null argument");
  *count = e->trace.size();
  return SGW_OK;
}

int sgw_trace_read(const sgw_engine *e, sgw_trace_rec *out, uint64_t capacity, uint64_t *count) {
  if (!e || !count) return fail(SGW_EINVAL, "null argument");
  uint64_t k = std::min<uint64_t>(capacity, e->trace.size());
  if (out && k) memcpy(out, e->trace.data(), k * sizeof(sgw_trace_rec));
  *count = k;
  return SGW_OK;
}

int sgw_trace_save(const sgw_engine *e, const char *path) {
  if (!e) return fail(SGW_EINVAL, "null engine");
  return sgw_trace_write_csv(e->trace.data(), e->trace.size(), path);
}

int sgw_read_values(sgw_engine *e, void *out_values) {
  clear_error();
  if (!e || !out_values) return fail(SGW_EINVAL, "null argument");
  if (!e->initialized) return fail(SGW_ESTATE, "engine not initialised");
  CK(cudaSetDevice(e->device));
  if (e->fam == FAM_PR) {  // ranks are kept in double: cast on the host
    std::vector<double> tmp(e->n);
    CK(cudaMemcpyAsync(tmp.data(), e->d_pval, 8ull * e->n, cudaMemcpyDeviceToHost, e->s_comp));
    CK(cudaStreamSynchronize(e->s_comp));
    float *o = static_cast<float *>(out_values);
    for (uint32_t v = 0; v < e->n; ++v) o[v] = (float)tmp[v];
    e->stats.d2h_bytes += 8ull * e->n;
    return SGW_OK;
  }
  CK(cudaMemcpyAsync(out_values, e->d_value, 4ull * e->n, cudaMemcpyDeviceToHost, e->s_comp));
  CK(cudaStreamSynchronize(e->s_comp));
  e->stats.d2h_bytes += 4ull * e->n;
  return SGW_OK;
}

int sgw_read_values_f64(sgw_engine *e, double *out_values) {
  clear_error();
  if (!e || !out_values) return fail(SGW_EINVAL, "null argument");
  if (!e->initialized || e->fam != FAM_PR) return fail(SGW_ESTATE, "no PageRank state");
  CK(cudaSetDevice(e->device));
  CK(cudaMemcpyAsync(out_values, e->d_pval, 8ull * e->n, cudaMemcpyDeviceToHost, e->s_comp));
  CK(cudaStreamSynchronize(e->s_comp));
  e->stats.d2h_bytes += 8ull * e->n;
  return SGW_OK;
}

int sgw_read_active(sgw_engine *e, uint32_t *nodes, uint32_t *ptr, uint32_t capacity, uint32_t *count) {
  clear_error();
  if (!e || !count) return fail(SGW_EINVAL, "null argument");
  if (!e->initialized) return fail(SGW_ESTATE, "engine not initialised");
  *count = e->num_active;
  if (e->num_active > capacity) return fail(SGW_ERANGE, "capacity %u < %u", capacity, e->num_active);
  CK(cudaSetDevice(e->device));
  if (nodes && e->num_active)
    CK(cudaMemcpyAsync(nodes, e->d_queue, 4ull * e->num_active, cudaMemcpyDeviceToHost, e->s_comp));
  if (ptr)
    CK(cudaMemcpyAsync(ptr, e->d_ptr, 4ull * (e->num_active + 1), cudaMemcpyDeviceToHost, e->s_comp));
  CK(cudaStreamSynchronize(e->s_comp));
  return SGW_OK;
}

int sgw_get_stats(const sgw_engine *e, sgw_run_stats *stats) {
  if (!e || !stats) return fail(SGW_EINVAL, "null argument");
  *stats = e->stats;
  return SGW_OK;
}

int sgw_run(sgw_engine *e, const sgw_run_params *p, void *out_values, sgw_run_stats *stats) {
  clear_error();
  if (!e) return fail(SGW_EINVAL, "null engine");
  TRY(state_init(e, p));
  const bool async = p->mode == SGW_ASYNC;
  CK(cudaEventRecord(e->ev_t0, e->s_comp));  // "timer.Start()" after the first generate
  uint32_t gitr = 0;
  while (e->num_active > 0) {
    ++gitr;
    e->gitr = gitr;
    e->stats.active_vertices += e->num_active;
    e->stats.active_edges += e->num_active_edges;
    if (e->policy == SGW_POLICY_LEARNED) {
      TRY(process_iteration_ranges(e));
      TRY(generate_and_stats(e, async ? 0 : 1));
    } else {
      TRY(process_iteration(e));
      TRY(generate_and_plan(e, async ? 0 : 1));
    }
  }
  CK(cudaEventRecord(e->ev_t1, e->s_comp));
  e->stats.global_iterations = gitr;
  // Graph500 m_reached (PR: every edge)
  const bool pr = p->algo == SGW_PR;
  if (!pr) {
    const uint32_t src = p->algo == SGW_CC ? 0xffffffffu : p->source;
    k_reached<<<grid_for(e, e->n, 256), 256, 0, e->s_comp>>>(e->n, p->algo, src, e->d_value, e->d_off, e->d_ctl);
    CK(cudaGetLastError());
  }
  if (out_values) {
    if (pr) {  // the queue is free once the loop is over: cast the ranks into it
      k_pr_to_f32<<<grid_for(e, e->n, 256), 256, 0, e->s_comp>>>(e->n, e->d_pval, (float *)e->d_queue);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(out_values, e->d_queue, 4ull * e->n, cudaMemcpyDeviceToHost, e->s_comp));
    } else {
      CK(cudaMemcpyAsync(out_values, e->d_value, 4ull * e->n, cudaMemcpyDeviceToHost, e->s_comp));
    }
    e->stats.d2h_bytes += 4ull * e->n;
  }
  CK(cudaMemcpyAsync(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->s_comp));
  CK(cudaStreamSynchronize(e->s_comp));
  TRY(check_ctl_error(e));
  e->stats.reached_edges = pr ? e->m : e->h_ctl->reached_edges;
  e->stats.relaxed_edges = e->h_ctl->relaxed_edges;
  e->stats.relaxed_sources = e->h_ctl->relaxed_sources;
  e->stats.inner_iterations = (uint64_t)e->h_ctl->iters_total + e->hub_iters;
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e->ev_t0, e->ev_t1));
  e->stats.ms_device = ms;
  TRY(prof_collect(e));
  if (stats) *stats = e->stats;
  return SGW_OK;
}

}  // extern "C"

// ---- allocation-free compaction ---------------------------------------------
// sgw_generate_noalloc runs the single-pass generate kernel (k_generate, one
// launch, decoupled look-back) on caller-owned device arrays, with the scan's tile state and counters in the
// file-scope array below instead of an engine arena.  Nothing here allocates.
//
// Limit: SGW_NOALLOC_MAX_VERTICES vertices = 16384 scan tiles of 4096.
// Size: 16384 x (4 B flag + 8 B aggregate + 8 B inclusive prefix) plus the
// control block, about 321 KB, held by every GPU that loads the library.

#include <mutex>

namespace {

constexpr uint32_t kNoAllocTiles = SGW_NOALLOC_MAX_VERTICES / kGenTile;
constexpr size_t kNaFlagOff = 0;
constexpr size_t kNaAggOff = kNaFlagOff + 4ull * kNoAllocTiles;
constexpr size_t kNaInclOff = kNaAggOff + 8ull * kNoAllocTiles;
constexpr size_t kNaCtlOff = kNaInclOff + 8ull * kNoAllocTiles;
constexpr size_t kNoAllocBytes = kNaCtlOff + ((sizeof(Ctl) + 255) / 256) * 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_ptr[kNoAllocMaxDevices] = {};  // device address per device
uint32_t g_noalloc_epoch[kNoAllocMaxDevices] = {};

}  // namespace

extern "C" int sgw_generate_noalloc(uint8_t *d_label1, uint8_t *d_label2,
                                    const uint32_t *d_node_pointer, uint32_t n, int consume,
                                    uint32_t *d_queue, uint32_t *d_ptr, void *stream,
                                    uint32_t *num_active, uint64_t *num_active_edges) {
  clear_error();
  if (n == 0 || n > SGW_NOALLOC_MAX_VERTICES)
    return fail(SGW_ERANGE, "sgw_generate_noalloc: n=%u outside 1..%u (static scratch limit)", n,
                SGW_NOALLOC_MAX_VERTICES);
  if (!d_label1 || !d_label2 || !d_node_pointer || !d_queue || !d_ptr)
    return fail(SGW_EINVAL, "sgw_generate_noalloc: null device pointer");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(SGW_ERANGE, "device %d", dev);
  unsigned char *scratch = nullptr;
  uint32_t epoch = 0;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {  // once per device, with that device current
      void *p = nullptr;
      cudaError_t ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (ce != cudaSuccess) {
        cudaGetLastError();
        return fail(SGW_ECUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(ce));
      }
      g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
    }
    scratch = g_noalloc_ptr[dev];
    epoch = g_noalloc_epoch[dev] = (g_noalloc_epoch[dev] + 1) & 0x3fffffffu;
    if (epoch == 0) epoch = g_noalloc_epoch[dev] = 1;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Ctl *ctl = reinterpret_cast<Ctl *>(scratch + kNaCtlOff);
  // the previous call's counters are not trusted: clear the control block
  CK(cudaMemsetAsync(ctl, 0, sizeof(Ctl), s));
  GenArgs a;
  a.n = n;
  a.l1 = d_label1;
  a.l2 = d_label2;
  a.off = d_node_pointer;
  a.queue = d_queue;
  a.ptr = d_ptr;
  a.tflag = reinterpret_cast<uint32_t *>(scratch + kNaFlagOff);
  a.tagg = reinterpret_cast<unsigned long long *>(scratch + kNaAggOff);
  a.tincl = reinterpret_cast<unsigned long long *>(scratch + kNaInclOff);
  a.ctl = ctl;
  a.gmask = nullptr;
  a.epoch = epoch;
  a.num_tiles = (n + kGenTile - 1) / kGenTile;
  a.consume = consume ? 1 : 0;
  a.delta = a.pval = a.qpush = nullptr;
  a.acc = a.damping = 0.0;
  k_generate<<<a.num_tiles, kGenThreads, 0, s>>>(a);
  CK(cudaGetLastError());
  Ctl h;
  CK(cudaMemcpyAsync(&h, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h.error == 1) return fail(SGW_ETIMEOUT, "scan look-back wait timed out");
  if (h.error) return fail(SGW_ESTATE, "scan error %u", h.error);
  if (num_active) *num_active = h.num_active;
  if (num_active_edges) *num_active_edges = h.num_active_edges;
  return SGW_OK;
}

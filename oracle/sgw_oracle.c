/*
 * sgw_oracle.c — CPU oracle for the Subway hot path.  TEST INFRASTRUCTURE:
 * only the tests, the smoke check and the benchmark's CPU-baseline leg load
 * this library, for expected answers and as the reported CPU baseline; the engine
 * never calls it.
 *
 * Two groups of functions:
 *  - orc_*  exact serial restatements of the reference's algorithms and of its
 *           subgraph-generation and partitioning steps;
 *  - omp_*  OpenMP implementations of the same algorithms (the CPU baseline).
 *
 * Semantics follow the reference (paths relative to the Subway tree):
 *  - DIST_INFINITY = UINT_MAX - 1 (shared/globals.hpp:27);
 *  - BFS: value[s] = 0, others INF, relax value+1 / atomicMin
 *    (subway/bfs-sync.cu:28-36, shared/gpu_kernels.cu:41-52);
 *  - SSSP: relax value+w8 / atomicMin (shared/gpu_kernels.cu:141-153);
 *  - SSWP: value[s] = INF, others 0, relax min(value,w8) / atomicMax
 *    (subway/sswp-sync.cu:28-36, shared/gpu_kernels.cu:191-203);
 *  - CC: value[v] = v, relax value / atomicMin along out-edges only
 *    (subway/cc-sync.cu:29-34, shared/gpu_kernels.cu:92-104), whose fixpoint
 *    is value[v] = min id of the vertices that reach v;
 *  - PR: delta = 0.15, value = 0, activation delta > acc, push
 *    damping * delta / outdeg (subway/pr-sync.cu:33-40,
 *    shared/gpu_kernels.cu:226-252), restated as a deterministic
 *    bulk-synchronous schedule in double precision.
 * Every integer algorithm has a unique fixpoint, so any exact method here
 * gives the same labels as the reference's schedule.
 *
 * Edge records are `stride` u32 words: word 0 the destination, word 1 the
 * weight when stride == 2 (OutEdge / OutEdgeWeighted, shared/globals.hpp:33-40).
 * Node pointers are u64 (n + 1 entries; the reference's are u32,
 * shared/graph.cu:46), so graphs of 2^32 edges or more are checked too; the
 * Python wrapper widens u32 arrays.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_INF 4294967294u

/* ------------------------------------------------------------------------ */
/* exact serial algorithms                                                   */
/* ------------------------------------------------------------------------ */

/* Queue BFS. */
int orc_bfs(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride,
            uint32_t src, uint32_t *out) {
  uint32_t *q = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  if (!q) return -1;
  for (uint32_t v = 0; v < n; ++v) out[v] = ORC_INF;
  size_t head = 0, tail = 0;
  out[src] = 0;
  q[tail++] = src;
  while (head < tail) {
    uint32_t u = q[head++];
    for (uint64_t i = np[u]; i < np[u + 1]; ++i) {
      uint32_t v = ed[(size_t)i * stride];
      if (out[v] == ORC_INF) {
        out[v] = out[u] + 1;
        q[tail++] = v;
      }
    }
  }
  free(q);
  return 0;
}

/* Binary heap of (key, vertex) with lazy deletion; max_heap flips order. */
typedef struct {
  uint64_t *a;
  size_t n, cap;
} heap_t;

static int heap_push(heap_t *h, uint64_t x) {
  if (h->n == h->cap) {
    size_t nc = h->cap ? 2 * h->cap : 1024;
    uint64_t *na = (uint64_t *)realloc(h->a, nc * sizeof(uint64_t));
    if (!na) return -1;
    h->a = na;
    h->cap = nc;
  }
  size_t i = h->n++;
  while (i > 0) {
    size_t p = (i - 1) / 2;
    if (h->a[p] <= x) break;
    h->a[i] = h->a[p];
    i = p;
  }
  h->a[i] = x;
  return 0;
}

static uint64_t heap_pop(heap_t *h) {
  uint64_t top = h->a[0];
  uint64_t x = h->a[--h->n];
  size_t i = 0;
  for (;;) {
    size_t l = 2 * i + 1, r = l + 1, m = i;
    uint64_t best = x;
    if (l < h->n && h->a[l] < best) { m = l; best = h->a[l]; }
    if (r < h->n && h->a[r] < best) { m = r; best = h->a[r]; }
    if (m == i) break;
    h->a[i] = h->a[m];
    i = m;
  }
  if (h->n) h->a[i] = x;
  return top;
}

/* Dijkstra (min-plus).  Distances wrap in u32 exactly like the reference's
 * `sourceWeight + w8` (they never come near 2^32 for the supported weights). */
int orc_sssp(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride,
             uint32_t src, uint32_t *out) {
  if (stride != 2) return -2;
  heap_t h = {0, 0, 0};
  for (uint32_t v = 0; v < n; ++v) out[v] = ORC_INF;
  out[src] = 0;
  if (heap_push(&h, (uint64_t)src)) return -1;
  while (h.n) {
    uint64_t x = heap_pop(&h);
    uint32_t d = (uint32_t)(x >> 32), u = (uint32_t)x;
    if (d != out[u]) continue;
    for (uint64_t i = np[u]; i < np[u + 1]; ++i) {
      uint32_t v = ed[(size_t)i * 2], w = ed[(size_t)i * 2 + 1];
      uint32_t c = d + w;
      if (c < out[v]) {
        out[v] = c;
        if (heap_push(&h, ((uint64_t)c << 32) | v)) { free(h.a); return -1; }
      }
    }
  }
  free(h.a);
  return 0;
}

/* Widest path (max-min) by a max-heap Dijkstra; unreached stay 0. */
int orc_sswp(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride,
             uint32_t src, uint32_t *out) {
  if (stride != 2) return -2;
  heap_t h = {0, 0, 0};
  for (uint32_t v = 0; v < n; ++v) out[v] = 0;
  out[src] = ORC_INF;
  /* key = ~width so that the min-heap pops the widest first */
  if (heap_push(&h, ((uint64_t)(~ORC_INF) << 32) | src)) return -1;
  while (h.n) {
    uint64_t x = heap_pop(&h);
    uint32_t wdt = ~(uint32_t)(x >> 32), u = (uint32_t)x;
    if (wdt != out[u]) continue;
    for (uint64_t i = np[u]; i < np[u + 1]; ++i) {
      uint32_t v = ed[(size_t)i * 2], w = ed[(size_t)i * 2 + 1];
      uint32_t c = wdt < w ? wdt : w;
      if (c > out[v]) {
        out[v] = c;
        if (heap_push(&h, ((uint64_t)(~c) << 32) | v)) { free(h.a); return -1; }
      }
    }
  }
  free(h.a);
  return 0;
}

/* value[v] = min id among the vertices that reach v along out-edges:
 * ascending sources, each BFS only over still-unlabelled vertices. */
int orc_cc(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride,
           uint32_t *out) {
  uint32_t *q = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  if (!q) return -1;
  const uint32_t unset = 0xffffffffu;
  for (uint32_t v = 0; v < n; ++v) out[v] = unset;
  for (uint32_t s = 0; s < n; ++s) {
    if (out[s] != unset) continue;
    size_t head = 0, tail = 0;
    out[s] = s;
    q[tail++] = s;
    while (head < tail) {
      uint32_t u = q[head++];
      for (uint64_t i = np[u]; i < np[u + 1]; ++i) {
        uint32_t v = ed[(size_t)i * stride];
        if (out[v] == unset) {
          out[v] = s;
          q[tail++] = v;
        }
      }
    }
  }
  free(q);
  return 0;
}

/* Bulk-synchronous delta PageRank in double precision.  Each round: every
 * vertex with delta > acc moves its delta into its value and pushes
 * damping * delta / outdeg to each out-neighbour; pushes land in the next
 * round's deltas.  Returns the number of rounds in *rounds. */
int orc_pr(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride,
           double init, double acc, double damping, uint32_t max_rounds,
           double *value, uint32_t *rounds) {
  double *delta = (double *)malloc(sizeof(double) * (size_t)n);
  double *push = (double *)malloc(sizeof(double) * (size_t)n);
  uint32_t *act = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  if (!delta || !push || !act) { free(delta); free(push); free(act); return -1; }
  for (uint32_t v = 0; v < n; ++v) { value[v] = 0.0; delta[v] = init; }
  uint32_t r = 0;
  for (; r < max_rounds; ++r) {
    size_t na = 0;
    for (uint32_t v = 0; v < n; ++v)
      if (delta[v] > acc) act[na++] = v;
    if (na == 0) break;
    for (size_t k = 0; k < na; ++k) {
      uint32_t v = act[k];
      double d = delta[v];
      value[v] += d;
      delta[v] = 0.0;
      uint32_t deg = (uint32_t)(np[v + 1] - np[v]);
      push[v] = deg ? damping * d / (double)deg : 0.0;
    }
    for (size_t k = 0; k < na; ++k) {
      uint32_t v = act[k];
      for (uint64_t i = np[v]; i < np[v + 1]; ++i) delta[ed[(size_t)i * stride]] += push[v];
    }
  }
  if (rounds) *rounds = r;
  free(delta);
  free(push);
  free(act);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* restatements of the reference's subgraph generation and partitioning     */
/* ------------------------------------------------------------------------ */

/* SubgraphGenerator<E>::generate without the host gather
 * (shared/subgraph_generator.cu:10-60, :128-162): activeness
 * lab = label1 || label2, masked degree, exclusive scans, queue and pointer
 * compaction.  Zero-degree active vertices are queued, as in the reference.
 * ptr gets count+1 entries (the sentinel of :155-160). Returns count. */
uint32_t orc_generate(uint32_t n, const uint8_t *label1, const uint8_t *label2,
                      const uint32_t *out_degree, uint32_t *queue, uint32_t *ptr) {
  uint32_t cnt = 0, edges = 0;
  for (uint32_t v = 0; v < n; ++v) {
    if (label1[v] || label2[v]) {
      queue[cnt] = v;
      ptr[cnt] = edges;
      edges += out_degree[v];
      ++cnt;
    }
  }
  ptr[cnt] = edges;
  return cnt;
}

/* Partitioner<E>::partition (shared/partitioner.cu:12-91) including its
 * ten extra bisection steps after the first fit.  Returns the number of
 * partitions, or 0xffffffff where the reference would loop forever or exit
 * (a single vertex above max_partition_size).  cap_out limits the output. */
uint32_t orc_partition(const uint32_t *ptr, uint32_t num_active, uint64_t max_partition_size,
                       uint32_t *from_node, uint32_t *node_size, uint32_t cap_out) {
  uint32_t from = 0, to = num_active, p = 0;
  do {
    uint32_t left = from, right = num_active, mid;
    uint64_t size = (uint64_t)ptr[right] - ptr[left];
    if (size <= max_partition_size) {
      to = right;
    } else {
      int found = 0, accur = 10;
      uint32_t steps = 0;
      while (!found || accur > 0) {
        mid = (left + right) / 2;
        size = (uint64_t)ptr[mid] - ptr[from];
        if (found) accur--;
        if (size <= max_partition_size) { left = mid; to = mid; found = 1; }
        else right = mid;
        if (++steps > 4096) return 0xffffffffu;
      }
      if (to == num_active) return 0xffffffffu;
    }
    if (to == from) return 0xffffffffu; /* empty partition: the reference spins */
    if (p < cap_out) {
      if (from_node) from_node[p] = from;
      if (node_size) node_size[p] = to - from;
    }
    ++p;
    from = to;
  } while (to != num_active);
  return p;
}

/* ------------------------------------------------------------------------ */
/* OpenMP CPU baseline                                                       */
/* ------------------------------------------------------------------------ */

static inline int cas_min(uint32_t *p, uint32_t v) {
  uint32_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (v < cur) {
    if (__atomic_compare_exchange_n(p, &cur, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return 1;
  }
  return 0;
}

static inline int cas_max(uint32_t *p, uint32_t v) {
  uint32_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (v > cur) {
    if (__atomic_compare_exchange_n(p, &cur, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return 1;
  }
  return 0;
}

/* Frontier-driven label correction shared by BFS/SSSP/SSWP/CC: each round
 * relaxes the out-edges of the vertices changed in the previous round
 * (algo 0 bfs, 1 sssp, 2 sswp, 3 cc), until no value changes. */
static int omp_frontier(int algo, uint32_t n, const uint64_t *np, const uint32_t *ed,
                        uint32_t stride, uint32_t src, uint32_t *val, uint32_t *rounds_out) {
  uint32_t *front = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t *next = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint8_t *inq = (uint8_t *)calloc(n, 1);
  if (!front || !next || !inq) { free(front); free(next); free(inq); return -1; }
  size_t nf = 0;
  if (algo == 3) {
#pragma omp parallel for
    for (int64_t v = 0; v < (int64_t)n; ++v) { val[v] = (uint32_t)v; front[v] = (uint32_t)v; }
    nf = n;
  } else {
    uint32_t init = (algo == 2) ? 0u : ORC_INF;
#pragma omp parallel for
    for (int64_t v = 0; v < (int64_t)n; ++v) val[v] = init;
    val[src] = (algo == 2) ? ORC_INF : 0u;
    front[0] = src;
    nf = 1;
  }
  uint32_t rounds = 0;
  while (nf) {
    ++rounds;
    size_t nn = 0;
#pragma omp parallel
    {
      uint32_t local[1024];
      int nl = 0;
#pragma omp for schedule(dynamic, 64) nowait
      for (int64_t k = 0; k < (int64_t)nf; ++k) {
        uint32_t u = front[k];
        uint32_t du = __atomic_load_n(&val[u], __ATOMIC_RELAXED);
        for (uint64_t i = np[u]; i < np[u + 1]; ++i) {
          uint32_t v = ed[(size_t)i * stride];
          uint32_t c;
          int upd;
          switch (algo) {
            case 0: c = du + 1; upd = cas_min(&val[v], c); break;
            case 1: c = du + ed[(size_t)i * stride + 1]; upd = cas_min(&val[v], c); break;
            case 2: { uint32_t w = ed[(size_t)i * stride + 1]; c = du < w ? du : w; upd = cas_max(&val[v], c); break; }
            default: c = du; upd = cas_min(&val[v], c); break;
          }
          if (upd && !__atomic_exchange_n(&inq[v], 1, __ATOMIC_RELAXED)) {
            local[nl++] = v;
            if (nl == 1024) {
              size_t at = __atomic_fetch_add(&nn, (size_t)nl, __ATOMIC_RELAXED);
              memcpy(next + at, local, sizeof(uint32_t) * nl);
              nl = 0;
            }
          }
        }
      }
      if (nl) {
        size_t at = __atomic_fetch_add(&nn, (size_t)nl, __ATOMIC_RELAXED);
        memcpy(next + at, local, sizeof(uint32_t) * nl);
      }
    }
#pragma omp parallel for
    for (int64_t k = 0; k < (int64_t)nn; ++k) inq[next[k]] = 0;
    uint32_t *t = front; front = next; next = t;
    nf = nn;
  }
  if (rounds_out) *rounds_out = rounds;
  free(front);
  free(next);
  free(inq);
  return 0;
}

int omp_bfs(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride, uint32_t src, uint32_t *out) {
  return omp_frontier(0, n, np, ed, stride, src, out, 0);
}
/* Appends v to a shared array through a thread-local block of 1024. */
typedef struct { uint32_t buf[1024]; int n; } tl_buf;
static inline void tl_push(tl_buf *b, uint32_t v, uint32_t *out, size_t *cnt) {
  b->buf[b->n++] = v;
  if (b->n == 1024) {
    size_t at = __atomic_fetch_add(cnt, (size_t)b->n, __ATOMIC_RELAXED);
    memcpy(out + at, b->buf, sizeof(uint32_t) * b->n);
    b->n = 0;
  }
}
static inline void tl_flush(tl_buf *b, uint32_t *out, size_t *cnt) {
  if (b->n) {
    size_t at = __atomic_fetch_add(cnt, (size_t)b->n, __ATOMIC_RELAXED);
    memcpy(out + at, b->buf, sizeof(uint32_t) * b->n);
    b->n = 0;
  }
}

/* Delta-stepping SSSP (Meyer and Sanders, J. Algorithms 2003), in the
 * label-correcting form: bucket k holds the vertices whose distance lies in
 * [k*delta, (k+1)*delta).  Rounds relax the out-edges of the current bucket's
 * changed vertices until the bucket is empty; an improvement beyond the
 * bucket parks the vertex in a pending list, from which the next non-empty
 * bucket is taken.  Every vertex whose distance changes has its out-edges
 * relaxed afterwards, so the result is the exact fixpoint (the same labels as
 * orc_sssp); the buckets only cut repeated relaxations. */
static int omp_delta_sssp(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t src,
                          uint32_t delta, uint32_t *val) {
  uint32_t *front = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t *next = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t *pend = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint8_t *inq = (uint8_t *)calloc(n, 1);   /* queued for the next round */
  uint8_t *inp = (uint8_t *)calloc(n, 1);   /* in the pending list */
  if (!front || !next || !pend || !inq || !inp) {
    free(front); free(next); free(pend); free(inq); free(inp);
    return -1;
  }
#pragma omp parallel for
  for (int64_t v = 0; v < (int64_t)n; ++v) val[v] = ORC_INF;
  val[src] = 0;
  front[0] = src;
  size_t nf = 1, np_ = 0;
  uint64_t bucket = 0;
  for (;;) {
    const uint64_t hi = (bucket + 1) * (uint64_t)delta;  /* bucket's end */
    while (nf) {
      size_t nn = 0;
#pragma omp parallel
      {
        tl_buf bn, bp;
        bn.n = bp.n = 0;
#pragma omp for schedule(dynamic, 64) nowait
        for (int64_t k = 0; k < (int64_t)nf; ++k) {
          const uint32_t u = front[k];
          const uint32_t du = __atomic_load_n(&val[u], __ATOMIC_RELAXED);
          for (uint64_t i = np[u]; i < np[u + 1]; ++i) {
            const uint32_t v = ed[2 * (size_t)i];
            const uint32_t c = du + ed[2 * (size_t)i + 1];
            if (!cas_min(&val[v], c)) continue;
            if (c < hi) {
              if (!__atomic_exchange_n(&inq[v], 1, __ATOMIC_RELAXED)) tl_push(&bn, v, next, &nn);
            } else if (!__atomic_exchange_n(&inp[v], 1, __ATOMIC_RELAXED)) {
              tl_push(&bp, v, pend, &np_);
            }
          }
        }
        tl_flush(&bn, next, &nn);
        tl_flush(&bp, pend, &np_);
      }
#pragma omp parallel for
      for (int64_t k = 0; k < (int64_t)nn; ++k) inq[next[k]] = 0;
      uint32_t *t = front; front = next; next = t;
      nf = nn;
    }
    /* next bucket: the smallest among pending vertices still beyond this
     * one (the others were improved into a bucket already relaxed) */
    uint64_t best = UINT64_MAX;
#pragma omp parallel for reduction(min : best)
    for (int64_t k = 0; k < (int64_t)np_; ++k) {
      const uint32_t d = val[pend[k]];
      if ((uint64_t)d >= hi && (uint64_t)d / delta < best) best = (uint64_t)d / delta;
    }
    if (best == UINT64_MAX) break;
    bucket = best;
    const uint64_t lo2 = bucket * (uint64_t)delta, hi2 = lo2 + delta;
    size_t keep = 0;
    nf = 0;
    for (size_t k = 0; k < np_; ++k) {  /* serial: stable and simple */
      const uint32_t v = pend[k];
      const uint32_t d = val[v];
      if ((uint64_t)d >= hi2) {
        pend[keep++] = v;
      } else {
        inp[v] = 0;
        if ((uint64_t)d >= lo2) front[nf++] = v;
      }
    }
    np_ = keep;
  }
  free(front); free(next); free(pend); free(inq); free(inp);
  return 0;
}

int omp_sssp(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride, uint32_t src, uint32_t *out) {
  if (stride != 2) return -2;
  return omp_delta_sssp(n, np, ed, src, 32, out);
}

/* Frontier form of omp_sssp (Bellman-Ford rounds without buckets), kept as a
 * second exact method for the tests. */
int omp_sssp_frontier(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride, uint32_t src,
                      uint32_t *out) {
  if (stride != 2) return -2;
  return omp_frontier(1, n, np, ed, stride, src, out, 0);
}

/* Edges reachable from each of nsrc <= 64 sources (the sum of the out-degrees
 * of the vertices a source reaches, Graph500's m_reached for BFS, SSSP and
 * SSWP), by one bit-parallel search: every vertex carries a 64-bit mask of the
 * sources that reach it, and a vertex whose mask gains bits pushes them along
 * its out-edges in the next round. */
int omp_reach_multi(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride, uint32_t nsrc,
                    const uint32_t *src, uint64_t *reached) {
  if (nsrc == 0 || nsrc > 64) return -2;
  uint64_t *mask = (uint64_t *)calloc(n, sizeof(uint64_t));
  uint32_t *front = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t *next = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint8_t *inq = (uint8_t *)calloc(n, 1);
  if (!mask || !front || !next || !inq) { free(mask); free(front); free(next); free(inq); return -1; }
  size_t nf = 0;
  for (uint32_t k = 0; k < nsrc; ++k) {
    if (!mask[src[k]]) front[nf++] = src[k];
    mask[src[k]] |= 1ULL << k;
  }
  while (nf) {
    size_t nn = 0;
#pragma omp parallel
    {
      tl_buf b;
      b.n = 0;
#pragma omp for schedule(dynamic, 64) nowait
      for (int64_t k = 0; k < (int64_t)nf; ++k) {
        const uint32_t u = front[k];
        const uint64_t mu = __atomic_load_n(&mask[u], __ATOMIC_RELAXED);
        for (uint64_t i = np[u]; i < np[u + 1]; ++i) {
          const uint32_t v = ed[(size_t)i * stride];
          const uint64_t mv = __atomic_load_n(&mask[v], __ATOMIC_RELAXED);
          if ((mu & ~mv) == 0) continue;
          const uint64_t old = __atomic_fetch_or(&mask[v], mu, __ATOMIC_RELAXED);
          if ((mu & ~old) && !__atomic_exchange_n(&inq[v], 1, __ATOMIC_RELAXED)) tl_push(&b, v, next, &nn);
        }
      }
      tl_flush(&b, next, &nn);
    }
#pragma omp parallel for
    for (int64_t k = 0; k < (int64_t)nn; ++k) inq[next[k]] = 0;
    uint32_t *t = front; front = next; next = t;
    nf = nn;
  }
  for (uint32_t k = 0; k < nsrc; ++k) reached[k] = 0;
#pragma omp parallel
  {
    uint64_t loc[64] = {0};
#pragma omp for schedule(static)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
      uint64_t m = mask[v];
      const uint64_t deg = np[v + 1] - np[v];
      while (m) {
        loc[__builtin_ctzll(m)] += deg;
        m &= m - 1;
      }
    }
    for (uint32_t k = 0; k < nsrc; ++k) {
#pragma omp atomic
      reached[k] += loc[k];
    }
  }
  free(mask); free(front); free(next); free(inq);
  return 0;
}
int omp_sswp(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride, uint32_t src, uint32_t *out) {
  if (stride != 2) return -2;
  return omp_frontier(2, n, np, ed, stride, src, out, 0);
}
int omp_cc(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride, uint32_t *out) {
  return omp_frontier(3, n, np, ed, stride, 0, out, 0);
}

/* Same rounds as orc_pr, in parallel (atomic double adds). */
int omp_pr(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride, double init,
           double acc, double damping, uint32_t max_rounds, double *value, uint32_t *rounds) {
  double *delta = (double *)malloc(sizeof(double) * (size_t)n);
  double *push = (double *)malloc(sizeof(double) * (size_t)n);
  if (!delta || !push) { free(delta); free(push); return -1; }
#pragma omp parallel for
  for (int64_t v = 0; v < (int64_t)n; ++v) { value[v] = 0.0; delta[v] = init; }
  uint32_t r = 0;
  for (; r < max_rounds; ++r) {
    int64_t na = 0;
#pragma omp parallel for reduction(+ : na)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
      double d = delta[v];
      if (d > acc) {
        value[v] += d;
        delta[v] = 0.0;
        uint32_t deg = (uint32_t)(np[v + 1] - np[v]);
        push[v] = deg ? damping * d / (double)deg : 0.0;
        ++na;
      } else {
        push[v] = 0.0;
      }
    }
    if (na == 0) break;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
      double p = push[v];
      if (p == 0.0) continue;
      for (uint64_t i = np[v]; i < np[v + 1]; ++i) {
        double *t = &delta[ed[(size_t)i * stride]];
#pragma omp atomic
        *t += p;
      }
    }
  }
  if (rounds) *rounds = r;
  free(delta);
  free(push);
  return 0;
}

int orc_num_threads(void) { return omp_get_max_threads(); }

/* ------------------------------------------------------------------------ */
/* Seeded synthetic inputs, independent of the engine library               */
/* ------------------------------------------------------------------------ */
/* The benchmark's reference arm must not load the engine library, so the
 * R-MAT graph and the source choice are restated here.  Both follow the
 * published algorithms the engine's generator documents (include/
 * sgw_graphgen.h): R-MAT (Chakrabarti, Zhan and Faloutsos, SDM 2004) drawn
 * with SplitMix64 (Steele, Lea and Flood, OOPSLA 2014) indexed by edge number,
 * self-loops, duplicates and vertex n-2's out-edges removed (so that the
 * reference's loader, which never writes outDegree[n-2], shared/graph.cu:
 * 179-181, means the same thing), rows sorted by destination, weight
 * 1 + hash(src, dst) mod wmax; sources uniform among the out-degree > 0
 * vertices of the largest weakly connected component.  The output file is
 * the reference's binary CSR [n][m][nodePointer x n][edge x m]
 * (shared/graph.cu:39-52).  tests/test_oracle.py checks the bytes and the
 * sources against the engine library's generator. */

static inline uint64_t sm_fin(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
#define SM_GAMMA 0x9e3779b97f4a7c15ULL

/* The (src, dst) pair of edge e: one quadrant per level, 32 random bits per
 * level, two levels per 64-bit draw (low half first). */
static inline uint64_t rmat_pair(uint32_t scale, uint64_t ta, uint64_t tab, uint64_t tabc,
                                 uint64_t key, uint64_t e) {
  uint64_t state = key ^ sm_fin(e * SM_GAMMA + 0x2545f4914f6cdd1dULL);
  uint64_t word = 0;
  uint32_t s = 0, d = 0;
  for (uint32_t l = 0; l < scale; ++l) {
    uint64_t u;
    if ((l & 1u) == 0) {
      state += SM_GAMMA;
      word = sm_fin(state);
      u = word & 0xffffffffULL;
    } else {
      u = word >> 32;
    }
    const uint32_t qs = u >= tab, qd = (u >= ta && u < tab) || u >= tabc;
    s = (s << 1) | qs;
    d = (d << 1) | qd;
  }
  return ((uint64_t)s << 32) | d;
}

static int cmp_u64(const void *x, const void *y) {
  const uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
  return (a > b) - (a < b);
}

/* Writes the R-MAT graph to `path` (.bwcsr when weighted, else .bcsr).
 * Returns 0, -1 (memory), -2 (I/O), -3 (m reaches 2^32). */
int orc_rmat_write(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                   uint64_t seed, int weighted, uint32_t wmax, const char *path,
                   uint64_t *m_out) {
  if (scale == 0 || scale > 31 || edge_factor == 0 || (weighted && wmax == 0)) return -4;
  const uint32_t n = 1u << scale, drop = n - 2;
  const uint64_t m0 = (uint64_t)edge_factor << scale;
  const uint64_t ta = (uint64_t)(a * 4294967296.0), tab = (uint64_t)((a + b) * 4294967296.0),
                 tabc = (uint64_t)((a + b + c) * 4294967296.0);
  const uint64_t key = sm_fin(seed ^ 0x6a09e667f3bcc909ULL);
  const uint64_t wkey = sm_fin(seed ^ 0xbb67ae8584caa73bULL);
  /* buckets of sources by their top bits: count, place, sort, deduplicate */
  const uint32_t bb = scale < 14 ? scale : 14, sh = scale - bb, B = 1u << bb;
  const int T = omp_get_max_threads();
  uint64_t *cnt = (uint64_t *)calloc((size_t)T * B, sizeof(uint64_t));
  uint64_t *start = (uint64_t *)calloc((size_t)B + 1, sizeof(uint64_t));
  uint64_t *uniq = (uint64_t *)calloc((size_t)B + 1, sizeof(uint64_t));
  uint32_t *np = (uint32_t *)calloc((size_t)n + 1, sizeof(uint32_t));
  if (!cnt || !start || !uniq || !np) { free(cnt); free(start); free(uniq); free(np); return -1; }
#pragma omp parallel num_threads(T)
  {
    const int t = omp_get_thread_num();
    uint64_t *h = cnt + (size_t)t * B;
    const uint64_t lo = m0 * t / T, hi = m0 * (t + 1) / T;
    for (uint64_t e = lo; e < hi; ++e) {
      const uint64_t p = rmat_pair(scale, ta, tab, tabc, key, e);
      const uint32_t s = (uint32_t)(p >> 32), d = (uint32_t)p;
      if (s != d && s != drop) h[s >> sh]++;
    }
  }
  uint64_t acc = 0;
  for (uint32_t k = 0; k < B; ++k) {
    start[k] = acc;
    for (int t = 0; t < T; ++t) {
      const uint64_t v = cnt[(size_t)t * B + k];
      cnt[(size_t)t * B + k] = acc;
      acc += v;
    }
  }
  start[B] = acc;
  uint64_t *pairs = (uint64_t *)malloc(sizeof(uint64_t) * (acc ? acc : 1));
  if (!pairs) { free(cnt); free(start); free(uniq); free(np); return -1; }
#pragma omp parallel num_threads(T)
  {
    const int t = omp_get_thread_num();
    uint64_t *cur = cnt + (size_t)t * B;
    const uint64_t lo = m0 * t / T, hi = m0 * (t + 1) / T;
    for (uint64_t e = lo; e < hi; ++e) {
      const uint64_t p = rmat_pair(scale, ta, tab, tabc, key, e);
      const uint32_t s = (uint32_t)(p >> 32), d = (uint32_t)p;
      if (s != d && s != drop) pairs[cur[s >> sh]++] = p;
    }
  }
  free(cnt);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < (int64_t)B; ++k) {
    uint64_t *p = pairs + start[k];
    const uint64_t len = start[k + 1] - start[k];
    qsort(p, len, sizeof(uint64_t), cmp_u64);
    uint64_t u = 0;
    for (uint64_t i = 0; i < len; ++i)
      if (u == 0 || p[u - 1] != p[i]) p[u++] = p[i];
    uniq[k] = u;
    for (uint64_t i = 0; i < u; ++i) np[(p[i] >> 32) + 1]++;
  }
  uint64_t m = 0;
  for (uint32_t k = 0; k < B; ++k) m += uniq[k];
  if (m >= 0xffffffffULL) { free(pairs); free(start); free(uniq); free(np); return -3; }
  for (uint32_t v = 0; v < n; ++v) np[v + 1] += np[v];
  /* records in place, bucket by bucket: (dst, weight) in the same 8 bytes,
   * or the 4-byte destination moved down within the bucket's own region */
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < (int64_t)B; ++k) {
    uint64_t *p = pairs + start[k];
    uint32_t *w32 = (uint32_t *)p;
    for (uint64_t i = 0; i < uniq[k]; ++i) {
      const uint32_t s = (uint32_t)(p[i] >> 32), d = (uint32_t)p[i];
      if (weighted) {
        const uint64_t h = sm_fin(wkey ^ sm_fin(((uint64_t)s << 32) | d) ^ 0x5851f42d4c957f2dULL);
        w32[2 * i] = d;
        w32[2 * i + 1] = 1u + (uint32_t)(h % wmax);
      } else {
        w32[i] = d;
      }
    }
  }
  int st = 0;
  FILE *f = fopen(path, "wb");
  if (!f) st = -2;
  if (!st) {
    const uint32_t hdr[2] = {n, (uint32_t)m};
    if (fwrite(hdr, 4, 2, f) != 2 || fwrite(np, 4, n, f) != n) st = -2;
  }
  const size_t rec = weighted ? 8 : 4;
  for (uint32_t k = 0; k < B && !st; ++k)
    if (uniq[k] && fwrite(pairs + start[k], rec, uniq[k], f) != uniq[k]) st = -2;
  if (f && fclose(f) != 0 && !st) st = -2;
  free(pairs);
  free(start);
  free(uniq);
  free(np);
  if (m_out) *m_out = m;
  return st;
}

/* Root (minimum id) of x's set; roots only ever gain smaller parents. */
static uint32_t uf_root(uint32_t *par, uint32_t x) {
  for (;;) {
    const uint32_t p = __atomic_load_n(&par[x], __ATOMIC_RELAXED);
    if (p == x) return x;
    const uint32_t gp = __atomic_load_n(&par[p], __ATOMIC_RELAXED);
    if (gp != p) __atomic_compare_exchange_n(&par[x], &(uint32_t){p}, gp, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
    x = gp;
  }
}

/* count sources (may repeat only when count exceeds the candidates), picked
 * uniformly among the out-degree > 0 vertices of the largest weakly
 * connected component (ties: the component with the smallest id). */
int orc_pick_sources(uint32_t n, const uint64_t *np, const uint32_t *ed, uint32_t stride,
                     uint32_t count, uint64_t seed, uint32_t *out) {
  uint32_t *par = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t *size = (uint32_t *)calloc(n, sizeof(uint32_t));
  if (!par || !size) { free(par); free(size); return -1; }
#pragma omp parallel for
  for (int64_t v = 0; v < (int64_t)n; ++v) par[v] = (uint32_t)v;
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t v = 0; v < (int64_t)n; ++v) {
    for (uint64_t i = np[v]; i < np[v + 1]; ++i) {
      uint32_t x = (uint32_t)v, y = ed[(size_t)i * stride];
      for (;;) {
        x = uf_root(par, x);
        y = uf_root(par, y);
        if (x == y) break;
        if (x < y) { const uint32_t t = x; x = y; y = t; }
        uint32_t expect = x;  /* hang the larger root under the smaller */
        if (__atomic_compare_exchange_n(&par[x], &expect, y, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) break;
      }
    }
  }
  /* parents always have smaller ids, so one ascending pass leaves roots */
  for (uint32_t v = 0; v < n; ++v) {
    par[v] = par[par[v]];
    size[par[v]]++;
  }
  uint32_t best = 0;
  for (uint32_t v = 1; v < n; ++v)
    if (size[v] > size[best]) best = v;
  uint32_t *cand = size;  /* sizes are no longer needed */
  size_t nc = 0;
  for (uint32_t v = 0; v < n; ++v)
    if (par[v] == best && np[v + 1] > np[v]) cand[nc++] = v;
  free(par);
  par = cand;
  if (nc == 0) { free(par); return -2; }
  uint64_t state = sm_fin(seed ^ 0xa54ff53a5f1d36f1ULL);
  for (uint32_t k = 0; k < count; ++k) {
    uint32_t v = 0;
    int tries = 0, dup;
    do {
      state += SM_GAMMA;
      v = par[(uint32_t)(((sm_fin(state) >> 32) * nc) >> 32)];
      dup = 0;
      for (uint32_t j = 0; j < k; ++j) dup |= out[j] == v;
    } while (count <= nc && ++tries < 1000 && dup);
    out[k] = v;
  }
  free(par);
  return 0;
}

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
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_INF 4294967294u

/* ------------------------------------------------------------------------ */
/* exact serial algorithms                                                   */
/* ------------------------------------------------------------------------ */

/* Queue BFS. */
int orc_bfs(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride,
            uint32_t src, uint32_t *out) {
  uint32_t *q = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  if (!q) return -1;
  for (uint32_t v = 0; v < n; ++v) out[v] = ORC_INF;
  size_t head = 0, tail = 0;
  out[src] = 0;
  q[tail++] = src;
  while (head < tail) {
    uint32_t u = q[head++];
    for (uint32_t i = np[u]; i < np[u + 1]; ++i) {
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
int orc_sssp(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride,
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
    for (uint32_t i = np[u]; i < np[u + 1]; ++i) {
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
int orc_sswp(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride,
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
    for (uint32_t i = np[u]; i < np[u + 1]; ++i) {
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
int orc_cc(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride,
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
      for (uint32_t i = np[u]; i < np[u + 1]; ++i) {
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
int orc_pr(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride,
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
      uint32_t deg = np[v + 1] - np[v];
      push[v] = deg ? damping * d / (double)deg : 0.0;
    }
    for (size_t k = 0; k < na; ++k) {
      uint32_t v = act[k];
      for (uint32_t i = np[v]; i < np[v + 1]; ++i) delta[ed[(size_t)i * stride]] += push[v];
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
static int omp_frontier(int algo, uint32_t n, const uint32_t *np, const uint32_t *ed,
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
        for (uint32_t i = np[u]; i < np[u + 1]; ++i) {
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

int omp_bfs(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride, uint32_t src, uint32_t *out) {
  return omp_frontier(0, n, np, ed, stride, src, out, 0);
}
int omp_sssp(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride, uint32_t src, uint32_t *out) {
  if (stride != 2) return -2;
  return omp_frontier(1, n, np, ed, stride, src, out, 0);
}
int omp_sswp(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride, uint32_t src, uint32_t *out) {
  if (stride != 2) return -2;
  return omp_frontier(2, n, np, ed, stride, src, out, 0);
}
int omp_cc(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride, uint32_t *out) {
  return omp_frontier(3, n, np, ed, stride, 0, out, 0);
}

/* Same rounds as orc_pr, in parallel (atomic double adds). */
int omp_pr(uint32_t n, const uint32_t *np, const uint32_t *ed, uint32_t stride, double init,
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
        uint32_t deg = np[v + 1] - np[v];
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
      for (uint32_t i = np[v]; i < np[v + 1]; ++i) {
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

// Host half of libsubwaygb: graph objects, file formats, seeded generators,
// connected-component helpers and the host partition planner.
//
// File formats follow the reference: binary CSR [u32 n][u32 m][u32
// nodePointer x n][edge x m] (shared/graph.cu:39-52, tools/converter.cpp:
// 88-95) and "src dst [w]" text lines (shared/graph.cu:56-170, README.md:16-30).

#include <omp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include "sgw_graphgen.h"
#include "sgw_internal.h"

namespace sgw {

static thread_local char g_err[512] = "";

int fail(int status, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return status;
}

void clear_error() { g_err[0] = 0; }

static const size_t kPage = size_t(1) << 16;

void *host_alloc(size_t bytes, size_t *rounded) {
  size_t r = (bytes + kPage - 1) / kPage * kPage;
  if (r == 0) r = kPage;
  void *p = nullptr;
  if (posix_memalign(&p, kPage, r) != 0) return nullptr;
  if (rounded) *rounded = r;
  return p;
}

void host_free(void *p) { free(p); }

int graph_alloc(uint32_t n, uint64_t m, int weighted, sgw_graph **out) {
  sgw_graph *g = new (std::nothrow) sgw_graph();
  if (!g) return fail(SGW_ENOMEM, "graph object");
  g->n = n;
  g->m = m;
  g->weighted = weighted ? 1 : 0;
  g->esz = weighted ? 8 : 4;
  g->owns = true;
  const bool wide = m >= (uint64_t(1) << 32);
  void *np = host_alloc((wide ? 8 : 4) * (size_t(n) + 1), nullptr);
  if (wide) g->node_pointer64 = (uint64_t *)np;
  else g->node_pointer = (uint32_t *)np;
  // 16 spare bytes: the engine's 16-byte reads of the last records stay inside
  g->edges = host_alloc(size_t(m) * g->esz + 16, &g->edges_bytes_alloc);
  if (!np || !g->edges) {
    host_free(np);
    host_free(g->edges);
    delete g;
    return fail(SGW_ENOMEM, "graph arrays (n=%u m=%llu)", n, (unsigned long long)m);
  }
  *out = g;
  return SGW_OK;
}

// Sets node pointer v of a graph being built, whichever its width.
static inline void np_set(sgw_graph *g, uint64_t v, uint64_t x) {
  if (g->node_pointer64) g->node_pointer64[v] = x;
  else g->node_pointer[v] = (uint32_t)x;
}

// Checks monotone node pointers (np[0] == 0, np[n] == m is the caller's) and
// edge endpoints below n, in parallel.  Returns 0, or 1 (pointers) / 2
// (endpoints) / 4 (an out-degree of 2^32 or more).
static int validate_csr(const sgw_graph *g) {
  int bad = 0;
  const uint32_t n = g->n;
#pragma omp parallel for reduction(| : bad)
  for (int64_t v = 0; v < (int64_t)n; ++v) {
    const uint64_t a = np_at(g, (uint64_t)v), b = np_at(g, (uint64_t)v + 1);
    if (a > b) bad |= 1;
    else if (b - a >= (uint64_t(1) << 32)) bad |= 4;
  }
  if (bad) return bad & 1 ? 1 : 4;
  const uint32_t *ed = (const uint32_t *)g->edges;
  const size_t stride = g->esz / 4;
#pragma omp parallel for reduction(| : bad)
  for (int64_t i = 0; i < (int64_t)g->m; ++i)
    if (ed[size_t(i) * stride] >= n) bad |= 2;
  return bad;
}

bool device_offsets(const sgw_graph *g, uint32_t *lo, unsigned long long *base) {
  const uint32_t n = g->n;
  if (!g->node_pointer64) {
    copy_bytes(lo, g->node_pointer, 4ull * (n + 1));
    return true;
  }
  const uint64_t *np = g->node_pointer64;
  const int64_t groups = (int64_t)(n >> kOffGroupLog2) + 2;
  int over = 0;
#pragma omp parallel for reduction(| : over)
  for (int64_t k = 0; k < groups; ++k) {
    const uint64_t v0 = std::min<uint64_t>(n, (uint64_t)k << kOffGroupLog2);
    const uint64_t v1 = std::min<uint64_t>(n, v0 + (1u << kOffGroupLog2));
    if (np[v1] - np[v0] >= (uint64_t(1) << 32)) over = 1;
  }
  if (over) return false;
#pragma omp parallel for
  for (int64_t k = 0; k < groups; ++k) base[k] = np[std::min<uint64_t>(n, (uint64_t)k << kOffGroupLog2)];
#pragma omp parallel for
  for (int64_t v = 0; v <= (int64_t)n; ++v) lo[v] = (uint32_t)np[v];
  return true;
}

static const char *csr_problem(int bad) {
  return bad & 1 ? "node pointers not monotone"
                 : bad & 4 ? "out-degree of 2^32 or more" : "edge endpoint out of range";
}

bool pack_bits_for(const sgw_graph *g, uint32_t wmax, uint32_t *nbits) {
  if (!g->weighted || g->m == 0) return false;
  uint32_t nb = 1;
  while (nb < 32 && (uint64_t(1) << nb) < g->n) ++nb;
  if (nb >= 31) return false;
  if ((uint64_t)wmax >= (uint64_t(1) << (32 - nb))) return false;
  *nbits = nb;
  return true;
}

bool pack_bits(const sgw_graph *g, uint32_t *nbits) { return pack_bits_for(g, max_weight(g), nbits); }

void copy_bytes(void *dst, const void *src, size_t bytes) {
  const size_t piece = size_t(64) << 20;
  const int64_t pieces = (int64_t)((bytes + piece - 1) / piece);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < pieces; ++k) {
    const size_t a = size_t(k) * piece, b = std::min(bytes, a + piece);
    memcpy((char *)dst + a, (const char *)src + a, b - a);
  }
}

void pack_into(const sgw_graph *g, uint32_t nb, uint32_t *p) {
  const uint32_t *ed = (const uint32_t *)g->edges;
#pragma omp parallel for
  for (int64_t i = 0; i < (int64_t)g->m; ++i) p[i] = (ed[2 * size_t(i) + 1] << nb) | ed[2 * size_t(i)];
}


uint32_t max_weight(const sgw_graph *g) {
  if (!g->weighted || g->m == 0) return 0;
  const bool cacheable = g->owns || g->map_base;
  if (cacheable) {
    const int64_t c = g->wmax_cache.load(std::memory_order_relaxed);
    if (c >= 0) return (uint32_t)c;
  }
  const uint32_t *ed = (const uint32_t *)g->edges;
  uint32_t wmax = 0;
#pragma omp parallel for reduction(max : wmax)
  for (int64_t i = 0; i < (int64_t)g->m; ++i) wmax = std::max(wmax, ed[2 * size_t(i) + 1]);
  if (cacheable) g->wmax_cache.store(wmax, std::memory_order_relaxed);
  return wmax;
}

// The same transforms for edges [e0, e1), written from out[0] on (one chunk
// of a transfer copy held in pieces).
void pack_range(const sgw_graph *g, uint32_t nb, uint32_t *out, uint64_t e0, uint64_t e1) {
  const uint32_t *ed = (const uint32_t *)g->edges;
#pragma omp parallel for
  for (int64_t i = (int64_t)e0; i < (int64_t)e1; ++i)
    out[i - e0] = (ed[2 * size_t(i) + 1] << nb) | ed[2 * size_t(i)];
}

void split_ends_range(const sgw_graph *g, uint32_t *ends, uint64_t e0, uint64_t e1) {
  const uint32_t *ed = (const uint32_t *)g->edges;
#pragma omp parallel for
  for (int64_t i = (int64_t)e0; i < (int64_t)e1; ++i) ends[i - e0] = ed[2 * size_t(i)];
}

void split_weights_range(const sgw_graph *g, uint8_t *w8, uint64_t e0, uint64_t e1) {
  const uint32_t *ed = (const uint32_t *)g->edges;
#pragma omp parallel for
  for (int64_t i = (int64_t)e0; i < (int64_t)e1; ++i) w8[i - e0] = (uint8_t)ed[2 * size_t(i) + 1];
}

void copy_records_range(const sgw_graph *g, void *out, uint64_t e0, uint64_t e1) {
  copy_bytes(out, (const char *)g->edges + e0 * g->esz, (e1 - e0) * g->esz);
}

bool pack_weighted(const sgw_graph *g, uint32_t **out, size_t *alloc_bytes, uint32_t *nbits) {
  *out = nullptr;
  uint32_t nb = 0;
  if (!pack_bits(g, &nb)) return false;
  uint32_t *p = (uint32_t *)host_alloc(sizeof(uint32_t) * size_t(g->m), alloc_bytes);
  if (!p) return false;
  pack_into(g, nb, p);
  *out = p;
  *nbits = nb;
  return true;
}

// ---- SplitMix64 ------------------------------------------------------------
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
static const uint64_t kGamma = 0x9e3779b97f4a7c15ULL;

struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed) {}
  uint64_t next() { s += kGamma; return mix64(s); }
};

static inline uint32_t edge_weight(uint64_t seed, uint32_t src, uint32_t dst,
                                   uint32_t wmax) {
  uint64_t h = mix64(seed ^ mix64((uint64_t(src) << 32) | dst) ^ 0x5851f42d4c957f2dULL);
  return 1u + (uint32_t)(h % wmax);
}

// Draws edge e of an R-MAT stream.  Thresholds are 32-bit fixed point.
struct RmatParams {
  uint32_t scale;
  uint64_t ta, tab, tabc;  // cumulative thresholds scaled to 2^32
  uint64_t seed;
};

static inline void rmat_edge(const RmatParams &p, uint64_t e, uint32_t *src,
                             uint32_t *dst) {
  SplitMix rng(p.seed ^ mix64(e * kGamma + 0x2545f4914f6cdd1dULL));
  uint32_t s = 0, d = 0;
  uint64_t bits = 0;
  int avail = 0;
  for (uint32_t l = 0; l < p.scale; ++l) {
    if (avail == 0) { bits = rng.next(); avail = 2; }
    uint64_t u = bits & 0xffffffffULL;
    bits >>= 32;
    --avail;
    uint32_t qs, qd;
    if (u < p.ta) { qs = 0; qd = 0; }
    else if (u < p.tab) { qs = 0; qd = 1; }
    else if (u < p.tabc) { qs = 1; qd = 0; }
    else { qs = 1; qd = 1; }
    s = (s << 1) | qs;
    d = (d << 1) | qd;
  }
  *src = s;
  *dst = d;
}

static inline void er_edge(uint64_t seed, uint32_t n, uint64_t e, uint32_t *src,
                           uint32_t *dst) {
  SplitMix rng(seed ^ mix64(e * kGamma + 0x14057b7ef767814fULL));
  uint64_t r = rng.next();
  *src = (uint32_t)(((r & 0xffffffffULL) * n) >> 32);
  *dst = (uint32_t)(((r >> 32) * n) >> 32);
}

// Builds a deduplicated CSR from an edge stream given as a functor
// draw(e, &src, &dst) for e in [0, m0).  Edges are bucketed by the top bits of
// the source without atomics (two passes over the stream), each bucket is
// sorted and deduplicated, and the CSR is written in one more pass.
template <class Draw>
static int build_csr(uint32_t n, uint64_t m0, Draw draw, uint32_t drop_vertex,
                     int weighted, uint32_t wmax, uint64_t wseed,
                     sgw_graph **out) {
  const int T = omp_get_max_threads();
  int bbits = 0;
  while ((1u << bbits) < n && bbits < 16) ++bbits;
  int shift = 0;
  while ((uint64_t(n) >> shift) > (uint64_t(1) << bbits)) ++shift;
  const uint32_t B = 1u << bbits;
  auto bucket_of = [&](uint32_t s) { return s >> shift; };

  std::vector<uint64_t> hist(size_t(T) * B, 0);
  const uint64_t per = (m0 + T - 1) / T;
#pragma omp parallel num_threads(T)
  {
    int t = omp_get_thread_num();
    uint64_t *h = &hist[size_t(t) * B];
    uint64_t lo = std::min<uint64_t>(m0, per * t), hi = std::min<uint64_t>(m0, lo + per);
    for (uint64_t e = lo; e < hi; ++e) {
      uint32_t s, d;
      draw(e, &s, &d);
      if (s == d || s == drop_vertex) continue;
      h[bucket_of(s)]++;
    }
  }
  // prefix over (bucket, thread)
  std::vector<uint64_t> bstart(B + 1, 0);
  {
    uint64_t acc = 0;
    for (uint32_t b = 0; b < B; ++b) {
      bstart[b] = acc;
      for (int t = 0; t < T; ++t) {
        uint64_t c = hist[size_t(t) * B + b];
        hist[size_t(t) * B + b] = acc;
        acc += c;
      }
    }
    bstart[B] = acc;
  }
  const uint64_t kept = bstart[B];
  uint64_t *pairs = (uint64_t *)host_alloc(sizeof(uint64_t) * std::max<uint64_t>(kept, 1), nullptr);
  if (!pairs) return fail(SGW_ENOMEM, "edge pairs (%llu)", (unsigned long long)kept);
#pragma omp parallel num_threads(T)
  {
    int t = omp_get_thread_num();
    uint64_t *cur = &hist[size_t(t) * B];
    uint64_t lo = std::min<uint64_t>(m0, per * t), hi = std::min<uint64_t>(m0, lo + per);
    for (uint64_t e = lo; e < hi; ++e) {
      uint32_t s, d;
      draw(e, &s, &d);
      if (s == d || s == drop_vertex) continue;
      pairs[cur[bucket_of(s)]++] = (uint64_t(s) << 32) | d;
    }
  }
  // sort + dedup each bucket, count rows
  std::vector<uint64_t> bunique(B, 0);
  std::vector<uint32_t> deg(size_t(n) + 1, 0);
#pragma omp parallel for schedule(dynamic, 1) num_threads(T)
  for (int64_t b = 0; b < (int64_t)B; ++b) {
    uint64_t *p = pairs + bstart[b];
    uint64_t len = bstart[b + 1] - bstart[b];
    std::sort(p, p + len);
    uint64_t u = 0;
    for (uint64_t i = 0; i < len; ++i) {
      if (u == 0 || p[u - 1] != p[i]) p[u++] = p[i];
    }
    bunique[b] = u;
    for (uint64_t i = 0; i < u; ++i) deg[p[i] >> 32]++;
  }
  uint64_t m = 0;
  for (uint32_t b = 0; b < B; ++b) m += bunique[b];
  sgw_graph *g = nullptr;
  int st = graph_alloc(n, m, weighted, &g);
  if (st != SGW_OK) { host_free(pairs); return st; }
  {
    uint64_t acc = 0;
    for (uint32_t v = 0; v < n; ++v) { np_set(g, v, acc); acc += deg[v]; }
    np_set(g, n, acc);
  }
  // bucket b's rows start at node_pointer[first source of bucket]
#pragma omp parallel for schedule(dynamic, 1) num_threads(T)
  for (int64_t b = 0; b < (int64_t)B; ++b) {
    const uint64_t *p = pairs + bstart[b];
    uint64_t u = bunique[b];
    if (u == 0) continue;
    uint64_t pos = np_at(g, p[0] >> 32);
    if (weighted) {
      uint32_t *ed = (uint32_t *)g->edges;
      for (uint64_t i = 0; i < u; ++i) {
        uint32_t s = (uint32_t)(p[i] >> 32), d = (uint32_t)p[i];
        ed[2 * (pos + i)] = d;
        ed[2 * (pos + i) + 1] = edge_weight(wseed, s, d, wmax);
      }
    } else {
      uint32_t *ed = (uint32_t *)g->edges;
      for (uint64_t i = 0; i < u; ++i) ed[pos + i] = (uint32_t)p[i];
    }
  }
  host_free(pairs);
  *out = g;
  return SGW_OK;
}

static std::string extension_of(const char *path) {
  std::string s(path);
  size_t dot = s.find_last_of('.');
  if (dot == std::string::npos) return "";
  return s.substr(dot + 1);
}

// Reads [off, off + bytes) of fd into dst with T threads, each issuing pread
// calls of at most 64 MiB on its own contiguous slice.  Returns false on a short
// read or an I/O error.
static bool pread_parallel(int fd, char *dst, size_t bytes, off_t off) {
  const size_t kPiece = size_t(64) << 20;
  const int T = (int)std::max<size_t>(1, std::min<size_t>(omp_get_max_threads(), (bytes >> 23) + 1));
  int bad = 0;
#pragma omp parallel num_threads(T) reduction(| : bad)
  {
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
    size_t lo = bytes * t / nt, hi = bytes * (t + 1) / nt;
    while (lo < hi && !bad) {
      ssize_t r = pread(fd, dst + lo, std::min(hi - lo, kPiece), off + (off_t)lo);
      if (r <= 0) bad = 1;
      else lo += size_t(r);
    }
  }
  return !bad;
}

// Binary CSR files.  .bcsr / .bwcsr (graph.cu:43-51): [u32 n][u32 m]
// [u32 nodePointer x n][edge x m], the sentinel nodePointer[n] = m implied.
// .bcsr64 / .bwcsr64, for graphs of 2^32 edges or more: [u64 n][u64 m]
// [u64 nodePointer x n][edge x m]; every field and the records stay 8-byte
// aligned, so the file maps in place.  Vertex ids stay u32 in both.
struct BinHeader {
  uint64_t n = 0, m = 0;
  size_t hdr = 0, npsz = 0;  // header bytes, bytes per node pointer
};

static int read_header(int fd, const char *path, bool wide_file, int weighted, BinHeader *h) {
  struct stat sb;
  if (fstat(fd, &sb) != 0) return fail(SGW_EIO, "cannot stat %s", path);
  if (wide_file) {
    uint64_t hd[2];
    if (pread(fd, hd, sizeof(hd), 0) != (ssize_t)sizeof(hd)) return fail(SGW_EFORMAT, "%s: truncated header", path);
    h->n = hd[0];
    h->m = hd[1];
    h->hdr = 16;
    h->npsz = 8;
  } else {
    uint32_t hd[2];
    if (pread(fd, hd, sizeof(hd), 0) != (ssize_t)sizeof(hd)) return fail(SGW_EFORMAT, "%s: truncated header", path);
    h->n = hd[0];
    h->m = hd[1];
    h->hdr = 8;
    h->npsz = 4;
  }
  if (h->n == 0) return fail(SGW_EFORMAT, "%s: zero vertices", path);
  if (h->n >= (uint64_t(1) << 32)) return fail(SGW_EFORMAT, "%s: %llu vertices (ids are u32)", path,
                                               (unsigned long long)h->n);
  const uint64_t esz = weighted ? 8 : 4;
  const unsigned long long want = h->hdr + h->npsz * h->n + h->m * esz;
  if (h->m > (uint64_t(1) << 40) || (unsigned long long)sb.st_size != want)
    return fail(SGW_EFORMAT, "%s: size %lld, expected %llu for n=%llu m=%llu", path, (long long)sb.st_size,
                want, (unsigned long long)h->n, (unsigned long long)h->m);
  return SGW_OK;
}

// Fills the graph's node pointers [0, n) from a file's array of npsz-byte
// pointers (u32 or u64, into a u32 or u64 array) and sets [n] = m.  False
// when a u64 pointer above m was to be narrowed to u32 (it would wrap and
// could pass the monotonicity check).
static bool fill_pointers(sgw_graph *g, const void *src, size_t npsz) {
  const uint32_t n = g->n;
  int over = 0;
  if (npsz == 4 && g->node_pointer) {
    copy_bytes(g->node_pointer, src, 4ull * n);
  } else if (npsz == 8 && g->node_pointer64) {
    copy_bytes(g->node_pointer64, src, 8ull * n);
  } else {
    const uint64_t m = g->m;
#pragma omp parallel for reduction(| : over)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
      const uint64_t x = npsz == 8 ? ((const uint64_t *)src)[v] : (uint64_t)((const uint32_t *)src)[v];
      if (x > m) over = 1;
      np_set(g, (uint64_t)v, x);
    }
  }
  np_set(g, n, g->m);
  return !over;
}

static int load_binary(const char *path, int weighted, bool wide_file, sgw_graph **out) {
  int fd = open(path, O_RDONLY);
  if (fd < 0) return fail(SGW_EIO, "cannot open %s", path);
  BinHeader h;
  int st = read_header(fd, path, wide_file, weighted, &h);
  if (st != SGW_OK) { close(fd); return st; }
  const uint32_t n = (uint32_t)h.n;
  const uint32_t esz = weighted ? 8 : 4;
  sgw_graph *g = nullptr;
  st = graph_alloc(n, h.m, weighted, &g);
  if (st != SGW_OK) { close(fd); return st; }
  bool ok;
  if ((h.npsz == 8) == (g->node_pointer64 != nullptr)) {
    ok = pread_parallel(fd, g->node_pointer64 ? (char *)g->node_pointer64 : (char *)g->node_pointer,
                        h.npsz * size_t(n), (off_t)h.hdr);
    np_set(g, n, h.m);
  } else {  // a 64-bit file of fewer than 2^32 edges: u32 pointers in memory
    char *tmp = (char *)host_alloc(h.npsz * size_t(n), nullptr);
    ok = tmp && pread_parallel(fd, tmp, h.npsz * size_t(n), (off_t)h.hdr);
    const bool fits = ok && fill_pointers(g, tmp, h.npsz);
    host_free(tmp);
    if (ok && !fits) {
      close(fd);
      sgw_graph_free(g);
      return fail(SGW_EFORMAT, "%s: %s", path, csr_problem(1));
    }
  }
  ok = ok && pread_parallel(fd, (char *)g->edges, size_t(h.m) * esz, (off_t)(h.hdr + h.npsz * size_t(n)));
  close(fd);
  if (!ok) {
    sgw_graph_free(g);
    return fail(SGW_EFORMAT, "%s: truncated body", path);
  }
  const int bad = validate_csr(g);
  if (bad) {
    sgw_graph_free(g);
    return fail(SGW_EFORMAT, "%s: %s", path, csr_problem(bad));
  }
  *out = g;
  return SGW_OK;
}

// Text edge lists: one "src dst" (.el) or "src dst w" (.wel) line per edge,
// decimal u32 values separated by blanks (graph.cu:65-82, 120-137).  Blank
// lines and lines starting with '#' or '%' are skipped; anything after the
// last value of a line is ignored.  n = max id + 1 (graph.cu:85) and rows keep
// file order, as the reference's counting sort does (graph.cu:92-113).
//
// The file is mapped and cut into one piece per thread at line starts; the
// threads parse their pieces, count degrees with relaxed atomics, and then
// place edges, each thread owning a vertex range of about m / T edges and
// walking all pieces in file order, so the result does not depend on the
// thread count.
struct TextPiece {
  std::vector<uint32_t> src, dst, w;
  uint32_t max_id = 0;
  size_t bad_at = SIZE_MAX;  // offset of the first bad line
  int bad_status = SGW_OK;
};

static inline bool is_blank(char c) { return c == ' ' || c == '\t'; }

// Parses one unsigned decimal at p (blanks skipped); false if there is none.
static inline bool parse_u32(const char *&p, const char *end, uint64_t *v, bool *over) {
  while (p < end && is_blank(*p)) ++p;
  if (p == end || *p < '0' || *p > '9') return false;
  uint64_t x = 0;
  while (p < end && *p >= '0' && *p <= '9') {
    x = x * 10 + uint64_t(*p - '0');
    if (x > 0xffffffffULL) { *over = true; x = 0xffffffffULL + 1; }
    ++p;
  }
  *v = x;
  return true;
}

static void parse_piece(const char *base, size_t lo, size_t hi, int weighted, TextPiece &pc) {
  const char *p = base + lo, *end = base + hi;
  pc.src.reserve((hi - lo) / (weighted ? 10 : 7) + 16);
  pc.dst.reserve(pc.src.capacity());
  if (weighted) pc.w.reserve(pc.src.capacity());
  while (p < end) {
    const char *line = p;
    const char *eol = (const char *)memchr(p, '\n', size_t(end - p));
    if (!eol) eol = end;
    while (p < eol && is_blank(*p)) ++p;
    if (p < eol && *p != '\r' && *p != '#' && *p != '%') {
      uint64_t s = 0, d = 0, w = 0;
      bool over = false;
      bool ok = parse_u32(p, eol, &s, &over) && parse_u32(p, eol, &d, &over) &&
                (!weighted || parse_u32(p, eol, &w, &over));
      if (!ok || over || s >= 0xffffffffULL || d >= 0xffffffffULL) {
        pc.bad_at = size_t(line - base);
        pc.bad_status = ok ? SGW_ERANGE : SGW_EFORMAT;
        return;
      }
      pc.src.push_back((uint32_t)s);
      pc.dst.push_back((uint32_t)d);
      if (weighted) pc.w.push_back((uint32_t)w);
      pc.max_id = std::max(pc.max_id, (uint32_t)std::max(s, d));
    }
    p = eol + 1;
  }
}

// Node pointers (T = u32 or u64) and rows of a graph from parsed pieces:
// degrees, an exclusive prefix in T blocks, then placement, where thread j
// owns the sources whose rows start in its 1/T of the edge range and scans
// every piece in file order, keeping rows stable.
template <class P>
static void place_text_rows(sgw_graph *g, const std::vector<TextPiece> &pcs, int T, P *np) {
  const uint32_t n = g->n;
  const uint64_t m = g->m;
  const int weighted = g->weighted;
#pragma omp parallel for num_threads(T)
  for (int64_t v = 0; v <= (int64_t)n; ++v) np[v] = 0;
#pragma omp parallel for schedule(static, 1) num_threads(T)
  for (int t = 0; t < T; ++t)
    for (uint32_t s : pcs[t].src) __atomic_fetch_add(&np[s], (P)1, __ATOMIC_RELAXED);
  std::vector<uint64_t> block(size_t(T) + 1, 0);
#pragma omp parallel num_threads(T)
  {
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
    const uint64_t lo = uint64_t(n) * t / nt, hi = uint64_t(n) * (t + 1) / nt;
    uint64_t acc = 0;
    for (uint64_t v = lo; v < hi; ++v) acc += np[v];
    block[t + 1] = acc;
#pragma omp barrier
#pragma omp single
    for (int k = 1; k <= nt; ++k) block[k] += block[k - 1];
    uint64_t run = block[t];
    for (uint64_t v = lo; v < hi; ++v) {
      const P c = np[v];
      np[v] = (P)run;
      run += c;
    }
  }
  np[n] = (P)m;
  std::vector<P> cur(np, np + n);
  uint32_t *ed = (uint32_t *)g->edges;
#pragma omp parallel num_threads(T)
  {
    const int j = omp_get_thread_num(), nt = omp_get_num_threads();
    const P e_lo = (P)(m * j / nt), e_hi = (P)(m * (j + 1) / nt);
    // first vertex whose row starts at or after e_lo / e_hi
    const uint32_t v_lo = j == 0 ? 0 : (uint32_t)(std::lower_bound(np, np + n, e_lo) - np);
    const uint32_t v_hi = j == nt - 1 ? n : (uint32_t)(std::lower_bound(np, np + n, e_hi) - np);
    if (v_lo < v_hi)
      for (const TextPiece &pc : pcs) {
        const size_t k = pc.src.size();
        for (size_t i = 0; i < k; ++i) {
          const uint32_t s = pc.src[i];
          if (s < v_lo || s >= v_hi) continue;
          const P pos = cur[s]++;
          if (weighted) { ed[2 * size_t(pos)] = pc.dst[i]; ed[2 * size_t(pos) + 1] = pc.w[i]; }
          else ed[pos] = pc.dst[i];
        }
      }
  }
}

static int load_text(const char *path, int weighted, sgw_graph **out) {
  int fd = open(path, O_RDONLY);
  if (fd < 0) return fail(SGW_EIO, "cannot open %s", path);
  struct stat sb;
  if (fstat(fd, &sb) != 0) { close(fd); return fail(SGW_EIO, "cannot stat %s", path); }
  const size_t size = (size_t)sb.st_size;
  if (size == 0) { close(fd); return fail(SGW_EFORMAT, "%s: no edges", path); }
  void *map = mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
  close(fd);
  if (map == MAP_FAILED) return fail(SGW_EIO, "cannot map %s", path);
  madvise(map, size, MADV_SEQUENTIAL);
  const char *base = (const char *)map;

  const int T = (int)std::max<size_t>(1, std::min<size_t>(omp_get_max_threads(), size / (1 << 20) + 1));
  std::vector<size_t> cut(size_t(T) + 1);
  for (int t = 0; t <= T; ++t) {
    size_t c = size * size_t(t) / size_t(T);
    if (t > 0 && t < T)
      while (c < size && base[c - 1] != '\n') ++c;  // first line starting at or after c
    cut[t] = c;
  }
  std::vector<TextPiece> pcs(T);
#pragma omp parallel for schedule(static, 1) num_threads(T)
  for (int t = 0; t < T; ++t)
    if (cut[t] < cut[t + 1]) parse_piece(base, cut[t], cut[t + 1], weighted, pcs[t]);

  for (int t = 0; t < T; ++t)  // pieces in file order: the first bad line wins
    if (pcs[t].bad_status != SGW_OK) {
      const char *line = base + pcs[t].bad_at;
      const char *eol = (const char *)memchr(line, '\n', size - pcs[t].bad_at);
      int len = (int)std::min<size_t>(eol ? size_t(eol - line) : size - pcs[t].bad_at, 200);
      std::string text(line, size_t(len));
      munmap(map, size);
      return pcs[t].bad_status == SGW_ERANGE
                 ? fail(SGW_ERANGE, "%s: value out of u32 range in '%s'", path, text.c_str())
                 : fail(SGW_EFORMAT, "%s: bad line '%s'", path, text.c_str());
    }
  munmap(map, size);

  uint64_t m = 0;
  uint32_t max_id = 0;
  bool any = false;
  for (const TextPiece &pc : pcs) {
    m += pc.src.size();
    if (!pc.src.empty()) { any = true; max_id = std::max(max_id, pc.max_id); }
  }
  if (!any) return fail(SGW_EFORMAT, "%s: no edges", path);
  const uint32_t n = max_id + 1;
  sgw_graph *g = nullptr;
  int st = graph_alloc(n, m, weighted, &g);
  if (st != SGW_OK) return st;
  if (g->node_pointer64) place_text_rows(g, pcs, T, g->node_pointer64);
  else place_text_rows(g, pcs, T, g->node_pointer);
  if (g->node_pointer64) {  // rows are built sorted and in range; only a degree can overflow
    int big = 0;
#pragma omp parallel for reduction(| : big)
    for (int64_t v = 0; v < (int64_t)n; ++v)
      if (g->node_pointer64[v + 1] - g->node_pointer64[v] >= (uint64_t(1) << 32)) big = 1;
    if (big) {
      sgw_graph_free(g);
      return fail(SGW_EFORMAT, "%s: %s", path, csr_problem(4));
    }
  }
  *out = g;
  return SGW_OK;
}

// Writes x in decimal at q and returns the end.
static inline char *put_u32(char *q, uint32_t x) {
  char d[10];
  int k = 0;
  do { d[k++] = char('0' + x % 10); x /= 10; } while (x);
  while (k) *q++ = d[--k];
  return q;
}

}  // namespace sgw

using namespace sgw;

extern "C" {

const char *sgw_strerror(int status) {
  switch (status) {
    case SGW_OK: return "ok";
    case SGW_EINVAL: return "invalid argument";
    case SGW_EIO: return "i/o error";
    case SGW_EFORMAT: return "unsupported or malformed graph file";
    case SGW_ENOMEM: return "out of host memory";
    case SGW_EBUDGET: return "device-memory budget too small";
    case SGW_ECUDA: return "CUDA error";
    case SGW_ETIMEOUT: return "bounded device wait timed out";
    case SGW_ESTATE: return "wrong engine state";
    case SGW_ERANGE: return "size out of range";
    default: return "unknown status";
  }
}

const char *sgw_last_error(void) { return g_err; }

int sgw_graph_load(const char *path, sgw_graph **out) {
  clear_error();
  if (!path || !out) return fail(SGW_EINVAL, "null argument");
  *out = nullptr;
  std::string ext = extension_of(path);
  if (ext == "bcsr") return load_binary(path, 0, false, out);
  if (ext == "bwcsr") return load_binary(path, 1, false, out);
  if (ext == "bcsr64") return load_binary(path, 0, true, out);
  if (ext == "bwcsr64") return load_binary(path, 1, true, out);
  if (ext == "el") return load_text(path, 0, out);
  if (ext == "wel") return load_text(path, 1, out);
  return fail(SGW_EFORMAT, "The graph format is not supported: '%s'", path);
}

int sgw_graph_from_csr(uint32_t n, uint32_t m, const uint32_t *node_pointer,
                       const void *edges, int weighted, sgw_graph **out) {
  clear_error();
  if (!out || !node_pointer || (m > 0 && !edges) || n == 0)
    return fail(SGW_EINVAL, "null argument or zero vertices");
  if (node_pointer[n] != m) return fail(SGW_EINVAL, "node_pointer[n] != m");
  sgw_graph *g = new (std::nothrow) sgw_graph();
  if (!g) return fail(SGW_ENOMEM, "graph object");
  g->n = n;
  g->m = m;
  g->weighted = weighted ? 1 : 0;
  g->esz = weighted ? 8 : 4;
  g->node_pointer = const_cast<uint32_t *>(node_pointer);
  g->edges = const_cast<void *>(edges);
  g->owns = false;
  // the device kernels index vertex arrays by edge endpoint: validate once
  if (const int bad = validate_csr(g)) {
    delete g;
    return fail(SGW_EINVAL, "%s", bad & 1 ? "node_pointer not monotone" : "edge endpoint >= n");
  }
  *out = g;
  return SGW_OK;
}

int sgw_graph_from_csr64(uint32_t n, uint64_t m, const uint64_t *node_pointer,
                         const void *edges, int weighted, sgw_graph **out) {
  clear_error();
  if (!out || !node_pointer || (m > 0 && !edges) || n == 0)
    return fail(SGW_EINVAL, "null argument or zero vertices");
  if (node_pointer[n] != m) return fail(SGW_EINVAL, "node_pointer[n] != m");
  sgw_graph *g = new (std::nothrow) sgw_graph();
  if (!g) return fail(SGW_ENOMEM, "graph object");
  g->n = n;
  g->m = m;
  g->weighted = weighted ? 1 : 0;
  g->esz = weighted ? 8 : 4;
  g->node_pointer64 = const_cast<uint64_t *>(node_pointer);
  g->edges = const_cast<void *>(edges);
  g->owns = false;
  if (const int bad = validate_csr(g)) {
    delete g;
    return fail(SGW_EINVAL, "%s", bad & 1 ? "node_pointer not monotone"
                                          : bad & 4 ? "out-degree of 2^32 or more" : "edge endpoint >= n");
  }
  *out = g;
  return SGW_OK;
}

int sgw_graph_info(const sgw_graph *g, uint32_t *n, uint32_t *m, int *weighted) {
  if (!g) return fail(SGW_EINVAL, "null graph");
  if (g->m >= (uint64_t(1) << 32))
    return fail(SGW_ERANGE, "%llu edges do not fit a u32 count (sgw_graph_info64)", (unsigned long long)g->m);
  if (n) *n = g->n;
  if (m) *m = (uint32_t)g->m;
  if (weighted) *weighted = g->weighted;
  return SGW_OK;
}

int sgw_graph_info64(const sgw_graph *g, uint32_t *n, uint64_t *m, int *weighted) {
  if (!g) return fail(SGW_EINVAL, "null graph");
  if (n) *n = g->n;
  if (m) *m = g->m;
  if (weighted) *weighted = g->weighted;
  return SGW_OK;
}

const uint32_t *sgw_graph_node_pointer(const sgw_graph *g) { return g ? g->node_pointer : nullptr; }
const uint64_t *sgw_graph_node_pointer64(const sgw_graph *g) { return g ? g->node_pointer64 : nullptr; }
const void *sgw_graph_edges(const sgw_graph *g) { return g ? g->edges : nullptr; }

int sgw_graph_out_degree(const sgw_graph *g, uint32_t *out_degree) {
  if (!g || !out_degree) return fail(SGW_EINVAL, "null argument");
#pragma omp parallel for
  for (int64_t v = 0; v < (int64_t)g->n; ++v) out_degree[v] = deg_at(g, (uint64_t)v);
  return SGW_OK;
}

int sgw_graph_save(const sgw_graph *g, const char *path) {
  clear_error();
  if (!g || !path) return fail(SGW_EINVAL, "null argument");
  std::string ext = extension_of(path);
  const bool bin64 = (ext == "bcsr64" || ext == "bwcsr64");
  const bool bin = bin64 || (ext == "bcsr" || ext == "bwcsr");
  bool txt = (ext == "el" || ext == "wel");
  if (!bin && !txt) return fail(SGW_EFORMAT, "unsupported extension for %s", path);
  bool want_w = (ext == "bwcsr" || ext == "bwcsr64" || ext == "wel");
  if (want_w && !g->weighted)
    return fail(SGW_EINVAL, "%s needs a weighted graph", path);
  if (bin && !bin64 && g->m >= (uint64_t(1) << 32))
    return fail(SGW_ERANGE, "%llu edges do not fit the u32 header of %s (write .%s64)",
                (unsigned long long)g->m, path, ext.c_str());
  FILE *f = fopen(path, "wb");
  if (!f) return fail(SGW_EIO, "cannot create %s", path);
  bool ok = true;
  const uint32_t *ed = (const uint32_t *)g->edges;
  const size_t stride = g->esz / 4;
  if (bin) {
    const size_t npsz = bin64 ? 8 : 4;
    if (bin64) {
      const uint64_t hdr[2] = {g->n, g->m};
      ok = fwrite(hdr, 8, 2, f) == 2;
    } else {
      const uint32_t hdr[2] = {g->n, (uint32_t)g->m};
      ok = fwrite(hdr, 4, 2, f) == 2;
    }
    if (ok && (npsz == 8) == (g->node_pointer64 != nullptr)) {
      const void *np = g->node_pointer64 ? (const void *)g->node_pointer64 : (const void *)g->node_pointer;
      ok = fwrite(np, npsz, g->n, f) == g->n;
    } else if (ok) {  // widen or narrow in blocks
      std::vector<char> buf(npsz << 20);
      for (uint32_t v0 = 0; ok && v0 < g->n; v0 += 1u << 20) {
        const uint32_t k = std::min<uint32_t>(g->n - v0, 1u << 20);
        for (uint32_t i = 0; i < k; ++i) {
          const uint64_t x = np_at(g, uint64_t(v0) + i);
          if (npsz == 8) reinterpret_cast<uint64_t *>(buf.data())[i] = x;
          else reinterpret_cast<uint32_t *>(buf.data())[i] = (uint32_t)x;
        }
        ok = fwrite(buf.data(), npsz, k, f) == k;
      }
    }
    if (ok && want_w == (bool)g->weighted) {
      size_t total = size_t(g->m) * g->esz, done = 0;
      while (ok && done < total) {
        size_t piece = std::min(total - done, size_t(256) << 20);
        ok = fwrite((const char *)g->edges + done, 1, piece, f) == piece;
        done += piece;
      }
    } else if (ok) {  // unweighted file from a weighted graph: ends only
      std::vector<uint32_t> buf;
      buf.reserve(1 << 20);
      for (size_t i = 0; ok && i < g->m; ++i) {
        buf.push_back(ed[i * stride]);
        if (buf.size() == (1u << 20) || i + 1 == g->m) {
          ok = fwrite(buf.data(), 4, buf.size(), f) == buf.size();
          buf.clear();
        }
      }
    }
  } else {
    // text: vertex blocks of about 2^24 edges, each formatted by T threads
    // into their own buffers and written in order
    const int T = omp_get_max_threads();
    std::vector<std::string> bufs(T);
    auto row_of = [&](uint32_t lo, uint32_t hi, uint64_t e) {  // last v in [lo, hi) with np[v] <= e
      while (hi - lo > 1) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (np_at(g, mid) <= e) lo = mid; else hi = mid;
      }
      return lo;
    };
    uint32_t v0 = 0;
    while (ok && v0 < g->n) {
      const uint64_t e0 = np_at(g, v0);
      uint32_t v1 = row_of(v0, g->n + 1, e0 + (1u << 24)) + 1;
      v1 = std::min(std::max(v1, v0 + 1), g->n);
      const uint64_t span = np_at(g, v1) - e0;
#pragma omp parallel num_threads(T)
      {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        const uint64_t lo_e = e0 + span * t / nt, hi_e = e0 + span * (t + 1) / nt;
        std::string &b = bufs[t];
        b.clear();
        b.reserve(size_t(hi_e - lo_e) * (want_w ? 24 : 20));
        // the vertex whose row holds edge lo_e
        uint32_t v = row_of(v0, v1 + 1, lo_e);
        char tmp[40];
        for (uint64_t i = lo_e; i < hi_e; ++i) {
          while (np_at(g, uint64_t(v) + 1) <= i) ++v;
          char *q = tmp;
          q = put_u32(q, v);
          *q++ = ' ';
          q = put_u32(q, ed[size_t(i) * stride]);
          if (want_w) { *q++ = ' '; q = put_u32(q, ed[size_t(i) * stride + 1]); }
          *q++ = '\n';
          b.append(tmp, size_t(q - tmp));
        }
      }
      for (int t = 0; ok && t < T; ++t)
        ok = bufs[t].empty() || fwrite(bufs[t].data(), 1, bufs[t].size(), f) == bufs[t].size();
      v0 = v1;
    }
  }
  if (fclose(f) != 0) ok = false;
  return ok ? SGW_OK : fail(SGW_EIO, "write failed for %s", path);
}

int sgw_graph_clear_out_edges(sgw_graph *g, uint32_t v) {
  clear_error();
  if (!g) return fail(SGW_EINVAL, "null graph");
  if (v >= g->n) return fail(SGW_EINVAL, "vertex %u out of range (n=%u)", v, g->n);
  if (!g->owns || g->map_base)
    return fail(SGW_EINVAL, "only a graph whose arrays the library owns (loaded or generated) can be changed");
  const uint64_t a = np_at(g, v), b = np_at(g, uint64_t(v) + 1), d = b - a;
  if (d == 0) return SGW_OK;
  char *ed = static_cast<char *>(g->edges);
  memmove(ed + a * g->esz, ed + b * g->esz, size_t(g->m - b) * g->esz);
#pragma omp parallel for
  for (int64_t u = (int64_t)v + 1; u <= (int64_t)g->n; ++u) np_set(g, (uint64_t)u, np_at(g, (uint64_t)u) - d);
  g->m -= d;
  g->wmax_cache.store(-1, std::memory_order_relaxed);
  return SGW_OK;
}

int sgw_trace_write_csv(const sgw_trace_rec *recs, uint64_t count, const char *path) {
  clear_error();
  if (!path || (count && !recs)) return fail(SGW_EINVAL, "null argument");
  FILE *f = fopen(path, "w");
  if (!f) return fail(SGW_EIO, "cannot create %s", path);
  bool ok = fprintf(f, "global_iteration,partition,num_partitions,inner_iterations,active_nodes,first_vertex,"
                       "active_edges,iteration_active_nodes,iteration_active_edges,bytes_h2d,transfer\n") > 0;
  for (uint64_t i = 0; ok && i < count; ++i) {
    const sgw_trace_rec &r = recs[i];
    ok = fprintf(f, "%u,%u,%u,%u,%u,%u,%llu,%llu,%llu,%llu,%u\n", r.global_iteration, r.partition,
                 r.num_partitions, r.inner_iterations, r.active_nodes, r.first_vertex,
                 (unsigned long long)r.active_edges, (unsigned long long)r.iteration_active_nodes,
                 (unsigned long long)r.iteration_active_edges, (unsigned long long)r.bytes_h2d,
                 r.transfer) > 0;
  }
  if (fclose(f) != 0) ok = false;
  return ok ? SGW_OK : fail(SGW_EIO, "write failed for %s", path);
}

void sgw_graph_free(sgw_graph *g) {
  if (!g) return;
  if (g->map_base) {
    host_free(g->node_pointer);
    host_free(g->node_pointer64);
    munmap(g->map_base, g->map_len);
  } else if (g->owns) {
    host_free(g->node_pointer);
    host_free(g->node_pointer64);
    host_free(g->edges);
  }
  delete g;
}

int sgw_graph_map(const char *path, sgw_graph **out) {
  clear_error();
  if (!path || !out) return fail(SGW_EINVAL, "null argument");
  *out = nullptr;
  const std::string ext = extension_of(path);
  const bool wide_file = ext == "bcsr64" || ext == "bwcsr64";
  if (ext != "bcsr" && ext != "bwcsr" && !wide_file)
    return fail(SGW_EFORMAT, "only .bcsr/.bwcsr(64) files can be mapped: '%s'", path);
  const int weighted = ext == "bwcsr" || ext == "bwcsr64";
  int fd = open(path, O_RDONLY);
  if (fd < 0) return fail(SGW_EIO, "cannot open %s", path);
  BinHeader h;
  int st = read_header(fd, path, wide_file, weighted, &h);
  if (st != SGW_OK) { close(fd); return st; }
  const uint32_t n = (uint32_t)h.n, esz = weighted ? 8 : 4;
  const size_t want = h.hdr + h.npsz * size_t(n) + size_t(h.m) * esz;
  if (weighted && !wide_file && (n & 1u)) {  // 8-byte records would start 4 bytes off an 8-byte boundary
    close(fd);
    return load_binary(path, weighted, wide_file, out);
  }
  void *base = mmap(nullptr, want, PROT_READ, MAP_SHARED, fd, 0);
  close(fd);
  if (base == MAP_FAILED) return fail(SGW_EIO, "cannot map %s", path);
  madvise(base, want, MADV_WILLNEED);
  // the node pointers are copied (u32 below 2^32 edges, else u64); the
  // records stay in the mapping
  const bool wide = h.m >= (uint64_t(1) << 32);
  void *np = host_alloc((wide ? 8 : 4) * (size_t(n) + 1), nullptr);
  sgw_graph *g = np ? new (std::nothrow) sgw_graph() : nullptr;
  if (!g) {
    host_free(np);
    munmap(base, want);
    return fail(SGW_ENOMEM, "graph arrays (n=%u)", n);
  }
  g->n = n;
  g->m = h.m;
  g->weighted = weighted;
  g->esz = esz;
  g->owns = false;
  if (wide) g->node_pointer64 = (uint64_t *)np;
  else g->node_pointer = (uint32_t *)np;
  const bool fits = fill_pointers(g, (const char *)base + h.hdr, h.npsz);
  g->edges = (char *)base + h.hdr + h.npsz * size_t(n);
  g->map_base = base;
  g->map_len = want;
  if (const int bad = fits ? validate_csr(g) : 1) {
    sgw_graph_free(g);
    return fail(SGW_EFORMAT, "%s: %s", path, csr_problem(bad));
  }
  *out = g;
  return SGW_OK;
}

int sgw_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b,
                 double c, uint64_t seed, int weighted, uint32_t wmax,
                 sgw_graph **out) {
  clear_error();
  if (!out || scale == 0 || scale > 31 || edge_factor == 0 || a < 0 || b < 0 ||
      c < 0 || a + b + c > 1.0 || (weighted && wmax == 0))
    return fail(SGW_EINVAL, "bad R-MAT parameters");
  RmatParams p;
  p.scale = scale;
  const double two32 = 4294967296.0;
  p.ta = (uint64_t)(a * two32);
  p.tab = (uint64_t)((a + b) * two32);
  p.tabc = (uint64_t)((a + b + c) * two32);
  p.seed = mix64(seed ^ 0x6a09e667f3bcc909ULL);
  uint32_t n = 1u << scale;
  uint64_t m0 = uint64_t(edge_factor) << scale;
  uint32_t drop = n >= 2 ? n - 2 : 0xffffffffu;
  return build_csr(n, m0, [&](uint64_t e, uint32_t *s, uint32_t *d) { rmat_edge(p, e, s, d); },
                   drop, weighted, wmax, mix64(seed ^ 0xbb67ae8584caa73bULL), out);
}

int sgw_gen_er(uint32_t n, uint64_t m, uint64_t seed, int weighted,
               uint32_t wmax, sgw_graph **out) {
  clear_error();
  if (!out || n < 2 || (weighted && wmax == 0)) return fail(SGW_EINVAL, "bad ER parameters");
  uint64_t s2 = mix64(seed ^ 0x3c6ef372fe94f82bULL);
  return build_csr(n, m, [&](uint64_t e, uint32_t *s, uint32_t *d) { er_edge(s2, n, e, s, d); },
                   n - 2, weighted, wmax, mix64(seed ^ 0xbb67ae8584caa73bULL), out);
}

int sgw_graph_symmetrize(const sgw_graph *g, sgw_graph **out) {
  clear_error();
  if (!g || !out) return fail(SGW_EINVAL, "null argument");
  if (g->weighted) return fail(SGW_EINVAL, "symmetrize expects an unweighted graph");
  const uint32_t *ed = (const uint32_t *)g->edges;
  const uint32_t n = g->n;
  // edge e < m is the forward edge, e >= m the reverse of edge e - m
  std::vector<uint32_t> srcof(g->m);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < (int64_t)n; ++v)
    for (uint64_t i = np_at(g, (uint64_t)v), e = np_at(g, (uint64_t)v + 1); i < e; ++i) srcof[i] = (uint32_t)v;
  const uint64_t m = g->m;
  // vertex n-2 keeps no out-edges, as in the generators
  return build_csr(n, 2 * m,
                   [&](uint64_t e, uint32_t *s, uint32_t *d) {
                     if (e < m) { *s = srcof[e]; *d = ed[e]; }
                     else { *s = ed[e - m]; *d = srcof[e - m]; }
                   },
                   n >= 2 ? n - 2 : 0xffffffffu, 0, 1, 0, out);
}

static uint32_t uf_find(std::atomic<uint32_t> *par, uint32_t x) {
  while (true) {
    uint32_t p = par[x].load(std::memory_order_relaxed);
    if (p == x) return x;
    uint32_t gp = par[p].load(std::memory_order_relaxed);
    if (gp != p) par[x].compare_exchange_weak(p, gp, std::memory_order_relaxed);
    x = gp;
  }
}

static void wcc_labels(const sgw_graph *g, std::vector<uint32_t> &root) {
  const uint32_t n = g->n;
  const uint32_t *ed = (const uint32_t *)g->edges;
  const size_t stride = g->esz / 4;
  std::atomic<uint32_t> *par = new std::atomic<uint32_t>[n];
#pragma omp parallel for
  for (int64_t v = 0; v < (int64_t)n; ++v) par[v].store((uint32_t)v, std::memory_order_relaxed);
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t v = 0; v < (int64_t)n; ++v) {
    for (uint64_t i = np_at(g, (uint64_t)v), e = np_at(g, (uint64_t)v + 1); i < e; ++i) {
      uint32_t a = (uint32_t)v, b = ed[size_t(i) * stride];
      while (true) {
        a = uf_find(par, a);
        b = uf_find(par, b);
        if (a == b) break;
        if (a < b) std::swap(a, b);  // link the larger root under the smaller
        uint32_t exp = a;
        if (par[a].compare_exchange_strong(exp, b, std::memory_order_relaxed)) break;
      }
    }
  }
  root.resize(n);
#pragma omp parallel for
  for (int64_t v = 0; v < (int64_t)n; ++v) root[v] = uf_find(par, (uint32_t)v);
  delete[] par;
}

int sgw_largest_wcc(const sgw_graph *g, uint32_t *vertices, uint64_t *edges) {
  clear_error();
  if (!g) return fail(SGW_EINVAL, "null graph");
  std::vector<uint32_t> root;
  wcc_labels(g, root);
  std::vector<uint32_t> size(g->n, 0);
  std::vector<uint64_t> esum(g->n, 0);
  for (uint32_t v = 0; v < g->n; ++v) {
    size[root[v]]++;
    esum[root[v]] += deg_at(g, v);
  }
  uint32_t best = 0;
  for (uint32_t v = 1; v < g->n; ++v)
    if (size[v] > size[best]) best = v;
  if (vertices) *vertices = size[best];
  if (edges) *edges = esum[best];
  return SGW_OK;
}

int sgw_pick_sources(const sgw_graph *g, uint32_t count, uint64_t seed, uint32_t *out) {
  clear_error();
  if (!g || (!out && count)) return fail(SGW_EINVAL, "null argument");
  std::vector<uint32_t> root;
  wcc_labels(g, root);
  std::vector<uint32_t> size(g->n, 0);
  for (uint32_t v = 0; v < g->n; ++v) size[root[v]]++;
  uint32_t best = 0;
  for (uint32_t v = 1; v < g->n; ++v)
    if (size[v] > size[best]) best = v;
  std::vector<uint32_t> cand;
  for (uint32_t v = 0; v < g->n; ++v)
    if (root[v] == best && deg_at(g, v) > 0) cand.push_back(v);
  if (cand.empty()) return fail(SGW_EINVAL, "no vertex with out-edges");
  SplitMix rng(mix64(seed ^ 0xa54ff53a5f1d36f1ULL));
  std::vector<uint32_t> chosen;
  for (uint32_t k = 0; k < count; ++k) {
    uint32_t v;
    int tries = 0;
    do {
      v = cand[(uint32_t)(((rng.next() >> 32) * cand.size()) >> 32)];
    } while (count <= cand.size() && ++tries < 1000 &&
             std::find(chosen.begin(), chosen.end(), v) != chosen.end());
    chosen.push_back(v);
    out[k] = v;
  }
  return SGW_OK;
}

int sgw_plan_partitions(const uint32_t *ptr, uint32_t count, uint64_t cap,
                        uint32_t *from_node, uint32_t *node_size,
                        uint32_t capacity, uint32_t *num_partitions) {
  clear_error();
  if (!ptr || !num_partitions || cap == 0) return fail(SGW_EINVAL, "bad arguments");
  uint32_t p = 0, from = 0;
  while (from < count) {
    uint32_t to = plan_next(ptr, from, count, cap);
    if (p < capacity) {
      if (from_node) from_node[p] = from;
      if (node_size) node_size[p] = to - from;
    }
    ++p;
    from = to;
  }
  *num_partitions = p;
  if (p > capacity) return fail(SGW_ERANGE, "%u partitions exceed capacity %u", p, capacity);
  return SGW_OK;
}

}  // extern "C"

/*
 * sst_oracle.c -- CPU restatement of SSTGraph's hot path (TEST
 * INFRASTRUCTURE: the checker for the CUDA library, and the "port" CPU
 * baseline; see sst_oracle.h for what is restated from where).
 *
 * Storage is one sorted, duplicate-free uint32 array per vertex.  A batch is
 * sorted by (row, col) with an LSD radix sort, then each touched row merges
 * its run (insert) or subtracts it (remove); rows are independent, so rows
 * run in parallel, as the reference parallelises over row chunks
 * (include/SSTGraph/SparseMatrix.hpp:582-607).
 */
#include "sst_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* hashes                                                               */
/* ------------------------------------------------------------------ */

/* splitmix64 output function (Steele, Lea, Flood 2014; constants as
 * published by Vigna) */
uint64_t sst_o_mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}

/* counter-based draw j of item i in stream seed */
uint64_t sst_o_draw(uint64_t seed, uint64_t i, uint64_t j) {
  return sst_o_mix64(sst_o_mix64(seed * 0x9E3779B97F4A7C15ULL + i) ^
                     (j * 0xD1B54A32D192ED03ULL + 0x8CB92BA72F3D8DD7ULL));
}

/* include/SSTGraph/internal/rmat_util.h:29-39 */
uint64_t sst_o_ref_hash64(uint64_t u) {
  uint64_t v = u * 3935559000370003845ULL + 2691343689449507681ULL;
  v ^= v >> 21;
  v ^= v << 37;
  v ^= v >> 4;
  v *= 4768777513237032717ULL;
  v ^= v << 20;
  v ^= v >> 41;
  v ^= v << 5;
  return v;
}

/* include/SSTGraph/internal/rmat_util.h:42-50 */
uint32_t sst_o_ref_hash32(uint32_t a) {
  a = (a + 0x7ed55d16u) + (a << 12);
  a = (a ^ 0xc761c23cu) ^ (a >> 19);
  a = (a + 0x165667b1u) + (a << 5);
  a = (a + 0xd3a2646cu) ^ (a << 9);
  a = (a + 0xfd7046c5u) + (a << 3);
  a = (a ^ 0xb55a4f09u) ^ (a >> 16);
  return a;
}

/* ------------------------------------------------------------------ */
/* generators                                                           */
/* ------------------------------------------------------------------ */

static void rmat_thresholds(double a, double b, double c, uint64_t t[3]) {
  t[0] = (uint64_t)(a * 4294967296.0);
  t[1] = (uint64_t)((a + b) * 4294967296.0);
  t[2] = (uint64_t)((a + b + c) * 4294967296.0);
}

/* Recursive-matrix edges: level l (most significant bit first) picks a
 * quadrant with a 32-bit uniform draw against fixed-point thresholds. */
void sst_o_rmat(uint32_t scale, double a, double b, double c, uint64_t seed,
                uint64_t first, uint64_t count, uint32_t *pairs) {
  uint64_t t[3];
  rmat_thresholds(a, b, c, t);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)count; i++) {
    uint64_t idx = first + (uint64_t)i;
    uint32_t u = 0, v = 0;
    uint64_t h = 0;
    for (uint32_t l = 0; l < scale; l++) {
      if ((l & 1) == 0) h = sst_o_draw(seed, idx, l >> 1);
      uint64_t r = (l & 1) ? (h >> 32) : (h & 0xffffffffULL);
      uint32_t bit = 1u << (scale - 1 - l);
      if (r < t[0]) {
      } else if (r < t[1]) {
        v |= bit;
      } else if (r < t[2]) {
        u |= bit;
      } else {
        u |= bit;
        v |= bit;
      }
    }
    pairs[2 * i] = u;
    pairs[2 * i + 1] = v;
  }
}

void sst_o_er(uint32_t n, uint64_t seed, uint64_t first, uint64_t count,
              uint32_t *pairs) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)count; i++) {
    uint64_t h = sst_o_draw(seed, first + (uint64_t)i, 0);
    pairs[2 * i] = (uint32_t)(((h & 0xffffffffULL) * n) >> 32);
    pairs[2 * i + 1] = (uint32_t)(((h >> 32) * n) >> 32);
  }
}

/* rMat<uint32_t>::operator() of include/SSTGraph/internal/rmat_util.h:82-131
 * unrolled: level k (k = 0 for the top, n/2 bit) draws
 * hash32(randStart + k*randStride) / INT32_MAX, which lies in [0, 2). */
void sst_o_ref_rmat_stream(uint32_t nn, double a, double b, double c,
                           uint64_t first, uint64_t count, uint32_t *pairs) {
  const double ab = a + b, abc = a + b + c;
  /* random_aspen().ith_rand(0) = hash64(0), truncated to the uint32 seed */
  const uint32_t h = sst_o_ref_hash32((uint32_t)sst_o_ref_hash64(0));
  uint32_t levels = 0;
  while ((1u << levels) < nn) levels++;
#pragma omp parallel for schedule(static)
  for (int64_t ii = 0; ii < (int64_t)count; ii++) {
    uint32_t i = (uint32_t)(first + (uint64_t)ii);
    uint32_t start = sst_o_ref_hash32((uint32_t)(2u * i) * h);
    uint32_t stride = sst_o_ref_hash32((uint32_t)(2u * i + 1u) * h);
    uint32_t u = 0, v = 0;
    for (uint32_t k = 0; k < levels; k++) {
      uint32_t half = (nn >> k) / 2;
      double r = (double)sst_o_ref_hash32(start + k * stride) / 2147483647.0;
      if (r < a) {
      } else if (r < ab) {
        v += half;
      } else if (r < abc) {
        u += half;
      } else {
        u += half;
        v += half;
      }
    }
    pairs[2 * ii] = u;
    pairs[2 * ii + 1] = v;
  }
}

/* ------------------------------------------------------------------ */
/* graph storage                                                        */
/* ------------------------------------------------------------------ */

struct sst_o_graph {
  uint32_t n;
  uint32_t width; /* column ids are < width (SparseMatrixV(height, width)) */
  uint32_t *deg;
  uint32_t *cap;
  uint32_t **adj;
};

sst_o_graph *sst_o_new2(uint32_t n, uint32_t width) {
  sst_o_graph *g = (sst_o_graph *)calloc(1, sizeof(sst_o_graph));
  g->n = n;
  g->width = width;
  g->deg = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
  g->cap = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
  g->adj = (uint32_t **)calloc(n ? n : 1, sizeof(uint32_t *));
  return g;
}

void sst_o_free(sst_o_graph *g) {
  if (!g) return;
  for (uint32_t v = 0; v < g->n; v++) free(g->adj[v]);
  free(g->adj);
  free(g->cap);
  free(g->deg);
  free(g);
}

uint32_t sst_o_num_nodes(const sst_o_graph *g) { return g->n; }

/* LSD radix sort of 64-bit keys, 16-bit digits, parallel histograms */
static void radix_sort_u64(uint64_t *keys, uint64_t n, int key_bits) {
  if (n < 2) return;
  uint64_t *tmp = (uint64_t *)malloc(n * sizeof(uint64_t));
  int nthreads = 1;
#ifdef _OPENMP
  nthreads = omp_get_max_threads();
#endif
  const int R = 1 << 16;
  uint64_t *hist = (uint64_t *)malloc((size_t)nthreads * R * sizeof(uint64_t));
  uint64_t *src = keys, *dst = tmp;
  int passes = 0;
  for (int shift = 0; shift < key_bits; shift += 16, passes++) {
    memset(hist, 0, (size_t)nthreads * R * sizeof(uint64_t));
#pragma omp parallel num_threads(nthreads)
    {
      int t = 0;
#ifdef _OPENMP
      t = omp_get_thread_num();
#endif
      uint64_t lo = n * (uint64_t)t / nthreads, hi = n * (uint64_t)(t + 1) / nthreads;
      uint64_t *h = hist + (size_t)t * R;
      for (uint64_t i = lo; i < hi; i++) h[(src[i] >> shift) & (R - 1)]++;
#pragma omp barrier
#pragma omp single
      {
        uint64_t sum = 0;
        for (int d = 0; d < R; d++)
          for (int tt = 0; tt < nthreads; tt++) {
            uint64_t c = hist[(size_t)tt * R + d];
            hist[(size_t)tt * R + d] = sum;
            sum += c;
          }
      }
      for (uint64_t i = lo; i < hi; i++) {
        uint64_t k = src[i];
        dst[h[(k >> shift) & (R - 1)]++] = k;
      }
    }
    uint64_t *s = src;
    src = dst;
    dst = s;
  }
  if (src != keys) memcpy(keys, src, n * sizeof(uint64_t));
  free(hist);
  free(tmp);
}

static int bits_for(uint64_t x) {
  int b = 0;
  while (b < 64 && (x >> b) != 0) b++;
  return b;
}

/* sorted, duplicate-free (row<<32|col) keys of the valid pairs; self-loops
 * are dropped when drop_loops is set */
static uint64_t prepare_batch(const sst_o_graph *g, const uint32_t *pairs,
                              uint64_t b, int drop_loops, uint64_t **out) {
  uint64_t *keys = (uint64_t *)malloc((b ? b : 1) * sizeof(uint64_t));
  uint64_t k = 0;
  for (uint64_t i = 0; i < b; i++) {
    uint32_t r = pairs[2 * i], c = pairs[2 * i + 1];
    if (r >= g->n || c >= g->width) continue;
    if (drop_loops && r == c) continue;
    keys[k++] = ((uint64_t)r << 32) | c;
  }
  radix_sort_u64(keys, k, 32 + bits_for(g->n ? g->n - 1 : 0));
  uint64_t u = 0;
  for (uint64_t i = 0; i < k; i++)
    if (i == 0 || keys[i] != keys[i - 1]) keys[u++] = keys[i];
  *out = keys;
  return u;
}

static uint64_t row_runs(const uint64_t *keys, uint64_t k, uint64_t **starts) {
  uint64_t *s = (uint64_t *)malloc((k + 1) * sizeof(uint64_t));
  uint64_t r = 0;
  for (uint64_t i = 0; i < k; i++)
    if (i == 0 || (keys[i] >> 32) != (keys[i - 1] >> 32)) s[r++] = i;
  s[r] = k;
  *starts = s;
  return r;
}

/* SparseMatrixV::insert_batch semantics (SparseMatrix.hpp:556-643): set
 * union per row, self-loops skipped (:570,602) */
void sst_o_insert_batch(sst_o_graph *g, const uint32_t *pairs, uint64_t b) {
  uint64_t *keys, *runs;
  uint64_t k = prepare_batch(g, pairs, b, 1, &keys);
  uint64_t nr = row_runs(keys, k, &runs);
#pragma omp parallel for schedule(dynamic, 8)
  for (int64_t r = 0; r < (int64_t)nr; r++) {
    uint64_t s = runs[r], e = runs[r + 1];
    uint32_t v = (uint32_t)(keys[s] >> 32);
    uint32_t d = g->deg[v];
    uint64_t need = (uint64_t)d + (e - s);
    uint32_t *out = (uint32_t *)malloc(need * sizeof(uint32_t));
    const uint32_t *a = g->adj[v];
    uint64_t i = 0, j = s, o = 0;
    while (i < d || j < e) {
      if (j == e || (i < d && a[i] < (uint32_t)keys[j])) {
        out[o++] = a[i++];
      } else if (i == d || (uint32_t)keys[j] < a[i]) {
        out[o++] = (uint32_t)keys[j++];
      } else {
        out[o++] = a[i++];
        j++;
      }
    }
    free(g->adj[v]);
    g->adj[v] = out;
    g->deg[v] = (uint32_t)o;
    g->cap[v] = (uint32_t)need;
  }
  free(runs);
  free(keys);
}

/* SparseMatrixV::remove_batch semantics (SparseMatrix.hpp:645-718): set
 * difference per row; removing an absent edge is a no-op
 * (PMA.hpp:1226-1228) */
void sst_o_remove_batch(sst_o_graph *g, const uint32_t *pairs, uint64_t b) {
  uint64_t *keys, *runs;
  uint64_t k = prepare_batch(g, pairs, b, 0, &keys);
  uint64_t nr = row_runs(keys, k, &runs);
#pragma omp parallel for schedule(dynamic, 8)
  for (int64_t r = 0; r < (int64_t)nr; r++) {
    uint64_t s = runs[r], e = runs[r + 1];
    uint32_t v = (uint32_t)(keys[s] >> 32);
    uint32_t d = g->deg[v];
    uint32_t *a = g->adj[v];
    uint64_t i = 0, j = s, o = 0;
    while (i < d) {
      while (j < e && (uint32_t)keys[j] < a[i]) j++;
      if (j < e && (uint32_t)keys[j] == a[i]) {
        i++;
        j++;
      } else {
        a[o++] = a[i++];
      }
    }
    g->deg[v] = (uint32_t)o;
    if (o == 0) {
      free(g->adj[v]);
      g->adj[v] = NULL;
      g->cap[v] = 0;
    }
  }
  free(runs);
  free(keys);
}

uint64_t sst_o_M(const sst_o_graph *g) {
  uint64_t m = 0;
  for (uint32_t v = 0; v < g->n; v++) m += g->deg[v];
  return m;
}

uint32_t sst_o_degree(const sst_o_graph *g, uint32_t v) { return g->deg[v]; }

void sst_o_degrees(const sst_o_graph *g, uint32_t *out) {
  memcpy(out, g->deg, (size_t)g->n * sizeof(uint32_t));
}

static int64_t lower_bound_u32(const uint32_t *a, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo) / 2;
    if (a[mid] < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

int sst_o_has(const sst_o_graph *g, uint32_t r, uint32_t c) {
  if (r >= g->n) return 0;
  int64_t p = lower_bound_u32(g->adj[r], g->deg[r], c);
  return p < g->deg[r] && g->adj[r][p] == c;
}

void sst_o_to_csr(const sst_o_graph *g, uint64_t *offsets, uint32_t *cols) {
  uint64_t pos = 0;
  for (uint32_t v = 0; v < g->n; v++) {
    offsets[v] = pos;
    if (g->deg[v]) memcpy(cols + pos, g->adj[v], g->deg[v] * sizeof(uint32_t));
    pos += g->deg[v];
  }
  offsets[g->n] = pos;
}

/* |N(a) n N(b)|, or with early_end only the common w < a, w < b
 * (SparseMatrix.hpp:61-71, TinySet_small.hpp:357-407) */
uint64_t sst_o_common_neighbors(const sst_o_graph *g, uint32_t a, uint32_t b,
                                int early_end) {
  const uint32_t *x = g->adj[a], *y = g->adj[b];
  uint32_t nx = g->deg[a], ny = g->deg[b];
  if (early_end) {
    nx = (uint32_t)lower_bound_u32(x, nx, a);
    ny = (uint32_t)lower_bound_u32(y, ny, b);
  }
  uint64_t cnt = 0;
  uint32_t i = 0, j = 0;
  while (i < nx && j < ny) {
    if (x[i] < y[j])
      i++;
    else if (y[j] < x[i])
      j++;
    else {
      cnt++;
      i++;
      j++;
    }
  }
  return cnt;
}

/* SparseMatrix.hpp:436-454 */
uint64_t sst_o_touch_all_sum(const sst_o_graph *g) {
  uint64_t s = 0;
#pragma omp parallel for reduction(+ : s) schedule(dynamic, 1024)
  for (int64_t v = 0; v < (int64_t)g->n; v++)
    for (uint32_t i = 0; i < g->deg[v]; i++) s += g->adj[v][i];
  return s;
}

static uint64_t mulhi64(uint64_t a, uint64_t b) {
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
}

void sst_o_sample_edges(const sst_o_graph *g, uint64_t seed, uint64_t first,
                        uint64_t count, uint32_t *pairs) {
  uint64_t *pre = (uint64_t *)malloc(((size_t)g->n + 1) * sizeof(uint64_t));
  pre[0] = 0;
  for (uint32_t v = 0; v < g->n; v++) pre[v + 1] = pre[v] + g->deg[v];
  uint64_t m = pre[g->n];
  for (uint64_t i = 0; i < count; i++) {
    if (m == 0) {
      pairs[2 * i] = pairs[2 * i + 1] = 0;
      continue;
    }
    uint64_t rank = mulhi64(sst_o_draw(seed, first + i, 0), m);
    /* last v with pre[v] <= rank */
    uint32_t lo = 0, hi = g->n;
    while (hi - lo > 1) {
      uint32_t mid = lo + (hi - lo) / 2;
      if (pre[mid] <= rank)
        lo = mid;
      else
        hi = mid;
    }
    pairs[2 * i] = lo;
    pairs[2 * i + 1] = g->adj[lo][rank - pre[lo]];
  }
  free(pre);
}

/* ------------------------------------------------------------------ */
/* algorithms                                                           */
/* ------------------------------------------------------------------ */

/* BFS depths; -1 = unreached.  The reference returns parents and derives
 * depths by chasing them (internal/test.hpp:486-509); depths are unique, so
 * they are the parity target.  Level-synchronous over the host threads:
 * each level's vertices claim unvisited neighbours with a compare-and-swap,
 * so the depths do not depend on the claim order. */
static int nthreads_max(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
static int thread_id(void) {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

/* vertices reached, in level order, into order[] (may be NULL); returns
 * their count */
static uint64_t bfs_levels(const sst_o_graph *g, uint32_t src, int32_t *depth,
                           uint32_t *order) {
  const uint32_t n = g->n;
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; v++) depth[v] = -1;
  if (src >= n) return 0;
  uint32_t *q = order ? order : (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
  const int nt = nthreads_max();
  uint32_t **buf = (uint32_t **)calloc((size_t)nt, sizeof(uint32_t *));
  uint64_t *bcap = (uint64_t *)calloc((size_t)nt, sizeof(uint64_t));
  uint64_t *bcnt = (uint64_t *)calloc((size_t)nt + 1, sizeof(uint64_t));
  uint64_t head = 0, tail = 1;
  q[0] = src;
  depth[src] = 0;
  for (int32_t d = 0; head < tail; d++) {
    memset(bcnt, 0, ((size_t)nt + 1) * sizeof(uint64_t));
#pragma omp parallel
    {
      const int t = thread_id();
#pragma omp for schedule(dynamic, 64)
      for (int64_t k = (int64_t)head; k < (int64_t)tail; k++) {
        const uint32_t v = q[k];
        for (uint32_t i = 0; i < g->deg[v]; i++) {
          const uint32_t w = g->adj[v][i];
          int32_t expect = -1;
          if (depth[w] < 0 &&
              __atomic_compare_exchange_n(&depth[w], &expect, d + 1, 0, __ATOMIC_RELAXED,
                                          __ATOMIC_RELAXED)) {
            if (bcnt[t] == bcap[t]) {
              bcap[t] = bcap[t] ? 2 * bcap[t] : 1024;
              buf[t] = (uint32_t *)realloc(buf[t], bcap[t] * sizeof(uint32_t));
            }
            buf[t][bcnt[t]++] = w;
          }
        }
      }
    }
    uint64_t at = tail;
    for (int t = 0; t < nt; t++) {
      memcpy(q + at, buf[t], bcnt[t] * sizeof(uint32_t));
      at += bcnt[t];
    }
    head = tail;
    tail = at;
  }
  for (int t = 0; t < nt; t++) free(buf[t]);
  free(buf);
  free(bcap);
  free(bcnt);
  if (!order) free(q);
  return tail;
}

void sst_o_bfs(const sst_o_graph *g, uint32_t src, int32_t *depth) {
  bfs_levels(g, src, depth, NULL);
}

/* PageRank, pull form over the (symmetric) neighbour sets, in FP64:
 *   p_0(v) = 1/n
 *   p_{k+1}(v) = (1-d)/n + d * sum_{u in N(v)} p_k(u) / deg(u)
 * summed in ascending u; rank held by a vertex of degree 0 is not
 * redistributed.  Exactly `iters` iterations (the reference drivers call
 * PR_S<double>(g, 10), internal/test.hpp:527). */
void sst_o_pagerank(const sst_o_graph *g, uint32_t iters, double damping,
                    double *rank) {
  uint32_t n = g->n;
  double *contrib = (double *)malloc((size_t)(n ? n : 1) * sizeof(double));
  const double base = (1.0 - damping) / (double)n;
  for (uint32_t v = 0; v < n; v++) rank[v] = 1.0 / (double)n;
  for (uint32_t it = 0; it < iters; it++) {
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t)n; v++)
      contrib[v] = g->deg[v] ? rank[v] / (double)g->deg[v] : 0.0;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t v = 0; v < (int64_t)n; v++) {
      double s = 0.0;
      for (uint32_t i = 0; i < g->deg[v]; i++) s += contrib[g->adj[v][i]];
      rank[v] = base + damping * s;
    }
  }
  free(contrib);
}

/* connected components: label = smallest vertex id in the component.
 * Concurrent union-find over the host threads: a root is only ever linked
 * below a smaller root (compare-and-swap on the larger one), so every
 * component's final root is its smallest id. */
static uint32_t uf_find(uint32_t *par, uint32_t v) {
  for (;;) {
    uint32_t p = __atomic_load_n(&par[v], __ATOMIC_RELAXED);
    if (p == v) return v;
    uint32_t gp = __atomic_load_n(&par[p], __ATOMIC_RELAXED);
    if (gp != p) __atomic_compare_exchange_n(&par[v], &p, gp, 0, __ATOMIC_RELAXED,
                                             __ATOMIC_RELAXED); /* halving */
    v = gp;
  }
}

void sst_o_cc(const sst_o_graph *g, uint32_t *label) {
  const uint32_t n = g->n;
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; v++) label[v] = (uint32_t)v;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t uu = 0; uu < (int64_t)n; uu++) {
    const uint32_t u = (uint32_t)uu;
    for (uint32_t i = 0; i < g->deg[u]; i++) {
      const uint32_t w = g->adj[u][i];
      if (w >= n) continue;
      for (;;) {
        uint32_t a = uf_find(label, u), b = uf_find(label, w);
        if (a == b) break;
        uint32_t hi = a > b ? a : b, lo = a > b ? b : a, expect = hi;
        if (__atomic_compare_exchange_n(&label[hi], &expect, lo, 0, __ATOMIC_RELAXED,
                                        __ATOMIC_RELAXED))
          break;
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; v++) label[v] = uf_find(label, (uint32_t)v);
  /* the finds above only shorten paths: a second pass settles every label
   * on its root */
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; v++) label[v] = label[label[v]];
}

/* Single-source betweenness dependencies (Brandes 2001), FP64:
 *   sigma(src) = 1, sigma(w) = sum_{v in N(w), depth v = depth w - 1} sigma(v)
 *   dep(v) = sum_{w in N(v), depth w = depth v + 1} sigma(v)/sigma(w) * (1 + dep(w))
 * sums in ascending neighbour order; unreached vertices get 0; the source
 * keeps its own dep by the same formula.  Each level's vertices run in
 * parallel (their sums read only the levels before, resp. after, them), so
 * every value is the same sum in the same order as a serial pass. */
void sst_o_bc(const sst_o_graph *g, uint32_t src, double *dep) {
  const uint32_t n = g->n;
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; v++) dep[v] = 0.0;
  if (src >= n) return;
  int32_t *depth = (int32_t *)malloc((size_t)n * sizeof(int32_t));
  double *sigma = (double *)calloc(n, sizeof(double));
  uint32_t *order = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
  const uint64_t t = bfs_levels(g, src, depth, order);
  /* level boundaries in order[] (level-synchronous BFS emits by level) */
  const int32_t maxd = depth[order[t - 1]];
  uint64_t *lvl = (uint64_t *)calloc((size_t)maxd + 2, sizeof(uint64_t));
  for (uint64_t k = 0; k < t; k++) lvl[depth[order[k]] + 1]++;
  for (int32_t d = 0; d <= maxd; d++) lvl[d + 1] += lvl[d];
  sigma[src] = 1.0;
  for (int32_t d = 1; d <= maxd; d++) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = (int64_t)lvl[d]; k < (int64_t)lvl[d + 1]; k++) {
      const uint32_t w = order[k];
      double s = 0.0;
      for (uint32_t i = 0; i < g->deg[w]; i++) {
        const uint32_t v = g->adj[w][i];
        if (depth[v] == d - 1) s += sigma[v];
      }
      sigma[w] = s;
    }
  }
  for (int32_t d = maxd; d >= 0; d--) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = (int64_t)lvl[d]; k < (int64_t)lvl[d + 1]; k++) {
      const uint32_t v = order[k];
      double s = 0.0;
      for (uint32_t i = 0; i < g->deg[v]; i++) {
        const uint32_t w = g->adj[v][i];
        if (depth[w] == d + 1) s += sigma[v] / sigma[w] * (1.0 + dep[w]);
      }
      dep[v] = s;
    }
  }
  free(lvl);
  free(order);
  free(sigma);
  free(depth);
}

/* triangle count: sum over u, v in N(u), v < u of common_neighbors(u, v,
 * early_end) -- each triangle w < v < u once (SparseMatrix.hpp:61-71).
 * per_vertex (optional): triangles containing each vertex. */
uint64_t sst_o_tc(const sst_o_graph *g, uint64_t *per_vertex) {
  uint32_t n = g->n;
  uint64_t total = 0;
  if (per_vertex) memset(per_vertex, 0, (size_t)n * sizeof(uint64_t));
#pragma omp parallel for reduction(+ : total) schedule(dynamic, 64)
  for (int64_t uu = 0; uu < (int64_t)n; uu++) {
    uint32_t u = (uint32_t)uu;
    const uint32_t *a = g->adj[u];
    uint32_t na = g->deg[u];
    for (uint32_t k = 0; k < na && a[k] < u; k++) {
      uint32_t v = a[k];
      const uint32_t *b = g->adj[v];
      uint32_t nb = g->deg[v];
      uint32_t i = 0, j = 0;
      while (i < na && j < nb && a[i] < v && b[j] < v) {
        if (a[i] < b[j])
          i++;
        else if (b[j] < a[i])
          j++;
        else {
          total++;
          if (per_vertex) {
#pragma omp atomic
            per_vertex[u]++;
#pragma omp atomic
            per_vertex[v]++;
#pragma omp atomic
            per_vertex[a[i]]++;
          }
          i++;
          j++;
        }
      }
    }
  }
  return total;
}

sst_o_graph *sst_o_new(uint32_t n) { return sst_o_new2(n, n); }

// Traversal kernels over the device PMA (the EdgeMap/VertexMap algorithms the
// reference drivers call at internal/test.hpp:476-618; the algorithm
// library itself, EdgeMapVertexMap, is absent from the reference tree).
//
// Work decomposition, rebuilt when the graph version changes:
//  - a vertex whose segment is one leaf (cap <= 32) is handled by one thread
//    that walks its packed leaf;
//  - a vertex with a multi-leaf segment is cut into chunks of kChunkLeaves
//    leaves; one warp walks a chunk leaf by leaf (lane = slot, one 128-byte
//    line per leaf, only the occupied prefix is read); chunks of one vertex
//    are combined in chunk order, so sums are deterministic.
#include <algorithm>
#include <vector>

#include "ccshared.cuh"
#include "prfixed.cuh"
#include "tcshared.cuh"
#include "traverse.cuh"

namespace sst {

namespace {
constexpr int kTB = 256;
constexpr uint32_t kChunkLeaves = 32;
// leaves per work item of the push-style kernels (frontier expansion):
// smaller than kChunkLeaves so a hub's chunks spread over more warps
constexpr uint32_t kPushLeaves = 8;

inline unsigned blocks_for(uint64_t n, int per = kTB) {
  uint64_t b = (n + per - 1) / per;
  return (unsigned)(b == 0 ? 1 : b);
}
inline unsigned warp_blocks(uint64_t nwarps) { return blocks_for(nwarps * 32); }

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  return v;
}
}  // namespace

template <typename T> struct DevBuf {
  T *p = nullptr;
  uint64_t cap = 0;
  cudaError_t ensure(uint64_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    uint64_t want = n + n / 8 + 64;
    cudaError_t e = cudaMalloc(&p, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct TravState {
  uint64_t version = ~0ull;
  // tuning (sst_autotune): leaves per work-list chunk (<= 32), lanes per
  // one-leaf vertex in PageRank, and the BFS switch to pull once
  // (frontier + its edges) * bfs_alpha > m
  uint32_t chunk_leaves = 32, pr_lanes = 8, bfs_alpha = 20;
  uint32_t pr_hot = 0;        // contributions staged in shared memory
  uint32_t pr_hot_used = ~0u; // pr_hot of the captured graph
  uint32_t lists_cl = 0;      // chunk size the lists were built with
  uint64_t lists_stamp = 0;   // bumped on every rebuild of the lists
  // chunk list of multi-leaf vertices
  uint64_t nchunks = 0, nmulti = 0, nbig = 0, nsmall = 0;
  uint64_t inv_version = ~0ull;
  DevBuf<uint64_t> choff;   // per vertex: first chunk (n+1)
  DevBuf<uint32_t> cv, cl0; // per chunk: vertex, first leaf
  DevBuf<unsigned long long> cdesc, sdesc;  // packed chunk / one-leaf items
  DevBuf<uint32_t> multi;   // vertices with more than one chunk
  DevBuf<uint32_t> big;     // vertices with a multi-leaf segment
  DevBuf<uint32_t> small;   // vertices with a one-leaf segment (deg >= 1)
  DevBuf<uint32_t> flag, pos;
  // pagerank
  DevBuf<double> inv_deg, ca, cb, partial;
  // bfs
  DevBuf<uint32_t> qa, qb, fbits, icnt, ioff, iv, il0;
  DevBuf<int32_t> depth_tmp, parent_tmp;
  // bc
  DevBuf<double> sigma, ratio;
  DevBuf<uint32_t> lvl_list, lvl_cnt;
  // cc
  DevBuf<uint32_t> par;
  // tc
  DevBuf<uint64_t> toff, tlpre, tlcnt, titems;
  DevBuf<uint32_t> tadj, tmask;
  // multi-source bfs: per-vertex source masks (visited, frontier, next)
  DevBuf<unsigned long long> mvis, mfr, mfr2, mnx, msrc;
  DevBuf<int32_t> mdepth;
  // multi-source bc: per (source, vertex) values and per-source level tables
  DevBuf<double> msig, mrat, mpart;
  DevBuf<uint32_t> mlist, micnt, mioff, miv, mil0, mtab;
  // PageRank iterations captured as one CUDA graph, replayed while the
  // graph version and the call's arguments stay the same
  cudaGraphExec_t pr_exec = nullptr;
  uint64_t pr_version = ~0ull;  // lists_stamp the graph was captured with
  uint32_t pr_lanes_used = 0;
  uint32_t pr_iters = 0;
  double pr_damping = 0.0;
  const void *pr_key[6] = {};  // output, stream and the buffers it reads
  int64_t pr_kernels = 0;      // kernels in the captured graph
  uint64_t *h_small = nullptr;  // pinned readback slots
  unsigned long long *d_small = nullptr;
};

// frees every buffer and the captured PageRank graph; the tuning stays, and
// the work lists are rebuilt by the next traversal
static void trav_buffers_release(TravState *t) {
  t->choff.release();
  t->cv.release();
  t->cl0.release();
  t->cdesc.release();
  t->sdesc.release();
  t->multi.release();
  t->big.release();
  t->small.release();
  t->flag.release();
  t->pos.release();
  t->inv_deg.release();
  t->ca.release();
  t->cb.release();
  t->partial.release();
  t->qa.release();
  t->qb.release();
  t->fbits.release();
  t->icnt.release();
  t->ioff.release();
  t->iv.release();
  t->il0.release();
  t->depth_tmp.release();
  t->parent_tmp.release();
  t->sigma.release();
  t->ratio.release();
  t->lvl_list.release();
  t->lvl_cnt.release();
  t->par.release();
  t->toff.release();
  t->tlpre.release();
  t->tlcnt.release();
  t->tadj.release();
  t->titems.release();
  t->tmask.release();
  t->mvis.release();
  t->mfr.release();
  t->mfr2.release();
  t->mnx.release();
  t->msrc.release();
  t->mdepth.release();
  t->msig.release();
  t->mrat.release();
  t->mpart.release();
  t->mlist.release();
  t->micnt.release();
  t->mioff.release();
  t->miv.release();
  t->mil0.release();
  t->mtab.release();
  if (t->pr_exec) cudaGraphExecDestroy(t->pr_exec);
  t->pr_exec = nullptr;
  t->version = ~0ull;
  t->inv_version = ~0ull;
  t->lists_stamp++;
}

void trav_trim(sst_graph *g) {
  if (g->trav) trav_buffers_release(g->trav);
}

void trav_release(sst_graph *g) {
  TravState *t = g->trav;
  if (!t) return;
  trav_buffers_release(t);
  if (t->h_small) cudaFreeHost(t->h_small);
  if (t->d_small) cudaFree(t->d_small);
  delete t;
  g->trav = nullptr;
}

uint64_t trav_device_bytes(const sst_graph *g) {
  const TravState *t = g->trav;
  if (!t) return 0;
  uint64_t b = 0;
  auto add = [&](uint64_t cap, size_t elem) { b += cap * elem; };
  add(t->choff.cap, 8); add(t->cv.cap, 4); add(t->cl0.cap, 4); add(t->cdesc.cap, 8);
  add(t->sdesc.cap, 8); add(t->multi.cap, 4); add(t->big.cap, 4); add(t->small.cap, 4);
  add(t->flag.cap, 4); add(t->pos.cap, 4); add(t->inv_deg.cap, 8); add(t->ca.cap, 8);
  add(t->cb.cap, 8); add(t->partial.cap, 8); add(t->qa.cap, 4); add(t->qb.cap, 4);
  add(t->fbits.cap, 4); add(t->icnt.cap, 4); add(t->ioff.cap, 4); add(t->iv.cap, 4);
  add(t->il0.cap, 4); add(t->depth_tmp.cap, 4); add(t->parent_tmp.cap, 4);
  add(t->sigma.cap, 8); add(t->ratio.cap, 8); add(t->lvl_list.cap, 4);
  add(t->lvl_cnt.cap, 4); add(t->par.cap, 4); add(t->toff.cap, 8); add(t->tlpre.cap, 8);
  add(t->tlcnt.cap, 8); add(t->tadj.cap, 4); add(t->titems.cap, 8); add(t->tmask.cap, 4);
  add(t->mvis.cap, 8); add(t->mfr.cap, 8);
  add(t->mfr2.cap, 8); add(t->mnx.cap, 8); add(t->msrc.cap, 8); add(t->mdepth.cap, 4);
  add(t->msig.cap, 8); add(t->mrat.cap, 8); add(t->mpart.cap, 8); add(t->mlist.cap, 4);
  add(t->micnt.cap, 4); add(t->mioff.cap, 4); add(t->miv.cap, 4); add(t->mil0.cap, 4);
  add(t->mtab.cap, 4);
  return b;
}

namespace {

// ------------------------------------------------------------- work lists
__global__ void k_chunk_counts(const uint32_t *__restrict__ cap, uint32_t n,
                               uint64_t *__restrict__ nch,
                               uint32_t *__restrict__ bigf,
                               uint32_t *__restrict__ multif,
                               uint32_t *__restrict__ smallf, uint32_t cl) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  uint32_t c = cap[v];
  uint64_t k = c > kLeaf ? ((c >> kLeafLog) + cl - 1) / cl : 0;
  nch[v] = k;
  bigf[v] = c > kLeaf;
  multif[v] = k > 1;
  smallf[v] = c > 0 && c <= kLeaf;
}

__global__ void k_chunk_fill(const uint32_t *__restrict__ cap,
                             const uint64_t *__restrict__ base, uint32_t n,
                             const uint64_t *__restrict__ choff,
                             uint32_t *__restrict__ cv,
                             uint32_t *__restrict__ cl0,
                             unsigned long long *__restrict__ cdesc,
                             uint32_t cl) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  uint64_t c0 = choff[v], c1 = choff[v + 1];
  uint32_t nl = cap[v] >> kLeafLog;
  uint64_t leaf = base[v] >> kLeafLog;
  unsigned long long single = (c1 - c0) == 1 ? 128ull : 0ull;
  for (uint64_t c = c0; c < c1; c++) {
    uint32_t l0 = (uint32_t)((c - c0) * cl);
    cv[c] = v;
    cl0[c] = l0;
    cdesc[c] = ((leaf + l0) << 8) | single | (unsigned long long)min(cl, nl - l0);
  }
}

__global__ void k_small_desc(const uint32_t *__restrict__ small, uint64_t nsmall,
                             const uint64_t *__restrict__ base,
                             const uint32_t *__restrict__ deg,
                             unsigned long long *__restrict__ sdesc) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsmall) return;
  uint32_t v = small[i];
  sdesc[i] = ((unsigned long long)base[v] << 6) | deg[v];
}

__global__ void k_compact_ids(const uint32_t *__restrict__ flag,
                              const uint32_t *__restrict__ pos, uint32_t n,
                              uint32_t *__restrict__ out) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n && flag[v]) out[pos[v]] = v;
}

// ------------------------------------------------------------- pagerank
// The fixed-point arithmetic (units of 2^-63, exact integer sums) is in
// prfixed.cuh, shared with the byte-width snapshot's PageRank.

// per vertex: round(2^64 / deg) for deg >= 2 (deg 1 passes rank through)
__global__ void k_pr_rdeg(const uint32_t *__restrict__ deg, uint32_t n,
                          unsigned long long *__restrict__ rdeg) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  rdeg[v] = pr_rdeg_of(deg[v]);
}

// a vertex with an empty row is in no work list, so no iteration writes its
// contribution: zero it in both buffers (a directed graph's rows may still
// name it)
__global__ void k_pr_start(const uint32_t *__restrict__ deg, uint32_t n,
                           unsigned long long r0,
                           const unsigned long long *__restrict__ rdeg,
                           unsigned long long *__restrict__ contrib,
                           unsigned long long *__restrict__ contrib2,
                           double *__restrict__ rank, double base) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  uint32_t d = deg[v];
  contrib[v] = d ? contrib_of(r0, d, rdeg[v]) : 0ull;
  if (d == 0) {
    contrib2[v] = 0ull;
    rank[v] = base;  // no in-edges: constant term only
  }
}


// One-leaf segments (cap <= 32): a group of G lanes per vertex (G = 8: one
// 32-byte sector of the leaf per lane step), four vertices per group in
// flight.  sdesc[i] = (segment base << 6) | degree.
constexpr int kSmallPer = 4;

template <int G>
__global__ void k_pr_small(DGraph g, const unsigned long long *__restrict__ sdesc,
                           const uint32_t *__restrict__ small, uint64_t nsmall,
                           const unsigned long long *__restrict__ cin,
                           unsigned long long *__restrict__ cout,
                           double *__restrict__ rank,
                           const unsigned long long *__restrict__ rdeg,
                           PrConst k, bool last) {
  static_assert(G >= kSmallPer && G <= 32 && (G & (G - 1)) == 0, "lanes per vertex");
  constexpr int Q = 32 / G;  // slots per lane
  uint64_t grp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const uint32_t sub = threadIdx.x & (G - 1);
  const unsigned long long pol = l2_evict_first();
  const uint64_t i0 = grp * kSmallPer;
  uint32_t x[kSmallPer][Q];
  uint32_t dg[kSmallPer];
#pragma unroll
  for (int u = 0; u < kSmallPer; u++) {
    uint64_t i = i0 + u;
    unsigned long long dsc = i < nsmall ? sdesc[i] : 0ull;
    dg[u] = (uint32_t)(dsc & 63);
    const uint32_t *p = g.slots + (dsc >> 6);
#pragma unroll
    for (int q = 0; q < Q; q++) {
      uint32_t j = sub + G * q;
      x[u][q] = j < dg[u] ? ld_stream(p + j, pol) : kEmpty;
    }
  }
  unsigned long long acc[kSmallPer];
#pragma unroll
  for (int u = 0; u < kSmallPer; u++) {
    acc[u] = 0;
#pragma unroll
    for (int q = 0; q < Q; q++)
      if (x[u][q] != kEmpty) acc[u] += ld_keep(cin + x[u][q]);
  }
  unsigned long long mine = 0;
  uint32_t mydeg = 0;
#pragma unroll
  for (int u = 0; u < kSmallPer; u++) {
    unsigned long long a = acc[u];
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (sub == (uint32_t)u) {
      mine = a;
      mydeg = dg[u];
    }
  }
  if (sub < (uint32_t)kSmallPer && i0 + sub < nsmall)
    pr_finish(small[i0 + sub], mine, k, mydeg, rdeg, cout, rank, last);
}

// warp per chunk of <= 32 leaves of a multi-leaf segment (lane = slot);
// the chunk's leaf counts come in with one coalesced load, and eight leaves'
// ids, then their eight gathers, are in flight per step.
// cdesc[c] = (first leaf << 8) | (single chunk << 7) | leaves in the chunk.
__global__ void k_pr_chunks(DGraph g, const unsigned long long *__restrict__ cdesc,
                            const uint32_t *__restrict__ cv, uint64_t nchunks,
                            const unsigned long long *__restrict__ cin,
                            unsigned long long *__restrict__ cout,
                            double *__restrict__ rank,
                            const unsigned long long *__restrict__ rdeg,
                            unsigned long long *__restrict__ partial, PrConst k,
                            bool last) {
  uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= nchunks) return;
  const unsigned long long pol = l2_evict_first();
  unsigned long long dsc = cdesc[c];
  const uint64_t leaf0 = dsc >> 8;
  const uint32_t l1 = (uint32_t)(dsc & 63);
  const bool single = (dsc >> 7) & 1;
  const uint32_t mycnt = (uint32_t)lane < l1 ? g.lcnt[leaf0 + lane] : 0u;
  const uint32_t *sl = g.slots + (leaf0 << kLeafLog) + lane;
  unsigned long long acc = 0;
  for (uint32_t l = 0; l < l1; l += 8) {
    uint32_t x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint32_t cq = __shfl_sync(0xffffffffu, mycnt, (l + q) & 31);
      if (l + q >= l1) cq = 0;
      x[q] = (uint32_t)lane < cq ? ld_stream(sl + ((uint64_t)(l + q) << kLeafLog), pol)
                                 : kEmpty;
    }
#pragma unroll
    for (int q = 0; q < 8; q++)
      if (x[q] != kEmpty) acc += ld_keep(cin + x[q]);
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
  if (lane == 0) {
    if (single) {
      uint32_t v = cv[c];
      pr_finish(v, acc, k, g.deg[v], rdeg, cout, rank, last);
    } else {
      partial[c] = acc;
    }
  }
}

// ---- PageRank with the contributions of ids below `hot` staged in shared
// memory once per block: on a degree-ordered graph (highest degree first,
// sst_degree_order_map) those are the vertices most edges point to, so
// their gathers leave L2 alone.  Blocks are persistent and stride over the
// work; the loops stay warp-uniform for the shuffles.
__device__ __forceinline__ void stage_hot(unsigned long long *sh,
                                          const unsigned long long *cin,
                                          uint32_t hot) {
  for (uint32_t i = threadIdx.x; i < hot; i += blockDim.x) sh[i] = cin[i];
  __syncthreads();
}
__device__ __forceinline__ unsigned long long gather(const unsigned long long *sh,
                                                     const unsigned long long *cin,
                                                     uint32_t x, uint32_t hot) {
  return x < hot ? sh[x] : ld_keep(cin + x);
}

constexpr int kHotThreads = 512;  // 4 blocks of 16 warps per SM
// a cache above kHotBig entries leaves room for one block per SM: that block
// takes 1024 threads
constexpr uint32_t kHotBig = 8192;

// launch bounds: 512-thread blocks at least two to an SM (64 registers a
// thread), 1024-thread blocks (large caches) one to an SM
template <int G, int T = kHotThreads>
__global__ void __launch_bounds__(T, T == 1024 ? 1 : 2) k_pr_small_hot(DGraph g, const unsigned long long *__restrict__ sdesc,
                               const uint32_t *__restrict__ small, uint64_t nsmall,
                               const unsigned long long *__restrict__ cin,
                               unsigned long long *__restrict__ cout,
                               double *__restrict__ rank,
                               const unsigned long long *__restrict__ rdeg,
                               PrConst k, bool last, uint32_t hot) {
  extern __shared__ unsigned long long sh[];
  constexpr int Q = 32 / G;
  stage_hot(sh, cin, hot);
  const unsigned long long pol = l2_evict_first();
  const uint32_t sub = threadIdx.x & (G - 1);
  const uint64_t per_warp = (32 / G) * kSmallPer;  // vertices per warp round
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t rounds = (nsmall + per_warp - 1) / per_warp;
  for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       w < rounds; w += nwarps) {
    const uint64_t i0 = (w * (32 / G) + ((threadIdx.x & 31) / G)) * kSmallPer;
    uint32_t x[kSmallPer][Q];
    uint32_t dg[kSmallPer];
#pragma unroll
    for (int u = 0; u < kSmallPer; u++) {
      uint64_t i = i0 + u;
      unsigned long long dsc = i < nsmall ? sdesc[i] : 0ull;
      dg[u] = (uint32_t)(dsc & 63);
      const uint32_t *p = g.slots + (dsc >> 6);
#pragma unroll
      for (int q = 0; q < Q; q++) {
        uint32_t j = sub + G * q;
        x[u][q] = j < dg[u] ? ld_stream(p + j, pol) : kEmpty;
      }
    }
    unsigned long long mine = 0;
    uint32_t mydeg = 0;
#pragma unroll
    for (int u = 0; u < kSmallPer; u++) {
      unsigned long long a = 0;
#pragma unroll
      for (int q = 0; q < Q; q++)
        if (x[u][q] != kEmpty) a += gather(sh, cin, x[u][q], hot);
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (sub == (uint32_t)u) {
        mine = a;
        mydeg = dg[u];
      }
    }
    if (sub < (uint32_t)kSmallPer && i0 + sub < nsmall)
      pr_finish(small[i0 + sub], mine, k, mydeg, rdeg, cout, rank, last);
  }
}

template <int T = kHotThreads>
__global__ void __launch_bounds__(T, T == 1024 ? 1 : 2) k_pr_chunks_hot(DGraph g, const unsigned long long *__restrict__ cdesc,
                                const uint32_t *__restrict__ cv, uint64_t nchunks,
                                const unsigned long long *__restrict__ cin,
                                unsigned long long *__restrict__ cout,
                                double *__restrict__ rank,
                                const unsigned long long *__restrict__ rdeg,
                                unsigned long long *__restrict__ partial, PrConst k,
                                bool last, uint32_t hot) {
  extern __shared__ unsigned long long sh[];
  stage_hot(sh, cin, hot);
  const int lane = threadIdx.x & 31;
  const unsigned long long pol = l2_evict_first();
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       c < nchunks; c += nwarps) {
    unsigned long long dsc = cdesc[c];
    const uint64_t leaf0 = dsc >> 8;
    const uint32_t l1 = (uint32_t)(dsc & 63);
    const bool single = (dsc >> 7) & 1;
    const uint32_t mycnt = (uint32_t)lane < l1 ? g.lcnt[leaf0 + lane] : 0u;
    const uint32_t *sl = g.slots + (leaf0 << kLeafLog) + lane;
    unsigned long long acc = 0;
    for (uint32_t l = 0; l < l1; l += 8) {
      uint32_t x[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        uint32_t cq = __shfl_sync(0xffffffffu, mycnt, (l + q) & 31);
        if (l + q >= l1) cq = 0;
        x[q] = (uint32_t)lane < cq ? ld_stream(sl + ((uint64_t)(l + q) << kLeafLog), pol)
                                   : kEmpty;
      }
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (x[q] != kEmpty) acc += gather(sh, cin, x[q], hot);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
    if (lane == 0) {
      if (single) {
        uint32_t v = cv[c];
        pr_finish(v, acc, k, g.deg[v], rdeg, cout, rank, last);
      } else {
        partial[c] = acc;
      }
    }
  }
}

__global__ void k_pr_fix(DGraph g, const uint32_t *__restrict__ multi,
                         uint64_t nmulti, const uint64_t *__restrict__ choff,
                         const unsigned long long *__restrict__ partial,
                         unsigned long long *__restrict__ cout,
                         double *__restrict__ rank,
                         const unsigned long long *__restrict__ rdeg, PrConst k,
                         bool last) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nmulti) return;
  uint32_t v = multi[i];
  unsigned long long s = 0;
  for (uint64_t c = choff[v]; c < choff[v + 1]; c++) s += partial[c];
  pr_finish(v, s, k, g.deg[v], rdeg, cout, rank, last);
}

__global__ void k_fill_d(double *__restrict__ p, uint32_t n, double x) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) p[v] = x;
}

// ------------------------------------------------------------- bfs
__global__ void k_bfs_init(int32_t *__restrict__ depth, int32_t *__restrict__ parent,
                           uint32_t n, uint32_t src) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  depth[v] = v == src ? 0 : -1;
  parent[v] = v == src ? (int32_t)src : -1;
}

// warp-aggregated append of `mine` to the next queue
// counters: [0] queue length, [1] degree sum, [2] work items of the queue
__device__ __forceinline__ void enqueue(bool mine, uint32_t w, uint32_t wdeg,
                                        uint32_t witems, uint32_t *q,
                                        unsigned long long *qlen_deg) {
  const int lane = threadIdx.x & 31;
  uint32_t m = __ballot_sync(0xffffffffu, mine);
  if (!m) return;
  uint32_t dsum = __reduce_add_sync(0xffffffffu, mine ? wdeg : 0u);
  uint32_t isum = __reduce_add_sync(0xffffffffu, mine ? witems : 0u);
  int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) {
    base = atomicAdd(&qlen_deg[0], (unsigned long long)__popc(m));
    atomicAdd(&qlen_deg[1], (unsigned long long)dsum);
    atomicAdd(&qlen_deg[2], (unsigned long long)isum);
  }
  base = __shfl_sync(0xffffffffu, base, leader);
  if (mine) q[base + __popc(m & ((1u << lane) - 1u))] = w;
}

// Block-aggregated form of enqueue for kernels in which every thread of the
// block calls it once: one atomic per counter per block (the three queue
// counters are single addresses, so per-warp atomics from a whole grid
// serialise on them).
__device__ __forceinline__ void enqueue_block(bool mine, uint32_t w, uint32_t wdeg,
                                              uint32_t witems, uint32_t *q,
                                              unsigned long long *qlen_deg) {
  __shared__ uint32_t s_cnt[kTB / 32];
  __shared__ unsigned long long s_base, s_deg, s_items;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t m = __ballot_sync(0xffffffffu, mine);
  const uint32_t dsum = __reduce_add_sync(0xffffffffu, mine ? wdeg : 0u);
  const uint32_t isum = __reduce_add_sync(0xffffffffu, mine ? witems : 0u);
  if (threadIdx.x == 0) {
    s_deg = 0;
    s_items = 0;
  }
  if (lane == 0) s_cnt[warp] = __popc(m);
  __syncthreads();
  if (lane == 0 && m) {
    atomicAdd(&s_deg, (unsigned long long)dsum);
    atomicAdd(&s_items, (unsigned long long)isum);
  }
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
#pragma unroll
    for (int k = 0; k < kTB / 32; k++) {
      uint32_t c = s_cnt[k];
      s_cnt[k] = tot;
      tot += c;
    }
    s_base = tot ? atomicAdd(&qlen_deg[0], (unsigned long long)tot) : 0ull;
  }
  __syncthreads();
  if (threadIdx.x == 0 && (s_deg || s_items)) {
    atomicAdd(&qlen_deg[1], s_deg);
    atomicAdd(&qlen_deg[2], s_items);
  }
  if (mine) q[s_base + s_cnt[warp] + __popc(m & ((1u << lane) - 1u))] = w;
}

// push work items of one vertex: 1 for a one-leaf segment, else one per
// chunk of kPushLeaves leaves
__device__ __forceinline__ uint32_t items_of(uint32_t cap) {
  return cap > kLeaf ? ((cap >> kLeafLog) + kPushLeaves - 1) / kPushLeaves : 1u;
}

__global__ void k_front_items(const uint32_t *__restrict__ q, uint32_t qn,
                              const uint32_t *__restrict__ cap,
                              uint32_t *__restrict__ cnt) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < qn) cnt[i] = items_of(cap[q[i]]);
}

__global__ void k_front_expand(const uint32_t *__restrict__ q, uint32_t qn,
                               const uint32_t *__restrict__ cap,
                               const uint32_t *__restrict__ off,
                               uint32_t *__restrict__ iv,
                               uint32_t *__restrict__ il0) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= qn) return;
  uint32_t v = q[i], k = items_of(cap[v]), o = off[i];
  for (uint32_t j = 0; j < k; j++) {
    iv[o + j] = v;
    il0[o + j] = j * kPushLeaves;
  }
}

// push: warp per work item (a frontier vertex's leaf chunk), lane = slot;
// four leaves' slots, depths and claims are in flight at once, their newly
// reached vertices take queue positions with one atomic per warp and batch,
// and the warp adds its degree and work-item sums once
__global__ void __launch_bounds__(kTB, 8)
k_bfs_push(DGraph g, const uint32_t *__restrict__ iv,
           const uint32_t *__restrict__ il0, uint32_t nitems,
           int32_t *__restrict__ depth, int32_t *__restrict__ parent,
           uint32_t *__restrict__ nq, unsigned long long *__restrict__ cnt,
           int lvl) {
  constexpr int kBatch = 4;  // leaves whose slots are in flight at once
  const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= nitems) return;
  const uint32_t u = iv[i];
  const uint64_t base = g.base[u];
  const uint32_t cap = g.cap[u], deg = g.deg[u];
  const uint32_t nl = cap ? nleaves_of(cap) : 0;
  const uint32_t l0 = il0[i], l1 = min(l0 + kPushLeaves, nl);
  // a one-leaf segment holds deg ids; a multi-leaf segment's leaves hold
  // their ids packed left with EMPTY after them, so no leaf counts are read
  const uint32_t lim = cap <= kLeaf ? deg : kLeaf;
  const uint32_t below = (1u << lane) - 1u;
  unsigned long long dsum = 0, isum = 0;
  for (uint32_t l = l0; l < l1; l += kBatch) {
    uint32_t w[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; k++)
      w[k] = (l + k < l1 && (uint32_t)lane < lim)
                 ? g.slots[base + ((uint64_t)(l + k) << kLeafLog) + lane]
                 : kEmpty;
    int32_t dd[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; k++) dd[k] = w[k] != kEmpty ? depth[w[k]] : 0;
    uint32_t mine = 0;  // bit k: this lane claimed w[k]
#pragma unroll
    for (int k = 0; k < kBatch; k++)
      if (dd[k] < 0 && atomicCAS(&depth[w[k]], -1, lvl + 1) == -1)
        mine |= 1u << k;
    // one queue reservation per batch, in (leaf, lane) order; leaves past
    // the chunk's end (warp-uniform) take no ballot
    uint32_t mm[kBatch], total = 0;
#pragma unroll
    for (int k = 0; k < kBatch; k++) {
      mm[k] = l + k < l1 ? __ballot_sync(0xffffffffu, (mine >> k) & 1u) : 0u;
      total += __popc(mm[k]);
    }
    if (total == 0) continue;
    unsigned long long at = 0;
    if (lane == 0) at = atomicAdd(&cnt[0], (unsigned long long)total);
    at = __shfl_sync(0xffffffffu, at, 0);
#pragma unroll
    for (int k = 0; k < kBatch; k++) {
      if ((mine >> k) & 1u) {
        nq[at + __popc(mm[k] & below)] = w[k];
        parent[w[k]] = (int32_t)u;
        dsum += g.deg[w[k]];
        isum += items_of(g.cap[w[k]]);
      }
      at += __popc(mm[k]);
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    dsum += __shfl_xor_sync(0xffffffffu, dsum, d);
    isum += __shfl_xor_sync(0xffffffffu, isum, d);
  }
  if (lane == 0 && (dsum || isum)) {
    atomicAdd(&cnt[1], dsum);
    atomicAdd(&cnt[2], isum);
  }
}

__global__ void k_q2bits(const uint32_t *__restrict__ q, uint32_t qn,
                         uint32_t *__restrict__ bits) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= qn) return;
  uint32_t u = q[i];
  atomicOr(&bits[u >> 5], 1u << (u & 31));
}

__device__ __forceinline__ bool in_front(const uint32_t *bits, uint32_t u) {
  return (bits[u >> 5] >> (u & 31)) & 1u;
}

// pull, one-leaf vertices (the one-leaf list): a group of 8 lanes per
// vertex, 4 slots per lane, four vertices per group in flight; the parent is
// the smallest frontier neighbour
__global__ void k_bfs_pull_small8(DGraph g, const unsigned long long *__restrict__ sdesc,
                                  const uint32_t *__restrict__ small, uint64_t nsmall,
                                  const uint32_t *__restrict__ fbits,
                                  int32_t *__restrict__ depth,
                                  int32_t *__restrict__ parent,
                                  uint32_t *__restrict__ nq,
                                  unsigned long long *__restrict__ cnt, int lvl) {
  const uint64_t grp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const uint32_t sub = threadIdx.x & 7;
  const uint64_t i0 = grp * 4;
  // each stage's loads for the group's four vertices go out together: the
  // list entries, then their depths, then the open ones' slots, then the
  // frontier bits of those neighbours
  uint32_t v[4], d[4];
  unsigned long long dsc[4];
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const bool in = i0 + u < nsmall;
    v[u] = in ? small[i0 + u] : 0u;
    dsc[u] = in ? sdesc[i0 + u] : 0ull;
    d[u] = (uint32_t)(dsc[u] & 63);
  }
  bool open[4];
#pragma unroll
  for (int u = 0; u < 4; u++) open[u] = i0 + u < nsmall && depth[v[u]] < 0;
  uint32_t w[4][4];
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint32_t j = sub + 8 * q;
      w[u][q] = (open[u] && j < d[u]) ? g.slots[(dsc[u] >> 6) + j] : kEmpty;
    }
  uint32_t fb[4][4];
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int q = 0; q < 4; q++) fb[u][q] = w[u][q] != kEmpty ? fbits[w[u][q] >> 5] : 0u;
  bool mine = false;
  uint32_t myv = 0, mydeg = 0;
#pragma unroll
  for (int u = 0; u < 4; u++) {
    uint32_t best = kEmpty;
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (((fb[u][q] >> (w[u][q] & 31)) & 1u) && w[u][q] < best) best = w[u][q];
    // smallest frontier neighbour over the group's 8 lanes
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (sub == (uint32_t)u && open[u] && best != kEmpty) {
      depth[v[u]] = lvl + 1;
      parent[v[u]] = (int32_t)best;
      mine = true;
      myv = v[u];
      mydeg = d[u];
    }
  }
  enqueue_block(mine, myv, mydeg, 1u, nq, cnt);
}

// pull, multi-leaf vertices: warp per chunk of the work lists (lane = slot,
// eight leaves in flight), stops at the first frontier neighbour or once
// another chunk has claimed the vertex; the claim is a compare-and-swap on
// its depth, so one chunk records it
__global__ void k_bfs_pull_chunks(DGraph g, const unsigned long long *__restrict__ cdesc,
                                  const uint32_t *__restrict__ cv, uint64_t nchunks,
                                  const uint32_t *__restrict__ fbits,
                                  int32_t *__restrict__ depth,
                                  int32_t *__restrict__ parent,
                                  uint32_t *__restrict__ nq,
                                  unsigned long long *__restrict__ cnt, int lvl) {
  const uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  bool mine = false;
  uint32_t v = 0;
  if (c < nchunks) {
    v = cv[c];
    // the chunk's descriptor and leaf counts load beside the depth check
    const unsigned long long dsc = cdesc[c];
    const uint64_t leaf0 = dsc >> 8;
    const uint32_t l1 = (uint32_t)(dsc & 63);
    const uint32_t mycnt = (uint32_t)lane < l1 ? g.lcnt[leaf0 + lane] : 0u;
    // another chunk may claim v at any time: every lane follows lane 0's
    // reading, so the warp stays converged for its shuffles
    if (__shfl_sync(0xffffffffu, __ldcg(depth + v), 0) < 0) {
      const uint32_t *sl = g.slots + (leaf0 << kLeafLog) + lane;
      uint32_t found = kEmpty;
      for (uint32_t l = 0; l < l1 && found == kEmpty; l += 8) {
        uint32_t x[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          uint32_t cq = __shfl_sync(0xffffffffu, mycnt, (l + q) & 31);
          if (l + q >= l1) cq = 0;
          x[q] = (uint32_t)lane < cq ? sl[(uint64_t)(l + q) << kLeafLog] : kEmpty;
        }
        // the eight frontier words load together, then the smallest hit
        uint32_t fw[8];
#pragma unroll
        for (int q = 0; q < 8; q++) fw[q] = x[q] != kEmpty ? fbits[x[q] >> 5] : 0u;
        uint32_t best = kEmpty;
#pragma unroll
        for (int q = 0; q < 8; q++)
          if (((fw[q] >> (x[q] & 31)) & 1u) && x[q] < best) best = x[q];
        found = __reduce_min_sync(0xffffffffu, best);
        if (found == kEmpty && __shfl_sync(0xffffffffu, __ldcg(depth + v), 0) >= 0)
          break;  // claimed by another chunk
      }
      if (found != kEmpty && lane == 0 && atomicCAS(&depth[v], -1, lvl + 1) == -1) {
        parent[v] = (int32_t)found;
        mine = true;
      }
    }
  }
  enqueue_block(mine, v, mine ? g.deg[v] : 0u, mine ? items_of(g.cap[v]) : 0u, nq, cnt);
}

// ------------------------------------------------------------- cc
// Afforest, with the helpers in ccshared.cuh
// round r of the sampling: u links to its r-th neighbour in its first leaf
__global__ void k_cc_sample(DGraph g, uint32_t r, uint32_t *__restrict__ par,
                            unsigned long long *__restrict__ err) {
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= g.n) return;
  const uint32_t cap = g.cap[u];
  if (!cap) return;
  const uint64_t base = g.base[u];
  const uint32_t c0 = leaf_count(g, base, cap, g.deg[u], 0);
  if (r < c0) cc_link(par, u, g.slots[base + r], err);
}

// phase 3, one-leaf vertices: thread per vertex
__global__ void k_cc_rest_small(DGraph g, const unsigned long long *__restrict__ sdesc,
                                const uint32_t *__restrict__ small, uint64_t nsmall,
                                const unsigned long long *__restrict__ giant,
                                uint32_t *__restrict__ par,
                                unsigned long long *__restrict__ err) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsmall) return;
  const uint32_t u = small[i];
  if (ld_par(par, u) == (uint32_t)*giant) return;
  const unsigned long long d = sdesc[i];
  const uint32_t *p = g.slots + (d >> 6);
  const uint32_t deg = (uint32_t)(d & 63);
  for (uint32_t j = 0; j < deg; j++) cc_link(par, u, p[j], err);
}

// phase 3, multi-leaf vertices: warp per chunk of leaves, lane = slot
__global__ void k_cc_rest_chunks(DGraph g, const unsigned long long *__restrict__ cdesc,
                                 const uint32_t *__restrict__ cv, uint64_t nchunks,
                                 const unsigned long long *__restrict__ giant,
                                 uint32_t *__restrict__ par,
                                 unsigned long long *__restrict__ err) {
  const uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= nchunks) return;
  const uint32_t u = cv[c];
  if (ld_par(par, u) == (uint32_t)*giant) return;
  const unsigned long long dsc = cdesc[c];
  const uint64_t leaf0 = dsc >> 8;
  const uint32_t nl = (uint32_t)(dsc & 63);
  for (uint32_t l = 0; l < nl; l++) {
    const uint32_t cnt = g.lcnt[leaf0 + l];
    if ((uint32_t)lane < cnt) cc_link(par, u, g.slots[((leaf0 + l) << kLeafLog) + lane], err);
  }
}

// ------------------------------------------------------------- bc
// Level bookkeeping: the per-level counters are a handful of addresses hit
// by every vertex, so lanes of a warp that share a level add once (match),
// and the maximum depth is taken per block before its one atomic.
__device__ __forceinline__ uint32_t level_add(uint32_t *ctr, int32_t d, bool on) {
  const uint32_t key = on ? (uint32_t)d : 0xffffffffu;
  const uint32_t peers = __match_any_sync(0xffffffffu, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (on && lane == leader) base = atomicAdd(ctr, (uint32_t)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

__device__ __forceinline__ void block_max_to(int32_t d, unsigned long long *out) {
  __shared__ int32_t s_max;
  if (threadIdx.x == 0) s_max = -1;
  __syncthreads();
  for (int o = 16; o > 0; o >>= 1) d = max(d, __shfl_down_sync(0xffffffffu, d, o));
  if ((threadIdx.x & 31) == 0 && d >= 0) atomicMax(&s_max, d);
  __syncthreads();
  if (threadIdx.x == 0 && s_max >= 0) atomicMax(out, (unsigned long long)s_max);
}

__global__ void k_bc_init(double *__restrict__ sigma, double *__restrict__ ratio,
                          double *__restrict__ dep, uint32_t n, uint32_t src) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  sigma[v] = v == src ? 1.0 : 0.0;
  ratio[v] = 0.0;
  dep[v] = 0.0;
}

// neighbours (or leaves) whose loads the BC kernels keep in flight together
constexpr int kBcAhead = 8;

// sigma(v) = sum of sigma over neighbours one level up (thread per vertex)
__global__ void k_sigma_small(DGraph g, const uint32_t *__restrict__ list,
                              uint32_t cnt, const int32_t *__restrict__ depth,
                              double *__restrict__ sigma, int32_t d) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  uint32_t v = list[i];
  if (g.cap[v] > kLeaf) return;
  const uint32_t *p = g.slots + g.base[v];
  uint32_t dg = g.deg[v];
  double s = 0.0;
  // kBcAhead neighbours at a time, each load stage issued for all of them
  // before any is used; the sum keeps neighbour order
  for (uint32_t k0 = 0; k0 < dg; k0 += kBcAhead) {
    uint32_t u[kBcAhead];
    bool on[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) u[q] = k0 + q < dg ? p[k0 + q] : 0u;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) on[q] = k0 + q < dg && depth[u[q]] == d - 1;
    double x[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) x[q] = on[q] ? sigma[u[q]] : 0.0;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++)
      if (on[q]) s += x[q];
  }
  sigma[v] = s;
}

// items (big vertices of the level list, one per leaf chunk)
__global__ void k_bc_item_counts(const uint32_t *__restrict__ list, uint32_t nl,
                                 const uint32_t *__restrict__ cap,
                                 uint32_t *__restrict__ cnt) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nl) return;
  uint32_t c = cap[list[p]];
  cnt[p] = c > kLeaf ? ((c >> kLeafLog) + kChunkLeaves - 1) / kChunkLeaves : 0;
}

__global__ void k_bc_expand(const uint32_t *__restrict__ list, uint32_t nl,
                            const uint32_t *__restrict__ cnt,
                            const uint32_t *__restrict__ off,
                            uint32_t *__restrict__ iv, uint32_t *__restrict__ il0) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nl) return;
  for (uint32_t j = 0; j < cnt[p]; j++) {
    iv[off[p] + j] = list[p];
    il0[off[p] + j] = j * kChunkLeaves;
  }
}

__global__ void k_gather_bounds(const uint32_t *__restrict__ off,
                                const uint32_t *__restrict__ pos, uint32_t k,
                                uint32_t *__restrict__ out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) out[i] = off[pos[i]];
}

// warp per chunk: partial sum of val[u] over the chunk's neighbours u at
// depth want (sigma pass: want = d-1 over sigma; dependency pass: want =
// d+1 over ratio)
__global__ void k_bc_chunks(DGraph g, const uint32_t *__restrict__ iv,
                            const uint32_t *__restrict__ il0, uint32_t i0,
                            uint32_t ni, const int32_t *__restrict__ depth,
                            const double *__restrict__ val, int32_t want,
                            double *__restrict__ partial) {
  uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= ni) return;
  i += i0;
  uint32_t v = iv[i];
  uint32_t nl = g.cap[v] >> kLeafLog;
  uint32_t l0 = il0[i], l1 = min(l0 + kChunkLeaves, nl);
  uint64_t base = g.base[v];
  const uint8_t *lc = g.lcnt + (base >> kLeafLog);
  double acc = 0.0;
  // kBcAhead leaves at a time, each load stage issued for all of them before
  // any is used; the sum keeps leaf order
  for (uint32_t l = l0; l < l1; l += kBcAhead) {
    uint32_t u[kBcAhead];
    bool on[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) on[q] = l + q < l1 && (uint32_t)lane < lc[l + q];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++)
      u[q] = on[q] ? g.slots[base + ((uint64_t)(l + q) << kLeafLog) + lane] : 0u;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) on[q] = on[q] && depth[u[q]] == want;
    double x[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) x[q] = on[q] ? val[u[q]] : 0.0;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++)
      if (on[q]) acc += x[q];
  }
  double s = warp_sum_d(acc);
  if (lane == 0) partial[i] = s;
}

// thread per big vertex of the level: combine its chunk partials in order
__global__ void k_bc_fix(const uint32_t *__restrict__ list, uint32_t p0,
                         uint32_t np, const uint32_t *__restrict__ cnt,
                         const uint32_t *__restrict__ off,
                         const double *__restrict__ partial, bool sigma_pass,
                         double *__restrict__ sigma, double *__restrict__ ratio,
                         double *__restrict__ dep) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  p += p0;
  uint32_t k = cnt[p];
  if (k == 0) return;
  double s = 0.0;
  for (uint32_t j = 0; j < k; j++) s += partial[off[p] + j];
  uint32_t v = list[p];
  if (sigma_pass) {
    sigma[v] = s;
  } else {
    double dv = sigma[v] * s;
    dep[v] = dv;
    ratio[v] = (1.0 + dv) / sigma[v];
  }
}

// dep(v) = sigma(v) * sum over neighbours one level down of (1+dep(w))/sigma(w)
__global__ void k_delta_small(DGraph g, const uint32_t *__restrict__ list,
                              uint32_t cnt, const int32_t *__restrict__ depth,
                              const double *__restrict__ sigma,
                              double *__restrict__ ratio,
                              double *__restrict__ dep, int32_t d) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  uint32_t v = list[i];
  if (g.cap[v] > kLeaf) return;
  const uint32_t *p = g.slots + g.base[v];
  uint32_t dg = g.deg[v];
  double s = 0.0;
  for (uint32_t k0 = 0; k0 < dg; k0 += kBcAhead) {  // as in k_sigma_small
    uint32_t w[kBcAhead];
    bool on[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) w[q] = k0 + q < dg ? p[k0 + q] : 0u;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) on[q] = k0 + q < dg && depth[w[q]] == d + 1;
    double x[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) x[q] = on[q] ? ratio[w[q]] : 0.0;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++)
      if (on[q]) s += x[q];
  }
  double dv = sigma[v] * s;
  dep[v] = dv;
  ratio[v] = (1.0 + dv) / sigma[v];
}

// ------------------------------------------------------------- tc
// orientation and counting in tcshared.cuh

// The orientation passes take kTcLeaves leaves a warp, all their loads
// issued before any is used (a leaf alone is three dependent round trips:
// its directory entry, its line, its ids' degrees).  The count pass also
// records each leaf's keep mask, so the fill pass needs no degree lookups.
constexpr int kTcLeaves = 4;

__global__ void k_tc_leafcount(const uint32_t *__restrict__ slots,
                               const uint32_t *__restrict__ owner,
                               const uint64_t *__restrict__ slot,
                               const uint32_t *__restrict__ cnt,
                               uint64_t nleaves, const uint32_t *__restrict__ deg,
                               uint64_t *__restrict__ out, uint32_t *__restrict__ kmask) {
  const uint64_t k0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kTcLeaves;
  const int lane = threadIdx.x & 31;
  if (k0 >= nleaves) return;
  uint32_t u[kTcLeaves], c[kTcLeaves], x[kTcLeaves];
  uint64_t sl[kTcLeaves];
#pragma unroll
  for (int j = 0; j < kTcLeaves; j++) {
    const uint64_t k = k0 + j;
    u[j] = 0;
    c[j] = 0;
    sl[j] = 0;
    if (k < nleaves) {
      u[j] = owner[k];
      sl[j] = slot[k];
      c[j] = cnt[k];
    }
  }
#pragma unroll
  for (int j = 0; j < kTcLeaves; j++) x[j] = (uint32_t)lane < c[j] ? slots[sl[j] + lane] : 0u;
#pragma unroll
  for (int j = 0; j < kTcLeaves; j++) {
    const bool keep = (uint32_t)lane < c[j] && ranks_above(deg, x[j], u[j]);
    const uint32_t m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0 && k0 + j < nleaves) {
      out[k0 + j] = __popc(m);
      kmask[k0 + j] = m;
    }
  }
}

__global__ void k_tc_fill(const uint32_t *__restrict__ slots,
                          const uint64_t *__restrict__ slot, uint64_t nleaves,
                          const uint32_t *__restrict__ kmask,
                          const uint64_t *__restrict__ lpre,
                          uint32_t *__restrict__ adj) {
  const uint64_t k0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kTcLeaves;
  const int lane = threadIdx.x & 31;
  if (k0 >= nleaves) return;
  uint32_t m[kTcLeaves], x[kTcLeaves];
  uint64_t sl[kTcLeaves], at[kTcLeaves];
#pragma unroll
  for (int j = 0; j < kTcLeaves; j++) {
    const uint64_t k = k0 + j;
    m[j] = 0;
    sl[j] = 0;
    at[j] = 0;
    if (k < nleaves) {
      m[j] = kmask[k];
      sl[j] = slot[k];
      at[j] = lpre[k];
    }
  }
#pragma unroll
  for (int j = 0; j < kTcLeaves; j++) x[j] = (m[j] >> lane) & 1u ? slots[sl[j] + lane] : 0u;
#pragma unroll
  for (int j = 0; j < kTcLeaves; j++)
    if ((m[j] >> lane) & 1u) adj[at[j] + __popc(m[j] & ((1u << lane) - 1u))] = x[j];
}

__global__ void k_tc_off(const uint64_t *__restrict__ vleaf,
                         const uint64_t *__restrict__ lpre, uint32_t n,
                         uint64_t *__restrict__ off) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v <= n) off[v] = lpre[vleaf[v]];
}

// ------------------------------------------------------------- pairs
__device__ __forceinline__ bool pma_has(const DGraph &g, uint32_t u, uint32_t x) {
  uint32_t cap = g.cap[u];
  if (!cap) return false;
  uint64_t base = g.base[u];
  uint32_t l = find_leaf(g.slots, base, cap, x);
  uint32_t c = leaf_count(g, base, cap, g.deg[u], l);
  const uint32_t *p = g.slots + base + ((uint64_t)l << kLeafLog);
  uint32_t pos = leaf_lower_bound(p, c, x);
  return pos < c && p[pos] == x;
}

// thread per pair: walk the smaller set in order, probe the other
__global__ void k_common(DGraph g, const uint32_t *__restrict__ pairs, uint64_t n,
                         bool early, uint64_t *__restrict__ out) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a = pairs[2 * i], b = pairs[2 * i + 1];
  if (a >= g.n || b >= g.n) {
    out[i] = 0;
    return;
  }
  uint32_t lim = early ? min(a, b) : 0xFFFFFFFFu;
  uint32_t s = g.deg[a] <= g.deg[b] ? a : b, o = s == a ? b : a;
  uint64_t base = g.base[s];
  uint32_t cap = g.cap[s], deg = g.deg[s];
  uint32_t nl = cap ? nleaves_of(cap) : 0;
  uint64_t c = 0;
  for (uint32_t l = 0; l < nl; l++) {
    uint32_t k = leaf_count(g, base, cap, deg, l);
    const uint32_t *p = g.slots + base + ((uint64_t)l << kLeafLog);
    for (uint32_t j = 0; j < k; j++) {
      uint32_t x = p[j];
      if (x >= lim) goto done;
      c += pma_has(g, o, x);
    }
  }
done:
  out[i] = c;
}

}  // namespace

// ================================================================== host
static TravState *state(sst_graph *g) {
  if (!g->trav) {
    g->trav = new TravState();
    cudaMallocHost(&g->trav->h_small, 64 * sizeof(uint64_t));
    cudaMalloc(&g->trav->d_small, 64 * sizeof(unsigned long long));
  }
  return g->trav;
}

static sst_status ensure_lists(sst_graph *g) {
  TravState *t = state(g);
  if (t->version == g->version && t->lists_cl == t->chunk_leaves) return SST_OK;
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  SST_CUDA_TRY(t->choff.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->flag.ensure((uint64_t)n * 3 + 3));
  SST_CUDA_TRY(t->pos.ensure((uint64_t)n * 3 + 3));
  uint32_t *bigf = t->flag.p, *multif = t->flag.p + n + 1, *smallf = t->flag.p + 2 * (n + 1);
  uint32_t *bigp = t->pos.p, *multip = t->pos.p + n + 1, *smallp = t->pos.p + 2 * (n + 1);
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(4 * scan_scratch_bytes((uint64_t)n + 1, 8) + 4096));
  uint64_t *tot = g->arena.take<uint64_t>(1);
  uint32_t *tot32 = g->arena.take<uint32_t>(3);
  const uint32_t cl = t->chunk_leaves;
  if (n) SST_LAUNCH(k_chunk_counts, blocks_for(n), kTB, 0, s, g->d_cap, n,
                    t->choff.p, bigf, multif, smallf, cl);
  SST_CUDA_TRY((scan<uint64_t, OpAdd>(t->choff.p, t->choff.p, n, 0ull, OpAdd{},
                                      true, false, tot, g->arena, s)));
  SST_CUDA_TRY((scan<uint32_t, OpAdd>(bigf, bigp, n, 0u, OpAdd{}, true, false,
                                      tot32, g->arena, s)));
  SST_CUDA_TRY((scan<uint32_t, OpAdd>(multif, multip, n, 0u, OpAdd{}, true,
                                      false, tot32 + 1, g->arena, s)));
  SST_CUDA_TRY((scan<uint32_t, OpAdd>(smallf, smallp, n, 0u, OpAdd{}, true,
                                      false, tot32 + 2, g->arena, s)));
  uint64_t h[2];
  uint32_t h32[3];
  SST_CUDA_TRY(cudaMemcpyAsync(h, tot, 8, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaMemcpyAsync(h32, tot32, 12, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  t->nchunks = h[0];
  t->nbig = h32[0];
  t->nmulti = h32[1];
  t->nsmall = h32[2];
  SST_CUDA_TRY(cudaMemcpyAsync(t->choff.p + n, &t->nchunks, 8, cudaMemcpyHostToDevice, s));
  SST_CUDA_TRY(t->cv.ensure(t->nchunks + 1));
  SST_CUDA_TRY(t->cl0.ensure(t->nchunks + 1));
  SST_CUDA_TRY(t->big.ensure(t->nbig + 1));
  SST_CUDA_TRY(t->multi.ensure(t->nmulti + 1));
  SST_CUDA_TRY(t->small.ensure(t->nsmall + 1));
  SST_CUDA_TRY(t->cdesc.ensure(t->nchunks + 1));
  SST_CUDA_TRY(t->sdesc.ensure(t->nsmall + 1));
  if (n) {
    SST_LAUNCH(k_chunk_fill, blocks_for(n), kTB, 0, s, g->d_cap, g->d_base, n,
               t->choff.p, t->cv.p, t->cl0.p, t->cdesc.p, cl);
    SST_LAUNCH(k_compact_ids, blocks_for(n), kTB, 0, s, bigf, bigp, n, t->big.p);
    SST_LAUNCH(k_compact_ids, blocks_for(n), kTB, 0, s, multif, multip, n, t->multi.p);
    SST_LAUNCH(k_compact_ids, blocks_for(n), kTB, 0, s, smallf, smallp, n, t->small.p);
    if (t->nsmall)
      SST_LAUNCH(k_small_desc, blocks_for(t->nsmall), kTB, 0, s, t->small.p,
                 t->nsmall, g->d_base, g->d_deg, t->sdesc.p);
  }
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  SST_CUDA_TRY(cudaGetLastError());
  t->version = g->version;
  t->lists_cl = cl;
  t->lists_stamp++;
  return SST_OK;
}

sst_status pagerank(sst_graph *g, uint32_t iters, double damping, double *d_rank) {
  sst_status st = ensure_lists(g);
  if (st != SST_OK) return st;
  TravState *t = g->trav;
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  if (n == 0) return SST_OK;
  SST_CUDA_TRY(t->ca.ensure(n));
  SST_CUDA_TRY(t->cb.ensure(n));
  SST_CUDA_TRY(t->partial.ensure(t->nchunks + 1));
  unsigned long long *rdeg = reinterpret_cast<unsigned long long *>(t->inv_deg.p);
  if (t->inv_version != g->version) {
    SST_CUDA_TRY(t->inv_deg.ensure(n));
    rdeg = reinterpret_cast<unsigned long long *>(t->inv_deg.p);
    SST_LAUNCH(k_pr_rdeg, blocks_for(n), kTB, 0, s, g->d_deg, n, rdeg);
    t->inv_version = g->version;
  }
  static bool carveout = false;
  if (!carveout) {
    // these kernels use no shared memory: give the SM's storage to L1
    cudaFuncSetAttribute(k_pr_small<4>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    cudaFuncSetAttribute(k_pr_small<8>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    cudaFuncSetAttribute(k_pr_small<16>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    cudaFuncSetAttribute(k_pr_chunks, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    carveout = true;
  }
  double r0 = 1.0 / (double)n;
  double base = (1.0 - damping) / (double)n;
  if (iters == 0) {
    SST_LAUNCH(k_fill_d, blocks_for(n), kTB, 0, s, d_rank, n, r0);
    SST_CUDA_TRY(cudaGetLastError());
    return SST_OK;
  }
  unsigned long long r0f = 0;
  const PrConst K = pr_const(n, damping, &r0f);
  unsigned long long *cin = reinterpret_cast<unsigned long long *>(t->ca.p);
  unsigned long long *cout = reinterpret_cast<unsigned long long *>(t->cb.p);
  unsigned long long *part = reinterpret_cast<unsigned long long *>(t->partial.p);
  // the shared-memory cache: at most the rows, at most 24,576 entries
  // (192 KiB), one copy per block; persistent grids sized by occupancy at
  // that footprint (more than 8,192 entries leaves under three blocks/SM)
  const uint32_t hot = std::min<uint32_t>(t->pr_hot, std::min<uint32_t>(n, 24576));
  const size_t hot_bytes = (size_t)hot * 8;
  const bool big = hot > kHotBig;  // 1024-thread blocks
  const int hot_threads = big ? 1024 : kHotThreads;
  unsigned hot_grid[4] = {1, 1, 1, 1};
  if (hot) {
    const void *fns[4] = {
        big ? (const void *)k_pr_small_hot<4, 1024> : (const void *)k_pr_small_hot<4>,
        big ? (const void *)k_pr_small_hot<8, 1024> : (const void *)k_pr_small_hot<8>,
        big ? (const void *)k_pr_small_hot<16, 1024> : (const void *)k_pr_small_hot<16>,
        big ? (const void *)k_pr_chunks_hot<1024> : (const void *)k_pr_chunks_hot<>};
    for (int i = 0; i < 4; i++) {
      SST_CUDA_TRY(cudaFuncSetAttribute(fns[i], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)hot_bytes));
      int per_sm = 0;
      SST_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fns[i], hot_threads,
                                                                 hot_bytes));
      hot_grid[i] = (unsigned)std::max(1, per_sm) * (unsigned)g->sms;
    }
  }
  auto launch_all = [&]() {
    unsigned long long *ci = cin, *co = cout;
    SST_LAUNCH(k_pr_start, blocks_for(n), kTB, 0, s, g->d_deg, n, r0f, rdeg, ci, co,
               d_rank, base);
    DGraph dg = g->view();
    for (uint32_t it = 0; it < iters; it++) {
      bool last = it + 1 == iters;
      if (hot && t->nsmall) {
#define SST_PR_SMALL_HOT(G, I)                                                        \
  do {                                                                              \
    if (big)                                                                        \
      SST_LAUNCH((k_pr_small_hot<G, 1024>), hot_grid[I], 1024, hot_bytes, s, dg,    \
                 t->sdesc.p, t->small.p, t->nsmall, ci, co, d_rank, rdeg, K, last, hot); \
    else                                                                            \
      SST_LAUNCH((k_pr_small_hot<G>), hot_grid[I], kHotThreads, hot_bytes, s, dg,   \
                 t->sdesc.p, t->small.p, t->nsmall, ci, co, d_rank, rdeg, K, last, hot); \
  } while (0)
        if (t->pr_lanes == 4)
          SST_PR_SMALL_HOT(4, 0);
        else if (t->pr_lanes == 16)
          SST_PR_SMALL_HOT(16, 2);
        else
          SST_PR_SMALL_HOT(8, 1);
#undef SST_PR_SMALL_HOT
      } else if (t->nsmall) {
        const uint64_t groups = (t->nsmall + kSmallPer - 1) / kSmallPer;
        if (t->pr_lanes == 4)
          SST_LAUNCH(k_pr_small<4>, blocks_for(groups * 4), kTB, 0, s, dg,
                     t->sdesc.p, t->small.p, t->nsmall, ci, co, d_rank, rdeg, K, last);
        else if (t->pr_lanes == 16)
          SST_LAUNCH(k_pr_small<16>, blocks_for(groups * 16), kTB, 0, s, dg,
                     t->sdesc.p, t->small.p, t->nsmall, ci, co, d_rank, rdeg, K, last);
        else
          SST_LAUNCH(k_pr_small<8>, blocks_for(groups * 8), kTB, 0, s, dg,
                     t->sdesc.p, t->small.p, t->nsmall, ci, co, d_rank, rdeg, K, last);
      }
      if (hot && t->nchunks && big)
        SST_LAUNCH(k_pr_chunks_hot<1024>, hot_grid[3], 1024, hot_bytes, s, dg, t->cdesc.p,
                   t->cv.p, t->nchunks, ci, co, d_rank, rdeg, part, K, last, hot);
      else if (hot && t->nchunks)
        SST_LAUNCH(k_pr_chunks_hot<>, hot_grid[3], kHotThreads, hot_bytes, s, dg, t->cdesc.p,
                   t->cv.p, t->nchunks, ci, co, d_rank, rdeg, part, K, last, hot);
      else if (t->nchunks)
        SST_LAUNCH(k_pr_chunks, warp_blocks(t->nchunks), kTB, 0, s, dg, t->cdesc.p,
                   t->cv.p, t->nchunks, ci, co, d_rank, rdeg, part, K, last);
      if (t->nmulti)
        SST_LAUNCH(k_pr_fix, blocks_for(t->nmulti), kTB, 0, s, dg, t->multi.p,
                   t->nmulti, t->choff.p, part, co, d_rank, rdeg, K, last);
      std::swap(ci, co);
    }
  };
  // replay the captured iterations when nothing they depend on changed;
  // with the kernel profiler on, launch them one by one so each is timed
  const void *key[6] = {d_rank, s, cin, cout, part, rdeg};
  bool same = t->pr_exec && t->pr_version == t->lists_stamp &&
              t->pr_lanes_used == t->pr_lanes && t->pr_hot_used == t->pr_hot &&
              t->pr_iters == iters && t->pr_damping == damping;
  for (int i = 0; i < 6 && same; i++) same = t->pr_key[i] == key[i];
  if (profiling("k_pr_chunks") || profiling("k_pr_small")) {
    launch_all();
    SST_CUDA_TRY(cudaGetLastError());
    return SST_OK;
  }
  if (!same) {
    if (t->pr_exec) cudaGraphExecDestroy(t->pr_exec);
    t->pr_exec = nullptr;
    cudaGraph_t graph = nullptr;
    const uint64_t l0 = launches();
    SST_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    launch_all();
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    t->pr_kernels = (int64_t)(launches() - l0);
    note_launches(-t->pr_kernels);  // captured, not launched
    if (e == cudaSuccess) e = cudaGraphInstantiate(&t->pr_exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      t->pr_exec = nullptr;
      SST_CUDA_TRY(e);
    }
    t->pr_version = t->lists_stamp;
    t->pr_lanes_used = t->pr_lanes;
    t->pr_hot_used = t->pr_hot;
    t->pr_iters = iters;
    t->pr_damping = damping;
    for (int i = 0; i < 6; i++) t->pr_key[i] = key[i];
  }
  SST_CUDA_TRY(cudaGraphLaunch(t->pr_exec, s));
  note_launches(t->pr_kernels);
  return SST_OK;
}

// BFS from src; with d_levels (n entries, device) it also lists the vertices
// level by level, as the level queues come (each level's new queue is
// copied after the level), their counts in *level_counts.
static sst_status bfs_run(sst_graph *g, uint32_t src, int32_t *d_parents, int32_t *d_depths,
                          uint32_t *d_levels, std::vector<uint32_t> *level_counts) {
  sst_status st = ensure_lists(g);
  if (st != SST_OK) return st;
  TravState *t = g->trav;
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  SST_CUDA_TRY(t->qa.ensure(n + 1));
  SST_CUDA_TRY(t->qb.ensure(n + 1));
  SST_CUDA_TRY(t->fbits.ensure(n / 32 + 2));
  int32_t *depth = d_depths, *parent = d_parents;
  if (!depth) {
    SST_CUDA_TRY(t->depth_tmp.ensure(n));
    depth = t->depth_tmp.p;
  }
  if (!parent) {
    SST_CUDA_TRY(t->parent_tmp.ensure(n));
    parent = t->parent_tmp.p;
  }
  DGraph dg = g->view();
  SST_LAUNCH(k_bfs_init, blocks_for(n), kTB, 0, s, depth, parent, n, src);
  SST_CUDA_TRY(cudaMemcpyAsync(t->qa.p, &src, 4, cudaMemcpyHostToDevice, s));
  uint32_t sinfo[2] = {0, 0};
  SST_CUDA_TRY(cudaMemcpyAsync(&sinfo[0], g->d_deg + src, 4, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaMemcpyAsync(&sinfo[1], g->d_cap + src, 4, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t qn = 1, qdeg = sinfo[0];
  uint64_t qitems = sinfo[1] > kLeaf ? ((sinfo[1] >> kLeafLog) + kPushLeaves - 1) / kPushLeaves : 1;
  uint32_t *q = t->qa.p, *nq = t->qb.p;
  unsigned long long *cnt = t->d_small;
  const uint64_t m = g->m;
  uint64_t listed = 0;  // vertices listed in d_levels so far
  if (d_levels) {
    level_counts->assign(1, 1u);  // level 0: the source
    SST_CUDA_TRY(cudaMemcpyAsync(d_levels, &src, 4, cudaMemcpyHostToDevice, s));
    listed = 1;
  }
  SST_CUDA_TRY(t->icnt.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->ioff.ensure((uint64_t)n + 1));
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes((uint64_t)n + 1, 4) + 4096));
  for (int lvl = 0; qn > 0; lvl++) {
    if ((uint64_t)lvl > n) {
      set_error_message("BFS exceeded n levels");
      return SST_ETIMEDOUT;
    }
    SST_CUDA_TRY(cudaMemsetAsync(cnt, 0, 24, s));
    if ((qn + qdeg) * t->bfs_alpha > m) {
      SST_CUDA_TRY(cudaMemsetAsync(t->fbits.p, 0, ((uint64_t)n / 32 + 1) * 4, s));
      SST_LAUNCH(k_q2bits, blocks_for(qn), kTB, 0, s, q, (uint32_t)qn, t->fbits.p);
      if (t->nsmall)
        SST_LAUNCH(k_bfs_pull_small8, blocks_for((t->nsmall + 3) / 4 * 8), kTB, 0,
                   s, dg, t->sdesc.p, t->small.p, t->nsmall, t->fbits.p, depth,
                   parent, nq, cnt, lvl);
      if (t->nchunks)
        SST_LAUNCH(k_bfs_pull_chunks, warp_blocks(t->nchunks), kTB, 0, s, dg,
                   t->cdesc.p, t->cv.p, t->nchunks, t->fbits.p, depth, parent,
                   nq, cnt, lvl);
    } else {
      SST_CUDA_TRY(t->iv.ensure(qitems + 1));
      SST_CUDA_TRY(t->il0.ensure(qitems + 1));
      SST_LAUNCH(k_front_items, blocks_for(qn), kTB, 0, s, q, (uint32_t)qn,
                 g->d_cap, t->icnt.p);
      g->arena.reset();
      SST_CUDA_TRY((scan<uint32_t, OpAdd>(t->icnt.p, t->ioff.p, qn, 0u, OpAdd{},
                                          true, false, nullptr, g->arena, s)));
      SST_LAUNCH(k_front_expand, blocks_for(qn), kTB, 0, s, q, (uint32_t)qn,
                 g->d_cap, t->ioff.p, t->iv.p, t->il0.p);
      SST_LAUNCH(k_bfs_push, warp_blocks(qitems), kTB, 0, s, dg, t->iv.p, t->il0.p,
                 (uint32_t)qitems, depth, parent, nq, cnt, lvl);
    }
    SST_CUDA_TRY(cudaMemcpyAsync(t->h_small, cnt, 24, cudaMemcpyDeviceToHost, s));
    SST_CUDA_TRY(cudaStreamSynchronize(s));
    qn = t->h_small[0];
    qdeg = t->h_small[1];
    qitems = t->h_small[2];
    if (d_levels && qn) {
      if (listed + qn > n) {
        set_error_message("BFS listed more than n vertices");
        return SST_EDEVICE;
      }
      SST_CUDA_TRY(cudaMemcpyAsync(d_levels + listed, nq, qn * 4, cudaMemcpyDeviceToDevice, s));
      level_counts->push_back((uint32_t)qn);
      listed += qn;
    }
    std::swap(q, nq);
  }
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status bfs(sst_graph *g, uint32_t src, int32_t *d_parents, int32_t *d_depths) {
  return bfs_run(g, src, d_parents, d_depths, nullptr, nullptr);
}

sst_status cc(sst_graph *g, uint32_t *d_labels) {
  sst_status st = ensure_lists(g);
  if (st != SST_OK) return st;
  TravState *t = g->trav;
  cudaStream_t s = g->stream;
  const uint32_t n = g->n;
  if (n == 0) return SST_OK;
  uint32_t *par = d_labels;
  unsigned long long *giant = t->d_small, *err = t->d_small + 1;
  SST_CUDA_TRY(cudaMemsetAsync(t->d_small, 0, 16, s));
  const DGraph dg = g->view();
  SST_LAUNCH(k_iota, blocks_for(n), kTB, 0, s, par, n);
  for (uint32_t r = 0; r < 2; r++) {
    SST_LAUNCH(k_cc_sample, blocks_for(n), kTB, 0, s, dg, r, par, err);
    SST_LAUNCH(k_cc_compress, blocks_for(n), kTB, 0, s, par, n);
  }
  SST_LAUNCH(k_cc_giant, 1, 1024, 0, s, par, n, giant);
  if (t->nsmall)
    SST_LAUNCH(k_cc_rest_small, blocks_for(t->nsmall), kTB, 0, s, dg, t->sdesc.p,
               t->small.p, t->nsmall, giant, par, err);
  if (t->nchunks)
    SST_LAUNCH(k_cc_rest_chunks, warp_blocks(t->nchunks), kTB, 0, s, dg, t->cdesc.p,
               t->cv.p, t->nchunks, giant, par, err);
  SST_LAUNCH(k_cc_compress, blocks_for(n), kTB, 0, s, par, n);
  SST_CUDA_TRY(cudaMemcpyAsync(t->h_small, t->d_small, 16, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  SST_CUDA_TRY(cudaGetLastError());
  if (t->h_small[1]) {
    set_error_message("connected components: %llu links gave up",
                      (unsigned long long)t->h_small[1]);
    return SST_ETIMEDOUT;
  }
  return SST_OK;
}

sst_status bc(sst_graph *g, uint32_t src, double *d_dep) {
  TravState *t = state(g);
  uint32_t n = g->n;
  SST_CUDA_TRY(t->depth_tmp.ensure(n));
  SST_CUDA_TRY(t->lvl_list.ensure(n + 1));
  // the BFS lists the vertices level by level as its queues come (their
  // order within a level does not enter any per-vertex sum below)
  std::vector<uint32_t> hc;
  sst_status st = bfs_run(g, src, nullptr, t->depth_tmp.p, t->lvl_list.p, &hc);
  if (st != SST_OK) return st;
  cudaStream_t s = g->stream;
  const int32_t *depth = t->depth_tmp.p;
  const uint32_t D = (uint32_t)hc.size() - 1;  // deepest level
  hc.resize(D + 2, 0u);
  SST_CUDA_TRY(t->lvl_cnt.ensure(2 * ((uint64_t)D + 2)));
  SST_CUDA_TRY(t->sigma.ensure(n));
  SST_CUDA_TRY(t->ratio.ensure(n));
  uint32_t *off = t->lvl_cnt.p, *ibound = off + D + 2;
  std::vector<uint32_t> ho(D + 2), hib(D + 2);
  uint32_t acc = 0;
  for (uint32_t d = 0; d <= D; d++) {
    ho[d] = acc;
    acc += hc[d];
  }
  ho[D + 1] = acc;
  const uint32_t R = acc;  // reached vertices
  SST_CUDA_TRY(cudaMemcpyAsync(off, ho.data(), (D + 2) * 4, cudaMemcpyHostToDevice, s));
  // chunk items of the big vertices, in level-list order
  SST_CUDA_TRY(t->icnt.ensure((uint64_t)R + 1));
  SST_CUDA_TRY(t->ioff.ensure((uint64_t)R + 1));
  const uint32_t *list = t->lvl_list.p;
  SST_LAUNCH(k_bc_item_counts, blocks_for(R), kTB, 0, s, list, R, g->d_cap, t->icnt.p);
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes((uint64_t)R + 1, 4) + 4096));
  SST_CUDA_TRY((scan<uint32_t, OpAdd>(t->icnt.p, t->ioff.p, R, 0u, OpAdd{}, true,
                                      false, t->ioff.p + R, g->arena, s)));
  SST_LAUNCH(k_gather_bounds, blocks_for(D + 2), kTB, 0, s, t->ioff.p, off,
             D + 2, ibound);
  SST_CUDA_TRY(cudaMemcpyAsync(hib.data(), ibound, (D + 2) * 4, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint32_t items = hib[D + 1];
  SST_CUDA_TRY(t->iv.ensure((uint64_t)items + 1));
  SST_CUDA_TRY(t->il0.ensure((uint64_t)items + 1));
  SST_CUDA_TRY(t->partial.ensure((uint64_t)items + 1));
  if (items)
    SST_LAUNCH(k_bc_expand, blocks_for(R), kTB, 0, s, list, R, t->icnt.p,
               t->ioff.p, t->iv.p, t->il0.p);
  SST_LAUNCH(k_bc_init, blocks_for(n), kTB, 0, s, t->sigma.p, t->ratio.p, d_dep, n, src);
  DGraph dg = g->view();
  double *part = t->partial.p;
  for (uint32_t d = 1; d <= D; d++) {
    uint32_t c = hc[d], ni = hib[d + 1] - hib[d];
    const uint32_t *lst = list + ho[d];
    SST_LAUNCH(k_sigma_small, blocks_for(c), kTB, 0, s, dg, lst, c, depth, t->sigma.p, (int32_t)d);
    if (ni) {
      SST_LAUNCH(k_bc_chunks, warp_blocks(ni), kTB, 0, s, dg, t->iv.p, t->il0.p,
                 hib[d], ni, depth, t->sigma.p, (int32_t)d - 1, part);
      SST_LAUNCH(k_bc_fix, blocks_for(c), kTB, 0, s, list, ho[d], c, t->icnt.p,
                 t->ioff.p, part, true, t->sigma.p, t->ratio.p, d_dep);
    }
  }
  for (int32_t d = (int32_t)D; d >= 0; d--) {
    uint32_t c = hc[d], ni = hib[d + 1] - hib[d];
    const uint32_t *lst = list + ho[d];
    SST_LAUNCH(k_delta_small, blocks_for(c), kTB, 0, s, dg, lst, c, depth,
               t->sigma.p, t->ratio.p, d_dep, d);
    if (ni) {
      SST_LAUNCH(k_bc_chunks, warp_blocks(ni), kTB, 0, s, dg, t->iv.p, t->il0.p,
                 hib[d], ni, depth, t->ratio.p, d + 1, part);
      SST_LAUNCH(k_bc_fix, blocks_for(c), kTB, 0, s, list, ho[d], c, t->icnt.p,
                 t->ioff.p, part, false, t->sigma.p, t->ratio.p, d_dep);
    }
  }
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status tc(sst_graph *g, uint64_t *total, uint64_t *d_pv) {
  sst_status st = ensure_leaf_dir(g);
  if (st != SST_OK) return st;
  TravState *t = state(g);
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  LeafDir &D = g->dir;
  uint64_t nl = D.nleaves;
  SST_CUDA_TRY(t->tlcnt.ensure(nl + 1));
  SST_CUDA_TRY(t->tlpre.ensure(nl + 1));
  SST_CUDA_TRY(t->tmask.ensure(nl + 1));
  SST_CUDA_TRY(t->toff.ensure((uint64_t)n + 1));
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes(nl + 1, 8) + 4096));
  const uint64_t tc_warps = (nl + kTcLeaves - 1) / kTcLeaves;
  if (nl)
    SST_LAUNCH(k_tc_leafcount, warp_blocks(tc_warps), kTB, 0, s, g->d_slots, D.owner,
               D.slot, D.cnt, nl, g->d_deg, t->tlcnt.p, t->tmask.p);
  SST_CUDA_TRY((scan<uint64_t, OpAdd>(t->tlcnt.p, t->tlpre.p, nl, 0ull, OpAdd{},
                                      true, false, t->tlpre.p + nl, g->arena, s)));
  uint64_t madj = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(&madj, t->tlpre.p + nl, 8, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  SST_CUDA_TRY(t->tadj.ensure(madj + 1));
  SST_CUDA_TRY(t->icnt.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->ioff.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->titems.ensure(tc_items_bound(n, madj)));
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes((uint64_t)n + 1, 4) + 4096));
  if (nl)
    SST_LAUNCH(k_tc_fill, warp_blocks(tc_warps), kTB, 0, s, g->d_slots, D.slot, nl,
               t->tmask.p, t->tlpre.p, t->tadj.p);
  SST_LAUNCH(k_tc_off, blocks_for((uint64_t)n + 1), kTB, 0, s, D.vleaf,
             t->tlpre.p, n, t->toff.p);
  SST_CUDA_TRY(cudaMemsetAsync(t->d_small, 0, 16, s));  // count, work cursor
  if (d_pv) SST_CUDA_TRY(cudaMemsetAsync(d_pv, 0, (uint64_t)n * 8, s));
  if (n)
    SST_CUDA_TRY(tc_count_launch(t->toff.p, t->tadj.p, n, madj,
                                 TcScratch{t->icnt.p, t->ioff.p, t->titems.p}, g->arena,
                                 t->d_small,
                                 reinterpret_cast<unsigned long long *>(d_pv), g->sms, s));
  SST_CUDA_TRY(cudaMemcpyAsync(t->h_small, t->d_small, 8, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  SST_CUDA_TRY(cudaGetLastError());
  *total = t->h_small[0];
  return SST_OK;
}

sst_status common_neighbors_batch(sst_graph *g, const uint32_t *d_pairs,
                                  uint64_t n, bool early_end, uint64_t *d_out) {
  if (n == 0) return SST_OK;
  SST_LAUNCH(k_common, blocks_for(n), kTB, 0, g->stream, g->view(), d_pairs, n,
             early_end, d_out);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}


// ================================================ multi-source BFS and BC
// Multi-source BFS: k <= 64 sources traverse together.  Each vertex holds a
// mask of the sources that have reached it (vis) and of those for which it
// is on the current level (fr); one level is one pass for all sources -- a
// push from the frontier queue while the frontier's edges are few, else a
// pull over all unfinished vertices -- followed by one update pass that
// turns the collected masks into new depths and the next queue.
namespace {

__global__ void k_msbfs_seed(const uint32_t *__restrict__ sv,
                             const unsigned long long *__restrict__ sm,
                             uint32_t cnt, uint32_t n,
                             unsigned long long *__restrict__ vis,
                             unsigned long long *__restrict__ fr,
                             int32_t *__restrict__ depth,
                             const uint32_t *__restrict__ deg,
                             const uint32_t *__restrict__ cap,
                             uint32_t *__restrict__ q,
                             unsigned long long *__restrict__ qc) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  uint32_t v = sv[i];
  unsigned long long m = sm[i];
  vis[v] = m;
  fr[v] = m;
  for (unsigned long long b = m; b; b &= b - 1)
    depth[(uint64_t)(__ffsll((long long)b) - 1) * n + v] = 0;
  q[i] = v;
  atomicAdd(&qc[1], (unsigned long long)deg[v]);
  atomicAdd(&qc[2], (unsigned long long)items_of(cap[v]));
}

// push: warp per work item (a frontier vertex's leaf chunk), lane = slot
__global__ void __launch_bounds__(kTB, 8)
k_msbfs_push(DGraph g, const uint32_t *__restrict__ iv,
             const uint32_t *__restrict__ il0, uint32_t nitems,
             const unsigned long long *__restrict__ fr,
             const unsigned long long *__restrict__ vis,
             unsigned long long *__restrict__ nx) {
  uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= nitems) return;
  uint32_t u = iv[i];
  const unsigned long long f = fr[u];
  uint64_t base = g.base[u];
  uint32_t cap = g.cap[u], deg = g.deg[u];
  uint32_t nl = cap ? nleaves_of(cap) : 0;
  uint32_t l0 = il0[i], l1 = min(l0 + kPushLeaves, nl);
  // four leaves' slots and visited masks in flight at once; leaves keep
  // their ids packed left with EMPTY after them
  constexpr int kBatch = 4;
  const uint32_t lim = cap <= kLeaf ? deg : kLeaf;
  for (uint32_t l = l0; l < l1; l += kBatch) {
    uint32_t w[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; k++)
      w[k] = (l + k < l1 && (uint32_t)lane < lim)
                 ? g.slots[base + ((uint64_t)(l + k) << kLeafLog) + lane]
                 : kEmpty;
    unsigned long long add[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; k++) add[k] = w[k] != kEmpty ? f & ~vis[w[k]] : 0ull;
#pragma unroll
    for (int k = 0; k < kBatch; k++)
      if (add[k]) atomicOr(&nx[w[k]], add[k]);
  }
}

// pull, one-leaf vertices: thread per vertex, stops once every source that
// has not reached v is seen in the frontier
__global__ void k_msbfs_pull_small(DGraph g, const uint32_t *__restrict__ small,
                                   uint64_t nsmall,
                                   const unsigned long long *__restrict__ fr,
                                   const unsigned long long *__restrict__ vis,
                                   unsigned long long *__restrict__ nx,
                                   unsigned long long full) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsmall) return;
  uint32_t v = small[i];
  const unsigned long long need = full & ~vis[v];
  if (!need) return;
  const uint32_t *p = g.slots + g.base[v];
  uint32_t d = g.deg[v];
  unsigned long long acc = 0;
  // four neighbours' ids, then their four masks, in flight per step
  for (uint32_t k = 0; k < d; k += 4) {
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; q++) w[q] = k + q < d ? p[k + q] : kEmpty;
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (w[q] != kEmpty) acc |= fr[w[q]];
    if ((acc & need) == need) break;
  }
  acc &= need;
  if (acc) nx[v] = acc;
}

__device__ __forceinline__ unsigned long long warp_or64(unsigned long long x) {
  unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)x);
  unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(x >> 32));
  return ((unsigned long long)hi << 32) | lo;
}

// pull, multi-leaf vertices: warp per chunk (lane = slot), early exit
__global__ void k_msbfs_pull_chunks(DGraph g,
                                    const unsigned long long *__restrict__ cdesc,
                                    const uint32_t *__restrict__ cv,
                                    uint64_t nchunks,
                                    const unsigned long long *__restrict__ fr,
                                    const unsigned long long *__restrict__ vis,
                                    unsigned long long *__restrict__ nx,
                                    unsigned long long full) {
  uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= nchunks) return;
  const uint32_t v = cv[c];
  const unsigned long long need = full & ~vis[v];
  if (!need) return;
  const unsigned long long dsc = cdesc[c];
  const uint64_t leaf0 = dsc >> 8;
  const uint32_t l1 = (uint32_t)(dsc & 63);
  const bool single = (dsc >> 7) & 1;
  const uint32_t mycnt = (uint32_t)lane < l1 ? g.lcnt[leaf0 + lane] : 0u;
  const uint32_t *sl = g.slots + (leaf0 << kLeafLog) + lane;
  unsigned long long acc = 0;
  for (uint32_t l = 0; l < l1; l += 4) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      uint32_t cq = __shfl_sync(0xffffffffu, mycnt, (l + q) & 31);
      if (l + q >= l1) cq = 0;
      if ((uint32_t)lane < cq) acc |= fr[sl[(uint64_t)(l + q) << kLeafLog]];
    }
    if ((warp_or64(acc) & need) == need) break;
  }
  acc = warp_or64(acc) & need;
  if (lane == 0 && acc) {
    if (single)
      nx[v] = acc;
    else
      atomicOr(&nx[v], acc);
  }
}

// new sources per vertex -> depths, next frontier masks and queue
__global__ void k_msbfs_update(uint32_t n, unsigned long long *__restrict__ vis,
                               unsigned long long *__restrict__ nx,
                               unsigned long long *__restrict__ fr_next,
                               int32_t *__restrict__ depth, int32_t lvl,
                               const uint32_t *__restrict__ deg,
                               const uint32_t *__restrict__ cap,
                               uint32_t *__restrict__ q,
                               unsigned long long *__restrict__ qc) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long nw = 0;
  if (v < n) {
    unsigned long long x = nx[v];
    if (x) {
      nx[v] = 0;
      unsigned long long old = vis[v];
      nw = x & ~old;
      if (nw) {
        vis[v] = old | nw;
        for (unsigned long long b = nw; b; b &= b - 1)
          depth[(uint64_t)(__ffsll((long long)b) - 1) * n + v] = lvl;
      }
    }
    fr_next[v] = nw;
  }
  enqueue_block(nw != 0, v, nw ? deg[v] : 0u, nw ? items_of(cap[v]) : 0u, q, qc);
}

// ---- multi-source BC: the single-source passes with the source on
// blockIdx.y; per (source, level) the list start, list count, item start and
// item count come from tab[(s * L + d) * 4 + 0..3]
__global__ void k_msbc_maxdepth(const int32_t *__restrict__ depth, uint32_t n,
                                unsigned long long *__restrict__ out) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  block_max_to(v < n ? depth[(uint64_t)blockIdx.y * n + v] : -1, out);
}

__global__ void k_msbc_level_count(const int32_t *__restrict__ depth, uint32_t n,
                                   uint32_t L, uint32_t *__restrict__ cnt) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t d = v < n ? depth[(uint64_t)blockIdx.y * n + v] : -1;
  level_add(cnt + blockIdx.y * L + (d >= 0 ? d : 0), d, d >= 0);
}

__global__ void k_msbc_level_scatter(const int32_t *__restrict__ depth,
                                     uint32_t n, uint32_t L,
                                     const uint32_t *__restrict__ start,
                                     uint32_t *__restrict__ ctr,
                                     uint32_t *__restrict__ list) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t d = v < n ? depth[(uint64_t)blockIdx.y * n + v] : -1;
  const uint32_t a = blockIdx.y * L + (d >= 0 ? d : 0);
  const uint32_t at = level_add(ctr + a, d, d >= 0);
  if (d >= 0) list[start[a] + at] = v;
}

__global__ void k_msbc_init(const uint32_t *__restrict__ srcs, uint32_t n,
                            double *__restrict__ sigma, double *__restrict__ ratio,
                            double *__restrict__ dep) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  uint64_t at = (uint64_t)blockIdx.y * n + v;
  sigma[at] = v == srcs[blockIdx.y] ? 1.0 : 0.0;
  ratio[at] = 0.0;
  dep[at] = 0.0;
}

__global__ void k_msbc_sigma_small(DGraph g, const uint32_t *__restrict__ list,
                                   const uint32_t *__restrict__ tab, uint32_t L,
                                   int32_t d, const int32_t *__restrict__ depth,
                                   double *__restrict__ sigma) {
  const uint32_t *e = tab + ((uint64_t)blockIdx.y * L + d) * 4;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= e[1]) return;
  uint32_t v = list[e[0] + i];
  if (g.cap[v] > kLeaf) return;
  const uint64_t so = (uint64_t)blockIdx.y * g.n;
  const uint32_t *p = g.slots + g.base[v];
  uint32_t dg = g.deg[v];
  double acc = 0.0;
  for (uint32_t k0 = 0; k0 < dg; k0 += kBcAhead) {  // as in k_sigma_small
    uint32_t u[kBcAhead];
    bool on[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) u[q] = k0 + q < dg ? p[k0 + q] : 0u;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) on[q] = k0 + q < dg && depth[so + u[q]] == d - 1;
    double x[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) x[q] = on[q] ? sigma[so + u[q]] : 0.0;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++)
      if (on[q]) acc += x[q];
  }
  sigma[so + v] = acc;
}

__global__ void k_msbc_chunks(DGraph g, const uint32_t *__restrict__ iv,
                              const uint32_t *__restrict__ il0,
                              const uint32_t *__restrict__ tab, uint32_t L,
                              int32_t d, const int32_t *__restrict__ depth,
                              const double *__restrict__ val, int32_t want,
                              double *__restrict__ partial) {
  const uint32_t *e = tab + ((uint64_t)blockIdx.y * L + d) * 4;
  uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= e[3]) return;
  i += e[2];
  const uint64_t so = (uint64_t)blockIdx.y * g.n;
  uint32_t v = iv[i];
  uint32_t nl = g.cap[v] >> kLeafLog;
  uint32_t l0 = il0[i], l1 = min(l0 + kChunkLeaves, nl);
  uint64_t base = g.base[v];
  // eight leaves' slots, depths and values in flight at once (the leaves of
  // a multi-leaf segment keep their ids packed left with EMPTY after them);
  // each lane still adds in leaf order
  constexpr int kBatch = 8;
  double acc = 0.0;
  for (uint32_t l = l0; l < l1; l += kBatch) {
    uint32_t u[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; k++)
      u[k] = l + k < l1 ? g.slots[base + ((uint64_t)(l + k) << kLeafLog) + lane] : kEmpty;
    bool on[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; k++) on[k] = u[k] != kEmpty && depth[so + u[k]] == want;
    double x[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; k++) x[k] = on[k] ? val[so + u[k]] : 0.0;
#pragma unroll
    for (int k = 0; k < kBatch; k++)
      if (on[k]) acc += x[k];
  }
  double sum = warp_sum_d(acc);
  if (lane == 0) partial[i] = sum;
}

__global__ void k_msbc_fix(DGraph g, const uint32_t *__restrict__ list,
                           const uint32_t *__restrict__ tab, uint32_t L,
                           int32_t d, const uint32_t *__restrict__ cnt,
                           const uint32_t *__restrict__ off,
                           const double *__restrict__ partial, bool sigma_pass,
                           double *__restrict__ sigma, double *__restrict__ ratio,
                           double *__restrict__ dep) {
  const uint32_t *e = tab + ((uint64_t)blockIdx.y * L + d) * 4;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= e[1]) return;
  uint32_t p = e[0] + i;
  uint32_t k = cnt[p];
  if (k == 0) return;
  double acc = 0.0;
  for (uint32_t j = 0; j < k; j++) acc += partial[off[p] + j];
  const uint64_t at = (uint64_t)blockIdx.y * g.n + list[p];
  if (sigma_pass) {
    sigma[at] = acc;
  } else {
    double dv = sigma[at] * acc;
    dep[at] = dv;
    ratio[at] = (1.0 + dv) / sigma[at];
  }
}

__global__ void k_msbc_delta_small(DGraph g, const uint32_t *__restrict__ list,
                                   const uint32_t *__restrict__ tab, uint32_t L,
                                   int32_t d, const int32_t *__restrict__ depth,
                                   const double *__restrict__ sigma,
                                   double *__restrict__ ratio,
                                   double *__restrict__ dep) {
  const uint32_t *e = tab + ((uint64_t)blockIdx.y * L + d) * 4;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= e[1]) return;
  uint32_t v = list[e[0] + i];
  if (g.cap[v] > kLeaf) return;
  const uint64_t so = (uint64_t)blockIdx.y * g.n;
  const uint32_t *p = g.slots + g.base[v];
  uint32_t dg = g.deg[v];
  double acc = 0.0;
  for (uint32_t k0 = 0; k0 < dg; k0 += kBcAhead) {  // as in k_sigma_small
    uint32_t w[kBcAhead];
    bool on[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) w[q] = k0 + q < dg ? p[k0 + q] : 0u;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) on[q] = k0 + q < dg && depth[so + w[q]] == d + 1;
    double x[kBcAhead];
#pragma unroll
    for (int q = 0; q < kBcAhead; q++) x[q] = on[q] ? ratio[so + w[q]] : 0.0;
#pragma unroll
    for (int q = 0; q < kBcAhead; q++)
      if (on[q]) acc += x[q];
  }
  double dv = sigma[so + v] * acc;
  dep[so + v] = dv;
  ratio[so + v] = (1.0 + dv) / sigma[so + v];
}

}  // namespace

sst_status bfs_multi(sst_graph *g, const uint32_t *h_srcs, uint32_t k,
                     int32_t *d_depth) {
  if (k == 0) return SST_OK;
  if (k > 64) {
    set_error_message("at most 64 sources per multi-source BFS");
    return SST_EINVAL;
  }
  sst_status st = ensure_lists(g);
  if (st != SST_OK) return st;
  TravState *t = g->trav;
  cudaStream_t s = g->stream;
  const uint32_t n = g->n;
  // distinct sources with their source masks
  std::vector<uint32_t> sv;
  std::vector<unsigned long long> sm;
  for (uint32_t i = 0; i < k; i++) {
    if (h_srcs[i] >= n) {
      set_error_message("source %u out of range", h_srcs[i]);
      return SST_EINVAL;
    }
    auto it = std::find(sv.begin(), sv.end(), h_srcs[i]);
    if (it == sv.end()) {
      sv.push_back(h_srcs[i]);
      sm.push_back(1ull << i);
    } else {
      sm[it - sv.begin()] |= 1ull << i;
    }
  }
  const unsigned long long full = k == 64 ? ~0ull : (1ull << k) - 1;
  SST_CUDA_TRY(t->mvis.ensure(n));
  SST_CUDA_TRY(t->mfr.ensure(n));
  SST_CUDA_TRY(t->mfr2.ensure(n));
  SST_CUDA_TRY(t->mnx.ensure(n));
  SST_CUDA_TRY(t->qa.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->qb.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->icnt.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->ioff.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->msrc.ensure(2 * (uint64_t)sv.size()));
  SST_CUDA_TRY(cudaMemsetAsync(t->mvis.p, 0, (uint64_t)n * 8, s));
  SST_CUDA_TRY(cudaMemsetAsync(t->mfr.p, 0, (uint64_t)n * 8, s));
  SST_CUDA_TRY(cudaMemsetAsync(t->mnx.p, 0, (uint64_t)n * 8, s));
  SST_CUDA_TRY(cudaMemsetAsync(d_depth, 0xFF, (uint64_t)k * n * 4, s));
  unsigned long long *d_sm = t->msrc.p;
  uint32_t *d_sv = reinterpret_cast<uint32_t *>(t->msrc.p + sv.size());
  SST_CUDA_TRY(cudaMemcpyAsync(d_sv, sv.data(), sv.size() * 4, cudaMemcpyHostToDevice, s));
  SST_CUDA_TRY(cudaMemcpyAsync(d_sm, sm.data(), sm.size() * 8, cudaMemcpyHostToDevice, s));
  unsigned long long *qc = t->d_small;
  SST_CUDA_TRY(cudaMemsetAsync(qc, 0, 24, s));
  uint32_t *q = t->qa.p, *nq = t->qb.p;
  unsigned long long *fr = t->mfr.p, *fr2 = t->mfr2.p;
  SST_LAUNCH(k_msbfs_seed, blocks_for(sv.size()), kTB, 0, s, d_sv, d_sm,
             (uint32_t)sv.size(), n, t->mvis.p, fr, d_depth, g->d_deg, g->d_cap,
             q, qc);
  SST_CUDA_TRY(cudaMemcpyAsync(t->h_small, qc, 24, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t qn = sv.size(), qdeg = t->h_small[1], qitems = t->h_small[2];
  const uint64_t m = g->m;
  DGraph dg = g->view();
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes((uint64_t)n + 1, 4) + 4096));
  for (int32_t lvl = 0; qn > 0; lvl++) {
    if ((uint64_t)lvl > n) {
      set_error_message("multi-source BFS exceeded n levels");
      return SST_ETIMEDOUT;
    }
    if ((qn + qdeg) * t->bfs_alpha > m) {
      if (t->nsmall)
        SST_LAUNCH(k_msbfs_pull_small, blocks_for(t->nsmall), kTB, 0, s, dg,
                   t->small.p, t->nsmall, fr, t->mvis.p, t->mnx.p, full);
      if (t->nchunks)
        SST_LAUNCH(k_msbfs_pull_chunks, warp_blocks(t->nchunks), kTB, 0, s, dg,
                   t->cdesc.p, t->cv.p, t->nchunks, fr, t->mvis.p, t->mnx.p, full);
    } else {
      SST_CUDA_TRY(t->iv.ensure(qitems + 1));
      SST_CUDA_TRY(t->il0.ensure(qitems + 1));
      SST_LAUNCH(k_front_items, blocks_for(qn), kTB, 0, s, q, (uint32_t)qn,
                 g->d_cap, t->icnt.p);
      g->arena.reset();
      SST_CUDA_TRY((scan<uint32_t, OpAdd>(t->icnt.p, t->ioff.p, qn, 0u, OpAdd{},
                                          true, false, nullptr, g->arena, s)));
      SST_LAUNCH(k_front_expand, blocks_for(qn), kTB, 0, s, q, (uint32_t)qn,
                 g->d_cap, t->ioff.p, t->iv.p, t->il0.p);
      SST_LAUNCH(k_msbfs_push, warp_blocks(qitems), kTB, 0, s, dg, t->iv.p,
                 t->il0.p, (uint32_t)qitems, fr, t->mvis.p, t->mnx.p);
    }
    SST_CUDA_TRY(cudaMemsetAsync(qc, 0, 24, s));
    SST_LAUNCH(k_msbfs_update, blocks_for(n), kTB, 0, s, n, t->mvis.p, t->mnx.p,
               fr2, d_depth, lvl + 1, g->d_deg, g->d_cap, nq, qc);
    SST_CUDA_TRY(cudaMemcpyAsync(t->h_small, qc, 24, cudaMemcpyDeviceToHost, s));
    SST_CUDA_TRY(cudaStreamSynchronize(s));
    qn = t->h_small[0];
    qdeg = t->h_small[1];
    qitems = t->h_small[2];
    std::swap(q, nq);
    std::swap(fr, fr2);
  }
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status bc_multi(sst_graph *g, const uint32_t *h_srcs, uint32_t k,
                    double *d_dep) {
  if (k == 0) return SST_OK;
  TravState *t = state(g);
  const uint32_t n = g->n;
  SST_CUDA_TRY(t->mdepth.ensure((uint64_t)k * n));
  sst_status st = bfs_multi(g, h_srcs, k, t->mdepth.p);
  if (st != SST_OK) return st;
  cudaStream_t s = g->stream;
  const int32_t *depth = t->mdepth.p;
  const dim3 vgrid(blocks_for(n), k);
  SST_CUDA_TRY(cudaMemsetAsync(t->d_small, 0, 8, s));
  SST_LAUNCH(k_msbc_maxdepth, vgrid, kTB, 0, s, depth, n, t->d_small);
  SST_CUDA_TRY(cudaMemcpyAsync(t->h_small, t->d_small, 8, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  const uint32_t D = (uint32_t)t->h_small[0];
  const uint32_t L = D + 2;  // levels 0..D plus an end marker
  // per (source, level): vertex counts -> list starts
  SST_CUDA_TRY(t->mtab.ensure((uint64_t)k * L * 7));
  uint32_t *cnt = t->mtab.p, *start = cnt + (uint64_t)k * L, *ctr = start + (uint64_t)k * L;
  uint32_t *tab = ctr + (uint64_t)k * L;  // k * L * 4 words
  SST_CUDA_TRY(cudaMemsetAsync(cnt, 0, (uint64_t)k * L * 4, s));
  SST_CUDA_TRY(cudaMemsetAsync(ctr, 0, (uint64_t)k * L * 4, s));
  SST_LAUNCH(k_msbc_level_count, vgrid, kTB, 0, s, depth, n, L, cnt);
  std::vector<uint32_t> hc((uint64_t)k * L), hs((uint64_t)k * L);
  SST_CUDA_TRY(cudaMemcpyAsync(hc.data(), cnt, hc.size() * 4, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t acc = 0;
  for (uint64_t i = 0; i < hc.size(); i++) {
    hs[i] = (uint32_t)acc;
    acc += hc[i];
  }
  if (acc >= 0xFFFFFFFFull) {
    set_error_message("too many (source, vertex) pairs for one multi-source BC");
    return SST_EINVAL;
  }
  const uint32_t RR = (uint32_t)acc;
  SST_CUDA_TRY(cudaMemcpyAsync(start, hs.data(), hs.size() * 4, cudaMemcpyHostToDevice, s));
  SST_CUDA_TRY(t->mlist.ensure((uint64_t)RR + 1));
  SST_LAUNCH(k_msbc_level_scatter, vgrid, kTB, 0, s, depth, n, L, start, ctr,
             t->mlist.p);
  // leaf-chunk items of the multi-leaf vertices, in list order
  SST_CUDA_TRY(t->micnt.ensure((uint64_t)RR + 1));
  SST_CUDA_TRY(t->mioff.ensure((uint64_t)RR + 1));
  const uint32_t *list = t->mlist.p;
  if (RR) SST_LAUNCH(k_bc_item_counts, blocks_for(RR), kTB, 0, s, list, RR, g->d_cap, t->micnt.p);
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes((uint64_t)RR + 1, 4) + 4096));
  SST_CUDA_TRY((scan<uint32_t, OpAdd>(t->micnt.p, t->mioff.p, RR, 0u, OpAdd{},
                                      true, false, t->mioff.p + RR, g->arena, s)));
  // item starts at each (source, level) list start, and the total
  std::vector<uint32_t> hpos(hs.size() + 1);
  for (uint64_t i = 0; i < hs.size(); i++) hpos[i] = hs[i];
  hpos[hs.size()] = RR;
  SST_CUDA_TRY(cudaMemcpyAsync(ctr, hpos.data(), (uint64_t)k * L * 4, cudaMemcpyHostToDevice, s));
  std::vector<uint32_t> hib((uint64_t)k * L + 1);
  SST_CUDA_TRY(t->mpart.ensure((uint64_t)k * L + 2));
  uint32_t *d_ib = reinterpret_cast<uint32_t *>(t->mpart.p);
  SST_LAUNCH(k_gather_bounds, blocks_for((uint64_t)k * L), kTB, 0, s, t->mioff.p,
             ctr, (uint32_t)(k * L), d_ib);
  SST_CUDA_TRY(cudaMemcpyAsync(hib.data(), d_ib, (uint64_t)k * L * 4, cudaMemcpyDeviceToHost, s));
  uint32_t items = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(&items, t->mioff.p + RR, 4, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  hib[(uint64_t)k * L] = items;
  // the table: list start, count, item start, item count per (source, level)
  std::vector<uint32_t> ht((uint64_t)k * L * 4);
  std::vector<uint32_t> maxc(L, 0), maxi(L, 0);
  for (uint32_t sidx = 0; sidx < k; sidx++)
    for (uint32_t d = 0; d < L; d++) {
      uint64_t at = (uint64_t)sidx * L + d;
      uint32_t i0 = hib[at], i1 = hib[at + 1];
      ht[at * 4 + 0] = hs[at];
      ht[at * 4 + 1] = hc[at];
      ht[at * 4 + 2] = i0;
      ht[at * 4 + 3] = i1 - i0;
      maxc[d] = std::max(maxc[d], hc[at]);
      maxi[d] = std::max(maxi[d], i1 - i0);
    }
  SST_CUDA_TRY(cudaMemcpyAsync(tab, ht.data(), ht.size() * 4, cudaMemcpyHostToDevice, s));
  SST_CUDA_TRY(t->miv.ensure((uint64_t)items + 1));
  SST_CUDA_TRY(t->mil0.ensure((uint64_t)items + 1));
  SST_CUDA_TRY(t->mpart.ensure((uint64_t)items + 1));
  if (items && RR)
    SST_LAUNCH(k_bc_expand, blocks_for(RR), kTB, 0, s, list, RR, t->micnt.p,
               t->mioff.p, t->miv.p, t->mil0.p);
  SST_CUDA_TRY(t->msig.ensure((uint64_t)k * n));
  SST_CUDA_TRY(t->mrat.ensure((uint64_t)k * n));
  // the sources, staged in the (now free) scatter counters
  SST_CUDA_TRY(cudaMemcpyAsync(ctr, h_srcs, (uint64_t)k * 4, cudaMemcpyHostToDevice, s));
  SST_LAUNCH(k_msbc_init, vgrid, kTB, 0, s, ctr, n, t->msig.p, t->mrat.p, d_dep);
  DGraph dg = g->view();
  double *part = t->mpart.p;
  for (uint32_t d = 1; d <= D; d++) {
    if (maxc[d])
      SST_LAUNCH(k_msbc_sigma_small, dim3(blocks_for(maxc[d]), k), kTB, 0, s, dg,
                 list, tab, L, (int32_t)d, depth, t->msig.p);
    if (maxi[d]) {
      SST_LAUNCH(k_msbc_chunks, dim3(warp_blocks(maxi[d]), k), kTB, 0, s, dg,
                 t->miv.p, t->mil0.p, tab, L, (int32_t)d, depth, t->msig.p,
                 (int32_t)d - 1, part);
      SST_LAUNCH(k_msbc_fix, dim3(blocks_for(maxc[d]), k), kTB, 0, s, dg, list,
                 tab, L, (int32_t)d, t->micnt.p, t->mioff.p, part, true,
                 t->msig.p, t->mrat.p, d_dep);
    }
  }
  for (int32_t d = (int32_t)D; d >= 0; d--) {
    if (maxc[d])
      SST_LAUNCH(k_msbc_delta_small, dim3(blocks_for(maxc[d]), k), kTB, 0, s, dg,
                 list, tab, L, d, depth, t->msig.p, t->mrat.p, d_dep);
    if (maxi[d]) {
      SST_LAUNCH(k_msbc_chunks, dim3(warp_blocks(maxi[d]), k), kTB, 0, s, dg,
                 t->miv.p, t->mil0.p, tab, L, d, depth, t->mrat.p, d + 1, part);
      SST_LAUNCH(k_msbc_fix, dim3(blocks_for(maxc[d]), k), kTB, 0, s, dg, list,
                 tab, L, d, t->micnt.p, t->mioff.p, part, false, t->msig.p,
                 t->mrat.p, d_dep);
    }
  }
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}


// ------------------------------------------------------------- autotuner
// Times the traversal knobs on this graph and keeps the fastest: PageRank
// (3 iterations) over chunk sizes {8, 16, 32} x lanes {4, 8, 16}, then its
// shared-memory cache {0, 2048, 4096, 8192}, then BFS from three sources
// over push/pull thresholds {5, 10, 20, 40, 80}.
sst_status get_tuning(sst_graph *g, sst_tuning *out) {
  TravState *t = state(g);
  out->chunk_leaves = t->chunk_leaves;
  out->pr_lanes = t->pr_lanes;
  out->bfs_alpha = t->bfs_alpha;
  out->pr_hot = t->pr_hot;
  out->pr_ms = 0.f;
  out->bfs_ms = 0.f;
  return SST_OK;
}

sst_status set_tuning(sst_graph *g, const sst_tuning *in) {
  if (in->chunk_leaves < 1 || in->chunk_leaves > 32 ||
      (in->pr_lanes != 4 && in->pr_lanes != 8 && in->pr_lanes != 16) ||
      in->bfs_alpha < 1 || in->pr_hot > 24576) {
    set_error_message("tuning out of range (chunk_leaves 1..32, pr_lanes 4/8/16, "
                      "bfs_alpha >= 1, pr_hot <= 24576)");
    return SST_EINVAL;
  }
  TravState *t = state(g);
  t->chunk_leaves = in->chunk_leaves;
  t->pr_lanes = in->pr_lanes;
  t->bfs_alpha = in->bfs_alpha;
  t->pr_hot = in->pr_hot;
  return SST_OK;
}

sst_status autotune(sst_graph *g, sst_tuning *out) {
  TravState *t = state(g);
  const uint32_t n = g->n;
  sst_status st = get_tuning(g, out);
  if (st != SST_OK || n == 0 || g->m == 0) return st;
  cudaStream_t s = g->stream;
  double *rank = nullptr;
  int32_t *dep = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  SST_CUDA_TRY(cudaMalloc(&rank, (uint64_t)n * 8));
  SST_CUDA_TRY(cudaMalloc(&dep, (uint64_t)n * 4));
  SST_CUDA_TRY(cudaEventCreate(&e0));
  SST_CUDA_TRY(cudaEventCreate(&e1));
  float best_pr = 1e30f, best_bfs = 1e30f;
  uint32_t bcl = t->chunk_leaves, blanes = t->pr_lanes, balpha = t->bfs_alpha;
  auto timed = [&](auto fn, float *ms) -> sst_status {
    sst_status r = fn();  // warm (lists, captured graph)
    if (r != SST_OK) return r;
    SST_CUDA_TRY(cudaEventRecord(e0, s));
    r = fn();
    if (r != SST_OK) return r;
    SST_CUDA_TRY(cudaEventRecord(e1, s));
    SST_CUDA_TRY(cudaEventSynchronize(e1));
    SST_CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
    return SST_OK;
  };
  const uint32_t cls[3] = {8, 16, 32}, lanes[3] = {4, 8, 16};
  for (uint32_t a = 0; a < 3 && st == SST_OK; a++)
    for (uint32_t b = 0; b < 3 && st == SST_OK; b++) {
      t->chunk_leaves = cls[a];
      t->pr_lanes = lanes[b];
      float ms = 0.f;
      st = timed([&] { return pagerank(g, 3, 0.85, rank); }, &ms);
      if (st == SST_OK && ms < best_pr) {
        best_pr = ms;
        bcl = cls[a];
        blanes = lanes[b];
      }
    }
  t->chunk_leaves = bcl;
  t->pr_lanes = blanes;
  // then the shared-memory cache of the lowest ids (pays on degree-ordered
  // graphs)
  uint32_t bhot = 0;
  const uint32_t hots[5] = {2048, 4096, 8192, 16384, 24576};
  for (uint32_t a = 0; a < 5 && st == SST_OK; a++) {
    t->pr_hot = hots[a];
    float ms = 0.f;
    st = timed([&] { return pagerank(g, 3, 0.85, rank); }, &ms);
    if (st == SST_OK && ms < best_pr) {
      best_pr = ms;
      bhot = hots[a];
    }
  }
  t->pr_hot = bhot;
  // BFS sources: the first three vertices with edges along a fixed stride
  std::vector<uint32_t> deg(n), src;
  if (st == SST_OK) {
    SST_CUDA_TRY(cudaMemcpy(deg.data(), g->d_deg, (uint64_t)n * 4, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < n && src.size() < 3; i++) {
      uint32_t v = (uint32_t)((i * 2654435761ull) % n);
      if (deg[v]) src.push_back(v);
    }
  }
  const uint32_t alphas[5] = {5, 10, 20, 40, 80};
  for (uint32_t a = 0; a < 5 && st == SST_OK && !src.empty(); a++) {
    t->bfs_alpha = alphas[a];
    float tot = 0.f;
    for (uint32_t v : src) {
      float ms = 0.f;
      st = timed([&] { return bfs(g, v, nullptr, dep); }, &ms);
      if (st != SST_OK) break;
      tot += ms;
    }
    if (st == SST_OK && tot < best_bfs) {
      best_bfs = tot;
      balpha = alphas[a];
    }
  }
  t->bfs_alpha = balpha;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(rank);
  cudaFree(dep);
  if (st != SST_OK) return st;
  get_tuning(g, out);
  out->pr_ms = best_pr;
  out->bfs_ms = src.empty() ? 0.f : best_bfs / (float)src.size();
  return SST_OK;
}


// ------------------------------------------------------------- bellman-ford
// Single-source shortest paths over a weighted graph (edge values as
// lengths): the reference drivers' BF(g, src) (internal/test.hpp:611-634;
// the algorithm library itself is absent).  Rounds of push relaxation from
// the vertices whose distance dropped in the previous round: a warp per
// frontier chunk (lane = slot) lowers dist[v] to dist[u] + w(u, v) by
// atomicMin on 64-bit distances, and the first thread to stamp v with the
// round enqueues it.  Lengths are unsigned, so no round count exceeds n.
namespace {
constexpr unsigned long long kInfDist = ~0ull;

__global__ void k_bf_init(unsigned long long *__restrict__ dist,
                          uint32_t *__restrict__ stamp, uint32_t n, uint32_t src) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  dist[v] = v == src ? 0ull : kInfDist;
  stamp[v] = 0;
}

__global__ void __launch_bounds__(kTB, 5)
k_bf_push(DGraph g, const uint32_t *__restrict__ iv,
          const uint32_t *__restrict__ il0, uint32_t nitems,
          unsigned long long *__restrict__ dist,
          uint32_t *__restrict__ stamp, uint32_t round,
          uint32_t *__restrict__ nq,
          unsigned long long *__restrict__ cnt) {
  // next-round vertices staged in shared memory, one queue reservation per
  // block (as in the BFS push)
  __shared__ uint32_t stage[(kTB / 32) * kPushLeaves * 32];
  __shared__ uint32_t s_n;
  __shared__ unsigned long long s_deg, s_items, s_base;
  if (threadIdx.x == 0) {
    s_n = 0;
    s_deg = 0;
    s_items = 0;
  }
  __syncthreads();
  const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i < nitems) {
    const uint32_t u = iv[i];
    const unsigned long long du = __ldcg(dist + u);
    const uint64_t base = g.base[u];
    const uint32_t cap = g.cap[u], deg = g.deg[u];
    const uint32_t nl = cap ? nleaves_of(cap) : 0;
    const uint32_t l0 = il0[i], l1 = min(l0 + kPushLeaves, nl);
    unsigned long long dsum = 0, isum = 0;
    // four leaves' slots, lengths and distances in flight at once; leaves
    // keep their ids packed left with EMPTY after them
    constexpr int kBatch = 4;
    const uint32_t lim = cap <= kLeaf ? deg : kLeaf;
    const uint32_t below = (1u << lane) - 1u;
    for (uint32_t l = l0; l < l1; l += kBatch) {
      uint32_t v[kBatch], len[kBatch];
#pragma unroll
      for (int k = 0; k < kBatch; k++) {
        const uint64_t at = base + ((uint64_t)(l + k) << kLeafLog) + lane;
        const bool in = l + k < l1 && (uint32_t)lane < lim;
        v[k] = in ? g.slots[at] : kEmpty;
        len[k] = in ? g.vals[at] : 0u;
      }
      unsigned long long dv[kBatch];
#pragma unroll
      for (int k = 0; k < kBatch; k++) dv[k] = v[k] != kEmpty ? __ldcg(dist + v[k]) : 0ull;
      uint32_t mine = 0;  // bit k: this lane enqueues v[k]
#pragma unroll
      for (int k = 0; k < kBatch; k++) {
        const unsigned long long nd = du + len[k];
        if (v[k] != kEmpty && nd < dv[k] && atomicMin(dist + v[k], nd) > nd &&
            atomicExch(stamp + v[k], round) != round)
          mine |= 1u << k;
      }
      uint32_t mm[kBatch], total = 0;
#pragma unroll
      for (int k = 0; k < kBatch; k++) {
        mm[k] = l + k < l1 ? __ballot_sync(0xffffffffu, (mine >> k) & 1u) : 0u;
        total += __popc(mm[k]);
      }
      if (total == 0) continue;
      uint32_t at = 0;
      if (lane == 0) at = atomicAdd(&s_n, total);
      at = __shfl_sync(0xffffffffu, at, 0);
#pragma unroll
      for (int k = 0; k < kBatch; k++) {
        if ((mine >> k) & 1u) {
          stage[at + __popc(mm[k] & below)] = v[k];
          dsum += g.deg[v[k]];
          isum += items_of(g.cap[v[k]]);
        }
        at += __popc(mm[k]);
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      dsum += __shfl_xor_sync(0xffffffffu, dsum, d);
      isum += __shfl_xor_sync(0xffffffffu, isum, d);
    }
    if (lane == 0 && (dsum || isum)) {
      atomicAdd(&s_deg, dsum);
      atomicAdd(&s_items, isum);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    s_base = s_n ? atomicAdd(&cnt[0], (unsigned long long)s_n) : 0ull;
    if (s_deg || s_items) {
      atomicAdd(&cnt[1], s_deg);
      atomicAdd(&cnt[2], s_items);
    }
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < s_n; k += blockDim.x) nq[s_base + k] = stage[k];
}

__global__ void k_bf_out(const unsigned long long *__restrict__ dist, uint32_t n,
                         int32_t *__restrict__ out) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const unsigned long long d = dist[v];
  out[v] = d >= 0x7FFFFFFFull ? 0x7FFFFFFF : (int32_t)d;
}
}  // namespace

static uint64_t items_of_host(uint32_t cap) {
  return cap > kLeaf ? ((cap >> kLeafLog) + kPushLeaves - 1) / kPushLeaves : 1;
}

sst_status bellman_ford(sst_graph *g, uint32_t src, int32_t *d_out) {
  if (!g->weighted || !g->d_vals) {
    set_error_message("Bellman-Ford needs a weighted graph (sst_config.weighted)");
    return SST_ESTATE;
  }
  TravState *t = state(g);
  cudaStream_t s = g->stream;
  const uint32_t n = g->n;
  if (n == 0) return SST_OK;
  SST_CUDA_TRY(t->msrc.ensure(n));  // 64-bit distances
  SST_CUDA_TRY(t->qa.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->qb.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->fbits.ensure((uint64_t)n + 1));  // round stamps
  SST_CUDA_TRY(t->icnt.ensure((uint64_t)n + 1));
  SST_CUDA_TRY(t->ioff.ensure((uint64_t)n + 1));
  unsigned long long *dist = t->msrc.p;
  uint32_t *stamp = t->fbits.p;
  SST_LAUNCH(k_bf_init, blocks_for(n), kTB, 0, s, dist, stamp, n, src);
  SST_CUDA_TRY(cudaMemcpyAsync(t->qa.p, &src, 4, cudaMemcpyHostToDevice, s));
  uint32_t scap = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(&scap, g->d_cap + src, 4, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t qn = 1, qitems = items_of_host(scap);
  uint32_t *q = t->qa.p, *nq = t->qb.p;
  unsigned long long *cnt = t->d_small;
  DGraph dg = g->view();
  for (uint32_t round = 1; qn > 0; round++) {
    if (round > n + 1) {
      set_error_message("Bellman-Ford did not settle in n rounds");
      return SST_ETIMEDOUT;
    }
    SST_CUDA_TRY(t->iv.ensure(qitems + 1));
    SST_CUDA_TRY(t->il0.ensure(qitems + 1));
    SST_CUDA_TRY(cudaMemsetAsync(cnt, 0, 24, s));
    SST_LAUNCH(k_front_items, blocks_for(qn), kTB, 0, s, q, (uint32_t)qn,
               g->d_cap, t->icnt.p);
    g->arena.reset();
    SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes(qn, 4) + 4096));
    SST_CUDA_TRY((scan<uint32_t, OpAdd>(t->icnt.p, t->ioff.p, qn, 0u, OpAdd{},
                                        true, false, nullptr, g->arena, s)));
    SST_LAUNCH(k_front_expand, blocks_for(qn), kTB, 0, s, q, (uint32_t)qn,
               g->d_cap, t->ioff.p, t->iv.p, t->il0.p);
    SST_LAUNCH(k_bf_push, warp_blocks(qitems), kTB, 0, s, dg, t->iv.p, t->il0.p,
               (uint32_t)qitems, dist, stamp, round, nq, cnt);
    SST_CUDA_TRY(cudaMemcpyAsync(t->h_small, cnt, 24, cudaMemcpyDeviceToHost, s));
    SST_CUDA_TRY(cudaStreamSynchronize(s));
    qn = t->h_small[0];
    qitems = t->h_small[2];
    std::swap(q, nq);
  }
  SST_LAUNCH(k_bf_out, blocks_for(n), kTB, 0, s, dist, n, d_out);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

}  // namespace sst

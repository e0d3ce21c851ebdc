// Byte-width snapshot of a graph: the device form of the reference's
// byte-width rows (TinySetV_small, TinySet_small.hpp:204-293,852-881).
//
// The reference stores each row as a set whose elements keep only their low
// B bytes (B = 4, 3, 2 or 1, chosen from the row's element count), split
// into buckets by the high part (bucket = e >> 8B, TinySet_small.hpp:852-870);
// the count thresholds come from a memory model over the column count
// (get_thresholds, TinySet_small.hpp:227-293).  The live graph here keeps
// uint32 PMA rows, which the update kernels need; this snapshot is a
// read-only copy in the byte-width layout, for queries that want the
// smaller HBM footprint (serving slots under a budget).
//
// Layout (device):
//   deg[v]  row length;  B and the bucket count nb follow from deg and the
//           column count, so they are not stored;
//   off[v]  byte offset of row v in `bytes`;
//   row v   nb == 1: deg x B bytes, element i at off + i*B, little endian;
//           nb > 1:  at align4(off) a directory of nb + 1 uint32 (element
//           index where each bucket starts; the last entry is deg), then
//           deg x B low bytes.
// A row's size is deg*B, plus 4*(nb+1) + 3 when it has a directory (the 3
// bytes of slack pay for aligning the directory).
//
// Built from the graph's CSR in element-parallel kernels; read by a decode
// to CSR, a batched membership test and a PageRank whose fixed-point
// arithmetic (prfixed.cuh) is the PMA PageRank's, so the ranks are equal
// bit for bit.
#include <algorithm>
#include <cstring>
#include <vector>

#include "ccshared.cuh"
#include "graph.cuh"
#include "prfixed.cuh"
#include "tcshared.cuh"

namespace sst {
namespace {

constexpr int kTB = 256;
// elements per work item of the element-parallel kernels and of the
// PageRank chunks
constexpr uint32_t kElemsPerWarp = 1024;
constexpr uint32_t kSmallRow = 32;  // PageRank rows up to this length: 8 lanes each

inline unsigned blocks_for(uint64_t n, int per = kTB) {
  uint64_t b = (n + per - 1) / per;
  return (unsigned)(b == 0 ? 1 : b);
}
inline unsigned warp_blocks(uint64_t nwarps) { return blocks_for(nwarps * 32); }

// ------------------------------------------------------- width choice
// The reference's per-PMA header size in its memory model
// (sizeof(PMA<sized_uint<4>>), PMA.hpp:170-175); its bucket bit array is
// compiled out (use_bit_array = false, TinySet_small.hpp:54).
constexpr uint64_t kBucketHeaderBytes = 12;

// calc_pma_count (TinySet_small.hpp:216-224): buckets of a b-byte row
__host__ __device__ inline uint64_t bucket_count(uint64_t max_el, uint32_t b) {
  uint64_t c = max_el >> (8 * b);
  if (c < 1) c = 1;
  if ((c << (8 * b)) < max_el) c += 1;
  return c;
}

// find_best_b_for_given_element_count (TinySet_small.hpp:265-293)
uint32_t best_width(uint64_t count, uint64_t max_el) {
  static const uint32_t opts[4] = {4, 3, 2, 1};
  uint32_t best = opts[0];
  uint64_t best_mem = 0;
  for (int i = 0; i < 4; i++) {
    const uint32_t b = opts[i];
    const uint64_t pmas = bucket_count(max_el, b);
    const uint64_t mem = count * b * 2 + (pmas == 1 ? 0 : pmas * kBucketHeaderBytes);
    if (i == 0 || mem < best_mem) {
      best = b;
      best_mem = mem;
    }
  }
  return best;
}

}  // namespace

// get_thresholds (TinySet_small.hpp:227-263): rows with fewer than t[0]
// elements keep 4-byte keys, fewer than t[1] 3-byte, fewer than t[2] 2-byte,
// the rest 1-byte
void compact_widths(uint64_t max_el, uint32_t t[3]) {
  uint32_t t24 = 2, t16 = 0, t8 = 0, cur = 32;
  for (uint32_t c = 2; c < UINT32_MAX / 2; c *= 2) {
    const uint32_t b = best_width(c, max_el);
    if (b < cur) {
      cur = b;
      if (b == 3) t24 = c * 2;
      if (b == 2) t16 = c * 2;
      if (b == 1) t8 = c * 2;
    }
  }
  if (t16 <= t24) t16 = t24 * 2;
  if (t8 <= t16) t8 = t16 * 2;
  t[0] = t24;
  t[1] = t16;
  t[2] = t8;
}

namespace {

struct DCompact {
  uint32_t n, width;
  uint32_t t24, t16, t8;
  const uint64_t *off;
  const uint32_t *deg;
  const uint8_t *bytes;
};

// find_b_for_el_count (TinySet_small.hpp:204-214)
__host__ __device__ inline uint32_t width_of(uint32_t d, uint32_t t24,
                                             uint32_t t16, uint32_t t8) {
  return d < t24 ? 4u : d < t16 ? 3u : d < t8 ? 2u : 1u;
}

struct Row {
  uint32_t d, B, nb;
  const uint32_t *dir;  // nb + 1 entries, or null when nb == 1
  const uint8_t *lows;
};

__device__ __forceinline__ Row row_of(const DCompact &c, uint32_t v) {
  Row r;
  r.d = c.deg[v];
  r.B = width_of(r.d, c.t24, c.t16, c.t8);
  r.nb = (uint32_t)bucket_count(c.width, r.B);
  const uint64_t o = c.off[v];
  if (r.nb > 1) {
    const uint64_t a = (o + 3) & ~uint64_t(3);
    r.dir = reinterpret_cast<const uint32_t *>(c.bytes + a);
    r.lows = c.bytes + a + 4ull * (r.nb + 1);
  } else {
    r.dir = nullptr;
    r.lows = c.bytes + o;
  }
  return r;
}

__device__ __forceinline__ uint32_t low_at(const uint8_t *p, uint32_t B) {
  uint32_t x = p[0];
  if (B > 1) x |= (uint32_t)p[1] << 8;
  if (B > 2) x |= (uint32_t)p[2] << 16;
  if (B > 3) x |= (uint32_t)p[3] << 24;
  return x;
}

// B-byte id at byte p of the array: two aligned word loads and a funnel
// shift (the array carries 16 bytes of tail padding, so the second word is
// always inside it); streamed past L1, first out of L2
__device__ __forceinline__ uint32_t low_fast(const uint8_t *bytes, uint64_t p,
                                             uint32_t B, unsigned long long pol) {
  const uint32_t *w = reinterpret_cast<const uint32_t *>(bytes + (p & ~uint64_t(3)));
  const uint32_t x = __funnelshift_r(ld_stream(w, pol), ld_stream(w + 1, pol),
                                     (uint32_t)(p & 3) * 8);
  return B == 4 ? x : x & ((1u << (8 * B)) - 1u);
}

// bucket of element i: the last b with dir[b] <= i
__device__ __forceinline__ uint32_t bucket_of(const Row &r, uint32_t i) {
  uint32_t lo = 0, hi = r.nb;  // dir[lo] <= i < dir[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (r.dir[mid] <= i)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t elem_at(const Row &r, uint32_t i, uint32_t b) {
  const uint32_t lo = low_at(r.lows + (uint64_t)i * r.B, r.B);
  return r.nb > 1 ? (b << (8 * r.B)) | lo : lo;
}

// last row whose CSR offset is <= i
__device__ __forceinline__ uint32_t row_of_pos(const uint64_t *csr, uint32_t n,
                                               uint64_t i) {
  uint32_t lo = 0, hi = n;  // csr[lo] <= i < csr[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (csr[mid] <= i)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// ------------------------------------------------------------- build
__global__ void k_cg_sizes(const uint64_t *__restrict__ csr, uint32_t n,
                           uint32_t width, uint32_t t24, uint32_t t16, uint32_t t8,
                           uint32_t *__restrict__ deg, uint64_t *__restrict__ size,
                           unsigned long long *__restrict__ per_width) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  const bool ok = v < n;
  uint32_t B = 0;
  if (ok) {
    const uint32_t d = (uint32_t)(csr[v + 1] - csr[v]);
    B = width_of(d, t24, t16, t8);
    const uint64_t nb = bucket_count(width, B);
    deg[v] = d;
    size[v] = (uint64_t)d * B + (nb > 1 ? 4 * (nb + 1) + 3 : 0);
  }
  // rows per width, one atomic per warp and width
#pragma unroll
  for (uint32_t b = 1; b <= 4; b++) {
    const uint32_t k = __popc(__ballot_sync(0xffffffffu, B == b));
    if ((threadIdx.x & 31) == 0 && k) atomicAdd(&per_width[b - 1], (unsigned long long)k);
  }
}

// warp per kElemsPerWarp CSR positions: each element's low bytes
__global__ void k_cg_lows(const uint64_t *__restrict__ csr,
                          const uint32_t *__restrict__ cols, uint64_t m,
                          DCompact c) {
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t p0 = w * kElemsPerWarp;
  if (p0 >= m) return;
  const uint64_t p1 = min(p0 + kElemsPerWarp, m);
  uint32_t v = __shfl_sync(0xffffffffu, lane == 0 ? row_of_pos(csr, c.n, p0) : 0u, 0);
  for (uint64_t i = p0 + lane; i < p1; i += 32) {
    while (csr[v + 1] <= i) v++;
    const Row r = row_of(c, v);
    const uint32_t x = cols[i];
    uint8_t *p = const_cast<uint8_t *>(r.lows) + (i - csr[v]) * r.B;
    p[0] = (uint8_t)x;
    if (r.B > 1) p[1] = (uint8_t)(x >> 8);
    if (r.B > 2) p[2] = (uint8_t)(x >> 16);
    if (r.B > 3) p[3] = (uint8_t)(x >> 24);
  }
}

__global__ void k_cg_dir_rows(const uint32_t *__restrict__ deg, uint32_t n,
                              uint32_t width, uint32_t t24, uint32_t t16,
                              uint32_t t8, uint32_t *__restrict__ list,
                              unsigned int *__restrict__ cnt) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  if (bucket_count(width, width_of(deg[v], t24, t16, t8)) > 1)
    list[atomicAdd(cnt, 1u)] = v;
}

// warp per row with a directory: dir[b] = first element >= b << 8B
__global__ void k_cg_dir(const uint64_t *__restrict__ csr,
                         const uint32_t *__restrict__ cols,
                         const uint32_t *__restrict__ list,
                         const unsigned int *__restrict__ cnt, DCompact c) {
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= *cnt) return;
  const uint32_t v = list[w];
  const Row r = row_of(c, v);
  uint32_t *dir = const_cast<uint32_t *>(r.dir);
  const uint32_t *row = cols + csr[v];
  for (uint32_t b = lane; b <= r.nb; b += 32) {
    uint32_t at = r.d;
    if (b < r.nb) {
      const uint64_t key = (uint64_t)b << (8 * r.B);
      uint32_t lo = 0, hi = r.d;  // first element >= key
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (row[mid] < key)
          lo = mid + 1;
        else
          hi = mid;
      }
      at = lo;
    }
    dir[b] = at;
  }
}

// PageRank work lists: rows of 1..kSmallRow elements in one bucket (a
// descriptor each); chunks of kElemsPerWarp elements of the other rows
__global__ void k_cg_flags(const uint32_t *__restrict__ deg, uint32_t n,
                           uint32_t width, uint32_t t24, uint32_t t16, uint32_t t8,
                           uint32_t *__restrict__ small_f,
                           uint32_t *__restrict__ chunks) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const uint32_t d = deg[v];
  const bool small = d >= 1 && d <= kSmallRow &&
                     bucket_count(width, width_of(d, t24, t16, t8)) == 1;
  small_f[v] = small;
  chunks[v] = (d >= 1 && !small) ? (d + kElemsPerWarp - 1) / kElemsPerWarp : 0;
}

__global__ void k_cg_lists(const uint32_t *__restrict__ deg,
                           const uint64_t *__restrict__ off, uint32_t n,
                           const uint32_t *__restrict__ small_f,
                           const uint32_t *__restrict__ small_pos,
                           const uint32_t *__restrict__ chunks,
                           const uint64_t *__restrict__ chunk_pos,
                           uint32_t *__restrict__ small,
                           unsigned long long *__restrict__ sdesc,
                           uint32_t *__restrict__ cv, uint32_t *__restrict__ c0) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  if (small_f[v]) {
    small[small_pos[v]] = v;
    sdesc[small_pos[v]] = (off[v] << 6) | deg[v];
  }
  const uint32_t k = chunks[v];
  const uint64_t at = chunk_pos[v];
  for (uint32_t j = 0; j < k; j++) {
    cv[at + j] = v;
    c0[at + j] = j * kElemsPerWarp;
  }
}

// ------------------------------------------------------------ queries
__global__ void k_cg_decode(const uint64_t *__restrict__ csr, uint64_t m,
                            DCompact c, uint32_t *__restrict__ cols) {
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t p0 = w * kElemsPerWarp;
  if (p0 >= m) return;
  const uint64_t p1 = min(p0 + kElemsPerWarp, m);
  uint32_t v = __shfl_sync(0xffffffffu, lane == 0 ? row_of_pos(csr, c.n, p0) : 0u, 0);
  for (uint64_t i = p0 + lane; i < p1; i += 32) {
    while (csr[v + 1] <= i) v++;
    const Row r = row_of(c, v);
    const uint32_t e = (uint32_t)(i - csr[v]);
    cols[i] = elem_at(r, e, r.nb > 1 ? bucket_of(r, e) : 0u);
  }
}

__global__ void k_cg_has(DCompact c, const uint32_t *__restrict__ pairs,
                         uint64_t q, uint8_t *__restrict__ out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= q) return;
  const uint32_t u = pairs[2 * i], x = pairs[2 * i + 1];
  uint8_t found = 0;
  if (u < c.n && x < c.width) {
    const Row r = row_of(c, u);
    uint32_t lo = 0, hi = r.d, t = x;
    if (r.nb > 1) {  // the bucket's range; x < width keeps b below nb
      const uint32_t b = x >> (8 * r.B);
      lo = r.dir[b];
      hi = r.dir[b + 1];
      t = x & ((1u << (8 * r.B)) - 1u);
    }
    const uint32_t end = hi;
    while (lo < hi) {  // first low >= t
      const uint32_t mid = (lo + hi) >> 1;
      if (low_at(r.lows + (uint64_t)mid * r.B, r.B) < t)
        lo = mid + 1;
      else
        hi = mid;
    }
    found = lo < end && low_at(r.lows + (uint64_t)lo * r.B, r.B) == t;
  }
  out[i] = found;
}

// ----------------------------------------------------------- pagerank
// as the PMA PageRank's start: an empty row's contribution is zero in both
// buffers, its rank the constant term
__global__ void k_cpr_start(const uint32_t *__restrict__ deg, uint32_t n,
                            unsigned long long r0,
                            unsigned long long *__restrict__ rdeg,
                            unsigned long long *__restrict__ contrib,
                            unsigned long long *__restrict__ contrib2,
                            double *__restrict__ rank, double base) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const uint32_t d = deg[v];
  const unsigned long long rd = pr_rdeg_of(d);
  rdeg[v] = rd;
  contrib[v] = d ? contrib_of(r0, d, rd) : 0ull;
  if (d == 0) {
    contrib2[v] = 0ull;
    rank[v] = base;
  }
}

// rows of up to 32 ids in one bucket: 8 lanes per row, four ids per lane,
// four rows per 8-lane group in flight.  sdesc[i] = (byte offset << 6) | ids.
constexpr int kSmallPer = 4;

__global__ void __launch_bounds__(kTB, 8)
k_cpr_small(DCompact c, const unsigned long long *__restrict__ sdesc,
                            const uint32_t *__restrict__ small, uint64_t nsmall,
                            const unsigned long long *__restrict__ cin,
                            unsigned long long *__restrict__ cout,
                            double *__restrict__ rank,
                            const unsigned long long *__restrict__ rdeg,
                            PrConst k, bool last) {
  const uint64_t grp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const uint32_t sub = threadIdx.x & 7;
  const unsigned long long pol = l2_evict_first();
  const uint64_t i0 = grp * kSmallPer;
  uint32_t x[kSmallPer][4];
  uint32_t dg[kSmallPer];
#pragma unroll
  for (int u = 0; u < kSmallPer; u++) {
    const uint64_t i = i0 + u;
    const unsigned long long dsc = i < nsmall ? sdesc[i] : 0ull;
    dg[u] = (uint32_t)(dsc & 63);
    const uint32_t B = width_of(dg[u], c.t24, c.t16, c.t8);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint32_t j = sub + 8 * q;
      x[u][q] = j < dg[u] ? low_fast(c.bytes, (dsc >> 6) + (uint64_t)j * B, B, pol) : kEmpty;
    }
  }
  unsigned long long acc[kSmallPer];
#pragma unroll
  for (int u = 0; u < kSmallPer; u++) {
    acc[u] = 0;
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (x[u][q] != kEmpty) acc[u] += ld_keep(cin + x[u][q]);
  }
  unsigned long long mine = 0;
  uint32_t mydeg = 0;
#pragma unroll
  for (int u = 0; u < kSmallPer; u++) {
    unsigned long long a = acc[u];
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (sub == (uint32_t)u) {
      mine = a;
      mydeg = dg[u];
    }
  }
  if (sub < (uint32_t)kSmallPer && i0 + sub < nsmall)
    pr_finish(small[i0 + sub], mine, k, mydeg, rdeg, cout, rank, last);
}

// warp per chunk of kElemsPerWarp ids of the other rows (longer ones, or
// with a bucket directory); each lane has eight ids' loads, then their
// eight gathers, in flight.  A row of one chunk finishes here, the others
// leave a partial sum per chunk.
__global__ void __launch_bounds__(kTB, 8)
k_cpr_chunks(DCompact c, const uint32_t *__restrict__ cv,
                             const uint32_t *__restrict__ c0, uint64_t nchunks,
                             const unsigned long long *__restrict__ cin,
                             unsigned long long *__restrict__ cout,
                             double *__restrict__ rank,
                             const unsigned long long *__restrict__ rdeg,
                             unsigned long long *__restrict__ partial,
                             PrConst k, bool last) {
  constexpr int kIn = 8;
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  const unsigned long long pol = l2_evict_first();
  const uint32_t v = cv[w], e0 = c0[w];
  const Row r = row_of(c, v);
  const uint64_t lows = (uint64_t)(r.lows - c.bytes);
  const uint32_t e1 = min(e0 + kElemsPerWarp, r.d);
  unsigned long long acc = 0;
  if (r.nb == 1) {
    for (uint32_t i = e0 + lane; i < e1; i += 32 * kIn) {
      uint32_t x[kIn];
#pragma unroll
      for (int q = 0; q < kIn; q++) {
        const uint32_t e = i + 32 * q;
        x[q] = e < e1 ? low_fast(c.bytes, lows + (uint64_t)e * r.B, r.B, pol) : kEmpty;
      }
#pragma unroll
      for (int q = 0; q < kIn; q++)
        if (x[q] != kEmpty) acc += ld_keep(cin + x[q]);
    }
  } else {
    // a row with a bucket directory: each lane walks the buckets upwards
    uint32_t b = e0 + lane < e1 ? bucket_of(r, e0 + lane) : 0u;
    for (uint32_t i = e0 + lane; i < e1; i += 32) {
      while (r.dir[b + 1] <= i) b++;
      acc += ld_keep(cin + ((b << (8 * r.B)) | low_fast(c.bytes, lows + (uint64_t)i * r.B,
                                                         r.B, pol)));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    if (r.d <= kElemsPerWarp)
      pr_finish(v, acc, k, r.d, rdeg, cout, rank, last);
    else
      partial[w] = acc;
  }
}

// rows of several chunks: the chunks' partial sums (consecutive, from
// first[j]) in chunk order
__global__ void k_cpr_fix(DCompact c, const uint32_t *__restrict__ multi,
                          const uint64_t *__restrict__ first, uint64_t nmulti,
                          const unsigned long long *__restrict__ partial,
                          unsigned long long *__restrict__ cout,
                          double *__restrict__ rank,
                          const unsigned long long *__restrict__ rdeg,
                          PrConst k, bool last) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nmulti) return;
  const uint32_t v = multi[j];
  const uint32_t d = c.deg[v];
  const uint32_t nc = (d + kElemsPerWarp - 1) / kElemsPerWarp;
  unsigned long long s = 0;
  for (uint32_t t = 0; t < nc; t++) s += partial[first[j] + t];
  pr_finish(v, s, k, d, rdeg, cout, rank, last);
}

__global__ void k_cg_multi(const uint32_t *__restrict__ deg, uint32_t n,
                           const uint64_t *__restrict__ chunk_pos,
                           uint32_t *__restrict__ multi, uint64_t *__restrict__ first,
                           unsigned int *__restrict__ cnt) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  if (deg[v] > kElemsPerWarp) {
    const unsigned int j = atomicAdd(cnt, 1u);
    multi[j] = v;
    first[j] = chunk_pos[v];
  }
}

__global__ void k_widen(const uint32_t *__restrict__ in, uint32_t n,
                        uint64_t *__restrict__ out) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v <= n) out[v] = v < n ? in[v] : 0ull;
}

__global__ void k_fill_d(double *__restrict__ out, uint32_t n, double x) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) out[v] = x;
}

// ------------------------------------------------------ traversals
// BFS and CC read the snapshot's rows through the PageRank work lists:
// one-bucket rows of up to kSmallRow ids (a thread each) and chunks of
// kElemsPerWarp ids of the other rows (a warp each).

// id of element i of a one-bucket small row at byte offset o (B bytes)
__device__ __forceinline__ uint32_t small_id(const uint8_t *bytes, uint64_t o,
                                             uint32_t i, uint32_t B) {
  return low_at(bytes + o + (uint64_t)i * B, B);
}

// ---- connected components (Afforest; the shared parts in ccshared.cuh)
// round r: v links to its r-th smallest neighbour
__global__ void k_ccc_sample(DCompact c, uint32_t r, uint32_t *__restrict__ par,
                             unsigned long long *__restrict__ err) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= c.n) return;
  const uint32_t d = c.deg[v];
  if (r >= d) return;
  const Row row = row_of(c, v);
  cc_link(par, v, elem_at(row, r, row.nb > 1 ? bucket_of(row, r) : 0u), err);
}

__global__ void k_ccc_rest_small(DCompact c, const unsigned long long *__restrict__ sdesc,
                                 const uint32_t *__restrict__ small, uint64_t nsmall,
                                 const unsigned long long *__restrict__ giant,
                                 uint32_t *__restrict__ par,
                                 unsigned long long *__restrict__ err) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsmall) return;
  const uint32_t v = small[i];
  if (ld_par(par, v) == (uint32_t)*giant) return;
  const unsigned long long dsc = sdesc[i];
  const uint32_t d = (uint32_t)(dsc & 63);
  const uint32_t B = width_of(d, c.t24, c.t16, c.t8);
  for (uint32_t j = 0; j < d; j++) cc_link(par, v, small_id(c.bytes, dsc >> 6, j, B), err);
}

__global__ void k_ccc_rest_chunks(DCompact c, const uint32_t *__restrict__ cv,
                                  const uint32_t *__restrict__ c0, uint64_t nchunks,
                                  const unsigned long long *__restrict__ giant,
                                  uint32_t *__restrict__ par,
                                  unsigned long long *__restrict__ err) {
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  const uint32_t v = cv[w], e0 = c0[w];
  if (ld_par(par, v) == (uint32_t)*giant) return;
  const Row r = row_of(c, v);
  const uint32_t e1 = min(e0 + kElemsPerWarp, r.d);
  uint32_t b = (r.nb > 1 && e0 + lane < e1) ? bucket_of(r, e0 + lane) : 0u;
  for (uint32_t i = e0 + lane; i < e1; i += 32) {
    if (r.nb > 1)
      while (r.dir[b + 1] <= i) b++;
    cc_link(par, v, elem_at(r, i, b), err);
  }
}

// ---- BFS (depths), push or pull per level as on the PMA graph
__device__ __forceinline__ void cbfs_enqueue(uint32_t w, uint32_t d,
                                             uint32_t *__restrict__ nq,
                                             unsigned long long *__restrict__ cnt) {
  const unsigned long long at = atomicAdd(&cnt[0], 1ull);
  nq[at] = w;
  atomicAdd(&cnt[1], (unsigned long long)d);
  atomicAdd(&cnt[2], (unsigned long long)((d + kElemsPerWarp - 1) / kElemsPerWarp));
}

__device__ __forceinline__ uint32_t cbfs_items(uint32_t d) {
  return (d + kElemsPerWarp - 1) / kElemsPerWarp;
}

// every lane of the warp calls it: the lanes with `want` append w (degree
// d) to the next queue with one set of counter atomics for the warp
__device__ __forceinline__ void cbfs_enqueue_warp(bool want, uint32_t w, uint32_t d,
                                                  uint32_t *__restrict__ nq,
                                                  unsigned long long *__restrict__ cnt) {
  const uint32_t m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const uint32_t dsum = __reduce_add_sync(0xffffffffu, want ? d : 0u);
  const uint32_t isum = __reduce_add_sync(0xffffffffu, want ? cbfs_items(d) : 0u);
  const int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) {
    base = atomicAdd(&cnt[0], (unsigned long long)__popc(m));
    atomicAdd(&cnt[1], (unsigned long long)dsum);
    atomicAdd(&cnt[2], (unsigned long long)isum);
  }
  base = __shfl_sync(0xffffffffu, base, leader);
  if (want) nq[base + __popc(m & ((1u << lane) - 1u))] = w;
}

// every thread of the block calls it: one set of counter atomics a block
__device__ __forceinline__ void cbfs_enqueue_block(bool want, uint32_t w, uint32_t d,
                                                   uint32_t *__restrict__ nq,
                                                   unsigned long long *__restrict__ cnt) {
  __shared__ uint32_t s_cnt[kTB / 32];
  __shared__ unsigned long long s_base, s_deg, s_items;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t m = __ballot_sync(0xffffffffu, want);
  const uint32_t dsum = __reduce_add_sync(0xffffffffu, want ? d : 0u);
  const uint32_t isum = __reduce_add_sync(0xffffffffu, want ? cbfs_items(d) : 0u);
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
    for (int k = 0; k < kTB / 32; k++) {
      const uint32_t c = s_cnt[k];
      s_cnt[k] = tot;
      tot += c;
    }
    s_base = tot ? atomicAdd(&cnt[0], (unsigned long long)tot) : 0ull;
  }
  __syncthreads();
  if (threadIdx.x == 0 && (s_deg || s_items)) {
    atomicAdd(&cnt[1], s_deg);
    atomicAdd(&cnt[2], s_items);
  }
  if (want) nq[s_base + s_cnt[warp] + __popc(m & ((1u << lane) - 1u))] = w;
}

__global__ void k_cbfs_init(int32_t *__restrict__ depth, uint32_t n, uint32_t src) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) depth[v] = v == src ? 0 : -1;
}

__global__ void k_cbfs_bits(const uint32_t *__restrict__ q, uint64_t qn,
                            uint32_t *__restrict__ bits) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < qn) atomicOr(&bits[q[i] >> 5], 1u << (q[i] & 31));
}

__device__ __forceinline__ bool in_front(const uint32_t *bits, uint32_t x) {
  return (__ldg(bits + (x >> 5)) >> (x & 31)) & 1u;
}

// B-byte id at byte p: two aligned words and a funnel shift (the byte
// array carries 16 bytes of tail padding)
__device__ __forceinline__ uint32_t id_words(const uint8_t *bytes, uint64_t p, uint32_t B) {
  const uint32_t *w = reinterpret_cast<const uint32_t *>(bytes + (p & ~uint64_t(3)));
  const uint32_t x = __funnelshift_r(__ldg(w), __ldg(w + 1), (uint32_t)(p & 3) * 8);
  return B == 4 ? x : x & ((1u << (8 * B)) - 1u);
}

// id of element i (bucket b) of a row, by word loads
__device__ __forceinline__ uint32_t elem_words(const DCompact &c, const Row &r, uint32_t i,
                                               uint32_t b) {
  const uint32_t lo = id_words(c.bytes, (uint64_t)(r.lows - c.bytes) + (uint64_t)i * r.B, r.B);
  return r.nb > 1 ? (b << (8 * r.B)) | lo : lo;
}

// pull, small rows: 8 lanes per row (four ids a lane), an unreached vertex
// looks for a neighbour in the frontier
__global__ void k_cbfs_pull_small(DCompact c, const unsigned long long *__restrict__ sdesc,
                                  const uint32_t *__restrict__ small, uint64_t nsmall,
                                  const uint32_t *__restrict__ bits,
                                  int32_t *__restrict__ depth, uint32_t *__restrict__ nq,
                                  unsigned long long *__restrict__ cnt, int32_t lvl) {
  const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const uint32_t sub = threadIdx.x & 7;
  const int lane = threadIdx.x & 31;
  const bool ok = i < nsmall;
  const uint32_t v = ok ? small[i] : 0u;
  bool hit = false;
  uint32_t d = 0;
  if (ok && depth[v] < 0) {
    const unsigned long long dsc = sdesc[i];
    d = (uint32_t)(dsc & 63);
    const uint32_t B = width_of(d, c.t24, c.t16, c.t8);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint32_t j = sub + 8 * q;
      if (j < d) hit |= in_front(bits, id_words(c.bytes, (dsc >> 6) + (uint64_t)j * B, B));
    }
  }
  const uint32_t group = (__ballot_sync(0xffffffffu, hit) >> (lane & ~7)) & 0xffu;
  // a small row is its vertex's only work item: no claim race
  const bool claim = group && sub == 0;
  if (claim) depth[v] = lvl + 1;
  cbfs_enqueue_block(claim, v, d, nq, cnt);
}

// pull, chunks: a warp per chunk, 32 ids a step, until one is in the
// frontier; the chunks of one row claim their vertex with a
// compare-and-swap
__global__ void k_cbfs_pull_chunks(DCompact c, const uint32_t *__restrict__ cv,
                                   const uint32_t *__restrict__ c0, uint64_t nchunks,
                                   const uint32_t *__restrict__ bits,
                                   int32_t *__restrict__ depth, uint32_t *__restrict__ nq,
                                   unsigned long long *__restrict__ cnt, int32_t lvl) {
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  const uint32_t v = cv[w], e0 = c0[w];
  if (__ldcg(depth + v) >= 0) return;
  const Row r = row_of(c, v);
  const uint32_t e1 = min(e0 + kElemsPerWarp, r.d);
  uint32_t b = (r.nb > 1 && e0 + lane < e1) ? bucket_of(r, e0 + lane) : 0u;
  for (uint32_t i0 = e0; i0 < e1; i0 += 32) {
    const uint32_t i = i0 + lane;
    bool hit = false;
    if (i < e1) {
      if (r.nb > 1)
        while (r.dir[b + 1] <= i) b++;
      hit = in_front(bits, elem_words(c, r, i, b));
    }
    if (__any_sync(0xffffffffu, hit)) {
      if (lane == 0 && atomicCAS(depth + v, -1, lvl + 1) == -1) cbfs_enqueue(v, r.d, nq, cnt);
      return;
    }
  }
}

// ---- triangle counting: the decoded rows oriented towards the higher
// (degree, id) rank, then the shared counting kernel (tcshared.cuh)
// warp per row: keep[e] = 1 where the row's e-th id ranks above the row
__global__ void k_ctc_keep(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                           const uint32_t *__restrict__ deg, uint32_t n,
                           uint32_t *__restrict__ keep) {
  const uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (v >= n) return;
  for (uint64_t e = off[v] + lane; e < off[v + 1]; e += 32)
    keep[e] = ranks_above(deg, cols[e], (uint32_t)v) ? 1u : 0u;
}

__global__ void k_ctc_fill(const uint32_t *__restrict__ cols, const uint32_t *__restrict__ keep,
                           const uint32_t *__restrict__ pos, uint64_t m,
                           uint32_t *__restrict__ adj) {
  const uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < m && keep[e]) adj[pos[e]] = cols[e];
}

// a row's oriented list starts where its first kept id lands
__global__ void k_ctc_off(const uint64_t *__restrict__ off, const uint32_t *__restrict__ pos,
                          uint32_t n, uint64_t m, uint64_t *__restrict__ doff) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v <= n) doff[v] = pos[off[v] < m ? off[v] : m];
}

// ---- betweenness (Brandes) over the decoded rows, level by level
__global__ void k_cbc_maxdepth(const int32_t *__restrict__ depth, uint32_t n,
                               unsigned long long *__restrict__ out) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n && depth[v] >= 0) atomicMax(out, (unsigned long long)depth[v]);
}

__global__ void k_cbc_count(const int32_t *__restrict__ depth, uint32_t n,
                            uint32_t *__restrict__ cnt) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n && depth[v] >= 0) atomicAdd(&cnt[depth[v]], 1u);
}

__global__ void k_cbc_scatter(const int32_t *__restrict__ depth, uint32_t n,
                              const uint32_t *__restrict__ off, uint32_t *__restrict__ ctr,
                              uint32_t *__restrict__ list) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n && depth[v] >= 0) list[off[depth[v]] + atomicAdd(&ctr[depth[v]], 1u)] = v;
}

__global__ void k_cbc_init(double *__restrict__ sigma, double *__restrict__ dep, uint32_t n,
                           uint32_t src) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  sigma[v] = v == src ? 1.0 : 0.0;
  dep[v] = 0.0;
}

// warp per vertex w of level d: sigma(w) = sum of sigma over its neighbours
// one level up
__global__ void k_cbc_sigma(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                            const int32_t *__restrict__ depth, const uint32_t *__restrict__ list,
                            uint32_t count, int32_t d, double *__restrict__ sigma) {
  const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= count) return;
  const uint32_t w = list[i];
  double acc = 0.0;
  for (uint64_t e = off[w] + lane; e < off[w + 1]; e += 32) {
    const uint32_t v = cols[e];
    if (depth[v] == d - 1) acc += sigma[v];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) sigma[w] = acc;
}

// warp per vertex v of level d: dep(v) = sum over neighbours w one level
// down of sigma(v) / sigma(w) * (1 + dep(w))
__global__ void k_cbc_dep(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                          const int32_t *__restrict__ depth, const uint32_t *__restrict__ list,
                          uint32_t count, int32_t d, const double *__restrict__ sigma,
                          double *__restrict__ dep) {
  const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= count) return;
  const uint32_t v = list[i];
  const double sv = sigma[v];
  double acc = 0.0;
  for (uint64_t e = off[v] + lane; e < off[v + 1]; e += 32) {
    const uint32_t w = cols[e];
    if (depth[w] == d + 1) acc += sv / sigma[w] * (1.0 + dep[w]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) dep[v] = acc;
}

// push: work items of kElemsPerWarp ids of the frontier's rows
__global__ void k_cbfs_items(const uint32_t *__restrict__ q, uint64_t qn,
                             const uint32_t *__restrict__ deg, uint32_t *__restrict__ k) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < qn) k[i] = (deg[q[i]] + kElemsPerWarp - 1) / kElemsPerWarp;
}

__global__ void k_cbfs_expand(const uint32_t *__restrict__ q, uint64_t qn,
                              const uint32_t *__restrict__ k,
                              const uint32_t *__restrict__ koff,
                              uint32_t *__restrict__ iv, uint32_t *__restrict__ ie0) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= qn) return;
  for (uint32_t j = 0; j < k[i]; j++) {
    iv[koff[i] + j] = q[i];
    ie0[koff[i] + j] = j * kElemsPerWarp;
  }
}

__global__ void k_cbfs_push(DCompact c, const uint32_t *__restrict__ iv,
                            const uint32_t *__restrict__ ie0, uint64_t nitems,
                            int32_t *__restrict__ depth, uint32_t *__restrict__ nq,
                            unsigned long long *__restrict__ cnt, int32_t lvl) {
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nitems) return;
  const uint32_t u = iv[w], e0 = ie0[w];
  const Row r = row_of(c, u);
  const uint32_t e1 = min(e0 + kElemsPerWarp, r.d);
  uint32_t b = (r.nb > 1 && e0 + lane < e1) ? bucket_of(r, e0 + lane) : 0u;
  for (uint32_t i0 = e0; i0 < e1; i0 += 32) {  // warp-uniform steps
    const uint32_t i = i0 + lane;
    bool won = false;
    uint32_t x = 0;
    if (i < e1) {
      if (r.nb > 1)
        while (r.dir[b + 1] <= i) b++;
      x = elem_words(c, r, i, b);
      won = __ldcg(depth + x) < 0 && atomicCAS(depth + x, -1, lvl + 1) == -1;
    }
    cbfs_enqueue_warp(won, x, won ? c.deg[x] : 0u, nq, cnt);
  }
}

}  // namespace
}  // namespace sst

struct sst_compact {
  int device = 0;
  cudaStream_t stream = nullptr;      // where the snapshot's work runs
  cudaStream_t own_stream = nullptr;  // created with it
  uint32_t n = 0, width = 0;
  uint64_t m = 0;
  uint32_t t[3] = {0, 0, 0};
  uint64_t *d_off = nullptr;   // n + 1
  uint32_t *d_deg = nullptr;   // n
  uint8_t *d_bytes = nullptr;  // nbytes
  uint64_t nbytes = 0;
  uint64_t per_width[4] = {0, 0, 0, 0};  // rows stored with 1..4-byte keys
  // PageRank work lists and buffers
  uint32_t *d_small = nullptr;
  unsigned long long *d_sdesc = nullptr;
  uint64_t nsmall = 0;
  uint32_t *d_cv = nullptr, *d_c0 = nullptr;
  uint64_t nchunks = 0;
  uint32_t *d_multi = nullptr;
  uint64_t *d_first = nullptr;
  uint64_t nmulti = 0;
  unsigned long long *d_rdeg = nullptr, *d_ca = nullptr, *d_cb = nullptr,
                     *d_partial = nullptr;
  // traversal buffers (BFS queues, frontier bits, push items; counters)
  uint32_t *d_qa = nullptr, *d_qb = nullptr, *d_bits = nullptr;
  uint32_t *d_ik = nullptr, *d_ikoff = nullptr, *d_iv = nullptr, *d_ie0 = nullptr;
  uint64_t items_cap = 0;
  unsigned long long *d_cnt = nullptr, *h_cnt = nullptr;  // h_cnt pinned
  sst::Arena arena;  // scans and staging

  sst::DCompact view() const {
    return sst::DCompact{n, width, t[0], t[1], t[2], d_off, d_deg, d_bytes};
  }
};

namespace sst {

void compact_release(sst_compact *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (void *p : {(void *)c->d_off, (void *)c->d_deg, (void *)c->d_bytes,
                  (void *)c->d_small, (void *)c->d_sdesc, (void *)c->d_cv, (void *)c->d_c0,
                  (void *)c->d_multi, (void *)c->d_first, (void *)c->d_rdeg,
                  (void *)c->d_ca, (void *)c->d_cb, (void *)c->d_partial,
                  (void *)c->d_qa, (void *)c->d_qb, (void *)c->d_bits, (void *)c->d_ik,
                  (void *)c->d_ikoff, (void *)c->d_iv, (void *)c->d_ie0, (void *)c->d_cnt})
    if (p) cudaFree(p);
  if (c->h_cnt) cudaFreeHost(c->h_cnt);
  c->arena.release();
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  c->stream = c->own_stream = nullptr;
}

sst_status compact_build(sst_graph *g, sst_compact *c) {
  SST_CUDA_TRY(cudaSetDevice(g->device));
  c->device = g->device;
  c->n = g->n;
  c->width = g->width;
  compact_widths(g->width, c->t);
  SST_CUDA_TRY(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
  c->stream = c->own_stream;
  const uint32_t n = g->n;
  // the graph's rows as CSR, on the graph's stream
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  const uint64_t m = g->m;
  c->m = m;
  uint64_t *csr = nullptr;
  uint32_t *cols = nullptr;
  SST_CUDA_TRY(cudaMalloc(&csr, ((uint64_t)n + 1) * 8));
  SST_CUDA_TRY(cudaMalloc(&cols, std::max<uint64_t>(m, 1) * 4));
  sst_status st = to_csr(g, csr, cols, nullptr);
  if (st == SST_OK && cudaStreamSynchronize(g->stream) != cudaSuccess) st = SST_EDEVICE;
  if (st != SST_OK) {
    cudaFree(csr);
    cudaFree(cols);
    return st;
  }
  cudaStream_t s = c->stream;
  auto fail = [&](cudaError_t e, const char *what) {
    cudaFree(csr);
    cudaFree(cols);
    set_cuda_error(e, what, __FILE__, __LINE__);
    return SST_EDEVICE;
  };
#define CG_TRY(expr)                          \
  do {                                        \
    cudaError_t _e = (expr);                  \
    if (_e != cudaSuccess) return fail(_e, #expr); \
  } while (0)
  CG_TRY(cudaMalloc(&c->d_off, ((uint64_t)n + 1) * 8));
  CG_TRY(cudaMalloc(&c->d_deg, std::max<uint32_t>(n, 1) * 4));
  CG_TRY(c->arena.reserve(((uint64_t)n + 1) * 8 * 2 + ((uint64_t)n + 1) * 4 * 4 +
                          4 * scan_scratch_bytes((uint64_t)n + 1, 8) + 4096));
  Arena &A = c->arena;
  A.reset();
  uint64_t *size = A.take<uint64_t>((uint64_t)n + 1);
  unsigned long long *pw = A.take<unsigned long long>(4);
  CG_TRY(cudaMemsetAsync(pw, 0, 32, s));
  CG_TRY(cudaMemsetAsync(size + n, 0, 8, s));
  SST_LAUNCH(k_cg_sizes, blocks_for(n), kTB, 0, s, csr, n, c->width, c->t[0], c->t[1],
             c->t[2], c->d_deg, size, pw);
  CG_TRY((scan<uint64_t, OpAdd>(size, c->d_off, (uint64_t)n + 1, 0ull, OpAdd{}, true,
                                false, nullptr, A, s)));
  unsigned long long h_pw[4];
  CG_TRY(cudaMemcpyAsync(&c->nbytes, c->d_off + n, 8, cudaMemcpyDeviceToHost, s));
  CG_TRY(cudaMemcpyAsync(h_pw, pw, 32, cudaMemcpyDeviceToHost, s));
  CG_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < 4; i++) c->per_width[i] = h_pw[i];
  CG_TRY(cudaMalloc(&c->d_bytes, c->nbytes + 16));
  DCompact dc = c->view();
  if (m)
    SST_LAUNCH(k_cg_lows, warp_blocks((m + kElemsPerWarp - 1) / kElemsPerWarp), kTB, 0, s,
               csr, cols, m, dc);
  uint32_t *dlist = A.take<uint32_t>(std::max<uint32_t>(n, 1));
  unsigned int *dcnt = A.take<unsigned int>(1);
  CG_TRY(cudaMemsetAsync(dcnt, 0, 4, s));
  SST_LAUNCH(k_cg_dir_rows, blocks_for(n), kTB, 0, s, c->d_deg, n, c->width, c->t[0],
             c->t[1], c->t[2], dlist, dcnt);
  uint64_t hubs = 0;  // rows with a directory: their width has several buckets
  for (uint32_t b = 1; b <= 4; b++)
    if (bucket_count(c->width, b) > 1) hubs += c->per_width[b - 1];
  if (hubs)
    SST_LAUNCH(k_cg_dir, warp_blocks(hubs), kTB, 0, s, csr, cols, dlist, dcnt, dc);
  // PageRank work lists
  uint32_t *sf = A.take<uint32_t>((uint64_t)n + 1), *spos = A.take<uint32_t>((uint64_t)n + 1);
  uint32_t *ck = A.take<uint32_t>((uint64_t)n + 1);
  uint64_t *ck64 = A.take<uint64_t>((uint64_t)n + 1), *cpos = A.take<uint64_t>((uint64_t)n + 1);
  if (!sf || !spos || !ck || !ck64 || !cpos) return fail(cudaErrorMemoryAllocation, "scratch");
  SST_LAUNCH(k_cg_flags, blocks_for(n), kTB, 0, s, c->d_deg, n, c->width, c->t[0],
             c->t[1], c->t[2], sf, ck);
  uint32_t *d_ns = A.take<uint32_t>(1);
  uint64_t *d_nc = A.take<uint64_t>(1);
  CG_TRY((scan<uint32_t, OpAdd>(sf, spos, n, 0u, OpAdd{}, true, false, d_ns, A, s)));
  // chunk counts widened to 64 bits for the prefix
  SST_LAUNCH(k_widen, blocks_for((uint64_t)n + 1), kTB, 0, s, ck, n, ck64);
  CG_TRY((scan<uint64_t, OpAdd>(ck64, cpos, n, 0ull, OpAdd{}, true, false, d_nc, A, s)));
  uint32_t h_ns = 0;
  uint64_t h_nc = 0;
  CG_TRY(cudaMemcpyAsync(&h_ns, d_ns, 4, cudaMemcpyDeviceToHost, s));
  CG_TRY(cudaMemcpyAsync(&h_nc, d_nc, 8, cudaMemcpyDeviceToHost, s));
  CG_TRY(cudaStreamSynchronize(s));
  c->nsmall = h_ns;
  c->nchunks = h_nc;
  CG_TRY(cudaMalloc(&c->d_small, std::max<uint64_t>(h_ns, 1) * 4));
  CG_TRY(cudaMalloc(&c->d_sdesc, std::max<uint64_t>(h_ns, 1) * 8));
  CG_TRY(cudaMalloc(&c->d_cv, std::max<uint64_t>(h_nc, 1) * 4));
  CG_TRY(cudaMalloc(&c->d_c0, std::max<uint64_t>(h_nc, 1) * 4));
  SST_LAUNCH(k_cg_lists, blocks_for(n), kTB, 0, s, c->d_deg, c->d_off, n, sf, spos, ck,
             cpos, c->d_small, c->d_sdesc, c->d_cv, c->d_c0);
  CG_TRY(cudaMemsetAsync(dcnt, 0, 4, s));
  CG_TRY(cudaMalloc(&c->d_multi, std::max<uint32_t>(n, 1) * 4));
  CG_TRY(cudaMalloc(&c->d_first, std::max<uint32_t>(n, 1) * 8));
  SST_LAUNCH(k_cg_multi, blocks_for(n), kTB, 0, s, c->d_deg, n, cpos, c->d_multi,
             c->d_first, dcnt);
  unsigned int h_nm = 0;
  CG_TRY(cudaMemcpyAsync(&h_nm, dcnt, 4, cudaMemcpyDeviceToHost, s));
  CG_TRY(cudaStreamSynchronize(s));
  c->nmulti = h_nm;
  CG_TRY(cudaGetLastError());
#undef CG_TRY
  cudaFree(csr);
  cudaFree(cols);
  return SST_OK;
}

// device CSR of the snapshot (offsets n + 1, cols m)
sst_status compact_to_csr(sst_compact *c, uint64_t *d_off, uint32_t *d_cols) {
  SST_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  Arena &A = c->arena;
  SST_CUDA_TRY(A.reserve(((uint64_t)n + 1) * 8 + scan_scratch_bytes((uint64_t)n + 1, 8) + 4096));
  A.reset();
  uint64_t *d64 = A.take<uint64_t>((uint64_t)n + 1);
  SST_LAUNCH(k_widen, blocks_for((uint64_t)n + 1), kTB, 0, s, c->d_deg, n, d64);
  SST_CUDA_TRY((scan<uint64_t, OpAdd>(d64, d_off, (uint64_t)n + 1, 0ull, OpAdd{}, true,
                                      false, nullptr, A, s)));
  if (c->m)
    SST_LAUNCH(k_cg_decode, warp_blocks((c->m + kElemsPerWarp - 1) / kElemsPerWarp), kTB,
               0, s, d_off, c->m, c->view(), d_cols);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status compact_has_batch(sst_compact *c, const uint32_t *d_pairs, uint64_t q,
                             uint8_t *d_out) {
  SST_CUDA_TRY(cudaSetDevice(c->device));
  if (q)
    SST_LAUNCH(k_cg_has, blocks_for(q), kTB, 0, c->stream, c->view(), d_pairs, q, d_out);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status compact_pagerank(sst_compact *c, uint32_t iters, double damping,
                            double *d_rank) {
  SST_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  if (n == 0) return SST_OK;
  if (!c->d_ca) {
    SST_CUDA_TRY(cudaMalloc(&c->d_rdeg, (uint64_t)n * 8));
    SST_CUDA_TRY(cudaMalloc(&c->d_ca, (uint64_t)n * 8));
    SST_CUDA_TRY(cudaMalloc(&c->d_cb, (uint64_t)n * 8));
    SST_CUDA_TRY(cudaMalloc(&c->d_partial, std::max<uint64_t>(c->nchunks, 1) * 8));
  }
  const double r0 = 1.0 / (double)n;
  const double base = (1.0 - damping) / (double)n;
  if (iters == 0) {
    SST_LAUNCH(k_fill_d, blocks_for(n), kTB, 0, s, d_rank, n, r0);
    SST_CUDA_TRY(cudaGetLastError());
    return SST_OK;
  }
  unsigned long long r0f = 0;
  const PrConst K = pr_const(n, damping, &r0f);
  unsigned long long *ci = c->d_ca, *co = c->d_cb;
  SST_LAUNCH(k_cpr_start, blocks_for(n), kTB, 0, s, c->d_deg, n, r0f, c->d_rdeg, ci, co,
             d_rank, base);
  const DCompact dc = c->view();
  for (uint32_t it = 0; it < iters; it++) {
    const bool last = it + 1 == iters;
    if (c->nsmall)
      SST_LAUNCH(k_cpr_small,
                 blocks_for((c->nsmall + kSmallPer - 1) / kSmallPer * 8), kTB, 0, s, dc,
                 c->d_sdesc, c->d_small, c->nsmall, ci, co, d_rank, c->d_rdeg, K, last);
    if (c->nchunks)
      SST_LAUNCH(k_cpr_chunks, warp_blocks(c->nchunks), kTB, 0, s, dc, c->d_cv, c->d_c0,
                 c->nchunks, ci, co, d_rank, c->d_rdeg, c->d_partial, K, last);
    if (c->nmulti)
      SST_LAUNCH(k_cpr_fix, blocks_for(c->nmulti), kTB, 0, s, dc, c->d_multi, c->d_first,
                 c->nmulti, c->d_partial, co, d_rank, c->d_rdeg, K, last);
    std::swap(ci, co);
  }
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

static sst_status compact_trav_buffers(sst_compact *c) {
  if (c->d_cnt) return SST_OK;
  const uint64_t n = std::max<uint32_t>(c->n, 1);
  SST_CUDA_TRY(cudaMalloc(&c->d_cnt, 8 * sizeof(unsigned long long)));
  SST_CUDA_TRY(cudaMallocHost(&c->h_cnt, 8 * sizeof(unsigned long long)));
  SST_CUDA_TRY(cudaMalloc(&c->d_qa, n * 4));
  SST_CUDA_TRY(cudaMalloc(&c->d_qb, n * 4));
  SST_CUDA_TRY(cudaMalloc(&c->d_bits, (n / 32 + 2) * 4));
  SST_CUDA_TRY(cudaMalloc(&c->d_ik, (n + 1) * 4));
  SST_CUDA_TRY(cudaMalloc(&c->d_ikoff, (n + 1) * 4));
  return SST_OK;
}

// BFS(g, src) on the snapshot: depths, -1 unreached (the same pull / push
// switch as on the PMA graph: pull once (frontier + its edges) * 20 > m)
sst_status compact_bfs(sst_compact *c, uint32_t src, int32_t *d_depth) {
  SST_CUDA_TRY(cudaSetDevice(c->device));
  sst_status st = compact_trav_buffers(c);
  if (st != SST_OK) return st;
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  const DCompact dc = c->view();
  SST_LAUNCH(k_cbfs_init, blocks_for(n), kTB, 0, s, d_depth, n, src);
  uint32_t d0 = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(c->d_qa, &src, 4, cudaMemcpyHostToDevice, s));
  SST_CUDA_TRY(cudaMemcpyAsync(&d0, c->d_deg + src, 4, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t qn = 1, qdeg = d0, qitems = (d0 + kElemsPerWarp - 1) / kElemsPerWarp;
  uint32_t *q = c->d_qa, *nq = c->d_qb;
  const uint64_t m = c->m;
  Arena &A = c->arena;
  SST_CUDA_TRY(A.reserve(scan_scratch_bytes((uint64_t)n + 1, 4) + 4096));
  for (int32_t lvl = 0; qn > 0; lvl++) {
    if ((uint64_t)lvl > n) {
      set_error_message("BFS exceeded n levels");
      return SST_ETIMEDOUT;
    }
    SST_CUDA_TRY(cudaMemsetAsync(c->d_cnt, 0, 24, s));
    if ((qn + qdeg) * 20 > m) {
      SST_CUDA_TRY(cudaMemsetAsync(c->d_bits, 0, ((uint64_t)n / 32 + 1) * 4, s));
      SST_LAUNCH(k_cbfs_bits, blocks_for(qn), kTB, 0, s, q, qn, c->d_bits);
      if (c->nsmall)
        SST_LAUNCH(k_cbfs_pull_small, blocks_for(c->nsmall * 8), kTB, 0, s, dc, c->d_sdesc,
                   c->d_small, c->nsmall, c->d_bits, d_depth, nq, c->d_cnt, lvl);
      if (c->nchunks)
        SST_LAUNCH(k_cbfs_pull_chunks, warp_blocks(c->nchunks), kTB, 0, s, dc, c->d_cv,
                   c->d_c0, c->nchunks, c->d_bits, d_depth, nq, c->d_cnt, lvl);
    } else if (qitems) {
      if (qitems > c->items_cap) {
        cudaFree(c->d_iv);
        cudaFree(c->d_ie0);
        c->d_iv = c->d_ie0 = nullptr;
        c->items_cap = 0;
        const uint64_t want = qitems + qitems / 4 + 64;
        SST_CUDA_TRY(cudaMalloc(&c->d_iv, want * 4));
        SST_CUDA_TRY(cudaMalloc(&c->d_ie0, want * 4));
        c->items_cap = want;
      }
      SST_LAUNCH(k_cbfs_items, blocks_for(qn), kTB, 0, s, q, qn, c->d_deg, c->d_ik);
      A.reset();
      SST_CUDA_TRY((scan<uint32_t, OpAdd>(c->d_ik, c->d_ikoff, qn, 0u, OpAdd{}, true,
                                          false, nullptr, A, s)));
      SST_LAUNCH(k_cbfs_expand, blocks_for(qn), kTB, 0, s, q, qn, c->d_ik, c->d_ikoff,
                 c->d_iv, c->d_ie0);
      SST_LAUNCH(k_cbfs_push, warp_blocks(qitems), kTB, 0, s, dc, c->d_iv, c->d_ie0, qitems,
                 d_depth, nq, c->d_cnt, lvl);
    }
    SST_CUDA_TRY(cudaMemcpyAsync(c->h_cnt, c->d_cnt, 24, cudaMemcpyDeviceToHost, s));
    SST_CUDA_TRY(cudaStreamSynchronize(s));
    qn = c->h_cnt[0];
    qdeg = c->h_cnt[1];
    qitems = c->h_cnt[2];
    std::swap(q, nq);
  }
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

// TC(g) on the snapshot: triangles (each once); d_pv (may be null) gets
// the triangles containing each vertex
sst_status compact_tc(sst_compact *c, uint64_t *total, uint64_t *d_pv, int sms) {
  SST_CUDA_TRY(cudaSetDevice(c->device));
  sst_status st = compact_trav_buffers(c);
  if (st != SST_OK) return st;
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  const uint64_t m = c->m;
  *total = 0;
  if (d_pv) SST_CUDA_TRY(cudaMemsetAsync(d_pv, 0, (uint64_t)n * 8, s));
  if (n == 0 || m == 0) return SST_OK;
  if (m >= (1ull << 32)) {
    set_error_message("sst_compact_tc: more than 2^32 stored edges");
    return SST_EINVAL;
  }
  uint64_t *off = nullptr, *doff = nullptr;
  uint32_t *cols = nullptr, *keep = nullptr, *pos = nullptr, *adj = nullptr;
  uint32_t *icnt = nullptr, *ioff = nullptr;
  uint64_t *items = nullptr;
  cudaError_t e = cudaMalloc(&off, ((uint64_t)n + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&doff, ((uint64_t)n + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&cols, m * 4);
  if (e == cudaSuccess) e = cudaMalloc(&keep, m * 4);
  if (e == cudaSuccess) e = cudaMalloc(&pos, (m + 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&adj, m * 4);
  if (e == cudaSuccess) e = cudaMalloc(&icnt, ((uint64_t)n + 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&ioff, ((uint64_t)n + 1) * 4);
  // m bounds the oriented entries
  if (e == cudaSuccess) e = cudaMalloc(&items, tc_items_bound(n, m) * 8);
  if (e == cudaSuccess) {
    st = compact_to_csr(c, off, cols);
    if (st == SST_OK) {
      Arena &A = c->arena;
      e = A.reserve(std::max(scan_scratch_bytes(m, 4), scan_scratch_bytes((uint64_t)n + 1, 4)) +
                    4096);
      if (e == cudaSuccess) {
        A.reset();
        const DCompact dc = c->view();
        SST_LAUNCH(k_ctc_keep, warp_blocks(n), kTB, 0, s, off, cols, dc.deg, n, keep);
        e = scan<uint32_t, OpAdd>(keep, pos, m, 0u, OpAdd{}, true, false, pos + m, A, s);
        if (e == cudaSuccess) {
          SST_LAUNCH(k_ctc_fill, blocks_for(m), kTB, 0, s, cols, keep, pos, m, adj);
          SST_LAUNCH(k_ctc_off, blocks_for((uint64_t)n + 1), kTB, 0, s, off, pos, n, m, doff);
          e = cudaMemsetAsync(c->d_cnt, 0, 16, s);  // count, work cursor
          A.reset();
          if (e == cudaSuccess)
            e = tc_count_launch(doff, adj, n, m, TcScratch{icnt, ioff, items}, A, c->d_cnt,
                                reinterpret_cast<unsigned long long *>(d_pv), sms, s);
          if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->h_cnt, c->d_cnt, 8, cudaMemcpyDeviceToHost, s);
          if (e == cudaSuccess) e = cudaStreamSynchronize(s);
          if (e == cudaSuccess) *total = c->h_cnt[0];
        }
      }
    }
  }
  for (void *p : {(void *)off, (void *)doff, (void *)cols, (void *)keep, (void *)pos,
                  (void *)adj, (void *)icnt, (void *)ioff, (void *)items})
    if (p) cudaFree(p);
  if (st != SST_OK) return st;
  SST_CUDA_TRY(e);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

// BC(g, src) on the snapshot: single-source dependencies (Brandes), FP64
sst_status compact_bc(sst_compact *c, uint32_t src, double *d_dep) {
  SST_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  const uint64_t m = c->m;
  int32_t *depth = nullptr;
  uint64_t *off = nullptr;
  uint32_t *cols = nullptr, *list = nullptr, *lv = nullptr;
  double *sigma = nullptr;
  cudaError_t e = cudaMalloc(&depth, (uint64_t)n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&off, ((uint64_t)n + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&cols, std::max<uint64_t>(m, 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&list, (uint64_t)n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&sigma, (uint64_t)n * 8);
  sst_status st = SST_OK;
  std::vector<uint32_t> ho;
  if (e == cudaSuccess) st = compact_bfs(c, src, depth);
  if (e == cudaSuccess && st == SST_OK) st = compact_to_csr(c, off, cols);
  if (e == cudaSuccess && st == SST_OK) {
    SST_LAUNCH(k_cbc_init, blocks_for(n), kTB, 0, s, sigma, d_dep, n, src);
    e = cudaMemsetAsync(c->d_cnt, 0, 8, s);
    if (e == cudaSuccess)
      SST_LAUNCH(k_cbc_maxdepth, blocks_for(n), kTB, 0, s, depth, n, c->d_cnt);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_cnt, c->d_cnt, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    const uint32_t D = (uint32_t)c->h_cnt[0];
    // level counts, offsets and cursors
    if (e == cudaSuccess) e = cudaMalloc(&lv, 3 * ((uint64_t)D + 2) * 4);
    uint32_t *cnt = lv, *loff = lv + D + 2, *ctr = loff + D + 2;
    if (e == cudaSuccess) e = cudaMemsetAsync(lv, 0, 3 * ((uint64_t)D + 2) * 4, s);
    if (e == cudaSuccess) SST_LAUNCH(k_cbc_count, blocks_for(n), kTB, 0, s, depth, n, cnt);
    std::vector<uint32_t> hc(D + 2);
    ho.assign(D + 2, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), cnt, (D + 1) * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    uint32_t acc = 0;
    for (uint32_t d = 0; d <= D; d++) {
      ho[d] = acc;
      acc += hc[d];
    }
    ho[D + 1] = acc;
    if (e == cudaSuccess) e = cudaMemcpyAsync(loff, ho.data(), (D + 2) * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      SST_LAUNCH(k_cbc_scatter, blocks_for(n), kTB, 0, s, depth, n, loff, ctr, list);
    for (uint32_t d = 1; e == cudaSuccess && d <= D; d++) {
      const uint32_t k = ho[d + 1] - ho[d];
      if (k) SST_LAUNCH(k_cbc_sigma, warp_blocks(k), kTB, 0, s, off, cols, depth, list + ho[d],
                        k, (int32_t)d, sigma);
    }
    for (int64_t d = D; e == cudaSuccess && d >= 0; d--) {
      const uint32_t k = ho[d + 1] - ho[d];
      if (k) SST_LAUNCH(k_cbc_dep, warp_blocks(k), kTB, 0, s, off, cols, depth, list + ho[d],
                        k, (int32_t)d, sigma, d_dep);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  for (void *p : {(void *)depth, (void *)off, (void *)cols, (void *)list, (void *)lv,
                  (void *)sigma})
    if (p) cudaFree(p);
  if (st != SST_OK) return st;
  SST_CUDA_TRY(e);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

// CC(g) on the snapshot: label = the component's smallest vertex id
sst_status compact_cc(sst_compact *c, uint32_t *d_labels) {
  SST_CUDA_TRY(cudaSetDevice(c->device));
  sst_status st = compact_trav_buffers(c);
  if (st != SST_OK) return st;
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  if (n == 0) return SST_OK;
  const DCompact dc = c->view();
  unsigned long long *giant = c->d_cnt, *err = c->d_cnt + 1;
  SST_CUDA_TRY(cudaMemsetAsync(c->d_cnt, 0, 16, s));
  SST_LAUNCH(k_iota, blocks_for(n), kTB, 0, s, d_labels, n);
  for (uint32_t r = 0; r < 2; r++) {
    SST_LAUNCH(k_ccc_sample, blocks_for(n), kTB, 0, s, dc, r, d_labels, err);
    SST_LAUNCH(k_cc_compress, blocks_for(n), kTB, 0, s, d_labels, n);
  }
  SST_LAUNCH(k_cc_giant, 1, 1024, 0, s, d_labels, n, giant);
  if (c->nsmall)
    SST_LAUNCH(k_ccc_rest_small, blocks_for(c->nsmall), kTB, 0, s, dc, c->d_sdesc,
               c->d_small, c->nsmall, giant, d_labels, err);
  if (c->nchunks)
    SST_LAUNCH(k_ccc_rest_chunks, warp_blocks(c->nchunks), kTB, 0, s, dc, c->d_cv, c->d_c0,
               c->nchunks, giant, d_labels, err);
  SST_LAUNCH(k_cc_compress, blocks_for(n), kTB, 0, s, d_labels, n);
  SST_CUDA_TRY(cudaMemcpyAsync(c->h_cnt, c->d_cnt, 16, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  SST_CUDA_TRY(cudaGetLastError());
  if (c->h_cnt[1]) {
    set_error_message("connected components: %llu links gave up",
                      (unsigned long long)c->h_cnt[1]);
    return SST_ETIMEDOUT;
  }
  return SST_OK;
}

// device bytes the snapshot holds: its rows and index, and (after a
// PageRank, BFS or CC) the work lists and iteration buffers
void compact_bytes(const sst_compact *c, uint64_t *storage, uint64_t *total) {
  const uint64_t n = c->n;
  *storage = (n + 1) * 8 + n * 4 + c->nbytes;
  uint64_t t = *storage + c->nsmall * 12 + c->nchunks * 8 + n * 12 + c->arena.cap;
  if (c->d_ca) t += n * 24 + std::max<uint64_t>(c->nchunks, 1) * 8;
  if (c->d_cnt) t += n * 16 + n / 8 + c->items_cap * 8 + 64;  // BFS / CC buffers
  *total = t;
}

}  // namespace sst

// ---------------------------------------------------------------- C ABI
namespace {

sst_status compact_dev_check(sst_compact *c) {
  if (!c) {
    sst::set_error_message("null snapshot handle");
    return SST_EINVAL;
  }
  return SST_OK;
}

// traversal output of n entries of T: written on the device directly, or
// through a temporary for a host pointer
template <typename T, typename Fn>
sst_status compact_out(sst_compact *c, T *out, uint32_t flags, const char *what,
                              Fn run) {
  sst_status st = compact_dev_check(c);
  if (st != SST_OK) return st;
  if (!out) return SST_EINVAL;
  if (c->n != c->width) {  // column ids index per-row arrays
    sst::set_error_message("%s needs as many rows as columns (%u x %u)", what, c->n,
                           c->width);
    return SST_EINVAL;
  }
  SST_CUDA_TRY(cudaSetDevice(c->device));
  if (flags & SST_DEVICE_PTR) {
    st = run(out);
    if (st == SST_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) st = SST_EDEVICE;
    return st;
  }
  T *d = nullptr;
  SST_CUDA_TRY(cudaMalloc(&d, std::max<uint64_t>(c->n, 1) * sizeof(T)));
  st = run(d);
  if (st == SST_OK) {
    cudaMemcpyAsync(out, d, (uint64_t)c->n * sizeof(T), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) st = SST_EDEVICE;
  }
  cudaFree(d);
  return st;
}


}  // namespace

extern "C" {

sst_status sst_compact_widths(uint64_t max_el, uint32_t thresholds[3]) {
  if (!thresholds) return SST_EINVAL;
  sst::compact_widths(max_el, thresholds);
  return SST_OK;
}

sst_status sst_compact_create(sst_graph *g, sst_compact **out) {
  if (!g || !out) {
    sst::set_error_message("null graph or output handle");
    return SST_EINVAL;
  }
  if (g->weighted) {
    sst::set_error_message("byte-width snapshots hold ids only: the graph is weighted");
    return SST_ESTATE;
  }
  *out = nullptr;
  sst_compact *c = new sst_compact();
  sst_status st = sst::compact_build(g, c);
  if (st != SST_OK) {
    sst::compact_release(c);
    delete c;
    return st;
  }
  *out = c;
  return SST_OK;
}

sst_status sst_compact_destroy(sst_compact *c) {
  if (!c) return SST_OK;
  sst::compact_release(c);
  delete c;
  return SST_OK;
}

sst_status sst_compact_info(sst_compact *c, uint64_t *storage_bytes,
                            uint64_t *device_bytes, uint64_t *edges,
                            uint64_t rows_per_width[4]) {
  sst_status st = compact_dev_check(c);
  if (st != SST_OK) return st;
  uint64_t sb = 0, tb = 0;
  sst::compact_bytes(c, &sb, &tb);
  if (storage_bytes) *storage_bytes = sb;
  if (device_bytes) *device_bytes = tb;
  if (edges) *edges = c->m;
  if (rows_per_width)
    for (int i = 0; i < 4; i++) rows_per_width[i] = c->per_width[i];
  return SST_OK;
}

sst_status sst_compact_to_csr(sst_compact *c, uint64_t *offsets, uint32_t *cols,
                              uint32_t flags) {
  sst_status st = compact_dev_check(c);
  if (st != SST_OK) return st;
  if (!offsets || (c->m && !cols)) return SST_EINVAL;
  SST_CUDA_TRY(cudaSetDevice(c->device));
  if (flags & SST_DEVICE_PTR) {
    st = sst::compact_to_csr(c, offsets, cols);
    if (st == SST_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) st = SST_EDEVICE;
    return st;
  }
  uint64_t *doff = nullptr;
  uint32_t *dcols = nullptr;
  SST_CUDA_TRY(cudaMalloc(&doff, ((uint64_t)c->n + 1) * 8));
  if (cudaMalloc(&dcols, std::max<uint64_t>(c->m, 1) * 4) != cudaSuccess) {
    cudaFree(doff);
    sst::set_error_message("device allocation for the CSR copy failed");
    return SST_ENOMEM;
  }
  st = sst::compact_to_csr(c, doff, dcols);
  if (st == SST_OK) {
    cudaMemcpyAsync(offsets, doff, ((uint64_t)c->n + 1) * 8, cudaMemcpyDeviceToHost, c->stream);
    if (c->m) cudaMemcpyAsync(cols, dcols, c->m * 4, cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) st = SST_EDEVICE;
  }
  cudaFree(doff);
  cudaFree(dcols);
  return st;
}

sst_status sst_compact_has_batch(sst_compact *c, const uint32_t *pairs, uint64_t n,
                                 uint8_t *out, uint32_t flags) {
  sst_status st = compact_dev_check(c);
  if (st != SST_OK) return st;
  if (n && (!pairs || !out)) return SST_EINVAL;
  if (n == 0) return SST_OK;
  SST_CUDA_TRY(cudaSetDevice(c->device));
  if (flags & SST_DEVICE_PTR) {
    st = sst::compact_has_batch(c, pairs, n, out);
    if (st == SST_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) st = SST_EDEVICE;
    return st;
  }
  uint32_t *dp = nullptr;
  uint8_t *dout = nullptr;
  SST_CUDA_TRY(cudaMalloc(&dp, n * 8));
  if (cudaMalloc(&dout, n) != cudaSuccess) {
    cudaFree(dp);
    sst::set_error_message("device allocation for the query batch failed");
    return SST_ENOMEM;
  }
  cudaMemcpyAsync(dp, pairs, n * 8, cudaMemcpyHostToDevice, c->stream);
  st = sst::compact_has_batch(c, dp, n, dout);
  if (st == SST_OK) {
    cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) st = SST_EDEVICE;
  }
  cudaFree(dp);
  cudaFree(dout);
  return st;
}

sst_status sst_compact_pagerank(sst_compact *c, uint32_t iters, double damping,
                                double *out, uint32_t flags) {
  sst_status st = compact_dev_check(c);
  if (st != SST_OK) return st;
  if (!out) return SST_EINVAL;
  if (c->n != c->width) {  // column ids index per-row vectors
    sst::set_error_message("sst_compact_pagerank needs as many rows as columns (%u x %u)",
                           c->n, c->width);
    return SST_EINVAL;
  }
  SST_CUDA_TRY(cudaSetDevice(c->device));
  if (flags & SST_DEVICE_PTR) {
    st = sst::compact_pagerank(c, iters, damping, out);
    if (st == SST_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) st = SST_EDEVICE;
    return st;
  }
  double *d = nullptr;
  SST_CUDA_TRY(cudaMalloc(&d, std::max<uint64_t>(c->n, 1) * 8));
  st = sst::compact_pagerank(c, iters, damping, d);
  if (st == SST_OK) {
    cudaMemcpyAsync(out, d, (uint64_t)c->n * 8, cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) st = SST_EDEVICE;
  }
  cudaFree(d);
  return st;
}

sst_status sst_compact_bfs(sst_compact *c, uint32_t src, int32_t *depths, uint32_t flags) {
  if (c && src >= c->n) {
    sst::set_error_message("source out of range");
    return SST_EINVAL;
  }
  return compact_out(c, depths, flags, "sst_compact_bfs",
                     [&](int32_t *d) { return sst::compact_bfs(c, src, d); });
}

sst_status sst_compact_tc(sst_compact *c, uint64_t *total, uint64_t *per_vertex,
                          uint32_t flags) {
  if (!total) return SST_EINVAL;
  if (!per_vertex) {
    sst_status st = compact_dev_check(c);
    if (st != SST_OK) return st;
    if (c->n != c->width) {
      sst::set_error_message("sst_compact_tc needs as many rows as columns (%u x %u)", c->n,
                             c->width);
      return SST_EINVAL;
    }
    int sms = 0;
    SST_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    return sst::compact_tc(c, total, nullptr, sms);
  }
  return compact_out(c, per_vertex, flags, "sst_compact_tc", [&](uint64_t *d) {
    int sms = 0;
    SST_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    return sst::compact_tc(c, total, d, sms);
  });
}

sst_status sst_compact_bc(sst_compact *c, uint32_t src, double *out, uint32_t flags) {
  if (c && src >= c->n) {
    sst::set_error_message("source out of range");
    return SST_EINVAL;
  }
  return compact_out(c, out, flags, "sst_compact_bc",
                     [&](double *d) { return sst::compact_bc(c, src, d); });
}

sst_status sst_compact_cc(sst_compact *c, uint32_t *labels, uint32_t flags) {
  return compact_out(c, labels, flags, "sst_compact_cc",
                     [&](uint32_t *d) { return sst::compact_cc(c, d); });
}

sst_status sst_compact_set_stream(sst_compact *c, void *stream) {
  sst_status st = compact_dev_check(c);
  if (st != SST_OK) return st;
  SST_CUDA_TRY(cudaSetDevice(c->device));
  SST_CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  return SST_OK;
}

sst_status sst_compact_sync(sst_compact *c) {
  sst_status st = compact_dev_check(c);
  if (st != SST_OK) return st;
  SST_CUDA_TRY(cudaSetDevice(c->device));
  SST_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SST_OK;
}

}  // extern "C"

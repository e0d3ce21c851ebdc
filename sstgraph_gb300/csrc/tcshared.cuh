// Triangle counting over an oriented adjacency (each edge kept once, at its
// lower-ranked end), shared by the PMA graph (traverse.cu) and the
// byte-width snapshot (compact.cu), which build the orientation each from
// their own rows.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "primitives.cuh"

namespace sst {
namespace {

// rank order used to orient each undirected edge once: (degree, id).  Each
// vertex keeps the neighbours that rank above it (N+), so a hub keeps only
// the few neighbours of even higher degree and the lists stay short; every
// triangle is counted once, at its lowest-ranked vertex.
__device__ __forceinline__ bool rank_less(const uint32_t *deg, uint32_t a,
                                          uint32_t b) {
  uint32_t da = deg[a], db = deg[b];
  return da < db || (da == db && a < b);
}
__device__ __forceinline__ bool ranks_above(const uint32_t *deg, uint32_t w,
                                            uint32_t u) {
  return rank_less(deg, u, w);
}

__device__ __forceinline__ bool sorted_has(const uint32_t *a, uint64_t n,
                                           uint32_t x) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (a[mid] < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < n && a[lo] == x;
}

// The count runs over work items (u, j): the j-th batch of 32 entries of
// N+(u), for every u with |N+(u)| >= 2 (a triangle needs two neighbours
// above u).  A warp takes kTcGrab consecutive items at a time from a
// global cursor, so the serial work a warp can be left with at the end is a
// few items', whatever the degree distribution.  For an item the warp puts
// N+(u) into a hash set in its shared memory (kept while the next item has
// the same u), then reads the lists N+(v) of the item's 32 v as one
// flattened stream: lane i holds v_i's list bounds and the warp's inclusive
// prefix P of their lengths; stream item k lies in the first list i with
// P_i > k, which each lane tracks with a cursor that only moves forward
// (every lane's k grows by 32 a step); each lane issues kTcAhead loads
// before it probes the set, so a warp keeps kTcAhead * 32 list entries in
// flight.  A list N+(u) too long for the set is probed by binary search in
// global memory instead.
constexpr uint32_t kTcSlots = 2048;  // set slots per warp (8 KiB)
constexpr int kTcBucketBits = 9;     // up to 2^9 buckets of 4 slots
constexpr uint32_t kTcBatch = 32;    // v per work item
constexpr int kTcWarps = 8;          // warps per block
constexpr int kTcAhead = 4;          // stream items per lane in flight

// multiplicative hashing (Knuth): the top `bits` bits of x * 2^32/phi
__device__ __forceinline__ uint32_t tc_hash(uint32_t x, int bits) {
  return (x * 0x9E3779B1u) >> (32 - bits);
}

// The set: 2^bits buckets of four slots, one 16-byte shared load each.  An
// insert takes the first empty slot of its bucket (slots fill in order, so
// a bucket whose last slot is empty was never passed over), else moves on
// to the next bucket; a lookup stops at a match or at such a bucket.  At
// most half the slots are ever used, so every probe sequence ends.
__device__ __forceinline__ void tc_set_insert(uint4 *tab, uint32_t x, int bits) {
  uint32_t h = tc_hash(x, bits);
  const uint32_t mask = (1u << bits) - 1;
  for (;;) {
    uint32_t *b = reinterpret_cast<uint32_t *>(tab + h);
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (atomicCAS(b + j, kEmpty, x) == kEmpty) return;
    h = (h + 1) & mask;
  }
}

// One lookup per lane, warp-uniform: every lane reads its home bucket; the
// warp loops on only while some lane met a full bucket without its match
// (rare: the set keeps at least two buckets per entry where it can), so the
// probes do not diverge.  Lanes with on = false look nothing up.
__device__ __forceinline__ bool tc_set_has_warp(const uint4 *tab, uint32_t w, int bits,
                                                bool on) {
  const uint32_t mask = (1u << bits) - 1;
  uint32_t h = tc_hash(w, bits);
  uint4 b = on ? tab[h] : make_uint4(0, 0, 0, kEmpty);
  bool hit = on && (b.x == w || b.y == w || b.z == w || b.w == w);
  bool more = on && !hit && b.w != kEmpty;
  while (__any_sync(0xffffffffu, more)) {
    if (more) {
      h = (h + 1) & mask;
      b = tab[h];
      hit = b.x == w || b.y == w || b.z == w || b.w == w;
      more = !hit && b.w != kEmpty;
    }
  }
  return hit;
}

// per u: its number of work items
__global__ void k_tc_items_count(const uint64_t *__restrict__ off, uint32_t n,
                                 uint32_t *__restrict__ cnt) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n) return;
  const uint64_t na = off[u + 1] - off[u];
  cnt[u] = na < 2 ? 0u : (uint32_t)((na + kTcBatch - 1) / kTcBatch);
}

// per u: its items (j << 32 | u) at its exclusive prefix ioff[u]
__global__ void k_tc_items_fill(const uint32_t *__restrict__ cnt,
                                const uint32_t *__restrict__ ioff, uint32_t n,
                                uint64_t *__restrict__ items) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n) return;
  const uint32_t c = cnt[u], o = ioff[u];
  for (uint32_t j = 0; j < c; j++) items[(uint64_t)o + j] = ((uint64_t)j << 32) | u;
}

// items a warp takes per visit to the cursor; their descriptors load in
// parallel, one per lane
constexpr int kTcGrab = 8;

// PV: also count, per vertex, the triangles it is in
template <bool PV>
__global__ void __launch_bounds__(kTcWarps * 32, 3)
k_tc_count(const uint64_t *__restrict__ off, const uint32_t *__restrict__ adj,
           const uint64_t *__restrict__ items, const uint32_t *__restrict__ nitems,
           unsigned long long *__restrict__ total, unsigned long long *__restrict__ pv) {
  extern __shared__ uint4 tc_sh[];
  const int lane = threadIdx.x & 31;
  const uint32_t full = 0xffffffffu;
  uint4 *tab = tc_sh + (threadIdx.x >> 5) * (kTcSlots / 4);
  const uint32_t Q = *nitems;
  unsigned long long local = 0;
  uint32_t set_u = kEmpty;  // the u whose N+ the set holds
  for (;;) {
    unsigned long long q0 = 0;
    if (lane == 0) q0 = atomicAdd(total + 1, (unsigned long long)kTcGrab);
    q0 = __shfl_sync(full, q0, 0);
    if (q0 >= Q) break;
    // lane g < kTcGrab: item q0 + g and its u's list bounds
    uint64_t my_it = 0, my_a0 = 0, my_na = 0;
    if (lane < kTcGrab && q0 + lane < Q) {
      my_it = items[q0 + lane];
      const uint32_t uu = (uint32_t)my_it;
      my_a0 = off[uu];
      my_na = off[uu + 1] - my_a0;
    }
    const int ng = (int)((Q - q0) < (unsigned long long)kTcGrab ? (Q - q0) : kTcGrab);
    // The item's v (stage 1) and its list bounds (stage 2) load ahead: v two
    // items before the item's turn, the bounds one item before (they need
    // v), so a small item's three dependent loads overlap earlier items.
    auto load_v = [&](int g, bool &okv) -> uint32_t {
      const uint64_t itg = __shfl_sync(full, my_it, g & 31);
      const uint64_t a0g = __shfl_sync(full, my_a0, g & 31);
      const uint64_t nag = __shfl_sync(full, my_na, g & 31);
      const uint64_t e = (itg >> 32) * kTcBatch + lane;
      okv = g < ng && e < nag;
      return okv ? adj[a0g + e] : 0u;
    };
    bool ok_n1 = false, ok_n2 = false;
    uint32_t v_n1 = load_v(0, ok_n1);  // item gi's v
    uint32_t v_n2 = load_v(1, ok_n2);  // item gi + 1's v
    uint64_t b_n1 = ok_n1 ? off[v_n1] : 0, e_n1 = ok_n1 ? off[v_n1 + 1] : 0;
    for (int gi = 0; gi < ng; gi++) {
      const uint64_t it = __shfl_sync(full, my_it, gi);
      const uint64_t a0 = __shfl_sync(full, my_a0, gi);
      const uint64_t na = __shfl_sync(full, my_na, gi);
      const uint32_t u = (uint32_t)it;
      const uint32_t *A = adj + a0;
      // this lane's v and the bounds of N+(v), loaded ahead
      const bool okv = ok_n1;
      const uint32_t v = okv ? v_n1 : 0u;
      const uint64_t b0 = okv ? b_n1 : 0;
      const uint64_t l = okv ? e_n1 - b_n1 : 0;
      const uint32_t len = l > 0xffffffffull ? 0xffffffffu : (uint32_t)l;
      // the next items' loads go out before this item's work
      bool ok_n3 = false;
      const uint32_t v_n3 = load_v(gi + 2, ok_n3);
      ok_n1 = ok_n2;
      v_n1 = v_n2;
      b_n1 = ok_n2 ? off[v_n2] : 0;
      e_n1 = ok_n2 ? off[v_n2 + 1] : 0;
      ok_n2 = ok_n3;
      v_n2 = v_n3;
      const bool hashed = na <= kTcSlots / 2;
      int bits = 3;
      while (bits < kTcBucketBits && (1ull << bits) < 2 * na) bits++;
      if (hashed && u != set_u) {
        __syncwarp();  // the last item's lookups are done
        for (uint32_t i = lane; i < (1u << bits); i += 32)
          tab[i] = make_uint4(kEmpty, kEmpty, kEmpty, kEmpty);
        __syncwarp();
        for (uint64_t i = lane; i < na; i += 32) tc_set_insert(tab, A[i], bits);
        __syncwarp();
        set_u = u;
      }
      // inclusive prefix of the lengths.  It fits 32 bits: every w in N+(v)
      // has degree >= deg(v) >= |N+(v)|, so |N+(v)|^2 <= m and 32 lists
      // reach 2^32 items only past 2^54 edges
      uint32_t P = len;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(full, P, d);
        if (lane >= d) P += y;
      }
      const uint32_t T = __shfl_sync(full, P, 31);
      // item k of list i sits at adj[base_i + k], base_i = b0_i - (P_i - len_i)
      const uint64_t base = b0 - (uint64_t)(P - len);
      int cur = 0;  // this lane's list; P_31 = T > k keeps it below 32
      uint32_t cend = __shfl_sync(full, P, 0);
      uint64_t cb = __shfl_sync(full, base, 0);
      uint32_t cvx = PV ? __shfl_sync(full, v, 0) : 0u;
      unsigned long long cu = 0;
      for (uint32_t k0 = 0; k0 < T; k0 += 32 * kTcAhead) {
        uint32_t w[kTcAhead], vv[kTcAhead];
#pragma unroll
        for (int t = 0; t < kTcAhead; t++) {
          w[t] = kEmpty;
          vv[t] = 0;
          if (k0 + 32 * t >= T) continue;  // uniform: the stream ended
          const uint32_t k = k0 + 32 * t + lane;
          bool adv = k < T && k >= cend;
          while (__any_sync(full, adv)) {
            cur += adv ? 1 : 0;
            cend = __shfl_sync(full, P, cur);
            cb = __shfl_sync(full, base, cur);
            if (PV) cvx = __shfl_sync(full, v, cur);
            adv = k < T && k >= cend;
          }
          if (k < T) w[t] = adj[cb + k];  // ids are below n <= 2^32 - 1
          vv[t] = cvx;
        }
#pragma unroll
        for (int t = 0; t < kTcAhead; t++) {
          if (k0 + 32 * t >= T) continue;  // uniform
          const bool on = w[t] != kEmpty;
          bool hit;
          if (hashed) {
            hit = tc_set_has_warp(tab, w[t], bits, on);
          } else {
            hit = on && sorted_has(A, na, w[t]);
          }
          if (hit) {
            cu++;
            if (PV) {
              atomicAdd(&pv[w[t]], 1ull);
              atomicAdd(&pv[vv[t]], 1ull);
            }
          }
        }
      }
      if (PV) {
        unsigned long long c = cu;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(full, c, d);
        if (lane == 0 && c) atomicAdd(&pv[u], c);
      }
      local += cu;
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) local += __shfl_down_sync(full, local, d);
  if (lane == 0 && local) atomicAdd(total, local);
}

// Scratch of a count over n vertices and madj oriented entries: cnt and
// ioff n + 1 entries each, items tc_items_bound(n, madj) entries, and
// scan_scratch_bytes(n + 1, 4) of arena.
struct TcScratch {
  uint32_t *cnt, *ioff;
  uint64_t *items;
};
// an item per started batch of 32: sum ceil(na/32) <= madj/32 + n, and,
// counting only na >= 2, <= madj/2
inline uint64_t tc_items_bound(uint32_t n, uint64_t madj) {
  return std::min<uint64_t>(madj / 32 + n, madj / 2) + 1;
}

// Counts the triangles of off[n + 1] / adj (device, madj entries).  total
// (device) holds two counters the caller zeroes: total[0] gets the count,
// total[1] is the work cursor.  pv (device, zeroed, may be null) gets
// per-vertex counts.  One persistent grid of as many blocks as fit.
inline cudaError_t tc_count_launch(const uint64_t *off, const uint32_t *adj, uint32_t n,
                                   uint64_t madj, const TcScratch &sc, Arena &arena,
                                   unsigned long long *total, unsigned long long *pv,
                                   int sms, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (tc_items_bound(n, madj) >= (1ull << 32)) return cudaErrorInvalidValue;
  const unsigned vblocks = (unsigned)(((uint64_t)n + 255) / 256);
  SST_LAUNCH(k_tc_items_count, vblocks, 256, 0, s, off, n, sc.cnt);
  cudaError_t e = scan<uint32_t, OpAdd>(sc.cnt, sc.ioff, n, 0u, OpAdd{}, true, false,
                                        sc.ioff + n, arena, s);
  if (e != cudaSuccess) return e;
  SST_LAUNCH(k_tc_items_fill, vblocks, 256, 0, s, sc.cnt, sc.ioff, n, sc.items);
  const size_t shm = (size_t)kTcWarps * kTcSlots * 4;
  auto kern = pv ? k_tc_count<true> : k_tc_count<false>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTcWarps * 32, shm);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)(std::max(per_sm, 1) * sms);
  if (pv)
    SST_LAUNCH(k_tc_count<true>, grid, kTcWarps * 32, shm, s, off, adj, sc.items,
               sc.ioff + n, total, pv);
  else
    SST_LAUNCH(k_tc_count<false>, grid, kTcWarps * 32, shm, s, off, adj, sc.items,
               sc.ioff + n, total, pv);
  return cudaGetLastError();
}

}  // namespace
}  // namespace sst

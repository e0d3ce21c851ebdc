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

// Warp per vertex u (the lowest-ranked vertex of the triangles it counts):
// N+(u) goes into a hash set in the warp's shared memory (open addressing,
// at most half full); then for each v in N+(u) in turn the warp's lanes
// stride over N+(v) (coalesced) and probe the set for each w.  A list too
// long for the set is probed by binary search in global memory instead.
constexpr uint32_t kTcHash = 2048;  // set slots per warp (8 KiB)
// longest v list a lane walks alone (longer ones: the whole warp strides)
constexpr uint32_t kTcLaneWalk = 64;
constexpr int kTcWarps = 8;         // warps per block

// multiplicative hashing (Knuth): the top `bits` bits of x * 2^32/phi
__device__ __forceinline__ uint32_t tc_hash(uint32_t x, int bits) {
  return (x * 0x9E3779B1u) >> (32 - bits);
}

__global__ void __launch_bounds__(kTcWarps * 32, 3)
k_tc_count(const uint64_t *__restrict__ off, const uint32_t *__restrict__ adj,
           uint32_t n, unsigned long long *__restrict__ total,
           unsigned long long *__restrict__ pv) {
  extern __shared__ uint32_t tc_sh[];
  const int lane = threadIdx.x & 31;
  uint32_t *tab = tc_sh + (threadIdx.x >> 5) * kTcHash;
  const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  unsigned long long local = 0;
  for (uint64_t u = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n;
       u += warps) {
    const uint64_t a0 = off[u];
    const uint64_t na = off[u + 1] - a0;
    if (na < 2) continue;  // a triangle needs two neighbours above u
    const uint32_t *A = adj + a0;
    const bool hashed = na <= kTcHash / 2;
    uint32_t mask = 0;
    int bits = 5;
    if (hashed) {
      while ((1ull << bits) < 2 * na) bits++;
      mask = (1u << bits) - 1;
      for (uint32_t i = lane; i <= mask; i += 32) tab[i] = kEmpty;
      __syncwarp();
      for (uint64_t i = lane; i < na; i += 32) {
        const uint32_t x = A[i];
        uint32_t h = tc_hash(x, bits);
        while (atomicCAS(&tab[h], kEmpty, x) != kEmpty) h = (h + 1) & mask;
      }
      __syncwarp();
    }
    unsigned long long cu = 0;
    uint64_t mb0 = 0, mb1 = 0;  // this lane's v list, for a short N+(u)
    uint32_t longest = ~0u;
    if (hashed && na <= 32) {
      if ((uint64_t)lane < na) {
        const uint32_t v = A[lane];
        mb0 = off[v];
        mb1 = off[v + 1];
      }
      const uint64_t len = mb1 - mb0;
      longest = __reduce_max_sync(0xffffffffu, len > 0xffffffffull ? 0xffffffffu : (uint32_t)len);
    }
    if (longest <= kTcLaneWalk) {
      // a short N+(u) whose v lists are short too: each lane walks one v's
      // list alone, probing the set
      if ((uint64_t)lane < na) {
        const uint32_t v = A[lane];
        const uint64_t b0 = mb0, b1 = mb1;
        unsigned long long cv = 0;
        for (uint64_t j = b0; j < b1; j++) {
          const uint32_t w = adj[j];
          uint32_t h = tc_hash(w, bits), x;
          while ((x = tab[h]) != w && x != kEmpty) h = (h + 1) & mask;
          if (x == w) {
            cv++;
            if (pv) atomicAdd(&pv[w], 1ull);
          }
        }
        if (pv && cv) atomicAdd(&pv[v], cv);
        cu = cv;
      }
      if (pv) {
        unsigned long long t = cu;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(0xffffffffu, t, d);
        if (lane == 0 && t) atomicAdd(&pv[u], t);
      }
      local += cu;
      __syncwarp();
      continue;
    }
    for (uint64_t i = 0; i < na; i++) {
      const uint32_t v = A[i];
      const uint64_t b0 = off[v], b1 = off[v + 1];
      unsigned long long cv = 0;
      for (uint64_t j = b0 + lane; j < b1; j += 32) {
        const uint32_t w = adj[j];
        bool hit;
        if (hashed) {
          uint32_t h = tc_hash(w, bits), x;
          while ((x = tab[h]) != w && x != kEmpty) h = (h + 1) & mask;
          hit = x == w;
        } else {
          hit = sorted_has(A, na, w);
        }
        if (hit) {
          cv++;
          if (pv) atomicAdd(&pv[w], 1ull);
        }
      }
      if (pv) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) cv += __shfl_xor_sync(0xffffffffu, cv, d);
        if (lane == 0 && cv) atomicAdd(&pv[v], cv);
        if (lane != 0) cv = 0;  // counted once, by lane 0, below
      }
      cu += cv;
    }
    if (pv) {
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) cu += __shfl_xor_sync(0xffffffffu, cu, d);
      if (lane == 0 && cu) atomicAdd(&pv[u], cu);
      if (lane != 0) cu = 0;
    }
    local += cu;
    __syncwarp();  // the set is rebuilt for the next u
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) local += __shfl_down_sync(0xffffffffu, local, d);
  if (lane == 0 && local) atomicAdd(total, local);
}

// k_tc_count over off[n + 1] / adj (device); total (device, zeroed by the
// caller) gets the count, pv (device, zeroed, may be null) per-vertex counts
inline cudaError_t tc_count_launch(const uint64_t *off, const uint32_t *adj, uint32_t n,
                                   unsigned long long *total, unsigned long long *pv,
                                   int sms, cudaStream_t s) {
  const size_t shm = (size_t)kTcWarps * kTcHash * 4;
  cudaError_t e = cudaFuncSetAttribute(k_tc_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)shm);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tc_count, kTcWarps * 32, shm);
  if (e != cudaSuccess) return e;
  const uint64_t want = ((uint64_t)n + kTcWarps - 1) / kTcWarps;
  const unsigned grid =
      (unsigned)std::min<uint64_t>(want, (uint64_t)std::max(per_sm, 1) * sms * 8);
  SST_LAUNCH(k_tc_count, grid, kTcWarps * 32, shm, s, off, adj, n, total, pv);
  return cudaGetLastError();
}

}  // namespace
}  // namespace sst

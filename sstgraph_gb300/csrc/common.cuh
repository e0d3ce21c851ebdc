// Shared definitions of the device-resident dynamic graph.
//
// Layout in HBM (one graph):
//   vertex table (structure of arrays, n entries)
//     seg_base[v]  u64  first slot of v's segment in the slab
//     seg_cap[v]   u32  segment capacity in slots: 0 or a power of two
//     deg[v]       u32  number of neighbours stored
//   slab           u32 slots[nslots]; EMPTY (0xFFFFFFFF) marks a gap
//   leaf counts    u8  lcnt[nslots / 32]: elements in each 32-slot leaf
//
// A segment of capacity <= 32 is one leaf, packed left, holding deg
// elements (the reference's in-place / dense regimes, PMA.hpp:84-197).  A
// segment of capacity >= 64 is a packed memory array of cap/32 leaves of 32
// slots (one 128-byte line each); every leaf is packed left, holds
// lcnt[base/32 + leaf] >= 1 elements, and the leaves are in ascending key
// order, so leaf heads are strictly increasing (the reference's gapped PMA
// regime, PMA.hpp:19-74,570-664, with a fixed GPU-sized leaf instead of
// 2^floor(log2 log2 N) slots).  Segment bases are aligned to min(cap, 32)
// slots.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

namespace sst {

constexpr uint32_t kLeaf = 32;
constexpr uint32_t kLeafLog = 5;
constexpr uint32_t kEmpty = 0xFFFFFFFFu;
constexpr int kNumClasses = 34;  // capacities 2^0 .. 2^33

// Device view of one graph, passed by value to kernels.
struct DGraph {
  uint32_t n;
  uint32_t width;
  uint64_t *base;
  uint32_t *cap;
  uint32_t *deg;
  uint32_t *slots;
  uint8_t *lcnt;
  uint32_t *vals;  // per-slot edge values of a weighted graph, else null
};

// Density bounds of the device PMA (own choice, in the spirit of the
// reference's tables at PMA.hpp:19-74: the bounds tighten towards the root).
// A window of 2^t leaves in a segment of 2^H leaves may hold at most
// up(t) * 32 * 2^t elements after an insert and must hold at least
// low(t) * 32 * 2^t after a remove, with up/low interpolated linearly in t.
struct PmaParams {
  float upper_leaf = 1.0f;
  float upper_root = 0.85f;
  float lower_leaf = 4.0f / 32.0f;
  float lower_root = 0.20f;
  float grow_fill = 0.70f;  // target density when a segment is (re)sized
};

__host__ __device__ inline uint32_t nleaves_of(uint32_t cap) {
  return cap <= kLeaf ? 1u : (cap >> kLeafLog);
}

__host__ __device__ inline uint32_t log2_floor(uint64_t x) {
  uint32_t r = 0;
  while (x > 1) {
    x >>= 1;
    r++;
  }
  return r;
}

__host__ __device__ inline uint64_t next_pow2(uint64_t x) {
  if (x <= 1) return 1;
#ifdef __CUDA_ARCH__
  return 1ull << (64 - __clzll((long long)(x - 1)));
#else
  return 1ull << (64 - __builtin_clzll(x - 1));
#endif
}

// 2^24 / fill rounded up (fill clamped to [1/128, 1]): the resize target
// density as a fixed-point reciprocal, computed once on the host, so that
// sizing a segment takes one integer product instead of an FP64 division
// per resize.
inline uint64_t fill_inv_q24(float fill) {
  const double f = fill < 1.0f / 128 ? 1.0 / 128 : (fill > 1.0f ? 1.0 : (double)fill);
  return (uint64_t)ceil(16777216.0 / f);
}

// Capacity for a segment that must hold `total` (< 2^32) elements after a
// resize: at least total / fill + 1 slots, a power of two, and at least two
// leaves once above one leaf.
__host__ __device__ inline uint64_t cap_for(uint64_t total, uint64_t inv_q24) {
  if (total == 0) return 0;
  if (total <= kLeaf) return next_pow2(total);
  const uint64_t want = ((total * inv_q24) >> 24) + 1;
  const uint64_t c = next_pow2(want);
  return c < 2 * kLeaf ? 2 * kLeaf : c;
}

// maximum elements a window of 2^t leaves may hold in a segment of 2^H
// leaves after an insert
__host__ __device__ inline uint64_t window_upper(const PmaParams &p,
                                                 uint32_t t, uint32_t H) {
  double f = H == 0 ? p.upper_root
                    : p.upper_leaf + (double)(p.upper_root - p.upper_leaf) *
                                         (double)t / (double)H;
  return (uint64_t)(f * (double)((uint64_t)kLeaf << t));
}

// minimum elements such a window must hold after a remove
__host__ __device__ inline uint64_t window_lower(const PmaParams &p,
                                                 uint32_t t, uint32_t H) {
  double f = H == 0 ? p.lower_root
                    : p.lower_leaf + (double)(p.lower_root - p.lower_leaf) *
                                         (double)t / (double)H;
  uint64_t v = (uint64_t)(f * (double)((uint64_t)kLeaf << t));
  uint64_t leaves = 1ull << t;
  return v < leaves ? leaves : v;  // every leaf keeps >= 1 element
}

// splitmix64 output function (Steele, Lea, Flood 2014) and the
// counter-based draw used by every generator and sampler; the CPU oracle
// computes the same values.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}
__host__ __device__ __forceinline__ uint64_t draw(uint64_t seed, uint64_t i,
                                                  uint64_t j) {
  return mix64(mix64(seed * 0x9E3779B97F4A7C15ULL + i) ^
               (j * 0xD1B54A32D192ED03ULL + 0x8CB92BA72F3D8DD7ULL));
}

// number of elements in leaf l of vertex v
__device__ __forceinline__ uint32_t leaf_count(const DGraph &g, uint64_t base,
                                               uint32_t cap, uint32_t deg,
                                               uint32_t l) {
  return cap <= kLeaf ? deg : (uint32_t)g.lcnt[(base >> kLeafLog) + l];
}

// Leaf of a multi-leaf or single-leaf segment where x belongs: the last
// leaf whose head is <= x, or leaf 0.
__device__ __forceinline__ uint32_t find_leaf(const uint32_t *slots,
                                              uint64_t base, uint32_t cap,
                                              uint32_t x) {
  if (cap <= kLeaf) return 0;
  uint32_t lo = 0, hi = cap >> kLeafLog;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (slots[base + ((uint64_t)mid << kLeafLog)] <= x)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// position of the first element >= x in a packed leaf of c elements
__device__ __forceinline__ uint32_t leaf_lower_bound(const uint32_t *p,
                                                     uint32_t c, uint32_t x) {
  uint32_t lo = 0, hi = c;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (p[mid] < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

}  // namespace sst

#define SST_CUDA_TRY(expr)                                                    \
  do {                                                                        \
    cudaError_t _e = (expr);                                                  \
    if (_e != cudaSuccess) {                                                  \
      sst::set_cuda_error(_e, #expr, __FILE__, __LINE__);                     \
      return SST_EDEVICE;                                                     \
    }                                                                         \
  } while (0)

namespace sst {
void set_cuda_error(cudaError_t e, const char *what, const char *file,
                    int line);
void set_error_message(const char *fmt, ...);
}  // namespace sst

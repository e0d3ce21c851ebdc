// PageRank arithmetic shared by every PageRank kernel (the PMA lists in
// traverse.cu, the byte-width snapshot in compact.cu), so that all of them
// give bit-identical ranks.
//
// An iteration is integer-only fixed point in units of 2^-63: each
// contribution rank(u)/deg(u) is rounded once to a multiple of 2^-63, the
// per-edge sums are exact 64-bit integer additions (order-independent, so
// deterministic), and rank = (1-d)/n + d*sum uses a 64x64->128-bit product
// rounded to nearest.  GB300 runs FP64 at a small fraction of its integer
// rate; FP64 appears only when the final ranks are written.
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace sst {

__device__ __forceinline__ uint64_t mulhi_round(uint64_t a, uint64_t b) {
  return __umul64hi(a, b) + ((a * b) >> 63);
}

// round(2^64 / deg) for deg >= 2 (deg 1 passes rank through), 0 otherwise
__device__ __forceinline__ unsigned long long pr_rdeg_of(uint32_t d) {
  if (d < 2) return 0ull;
  unsigned __int128 num = ((unsigned __int128)1 << 64) + (d >> 1);
  return (unsigned long long)(num / d);
}

__device__ __forceinline__ unsigned long long contrib_of(unsigned long long rank,
                                                         uint32_t deg,
                                                         unsigned long long rd) {
  return deg == 1 ? rank : mulhi_round(rank, rd);
}

struct PrConst {
  unsigned long long B;  // (1-d)/n in 2^-63 units
  unsigned long long D;  // d in 2^-64 units
};

// the iteration constants and the starting rank 1/n in 2^-63 units
inline PrConst pr_const(uint32_t n, double damping, unsigned long long *r0f) {
  const double two63 = 9223372036854775808.0, two64 = 18446744073709551616.0;
  const double r0 = 1.0 / (double)n;
  const double base = (1.0 - damping) / (double)n;
  PrConst K;
  K.B = (unsigned long long)llrint(base * two63);
  K.D = damping >= 1.0 ? ~0ull : (unsigned long long)llrint(damping * two64 / 2.0) * 2ull;
  *r0f = (unsigned long long)llrint(r0 * two63);
  return K;
}

// rank of v from its in-sum: its next contribution, and (last iteration)
// the rank itself as FP64
__device__ __forceinline__ void pr_finish(uint32_t v, unsigned long long sum,
                                          PrConst k, uint32_t deg,
                                          const unsigned long long *rdeg,
                                          unsigned long long *cout,
                                          double *rank, bool last) {
  unsigned long long r = k.B + mulhi_round(sum, k.D);
  cout[v] = contrib_of(r, deg, rdeg[v]);
  if (last) rank[v] = __ull2double_rn(r) * (1.0 / 9223372036854775808.0);
}

// row ids are read once per iteration: keep them out of L1 and first in
// line for eviction from L2, so the contribution gathers keep both caches
__device__ __forceinline__ unsigned long long l2_evict_first() {
  unsigned long long pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ uint32_t ld_stream(const uint32_t *p,
                                              unsigned long long pol) {
  uint32_t v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;"
      : "=r"(v)
      : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ unsigned long long ld_keep(const unsigned long long *p) {
  unsigned long long v;
  asm("ld.global.nc.L1::evict_last.b64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}

}  // namespace sst

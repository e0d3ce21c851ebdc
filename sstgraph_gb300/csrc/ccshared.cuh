// Connected-components building blocks shared by the PMA graph
// (traverse.cu) and the byte-width snapshot (compact.cu): the
// layout-independent parts of Afforest (Sutton, Ben-Nun, Barak 2018).
//  1. link every vertex to its first two neighbours (two rounds, each
//     followed by compression);
//  2. sample 1024 vertices' roots and take the most frequent one, c: the
//     largest component so far;
//  3. link every edge of every vertex whose root is not c (on a symmetric
//     graph an edge with one end in c is linked from its other end), then
//     compress.
// A root is only ever linked below a smaller root (compare-and-swap on the
// larger one), so every component's final root -- its label -- is its
// smallest vertex id, independent of the order the links happen in.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sst {
namespace {

__device__ __forceinline__ uint32_t cc_root(const uint32_t *par, uint32_t x) {
  uint32_t p;
  while ((p = __ldcg(par + x)) != x) x = p;
  return x;
}

__global__ void k_iota(uint32_t *__restrict__ p, uint32_t n) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) p[v] = v;
}

__device__ __forceinline__ uint32_t ld_par(const uint32_t *par, uint32_t x) {
  return __ldcg(par + x);
}

// link the trees of u and v; err counts links that gave up (they cannot
// fail to progress; the bound only keeps every loop finite)
__device__ __forceinline__ void cc_link(uint32_t *par, uint32_t u, uint32_t v,
                                        unsigned long long *err) {
  uint32_t p1 = ld_par(par, u), p2 = ld_par(par, v);
  for (int it = 0; p1 != p2; it++) {
    if (it == (1 << 20)) {
      atomicAdd(err, 1ull);
      return;
    }
    const uint32_t hi = max(p1, p2), lo = min(p1, p2);
    const uint32_t ph = ld_par(par, hi);
    if (ph == lo) return;
    if (ph == hi && atomicCAS(&par[hi], hi, lo) == hi) return;
    p1 = ld_par(par, ld_par(par, hi));
    p2 = ld_par(par, lo);
  }
}

// the most frequent root among 1024 sampled vertices (ties: the smaller)
__global__ void __launch_bounds__(1024) k_cc_giant(const uint32_t *__restrict__ par,
                                                   uint32_t n,
                                                   unsigned long long *__restrict__ out) {
  __shared__ uint32_t lab[1024];
  __shared__ unsigned long long best;
  const uint32_t t = threadIdx.x;
  const uint32_t v = (uint32_t)(mix64(0x5EEDull + t) % n);
  lab[t] = par[v];
  if (t == 0) best = 0;
  __syncthreads();
  for (uint32_t k = 2; k <= 1024; k <<= 1)  // bitonic sort, ascending
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      const uint32_t o = t ^ j;
      if (o > t) {
        const uint32_t a = lab[t], b = lab[o];
        const bool up = (t & k) == 0;
        if ((a > b) == up) {
          lab[t] = b;
          lab[o] = a;
        }
      }
      __syncthreads();
    }
  if (t == 0 || lab[t] != lab[t - 1]) {
    uint32_t e = t + 1;
    while (e < 1024 && lab[e] == lab[t]) e++;
    // larger count first, then the smaller label
    atomicMax(&best, ((unsigned long long)(e - t) << 32) | (0xFFFFFFFFu - lab[t]));
  }
  __syncthreads();
  if (t == 0) out[0] = 0xFFFFFFFFu - (uint32_t)(best & 0xFFFFFFFFu);
}

__global__ void k_cc_compress(uint32_t *__restrict__ par, uint32_t n) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  par[v] = cc_root(par, v);
}

}  // namespace
}  // namespace sst

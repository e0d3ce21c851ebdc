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

// the root of x, halving the path on the way: a visited vertex is pointed
// at its grandparent.  Only roots are ever linked (compare-and-swap on a
// root's own entry), so a non-root's entry changes only here, and always to
// one of its ancestors: still its tree, and a smaller id.  Every step moves
// to a smaller id, so the walk ends.
__device__ __forceinline__ uint32_t cc_find(uint32_t *par, uint32_t x) {
  for (;;) {
    const uint32_t p = ld_par(par, x);
    if (p == x) return x;
    const uint32_t gp = ld_par(par, p);
    if (gp == p) return p;
    par[x] = gp;
    x = gp;
  }
}

// link the trees of u and v: find both roots, link the larger below the
// smaller; a failed compare-and-swap means that root was linked meanwhile,
// so the roots are looked up again.  err counts links that gave up (every
// failed attempt is another link's progress; the bound only keeps every
// loop finite).  Without halving, concurrent links build long chains of
// roots that later links walk again and again.
__device__ __forceinline__ void cc_link(uint32_t *par, uint32_t u, uint32_t v,
                                        unsigned long long *err) {
  // the finds start at the parents (usually the roots themselves)
  uint32_t p1 = ld_par(par, u), p2 = ld_par(par, v);
  if (p1 == p2) return;
  for (int it = 0;; it++) {
    if (it == (1 << 20)) {
      atomicAdd(err, 1ull);
      return;
    }
    const uint32_t r1 = cc_find(par, p1), r2 = cc_find(par, p2);
    if (r1 == r2) return;
    const uint32_t hi = max(r1, r2), lo = min(r1, r2);
    if (atomicCAS(&par[hi], hi, lo) == hi) return;
    p1 = hi;
    p2 = lo;
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

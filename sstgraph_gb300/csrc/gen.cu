// Device edge generators.  Each edge is a pure function of (stream, index),
// so any slice of a stream can be produced anywhere and the CPU oracle
// (oracle/sst_oracle.c) produces the identical pairs.
#include "common.cuh"
#include "primitives.cuh"

namespace sst {
namespace {

__global__ void k_rmat(uint32_t scale, uint64_t t0, uint64_t t1, uint64_t t2,
                       uint64_t seed, uint64_t first, uint64_t count,
                       uint32_t *__restrict__ pairs) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint64_t idx = first + i;
  uint32_t u = 0, v = 0;
  uint64_t h = 0;
  for (uint32_t l = 0; l < scale; l++) {
    if ((l & 1) == 0) h = draw(seed, idx, l >> 1);
    uint64_t r = (l & 1) ? (h >> 32) : (h & 0xffffffffULL);
    uint32_t bit = 1u << (scale - 1 - l);
    if (r >= t0) {
      if (r < t1) {
        v |= bit;
      } else if (r < t2) {
        u |= bit;
      } else {
        u |= bit;
        v |= bit;
      }
    }
  }
  pairs[2 * i] = u;
  pairs[2 * i + 1] = v;
}

__global__ void k_er(uint32_t n, uint64_t seed, uint64_t first, uint64_t count,
                     uint32_t *__restrict__ pairs) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint64_t h = draw(seed, first + i, 0);
  pairs[2 * i] = (uint32_t)(((h & 0xffffffffULL) * n) >> 32);
  pairs[2 * i + 1] = (uint32_t)(((h >> 32) * n) >> 32);
}

// rMat<uint32_t>::rMatRec of include/SSTGraph/internal/rmat_util.h:107-124,
// unrolled top level first; hash32 at :42-50.
__device__ __forceinline__ uint32_t ref_hash32(uint32_t a) {
  a = (a + 0x7ed55d16u) + (a << 12);
  a = (a ^ 0xc761c23cu) ^ (a >> 19);
  a = (a + 0x165667b1u) + (a << 5);
  a = (a + 0xd3a2646cu) ^ (a << 9);
  a = (a + 0xfd7046c5u) + (a << 3);
  a = (a ^ 0xb55a4f09u) ^ (a >> 16);
  return a;
}

__global__ void k_ref_rmat(uint32_t nn, uint32_t levels, uint32_t h, double a,
                           double ab, double abc, uint64_t first, uint64_t count,
                           uint32_t *__restrict__ pairs) {
  uint64_t ii = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= count) return;
  uint32_t i = (uint32_t)(first + ii);
  uint32_t start = ref_hash32((uint32_t)(2u * i) * h);
  uint32_t stride = ref_hash32((uint32_t)(2u * i + 1u) * h);
  uint32_t u = 0, v = 0;
  for (uint32_t k = 0; k < levels; k++) {
    uint32_t half = (nn >> k) / 2;
    // IEEE division, as on the host
    double r = __ddiv_rn((double)ref_hash32(start + k * stride), 2147483647.0);
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

uint64_t host_ref_hash64(uint64_t u) {
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
uint32_t host_ref_hash32(uint32_t a) {
  a = (a + 0x7ed55d16u) + (a << 12);
  a = (a ^ 0xc761c23cu) ^ (a >> 19);
  a = (a + 0x165667b1u) + (a << 5);
  a = (a + 0xd3a2646cu) ^ (a << 9);
  a = (a + 0xfd7046c5u) + (a << 3);
  a = (a ^ 0xb55a4f09u) ^ (a >> 16);
  return a;
}

}  // namespace

cudaError_t gen_rmat(uint32_t scale, double a, double b, double c, uint64_t seed,
                     uint64_t first, uint64_t count, uint32_t *d_pairs,
                     cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  uint64_t t0 = (uint64_t)(a * 4294967296.0);
  uint64_t t1 = (uint64_t)((a + b) * 4294967296.0);
  uint64_t t2 = (uint64_t)((a + b + c) * 4294967296.0);
  SST_LAUNCH(k_rmat, (unsigned)((count + 255) / 256), 256, 0, s, scale, t0, t1,
             t2, seed, first, count, d_pairs);
  return cudaGetLastError();
}

cudaError_t gen_er(uint32_t n, uint64_t seed, uint64_t first, uint64_t count,
                   uint32_t *d_pairs, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  SST_LAUNCH(k_er, (unsigned)((count + 255) / 256), 256, 0, s, n, seed, first,
             count, d_pairs);
  return cudaGetLastError();
}

cudaError_t gen_ref_rmat(uint32_t nn, double a, double b, double c,
                         uint64_t first, uint64_t count, uint32_t *d_pairs,
                         cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  uint32_t levels = 0;
  while ((1u << levels) < nn) levels++;
  // random_aspen().ith_rand(0) = hash64(0), truncated to the uint32 seed
  uint32_t h = host_ref_hash32((uint32_t)host_ref_hash64(0));
  SST_LAUNCH(k_ref_rmat, (unsigned)((count + 255) / 256), 256, 0, s, nn, levels,
             h, a, a + b, a + b + c, first, count, d_pairs);
  return cudaGetLastError();
}

}  // namespace sst

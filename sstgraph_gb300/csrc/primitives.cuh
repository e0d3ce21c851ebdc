// Device primitives shared by the update and traversal paths: a scratch
// arena, block/grid scans (any associative operator, forward or reverse),
// and a stable LSD radix sort of 64-bit keys.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sst {

void note_launch();
uint64_t launches();

// Kernel profiler: while enabled, every launch is bracketed by a pair of
// CUDA events on its own stream; profile_collect() folds the elapsed times
// per kernel name, with the algorithmic bytes the launch sites declare
// (SST_LAUNCH_B: the bytes the kernel must read and write at its launch
// size, independent of caching).
bool profiling(const char *kernel_name);
cudaEvent_t prof_begin(cudaStream_t s);
void prof_end(const char *name, cudaEvent_t start, cudaStream_t s,
              uint64_t bytes);

#define SST_LAUNCH_B(bytes, kernel, grid, block, smem, stream, ...)           \
  do {                                                                        \
    cudaEvent_t _sst_ev =                                                     \
        ::sst::profiling(#kernel) ? ::sst::prof_begin(stream) : nullptr;      \
    kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);               \
    ::sst::note_launch();                                                     \
    if (_sst_ev) ::sst::prof_end(#kernel, _sst_ev, stream, (bytes));          \
  } while (0)
#define SST_LAUNCH(kernel, grid, block, smem, stream, ...)                    \
  SST_LAUNCH_B(0, kernel, grid, block, smem, stream, __VA_ARGS__)

// ----------------------------------------------------------------- arena
// Bump allocator over one device buffer; reset at the start of each
// operation.  Growing it frees and reallocates (callers grow before use).
struct Arena {
  char *base = nullptr;
  size_t cap = 0;
  size_t used = 0;
  size_t peak = 0;

  cudaError_t reserve(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (base) {
      cudaError_t e = cudaFree(base);
      if (e != cudaSuccess) return e;
      base = nullptr;
      cap = 0;
    }
    size_t want = bytes + bytes / 4 + (1u << 20);
    cudaError_t e = cudaMalloc(&base, want);
    if (e != cudaSuccess) {
      base = nullptr;
      return e;
    }
    cap = want;
    return cudaSuccess;
  }
  // tile status words of the single-pass scan (32 B per tile), kept apart
  // from the bump memory so stale tags come only from earlier scans; each
  // scan tags its words with a fresh epoch
  uint4 *status = nullptr;
  uint64_t status_cap = 0;
  unsigned long long epoch = 0;
  unsigned long long *err = nullptr;  // counts look-back waits that ran out

  // the words are zeroed on the scan's own stream (the library's streams do
  // not synchronise with the legacy default stream), so the first scan never
  // sees uninitialised tags
  cudaError_t reserve_status(uint64_t tiles, cudaStream_t s) {
    if (tiles <= status_cap) return cudaSuccess;
    if (status) cudaFree(status);
    status = nullptr;
    status_cap = 0;
    uint64_t want = tiles + tiles / 4 + 64;
    cudaError_t e = cudaMalloc(&status, 2 * want * sizeof(uint4));
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(status, 0, 2 * want * sizeof(uint4), s);
    if (e != cudaSuccess) return e;
    status_cap = want;
    return cudaSuccess;
  }
  void release() {
    if (base) cudaFree(base);
    base = nullptr;
    cap = used = 0;
    if (status) cudaFree(status);
    status = nullptr;
    status_cap = 0;
  }
  void reset() { used = 0; }
  template <typename T> T *take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    if (used + bytes > cap) return nullptr;
    T *p = reinterpret_cast<T *>(base + used);
    used += bytes;
    if (used > peak) peak = used;
    return p;
  }
};

// ---------------------------------------------------------------- scans
struct OpAdd {
  template <typename T> __device__ __forceinline__ T operator()(T a, T b) const {
    return a + b;
  }
};
struct OpMax {
  template <typename T> __device__ __forceinline__ T operator()(T a, T b) const {
    return a > b ? a : b;
  }
};
struct OpMin {
  template <typename T> __device__ __forceinline__ T operator()(T a, T b) const {
    return a < b ? a : b;
  }
};

// 8192-element tiles: a 1e6-element scan is ~120 tiles, so the look-back
// of the single-pass scan meets an inclusive prefix within a few windows
constexpr int kScanThreads = 512;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T, typename Op>
__device__ __forceinline__ T warp_inclusive(T v, Op op) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v = op(o, v);
  }
  return v;
}

// exclusive scan of one value per thread across the block; returns the
// block total through *total
template <typename T, typename Op>
__device__ __forceinline__ T block_exclusive(T v, T identity, Op op, T *total) {
  __shared__ T warp_tot[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T inc = warp_inclusive(v, op);
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < kScanThreads / 32 ? warp_tot[lane] : identity;
    T wi = warp_inclusive(w, op);
    if (lane < kScanThreads / 32) warp_tot[lane] = wi;
  }
  __syncthreads();
  T prefix = warp == 0 ? identity : warp_tot[warp - 1];
  T excl_in_warp = __shfl_up_sync(0xffffffffu, inc, 1);
  if (lane == 0) excl_in_warp = identity;
  T res = warp == 0 ? excl_in_warp : (lane == 0 ? prefix : op(prefix, excl_in_warp));
  *total = warp_tot[kScanThreads / 32 - 1];
  __syncthreads();
  return res;
}

template <typename T, typename Op>
__global__ void k_scan_reduce(const T *__restrict__ in, uint64_t n, T identity,
                              Op op, bool reverse, T *__restrict__ block_sums,
                              const uint32_t *__restrict__ d_n) {
  if (d_n && *d_n < n) n = *d_n;
  uint64_t tile0 = (uint64_t)blockIdx.x * kScanTile;
  T acc = identity;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = tile0 + (uint64_t)threadIdx.x * kScanItems + k;
    if (i < n) acc = op(acc, in[reverse ? n - 1 - i : i]);
  }
  T total;
  block_exclusive(acc, identity, op, &total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

template <typename T, typename Op>
__global__ void k_scan_apply(const T *__restrict__ in, T *__restrict__ out,
                             uint64_t n, T identity, Op op, bool reverse,
                             bool exclusive, const T *__restrict__ block_prefix,
                             T *__restrict__ total_out,
                             const uint32_t *__restrict__ d_n) {
  if (d_n && *d_n < n) n = *d_n;
  uint64_t tile0 = (uint64_t)blockIdx.x * kScanTile;
  T vals[kScanItems];
  T acc = identity;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = tile0 + (uint64_t)threadIdx.x * kScanItems + k;
    vals[k] = i < n ? in[reverse ? n - 1 - i : i] : identity;
    acc = op(acc, vals[k]);
  }
  T total;
  T run = block_exclusive(acc, identity, op, &total);
  if (block_prefix) run = op(block_prefix[blockIdx.x], run);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = tile0 + (uint64_t)threadIdx.x * kScanItems + k;
    T nxt = op(run, vals[k]);
    if (i < n) out[reverse ? n - 1 - i : i] = exclusive ? run : nxt;
    run = nxt;
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    T t = block_prefix ? op(block_prefix[blockIdx.x], total) : total;
    *total_out = t;
  }
}

// Single-pass scan with decoupled look-back (Merrill & Garland 2016): each
// tile publishes its aggregate, then its inclusive prefix once the prefix of
// the tiles before it is known, so one launch scans the whole array.  Tiles
// rely on blocks being dispatched in index order; every wait on a
// predecessor is bounded and counts a failure in *err instead of hanging.
constexpr unsigned long long kScanAgg = 1, kScanIncl = 2;
constexpr uint32_t kLookbackSpins = 1u << 22;

// A tile's status is two 16-byte words: {tag, aggregate} and {inclusive
// prefix, -}.  The aggregate and the inclusive prefix live in separate
// fields, each written before the tag that announces it and never changed
// afterwards, so a reader takes the field that matches the tag it saw (a
// shared field could be overwritten between the reader's tag and value
// loads).
template <typename T>
__device__ __forceinline__ void tile_publish(uint4 *st, unsigned long long tag,
                                             T v) {
  volatile unsigned long long *w = reinterpret_cast<volatile unsigned long long *>(st);
  unsigned long long bits = 0;
  memcpy(&bits, &v, sizeof(T));
  w[(tag & 3) == kScanIncl ? 2 : 1] = bits;
  __threadfence();
  w[0] = tag;
}

template <typename T, typename Op>
__global__ void k_scan_single(const T *__restrict__ in, T *__restrict__ out,
                              uint64_t n, T identity, Op op, bool reverse,
                              bool exclusive, T *__restrict__ total_out,
                              const uint32_t *__restrict__ d_n, uint4 *status,
                              unsigned long long epoch,
                              unsigned long long *err) {
  if (d_n && *d_n < n) n = *d_n;
  const uint64_t tile = blockIdx.x;
  uint64_t tile0 = tile * kScanTile;
  T vals[kScanItems];
  T acc = identity;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = tile0 + (uint64_t)threadIdx.x * kScanItems + k;
    vals[k] = i < n ? in[reverse ? n - 1 - i : i] : identity;
    acc = op(acc, vals[k]);
  }
  T total;
  T run = block_exclusive(acc, identity, op, &total);
  __shared__ T s_prefix;
  if (threadIdx.x < 32) {
    // warp 0 looks back over 32 predecessors at a time: lane k reads tile
    // j - k; the window is folded up to the nearest tile that has published
    // its inclusive prefix (tile 0 always does)
    const int lane = threadIdx.x;
    const unsigned long long tagA = (epoch << 2) | kScanAgg;
    const unsigned long long tagI = (epoch << 2) | kScanIncl;
    T prefix = identity;
    if (tile == 0) {
      if (lane == 0) tile_publish(status, tagI, total);
    } else {
      if (lane == 0) tile_publish(status + 2 * tile, tagA, total);
      int64_t j = (int64_t)tile - 1;
      for (;;) {
        const int64_t mine = j - lane;
        bool incl = false, failed = false;
        T v = identity;
        if (mine >= 0) {
          volatile unsigned long long *w =
              reinterpret_cast<volatile unsigned long long *>(status + 2 * mine);
          unsigned long long tag = w[0];
          uint32_t spins = 0;
          while ((tag >> 2) != epoch && spins < kLookbackSpins) {
            __nanosleep(32);
            tag = w[0];
            spins++;
          }
          if ((tag >> 2) != epoch) {
            failed = true;
          } else {
            __threadfence();
            incl = (tag & 3) == kScanIncl;
            unsigned long long bits = incl ? w[2] : w[1];
            memcpy(&v, &bits, sizeof(T));
          }
        }
        const unsigned im = __ballot_sync(0xffffffffu, incl);
        const unsigned fm = __ballot_sync(0xffffffffu, failed);
        // lanes up to the nearest inclusive one contribute (the ops are
        // commutative, so the fold order within the window is free)
        const int stop = im ? __ffs(im) - 1 : 31;
        T c = lane <= stop ? v : identity;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) c = op(c, __shfl_xor_sync(0xffffffffu, c, d));
        prefix = op(c, prefix);
        if (fm) {
          if (lane == 0 && err) atomicAdd(err, 1ull);
          break;
        }
        if (im || j < 32) break;
        j -= 32;
      }
      if (lane == 0) tile_publish(status + 2 * tile, tagI, op(prefix, total));
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  run = op(s_prefix, run);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = tile0 + (uint64_t)threadIdx.x * kScanItems + k;
    T nxt = op(run, vals[k]);
    if (i < n) out[reverse ? n - 1 - i : i] = exclusive ? run : nxt;
    run = nxt;
  }
  if (total_out && tile == gridDim.x - 1 && threadIdx.x == 0)
    *total_out = op(s_prefix, total);
}

// Scan of n elements (in may equal out).  total_out (device, may be null)
// receives the reduction of all n elements.  With d_n (device, may be null)
// only the first min(n, *d_n) elements are scanned; n sizes the launch.
template <typename T, typename Op>
cudaError_t scan(const T *in, T *out, uint64_t n, T identity, Op op,
                 bool exclusive, bool reverse, T *total_out, Arena &arena,
                 cudaStream_t s, const uint32_t *d_n = nullptr) {
  if (n == 0) {
    if (total_out) return cudaMemcpyAsync(total_out, &identity, sizeof(T),
                                          cudaMemcpyHostToDevice, s);
    return cudaSuccess;
  }
  uint64_t blocks = (n + kScanTile - 1) / kScanTile;
  const uint64_t bytes = 2 * sizeof(T) * n;  // read in, write out
  if (blocks == 1) {
    SST_LAUNCH_B(bytes, (k_scan_apply<T, Op>), 1, kScanThreads, 0, s, in, out, n,
               identity, op, reverse, exclusive, (const T *)nullptr, total_out,
               d_n);
    return cudaGetLastError();
  }
  if (sizeof(T) <= 8 && arena.reserve_status(blocks, s) == cudaSuccess) {
    arena.epoch++;
    SST_LAUNCH_B(bytes, (k_scan_single<T, Op>), (unsigned)blocks, kScanThreads, 0, s, in,
               out, n, identity, op, reverse, exclusive, total_out, d_n,
               arena.status, arena.epoch, arena.err);
    return cudaGetLastError();
  }
  T *sums = arena.take<T>(blocks);
  if (!sums) return cudaErrorMemoryAllocation;
  SST_LAUNCH((k_scan_reduce<T, Op>), (unsigned)blocks, kScanThreads, 0, s, in,
             n, identity, op, reverse, sums, d_n);
  // block prefixes in block order (reverse handled inside the tiles)
  cudaError_t e = scan<T, Op>(sums, sums, blocks, identity, op, true, false,
                              (T *)nullptr, arena, s);
  if (e != cudaSuccess) return e;
  SST_LAUNCH((k_scan_apply<T, Op>), (unsigned)blocks, kScanThreads, 0, s, in,
             out, n, identity, op, reverse, exclusive, (const T *)sums,
             total_out, d_n);
  return cudaGetLastError();
}

// scratch bytes a scan of n elements of T takes from the arena
inline size_t scan_scratch_bytes(uint64_t n, size_t elem) {
  size_t bytes = 0;
  uint64_t blocks = (n + kScanTile - 1) / kScanTile;
  while (blocks > 1) {
    bytes += ((blocks * elem + 255) & ~size_t(255));
    blocks = (blocks + kScanTile - 1) / kScanTile;
  }
  return bytes + 256;
}

// ----------------------------------------------------------- radix sort
// Stable LSD radix sort of 64-bit keys on their low `bits` bits, 8-bit
// digits.  keys and tmp are both n long; *result points at whichever holds
// the sorted keys.  Batches up to kSmallSort keys sort in one CTA.
constexpr int kSmallSort = 2048;
// the same with a 32-bit payload per key moved along (stable)
cudaError_t radix_sort_kv(uint64_t *keys, uint64_t *tmp, uint32_t *vals,
                          uint32_t *vtmp, uint64_t n, int bits, Arena &arena,
                          cudaStream_t s, uint64_t **result, uint32_t **vresult);
cudaError_t radix_sort_u64(uint64_t *keys, uint64_t *tmp, uint64_t n, int bits,
                           Arena &arena, cudaStream_t s, uint64_t **result);
size_t radix_sort_scratch_bytes(uint64_t n);

}  // namespace sst

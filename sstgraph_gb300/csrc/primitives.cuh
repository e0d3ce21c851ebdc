// Device primitives shared by the update and traversal paths: a scratch
// arena, block/grid scans (any associative operator, forward or reverse),
// and a stable LSD radix sort of 64-bit keys.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <utility>

#include "common.cuh"

namespace sst {

// kernels launched by this library (a captured graph's kernels count when
// the graph is launched, not when it is captured)
void note_launch();
void note_launches(int64_t k);
uint64_t launches();
// a tag unique to one single-pass scan launch (see ScanStatus)
unsigned long long next_scan_tag();
// polls of a predecessor's flag before a single-pass scan tile reduces the
// predecessors' inputs itself (kLookbackPolls unless set; 0: no tile waits,
// every tile after the first takes that fallback)
int lookback_polls();
void set_lookback_polls(int polls);

// Kernel profiler: while enabled, every launch is bracketed by a pair of
// CUDA events on its own stream; profile_collect() folds the elapsed times
// per kernel name, with the algorithmic bytes the launch sites declare
// (SST_LAUNCH_B: the bytes the kernel must read and write at its launch
// size, independent of caching).
bool profiling(const char *kernel_name);
// While alive, launches from this thread are not timed one by one (a stream
// capture records them into a graph, whose replay is timed as a whole).
struct ProfPause {
  ProfPause();
  ~ProfPause();
  bool prev;
};
cudaEvent_t prof_begin(cudaStream_t s);
void prof_end(const char *name, cudaEvent_t start, cudaStream_t s,
              uint64_t bytes);

#define SST_LAUNCH_NB(name, bytes, kernel, grid, block, smem, stream, ...)    \
  do {                                                                        \
    cudaEvent_t _sst_ev =                                                     \
        ::sst::profiling(name) ? ::sst::prof_begin(stream) : nullptr;         \
    kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);               \
    ::sst::note_launch();                                                     \
    if (_sst_ev) ::sst::prof_end(name, _sst_ev, stream, (bytes));             \
  } while (0)
#define SST_LAUNCH_B(bytes, kernel, grid, block, smem, stream, ...)           \
  SST_LAUNCH_NB(#kernel, bytes, kernel, grid, block, smem, stream, __VA_ARGS__)
#define SST_LAUNCH(kernel, grid, block, smem, stream, ...)                    \
  SST_LAUNCH_B(0, kernel, grid, block, smem, stream, __VA_ARGS__)

// Programmatic dependent launch: the kernel may be scheduled while the
// kernel before it on the stream still runs (its launch and block set-up
// overlap that kernel's tail); it must call pdl_wait() before touching
// anything the earlier kernels read or write.  Used for the update
// pipeline's chains of dependent kernels (graph.cu, the scans and sorts);
// captured into a CUDA graph the dependency becomes a programmatic edge.
#define SST_LAUNCH_PDL_NB(name, bytes, kernel, grid, block, smem, stream, ...) \
  do {                                                                        \
    cudaEvent_t _sst_ev =                                                     \
        ::sst::profiling(name) ? ::sst::prof_begin(stream) : nullptr;         \
    ::sst::launch_pdl(kernel, (grid), (block), (smem), (stream), __VA_ARGS__); \
    ::sst::note_launch();                                                     \
    if (_sst_ev) ::sst::prof_end(name, _sst_ev, stream, (bytes));             \
  } while (0)
#define SST_LAUNCH_PDL_B(bytes, kernel, grid, block, smem, stream, ...)       \
  SST_LAUNCH_PDL_NB(#kernel, bytes, kernel, grid, block, smem, stream, __VA_ARGS__)
#define SST_LAUNCH_PDL(kernel, grid, block, smem, stream, ...)                \
  SST_LAUNCH_PDL_B(0, kernel, grid, block, smem, stream, __VA_ARGS__)

template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t s, Args &&...args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  // an error is left for the caller's cudaGetLastError, as a <<<>>> launch
  (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// wait for the kernels this one was launched after (a no-op for a kernel
// launched without programmatic serialization)
__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

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
  void release() {
    if (base) cudaFree(base);
    base = nullptr;
    cap = used = 0;
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

constexpr int kScanThreads = 256;
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

// Multi-tile scans run as two launches over kScanRanges contiguous tile
// ranges (about four blocks per SM): the first reduces each range, the
// second has every block fold the range sums before its own and then scan
// its range tile by tile with a running carry.  No block waits on another.
constexpr int kScanRanges = 608;
// scans of at most this many tiles (32K elements) run as one block
constexpr uint64_t kScanOneBlockTiles = 8;
// single-pass (look-back) scans up to this many tiles (4M elements)
constexpr uint64_t kScanLookbackTiles = 1024;

// A tile's results leave through shared memory (its inputs arrive the same
// way, load_tile below): each thread holds items
// t*kScanItems .. +kScanItems-1 of the tile, which it writes to a padded
// buffer (stride kScanItems+1, no bank conflicts for 4-byte elements), and
// the block then stores the tile striped, so each store instruction writes
// whole sectors.
// A scan's results go to an epilogue: epi(i, r) for element i (its index
// in the array, whatever the scan direction) and its result r.  StoreOut
// writes them out; a fused consumer (the update pipeline's compactions)
// uses them in place, saving the launch that would read them back.
template <typename T>
struct StoreOut {
  T *out;
  __device__ __forceinline__ void operator()(uint64_t i, T r) const { out[i] = r; }
};

// tile t of the scan order: element i of the array (forward or reversed)
template <typename T>
__device__ __forceinline__ T scan_load(const T *in, uint64_t i, uint64_t n,
                                       bool reverse, T identity) {
  return i < n ? in[reverse ? n - 1 - i : i] : identity;
}

// The tile's padded staging buffer (shared by its load and its store).
template <typename T>
__device__ __forceinline__ T *tile_sbuf() {
  __shared__ T sbuf[kScanThreads * (kScanItems + 1)];
  return sbuf;
}

// A tile's inputs arrive the same way in reverse: the block loads the tile
// striped (each load instruction reads whole sectors), into the padded
// buffer, and each thread then takes its kScanItems consecutive items.
template <typename T>
__device__ __forceinline__ void load_tile(const T *in, uint64_t base, uint64_t n,
                                          bool reverse, T identity, T *vals) {
  T *sbuf = tile_sbuf<T>();
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint32_t e = (uint32_t)k * kScanThreads + threadIdx.x;
    sbuf[(e / kScanItems) * (kScanItems + 1) + e % kScanItems] =
        scan_load(in, base + e, n, reverse, identity);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanItems; k++) vals[k] = sbuf[threadIdx.x * (kScanItems + 1) + k];
  __syncthreads();  // the buffer is free again
}

template <typename T, typename Epi>
__device__ __forceinline__ void store_tile(const Epi &epi, uint64_t base, uint64_t n,
                                           bool reverse, const T *vals) {
  T *sbuf = tile_sbuf<T>();
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    sbuf[threadIdx.x * (kScanItems + 1) + k] = vals[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const uint32_t e = (uint32_t)k * kScanThreads + threadIdx.x;
    const uint64_t i = base + e;
    if (i < n)
      epi(reverse ? n - 1 - i : i,
          sbuf[(e / kScanItems) * (kScanItems + 1) + e % kScanItems]);
  }
  __syncthreads();
}


template <typename T, typename Op>
__global__ void k_scan_reduce(const T *__restrict__ in, uint64_t n, T identity,
                              Op op, bool reverse, uint64_t tiles_per_range,
                              T *__restrict__ range_sums,
                              const uint32_t *__restrict__ d_n) {
  pdl_wait();
  if (d_n && *d_n < n) n = *d_n;
  const uint64_t t0 = (uint64_t)blockIdx.x * tiles_per_range;
  T acc = identity;
  for (uint64_t t = t0; t < t0 + tiles_per_range; t++) {
    const uint64_t base = t * kScanTile;
    if (base >= n) break;
    // order inside a range does not matter for the total: striped loads
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
      acc = op(acc, scan_load(in, base + (uint64_t)k * kScanThreads + threadIdx.x,
                              n, reverse, identity));
  }
  T total;
  block_exclusive(acc, identity, op, &total);
  if (threadIdx.x == 0) range_sums[blockIdx.x] = total;
}

template <typename T, typename Op, typename Epi = StoreOut<T>>
__global__ void k_scan_ranges(const T *__restrict__ in, Epi out,
                              uint64_t n, T identity, Op op, bool reverse,
                              bool exclusive, uint64_t tiles_per_range,
                              const T *__restrict__ range_sums,
                              T *__restrict__ total_out,
                              const uint32_t *__restrict__ d_n) {
  pdl_wait();
  if (d_n && *d_n < n) n = *d_n;
  __shared__ T s_carry;
  // carry into this range: the sums of the ranges before it
  {
    T a = identity;
    for (uint32_t r = threadIdx.x; r < blockIdx.x; r += kScanThreads)
      a = op(a, range_sums[r]);
    T tot;
    block_exclusive(a, identity, op, &tot);
    if (threadIdx.x == 0) s_carry = tot;
    __syncthreads();
  }
  T carry = s_carry;
  const uint64_t t0 = (uint64_t)blockIdx.x * tiles_per_range;
  for (uint64_t t = t0; t < t0 + tiles_per_range; t++) {
    const uint64_t base = t * kScanTile;
    if (base >= n) break;
    T vals[kScanItems];
    load_tile(in, base, n, reverse, identity, vals);
    T acc = identity;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) acc = op(acc, vals[k]);
    T total;
    T run = op(carry, block_exclusive(acc, identity, op, &total));
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
      T nxt = op(run, vals[k]);
      vals[k] = exclusive ? run : nxt;
      run = nxt;
    }
    store_tile(out, base, n, reverse, vals);
    carry = op(carry, total);
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
    *total_out = carry;
}

// one-tile scan (n <= kScanTile)
template <typename T, typename Op, typename Epi = StoreOut<T>>
__global__ void k_scan_tile(const T *__restrict__ in, Epi out,
                            uint64_t n, T identity, Op op, bool reverse,
                            bool exclusive, T *__restrict__ total_out,
                            const uint32_t *__restrict__ d_n) {
  pdl_wait();
  if (d_n && *d_n < n) n = *d_n;
  T vals[kScanItems];
  load_tile(in, 0, n, reverse, identity, vals);
  T acc = identity;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) acc = op(acc, vals[k]);
  T total;
  T run = block_exclusive(acc, identity, op, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    T nxt = op(run, vals[k]);
    vals[k] = exclusive ? run : nxt;
    run = nxt;
  }
  store_tile(out, 0, n, reverse, vals);
  if (total_out && threadIdx.x == 0) *total_out = total;
}

// ------------------------------------------------- single-pass scan
// Status of one tile of the single-pass scan.  flag = tag | state, where the
// tag (kScanTag | epoch << 2) is unique to the launch: a flag left in the
// same memory by an earlier launch, or by whatever the arena held there
// before, never matches.  State 1: agg holds the tile's reduction; state 2:
// incl holds the reduction of every tile up to and including this one.
// The two values sit in separate fields, so a reader that saw state 1 reads
// an aggregate that is never overwritten.
template <typename T>
struct ScanStatus {
  unsigned long long flag;
  T agg;
  T incl;
};
constexpr unsigned long long kScanTag = 0x5CA5ull << 48;
// scans a captured sequence may tag per device epoch (DeviceScanTags)
constexpr uint32_t kScanTagsPerEpoch = 64;
constexpr unsigned long long kScanEpochMask = (1ull << 46) - 1;
// polls of one predecessor's flag (with a growing sleep) before a tile stops
// waiting and reduces the inputs of the tiles it still lacks itself
constexpr int kLookbackPolls = 1 << 13;

template <typename T>
__device__ __forceinline__ void scan_publish(ScanStatus<T> *s,
                                             unsigned long long tag, int state,
                                             T v) {
  if (state == 1)
    *(volatile T *)&s->agg = v;
  else
    *(volatile T *)&s->incl = v;
  __threadfence();
  *(volatile unsigned long long *)&s->flag = tag | (unsigned long long)state;
}

template <typename T, typename Op>
__device__ __forceinline__ T warp_reduce_all(T v, Op op) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, d));
  return v;
}

// The reduction of tiles 0 .. tile-1, by the whole block of tile `tile`
// (> 0).  Each round thread k reads the flag of the tile k + 1 below the
// nearest tile not folded in yet, and the block folds every tile down to the
// nearest inclusive prefix (or all 256 when there is none and goes on).
// Every wait is bounded: if a predecessor that is needed has not published
// in time, the block reduces the inputs of tiles 0 .. j itself (the scan is
// out of place, so the inputs are intact).
template <typename T, typename Op>
__device__ T scan_lookback(const ScanStatus<T> *st, uint64_t tile,
                           unsigned long long tag, T identity, Op op,
                           const T *in, uint64_t n, bool reverse, int polls) {
  __shared__ int s_stop, s_fail;
  __shared__ T s_part[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T excl = identity;
  int64_t j = (int64_t)tile - 1;  // nearest tile not folded in yet
  for (;;) {
    if (threadIdx.x == 0) {
      s_stop = kScanThreads;
      s_fail = kScanThreads;
    }
    const int64_t t = j - (int64_t)threadIdx.x;
    // tiles below tile 0 act as an empty inclusive prefix
    unsigned long long f = tag | 2ull;
    if (t >= 0) {
      f = 0;  // polls == 0: treated as never published
      for (int p = 0; p < polls; p++) {
        const unsigned long long x = *(volatile const unsigned long long *)&st[t].flag;
        if ((x & ~3ull) == tag && (x & 3ull) != 0) {
          f = x;
          break;
        }
        __nanosleep(p < 64 ? 32 : 512);
      }
    }
    __syncthreads();  // s_stop / s_fail set
    if ((f & 3ull) == 2ull) atomicMin(&s_stop, (int)threadIdx.x);
    if (f == 0) atomicMin(&s_fail, (int)threadIdx.x);
    __syncthreads();
    const int stop = s_stop, fail = s_fail;
    if (fail <= stop && fail < kScanThreads) {
      // a needed predecessor never published: reduce its inputs and all below
      T a = identity;
      const uint64_t end = (uint64_t)(j + 1) * kScanTile;
      for (uint64_t i = threadIdx.x; i < end; i += kScanThreads)
        a = op(a, scan_load(in, i, n, reverse, identity));
      a = warp_reduce_all(a, op);
      if (lane == 0) s_part[warp] = a;
      __syncthreads();
      T r = identity;
#pragma unroll
      for (int w = 0; w < kScanThreads / 32; w++) r = op(r, s_part[w]);
      return op(r, excl);
    }
    __threadfence();
    T v = identity;
    if ((int)threadIdx.x <= stop && t >= 0)
      v = (int)threadIdx.x == stop ? *(volatile const T *)&st[t].incl
                                   : *(volatile const T *)&st[t].agg;
    v = warp_reduce_all(v, op);
    if (lane == 0) s_part[warp] = v;
    __syncthreads();
    T r = identity;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; w++) r = op(r, s_part[w]);
    excl = op(r, excl);
    if (stop < kScanThreads) return excl;
    j -= kScanThreads;
    __syncthreads();  // s_part read by every thread before the next round
  }
}

// Single-pass scan (out of place): block b scans tile b, publishes its
// aggregate, looks back for its prefix and publishes its inclusive prefix.
// Tile b waits only on the aggregates of tiles below it, which the hardware
// starts first and which depend on nothing.
template <typename T, typename Op, typename Epi = StoreOut<T>>
__global__ void __launch_bounds__(kScanThreads)
k_scan_lb(const T *__restrict__ in, Epi out, uint64_t n,
          T identity, Op op, bool reverse, bool exclusive,
          T *__restrict__ total_out, const uint32_t *__restrict__ d_n,
          ScanStatus<T> *st, unsigned long long tag, int polls,
          const unsigned long long *__restrict__ d_epoch) {
  pdl_wait();
  if (d_epoch)  // the epoch is written before this launch, in stream order
    tag = kScanTag |
          (((*d_epoch * kScanTagsPerEpoch + (tag & 0xFF)) & kScanEpochMask) << 2);
  if (d_n && *d_n < n) n = *d_n;
  const uint64_t tile = blockIdx.x, base = tile * kScanTile;
  if (base >= n) {
    if (tile == 0 && total_out && threadIdx.x == 0) *total_out = identity;
    return;
  }
  T vals[kScanItems];
  load_tile(in, base, n, reverse, identity, vals);
  T acc = identity;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) acc = op(acc, vals[k]);
  T total;
  T run = block_exclusive(acc, identity, op, &total);
  T carry = identity;
  if (tile == 0) {
    if (threadIdx.x == 0) scan_publish(&st[0], tag, 2, total);
  } else {
    if (threadIdx.x == 0) scan_publish(&st[tile], tag, 1, total);
    carry = scan_lookback(st, tile, tag, identity, op, in, n, reverse, polls);
    if (threadIdx.x == 0) scan_publish(&st[tile], tag, 2, op(carry, total));
  }
  run = op(carry, run);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    T nxt = op(run, vals[k]);
    vals[k] = exclusive ? run : nxt;
    run = nxt;
  }
  store_tile(out, base, n, reverse, vals);
  if (total_out && threadIdx.x == 0 && n - base <= (uint64_t)kScanTile)
    *total_out = op(carry, total);
}

// While alive, scans launched from this thread take the forms a stream
// capture would (no per-launch tag): kernels launched directly then match
// the ones a replayed capture runs, so they can be timed one by one.
extern thread_local bool t_capture_forms;
struct CaptureForms {
  bool prev;
  CaptureForms() : prev(t_capture_forms) { t_capture_forms = true; }
  ~CaptureForms() { t_capture_forms = prev; }
};

// Device-side scan tags, for single-pass scans that are captured into a
// CUDA graph (a tag fixed at capture would repeat in every replay).  While
// a DeviceScanTags is alive on a thread, the single-pass scans launched
// from it take their tag from a device epoch word instead of the host:
// bump() launches a one-thread kernel that advances the epoch (once per
// launched or replayed sequence, before its first scan), and the k-th scan
// after it tags its status words with (epoch * 64 + k), so no two scans of
// any two replays share a tag.
struct DeviceScanTags {
  unsigned long long *epoch = nullptr;  // device word
  uint32_t next = 0;                    // scans issued since bump()
  DeviceScanTags *prev = nullptr;
  explicit DeviceScanTags(unsigned long long *e);
  ~DeviceScanTags();
  cudaError_t bump(cudaStream_t s);
};
extern thread_local DeviceScanTags *t_scan_tags;

inline bool stream_capturing(cudaStream_t s) {
  if (t_capture_forms) return true;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    cudaGetLastError();
    return true;  // unknown: take the form that needs no per-launch tag
  }
  return cs != cudaStreamCaptureStatusNone;
}

// Scan of n elements whose results go to the epilogue epi (StoreOut for a
// plain scan; see store_tile).  total_out (device, may be null) receives the
// reduction of all n elements.  With d_n (device, may be null) only the first
// min(n, *d_n) elements are scanned; n sizes the launch.  in_place: the
// epilogue writes the input array (the single-pass form, whose bounded
// look-back may reread inputs, is not used then).
template <typename T, typename Op, typename Epi>
cudaError_t scan_epi(const T *in, uint64_t n, T identity, Op op, bool exclusive,
                     bool reverse, T *total_out, Arena &arena, cudaStream_t s,
                     const uint32_t *d_n, Epi epi, bool in_place) {
  if (n == 0) {
    if (total_out) return cudaMemcpyAsync(total_out, &identity, sizeof(T),
                                          cudaMemcpyHostToDevice, s);
    return cudaSuccess;
  }
  const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    SST_LAUNCH_PDL_B(2 * sizeof(T) * n, (k_scan_tile<T, Op, Epi>), 1, kScanThreads, 0, s,
                 in, epi, n, identity, op, reverse, exclusive, total_out, d_n);
    return cudaGetLastError();
  }
  // one launch with look-back, unless the scan is in place (the bounded
  // look-back's fallback rereads inputs), being captured into a graph (a
  // replay would reuse the launch's tag) or longer than kScanLookbackTiles
  // (past 256 tiles a look-back takes several rounds, and past about 1024
  // the two-launch form is faster)
  DeviceScanTags *dt = t_scan_tags;
  const bool dev_tags = dt && dt->epoch && dt->next < kScanTagsPerEpoch;
  if (!in_place && tiles <= kScanLookbackTiles && (dev_tags || !stream_capturing(s))) {
    ScanStatus<T> *st = arena.take<ScanStatus<T>>(tiles);
    if (st) {
      // a scan whose element count is on the device (d_n) is profiled
      // apart, with no declared bytes: its launch size overstates its work
      const unsigned long long tag = dev_tags ? (unsigned long long)dt->next++ : next_scan_tag();
      SST_LAUNCH_PDL_NB(d_n ? "(k_scan_lb<T, Op, Epi>, device count)" : "(k_scan_lb<T, Op, Epi>)",
                    d_n ? 0 : 2 * sizeof(T) * n, (k_scan_lb<T, Op, Epi>), (unsigned)tiles,
                    kScanThreads, 0, s, in, epi, n, identity, op, reverse,
                    exclusive, total_out, d_n, st, tag, lookback_polls(),
                    dev_tags ? (const unsigned long long *)dt->epoch : nullptr);
      return cudaGetLastError();
    }
  }
  if (tiles <= kScanOneBlockTiles) {
    // one block walks the tiles with a running carry: one launch, where the
    // two-launch form would pay a second launch's latency for little work
    SST_LAUNCH_PDL_B(2 * sizeof(T) * n, (k_scan_ranges<T, Op, Epi>), 1, kScanThreads, 0,
                 s, in, epi, n, identity, op, reverse, exclusive, tiles,
                 (const T *)nullptr, total_out, d_n);
    return cudaGetLastError();
  }
  const uint64_t ranges = tiles < (uint64_t)kScanRanges ? tiles : (uint64_t)kScanRanges;
  const uint64_t per = (tiles + ranges - 1) / ranges;
  const uint64_t used = (tiles + per - 1) / per;
  T *sums = arena.take<T>(used);
  if (!sums) return cudaErrorMemoryAllocation;
  // the reduce reads the input; the scan reads it again and writes the output
  SST_LAUNCH_PDL_B(sizeof(T) * n, (k_scan_reduce<T, Op>), (unsigned)used, kScanThreads,
               0, s, in, n, identity, op, reverse, per, sums, d_n);
  SST_LAUNCH_PDL_B(2 * sizeof(T) * n, (k_scan_ranges<T, Op, Epi>), (unsigned)used,
               kScanThreads, 0, s, in, epi, n, identity, op, reverse, exclusive,
               per, (const T *)sums, total_out, d_n);
  return cudaGetLastError();
}

// Scan of n elements into out (in may equal out).
template <typename T, typename Op>
cudaError_t scan(const T *in, T *out, uint64_t n, T identity, Op op,
                 bool exclusive, bool reverse, T *total_out, Arena &arena,
                 cudaStream_t s, const uint32_t *d_n = nullptr) {
  return scan_epi<T, Op, StoreOut<T>>(in, n, identity, op, exclusive, reverse, total_out,
                                      arena, s, d_n, StoreOut<T>{out}, in == out);
}

// scratch bytes a scan of n elements of T takes from the arena: the tile
// status of the single-pass form (8 + 2 * elem bytes a tile), else the range
// sums of the two-launch form
inline size_t scan_scratch_bytes(uint64_t n, size_t elem) {
  const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  const size_t st = (tiles * (8 + 2 * elem) + 255) & ~size_t(255);
  const size_t rs = ((kScanRanges * elem + 255) & ~size_t(255)) + 256;
  return st > rs ? st : rs;
}

// ----------------------------------------------------------- radix sort
// Stable LSD radix sort of 64-bit keys on their low `bits` bits, 8-bit
// digits.  keys and tmp are both n long; *result points at whichever holds
// the sorted keys.  Batches up to kSmallSort keys sort in one CTA (up to
// 1024 keys by radix passes, more by a bitonic network).
constexpr int kSmallSort = 2048;
// the same with a 32-bit payload per key moved along (stable)
cudaError_t radix_sort_kv(uint64_t *keys, uint64_t *tmp, uint32_t *vals,
                          uint32_t *vtmp, uint64_t n, int bits, Arena &arena,
                          cudaStream_t s, uint64_t **result, uint32_t **vresult);
// d_n (device, may be null): sort only the first min(n, *d_n) keys; n sizes
// the launches, the rest of the arrays is left as it was
// The digit counts of the one-sweep form (key-only sorts of more than
// kSmallSort keys), when the caller produces them: every pass's 256 digit
// totals of the keys (zero before the keys are counted) and the passes'
// tile status words (cleared).  The update pipeline's key build counts the
// digits of the keys it writes, so the sort skips its own counting read.
struct SortDigits {
  uint32_t *totals = nullptr;  // passes x 256
  uint32_t *status = nullptr;  // status_words
  uint64_t status_words = 0;
  int passes = 0;
};
// whether radix_sort_u64 of n keys on `bits` bits takes the one-sweep form;
// if so, its digit tables are taken from the arena into *d (call it where
// the sort would take them: before the sort's other scratch)
bool radix_sort_digits(uint64_t n, int bits, Arena &arena, SortDigits *d);
cudaError_t radix_sort_u64(uint64_t *keys, uint64_t *tmp, uint64_t n, int bits,
                           Arena &arena, cudaStream_t s, uint64_t **result,
                           const uint32_t *d_n = nullptr,
                           const SortDigits *pre = nullptr);
size_t radix_sort_scratch_bytes(uint64_t n);

}  // namespace sst

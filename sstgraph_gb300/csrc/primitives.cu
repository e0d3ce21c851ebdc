// Stable LSD radix sort of 64-bit keys (8-bit digits) and the launch
// counter.  Each pass: per-tile digit histograms, one exclusive scan over
// (digit, tile), then a stable scatter that ranks equal digits with
// warp match_any + per-warp prefix counts in shared memory.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "primitives.cuh"

namespace sst {

static std::atomic<uint64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(int64_t k) {
  g_launches.fetch_add((uint64_t)k, std::memory_order_relaxed);
}
uint64_t launches() { return g_launches.load(std::memory_order_relaxed); }

// ------------------------------------------------------------- profiler
namespace {
struct Pending {
  const char *name;
  cudaEvent_t a, b;
  uint64_t bytes;
};
struct Totals {
  uint64_t launches = 0;
  double ms = 0;
  uint64_t bytes = 0;  // declared algorithmic bytes (0 where undeclared)
};
std::mutex g_prof_mu;
bool g_prof_on = false;
std::vector<cudaEvent_t> g_pool;
std::vector<Pending> g_pending;
std::map<std::string, Totals> g_totals;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// fold finished pairs into the totals (caller holds the lock)
void drain(bool wait) {
  size_t keep = 0;
  for (size_t i = 0; i < g_pending.size(); i++) {
    Pending &p = g_pending[i];
    if (wait) cudaEventSynchronize(p.b);
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      Totals &t = g_totals[p.name];
      t.launches++;
      t.ms += ms;
      t.bytes += p.bytes;
      g_pool.push_back(p.a);
      g_pool.push_back(p.b);
    } else {
      cudaGetLastError();
      g_pending[keep++] = p;
    }
  }
  g_pending.resize(keep);
}
}  // namespace

std::string g_prof_filter;  // profile only kernels whose name contains it

bool profiling(const char *name) {
  if (!g_prof_on) return false;
  return g_prof_filter.empty() || strstr(name, g_prof_filter.c_str()) != nullptr;
}

cudaEvent_t prof_begin(cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaEvent_t e = take_event();
  cudaEventRecord(e, s);
  return e;
}

void prof_end(const char *name, cudaEvent_t start, cudaStream_t s,
              uint64_t bytes) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaEvent_t e = take_event();
  cudaEventRecord(e, s);
  g_pending.push_back({name, start, e, bytes});
  if (g_pending.size() > 4096) drain(false);
}

void profile_start(const char *filter) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  drain(true);
  g_totals.clear();
  g_prof_filter = filter ? filter : "";
  g_prof_on = true;
}

// JSON object {"kernel": {"launches": L, "ms": T}, ...}; stops profiling
std::string profile_collect() {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_on = false;
  drain(true);
  std::string out = "{";
  bool first = true;
  for (auto &kv : g_totals) {
    char buf[256];
    snprintf(buf, sizeof(buf),
             "%s\"%s\": {\"launches\": %llu, \"ms\": %.6f, \"bytes\": %llu}",
             first ? "" : ", ", kv.first.c_str(),
             (unsigned long long)kv.second.launches, kv.second.ms,
             (unsigned long long)kv.second.bytes);
    out += buf;
    first = false;
  }
  out += "}";
  g_totals.clear();
  return out;
}

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // 4096
constexpr int kRadix = 256;

// Stable ranking of one iteration's 256 keys (one per thread, in index
// order).  run[d] holds the next output position for digit d and is
// advanced.  Returns the output position of this thread's key.
__device__ __forceinline__ uint32_t rank_iteration(uint32_t d, bool valid,
                                                   uint32_t (*wcnt)[kRadix],
                                                   uint32_t *run) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < kWarps; w++) wcnt[w][threadIdx.x] = 0;
  __syncthreads();
  uint32_t key = valid ? d : 0xffffffffu;
  uint32_t peers = __match_any_sync(0xffffffffu, key);
  uint32_t lt = peers & ((1u << lane) - 1u);
  if (valid && lt == 0) wcnt[warp][d] = __popc(peers);
  __syncthreads();
  {
    uint32_t s = run[threadIdx.x];
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      uint32_t c = wcnt[w][threadIdx.x];
      wcnt[w][threadIdx.x] = s;
      s += c;
    }
    run[threadIdx.x] = s;
  }
  __syncthreads();
  uint32_t pos = valid ? wcnt[warp][d] + __popc(lt) : 0;
  __syncthreads();
  return pos;
}

__global__ void k_hist(const uint64_t *__restrict__ keys, uint64_t n, int shift,
                       uint32_t *__restrict__ hist, uint32_t nblocks) {
  __shared__ uint32_t h[kRadix];
  h[threadIdx.x] = 0;
  __syncthreads();
  uint64_t t0 = (uint64_t)blockIdx.x * kTile;
#pragma unroll 4
  for (int it = 0; it < kItems; it++) {
    uint64_t i = t0 + (uint64_t)it * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xff], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Scatter of one pass; with hist_next it also counts the next pass's digit
// of every key in the tile the key lands in (hist_next zeroed beforehand),
// so the next pass needs no histogram launch.
__global__ void k_scatter(const uint64_t *__restrict__ in,
                          uint64_t *__restrict__ out, uint64_t n, int shift,
                          const uint32_t *__restrict__ hist, uint32_t nblocks,
                          const uint32_t *__restrict__ vin,
                          uint32_t *__restrict__ vout,
                          uint32_t *__restrict__ hist_next, int next_shift) {
  __shared__ uint32_t wcnt[kWarps][kRadix];
  __shared__ uint32_t run[kRadix];
  run[threadIdx.x] = hist[(uint64_t)threadIdx.x * nblocks + blockIdx.x];
  // the tile's keys (and values) come in at once, ahead of the ranking
  // rounds, so the rounds do not wait on memory
  const uint64_t t0 = (uint64_t)blockIdx.x * kTile;
  uint64_t kk[kItems];
  uint32_t vv[kItems];
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    uint64_t i = t0 + (uint64_t)it * kThreads + threadIdx.x;
    kk[it] = i < n ? in[i] : 0;
    vv[it] = (vin && i < n) ? vin[i] : 0u;
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    uint64_t i = t0 + (uint64_t)it * kThreads + threadIdx.x;
    bool valid = i < n;
    uint32_t d = (uint32_t)(kk[it] >> shift) & 0xff;
    uint32_t pos = rank_iteration(d, valid, wcnt, run);
    if (valid) {
      out[pos] = kk[it];
      if (vin) vout[pos] = vv[it];
      if (hist_next)
        atomicAdd(&hist_next[(uint64_t)((kk[it] >> next_shift) & 0xff) * nblocks +
                             pos / kTile],
                  1u);
    }
  }
}

// whole sort in one CTA for n <= TILE: keys (and payloads) staged in shared
// memory
template <bool KV, int TILE>
__global__ void k_sort_small(uint64_t *__restrict__ keys,
                             uint32_t *__restrict__ vals, uint64_t n, int bits) {
  __shared__ uint64_t buf[2][TILE];
  __shared__ uint32_t vbuf[KV ? 2 : 1][KV ? TILE : 1];
  __shared__ uint32_t wcnt[kWarps][kRadix];
  __shared__ uint32_t run[kRadix];
  __shared__ uint32_t h[kRadix];
  for (uint64_t i = threadIdx.x; i < n; i += kThreads) {
    buf[0][i] = keys[i];
    if (KV) vbuf[0][i] = vals[i];
  }
  int cur = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    h[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t i = threadIdx.x; i < n; i += kThreads)
      atomicAdd(&h[(buf[cur][i] >> shift) & 0xff], 1u);
    __syncthreads();
    if (threadIdx.x < 32) {
      // exclusive scan of 256 bins by one warp, 8 bins per lane
      uint32_t loc[8], s = 0;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        loc[j] = s;
        s += h[threadIdx.x * 8 + j];
      }
      uint32_t inc = s;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, inc, d);
        if ((int)threadIdx.x >= d) inc += o;
      }
      uint32_t excl = inc - s;
#pragma unroll
      for (int j = 0; j < 8; j++) run[threadIdx.x * 8 + j] = excl + loc[j];
    }
    __syncthreads();
    int iters = (int)((n + kThreads - 1) / kThreads);
    for (int it = 0; it < iters; it++) {
      uint64_t i = (uint64_t)it * kThreads + threadIdx.x;
      bool valid = i < n;
      uint64_t k = valid ? buf[cur][i] : 0;
      uint32_t d = (uint32_t)(k >> shift) & 0xff;
      uint32_t pos = rank_iteration(d, valid, wcnt, run);
      if (valid) {
        buf[cur ^ 1][pos] = k;
        if (KV) vbuf[cur ^ 1][pos] = vbuf[cur][i];
      }
    }
    __syncthreads();
    cur ^= 1;
  }
  for (uint64_t i = threadIdx.x; i < n; i += kThreads) {
    keys[i] = buf[cur][i];
    if (KV) vals[i] = vbuf[cur][i];
  }
}

constexpr int kSmallSortKV = 1024;
constexpr uint32_t kFuseHistBlocks = 64;  // 256K keys

}  // namespace

size_t radix_sort_scratch_bytes(uint64_t n) {
  uint64_t nblocks = (n + kTile - 1) / kTile;
  uint64_t hn = nblocks * kRadix;
  return 2 * ((hn * 4 + 255) & ~size_t(255)) + scan_scratch_bytes(hn, 4) + 512;
}

static cudaError_t radix_sort_impl(uint64_t *keys, uint64_t *tmp,
                                   uint32_t *vals, uint32_t *vtmp, uint64_t n,
                                   int bits, Arena &arena, cudaStream_t s,
                                   uint64_t **result, uint32_t **vresult) {
  *result = keys;
  if (vresult) *vresult = vals;
  if (n < 2 || bits <= 0) return cudaSuccess;
  if (!vals && n <= (uint64_t)kSmallSort) {
    SST_LAUNCH_B(16 * n, (k_sort_small<false, kSmallSort>), 1, kThreads, 0, s, keys,
               (uint32_t *)nullptr, n, bits);
    return cudaGetLastError();
  }
  if (vals && n <= (uint64_t)kSmallSortKV) {
    SST_LAUNCH_B(24 * n, (k_sort_small<true, kSmallSortKV>), 1, kThreads, 0, s, keys, vals,
               n, bits);
    return cudaGetLastError();
  }
  uint32_t nblocks = (uint32_t)((n + kTile - 1) / kTile);
  uint64_t hn = (uint64_t)nblocks * kRadix;
  // digit-major tile histograms of this pass and the next (ping-pong)
  uint32_t *hist = arena.take<uint32_t>(hn);
  uint32_t *hnext = arena.take<uint32_t>(hn);
  if (!hist || !hnext) return cudaErrorMemoryAllocation;
  uint64_t *src = keys, *dst = tmp;
  uint32_t *vsrc = vals, *vdst = vtmp;
  // the first pass's histogram reads the keys; every scatter reads and
  // writes keys (and values) and touches the tile-digit tables
  const uint64_t hist_bytes = 8 * n + 4 * hn;
  const uint64_t scatter_bytes = (vals ? 24 : 16) * n + 8 * hn;
  SST_LAUNCH_B(hist_bytes, k_hist, nblocks, kThreads, 0, s, src, n, 0, hist, nblocks);
  for (int shift = 0; shift < bits; shift += 8) {
    size_t mark = arena.used;
    cudaError_t e = scan<uint32_t, OpAdd>(hist, hist, hn, 0u, OpAdd{}, true,
                                          false, nullptr, arena, s);
    arena.used = mark;
    if (e != cudaSuccess) return e;
    // the next pass's histogram rides on this scatter only for small sorts:
    // on large ones every block's keys of one digit land in the same one or
    // two destination tiles, and the atomics on those counters serialise
    const bool more = shift + 8 < bits;
    const bool fuse = more && nblocks <= kFuseHistBlocks;
    if (fuse) {
      e = cudaMemsetAsync(hnext, 0, hn * 4, s);
      if (e != cudaSuccess) return e;
    }
    SST_LAUNCH_B(scatter_bytes, k_scatter, nblocks, kThreads, 0, s, src, dst, n,
                 shift, hist, nblocks, vsrc, vdst, fuse ? hnext : nullptr,
                 shift + 8);
    std::swap(src, dst);
    std::swap(vsrc, vdst);
    // unfused: the next pass's histogram over this pass's output
    if (more && !fuse)
      SST_LAUNCH_B(hist_bytes, k_hist, nblocks, kThreads, 0, s, src, n, shift + 8,
                   hnext, nblocks);
    std::swap(hist, hnext);
  }
  *result = src;
  if (vresult) *vresult = vsrc;
  return cudaGetLastError();
}

cudaError_t radix_sort_u64(uint64_t *keys, uint64_t *tmp, uint64_t n, int bits,
                           Arena &arena, cudaStream_t s, uint64_t **result) {
  return radix_sort_impl(keys, tmp, nullptr, nullptr, n, bits, arena, s, result,
                         nullptr);
}

cudaError_t radix_sort_kv(uint64_t *keys, uint64_t *tmp, uint32_t *vals,
                          uint32_t *vtmp, uint64_t n, int bits, Arena &arena,
                          cudaStream_t s, uint64_t **result, uint32_t **vresult) {
  return radix_sort_impl(keys, tmp, vals, vtmp, n, bits, arena, s, result,
                         vresult);
}

}  // namespace sst

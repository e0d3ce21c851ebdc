// Stable LSD radix sort of 64-bit keys (8-bit digits) and the launch
// counter.  Each pass: per-tile digit counts, their exclusive scan over
// (digit, tile), then a stable scatter in which every warp ranks its own
// contiguous slice of the tile (a digit match from ballots, warp-private
// counters), the tile is reordered in shared memory and leaves in runs of
// one digit.  Sorts of up to 256 tiles fold the scan and the next pass's
// counts into the scatter: one launch a pass.
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

static std::atomic<unsigned long long> g_scan_epoch{0};
unsigned long long next_scan_tag() {
  const unsigned long long e =
      (g_scan_epoch.fetch_add(1, std::memory_order_relaxed) + 1) & kScanEpochMask;
  return kScanTag | (e << 2);
}

thread_local bool t_capture_forms = false;
thread_local DeviceScanTags *t_scan_tags = nullptr;

namespace {
__global__ void k_scan_epoch_bump(unsigned long long *epoch) {
  pdl_wait(); *epoch += 1; }
}  // namespace

DeviceScanTags::DeviceScanTags(unsigned long long *e) : epoch(e), prev(t_scan_tags) {
  t_scan_tags = this;  // with a null epoch: host tags, as without one
}
DeviceScanTags::~DeviceScanTags() { t_scan_tags = prev; }
cudaError_t DeviceScanTags::bump(cudaStream_t s) {
  next = 0;
  SST_LAUNCH_PDL(k_scan_epoch_bump, 1, 1, 0, s, epoch);
  return cudaGetLastError();
}

static std::atomic<int> g_lookback_polls{kLookbackPolls};
int lookback_polls() { return g_lookback_polls.load(std::memory_order_relaxed); }
void set_lookback_polls(int polls) {
  g_lookback_polls.store(polls < 0 ? 0 : polls, std::memory_order_relaxed);
}

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

static thread_local bool t_prof_paused = false;
ProfPause::ProfPause() : prev(t_prof_paused) { t_prof_paused = true; }
ProfPause::~ProfPause() { t_prof_paused = prev; }

bool profiling(const char *name) {
  if (!g_prof_on || t_prof_paused) return false;
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
// Sorts of at most kSmallTileKeys keys (without values) use tiles of
// kSmallItems items per thread: four times the blocks, each ranking a
// quarter of the keys, so a pass's dependent chain is shorter.
constexpr int kSmallItems = 4;
constexpr uint64_t kSmallTileKeys = 256ull * kThreads * kSmallItems;  // 2^18
// (1024-key tiles for larger one-sweep sorts were measured too: at 1e6 keys
// 977 tiles made a pass 29 us against 19 us for 245 tiles of 4096 -- the
// longer look-back walks cost more than the extra resident warps gain; and
// 2048-key tiles, three blocks an SM, made a 1e6-pair insert 567 us against
// 553 us; measured again with the match-word ranking: 21.3 against 17.8 us a
// pass)
constexpr int kRadix = 256;
constexpr uint32_t kNoDigit = 0xffffffffu;  // an item past the end
// Sorts of at most this many tiles run one launch per pass: every block
// prefixes the raw tile counts itself (reading all of them: the cost grows
// with the square of the tiles) and counts the next pass's digits as it
// scatters.  Larger sorts count and scan in separate launches.
constexpr uint32_t kFuseHistBlocks = 256;  // 1M keys

// Offset of this thread's item `it` in a warp-contiguous tile of ITEMS items
// per thread: warp w owns [w * ITEMS * 32, (w + 1) * ITEMS * 32), item it of
// lane l sits at w * ITEMS * 32 + it * 32 + l.  Loads stay coalesced, and a
// warp's items in (it, lane) order are in index order, so a warp ranks its
// own items without the rest of the block.
template <int ITEMS>
__device__ __forceinline__ uint32_t tile_offset(int it) {
  return (threadIdx.x >> 5) * (ITEMS * 32) + it * 32 + (threadIdx.x & 31);
}

// Stable rank of each of the warp's items among the warp's earlier items of
// the same digit.  The lanes holding one digit find each other through a
// warp-private word per digit in shared memory: each sets its bit with an
// atomic OR and reads the word back (far fewer instructions than eight
// ballots, one per digit bit, or __match_any_sync); the lowest of them then
// advances the digit's counter and clears the word.  wc (the warp's 256
// counters) and wm (its 256 match words) are zero and visible to the warp
// on entry; wc ends as the warp's count of each digit, wm zero again.  Items
// past the end carry kNoDigit.
template <int ITEMS>
__device__ __forceinline__ void warp_rank(const uint32_t (&dg)[ITEMS],
                                          uint32_t (&lr)[ITEMS], uint32_t *wc,
                                          uint32_t *wm) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t below = (1u << lane) - 1u;
#pragma unroll
  for (int it = 0; it < ITEMS; it++) {
    const uint32_t d = dg[it];
    const bool valid = d != kNoDigit;
    if (valid) atomicOr(&wm[d], 1u << lane);
    __syncwarp();
    const uint32_t peers = valid ? wm[d] : 0u;
    const uint32_t c = valid ? wc[d] : 0u;
    lr[it] = c + __popc(peers & below);
    __syncwarp();
    if (valid && (peers & below) == 0) {
      wc[d] = c + __popc(peers);
      wm[d] = 0;
    }
    __syncwarp();
  }
}
// a warp clears its 256 match words (then visible to the warp)
__device__ __forceinline__ void clear_match_words(uint32_t *wm) {
  const uint32_t lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < kRadix / 32; k++) wm[lane + 32 * k] = 0;
  __syncwarp();
}

// Exclusive scan of one value per thread over the block, in thread order
// (one __syncthreads inside).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint32_t off = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) off += w < warp ? wsum[w] : 0u;
  return off + inc - v;
}

// Per-tile digit counts at hist[d * dstride + tile * bstride]: digit-major
// (dstride = tiles, bstride = 1) for the scanned form, tile-major
// (dstride = 1, bstride = 256) for the fused one.  With `zero` the blocks
// also clear that table at the same indices.
template <int IT>
__global__ void __launch_bounds__(kThreads)
k_hist(const uint64_t *__restrict__ keys, uint64_t n, int shift,
       uint32_t *__restrict__ hist, uint32_t dstride, uint32_t bstride,
       uint32_t *__restrict__ zero, const uint32_t *__restrict__ d_n) {
  pdl_wait();
  if (d_n && *d_n < n) n = *d_n;
  __shared__ uint32_t h[kRadix];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * (kThreads * IT);
#pragma unroll 4
  for (int it = 0; it < IT; it++) {
    uint64_t i = t0 + (uint64_t)it * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xff], 1u);
  }
  __syncthreads();
  const uint64_t at = (uint64_t)threadIdx.x * dstride + (uint64_t)blockIdx.x * bstride;
  hist[at] = h[threadIdx.x];
  if (zero) zero[at] = 0;
}

// One pass's stable scatter of a tile.  The warps rank their slices, the
// tile is laid out in shared memory in (digit, index) order, and the block
// writes it out in that order, so the keys of one digit leave as one run of
// consecutive addresses (whole sectors, not one 8-byte write per lane).
//  raw: hist holds the raw tile-major counts (hist[tile * 256 + d]); every
//    block prefixes them itself (all digits below d over all tiles, plus
//    digit d over the tiles before its own), counts the next pass's digit
//    of each key into its destination tile's counter of hist_next (zero on
//    entry) and clears hist_zero (the counters of the pass after next).
//  otherwise: hist holds the scanned digit-major offsets.
// Dynamic shared memory: scatter_smem_bytes<KV, IT>(), IT items per thread.
// The staging area (keys and values of the tile) also holds the raw form's
// two [kWarps][kRadix] partial-sum tables before the ranking.
template <bool KV, int IT>
constexpr size_t scatter_stage_bytes() {
  return (size_t)kThreads * IT * (KV ? 12 : 8) > (size_t)2 * kWarps * kRadix * 4
             ? (size_t)kThreads * IT * (KV ? 12 : 8)
             : (size_t)2 * kWarps * kRadix * 4;
}
template <bool KV, int IT>
constexpr size_t scatter_smem_bytes() {
  return scatter_stage_bytes<KV, IT>() + (size_t)kWarps * kRadix * 4 + kRadix * 4 +
         kWarps * 4;
}

template <bool KV, int IT>
__global__ void __launch_bounds__(kThreads, 2)
k_scatter(const uint64_t *__restrict__ in, uint64_t *__restrict__ out,
          uint64_t n, int shift, const uint32_t *__restrict__ hist,
          uint32_t nblocks, bool raw, const uint32_t *__restrict__ vin,
          uint32_t *__restrict__ vout, uint32_t *__restrict__ hist_next,
          int next_shift, uint32_t *__restrict__ hist_zero,
          const uint32_t *__restrict__ d_n) {
  pdl_wait();
  constexpr int TILE = kThreads * IT;
  if (d_n && *d_n < n) n = *d_n;
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t *skeys = reinterpret_cast<uint64_t *>(smem);
  uint32_t *svals = reinterpret_cast<uint32_t *>(smem + (size_t)TILE * 8);
  uint32_t(*wcnt)[kRadix] = reinterpret_cast<uint32_t(*)[kRadix]>(
      smem + scatter_stage_bytes<KV, IT>());
  uint32_t *adj = &wcnt[kWarps - 1][kRadix - 1] + 1;  // [kRadix]
  uint32_t *wsum = adj + kRadix;                        // [kWarps]
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < kWarps; w++) wcnt[w][threadIdx.x] = 0;
  // the tile's keys (and values) come in at once, ahead of the ranking
  const uint64_t t0 = (uint64_t)blockIdx.x * TILE;
  uint64_t kk[IT];
  uint32_t vv[KV ? IT : 1];
  uint32_t dg[IT];
#pragma unroll
  for (int it = 0; it < IT; it++) {
    const uint64_t i = t0 + tile_offset<IT>(it);
    kk[it] = i < n ? in[i] : 0;
    if (KV) vv[it] = i < n ? vin[i] : 0u;
    dg[it] = i < n ? (uint32_t)(kk[it] >> shift) & 0xff : kNoDigit;
  }
  // gbase: output position of this tile's first key of digit threadIdx.x
  uint32_t gbase;
  if (raw) {
    // the tiles' counts summed by the block's warps: warp w takes every
    // kWarps-th tile row from w, each lane eight consecutive digits through
    // two 16-byte loads; the partial sums meet in shared memory (the key
    // staging area, unused until the write-out)
    const int lane = threadIdx.x & 31;
    uint32_t bef[8], tot[8];
#pragma unroll
    for (int k = 0; k < 8; k++) bef[k] = tot[k] = 0;
#pragma unroll 4
    for (uint32_t b = warp; b < nblocks; b += kWarps) {
      const uint4 *row = reinterpret_cast<const uint4 *>(hist + (uint64_t)b * kRadix) + lane * 2;
      const uint4 x0 = row[0], x1 = row[1];
      const uint32_t v[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
      const bool below = b < blockIdx.x;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        tot[k] += v[k];
        bef[k] += below ? v[k] : 0u;
      }
    }
    uint32_t *pb = reinterpret_cast<uint32_t *>(smem);  // [kWarps][kRadix]
    uint32_t *pt = pb + kWarps * kRadix;                // [kWarps][kRadix]
#pragma unroll
    for (int k = 0; k < 8; k++) {
      pb[warp * kRadix + lane * 8 + k] = bef[k];
      pt[warp * kRadix + lane * 8 + k] = tot[k];
    }
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      before += pb[w * kRadix + threadIdx.x];
      total += pt[w * kRadix + threadIdx.x];
    }
    gbase = block_excl_scan(total, wsum) + before;
  } else {
    gbase = hist[(uint64_t)threadIdx.x * nblocks + blockIdx.x];
    __syncthreads();
  }
  // the match words sit in the staging area, free until the reorder (the
  // raw form's partial-sum tables there are read: barrier above)
  uint32_t *wm = reinterpret_cast<uint32_t *>(smem) + warp * kRadix;
  clear_match_words(wm);
  uint32_t lr[IT];
  warp_rank<IT>(dg, lr, wcnt[warp], wm);
  __syncthreads();
  // tile-local start of each digit, then of each warp's share of it
  uint32_t tcount = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) tcount += wcnt[w][threadIdx.x];
  const uint32_t tstart = block_excl_scan(tcount, wsum);
  uint32_t s = tstart;
#pragma unroll
  for (int w = 0; w < kWarps; w++) {
    const uint32_t c = wcnt[w][threadIdx.x];
    wcnt[w][threadIdx.x] = s;
    s += c;
  }
  adj[threadIdx.x] = gbase - tstart;  // output position = adj[d] + local
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IT; it++) {
    if (dg[it] == kNoDigit) continue;
    const uint32_t lp = wcnt[warp][dg[it]] + lr[it];
    skeys[lp] = kk[it];
    if (KV) svals[lp] = vv[it];
  }
  __syncthreads();
  if (hist_zero) hist_zero[(uint64_t)blockIdx.x * kRadix + threadIdx.x] = 0;
  const uint32_t tn = t0 >= n ? 0u : (uint32_t)(n - t0 < (uint64_t)TILE ? n - t0 : TILE);
  for (uint32_t j = threadIdx.x; j < tn; j += kThreads) {
    const uint64_t key = skeys[j];
    const uint32_t pos = adj[(key >> shift) & 0xff] + j;
    out[pos] = key;
    if (KV) vout[pos] = svals[j];
    if (hist_next)
      atomicAdd(&hist_next[(uint64_t)(pos / TILE) * kRadix +
                           ((key >> next_shift) & 0xff)],
                1u);
  }
}

// ---- one-sweep passes (after Adinets and Merrill, "Onesweep", 2022).
// k_hist_all reads the keys once and counts every pass's digits (global
// totals, no per-tile tables) and clears the passes' tile status words.
// Each pass is then one launch: a block ranks its tile as k_scatter does,
// publishes its per-digit count, and thread d finds the count of digit d in
// all tiles before its own by looking back over their status words (an
// inclusive prefix ends the walk, an aggregate is added and the walk goes
// on).  A status word is (state << 30) | count, state 1 = this tile's
// count, 2 = the count of this and every earlier tile; 0 = not yet
// published.  Every wait is bounded: a tile that has not published in time
// is counted from its keys instead, and the walk goes on.
constexpr uint32_t kOsAgg = 1u << 30, kOsIncl = 2u << 30, kOsMask = kOsAgg - 1;
constexpr int kOsPolls = 1 << 14;

template <int IT>
__global__ void __launch_bounds__(kThreads)
k_hist_all(const uint64_t *__restrict__ keys, uint64_t n, int passes,
           uint32_t *__restrict__ totals, uint32_t *__restrict__ status,
           uint64_t status_words, const uint32_t *__restrict__ d_n) {
  pdl_wait();
  if (d_n && *d_n < n) n = *d_n;
  __shared__ uint32_t h[8][kRadix];
  for (int p = 0; p < passes; p++) h[p][threadIdx.x] = 0;
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * (kThreads * IT);
#pragma unroll 4
  for (int it = 0; it < IT; it++) {
    const uint64_t i = t0 + (uint64_t)it * kThreads + threadIdx.x;
    if (i < n) {
      const uint64_t k = keys[i];
      for (int p = 0; p < passes; p++) atomicAdd(&h[p][(k >> (8 * p)) & 0xff], 1u);
    }
  }
  __syncthreads();
  for (int p = 0; p < passes; p++)
    if (h[p][threadIdx.x]) atomicAdd(&totals[p * kRadix + threadIdx.x], h[p][threadIdx.x]);
  for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < status_words;
       i += (uint64_t)gridDim.x * kThreads)
    status[i] = 0;
}

// count of digit d among the keys of tile t (the bounded wait's fallback)
__device__ __forceinline__ uint32_t os_count_tile(const uint64_t *in, uint64_t n,
                                                  uint64_t t, int tile, int shift,
                                                  uint32_t d) {
  uint32_t c = 0;
  const uint64_t a = t * (uint64_t)tile;
  const uint64_t e = a + tile < n ? a + tile : n;
  for (uint64_t i = a; i < e; i++) c += ((uint32_t)(in[i] >> shift) & 0xff) == d;
  return c;
}

template <bool KV, int IT>
__global__ void __launch_bounds__(kThreads, IT == kSmallItems ? 3 : 2)
k_scatter_os(const uint64_t *__restrict__ in, uint64_t *__restrict__ out,
             uint64_t n, int shift, const uint32_t *__restrict__ totals,
             uint32_t *__restrict__ status, const uint32_t *__restrict__ vin,
             uint32_t *__restrict__ vout, const uint32_t *__restrict__ d_n) {
  pdl_wait();
  constexpr int TILE = kThreads * IT;
  if (d_n && *d_n < n) n = *d_n;
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t *skeys = reinterpret_cast<uint64_t *>(smem);
  uint32_t *svals = reinterpret_cast<uint32_t *>(smem + (size_t)TILE * 8);
  uint32_t(*wcnt)[kRadix] = reinterpret_cast<uint32_t(*)[kRadix]>(
      smem + scatter_stage_bytes<KV, IT>());
  uint32_t *adj = &wcnt[kWarps - 1][kRadix - 1] + 1;  // [kRadix]
  uint32_t *wsum = adj + kRadix;                        // [kWarps]
  const int warp = threadIdx.x >> 5;
  const uint32_t d = threadIdx.x;  // this thread's digit in the bookkeeping
#pragma unroll
  for (int w = 0; w < kWarps; w++) wcnt[w][d] = 0;
  const uint64_t tile = blockIdx.x;
  const uint64_t t0 = tile * TILE;
  uint64_t kk[IT];
  uint32_t vv[KV ? IT : 1];
  uint32_t dg[IT];
#pragma unroll
  for (int it = 0; it < IT; it++) {
    const uint64_t i = t0 + tile_offset<IT>(it);
    kk[it] = i < n ? in[i] : 0;
    if (KV) vv[it] = i < n ? vin[i] : 0u;
    dg[it] = i < n ? (uint32_t)(kk[it] >> shift) & 0xff : kNoDigit;
  }
  // the match words sit in the staging area, free until the reorder
  uint32_t *wm = reinterpret_cast<uint32_t *>(smem) + warp * kRadix;
  clear_match_words(wm);
  __syncthreads();
  uint32_t lr[IT];
  warp_rank<IT>(dg, lr, wcnt[warp], wm);
  __syncthreads();
  uint32_t tcount = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) tcount += wcnt[w][d];
  // publish this tile's count of digit d, then find the earlier tiles'
  uint32_t *mine = status + tile * kRadix + d;
  uint32_t before = 0;
  if (tile == 0) {
    atomicExch(mine, kOsIncl | tcount);
  } else {
    atomicExch(mine, kOsAgg | tcount);
    // the walk loads kOsAhead earlier tiles' words at once, then takes them
    // in order (a word not yet published is polled again on its own)
    constexpr int kOsAhead = 16;
    bool done = false;
    for (int64_t t0 = (int64_t)tile - 1; t0 >= 0 && !done; t0 -= kOsAhead) {
      uint32_t w[kOsAhead];
#pragma unroll
      for (int q = 0; q < kOsAhead; q++)
        w[q] = t0 - q >= 0 ? *(const volatile uint32_t *)(status + (uint64_t)(t0 - q) * kRadix + d)
                           : kOsIncl;
#pragma unroll
      for (int q = 0; q < kOsAhead; q++) {
        const int64_t t = t0 - q;
        if (done || t < 0) break;
        uint32_t v = w[q];
        const volatile uint32_t *sp = status + (uint64_t)t * kRadix + d;
        for (int p = 0; (v & ~kOsMask) == 0 && p < kOsPolls; p++) {
          __nanosleep(p < 32 ? 20 : 200);
          v = *sp;
        }
        if ((v & ~kOsMask) == 0) {  // never published: count its keys
          before += os_count_tile(in, n, (uint64_t)t, TILE, shift, d);
          continue;
        }
        before += v & kOsMask;
        if ((v & ~kOsMask) == kOsIncl) done = true;
      }
    }
    atomicExch(mine, kOsIncl | (before + tcount));
  }
  // global start of digit d: all keys of smaller digits, then the earlier
  // tiles' keys of digit d
  const uint32_t gbase = block_excl_scan(totals[d], wsum) + before;
  __syncthreads();  // wsum is read by every thread before it is reused
  const uint32_t tstart = block_excl_scan(tcount, wsum);
  uint32_t sacc = tstart;
#pragma unroll
  for (int w = 0; w < kWarps; w++) {
    const uint32_t c = wcnt[w][d];
    wcnt[w][d] = sacc;
    sacc += c;
  }
  adj[d] = gbase - tstart;
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IT; it++) {
    if (dg[it] == kNoDigit) continue;
    const uint32_t lp = wcnt[warp][dg[it]] + lr[it];
    skeys[lp] = kk[it];
    if (KV) svals[lp] = vv[it];
  }
  __syncthreads();
  const uint32_t tn = t0 >= n ? 0u : (uint32_t)(n - t0 < (uint64_t)TILE ? n - t0 : TILE);
  for (uint32_t j = threadIdx.x; j < tn; j += kThreads) {
    const uint64_t key = skeys[j];
    const uint32_t pos = adj[(key >> shift) & 0xff] + j;
    out[pos] = key;
    if (KV) vout[pos] = svals[j];
  }
}

// The key-value scatter's shared memory is above the 48 KB default: raise
// its limit once per device (before the first launch there).
cudaError_t scatter_smem_optin() {
  static std::atomic<uint64_t> done{0};  // one bit per device below 64
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 64 && ((done.load(std::memory_order_relaxed) >> dev) & 1)) return cudaSuccess;
  e = cudaFuncSetAttribute(k_scatter<true, kItems>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)scatter_smem_bytes<true, kItems>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_scatter_os<true, kItems>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)scatter_smem_bytes<true, kItems>());
  if (e == cudaSuccess && dev < 64) done.fetch_or(1ull << dev, std::memory_order_relaxed);
  return e;
}

// Whole sort in one CTA for n <= TILE: keys (and payloads) staged in shared
// memory; each pass ranks warp-contiguous items as k_scatter does, the digit
// offsets coming from a block scan of the warps' counts.
template <bool KV, int TILE>
__global__ void __launch_bounds__(kThreads)
k_sort_small(uint64_t *__restrict__ keys, uint32_t *__restrict__ vals,
             uint64_t n, int bits, const uint32_t *__restrict__ d_n) {
  pdl_wait();
  if (d_n && *d_n < n) n = *d_n;
  constexpr int IT = TILE / kThreads;
  __shared__ uint64_t buf[2][TILE];
  __shared__ uint32_t vbuf[KV ? 2 : 1][KV ? TILE : 1];
  __shared__ uint32_t wcnt[kWarps][kRadix];
  __shared__ uint32_t wmatch[kWarps][kRadix];
  __shared__ uint32_t wsum[kWarps];
  const int warp = threadIdx.x >> 5;
  clear_match_words(wmatch[warp]);  // warp_rank leaves them clear again
  for (uint64_t i = threadIdx.x; i < n; i += kThreads) {
    buf[0][i] = keys[i];
    if (KV) vbuf[0][i] = vals[i];
  }
  int cur = 0;
  for (int shift = 0; shift < bits; shift += 8) {
#pragma unroll
    for (int w = 0; w < kWarps; w++) wcnt[w][threadIdx.x] = 0;
    __syncthreads();  // counters clear; the previous pass's keys in place
    uint64_t kk[IT];
    uint32_t dg[IT], lr[IT];
#pragma unroll
    for (int it = 0; it < IT; it++) {
      const uint32_t o = tile_offset<IT>(it);
      kk[it] = o < n ? buf[cur][o] : 0;
      dg[it] = o < n ? (uint32_t)(kk[it] >> shift) & 0xff : kNoDigit;
    }
    warp_rank<IT>(dg, lr, wcnt[warp], wmatch[warp]);
    __syncthreads();
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) tot += wcnt[w][threadIdx.x];
    uint32_t s = block_excl_scan(tot, wsum);
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      const uint32_t c = wcnt[w][threadIdx.x];
      wcnt[w][threadIdx.x] = s;
      s += c;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < IT; it++) {
      if (dg[it] == kNoDigit) continue;
      const uint32_t pos = wcnt[warp][dg[it]] + lr[it];
      buf[cur ^ 1][pos] = kk[it];
      if (KV) vbuf[cur ^ 1][pos] = vbuf[cur][tile_offset<IT>(it)];
    }
    __syncthreads();  // all reads of the counters done before the next pass
    cur ^= 1;
  }
  for (uint64_t i = threadIdx.x; i < n; i += kThreads) {
    keys[i] = buf[cur][i];
    if (KV) vals[i] = vbuf[cur][i];
  }
}

constexpr int kSmallSortKV = 1024;

// Keys alone (no payload: equal keys are indistinguishable, so the order
// need not be stable) of 1025 .. kSmallSort: a bitonic sort in one CTA of
// kBitonicThreads, each thread taking the compare-exchanges of its pairs
// at every stage (66 stages for 2048 keys).  Up to 1024 keys the one-CTA
// radix form (k_sort_small, whose ranking by shared-memory match words is
// cheap) is faster: 10.5 against 12.9 us at 1e3 keys (serialised); its
// buffers for 2048 keys would pass the 48 KB of static shared memory.
// (Holding two keys a thread in registers, with warp shuffles for the
// stages within a warp and the shared array only for the rest, measured
// slower than this bitonic form: 15.7 against 13.0 us at 1e3 keys.)
constexpr int kBitonicThreads = 1024;
static_assert(kSmallSort <= 2 * kBitonicThreads, "one pair per thread and stage");
__global__ void __launch_bounds__(kBitonicThreads)
k_sort_bitonic(uint64_t *__restrict__ keys, uint64_t n, const uint32_t *__restrict__ d_n) {
  pdl_wait();
  __shared__ uint64_t sk[kSmallSort];
  if (d_n && *d_n < n) n = *d_n;
  uint32_t N = 2;
  while (N < n) N <<= 1;
  const uint32_t t = threadIdx.x;
  for (uint32_t i = t; i < N; i += kBitonicThreads) sk[i] = i < n ? keys[i] : ~0ull;
  __syncthreads();
  for (uint32_t k = 2; k <= N; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      // thread t takes the pair (i, i ^ j) whose lower index i is its t-th
      const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
      if (i + j < N) {
        const uint64_t a = sk[i], b = sk[i + j];
        if ((a > b) == ((i & k) == 0)) {
          sk[i] = b;
          sk[i + j] = a;
        }
      }
      __syncthreads();
    }
  for (uint32_t i = t; i < n; i += kBitonicThreads) keys[i] = sk[i];
}

}  // namespace

size_t radix_sort_scratch_bytes(uint64_t n) {
  const uint64_t tile = n <= kSmallTileKeys ? (uint64_t)kThreads * kSmallItems : kTile;
  uint64_t nblocks = (n + tile - 1) / tile;
  uint64_t hn = nblocks * kRadix;
  // the one-sweep form: digit totals and up to eight passes' tile status;
  // the counting forms: three count tables or counts and their scan
  const size_t os = 8 * kRadix * 4 + 8 * ((hn * 4 + 255) & ~size_t(255)) + 512;
  const size_t cnt = 3 * ((hn * 4 + 255) & ~size_t(255)) + scan_scratch_bytes(hn, 4) + 512;
  return os > cnt ? os : cnt;
}

// profiler name of a scatter pass, by its tile size
template <bool KV, int IT>
constexpr const char *scatter_name() {
  if constexpr (IT == kSmallItems)
    return KV ? "(k_scatter<true, 4>)" : "(k_scatter<false, 4>)";
  else
    return KV ? "(k_scatter<true, 16>)" : "(k_scatter<false, 16>)";
}

template <bool KV, int IT>
constexpr const char *scatter_os_name() {
  if constexpr (IT == kSmallItems)
    return KV ? "(k_scatter_os<true, 4>)" : "(k_scatter_os<false, 4>)";
  else
    return KV ? "(k_scatter_os<true, 16>)" : "(k_scatter_os<false, 16>)";
}

// The multi-tile sort with tiles of IT items per thread (see radix_sort_impl).
template <int IT>
static cudaError_t radix_sort_tiles(uint64_t *keys, uint64_t *tmp, uint32_t *vals,
                                    uint32_t *vtmp, uint64_t n, int bits, Arena &arena,
                                    cudaStream_t s, uint64_t **result,
                                    uint32_t **vresult, const uint32_t *d_n,
                                    const SortDigits *pre) {
  constexpr int TILE = kThreads * IT;
  const uint32_t nblocks = (uint32_t)((n + TILE - 1) / TILE);
  const uint64_t hn = (uint64_t)nblocks * kRadix;
  if (vals) {
    cudaError_t e = scatter_smem_optin();
    if (e != cudaSuccess) return e;
  }
  uint64_t *src = keys, *dst = tmp;
  uint32_t *vsrc = vals, *vdst = vtmp;
  // every scatter reads and writes keys (and values) and reads the counts
  const uint64_t hist_bytes = 8 * n + 4 * hn;
  const uint64_t scatter_bytes = (vals ? 24 : 16) * n + 8 * hn;
  const int passes = (bits + 7) / 8;
  if (n < (1ull << 30) && passes <= 8) {
    // one sweep: all passes' digit totals in one read, then one launch a
    // pass whose tiles find their offsets by looking back
    uint32_t *totals, *status;
    if (pre) {  // counted by the caller, status words cleared
      if (pre->passes != passes || pre->status_words != (uint64_t)passes * hn)
        return cudaErrorInvalidValue;
      totals = pre->totals;
      status = pre->status;
    } else {
      totals = arena.take<uint32_t>(8 * kRadix);
      status = arena.take<uint32_t>((uint64_t)passes * hn);
      if (!totals || !status) return cudaErrorMemoryAllocation;
      cudaError_t e = cudaMemsetAsync(totals, 0, (size_t)passes * kRadix * 4, s);
      if (e != cudaSuccess) return e;
      SST_LAUNCH_PDL_NB("(k_hist_all)", 8 * n, k_hist_all<IT>, nblocks, kThreads, 0, s, src, n,
                    passes, totals, status, (uint64_t)passes * hn, d_n);
    }
    for (int p = 0; p < passes; p++) {
      const uint64_t sb = (vals ? 24 : 16) * n + 8 * (uint64_t)kRadix * nblocks;
      if (vals)
        SST_LAUNCH_PDL_NB((scatter_os_name<true, IT>()), sb, (k_scatter_os<true, IT>), nblocks,
                      kThreads, (scatter_smem_bytes<true, IT>()), s, src, dst, n, 8 * p,
                      totals + p * kRadix, status + (uint64_t)p * hn, vsrc, vdst, d_n);
      else
        SST_LAUNCH_PDL_NB((scatter_os_name<false, IT>()), sb, (k_scatter_os<false, IT>), nblocks,
                      kThreads, (scatter_smem_bytes<false, IT>()), s, src, dst, n, 8 * p,
                      totals + p * kRadix, status + (uint64_t)p * hn, vsrc, vdst, d_n);
      std::swap(src, dst);
      std::swap(vsrc, vdst);
    }
  } else if (nblocks <= kFuseHistBlocks) {
    // three tile-major count tables in rotation: pass p reads table p % 3,
    // counts into (p + 1) % 3 and clears (p + 2) % 3
    uint32_t *h[3];
    for (auto &t : h)
      if (!(t = arena.take<uint32_t>(hn))) return cudaErrorMemoryAllocation;
    SST_LAUNCH_PDL_B(hist_bytes, k_hist<IT>, nblocks, kThreads, 0, s, src, n, 0, h[0],
                 1u, (uint32_t)kRadix, h[1], d_n);
    int p = 0;
    for (int shift = 0; shift < bits; shift += 8, p++) {
      const bool more = shift + 8 < bits;
      uint32_t *nx = more ? h[(p + 1) % 3] : nullptr;
      uint32_t *zr = more ? h[(p + 2) % 3] : nullptr;
      if (vals)
        SST_LAUNCH_PDL_NB((scatter_name<true, IT>()), scatter_bytes, (k_scatter<true, IT>), nblocks, kThreads,
                     (scatter_smem_bytes<true, IT>()), s, src,
                     dst, n, shift, h[p % 3], nblocks, true, vsrc, vdst, nx,
                     shift + 8, zr, d_n);
      else
        SST_LAUNCH_PDL_NB((scatter_name<false, IT>()), scatter_bytes, (k_scatter<false, IT>), nblocks, kThreads,
                     (scatter_smem_bytes<false, IT>()), s, src,
                     dst, n, shift, h[p % 3], nblocks, true, vsrc, vdst, nx,
                     shift + 8, zr, d_n);
      std::swap(src, dst);
      std::swap(vsrc, vdst);
    }
  } else {
    // counts and their scan in separate tables (the single-pass scan runs
    // out of place)
    uint32_t *cnts = arena.take<uint32_t>(hn);
    uint32_t *hist = arena.take<uint32_t>(hn);
    if (!cnts || !hist) return cudaErrorMemoryAllocation;
    for (int shift = 0; shift < bits; shift += 8) {
      SST_LAUNCH_PDL_B(hist_bytes, k_hist<IT>, nblocks, kThreads, 0, s, src, n, shift,
                   cnts, nblocks, 1u, (uint32_t *)nullptr, d_n);
      size_t mark = arena.used;
      cudaError_t e = scan<uint32_t, OpAdd>(cnts, hist, hn, 0u, OpAdd{}, true,
                                            false, nullptr, arena, s);
      arena.used = mark;
      if (e != cudaSuccess) return e;
      if (vals)
        SST_LAUNCH_PDL_NB((scatter_name<true, IT>()), scatter_bytes, (k_scatter<true, IT>), nblocks, kThreads,
                     (scatter_smem_bytes<true, IT>()), s, src,
                     dst, n, shift, hist, nblocks, false, vsrc, vdst,
                     (uint32_t *)nullptr, 0, (uint32_t *)nullptr, d_n);
      else
        SST_LAUNCH_PDL_NB((scatter_name<false, IT>()), scatter_bytes, (k_scatter<false, IT>), nblocks, kThreads,
                     (scatter_smem_bytes<false, IT>()), s, src,
                     dst, n, shift, hist, nblocks, false, vsrc, vdst,
                     (uint32_t *)nullptr, 0, (uint32_t *)nullptr, d_n);
      std::swap(src, dst);
      std::swap(vsrc, vdst);
    }
  }
  *result = src;
  if (vresult) *vresult = vsrc;
  return cudaGetLastError();
}

// the form radix_sort_impl takes: 0 none (n < 2), 1 one CTA, 2 tiles of
// kSmallItems a thread, 3 tiles of kItems
static int sort_form(uint64_t n, int bits, bool vals) {
  if (n < 2 || bits <= 0) return 0;
  if (!vals && n <= (uint64_t)kSmallSort) return 1;
  if (vals && n <= (uint64_t)kSmallSortKV) return 1;
  if (!vals && n <= kSmallTileKeys) return 2;
  return 3;
}

bool radix_sort_digits(uint64_t n, int bits, Arena &arena, SortDigits *d) {
  const int form = sort_form(n, bits, false);
  const int passes = (bits + 7) / 8;
  if (form < 2 || n >= (1ull << 30) || passes > 8) return false;
  const uint64_t tile = (uint64_t)kThreads * (form == 2 ? kSmallItems : kItems);
  const uint64_t hn = (n + tile - 1) / tile * kRadix;
  d->totals = arena.take<uint32_t>(8 * kRadix);
  d->status = arena.take<uint32_t>((uint64_t)passes * hn);
  d->status_words = (uint64_t)passes * hn;
  d->passes = passes;
  return d->totals && d->status;
}

static cudaError_t radix_sort_impl(uint64_t *keys, uint64_t *tmp,
                                   uint32_t *vals, uint32_t *vtmp, uint64_t n,
                                   int bits, Arena &arena, cudaStream_t s,
                                   uint64_t **result, uint32_t **vresult,
                                   const uint32_t *d_n, const SortDigits *pre = nullptr) {
  *result = keys;
  if (vresult) *vresult = vals;
  if (n < 2 || bits <= 0) return cudaSuccess;
  if (pre && (vals || sort_form(n, bits, false) < 2)) return cudaErrorInvalidValue;
  if (!vals && n <= (uint64_t)kSmallSortKV) {
    SST_LAUNCH_PDL_B(16 * n, (k_sort_small<false, kSmallSortKV>), 1, kThreads, 0, s, keys,
                     (uint32_t *)nullptr, n, bits, d_n);
    return cudaGetLastError();
  }
  if (!vals && n <= (uint64_t)kSmallSort) {
    SST_LAUNCH_PDL_B(16 * n, k_sort_bitonic, 1, kBitonicThreads, 0, s, keys, n, d_n);
    return cudaGetLastError();
  }
  if (vals && n <= (uint64_t)kSmallSortKV) {
    SST_LAUNCH_PDL_B(24 * n, (k_sort_small<true, kSmallSortKV>), 1, kThreads, 0, s, keys, vals,
               n, bits, d_n);
    return cudaGetLastError();
  }
  if (!vals && n <= kSmallTileKeys)
    return radix_sort_tiles<kSmallItems>(keys, tmp, vals, vtmp, n, bits, arena, s, result,
                                         vresult, d_n, pre);
  return radix_sort_tiles<kItems>(keys, tmp, vals, vtmp, n, bits, arena, s, result, vresult,
                                  d_n, pre);
}

cudaError_t radix_sort_u64(uint64_t *keys, uint64_t *tmp, uint64_t n, int bits,
                           Arena &arena, cudaStream_t s, uint64_t **result,
                           const uint32_t *d_n, const SortDigits *pre) {
  return radix_sort_impl(keys, tmp, nullptr, nullptr, n, bits, arena, s, result,
                         nullptr, d_n, pre);
}

cudaError_t radix_sort_kv(uint64_t *keys, uint64_t *tmp, uint32_t *vals,
                          uint32_t *vtmp, uint64_t n, int bits, Arena &arena,
                          cudaStream_t s, uint64_t **result, uint32_t **vresult) {
  return radix_sort_impl(keys, tmp, vals, vtmp, n, bits, arena, s, result,
                         vresult, nullptr);
}

}  // namespace sst

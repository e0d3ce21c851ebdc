// Graph lifetime, slab allocation and the batch update pipeline.
//
// A batch (insert or remove) runs as:
//   1. keys      (row << dbits | col) per pair; self-loops (insert) and ids
//                out of range become a sentinel that sorts last
//   2. sort      stable LSD radix sort of the keys (primitives.cu)
//   3. locate    per unique key: the leaf of its row's PMA where it belongs
//                (binary search over leaf heads) and whether it is present
//   4. pack      keys that change the graph, as (row, leaf) + col, in order
//   5. group     one group per (row, leaf)
//   6. classify  insert: a group fits its leaf (leaf merge) or climbs to the
//                smallest aligned window of 2^t leaves whose count stays
//                under the upper density bound, or the whole segment is
//                resized.  remove: deletions are applied leaf-locally first,
//                then leaves under the lower bound climb the same way.
//   7. dominance aligned windows nest, so a forward max-scan and a backward
//                min-scan over the groups find, for each group, the largest
//                window of its row that covers it; covered groups drop out
//   8. plan      window/resize tasks are sized and the summary is read back
//                (the one host synchronisation of a batch): it sizes the
//                staging buffer and the slab allocation
//   9. apply     leaf merges (one warp per leaf, shuffle-ranked), then each
//                task gathers old + new elements at their merged rank into
//                staging (parallel over leaves and items) and scatters them
//                evenly over the destination leaves (one warp per leaf)
// Reference counterparts: SparseMatrix.hpp:556-718 (batch split by row),
// PMA.hpp:1028-1082 (place: window climb + redistribute),
// PMA.hpp:612-702 (redistribute / double_list / half_list),
// PMA.hpp:1185-1222 (take: lower-bound climb).
#include <algorithm>
#include <cstddef>
#include <cstdarg>
#include <cstring>
#include <vector>

#include "graph.cuh"

namespace sst {

namespace {

enum : uint8_t { kNone = 0, kMerge = 1, kWindow = 2, kResize = 3 };

constexpr int kTB = 256;  // threads per block for element-wise kernels

inline unsigned blocks_for(uint64_t n, int per_block = kTB) {
  uint64_t b = (n + per_block - 1) / per_block;
  return (unsigned)(b == 0 ? 1 : b);
}
inline unsigned warp_blocks(uint64_t nwarps) {
  return blocks_for(nwarps * 32);
}

int bits_for(uint64_t x) {
  int b = 0;
  while (b < 64 && (x >> b) != 0) b++;
  return b;
}

// Lower bound (first index with a[i] >= x) of [lo, hi) in a sorted array,
// by a whole warp (every lane gets the answer): each round the 32 lanes
// probe 32 evenly spaced positions and the range shrinks to the gap between
// the last probe below x and the next one, so a range of 1e6 items takes
// four dependent rounds instead of twenty.
__device__ __forceinline__ uint32_t warp_lb_u64(const uint64_t *a, uint32_t lo,
                                                uint32_t hi, uint64_t x) {
  const uint32_t lane = threadIdx.x & 31;
  while (hi - lo > 32) {
    const uint32_t step = (hi - lo + 31) / 32;
    const uint32_t probe = lo + lane * step;
    const bool less = probe < hi && a[probe] < x;
    const uint32_t k = __popc(__ballot_sync(0xffffffffu, less));
    if (k == 0) return lo;  // a[lo] >= x
    const uint32_t nhi = lo + k * step;  // a[nhi] >= x, or nhi >= hi
    lo += (k - 1) * step + 1;
    if (nhi < hi) hi = nhi;
  }
  const uint32_t probe = lo + lane;
  return lo + __popc(__ballot_sync(0xffffffffu, probe < hi && a[probe] < x));
}

// index of the last element <= x in a sorted array (n >= 1, a[0] <= x)
__device__ __forceinline__ uint64_t last_le_u64(const uint64_t *a, uint64_t n,
                                                uint64_t x) {
  uint64_t lo = 0, hi = n;
  while (hi - lo > 1) {
    uint64_t mid = (lo + hi) >> 1;
    if (a[mid] <= x)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// elements of a[lo, hi) below each of four keys, found at once (the
// branchless lower bound: each step halves the range for all four searches,
// so their loads are in flight together)
__device__ __forceinline__ void count_less4(const uint32_t *a, uint32_t lo, uint32_t hi,
                                            const uint32_t (&x)[4], uint32_t (&out)[4]) {
  uint32_t b[4] = {lo, lo, lo, lo};
  uint32_t n = hi - lo;
  if (n == 0) {
#pragma unroll
    for (int r = 0; r < 4; r++) out[r] = 0;
    return;
  }
  while (n > 1) {
    const uint32_t half = n >> 1;
#pragma unroll
    for (int r = 0; r < 4; r++) b[r] = a[b[r] + half] < x[r] ? b[r] + half : b[r];
    n -= half;
  }
#pragma unroll
  for (int r = 0; r < 4; r++) out[r] = (b[r] - lo) + (a[b[r]] < x[r] ? 1u : 0u);
}

__device__ __forceinline__ uint32_t warp_sum_lcnt(const uint8_t *lc,
                                                  uint64_t lo, uint64_t hi) {
  const int lane = threadIdx.x & 31;
  uint32_t s = 0;
  for (uint64_t i = lo + lane; i < hi; i += 32) s += lc[i];
  return __reduce_add_sync(0xffffffffu, s);
}

// count word of an item's leaf: the leaf's element count (bits 0-7), plus
// this bit when the row is a multi-leaf segment (its leaves keep counts in
// lcnt), else the one-leaf row's capacity (0..32) from bit kCapShift
constexpr uint32_t kMultiLeaf = 1u << 8;
constexpr int kCapShift = 16;
__device__ __forceinline__ uint32_t one_leaf_cap(uint32_t cw) { return cw >> kCapShift; }

// ---------------------------------------------------------------- steps 1-5
// Keys of a batch, in one of two forms.
// k_make_keys: key i of pair i, the sentinel n << dbits for a pair that is
// dropped (an id out of range, or a self-loop the insert skips); the stable
// sort keeps equal keys in input order (weighted graphs: the last value
// given wins).
__global__ void k_make_keys(const uint32_t *__restrict__ pairs, uint64_t b,
                            uint32_t n, uint32_t width, int dbits,
                            bool drop_loops, uint64_t *__restrict__ keys,
                            unsigned long long *__restrict__ invalid,
                            const uint32_t *__restrict__ w,
                            uint32_t *__restrict__ wv) {
  pdl_wait();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b) return;
  // weighted graphs: the pair's value (1 when the call gives none) rides
  // with the key through the sort
  if (wv) wv[i] = w ? w[i] : 1u;
  const uint32_t r = pairs[2 * i], c = pairs[2 * i + 1];
  const bool ok = r < n && c < width && c != kEmpty;
  if (!ok) atomicAdd(invalid, 1ull);
  keys[i] = (!ok || (drop_loops && r == c)) ? (uint64_t)n << dbits
                                            : (((uint64_t)r << dbits) | c);
}

// k_make_keys_packed: only the kept keys, packed to the front in any order
// (*nkeys of them; one reservation per block of kPackItems x 256 pairs).
// Equal keys are equal, so their order does not matter (unweighted
// graphs), and the sort needs no bit for the sentinel row.  With V2 (the
// pairs 8-byte aligned) a pair comes in with one 8-byte load: the warp's
// load covers 256 contiguous bytes once, where two 4-byte loads a pair read
// each line twice (pinned host pairs are read across the host link).
// With sd.passes > 0 it also counts every radix pass's 8-bit digits of the
// keys it keeps into sd.totals (zero on entry) and clears the sort's tile
// status words (SortDigits): the sort then skips its own counting read.
constexpr int kPackItems = 8;
template <bool V2>
__global__ void __launch_bounds__(256)
k_make_keys_packed(const uint32_t *__restrict__ pairs, uint64_t b, uint32_t n,
                   uint32_t width, int dbits, bool drop_loops,
                   uint64_t *__restrict__ keys,
                   unsigned long long *__restrict__ invalid,
                   uint32_t *__restrict__ nkeys, SortDigits sd) {
  pdl_wait();
  __shared__ uint32_t s_warp[8];
  __shared__ uint32_t s_base;
  __shared__ uint32_t s_hist[8][256];
  for (int p = 0; p < sd.passes; p++) s_hist[p][threadIdx.x] = 0;
  const uint64_t t0 = (uint64_t)blockIdx.x * (256 * kPackItems);
  uint64_t key[kPackItems];
  uint32_t kept = 0, bad = 0;  // bit k: item k is kept
#pragma unroll
  for (int k = 0; k < kPackItems; k++) {
    const uint64_t i = t0 + (uint64_t)k * 256 + threadIdx.x;
    uint32_t r = 0, c = 0;
    if (i < b) {
      if (V2) {
        const uint2 rc = reinterpret_cast<const uint2 *>(pairs)[i];
        r = rc.x;
        c = rc.y;
      } else {
        r = pairs[2 * i];
        c = pairs[2 * i + 1];
      }
    }
    const bool ok = i < b && r < n && c < width && c != kEmpty;
    bad += i < b && !ok;
    if (ok && !(drop_loops && r == c)) kept |= 1u << k;
    key[k] = ((uint64_t)r << dbits) | c;
  }
  const uint32_t keep = __popc(kept);
  if (bad) atomicAdd(invalid, (unsigned long long)bad);
  // block prefix of the kept counts, one reservation for the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = keep;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int w = 0; w < 8; w++) {
      const uint32_t c = s_warp[w];
      s_warp[w] = tot;
      tot += c;
    }
    s_base = tot ? atomicAdd(nkeys, tot) : 0u;
  }
  if (sd.passes) {
#pragma unroll
    for (int k = 0; k < kPackItems; k++)
      if ((kept >> k) & 1u)
        for (int p = 0; p < sd.passes; p++)
          atomicAdd(&s_hist[p][(key[k] >> (8 * p)) & 0xff], 1u);
    for (uint64_t i = (uint64_t)blockIdx.x * 256 + threadIdx.x; i < sd.status_words;
         i += (uint64_t)gridDim.x * 256)
      sd.status[i] = 0;
  }
  __syncthreads();
  const uint64_t at = (uint64_t)s_base + s_warp[warp] + inc - keep;
#pragma unroll
  for (int k = 0; k < kPackItems; k++)
    if ((kept >> k) & 1u) keys[at + __popc(kept & ((1u << k) - 1u))] = key[k];
  for (int p = 0; p < sd.passes; p++)
    if (s_hist[p][threadIdx.x]) atomicAdd(&sd.totals[p * 256 + threadIdx.x], s_hist[p][threadIdx.x]);
}

// Of a run of equal keys the last (in input order: the sort is stable) is
// the one applied, so on a weighted graph the last value given wins, as
// sequential inserts would leave it (PMA.hpp:1137-1145).  A weighted insert
// of an edge already present overwrites its value here, in place.
__global__ void k_locate(const uint64_t *__restrict__ keys, uint64_t b,
                         int dbits, DGraph g, bool insert,
                         uint32_t *__restrict__ flag,
                         uint32_t *__restrict__ leaf_out,
                         const uint32_t *__restrict__ wv,
                         uint64_t *__restrict__ lS, uint32_t *__restrict__ lc,
                         const uint32_t *__restrict__ nkeys) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b) return;
  const uint64_t sent = (uint64_t)g.n << dbits;
  // a compacting key build leaves nkeys sorted keys and nothing after them
  const uint64_t nk = nkeys ? *nkeys : b;
  uint64_t k = i < nk ? keys[i] : sent;
  if (k >= sent || (i + 1 < nk && keys[i + 1] == k)) {
    flag[i] = 0;
    leaf_out[i] = 0;
    return;
  }
  uint64_t S = 0;
  uint32_t cw = 0;
  uint32_t u = (uint32_t)(k >> dbits);
  uint32_t x = (uint32_t)(k & ((1ull << dbits) - 1));
  uint64_t base = g.base[u];
  uint32_t cap = g.cap[u], deg = g.deg[u];
  bool present = false;
  uint32_t l = 0;
  if (cap > 0) {
    l = find_leaf(g.slots, base, cap, x);
    uint32_t c = leaf_count(g, base, cap, deg, l);
    const uint32_t *p = g.slots + base + ((uint64_t)l << kLeafLog);
    uint32_t pos = leaf_lower_bound(p, c, x);
    present = pos < c && p[pos] == x;
    if (present && insert && wv && g.vals)
      g.vals[base + ((uint64_t)l << kLeafLog) + pos] = wv[i];
    S = base + ((uint64_t)l << kLeafLog);
    cw = c | (cap > kLeaf ? kMultiLeaf : cap << kCapShift);
  }
  flag[i] = insert ? !present : present;
  leaf_out[i] = l;
  lS[i] = S;
  lc[i] = cw;
}

// k_locate for small batches, a warp per key (a batch of up to
// kLocateWarpKeys keys fills about one wave of warps): the leaf search
// probes 32 leaf heads at once, so a row of L leaves takes about log32(L)
// dependent steps where a thread takes log2(L), and the leaf's 32 slots come
// in with one coalesced load.  Same outputs as k_locate (the heads of a
// segment's leaves ascend, so the leaves whose head is <= x are a prefix).
constexpr uint64_t kLocateWarpKeys = 16384;
__global__ void k_locate_warp(const uint64_t *__restrict__ keys, uint64_t b,
                              int dbits, DGraph g, bool insert,
                              uint32_t *__restrict__ flag,
                              uint32_t *__restrict__ leaf_out,
                              const uint32_t *__restrict__ wv,
                              uint64_t *__restrict__ lS, uint32_t *__restrict__ lc,
                              const uint32_t *__restrict__ nkeys) {
  pdl_wait();
  const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= b) return;  // whole warps
  const uint64_t sent = (uint64_t)g.n << dbits;
  const uint64_t nk = nkeys ? *nkeys : b;
  const uint64_t k = i < nk ? keys[i] : sent;
  if (k >= sent || (i + 1 < nk && keys[i + 1] == k)) {
    if (lane == 0) {
      flag[i] = 0;
      leaf_out[i] = 0;
    }
    return;
  }
  const uint32_t u = (uint32_t)(k >> dbits);
  const uint32_t x = (uint32_t)(k & ((1ull << dbits) - 1));
  const uint64_t base = g.base[u];
  const uint32_t cap = g.cap[u], deg = g.deg[u];
  bool present = false;
  uint32_t l = 0, c = 0, pos = 0;
  uint64_t S = 0;
  uint32_t cw = 0;
  if (cap > 0) {
    if (cap > kLeaf) {
      // the answer lies in leaves [lo, lo + n); lane j probes leaf lo + j*step
      uint32_t lo = 0, n = cap >> kLeafLog;
      for (;;) {
        const uint32_t step = n > 32 ? (n + 31) / 32 : 1u;
        const uint32_t j = (uint32_t)lane * step;
        const bool le = lane > 0 && j < n && g.slots[base + ((uint64_t)(lo + j) << kLeafLog)] <= x;
        const uint32_t m = __ballot_sync(0xffffffffu, le);
        const uint32_t jj = m ? 31u - __clz(m) : 0u;
        lo += jj * step;
        if (step == 1) break;
        n = n - jj * step < step ? n - jj * step : step;
      }
      l = lo;
    }
    c = leaf_count(g, base, cap, deg, l);
    S = base + ((uint64_t)l << kLeafLog);
    const uint32_t a = (uint32_t)lane < c ? g.slots[S + lane] : kEmpty;
    pos = __popc(__ballot_sync(0xffffffffu, a < x));
    const uint32_t at = __shfl_sync(0xffffffffu, a, pos & 31);
    present = pos < c && at == x;
    cw = c | (cap > kLeaf ? kMultiLeaf : cap << kCapShift);
  }
  if (lane == 0) {
    if (present && insert && wv && g.vals) g.vals[S + pos] = wv[i];
    flag[i] = insert ? !present : present;
    leaf_out[i] = l;
    lS[i] = S;
    lc[i] = cw;
  }
}

__global__ void k_pack(const uint64_t *__restrict__ keys,
                       const uint32_t *__restrict__ flag,
                       const uint32_t *__restrict__ pos,
                       const uint32_t *__restrict__ leaf, uint64_t b, int dbits,
                       uint64_t *__restrict__ p_ul, uint32_t *__restrict__ p_x,
                       const uint32_t *__restrict__ wv, uint32_t *__restrict__ p_w,
                       const uint64_t *__restrict__ lS, const uint32_t *__restrict__ lc,
                       uint64_t *__restrict__ p_S, uint32_t *__restrict__ p_c) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b || !flag[i]) return;
  uint64_t k = keys[i];
  uint32_t j = pos[i];
  if (j >= b) return;  // positions come from a scan: never trust them blindly
  p_ul[j] = ((k >> dbits) << 32) | leaf[i];
  p_x[j] = (uint32_t)(k & ((1ull << dbits) - 1));
  if (p_w) p_w[j] = wv[i];
  p_S[j] = lS[i];
  p_c[j] = lc[i];
}

__global__ void k_group_flags(const uint64_t *__restrict__ p_ul,
                              const uint32_t *__restrict__ d_nitems, uint64_t b,
                              uint32_t *__restrict__ gflag) {
  pdl_wait();
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= b) return;
  uint32_t n = *d_nitems;
  gflag[j] = (j < n && (j == 0 || p_ul[j] != p_ul[j - 1])) ? 1u : 0u;
}

// Group starts, fused into the scan of the group flags: item j that opens
// a group records itself at its group's index; the last item closes the
// list with g_start[groups] = items (g_start[0] = 0 when there are none).
struct GroupStartEpi {
  const uint32_t *gflag;
  const uint32_t *d_nitems;
  uint64_t b;
  uint32_t *g_start;
  __device__ __forceinline__ void operator()(uint64_t j, uint32_t gp) const {
    const uint32_t f = gflag[j];
    if (f && gp < b) g_start[gp] = (uint32_t)j;
    const uint32_t ni = *d_nitems;
    if (ni == 0 ? j == 0 : j + 1 == ni) {
      const uint32_t ng = gp + f;
      if (ng <= b) g_start[ng] = ni;
    }
  }
};

// ---------------------------------------------------------------- step 6
// Group-level kernels run grid-stride over the device-side group count, so
// their grids do not scale with the batch bound.  Classification is one
// thread per group; the rare groups whose leaf over- or underflows are
// appended to a climb list and climbed by one warp each.
#define GRID_STRIDE(i, n)                                                     \
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
       i += (uint64_t)gridDim.x * blockDim.x)

// The count word of the group's first item (its leaf's count and, for a
// one-leaf row, the row's capacity, as k_locate read them; nothing has
// changed either since) decides, so no vertex record or leaf count is read
// again.
__global__ void k_classify_insert(const uint64_t *__restrict__ p_ul,
                                  const uint32_t *__restrict__ p_c,
                                  const uint32_t *__restrict__ g_start,
                                  const uint32_t *__restrict__ d_ngroups,
                                  uint8_t *__restrict__ gtype,
                                  uint8_t *__restrict__ glev,
                                  uint32_t *__restrict__ gw0,
                                  uint32_t *__restrict__ gw1,
                                  uint32_t *__restrict__ climb,
                                  uint32_t *__restrict__ nclimb) {
  pdl_wait();
  const uint32_t ng = *d_ngroups;
  GRID_STRIDE(gid, ng) {
    const uint32_t j0 = g_start[gid], k = g_start[gid + 1] - j0;
    const uint32_t leaf = (uint32_t)p_ul[j0];
    const uint32_t cw = p_c[j0], c = cw & 0xff;
    uint8_t type = kMerge;
    uint32_t lev = 0, w0 = leaf, w1 = leaf + 1;
    if (!(cw & kMultiLeaf)) {
      if (c + k > one_leaf_cap(cw)) {  // a one-leaf row's count is its degree
        type = kResize;
        lev = 31;
        w0 = 0;
        w1 = 1;
      }
    } else if (c + k > kLeaf) {
      type = kNone;  // decided by the climb
      climb[atomicAdd(nclimb, 1u)] = (uint32_t)gid;
    }
    gtype[gid] = type;
    glev[gid] = (uint8_t)lev;
    gw0[gid] = w0;
    gw1[gid] = w1;
  }
}

constexpr int kGroupsPerWarp = 4;

// The leaf holding slot S, read as its whole aligned 128-byte line (always
// inside the slab: slabs are whole lines, and a one-leaf segment never
// crosses a line), then each lane's slot of the leaf by a shuffle: the load
// does not wait on the leaf's count.
__device__ __forceinline__ uint32_t leaf_slot(uint32_t linev, uint64_t S,
                                              uint32_t c, int lane) {
  const uint32_t o = (uint32_t)(S & (kLeaf - 1));
  uint32_t a = __shfl_sync(0xffffffffu, linev, (o + lane) & 31);
  return (uint32_t)lane < c ? a : kEmpty;
}

// Groups of one item (nearly all of them: a batch rarely puts two ids in
// one leaf) take eight lanes, four at a time in a warp: lane `sub` of the
// eight holds the leaf's slots 4 sub .. 4 sub + 3 from S (kEmpty from c on),
// and the one id's place is the count of the slots below it.  The lists of
// a warp's one-item groups and of its other groups are built per chunk of
// 32 groups in shared memory (one byte per group).
constexpr int kLeafWarps = kTB / 32;  // warps of the leaf kernels' blocks
__device__ __forceinline__ void load_quarter(const uint32_t *slots, uint64_t S,
                                             uint32_t c, int sub, uint32_t (&a)[4]) {
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const uint32_t p = 4 * sub + r;
    a[r] = p < c ? slots[S + p] : kEmpty;
  }
}
// slots below x in the group's eight lanes (aligned lane octets)
__device__ __forceinline__ uint32_t below_in_octet(const uint32_t (&a)[4], uint32_t x) {
  uint32_t b = (uint32_t)(a[0] < x) + (a[1] < x) + (a[2] < x) + (a[3] < x);
  b += __shfl_xor_sync(0xffffffffu, b, 1);
  b += __shfl_xor_sync(0xffffffffu, b, 2);
  b += __shfl_xor_sync(0xffffffffu, b, 4);
  return b;
}
// list the chunk's groups, one-item groups first: list[0, n1) their lanes
// in order, list[n1, cnt) the others'; returns n1
__device__ __forceinline__ uint32_t list_groups(uint8_t *list, bool ok, bool one, int lane) {
  const uint32_t okm = __ballot_sync(0xffffffffu, ok);
  const uint32_t om = __ballot_sync(0xffffffffu, ok && one);
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t n1 = __popc(om);
  __syncwarp();  // the previous chunk's lists are read
  if (ok) list[one ? __popc(om & lt) : n1 + __popc(okm & ~om & lt)] = (uint8_t)lane;
  __syncwarp();
  return n1;
}

// remove: delete inside each touched leaf, take the count off the row's
// degree and classify the group: a leaf of a multi-leaf segment under the
// lower bound goes to the climb list; a one-leaf segment that emptied or
// fell to a quarter is resized.  (A one-leaf row has exactly one group, so
// its degree afterwards is its leaf's new count.)  lo_leaf is a one-leaf
// window's lower bound in a multi-leaf segment, window_lower(p, 0, H), the
// same for every H >= 1 (computed once on the host: no per-group FP64).
// A warp takes 32 groups at a time: lane l first loads group l's item
// range, its first item's leaf start, count word and key (two dependent
// loads for all 32 groups at once), then the
// groups' leaves go kGroupsPerWarp at a time with their items and leaf
// lines loaded together, one dependent load per batch; the bookkeeping
// (leaf count, degree, classification) runs once for all 32 groups, lane l
// for group l.
__global__ void __launch_bounds__(256, 4)
k_leaf_delete(DGraph g, uint32_t lo_leaf, const uint64_t *__restrict__ p_ul,
              const uint32_t *__restrict__ p_x,
              const uint64_t *__restrict__ p_S, const uint32_t *__restrict__ p_c,
              const uint32_t *__restrict__ g_start,
              const uint32_t *__restrict__ d_ngroups,
              uint8_t *__restrict__ gtype, uint8_t *__restrict__ glev,
              uint32_t *__restrict__ gw0, uint32_t *__restrict__ gw1,
              uint32_t *__restrict__ climb, uint32_t *__restrict__ nclimb) {
  pdl_wait();
  __shared__ uint8_t glist[kLeafWarps][32];
  const int lane = threadIdx.x & 31, sub = lane & 7;
  uint8_t *list = glist[threadIdx.x >> 5];
  constexpr int Q = kGroupsPerWarp;
  const uint32_t ng = *d_ngroups;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       w * 32 < ng; w += nw) {
    const uint64_t gl = w * 32 + lane;
    const bool okl = gl < ng;
    const uint32_t j0l = okl ? g_start[gl] : 0;
    const uint32_t kl = okl ? g_start[gl + 1] - j0l : 0;
    const uint64_t Sl = okl ? p_S[j0l] : 0;
    const uint32_t cwl = okl ? p_c[j0l] : 0;
    const uint64_t keyl = okl ? p_ul[j0l] : 0;
    const uint32_t ul = (uint32_t)(keyl >> 32), leafl = (uint32_t)keyl;
    // a one-leaf row's capacity is in its count word; a multi-leaf row
    // only needs to be told apart
    const uint32_t capl = (cwl & kMultiLeaf) ? kLeaf + 1 : one_leaf_cap(cwl);
    const uint32_t cnt = ng - w * 32 < 32 ? (uint32_t)(ng - w * 32) : 32u;
    // one-item groups: the slots from the deleted id's place on take their
    // right neighbour (kEmpty past the count)
    const uint32_t n1 = list_groups(list, okl, kl == 1 && !g.vals, lane);
    for (uint32_t f0 = 0; f0 < n1; f0 += 4) {
      const uint32_t f = f0 + (lane >> 3);
      const bool on = f < n1;
      const int src = list[on ? f : 0];
      const uint32_t j0 = __shfl_sync(0xffffffffu, j0l, src);
      const uint64_t S = __shfl_sync(0xffffffffu, Sl, src);
      const uint32_t cw = __shfl_sync(0xffffffffu, cwl, src);
      const uint32_t c = on ? (cw & 0xff) : 0u;
      const uint32_t d = on ? p_x[j0] : kEmpty;
      uint32_t a[4];
      load_quarter(g.slots, S, c, sub, a);
      const uint32_t pos = below_in_octet(a, d);
      const uint32_t nxt = __shfl_down_sync(0xffffffffu, a[0], 1, 8);
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const uint32_t p = 4 * sub + r;
        if (p >= pos && p < c) g.slots[S + p] = r < 3 ? a[r + 1] : (sub == 7 ? kEmpty : nxt);
      }
    }
    // the other groups: a warp each, kGroupsPerWarp at a time
    const uint32_t nrest = cnt - n1;
    for (uint32_t q0 = 0; q0 < nrest; q0 += Q) {
      uint32_t j0[Q], k[Q], d[Q], linev[Q], cw[Q];
      uint64_t S[Q];
      bool ok[Q];
#pragma unroll
      for (int q = 0; q < Q; q++) {
        ok[q] = q0 + q < nrest;
        const int src = list[n1 + (ok[q] ? q0 + q : 0)];
        j0[q] = __shfl_sync(0xffffffffu, j0l, src);
        k[q] = ok[q] ? __shfl_sync(0xffffffffu, kl, src) : 0;
        S[q] = __shfl_sync(0xffffffffu, Sl, src);
        cw[q] = __shfl_sync(0xffffffffu, cwl, src);
      }
#pragma unroll
      for (int q = 0; q < Q; q++) {
        d[q] = (uint32_t)lane < k[q] ? p_x[j0[q] + lane] : kEmpty;
        linev[q] = ok[q] ? g.slots[(S[q] & ~uint64_t(kLeaf - 1)) + lane] : kEmpty;
      }
#pragma unroll
      for (int q = 0; q < Q; q++) {
        if (!ok[q]) break;
        const uint32_t c = cw[q] & 0xff;
        const uint32_t a = leaf_slot(linev[q], S[q], c, lane);
        bool del = false;
        for (uint32_t j = 0; j < k[q]; j++) del |= (__shfl_sync(0xffffffffu, d[q], j) == a);
        const bool keep = (uint32_t)lane < c && !del;
        const uint32_t mask = __ballot_sync(0xffffffffu, keep);
        const uint32_t pos = __popc(mask & ((1u << lane) - 1u));
        if (g.vals) {
          const uint32_t av = (uint32_t)lane < c ? g.vals[S[q] + lane] : 0u;
          __syncwarp();  // every value read before any is moved
          if (keep) g.vals[S[q] + pos] = av;
        }
        // the ids come from registers: no lane reads the line again
        if (keep) g.slots[S[q] + pos] = a;
        if ((uint32_t)lane >= c - k[q] && (uint32_t)lane < c) g.slots[S[q] + lane] = kEmpty;
      }
    }
    // the chunk's bookkeeping, lane l for group l
    const uint32_t gid = (uint32_t)(w * 32) + lane;
    bool to_climb = false;
    if (okl) {
      const uint32_t nc = (cwl & 0xff) - kl;  // every item of a group is present
      if (cwl & kMultiLeaf) g.lcnt[Sl >> kLeafLog] = (uint8_t)nc;
      atomicSub(&g.deg[ul], kl);
      uint8_t type = kNone;
      uint32_t lev = 0, w0 = leafl, w1 = leafl + 1;
      if (capl <= kLeaf) {
        if (nc == 0 || (capl > 1 && 4 * nc <= capl)) {
          type = kResize;
          lev = 31;
          w0 = 0;
          w1 = 1;
        }
      } else if (nc < lo_leaf) {
        to_climb = true;
      }
      gtype[gid] = type;
      glev[gid] = (uint8_t)lev;
      gw0[gid] = w0;
      gw1[gid] = w1;
    }
    // one reservation in the climb list for the warp's climbing groups
    const uint32_t cm = __ballot_sync(0xffffffffu, to_climb);
    if (cm) {
      uint32_t at = 0;
      if (lane == __ffs(cm) - 1) at = atomicAdd(nclimb, (uint32_t)__popc(cm));
      at = __shfl_sync(0xffffffffu, at, __ffs(cm) - 1);
      if (to_climb) climb[at + __popc(cm & ((1u << lane) - 1u))] = gid;
    }
  }
}

// window density bounds by segment height H (2^H leaves, H < kBoundsH: a
// segment holds at most 2^33 slots) and window level t <= H: entry
// [H * kBoundsH + t] of the table, window_upper for inserts, window_lower
// (the second table) for removes
constexpr uint32_t kBoundsH = 32;

// warp per climbing group: the smallest aligned window of 2^t leaves that
// meets the density bound (insert: upper bound with the batch's new ids in
// the window counted; remove: lower bound), else a resize of the segment
__global__ void k_climb(DGraph g, const uint64_t *__restrict__ bound, bool insert,
                        const uint64_t *__restrict__ p_ul,
                        const uint32_t *__restrict__ g_start,
                        const uint32_t *__restrict__ d_nitems,
                        const uint32_t *__restrict__ climb,
                        const uint32_t *__restrict__ nclimb,
                        uint8_t *__restrict__ gtype, uint8_t *__restrict__ glev,
                        uint32_t *__restrict__ gw0, uint32_t *__restrict__ gw1) {
  pdl_wait();
  const int lane = threadIdx.x & 31;
  const uint32_t nc = *nclimb, nitems = *d_nitems;
  for (uint64_t ci = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       ci < nc; ci += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    uint32_t gid = climb[ci];
    uint32_t j0 = g_start[gid];
    uint64_t key = p_ul[j0];
    uint32_t u = (uint32_t)(key >> 32), leaf = (uint32_t)key;
    uint32_t cap = g.cap[u];
    uint64_t lbase = g.base[u] >> kLeafLog;
    uint32_t H = log2_floor(cap >> kLeafLog);
    uint64_t cur = g.lcnt[lbase + leaf];
    uint32_t w0 = leaf, size = 1, w1 = leaf + 1, lev = 31;
    uint8_t type = kResize;
    const uint64_t kk = (uint64_t)u << 32;
    // new items of the growing window: bounds inside the row's items, the
    // lower one only moving left and the upper one only right
    uint32_t rb = 0, re = 0, ib = 0, ie = 0;
    if (insert) {
      rb = warp_lb_u64(p_ul, 0, j0 + 1, kk);
      re = warp_lb_u64(p_ul, j0, nitems, kk + (1ull << 32));
      ib = j0;
      ie = j0;
    }
    for (uint32_t t = 1; t <= H; t++) {
      uint32_t nw0 = (leaf >> t) << t;
      if (nw0 == w0)
        cur += warp_sum_lcnt(g.lcnt, lbase + w0 + size, lbase + w0 + 2 * size);
      else
        cur += warp_sum_lcnt(g.lcnt, lbase + nw0, lbase + w0);
      w0 = nw0;
      size <<= 1;
      w1 = w0 + size;
      bool ok;
      if (insert) {
        ib = warp_lb_u64(p_ul, rb, ib + 1 < re ? ib + 1 : re, kk | w0);
        ie = warp_lb_u64(p_ul, ie, re, kk | w1);
        ok = cur + (ie - ib) <= bound[H * kBoundsH + t];
      } else {
        ok = cur >= bound[H * kBoundsH + t];
      }
      if (ok) {
        type = kWindow;
        lev = t;
        break;
      }
    }
    if (type == kResize) {
      w0 = 0;
      w1 = cap >> kLeafLog;
    }
    if (lane == 0) {
      gtype[gid] = type;
      glev[gid] = (uint8_t)lev;
      gw0[gid] = w0;
      gw1[gid] = w1;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- step 7
constexpr uint64_t kWinMask = (1ull << 27) - 1;

__global__ void k_dom_keys(const uint64_t *__restrict__ p_ul,
                           const uint32_t *__restrict__ g_start,
                           const uint8_t *__restrict__ gtype,
                           const uint8_t *__restrict__ glev,
                           const uint32_t *__restrict__ gw0,
                           const uint32_t *__restrict__ gw1,
                           const uint32_t *__restrict__ d_ngroups, uint64_t gmax,
                           uint64_t *__restrict__ fkey,
                           uint64_t *__restrict__ bkey) {
  pdl_wait();
  uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= gmax) return;
  uint64_t f = 0, bk = ~0ull;
  if (gid < *d_ngroups && gtype[gid] >= kWindow) {
    uint64_t u = p_ul[g_start[gid]] >> 32;
    uint64_t lev = glev[gid];
    f = (u << 32) | ((uint64_t)gw1[gid] << 5) | lev;
    bk = (u << 32) | ((uint64_t)gw0[gid] << 5) | (31 - lev);
  }
  fkey[gid] = f;
  bkey[gid] = bk;
}

// fscan[g] = max of fkey over groups before g, bscan[g] = min of bkey over
// groups after g.  A group is covered when a window of the same row from
// either side contains its leaf and is larger (or equal and earlier).
__global__ void k_dom_classify(const uint64_t *__restrict__ p_ul,
                               const uint32_t *__restrict__ g_start,
                               const uint8_t *__restrict__ gtype,
                               const uint8_t *__restrict__ glev,
                               const uint64_t *__restrict__ fscan,
                               const uint64_t *__restrict__ bscan,
                               const uint32_t *__restrict__ d_ngroups,
                               uint64_t gmax, uint64_t *__restrict__ mt) {
  pdl_wait();
  uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= gmax) return;
  uint32_t mf = 0, tf = 0;
  if (gid < *d_ngroups && gtype[gid] != kNone) {
    uint64_t key = p_ul[g_start[gid]];
    uint64_t u = key >> 32;
    uint32_t leaf = (uint32_t)key;
    uint64_t L = fscan[gid], R = bscan[gid];
    bool lcov = L != 0 && (L >> 32) == u && ((L >> 5) & kWinMask) > leaf;
    bool rcov = R != ~0ull && (R >> 32) == u && ((R >> 5) & kWinMask) <= leaf;
    uint32_t lt = (uint32_t)(L & 31), rt = 31u - (uint32_t)(R & 31);
    if (gtype[gid] == kMerge) {
      mf = !(lcov || rcov);
    } else {
      uint32_t lev = glev[gid];
      bool dom = (lcov && lt >= lev) || (rcov && rt > lev);
      tf = !dom;
    }
  }
  // merge flag in the low word, task flag in the high word: one scan of
  // the packed words gives both positions (the counts stay below 2^32)
  mt[gid] = ((uint64_t)tf << 32) | mf;
}


// ---------------------------------------------------------------- step 8
struct Tasks {
  uint32_t *u;
  uint32_t *w0;      // first source/destination leaf (0 for a resize)
  uint64_t *key;     // (u << 32) | w0, ascending
  uint64_t *nsrc;    // leaves read
  uint64_t *ndst;    // leaves written
  uint32_t *newbeg;  // range of packed items merged in (insert)
  uint32_t *newend;
  uint64_t *total;   // elements after the task
  uint64_t *capn;    // new capacity (resize), else 0
  uint32_t *rank;    // rank within the capacity class (resize)
  uint8_t *type;
  uint64_t *out;     // exclusive prefix of total: staging offset
  uint64_t *soff;    // exclusive prefix of nsrc
  uint64_t *doff;    // exclusive prefix of ndst
  unsigned long long *err;  // count of out-of-range staging ranks
  uint32_t *stage_v;        // weighted graphs: values staged beside the ids
  const uint32_t *p_w;      // weighted graphs: values of the packed items
};

// A task's record (the setup kernels below write it).
__device__ __forceinline__ void task_store(Tasks &t, uint64_t tid, uint32_t u, uint32_t w0,
                                           uint64_t nsrc, uint64_t ndst, uint32_t nb,
                                           uint32_t ne, uint64_t old, uint64_t capn,
                                           uint32_t rank, uint8_t type) {
  t.u[tid] = u;
  t.w0[tid] = w0;
  t.key[tid] = ((uint64_t)u << 32) | w0;
  t.nsrc[tid] = nsrc;
  t.ndst[tid] = ndst;
  t.newbeg[tid] = nb;
  t.newend[tid] = ne;
  t.total[tid] = old + (ne - nb);
  t.capn[tid] = capn;
  t.rank[tid] = rank;
  t.type[tid] = type;
}

// Each group's outputs from the merge/task scan: a merge group's item range
// (and, on an insert, "no task" for its items in itask), a task group's
// slot.  The lane of a task group then sets the task up when it is a
// resize of a one-leaf row -- the common task: the row has one group, so
// its new items are that group's (no search), and the lanes'
// capacity-class ranks come from one atomic per class and warp -- and
// lists every other task (windows, resizes of multi-leaf rows) for
// k_task_setup_hard, which takes them a warp each (a window's leaf counts
// and the row's item range by warp searches).
// k_emit's work for one group (gid with its packed flags f and positions
// p; f = 0 for a lane without a group).  Every lane of the warp calls it
// together: the class ranks and the hard list are reserved per warp.
struct EmitArgs {
  uint64_t gmax;
  const uint32_t *g_start;
  uint64_t *merge_jk;
  uint32_t *task_group;
  uint64_t inv_fill;
  bool insert;
  const uint64_t *p_ul;
  const uint32_t *p_c;  // items' count words (k_locate)
  const uint8_t *gtype;
  Tasks t;
  uint32_t *class_cnt, *hard, *nhard, *itask;
};

__device__ __forceinline__ void emit_group(const EmitArgs &a, uint64_t gid, uint64_t f,
                                           uint64_t p) {
  const uint64_t gmax = a.gmax;
  const uint32_t *__restrict__ g_start = a.g_start;
  const uint64_t *__restrict__ p_ul = a.p_ul;
  const uint8_t *__restrict__ gtype = a.gtype;
  const bool insert = a.insert;
  uint32_t *itask = a.itask;
  const int lane = threadIdx.x & 31;
  const uint32_t full = 0xffffffffu;
  const uint32_t mpos = (uint32_t)p, tpos = (uint32_t)(p >> 32);
  if ((uint32_t)f && mpos < gmax) {
    const uint32_t j0 = g_start[gid], j1 = g_start[gid + 1];
    a.merge_jk[mpos] = ((uint64_t)j0 << 32) | (j1 - j0);
    if (itask)
      for (uint32_t j = j0; j < j1; j++) itask[j] = kEmpty;
  }
  const bool task = (f >> 32) && tpos < gmax;
  bool simple = false;
  uint32_t cls = kEmpty;  // capacity class taking a rank, else none
  uint32_t u = 0, cap = 0, deg = 0, nb = 0, ne = 0;
  uint64_t capn = 0;
  uint8_t type = kNone;
  if (task) {
    a.task_group[tpos] = (uint32_t)gid;
    const uint32_t j0 = g_start[gid];
    type = gtype[gid];
    u = (uint32_t)(p_ul[j0] >> 32);
    // the count word of the group's first item holds a one-leaf row's
    // capacity and count as the batch found them (no vertex record read):
    // an insert has not changed the row yet; a remove's one group of the
    // row has taken its items off (all present)
    const uint32_t cw = a.p_c[j0];
    simple = type != kWindow && !(cw & kMultiLeaf);  // a resize of a one-leaf (or empty) row
    if (simple) {
      cap = one_leaf_cap(cw);
      const uint32_t j1 = g_start[gid + 1];
      deg = insert ? (cw & 0xff) : (cw & 0xff) - (j1 - j0);
      if (insert) {
        nb = j0;
        ne = j1;
      }
      capn = cap_for((uint64_t)deg + (ne - nb), a.inv_fill);
      if (capn > 0) cls = log2_floor(capn);
    }
  }
  // one rank reservation per class among the warp's simple lanes
  const uint32_t peers = __match_any_sync(full, cls);
  const int leader = __ffs(peers) - 1;
  uint32_t rbase = 0;
  if (cls != kEmpty && lane == leader) rbase = atomicAdd(&a.class_cnt[cls], (uint32_t)__popc(peers));
  rbase = __shfl_sync(full, rbase, leader);
  if (simple) {
    const uint32_t rank = cls != kEmpty ? rbase + __popc(peers & ((1u << lane) - 1u)) : 0u;
    const uint64_t ndst = capn == 0 ? 0 : nleaves_of((uint32_t)capn);
    Tasks t = a.t;
    task_store(t, tpos, u, 0, cap == 0 ? 0 : nleaves_of(cap), ndst, nb, ne, deg, capn, rank,
               type);
  }
  // the rest to k_task_setup_hard, one reservation for the warp
  const uint32_t hm = __ballot_sync(full, task && !simple);
  if (hm) {
    uint32_t at = 0;
    if (lane == __ffs(hm) - 1) at = atomicAdd(a.nhard, (uint32_t)__popc(hm));
    at = __shfl_sync(full, at, __ffs(hm) - 1);
    if (task && !simple) a.hard[at + __popc(hm & ((1u << lane) - 1u))] = tpos;
  }
}

__global__ void k_emit(const uint64_t *__restrict__ mt, const uint64_t *__restrict__ mtpos,
                       EmitArgs a) {
  pdl_wait();
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = gid < a.gmax;  // no early return: the warp votes in emit_group
  emit_group(a, gid, in ? mt[gid] : 0, in ? mtpos[gid] : 0);
}

__global__ void k_task_setup_hard(DGraph g, uint64_t inv_fill, bool insert,
                                  const uint64_t *__restrict__ p_ul,
                                  const uint32_t *__restrict__ g_start,
                                  const uint8_t *__restrict__ gtype,
                                  const uint32_t *__restrict__ gw0,
                                  const uint32_t *__restrict__ gw1,
                                  const uint32_t *__restrict__ task_group,
                                  const uint32_t *__restrict__ hard,
                                  const uint32_t *__restrict__ nhard,
                                  const uint32_t *__restrict__ d_nitems, Tasks t,
                                  uint32_t *__restrict__ class_cnt) {
  pdl_wait();
  const int lane = threadIdx.x & 31;
  const uint32_t nh = *nhard, nitems = *d_nitems;
  for (uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nh;
       i += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
    const uint32_t tid = hard[i];
    const uint32_t gid = task_group[tid];
    const uint32_t j0 = g_start[gid];
    const uint32_t u = (uint32_t)(p_ul[j0] >> 32);
    const uint8_t type = gtype[gid];
    const uint64_t base = g.base[u];
    const uint32_t cap = g.cap[u];
    const uint64_t kk = (uint64_t)u << 32;
    uint32_t w0, b = 0, e = 0, rank = 0;
    uint64_t nsrc, ndst, old, capn = 0;
    if (type == kWindow) {
      w0 = gw0[gid];
      const uint32_t w1 = gw1[gid];
      nsrc = w1 - w0;
      old = warp_sum_lcnt(g.lcnt, (base >> kLeafLog) + w0, (base >> kLeafLog) + w1);
      if (insert) {  // the group's first item lies between the two bounds
        b = warp_lb_u64(p_ul, 0, j0 + 1, kk | w0);
        e = warp_lb_u64(p_ul, j0, nitems, kk | w1);
      }
      ndst = nsrc;
    } else {
      w0 = 0;
      nsrc = cap == 0 ? 0 : nleaves_of(cap);
      old = g.deg[u];
      if (insert) {
        b = warp_lb_u64(p_ul, 0, j0 + 1, kk);
        e = warp_lb_u64(p_ul, j0, nitems, kk + (1ull << 32));
      }
      capn = cap_for(old + (e - b), inv_fill);
      ndst = capn == 0 ? 0 : nleaves_of((uint32_t)capn);
      if (lane == 0 && capn > 0) rank = atomicAdd(&class_cnt[log2_floor(capn)], 1u);
    }
    if (lane == 0) task_store(t, tid, u, w0, nsrc, ndst, b, e, old, capn, rank, type);
    __syncwarp();
  }
}

// The plan summary to the host, written by one block straight into the
// pinned host copy (mapped), with the staging-rank error count of the batches
// before it; a kernel follows the planning kernels at once (programmatic
// launch), where a copy-engine transfer would start only after they finish.
static_assert(sizeof(PlanSummary) % 8 == 0 && offsetof(PlanSummary, apply_err) % 8 == 0,
              "the plan summary is copied as 8-byte words");
__global__ void k_plan_out(const PlanSummary *__restrict__ P,
                           const unsigned long long *__restrict__ err,
                           PlanSummary *__restrict__ host) {
  pdl_wait();
  constexpr int kWords = (int)(sizeof(PlanSummary) / 8);
  constexpr int kErrWord = (int)(offsetof(PlanSummary, apply_err) / 8);
  const unsigned long long *src = reinterpret_cast<const unsigned long long *>(P);
  unsigned long long *dst = reinterpret_cast<unsigned long long *>(host);
  for (int i = threadIdx.x; i < kWords; i += blockDim.x) dst[i] = i == kErrWord ? *err : src[i];
}
// the staging-rank error count alone (the end of a host-pointer call)
__global__ void k_err_out(const unsigned long long *__restrict__ err,
                          unsigned long long *__restrict__ host) {
  pdl_wait();
  if (threadIdx.x == 0) *host = *err;
}

// ---------------------------------------------------------------- step 9
// merge_jk[t] = (first item << 32) | item count of merge group t.  A warp
// takes 32 groups at a time: lane l first loads group l's item range and its
// first item's leaf start and count word (two dependent loads for all 32
// groups at once), then the groups go kGroupsPerWarp at a time with their
// items and leaf lines loaded together, one dependent load per batch.
__global__ void __launch_bounds__(256, 4)
k_leaf_merge(DGraph g, const uint64_t *__restrict__ p_ul, const uint32_t *__restrict__ p_x,
             const uint64_t *__restrict__ p_S, const uint32_t *__restrict__ p_c,
             const uint64_t *__restrict__ merge_jk, const uint32_t *__restrict__ d_nmerge,
             const uint32_t *__restrict__ p_w) {
  pdl_wait();
  __shared__ uint8_t glist[kLeafWarps][32];
  const int lane = threadIdx.x & 31, sub = lane & 7;
  uint8_t *list = glist[threadIdx.x >> 5];
  constexpr int Q = kGroupsPerWarp;
  const uint32_t nmerge = *d_nmerge;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       w * 32 < nmerge; w += nw) {
    const uint64_t gl = w * 32 + lane;
    const bool okl = gl < nmerge;
    const uint64_t jkl = okl ? merge_jk[gl] : 0;
    const uint32_t j0l = (uint32_t)(jkl >> 32), kl = (uint32_t)jkl;
    const uint64_t Sl = okl ? p_S[j0l] : 0;
    const uint32_t cwl = okl ? p_c[j0l] : 0;
    const uint32_t ul = okl ? (uint32_t)(p_ul[j0l] >> 32) : 0u;
    const uint32_t cnt = nmerge - w * 32 < 32 ? (uint32_t)(nmerge - w * 32) : 32u;
    // one-item groups: the new id goes to the count of the slots below it,
    // the slots from there up move one place right
    const uint32_t n1 = list_groups(list, okl, kl == 1 && !g.vals, lane);
    for (uint32_t f0 = 0; f0 < n1; f0 += 4) {
      const uint32_t f = f0 + (lane >> 3);
      const bool on = f < n1;
      const int src = list[on ? f : 0];
      const uint32_t j0 = __shfl_sync(0xffffffffu, j0l, src);
      const uint64_t S = __shfl_sync(0xffffffffu, Sl, src);
      const uint32_t cw = __shfl_sync(0xffffffffu, cwl, src);
      const uint32_t c = on ? (cw & 0xff) : 0u;
      const uint32_t x = on ? p_x[j0] : kEmpty;
      uint32_t a[4];
      load_quarter(g.slots, S, c, sub, a);
      const uint32_t pos = below_in_octet(a, x);
      const uint32_t prev = __shfl_up_sync(0xffffffffu, a[3], 1, 8);
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const uint32_t p = 4 * sub + r;
        if (on && p >= pos && p <= c) g.slots[S + p] = p == pos ? x : (r ? a[r - 1] : prev);
      }
    }
    // the other groups: a warp each, kGroupsPerWarp at a time
    const uint32_t nrest = cnt - n1;
    for (uint32_t q0 = 0; q0 < nrest; q0 += Q) {
      uint32_t j0[Q], k[Q], x[Q], linev[Q], cw[Q];
      uint64_t S[Q];
      bool ok[Q];
#pragma unroll
      for (int q = 0; q < Q; q++) {
        ok[q] = q0 + q < nrest;
        const int src = list[n1 + (ok[q] ? q0 + q : 0)];
        j0[q] = __shfl_sync(0xffffffffu, j0l, src);
        k[q] = ok[q] ? __shfl_sync(0xffffffffu, kl, src) : 0;
        S[q] = __shfl_sync(0xffffffffu, Sl, src);
        cw[q] = __shfl_sync(0xffffffffu, cwl, src);
      }
#pragma unroll
      for (int q = 0; q < Q; q++) {
        x[q] = (uint32_t)lane < k[q] ? p_x[j0[q] + lane] : kEmpty;
        linev[q] = ok[q] ? g.slots[(S[q] & ~uint64_t(kLeaf - 1)) + lane] : kEmpty;
      }
#pragma unroll
      for (int q = 0; q < Q; q++) {
        if (!ok[q]) break;
        const uint32_t c = cw[q] & 0xff;
        const uint32_t a = leaf_slot(linev[q], S[q], c, lane);
        // merged ranks in O(k) steps (k new ids, usually one or two): an old
        // id moves up by the new ids below it; new id j lands at j + the old
        // ids below it (a ballot per new id)
        uint32_t pa = lane, px = lane;
        for (uint32_t j = 0; j < k[q]; j++) {
          uint32_t xj = __shfl_sync(0xffffffffu, x[q], j);
          pa += xj < a;
          uint32_t below = __popc(__ballot_sync(0xffffffffu, (uint32_t)lane < c && a < xj));
          if ((uint32_t)lane == j) px = j + below;
        }
        // values move with their ids (weighted graphs)
        if (g.vals) {
          const uint32_t av = (uint32_t)lane < c ? g.vals[S[q] + lane] : 0u;
          const uint32_t xv = (uint32_t)lane < k[q] ? (p_w ? p_w[j0[q] + lane] : 1u) : 0u;
          __syncwarp();  // every value read before any is moved
          if ((uint32_t)lane < c) g.vals[S[q] + pa] = av;
          if ((uint32_t)lane < k[q]) g.vals[S[q] + px] = xv;
        }
        // the ids come from registers: no lane reads the line again
        if ((uint32_t)lane < c) g.slots[S[q] + pa] = a;
        if ((uint32_t)lane < k[q]) g.slots[S[q] + px] = x[q];
      }
    }
    // the chunk's leaf counts and degrees, lane l for group l.  No task
    // reads these rows' degrees: a one-leaf row is one group (a merge or a
    // resize), and a row with a resize task has no merge group.
    if (okl) {
      if (cwl & kMultiLeaf) g.lcnt[Sl >> kLeafLog] = (uint8_t)((cwl & 0xff) + kl);
      atomicAdd(&g.deg[ul], kl);
    }
  }
}

// the task of every source and destination leaf of the window / resize
// tasks (a warp per task fills its two ranges), so the apply kernels find a
// leaf's task with one load, not a binary search over the offsets; the
// source leaves' element counts beside (scnt); and, on an insert, the task
// of each new item that a task takes (k_emit marked the merged items)
// (eight lanes a task: most tasks resize a one-leaf row, one leaf each way)
__global__ void k_task_index(DGraph g, Tasks t, uint32_t ntasks, uint32_t *__restrict__ stask,
                             uint32_t *__restrict__ dtask, uint32_t *__restrict__ itask,
                             uint64_t *__restrict__ scnt) {
  pdl_wait();
  const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const uint32_t sub = threadIdx.x & 7;
  if (w >= ntasks) return;
  const uint64_t s0 = t.soff[w], ns = t.nsrc[w], d0 = t.doff[w], nd = t.ndst[w];
  if (ns) {
    const uint32_t u = t.u[w], l0 = t.w0[w];
    const uint64_t base = g.base[u];
    const uint32_t cap = g.cap[u], deg = g.deg[u];
    for (uint64_t j = sub; j < ns; j += 8) {
      stask[s0 + j] = (uint32_t)w;
      scnt[s0 + j] = leaf_count(g, base, cap, deg, l0 + (uint32_t)j);
    }
  }
  for (uint64_t j = sub; j < nd; j += 8) dtask[d0 + j] = (uint32_t)w;
  if (itask)
    for (uint32_t j = t.newbeg[w] + sub; j < t.newend[w]; j += 8) itask[j] = (uint32_t)w;
}


// old elements to their merged rank: eight lanes per source leaf, lane
// `sub` taking slots sub, sub + 8, sub + 16, sub + 24, four leaves a warp
// (the chain of dependent loads -- task, row, count, ids, rank among the
// task's new ids -- is paid once per four leaves, not once per leaf)
__global__ void k_gather_old(DGraph g, Tasks t, uint32_t ntasks,
                             uint64_t nsrc_total,
                             const uint64_t *__restrict__ spre,
                             const uint32_t *__restrict__ p_x,
                             uint32_t *__restrict__ stage,
                             const uint32_t *__restrict__ stask) {
  pdl_wait();
  const uint64_t s = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const uint32_t sub = threadIdx.x & 7;
  if (s >= nsrc_total) return;
  const uint64_t tau = stask[s];
  const uint32_t u = t.u[tau];
  const uint64_t soff = t.soff[tau];
  const uint32_t l = t.w0[tau] + (uint32_t)(s - soff);
  const uint64_t base = g.base[u];
  const uint32_t c = leaf_count(g, base, g.cap[u], g.deg[u], l);
  if (sub >= c) return;
  const uint64_t at = base + ((uint64_t)l << kLeafLog);
  uint32_t a[4], below[4];
#pragma unroll
  for (int r = 0; r < 4; r++) a[r] = sub + 8 * r < c ? g.slots[at + sub + 8 * r] : kEmpty;
  count_less4(p_x, t.newbeg[tau], t.newend[tau], a, below);
  const uint64_t r0 = spre[s] - spre[soff], total = t.total[tau], out = t.out[tau];
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const uint32_t p = sub + 8 * r;
    if (p >= c) break;
    const uint64_t rank = r0 + p + below[r];
    if (rank >= total) {
      atomicAdd(t.err, 1ull);
      continue;
    }
    stage[out + rank] = a[r];
    if (t.stage_v) t.stage_v[out + rank] = g.vals[at + p];
  }
}

// thread per packed item owned by a task: new elements to their merged rank
__global__ void k_gather_new(DGraph g, Tasks t, uint32_t ntasks,
                             const uint64_t *__restrict__ spre,
                             const uint64_t *__restrict__ p_ul,
                             const uint32_t *__restrict__ p_x, uint32_t nitems,
                             uint32_t *__restrict__ stage,
                             const uint32_t *__restrict__ itask) {
  pdl_wait();
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nitems || ntasks == 0) return;
  const uint32_t tau = itask[j];
  if (tau >= ntasks) return;  // a leaf merge takes this item (kEmpty)
  const uint32_t u = (uint32_t)(p_ul[j] >> 32);
  uint32_t x = p_x[j];
  uint64_t base = g.base[u];
  uint32_t cap = g.cap[u], deg = g.deg[u];
  uint64_t old_less = 0;
  uint32_t nsrc = (uint32_t)t.nsrc[tau];
  if (nsrc > 0) {
    uint32_t w0 = t.w0[tau];
    uint32_t lo = 0, hi = nsrc;  // last leaf of the window with head <= x
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (g.slots[base + ((uint64_t)(w0 + mid) << kLeafLog)] <= x)
        lo = mid;
      else
        hi = mid;
    }
    uint32_t l = w0 + lo;
    uint32_t c = leaf_count(g, base, cap, deg, l);
    uint32_t pos = leaf_lower_bound(g.slots + base + ((uint64_t)l << kLeafLog), c, x);
    uint64_t s0 = t.soff[tau];
    old_less = (spre[s0 + lo] - spre[s0]) + pos;
  }
  uint64_t rank = (j - t.newbeg[tau]) + old_less;
  if (rank >= t.total[tau]) {
    atomicAdd(t.err, 1ull);
    return;
  }
  stage[t.out[tau] + rank] = x;
  if (t.stage_v) t.stage_v[t.out[tau] + rank] = t.p_w ? t.p_w[j] : 1u;
}

// first slab slot of each capacity class's new segments (largest class
// first), passed by value: the apply kernels need no copy of it on the device
struct ClassStarts {
  uint64_t s[kNumClasses];
};

__device__ __forceinline__ uint64_t task_new_base(const Tasks &t, uint64_t tau,
                                                  const ClassStarts &cs) {
  const uint64_t *class_start = cs.s;
  uint64_t capn = t.capn[tau];
  return class_start[log2_floor(capn)] + (uint64_t)t.rank[tau] * capn;
}

// even redistribution of the staged elements: eight lanes per destination
// leaf (slots sub, sub + 8, sub + 16, sub + 24), four leaves a warp.  Each
// lane finds the leaf's task and its share of the task's elements itself
// (the loads are the same address across the eight; 32-bit arithmetic: a
// task holds fewer than 2^32 elements).
__global__ void k_task_scatter(DGraph g, Tasks t, uint32_t ntasks,
                               uint64_t ndst_total,
                               const ClassStarts class_start,
                               const uint32_t *__restrict__ stage,
                               const uint32_t *__restrict__ dtask) {
  pdl_wait();
  const uint64_t d = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const uint32_t sub = threadIdx.x & 7;
  if (d >= ndst_total) return;
  const uint64_t tau = dtask[d];
  const uint32_t i = (uint32_t)(d - t.doff[tau]);
  const uint32_t NL = (uint32_t)t.ndst[tau], T = (uint32_t)t.total[tau];
  const uint32_t per = T / NL, ext = T - per * NL;
  const uint32_t cnt = per + (i < ext);
  const uint64_t src = t.out[tau] + (uint64_t)i * per + (i < ext ? i : ext);
  uint64_t S;
  uint32_t leafsize = kLeaf;
  bool multi = true;
  if (t.type[tau] == kResize) {
    const uint64_t capn = t.capn[tau];
    S = task_new_base(t, tau, class_start) + ((uint64_t)i << kLeafLog);
    if (capn <= kLeaf) {
      leafsize = (uint32_t)capn;
      multi = false;
    }
  } else {
    S = g.base[t.u[tau]] + ((uint64_t)(t.w0[tau] + i) << kLeafLog);
  }
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const uint32_t p = sub + 8 * r;
    if (p < leafsize) g.slots[S + p] = p < cnt ? stage[src + p] : kEmpty;
    if (g.vals && p < cnt) g.vals[S + p] = t.stage_v[src + p];
  }
  if (sub == 0 && multi) g.lcnt[S >> kLeafLog] = (uint8_t)cnt;
}

// resized rows get their new segment; every task's row gets the new items
// the task took (an insert's items are each taken by one merge group or one
// task, and the merge kernel counts its own)
__global__ void k_finalize(DGraph g, Tasks t, uint32_t ntasks,
                           const ClassStarts class_start) {
  pdl_wait();
  uint64_t tau = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tau >= ntasks) return;
  uint32_t u = t.u[tau];
  const uint32_t added = t.newend[tau] - t.newbeg[tau];
  if (added) atomicAdd(&g.deg[u], added);
  if (t.type[tau] != kResize) return;
  uint64_t capn = t.capn[tau];
  g.base[u] = capn ? task_new_base(t, tau, class_start) : 0;
  g.cap[u] = (uint32_t)capn;
}

// ---------------------------------------------------------------- repack
__global__ void k_class_count(const uint32_t *__restrict__ cap, uint32_t n,
                              uint32_t *__restrict__ cnt) {
  pdl_wait();
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n || cap[v] == 0) return;
  atomicAdd(&cnt[log2_floor(cap[v])], 1u);
}

__global__ void k_repack_assign(const uint32_t *__restrict__ cap, uint32_t n,
                                const uint64_t *__restrict__ class_start,
                                uint32_t *__restrict__ ctr,
                                uint64_t *__restrict__ newbase) {
  pdl_wait();
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  uint32_t c = cap[v];
  if (c == 0) {
    newbase[v] = 0;
    return;
  }
  uint32_t cls = log2_floor(c);
  newbase[v] = class_start[cls] + (uint64_t)atomicAdd(&ctr[cls], 1u) * c;
}

__global__ void k_repack_copy(const uint32_t *__restrict__ cap, uint32_t n,
                              const uint64_t *__restrict__ oldbase,
                              const uint64_t *__restrict__ newbase,
                              const uint32_t *__restrict__ oslots,
                              const uint8_t *__restrict__ olcnt,
                              uint32_t *__restrict__ nslots_,
                              uint8_t *__restrict__ nlcnt,
                              const uint32_t *__restrict__ ovals,
                              uint32_t *__restrict__ nvals) {
  pdl_wait();
  uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (v >= n) return;
  uint32_t c = cap[v];
  if (c == 0) return;
  uint64_t ob = oldbase[v], nb = newbase[v];
  for (uint64_t i = lane; i < c; i += 32) nslots_[nb + i] = oslots[ob + i];
  if (ovals)
    for (uint64_t i = lane; i < c; i += 32) nvals[nb + i] = ovals[ob + i];
  if (c > kLeaf)
    for (uint64_t l = lane; l < (c >> kLeafLog); l += 32)
      nlcnt[(nb >> kLeafLog) + l] = olcnt[(ob >> kLeafLog) + l];
}


}  // namespace

// ====================================================================== host

static thread_local char g_errmsg[512];

void set_error_message(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
  va_end(ap);
}
void set_cuda_error(cudaError_t e, const char *what, const char *file,
                    int line) {
  set_error_message("CUDA error %s (%s) at %s:%d: %s", cudaGetErrorName(e),
                    cudaGetErrorString(e), file, line, what);
}
const char *error_message() { return g_errmsg; }

void LeafDir::release() {
  cudaFree(owner);
  cudaFree(slot);
  cudaFree(cnt);
  cudaFree(pre);
  cudaFree(vleaf);
  owner = nullptr;
  slot = nullptr;
  cnt = nullptr;
  pre = nullptr;
  vleaf = nullptr;
  cap = 0;
  nleaves = 0;
  version = ~0ull;
}

void *pinned(sst_graph *g, size_t bytes) {
  if (bytes <= g->h_pinned_cap) return g->h_pinned;
  if (g->h_pinned) cudaFreeHost(g->h_pinned);
  size_t want = bytes + bytes / 4 + 4096;
  if (cudaMallocHost(&g->h_pinned, want) != cudaSuccess) {
    g->h_pinned = nullptr;
    g->h_pinned_cap = 0;
    return nullptr;
  }
  g->h_pinned_cap = want;
  return g->h_pinned;
}

uint64_t graph_device_bytes(const sst_graph *g) {
  return (uint64_t)g->n * 16 + g->nslots * (g->weighted ? 8 : 4) + g->nslots / kLeaf +
         g->arena.cap + g->work.cap + g->io.cap +
         g->dir.cap * (4 + 8 + 4 + 8) + (uint64_t)(g->n + 1) * 8 + trav_device_bytes(g);
}

sst_status release_scratch(sst_graph *g) {
  sst_status st = sync_checked(g);  // reads the last batch's device check
  if (st != SST_OK) return st;
  if (g->side) SST_CUDA_TRY(cudaStreamSynchronize(g->side));
  plan_cache_release(g);  // captured launches point into the arena
  g->arena.release();
  g->work.release();
  g->io.release();
  g->dir.release();
  trav_trim(g);
  return SST_OK;
}

static sst_status budget_check(sst_graph *g, uint64_t extra) {
  if (g->budget && graph_device_bytes(g) + extra > g->budget) {
    set_error_message("HBM budget of %llu bytes exceeded (need %llu more)",
                      (unsigned long long)g->budget,
                      (unsigned long long)extra);
    return SST_EBUDGET;
  }
  return SST_OK;
}

static sst_status alloc_slab(sst_graph *g, uint64_t nslots, uint32_t **slots,
                             uint8_t **lcnt, uint32_t **vals) {
  if (cudaMalloc(slots, nslots * 4) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("cannot allocate a slab of %llu slots",
                      (unsigned long long)nslots);
    return SST_ENOMEM;
  }
  if (cudaMalloc(lcnt, nslots / kLeaf + 1) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(*slots);
    set_error_message("cannot allocate leaf counts");
    return SST_ENOMEM;
  }
  *vals = nullptr;
  if (g->weighted && cudaMalloc(vals, nslots * 4) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(*slots);
    cudaFree(*lcnt);
    set_error_message("cannot allocate a value slab of %llu slots",
                      (unsigned long long)nslots);
    return SST_ENOMEM;
  }
  return SST_OK;
}

sst_status graph_init(sst_graph *g, uint32_t height, uint32_t width,
                      const sst_config *cfg) {
  g->n = height;
  g->width = width;
  g->rbits = bits_for(height);
  g->dbits = std::max(1, bits_for(width ? width - 1 : 0));
  if (cfg) {
    g->device = cfg->device;
    g->budget = cfg->hbm_budget_bytes;
    if (cfg->upper_root > 0) g->params.upper_root = cfg->upper_root;
    if (cfg->lower_root > 0) g->params.lower_root = cfg->lower_root;
    if (cfg->grow_fill > 0) g->params.grow_fill = cfg->grow_fill;
    g->keep_loops = cfg->keep_self_loops != 0;
    g->weighted = cfg->weighted != 0;
  }
  SST_CUDA_TRY(cudaSetDevice(g->device));
  SST_CUDA_TRY(cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, g->device));
  SST_CUDA_TRY(cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking));
  g->stream = g->own_stream;
  uint64_t n = std::max<uint64_t>(height, 1);
  SST_CUDA_TRY(cudaMalloc(&g->d_base, n * 8));
  SST_CUDA_TRY(cudaMalloc(&g->d_cap, n * 4));
  SST_CUDA_TRY(cudaMalloc(&g->d_deg, n * 4));
  SST_CUDA_TRY(cudaMemsetAsync(g->d_base, 0, n * 8, g->stream));
  SST_CUDA_TRY(cudaMemsetAsync(g->d_cap, 0, n * 4, g->stream));
  SST_CUDA_TRY(cudaMemsetAsync(g->d_deg, 0, n * 4, g->stream));
  uint64_t slots = cfg && cfg->initial_slots ? cfg->initial_slots : (1ull << 20);
  slots = (slots + kLeaf - 1) & ~uint64_t(kLeaf - 1);
  sst_status st = budget_check(g, slots * 4 + slots / kLeaf);
  if (st != SST_OK) return st;
  st = alloc_slab(g, slots, &g->d_slots, &g->d_lcnt, &g->d_vals);
  if (st != SST_OK) return st;
  g->nslots = slots;
  g->bump = 0;
  SST_CUDA_TRY(cudaMallocHost(&g->h_plan, sizeof(PlanSummary)));
  SST_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void **>(&g->h_plan_dev), g->h_plan, 0));
  SST_CUDA_TRY(cudaMalloc(&g->d_plan, sizeof(PlanSummary)));
  SST_CUDA_TRY(cudaMalloc(&g->d_err, sizeof(unsigned long long)));
  SST_CUDA_TRY(cudaMemsetAsync(g->d_err, 0, sizeof(unsigned long long), g->stream));
  SST_CUDA_TRY(cudaMalloc(&g->d_scan_epoch, sizeof(unsigned long long)));
  SST_CUDA_TRY(cudaMemsetAsync(g->d_scan_epoch, 0, sizeof(unsigned long long), g->stream));
  // the climb's density bounds per (segment height, window level), computed
  // once here with the graph's parameters: no FP64 on the device
  std::vector<uint64_t> wb(2 * kBoundsH * kBoundsH, 0);
  for (uint32_t H = 0; H < kBoundsH; H++)
    for (uint32_t t = 0; t <= H; t++) {
      wb[H * kBoundsH + t] = window_upper(g->params, t, H);
      wb[kBoundsH * kBoundsH + H * kBoundsH + t] = window_lower(g->params, t, H);
    }
  SST_CUDA_TRY(cudaMalloc(&g->d_bounds, wb.size() * 8));
  SST_CUDA_TRY(cudaMemcpy(g->d_bounds, wb.data(), wb.size() * 8, cudaMemcpyHostToDevice));
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  return SST_OK;
}

void graph_release(sst_graph *g) {
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  cudaFree(g->d_base);
  cudaFree(g->d_cap);
  cudaFree(g->d_deg);
  cudaFree(g->d_slots);
  cudaFree(g->d_vals);
  cudaFree(g->d_lcnt);
  cudaFree(g->d_plan);
  cudaFree(g->d_err);
  cudaFree(g->d_bounds);
  cudaFree(g->d_scan_epoch);
  if (g->h_plan) cudaFreeHost(g->h_plan);
  if (g->h_pinned) cudaFreeHost(g->h_pinned);
  g->arena.release();
  g->work.release();
  g->dir.release();
  trav_release(g);
  if (g->own_stream) cudaStreamDestroy(g->own_stream);
  g->own_stream = nullptr;
  if (g->plan_ready) cudaEventDestroy(g->plan_ready);
  g->plan_ready = nullptr;
  plan_cache_release(g);
  if (g->side) cudaStreamDestroy(g->side);
  if (g->fork_ev) cudaEventDestroy(g->fork_ev);
  if (g->merge_done) cudaEventDestroy(g->merge_done);
  g->side = nullptr;
  g->fork_ev = g->merge_done = nullptr;
  for (int k = 0; k < 2; k++) {
    if (g->aux[k]) cudaStreamDestroy(g->aux[k]);
    if (g->aux_join[k]) cudaEventDestroy(g->aux_join[k]);
    g->aux[k] = nullptr;
    g->aux_join[k] = nullptr;
  }
  if (g->aux_fork) cudaEventDestroy(g->aux_fork);
  g->aux_fork = nullptr;
  g->stream = nullptr;
}

sst_status graph_clone(const sst_graph *src, sst_graph *dst) {
  sst_config cfg{};
  cfg.device = src->device;
  cfg.hbm_budget_bytes = src->budget;
  cfg.initial_slots = std::max<uint64_t>(src->nslots, kLeaf);
  cfg.upper_root = src->params.upper_root;
  cfg.lower_root = src->params.lower_root;
  cfg.grow_fill = src->params.grow_fill;
  cfg.keep_self_loops = src->keep_loops ? 1u : 0u;
  cfg.weighted = src->weighted ? 1u : 0u;
  sst_status st = graph_init(dst, src->n, src->width, &cfg);
  if (st != SST_OK) return st;
  SST_CUDA_TRY(cudaStreamSynchronize(src->stream));
  uint64_t n = std::max<uint64_t>(src->n, 1);
  SST_CUDA_TRY(cudaMemcpyAsync(dst->d_base, src->d_base, n * 8, cudaMemcpyDeviceToDevice, dst->stream));
  SST_CUDA_TRY(cudaMemcpyAsync(dst->d_cap, src->d_cap, n * 4, cudaMemcpyDeviceToDevice, dst->stream));
  SST_CUDA_TRY(cudaMemcpyAsync(dst->d_deg, src->d_deg, n * 4, cudaMemcpyDeviceToDevice, dst->stream));
  SST_CUDA_TRY(cudaMemcpyAsync(dst->d_slots, src->d_slots, src->bump * 4, cudaMemcpyDeviceToDevice, dst->stream));
  if (src->d_vals)
    SST_CUDA_TRY(cudaMemcpyAsync(dst->d_vals, src->d_vals, src->bump * 4, cudaMemcpyDeviceToDevice, dst->stream));
  SST_CUDA_TRY(cudaMemcpyAsync(dst->d_lcnt, src->d_lcnt, src->bump / kLeaf + 1, cudaMemcpyDeviceToDevice, dst->stream));
  SST_CUDA_TRY(cudaStreamSynchronize(dst->stream));
  dst->bump = src->bump;
  dst->m = src->m;
  dst->version = 1;
  return SST_OK;
}

// Move every live segment into a fresh slab, packed by capacity class, with
// room for `extra` more slots.  Freed segments are reclaimed here.
sst_status repack(sst_graph *g, uint64_t extra) {
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  // own temporaries: the arena may hold a batch in flight
  char *tmp = nullptr;
  uint64_t tbytes = 512 + (uint64_t)std::max<uint32_t>(n, 1) * 8;
  SST_CUDA_TRY(cudaMalloc(&tmp, tbytes));
  uint32_t *cnt = reinterpret_cast<uint32_t *>(tmp);
  uint64_t *cstart = reinterpret_cast<uint64_t *>(tmp + 256);
  uint64_t *newbase = reinterpret_cast<uint64_t *>(tmp + 512);
  SST_CUDA_TRY(cudaMemsetAsync(cnt, 0, kNumClasses * 8, s));
  if (n) SST_LAUNCH_PDL(k_class_count, blocks_for(n), kTB, 0, s, g->d_cap, n, cnt);
  uint32_t hcnt[kNumClasses];
  SST_CUDA_TRY(cudaMemcpyAsync(hcnt, cnt, sizeof(hcnt), cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t hstart[kNumClasses];
  uint64_t off = 0;
  for (int c = kNumClasses - 1; c >= 0; c--) {
    hstart[c] = off;
    off += (uint64_t)hcnt[c] << c;
  }
  uint64_t live = off;
  uint64_t need = live + extra + kLeaf;
  uint64_t nsl = g->nslots;
  if (need > nsl / 2 + nsl / 4) nsl = std::max<uint64_t>(2 * need, 1ull << 20);
  nsl = (nsl + kLeaf - 1) & ~uint64_t(kLeaf - 1);
  // the new slab coexists with the old one while segments move
  sst_status st = budget_check(g, nsl * 4 + nsl / kLeaf);
  if (st != SST_OK) {
    cudaFree(tmp);
    return st;
  }
  uint32_t *nslots_, *nvals;
  uint8_t *nlcnt;
  st = alloc_slab(g, nsl, &nslots_, &nlcnt, &nvals);
  if (st != SST_OK) {
    cudaFree(tmp);
    return st;
  }
  SST_CUDA_TRY(cudaMemcpyAsync(cstart, hstart, sizeof(hstart), cudaMemcpyHostToDevice, s));
  if (n) {
    SST_LAUNCH_PDL(k_repack_assign, blocks_for(n), kTB, 0, s, g->d_cap, n, cstart,
               cnt + kNumClasses, newbase);
    SST_LAUNCH_PDL(k_repack_copy, warp_blocks(n), kTB, 0, s, g->d_cap, n, g->d_base,
               newbase, g->d_slots, g->d_lcnt, nslots_, nlcnt, g->d_vals, nvals);
    SST_CUDA_TRY(cudaMemcpyAsync(g->d_base, newbase, (uint64_t)n * 8, cudaMemcpyDeviceToDevice, s));
  }
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  SST_CUDA_TRY(cudaGetLastError());
  cudaFree(g->d_slots);
  cudaFree(g->d_lcnt);
  cudaFree(g->d_vals);
  g->d_slots = nslots_;
  g->d_lcnt = nlcnt;
  g->d_vals = nvals;
  g->nslots = nsl;
  g->bump = live;
  cudaFree(tmp);
  return SST_OK;
}

// The graph's stream waits for an update's leaf merges on the side stream:
// at wait(), or when the pipeline returns early.
struct MergeJoin {
  cudaStream_t s;
  cudaEvent_t ev;
  void wait() {
    if (ev) cudaStreamWaitEvent(s, ev, 0);
    ev = nullptr;
  }
  ~MergeJoin() { wait(); }
};

// ------------------------------------------------ captured planning
// An update's planning launches (sort to plan readback) replayed as one CUDA
// graph.  They depend on the batch size, the operation and where the graph
// and the scratch live; an entry is used only when all of these match.
constexpr uint64_t kPlanGraphMaxBatch = 1u << 20;
constexpr size_t kPlanGraphs = 56;

// Launch size of a replayed batch of b pairs: b rounded up to m * 2^k with
// m in 4..7 (at least 64), so batches of nearby sizes share one captured
// sequence; at most a third more launch size than b, about 12% on average.
inline uint64_t plan_size_class(uint64_t b) {
  if (b <= 64) return 64;
  const int k = 63 - __builtin_clzll(b) - 2;  // b >> k is 4..7
  const uint64_t m = (b + (1ull << k) - 1) >> k;
  return m << k;  // m may reach 8: the next power of two
}

struct PlanKey {
  uint64_t b;
  bool insert;
  DGraph dg;
  PmaParams params;
  const char *arena;
  bool operator==(const PlanKey &o) const {
    return b == o.b && insert == o.insert && arena == o.arena &&
           memcmp(&dg, &o.dg, sizeof(DGraph)) == 0 &&
           memcmp(&params, &o.params, sizeof(PmaParams)) == 0;
  }
};
struct PlanCache {
  struct Entry {
    PlanKey key;
    cudaGraphExec_t exec;
    int64_t kernels;  // kernel launches in the captured sequence
    uint64_t used;
  };
  std::vector<Entry> entries;
  uint64_t tick = 0;
};

void plan_cache_release(sst_graph *g) {
  if (!g->plans) return;
  for (auto &e : g->plans->entries) cudaGraphExecDestroy(e.exec);
  delete g->plans;
  g->plans = nullptr;
}

// Launch the planning sequence `body` (a function of the stream it issues
// on) for this key on stream s: replayed when captured before, else captured
// on the graph's side stream first.  A capture that fails turns replay off
// for the graph; the sequence then runs directly.
template <typename Body>
static sst_status plan_graph_launch(sst_graph *g, uint64_t b, bool insert,
                                    const DGraph &dg, cudaStream_t s, Body body) {
  if (!g->plans) g->plans = new PlanCache;
  PlanCache &C = *g->plans;
  PlanKey key{b, insert, dg, g->params, g->arena.base};
  PlanCache::Entry *hit = nullptr;
  for (auto &e : C.entries)
    if (e.key == key) hit = &e;
  if (!hit) {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const uint64_t l0 = launches();
    const size_t mark = g->arena.used;
    cudaError_t e = cudaStreamBeginCapture(g->side, cudaStreamCaptureModeThreadLocal);
    sst_status st = SST_OK;
    if (e == cudaSuccess) {
      ProfPause quiet;
      st = body(g->side);
      e = cudaStreamEndCapture(g->side, &graph);
    }
    const int64_t kernels = (int64_t)(launches() - l0);
    note_launches(-kernels);  // captured, not launched
    if (e == cudaSuccess && st == SST_OK) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess || st != SST_OK) {
      cudaGetLastError();
      g->plan_graphs = false;
      g->arena.used = mark;
      return body(s);
    }
    if (C.entries.size() >= kPlanGraphs) {
      auto lru = std::min_element(C.entries.begin(), C.entries.end(),
                                  [](const PlanCache::Entry &x, const PlanCache::Entry &y) {
                                    return x.used < y.used;
                                  });
      cudaGraphExecDestroy(lru->exec);
      C.entries.erase(lru);
    }
    C.entries.push_back({key, exec, kernels, 0});
    hit = &C.entries.back();
  }
  hit->used = ++C.tick;
  cudaEvent_t ev = profiling("update_plan_graph") ? prof_begin(s) : nullptr;
  SST_CUDA_TRY(cudaGraphLaunch(hit->exec, s));
  if (ev) prof_end("update_plan_graph", ev, s, 0);
  note_launches(hit->kernels);
  return SST_OK;
}

// bytes of arena scratch an update batch of b pairs takes
static size_t update_scratch_bytes(uint64_t b) {
  size_t per = 8 * 2 + 4 * 5 + 8 + 4 + 4 * 3 + 1 * 2 + 4 * 2 + 8 * 4 + 4 * 6 +
               8 * 8 + 4 * 4 + 1 + 64 + 4 * 3 /* values */ +
               8 + 4 + 8 + 4 + 4 /* leaf starts and counts, merge ranges */;
  return b * per + radix_sort_scratch_bytes(b) + 8 * scan_scratch_bytes(b, 8) +
         (1 << 16);
}

// One pass of the update pipeline.  Either d_pairs (raw pairs: steps 1-2
// make and sort the keys) or presorted (keys already (row << dbits | col),
// ascending and duplicate-free, in memory outside the arena) is given.
static sst_status run_pipeline(sst_graph *g, const uint32_t *d_pairs,
                               const uint64_t *presorted, uint64_t b,
                               bool insert, uint64_t *n_invalid,
                               const uint32_t *d_w);

sst_status update_batch(sst_graph *g, const uint32_t *d_pairs, uint64_t b,
                        bool insert, uint64_t *n_invalid, const uint32_t *d_w) {
  return run_pipeline(g, d_pairs, nullptr, b, insert, n_invalid, d_w);
}

// d_w: the pairs' values on a weighted graph (null: value 1)
static sst_status run_pipeline(sst_graph *g, const uint32_t *d_pairs,
                               const uint64_t *presorted, uint64_t b,
                               bool insert, uint64_t *n_invalid,
                               const uint32_t *d_w) {
  if (n_invalid) *n_invalid = 0;
  if (b == 0) return SST_OK;
  if (b > 0xFFFFFFF0ull) {
    set_error_message("batch of %llu pairs exceeds 2^32", (unsigned long long)b);
    return SST_EINVAL;
  }
  // Small batches are bound by the host's launch rate, so their planning
  // sequence (sort to plan readback) is captured once per size class and
  // graph layout and replayed as one graph launch.  Every launch after the
  // keys is sized by the class (b rounded up, see plan_size_class) and does
  // the work of the device-side key count.  Unweighted raw-pair batches only
  // (the keys, which read the caller's pairs, are launched directly).
  const bool wt = g->weighted && insert && !presorted;
  const uint64_t npairs = b;  // pairs the caller gave
  const bool replay = !presorted && !wt && b <= kPlanGraphMaxBatch && g->plan_graphs;
  if (replay) b = plan_size_class(b);
  cudaStream_t s = g->stream;
  size_t need = update_scratch_bytes(b);
  if (need > g->arena.cap) {
    sst_status st = budget_check(g, need - g->arena.cap);
    if (st != SST_OK) return st;
  }
  SST_CUDA_TRY(g->arena.reserve(need));
  Arena &A = g->arena;
  A.reset();
  PlanSummary *P = g->d_plan;
  SST_CUDA_TRY(cudaMemsetAsync(P, 0, sizeof(PlanSummary), s));

  const int dbits = g->dbits;
  DGraph dg = g->view();
  uint64_t *keys = A.take<uint64_t>(b), *ktmp = A.take<uint64_t>(b);
  uint32_t *flag = A.take<uint32_t>(b), *pos = A.take<uint32_t>(b + 1);
  uint32_t *leaf = A.take<uint32_t>(b);
  uint64_t *p_ul = A.take<uint64_t>(b);
  uint32_t *p_x = A.take<uint32_t>(b);
  uint32_t *gflag = A.take<uint32_t>(b);
  uint32_t *g_start = A.take<uint32_t>(b + 1);
  uint8_t *gtype = A.take<uint8_t>(b), *glev = A.take<uint8_t>(b);
  uint32_t *gw0 = A.take<uint32_t>(b), *gw1 = A.take<uint32_t>(b);
  uint64_t *fkey = A.take<uint64_t>(b), *bkey = A.take<uint64_t>(b);
  uint64_t *mt = A.take<uint64_t>(b), *mtpos = A.take<uint64_t>(b);
  uint64_t *merge_jk = A.take<uint64_t>(b);
  uint32_t *task_group = A.take<uint32_t>(b);
  // per key, then per packed item: the leaf's start slot and count word
  uint64_t *lS = A.take<uint64_t>(b), *p_S = A.take<uint64_t>(b);
  uint32_t *lc = A.take<uint32_t>(b), *p_c = A.take<uint32_t>(b);
  uint32_t *climb = A.take<uint32_t>(b);
  uint32_t *itask = A.take<uint32_t>(b);  // inserts: each item's task, or none
  Tasks T;
  T.u = A.take<uint32_t>(b);
  T.w0 = A.take<uint32_t>(b);
  T.key = A.take<uint64_t>(b);
  T.nsrc = A.take<uint64_t>(b);
  T.ndst = A.take<uint64_t>(b);
  T.newbeg = A.take<uint32_t>(b);
  T.newend = A.take<uint32_t>(b);
  T.total = A.take<uint64_t>(b);
  T.capn = A.take<uint64_t>(b);
  T.rank = A.take<uint32_t>(b);
  T.type = A.take<uint8_t>(b);
  T.out = A.take<uint64_t>(b);
  T.soff = A.take<uint64_t>(b);
  T.doff = A.take<uint64_t>(b);
  T.err = g->d_err;
  // weighted graphs: values beside the keys (sorted with them) and the packed
  // items
  uint32_t *wv = wt ? A.take<uint32_t>(b) : nullptr;
  uint32_t *wtmp = wt ? A.take<uint32_t>(b) : nullptr;
  uint32_t *p_w = wt ? A.take<uint32_t>(b) : nullptr;
  T.stage_v = nullptr;  // set with the staging below
  T.p_w = p_w;

  // 1: keys
  const uint64_t *sorted = presorted;
  uint32_t *nkeys = nullptr;
  const int sort_bits = bits_for(g->n ? g->n - 1 : 0) + dbits;  // unweighted keys
  SortDigits sdig;
  if (!presorted) {
    // pair in (8 B), key out (8 B)
    // unweighted keys are compacted (see k_make_keys): their rows are below
    // n, one bit fewer to sort when n is a power of two
    nkeys = wt ? nullptr : &P->n_keys;
    if (wt)
      SST_LAUNCH_PDL_B(16 * b, k_make_keys, blocks_for(b), kTB, 0, s, d_pairs, b, g->n,
                   g->width, dbits, insert && !g->keep_loops, keys,
                   reinterpret_cast<unsigned long long *>(&P->invalid), d_w, wv);
    else {
      // the sort's digit counts come from the key build when the sort takes
      // the one-sweep form (its tables taken here, before the sort's scratch)
      if (radix_sort_digits(b, sort_bits, A, &sdig)) {
        SST_CUDA_TRY(cudaMemsetAsync(sdig.totals, 0, (size_t)sdig.passes * 256 * 4, s));
      } else {
        sdig = SortDigits{};
      }
      if ((reinterpret_cast<uintptr_t>(d_pairs) & 7) == 0)
        SST_LAUNCH_PDL_NB("k_make_keys_packed", 16 * npairs, k_make_keys_packed<true>,
                     blocks_for(npairs, kTB * kPackItems), kTB, 0, s, d_pairs, npairs, g->n,
                     g->width, dbits, insert && !g->keep_loops, keys,
                     reinterpret_cast<unsigned long long *>(&P->invalid), nkeys, sdig);
      else
        SST_LAUNCH_PDL_NB("k_make_keys_packed", 16 * npairs, k_make_keys_packed<false>,
                     blocks_for(npairs, kTB * kPackItems), kTB, 0, s, d_pairs, npairs, g->n,
                     g->width, dbits, insert && !g->keep_loops, keys,
                     reinterpret_cast<unsigned long long *>(&P->invalid), nkeys, sdig);
    }
  }
  MergeJoin join{s, nullptr};
  // 9a (inserts): the leaf merges need only k_emit's output and their count
  // (on the device), so they run on a second stream from there, beside the
  // task planning, the plan readback and the window / resize tasks.  They
  // touch disjoint leaves: a group inside a task's window (or a resized row)
  // is that task's, not a merge, and the merges add their rows' degrees
  // themselves (no task reads those).  Every later step that could meet
  // them -- a repack of the slab, the end of the batch -- waits.
  auto fork_merges = [&](cudaStream_t from) -> sst_status {
    SST_CUDA_TRY(cudaEventRecord(g->fork_ev, from));
    SST_CUDA_TRY(cudaStreamWaitEvent(g->side, g->fork_ev, 0));
    SST_LAUNCH_PDL(k_leaf_merge, std::min(warp_blocks((b + 31) / 32), (unsigned)g->sms * 8),
               kTB, 0, g->side, dg, p_ul, p_x, p_S, p_c, merge_jk, &P->n_merge, p_w);
    SST_CUDA_TRY(cudaEventRecord(g->merge_done, g->side));
    join.ev = g->merge_done;
    return SST_OK;
  };
  if (!g->side) {
    SST_CUDA_TRY(cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking));
    SST_CUDA_TRY(cudaEventCreateWithFlags(&g->fork_ev, cudaEventDisableTiming));
    SST_CUDA_TRY(cudaEventCreateWithFlags(&g->merge_done, cudaEventDisableTiming));
  }
  if (!g->aux_fork) {
    for (int k = 0; k < 2; k++) {
      SST_CUDA_TRY(cudaStreamCreateWithFlags(&g->aux[k], cudaStreamNonBlocking));
      SST_CUDA_TRY(cudaEventCreateWithFlags(&g->aux_join[k], cudaEventDisableTiming));
    }
    SST_CUDA_TRY(cudaEventCreateWithFlags(&g->aux_fork, cudaEventDisableTiming));
  }
  // run k independent pieces of work on aux[0..k-1] beside the stream
  auto fork_aux = [&](cudaStream_t from, int k) -> cudaError_t {
    cudaError_t e = cudaEventRecord(g->aux_fork, from);
    for (int i = 0; i < k && e == cudaSuccess; i++)
      e = cudaStreamWaitEvent(g->aux[i], g->aux_fork, 0);
    return e;
  };
  auto join_aux = [&](cudaStream_t to, int k) -> cudaError_t {
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < k && e == cudaSuccess; i++) {
      e = cudaEventRecord(g->aux_join[i], g->aux[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(to, g->aux_join[i], 0);
    }
    return e;
  };

  // 2-8: sort to plan.  For a given batch size and graph layout this is a
  // fixed sequence of launches over device-resident counts; `fork` starts
  // the merges after k_emit (a captured sequence starts them after its end).
  auto plan = [&](cudaStream_t s, bool fork) -> sst_status {
    // a replayed sequence tags its single-pass scans from the device
    DeviceScanTags tags(replay ? g->d_scan_epoch : nullptr);
    if (replay) SST_CUDA_TRY(tags.bump(s));
    if (!presorted) {
      uint64_t *out = keys;
      if (wt) {
        uint32_t *wout = wv;
        SST_CUDA_TRY(radix_sort_kv(keys, ktmp, wv, wtmp, b, g->rbits + dbits, A, s,
                                   &out, &wout));
        wv = wout;
      } else {
        SST_CUDA_TRY(radix_sort_u64(keys, ktmp, b, sort_bits, A, s, &out, nkeys,
                                    sdig.passes ? &sdig : nullptr));
      }
      sorted = out;
    }
    // 3-5: locate, pack, group
    // sorted key in (8 B), flag and leaf out (8 B)
    if (b <= kLocateWarpKeys)
      SST_LAUNCH_PDL_B(16 * b, k_locate_warp, warp_blocks(b), kTB, 0, s, sorted, b, dbits, dg,
                   insert, flag, leaf, wt ? wv : nullptr, lS, lc, nkeys);
    else
      SST_LAUNCH_PDL_B(16 * b, k_locate, blocks_for(b), kTB, 0, s, sorted, b, dbits, dg,
                   insert, flag, leaf, wt ? wv : nullptr, lS, lc, nkeys);
    SST_CUDA_TRY((scan<uint32_t, OpAdd>(flag, pos, b, 0u, OpAdd{}, true, false,
                                        &P->n_items, A, s)));
    SST_LAUNCH_PDL(k_pack, blocks_for(b), kTB, 0, s, sorted, flag, pos, leaf, b, dbits,
                   p_ul, p_x, wv, p_w, lS, lc, p_S, p_c);
    SST_LAUNCH_PDL(k_group_flags, blocks_for(b), kTB, 0, s, p_ul, &P->n_items, b, gflag);
    SST_CUDA_TRY((scan_epi<uint32_t, OpAdd, GroupStartEpi>(
        gflag, b, 0u, OpAdd{}, true, false, &P->n_groups, A, s, nullptr,
        GroupStartEpi{gflag, &P->n_items, b, g_start}, false)));
    // 6: classify (grids capped: the kernels stride over the device count)
    const unsigned cap_blocks = (unsigned)g->sms * 8;
    const unsigned tgrid = std::min(blocks_for(b), cap_blocks);
    const unsigned wgrid = std::min(warp_blocks(b), cap_blocks);
    if (insert) {
      SST_LAUNCH_PDL(k_classify_insert, tgrid, kTB, 0, s, p_ul, p_c, g_start,
                 &P->n_groups, gtype, glev, gw0, gw1, climb, &P->n_climb);
    } else {
      // multi-leaf segments have H >= 1 (at least two leaves)
      SST_LAUNCH_PDL(k_leaf_delete, wgrid, kTB, 0, s, dg,
                 (uint32_t)window_lower(g->params, 0, 1), p_ul, p_x, p_S, p_c,
                 g_start, &P->n_groups, gtype, glev, gw0, gw1, climb, &P->n_climb);
    }
    SST_LAUNCH_PDL(k_climb, wgrid, kTB, 0, s, dg,
               g->d_bounds + (insert ? 0 : kBoundsH * kBoundsH), insert, p_ul, g_start,
               &P->n_items, climb, &P->n_climb, gtype, glev, gw0, gw1);
    // 7-8: dominance, classification and emit.  The climb list is free
    // again: it holds the tasks that k_task_setup_hard sets up
    const EmitArgs ea{b, g_start, merge_jk, task_group,
                      fill_inv_q24(g->params.grow_fill), insert, p_ul, p_c, gtype, T,
                      P->class_cnt, climb, &P->n_hard, insert ? itask : nullptr};
    // totals land as one word on (n_merge, n_tasks), adjacent in the plan
    static_assert(offsetof(PlanSummary, n_tasks) == offsetof(PlanSummary, n_merge) + 4 &&
                      offsetof(PlanSummary, n_merge) % 8 == 0,
                  "n_merge and n_tasks share one aligned 64-bit word");
    SST_LAUNCH_PDL(k_dom_keys, blocks_for(b), kTB, 0, s, p_ul, g_start, gtype, glev,
                   gw0, gw1, &P->n_groups, b, fkey, bkey);
    // the scans run out of place into merge_jk and mtpos, which hold
    // nothing until the merge/task scan and k_emit below overwrite them
    uint64_t *fscan = merge_jk, *bscan = mtpos;
    // the two are independent: the backward one runs beside the forward one
    SST_CUDA_TRY(fork_aux(s, 1));
    SST_CUDA_TRY((scan<uint64_t, OpMax>(fkey, fscan, b, 0ull, OpMax{}, true, false,
                                        nullptr, A, s)));
    SST_CUDA_TRY((scan<uint64_t, OpMin>(bkey, bscan, b, ~0ull, OpMin{}, true, true,
                                        nullptr, A, g->aux[0])));
    SST_CUDA_TRY(join_aux(s, 1));
    SST_LAUNCH_PDL(k_dom_classify, blocks_for(b), kTB, 0, s, p_ul, g_start, gtype, glev,
                   fscan, bscan, &P->n_groups, b, mt);
    SST_CUDA_TRY((scan<uint64_t, OpAdd>(mt, mtpos, b, 0ull, OpAdd{}, true, false,
                                        reinterpret_cast<uint64_t *>(&P->n_merge), A, s)));
    SST_LAUNCH_PDL(k_emit, blocks_for(b), kTB, 0, s, mt, mtpos, ea);
    if (fork && insert) {
      sst_status st = fork_merges(s);
      if (st != SST_OK) return st;
    }
    SST_LAUNCH_PDL(k_task_setup_hard, wgrid, kTB, 0, s, dg, fill_inv_q24(g->params.grow_fill),
               insert, p_ul, g_start, gtype, gw0, gw1, task_group, climb, &P->n_hard,
               &P->n_items, T, P->class_cnt);
    // three independent scans, two of them beside the stream
    SST_CUDA_TRY(fork_aux(s, 2));
    SST_CUDA_TRY((scan<uint64_t, OpAdd>(T.total, T.out, b, 0ull, OpAdd{}, true,
                                        false, &P->task_elems, A, s, &P->n_tasks)));
    SST_CUDA_TRY((scan<uint64_t, OpAdd>(T.nsrc, T.soff, b, 0ull, OpAdd{}, true,
                                        false, &P->src_leaves, A, g->aux[0], &P->n_tasks)));
    SST_CUDA_TRY((scan<uint64_t, OpAdd>(T.ndst, T.doff, b, 0ull, OpAdd{}, true,
                                        false, &P->dst_leaves, A, g->aux[1], &P->n_tasks)));
    SST_CUDA_TRY(join_aux(s, 2));
    SST_LAUNCH_PDL(k_plan_out, 1, 64, 0, s, P, g->d_err, g->h_plan_dev);
    return SST_OK;
  };

  // replayed for small batches (the kernel profiler times a replay as one
  // entry, update_plan_graph)
  if (replay) {
    sst_status st;
    if (g->plan_direct) {
      CaptureForms forms;
      st = plan(s, false);
    } else {
      st = plan_graph_launch(g, b, insert, dg, s, [&](cudaStream_t cs) {
        return plan(cs, false);
      });
    }
    if (st != SST_OK) return st;
    if (insert) {
      st = fork_merges(s);
      if (st != SST_OK) return st;
    }
  } else {
    sst_status st = plan(s, true);
    if (st != SST_OK) return st;
  }
  if (!g->plan_ready)
    SST_CUDA_TRY(cudaEventCreateWithFlags(&g->plan_ready, cudaEventDisableTiming));
  SST_CUDA_TRY(cudaEventRecord(g->plan_ready, s));
  SST_CUDA_TRY(cudaEventSynchronize(g->plan_ready));
  SST_CUDA_TRY(cudaGetLastError());
  PlanSummary ps = *g->h_plan;
  if (ps.apply_err) {
    set_error_message("internal error: %llu failed device checks (staging rank out of range)",
                      (unsigned long long)ps.apply_err);
    return SST_EDEVICE;
  }
  if (n_invalid) *n_invalid = ps.invalid;

  // slab space for resized segments, laid out largest class first so each
  // segment is aligned to min(cap, 32)
  uint64_t grow = 0;
  for (int c = 0; c < kNumClasses; c++) grow += (uint64_t)ps.class_cnt[c] << c;
  uint64_t start = (g->bump + kLeaf - 1) & ~uint64_t(kLeaf - 1);
  if (grow > 0 && start + grow > g->nslots) {
    join.wait();  // the merges write the slab the repack copies and frees
    sst_status st = repack(g, grow);
    if (st != SST_OK) return st;
    dg = g->view();
    start = (g->bump + kLeaf - 1) & ~uint64_t(kLeaf - 1);
    // the items' leaf starts (p_S) point into the old slab now, but the leaf
    // merges and deletes that read them have run already
  }
  ClassStarts cstart;
  uint64_t off = start;
  for (int c = kNumClasses - 1; c >= 0; c--) {
    cstart.s[c] = off;
    off += (uint64_t)ps.class_cnt[c] << c;
  }
  if (grow > 0) g->bump = off;

  // staging for window / resize tasks
  size_t wneed = ps.task_elems * (g->weighted ? 8 : 4) + ps.src_leaves * 20 +
                 ps.dst_leaves * 4 + scan_scratch_bytes(ps.src_leaves, 8) + 4096;
  if (wneed > g->work.cap) {
    sst_status st = budget_check(g, wneed - g->work.cap);
    if (st != SST_OK) return st;
  }
  SST_CUDA_TRY(g->work.reserve(wneed));
  g->work.reset();
  uint32_t *stage = g->work.take<uint32_t>(ps.task_elems);
  if (g->weighted) T.stage_v = g->work.take<uint32_t>(ps.task_elems);
  uint64_t *scnt = g->work.take<uint64_t>(ps.src_leaves);
  uint64_t *spre = g->work.take<uint64_t>(ps.src_leaves);
  uint32_t *stask = g->work.take<uint32_t>(ps.src_leaves);
  uint32_t *dtask = g->work.take<uint32_t>(ps.dst_leaves);
  uint32_t *const titem = insert && ps.n_tasks && ps.n_items ? itask : nullptr;

  // 9b: apply the window / resize tasks
  if (ps.n_tasks) {
    // eight lanes a task (k_task_index) and a leaf (k_gather_old,
    // k_task_scatter); the new ids' gather writes other staging slots than
    // the old ids', so it runs beside it on an aux stream
    SST_LAUNCH_PDL(k_task_index, blocks_for(8 * (uint64_t)ps.n_tasks), kTB, 0, s, dg, T,
               ps.n_tasks, stask, dtask, titem, scnt);
    if (ps.src_leaves)
      SST_CUDA_TRY((scan<uint64_t, OpAdd>(scnt, spre, ps.src_leaves, 0ull,
                                          OpAdd{}, true, false, nullptr,
                                          g->work, s)));
    const bool gnew = insert && ps.n_items;
    if (gnew && ps.src_leaves) {
      SST_CUDA_TRY(fork_aux(s, 1));
      SST_LAUNCH_PDL(k_gather_new, blocks_for(ps.n_items), kTB, 0, g->aux[0], dg, T,
                 ps.n_tasks, spre, p_ul, p_x, ps.n_items, stage, titem);
    } else if (gnew) {
      SST_LAUNCH_PDL(k_gather_new, blocks_for(ps.n_items), kTB, 0, s, dg, T,
                 ps.n_tasks, spre, p_ul, p_x, ps.n_items, stage, titem);
    }
    if (ps.src_leaves)
      SST_LAUNCH_PDL(k_gather_old, blocks_for(8 * ps.src_leaves), kTB, 0, s, dg, T,
                 ps.n_tasks, ps.src_leaves, spre, p_x, stage, stask);
    if (gnew && ps.src_leaves) SST_CUDA_TRY(join_aux(s, 1));
    if (ps.dst_leaves)
      SST_LAUNCH_PDL(k_task_scatter, blocks_for(8 * ps.dst_leaves), kTB, 0, s, dg, T,
                 ps.n_tasks, ps.dst_leaves, cstart, stage, dtask);
    SST_LAUNCH_PDL(k_finalize, blocks_for(ps.n_tasks), kTB, 0, s, dg, T, ps.n_tasks,
               cstart);
  }
  join.wait();
  // the staging-rank check of this batch is read back with the next plan
  // (or by sst_sync), so a batch ends without a second host synchronisation
  SST_CUDA_TRY(cudaGetLastError());
  if (insert)
    g->m += ps.n_items;
  else
    g->m -= ps.n_items;
  if (ps.n_items) g->version++;
  return SST_OK;
}

// ------------------------------------------------------------ batched form
// A sequence of update batches applied as one pipeline pass.  With set
// semantics only the last operation on an edge decides whether it is present
// afterwards, so a stable sort of all pairs by edge (payload: the batch's
// operation) and a last-one-wins selection give the net removals and net
// insertions, which touch disjoint edges and run as one remove pass and one
// insert pass over already sorted keys.  Self-loops are dropped from both
// (an inserted self-loop is skipped, a removed one is absent).
namespace {
__global__ void k_make_keys_batched(const uint32_t *__restrict__ pairs,
                                    uint64_t N, const uint64_t *__restrict__ boff,
                                    uint32_t nb, const uint8_t *__restrict__ ops,
                                    uint32_t n, uint32_t width, int dbits,
                                    bool drop_loops, uint64_t *__restrict__ keys,
                                    uint32_t *__restrict__ vals,
                                    unsigned long long *__restrict__ invalid) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  uint32_t lo = 0, hi = nb;  // batch: last with boff[b] <= i
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (boff[mid] <= i)
      lo = mid;
    else
      hi = mid;
  }
  uint32_t r = pairs[2 * i], c = pairs[2 * i + 1];
  const uint64_t sent = (uint64_t)n << dbits;
  bool ok = r < n && c < width && c != kEmpty;
  if (!ok) atomicAdd(invalid, 1ull);
  keys[i] = (!ok || (drop_loops && r == c)) ? sent : (((uint64_t)r << dbits) | c);
  vals[i] = ops[lo] ? 1u : 0u;
}

__global__ void k_last_op(const uint64_t *__restrict__ keys,
                          const uint32_t *__restrict__ vals, uint64_t N,
                          uint64_t sent, uint32_t *__restrict__ fins,
                          uint32_t *__restrict__ fdel) {
  pdl_wait();
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  uint64_t k = keys[j];
  bool last = k < sent && (j + 1 == N || keys[j + 1] != k);
  fins[j] = last && vals[j];
  fdel[j] = last && !vals[j];
}

__global__ void k_compact_keys(const uint64_t *__restrict__ keys,
                               const uint32_t *__restrict__ f,
                               const uint32_t *__restrict__ pos, uint64_t N,
                               uint64_t *__restrict__ out) {
  pdl_wait();
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < N && f[j]) out[pos[j]] = keys[j];
}
}  // namespace

sst_status update_batches(sst_graph *g, const uint32_t *d_pairs,
                          const uint64_t *d_boff, const uint8_t *d_ops,
                          uint32_t nb, uint64_t N, uint64_t *n_invalid) {
  if (n_invalid) *n_invalid = 0;
  if (N == 0 || nb == 0) return SST_OK;
  if (N > 0xFFFFFFF0ull) {
    set_error_message("batched update of %llu pairs exceeds 2^32", (unsigned long long)N);
    return SST_EINVAL;
  }
  cudaStream_t s = g->stream;
  size_t need = N * (8 * 2 + 4 * 6 + 64) + radix_sort_scratch_bytes(N) +
                4 * scan_scratch_bytes(N, 4) + (1 << 16);
  if (need > g->arena.cap) {
    sst_status st = budget_check(g, need - g->arena.cap);
    if (st != SST_OK) return st;
  }
  SST_CUDA_TRY(g->arena.reserve(need));
  Arena &A = g->arena;
  A.reset();
  PlanSummary *P = g->d_plan;
  SST_CUDA_TRY(cudaMemsetAsync(P, 0, sizeof(PlanSummary), s));
  uint64_t *keys = A.take<uint64_t>(N), *ktmp = A.take<uint64_t>(N);
  uint32_t *vals = A.take<uint32_t>(N), *vtmp = A.take<uint32_t>(N);
  uint32_t *fins = A.take<uint32_t>(N), *fdel = A.take<uint32_t>(N);
  uint32_t *pins = A.take<uint32_t>(N), *pdel = A.take<uint32_t>(N);
  if (!pdel) {
    set_error_message("batched update scratch sizing error");
    return SST_ENOMEM;
  }
  const int dbits = g->dbits;
  const uint64_t sent = (uint64_t)g->n << dbits;
  SST_LAUNCH_PDL(k_make_keys_batched, blocks_for(N), kTB, 0, s, d_pairs, N, d_boff,
             nb, d_ops, g->n, g->width, dbits, !g->keep_loops, keys, vals,
             reinterpret_cast<unsigned long long *>(&P->invalid));
  uint64_t *sk = keys;
  uint32_t *sv = vals;
  SST_CUDA_TRY(radix_sort_kv(keys, ktmp, vals, vtmp, N, g->rbits + dbits, A, s,
                             &sk, &sv));
  SST_LAUNCH_PDL(k_last_op, blocks_for(N), kTB, 0, s, sk, sv, N, sent, fins, fdel);
  SST_CUDA_TRY((scan<uint32_t, OpAdd>(fins, pins, N, 0u, OpAdd{}, true, false,
                                      &P->n_items, A, s)));
  SST_CUDA_TRY((scan<uint32_t, OpAdd>(fdel, pdel, N, 0u, OpAdd{}, true, false,
                                      &P->n_groups, A, s)));
  SST_CUDA_TRY(cudaMemcpyAsync(g->h_plan, P, sizeof(PlanSummary),
                               cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t n_ins = g->h_plan->n_items, n_del = g->h_plan->n_groups;
  if (n_invalid) *n_invalid = g->h_plan->invalid;
  if (n_ins + n_del == 0) return SST_OK;
  uint64_t *net = nullptr;
  SST_CUDA_TRY(cudaMallocAsync(&net, (n_ins + n_del) * 8, s));
  SST_LAUNCH_PDL(k_compact_keys, blocks_for(N), kTB, 0, s, sk, fins, pins, N, net);
  SST_LAUNCH_PDL(k_compact_keys, blocks_for(N), kTB, 0, s, sk, fdel, pdel, N, net + n_ins);
  sst_status st = run_pipeline(g, nullptr, net + n_ins, n_del, false, nullptr, nullptr);
  if (st == SST_OK) st = run_pipeline(g, nullptr, net, n_ins, true, nullptr, nullptr);
  cudaFreeAsync(net, s);
  return st;
}

// ------------------------------------------------------------ relabelling
// degree_order_map / rewrite_graph of SparseMatrix.hpp:737-766: vertices
// ranked by (degree, id) descending (std::greater on the pair, so among equal
// degrees the larger id comes first); the rewrite inserts every edge with
// both ends relabelled.
namespace {
__global__ void k_degkey(const uint32_t *__restrict__ deg, uint32_t n,
                         uint64_t *__restrict__ keys) {
  pdl_wait();
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) keys[v] = ((uint64_t)(0xFFFFFFFFu - deg[v]) << 32) | (0xFFFFFFFFu - v);
}
__global__ void k_rank_to_map(const uint64_t *__restrict__ sorted, uint32_t n,
                              uint32_t *__restrict__ map) {
  pdl_wait();
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) map[0xFFFFFFFFu - (uint32_t)sorted[r]] = r;
}
__global__ void k_csr_to_pairs(const uint64_t *__restrict__ off,
                               const uint32_t *__restrict__ cols, uint32_t n,
                               uint32_t *__restrict__ pairs);
__global__ void k_relabel_pairs(uint32_t *__restrict__ pairs, uint64_t m,
                                const uint32_t *__restrict__ map) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  pairs[2 * i] = map[pairs[2 * i]];
  pairs[2 * i + 1] = map[pairs[2 * i + 1]];
}
}  // namespace

sst_status degree_order_map(sst_graph *g, uint32_t *d_map) {
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  if (n == 0) return SST_OK;
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve((uint64_t)n * 16 + radix_sort_scratch_bytes(n) + 8192));
  uint64_t *keys = g->arena.take<uint64_t>(n), *tmp = g->arena.take<uint64_t>(n);
  SST_LAUNCH_PDL(k_degkey, blocks_for(n), kTB, 0, s, g->d_deg, n, keys);
  uint64_t *sorted = keys;
  SST_CUDA_TRY(radix_sort_u64(keys, tmp, n, 64, g->arena, s, &sorted));
  SST_LAUNCH_PDL(k_rank_to_map, blocks_for(n), kTB, 0, s, sorted, n, d_map);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status rewrite_graph(sst_graph *g, const uint32_t *d_map, sst_graph *out) {
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  uint64_t m = g->m;
  if (m == 0) return SST_OK;
  uint64_t *off = nullptr;
  uint32_t *cols = nullptr, *pairs = nullptr;
  SST_CUDA_TRY(cudaMallocAsync(&off, ((uint64_t)n + 1) * 8, s));
  SST_CUDA_TRY(cudaMallocAsync(&cols, m * 4, s));
  SST_CUDA_TRY(cudaMallocAsync(&pairs, m * 8, s));
  sst_status st = to_csr(g, off, cols);
  if (st == SST_OK) {
    SST_LAUNCH_PDL(k_csr_to_pairs, warp_blocks(n), kTB, 0, s, off, cols, n, pairs);
    SST_LAUNCH_PDL(k_relabel_pairs, blocks_for(m), kTB, 0, s, pairs, m, d_map);
    SST_CUDA_TRY(cudaStreamSynchronize(s));
    const uint64_t chunk = 1ull << 25;
    for (uint64_t first = 0; first < m && st == SST_OK; first += chunk)
      st = update_batch(out, pairs + 2 * first, std::min(chunk, m - first), true, nullptr);
    cudaStreamSynchronize(out->stream);
  }
  cudaFreeAsync(pairs, s);
  cudaFreeAsync(cols, s);
  cudaFreeAsync(off, s);
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  return st;
}

// Complete the graph's stream and report a staging-rank error left by an
// earlier batch (device-pointer updates do not wait for it).
sst_status sync_checked(sst_graph *g) {
  SST_LAUNCH_PDL(k_err_out, 1, 32, 0, g->stream, g->d_err, &g->h_plan_dev->apply_err);
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  if (g->h_plan->apply_err) {
    set_error_message("internal error: %llu failed device checks (staging rank out of range)",
                      (unsigned long long)g->h_plan->apply_err);
    return SST_EDEVICE;
  }
  return SST_OK;
}

// ------------------------------------------------------------ other paths
namespace {
__global__ void k_csr_to_pairs(const uint64_t *__restrict__ off,
                               const uint32_t *__restrict__ cols, uint32_t n,
                               uint32_t *__restrict__ pairs) {
  pdl_wait();
  uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (v >= n) return;
  for (uint64_t i = off[v] + lane; i < off[v + 1]; i += 32) {
    pairs[2 * i] = (uint32_t)v;
    pairs[2 * i + 1] = cols[i];
  }
}

// membership of each pair; with vals (weighted graphs) also the edge's
// value (0 where absent)
__global__ void k_has(DGraph g, const uint32_t *__restrict__ pairs, uint64_t n,
                      uint8_t *__restrict__ out, uint32_t *__restrict__ vals) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t u = pairs[2 * i], x = pairs[2 * i + 1];
  uint8_t r = 0;
  uint32_t v = 0;
  if (u < g.n) {
    uint64_t base = g.base[u];
    uint32_t cap = g.cap[u];
    if (cap) {
      uint32_t l = find_leaf(g.slots, base, cap, x);
      uint32_t c = leaf_count(g, base, cap, g.deg[u], l);
      const uint64_t S = base + ((uint64_t)l << kLeafLog);
      uint32_t pos = leaf_lower_bound(g.slots + S, c, x);
      r = pos < c && g.slots[S + pos] == x;
      if (r && vals) v = g.vals[S + pos];
    }
  }
  if (out) out[i] = r;
  if (vals) vals[i] = v;
}

__global__ void k_vertex_leaves(const uint32_t *__restrict__ cap, uint32_t n,
                                uint64_t *__restrict__ nl) {
  pdl_wait();
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  nl[v] = cap[v] ? nleaves_of(cap[v]) : 0;
}

// warp per vertex: its leaves into the directory
__global__ void k_dir_fill(DGraph g, const uint64_t *__restrict__ vleaf,
                           uint32_t *__restrict__ owner,
                           uint64_t *__restrict__ slot,
                           uint32_t *__restrict__ cnt) {
  pdl_wait();
  uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (v >= g.n) return;
  uint64_t k0 = vleaf[v], k1 = vleaf[v + 1];
  uint64_t base = g.base[v];
  uint32_t cap = g.cap[v], deg = g.deg[v];
  for (uint64_t k = k0 + lane; k < k1; k += 32) {
    uint32_t l = (uint32_t)(k - k0);
    owner[k] = (uint32_t)v;
    slot[k] = base + ((uint64_t)l << kLeafLog);
    cnt[k] = leaf_count(g, base, cap, deg, l);
  }
}

// warp per leaf: copy into CSR position
__global__ void k_dir_copy(const uint32_t *__restrict__ slots,
                           const uint64_t *__restrict__ slot,
                           const uint32_t *__restrict__ cnt,
                           const uint64_t *__restrict__ pre, uint64_t nleaves,
                           uint32_t *__restrict__ cols) {
  pdl_wait();
  uint64_t k = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= nleaves) return;
  if ((uint32_t)lane < cnt[k]) cols[pre[k] + lane] = slots[slot[k] + lane];
}

__global__ void k_widen(const uint32_t *__restrict__ in, uint64_t n,
                        uint64_t *__restrict__ out) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i];
}

__global__ void k_sample(const uint32_t *__restrict__ slots,
                         const uint32_t *__restrict__ owner,
                         const uint64_t *__restrict__ slot,
                         const uint64_t *__restrict__ pre, uint64_t nleaves,
                         uint64_t m, uint64_t seed, uint64_t first,
                         uint64_t count, uint32_t *__restrict__ pairs) {
  pdl_wait();
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  if (m == 0) {
    pairs[2 * i] = pairs[2 * i + 1] = 0;
    return;
  }
  uint64_t rank = __umul64hi(draw(seed, first + i, 0), m);
  uint64_t k = last_le_u64(pre, nleaves, rank);
  pairs[2 * i] = owner[k];
  pairs[2 * i + 1] = slots[slot[k] + (rank - pre[k])];
}

// warp per leaf; 64-bit sum of its elements added to *out
__global__ void k_sum_leaves(const uint32_t *__restrict__ slots,
                             const uint64_t *__restrict__ slot,
                             const uint32_t *__restrict__ cnt, uint64_t nleaves,
                             unsigned long long *__restrict__ out) {
  pdl_wait();
  uint64_t k = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= nleaves) return;
  uint64_t v = (uint32_t)lane < cnt[k] ? slots[slot[k] + lane] : 0;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  if (lane == 0 && v) atomicAdd(out, (unsigned long long)v);
}
}  // namespace

sst_status build_from_csr(sst_graph *g, const uint64_t *d_off,
                          const uint32_t *d_cols) {
  cudaStream_t s = g->stream;
  uint64_t m = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(&m, d_off + g->n, 8, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t n = std::max<uint64_t>(g->n, 1);
  SST_CUDA_TRY(cudaMemsetAsync(g->d_cap, 0, n * 4, s));
  SST_CUDA_TRY(cudaMemsetAsync(g->d_deg, 0, n * 4, s));
  SST_CUDA_TRY(cudaMemsetAsync(g->d_base, 0, n * 8, s));
  g->bump = 0;
  g->m = 0;
  g->version++;
  if (m == 0) return SST_OK;
  uint32_t *pairs = nullptr;
  SST_CUDA_TRY(cudaMallocAsync(&pairs, m * 8, s));
  SST_LAUNCH_PDL(k_csr_to_pairs, warp_blocks(g->n), kTB, 0, s, d_off, d_cols, g->n, pairs);
  sst_status st = update_batch(g, pairs, m, true, nullptr);
  cudaFreeAsync(pairs, s);
  return st;
}

sst_status has_batch(sst_graph *g, const uint32_t *d_pairs, uint64_t n,
                     uint8_t *d_out, uint32_t *d_vals) {
  if (n == 0) return SST_OK;
  SST_LAUNCH_PDL(k_has, blocks_for(n), kTB, 0, g->stream, g->view(), d_pairs, n, d_out,
             d_vals);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status ensure_leaf_dir(sst_graph *g) {
  LeafDir &D = g->dir;
  if (D.version == g->version && D.vleaf) return SST_OK;
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  if (!D.vleaf) SST_CUDA_TRY(cudaMalloc(&D.vleaf, ((uint64_t)n + 1) * 8));
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes((uint64_t)n + 1, 8) + 4096));
  uint64_t *total = g->arena.take<uint64_t>(1);
  if (n) SST_LAUNCH_PDL(k_vertex_leaves, blocks_for(n), kTB, 0, s, g->d_cap, n, D.vleaf);
  SST_CUDA_TRY((scan<uint64_t, OpAdd>(D.vleaf, D.vleaf, n, 0ull, OpAdd{}, true,
                                      false, total, g->arena, s)));
  uint64_t nl = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(&nl, total, 8, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  SST_CUDA_TRY(cudaMemcpyAsync(D.vleaf + n, &nl, 8, cudaMemcpyHostToDevice, s));
  if (nl > D.cap) {
    uint64_t want = nl + nl / 4 + 1024;
    sst_status st = budget_check(g, (want - D.cap) * 24);
    if (st != SST_OK) return st;
    SST_CUDA_TRY(cudaStreamSynchronize(s));
    cudaFree(D.owner);
    cudaFree(D.slot);
    cudaFree(D.cnt);
    cudaFree(D.pre);
    D.owner = nullptr;
    D.slot = nullptr;
    D.cnt = nullptr;
    D.pre = nullptr;
    D.cap = 0;
    SST_CUDA_TRY(cudaMalloc(&D.owner, want * 4));
    SST_CUDA_TRY(cudaMalloc(&D.slot, want * 8));
    SST_CUDA_TRY(cudaMalloc(&D.cnt, want * 4));
    SST_CUDA_TRY(cudaMalloc(&D.pre, (want + 1) * 8));
    D.cap = want;
  }
  D.nleaves = nl;
  if (n) SST_LAUNCH_PDL(k_dir_fill, warp_blocks(n), kTB, 0, s, g->view(), D.vleaf,
                    D.owner, D.slot, D.cnt);
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes(nl + 1, 8) + (nl + 1) * 8 + 4096));
  uint64_t *wide = g->arena.take<uint64_t>(nl + 1);
  if (nl) SST_LAUNCH_PDL(k_widen, blocks_for(nl), kTB, 0, s, D.cnt, nl, wide);
  SST_CUDA_TRY((scan<uint64_t, OpAdd>(wide, D.pre, nl, 0ull, OpAdd{}, true,
                                      false, D.pre + nl, g->arena, s)));
  SST_CUDA_TRY(cudaGetLastError());
  D.version = g->version;
  return SST_OK;
}

sst_status to_csr(sst_graph *g, uint64_t *d_off, uint32_t *d_cols,
                  uint32_t *d_vals) {
  sst_status st = ensure_leaf_dir(g);
  if (st != SST_OK) return st;
  cudaStream_t s = g->stream;
  uint32_t n = g->n;
  LeafDir &D = g->dir;
  // row offsets: CSR position of each vertex's first leaf
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(scan_scratch_bytes((uint64_t)n + 1, 8) + ((uint64_t)n + 1) * 8 + 4096));
  uint64_t *wide = g->arena.take<uint64_t>((uint64_t)n + 1);
  if (n) SST_LAUNCH_PDL(k_widen, blocks_for(n), kTB, 0, s, g->d_deg, n, wide);
  SST_CUDA_TRY((scan<uint64_t, OpAdd>(wide, d_off, n, 0ull, OpAdd{}, true, false,
                                      d_off + n, g->arena, s)));
  if (D.nleaves)
    SST_LAUNCH_PDL(k_dir_copy, warp_blocks(D.nleaves), kTB, 0, s, g->d_slots, D.slot,
               D.cnt, D.pre, D.nleaves, d_cols);
  if (D.nleaves && d_vals && g->d_vals)  // values in the same CSR order
    SST_LAUNCH_PDL(k_dir_copy, warp_blocks(D.nleaves), kTB, 0, s, g->d_vals, D.slot,
               D.cnt, D.pre, D.nleaves, d_vals);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status neighbors(sst_graph *g, uint32_t v, uint32_t *d_out, uint64_t cap,
                     uint64_t *deg) {
  sst_status st = ensure_leaf_dir(g);
  if (st != SST_OK) return st;
  cudaStream_t s = g->stream;
  LeafDir &D = g->dir;
  uint64_t k[2];
  SST_CUDA_TRY(cudaMemcpyAsync(k, D.vleaf + v, 16, cudaMemcpyDeviceToHost, s));
  uint32_t d = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(&d, g->d_deg + v, 4, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  *deg = d;
  if (k[1] == k[0] || cap == 0) return SST_OK;
  uint64_t p0 = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(&p0, D.pre + k[0], 8, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  if (cap >= d) {
    // copy leaves with positions rebased to the vertex's first element
    SST_LAUNCH_PDL(k_dir_copy, warp_blocks(k[1] - k[0]), kTB, 0, s, g->d_slots,
               D.slot + k[0], D.cnt + k[0], D.pre + k[0], k[1] - k[0],
               d_out - p0);
  } else {
    uint32_t *tmp = nullptr;
    SST_CUDA_TRY(cudaMallocAsync(&tmp, (uint64_t)d * 4, s));
    SST_LAUNCH_PDL(k_dir_copy, warp_blocks(k[1] - k[0]), kTB, 0, s, g->d_slots,
               D.slot + k[0], D.cnt + k[0], D.pre + k[0], k[1] - k[0], tmp - p0);
    SST_CUDA_TRY(cudaMemcpyAsync(d_out, tmp, cap * 4, cudaMemcpyDeviceToDevice, s));
    cudaFreeAsync(tmp, s);
  }
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status sample_edges(sst_graph *g, uint64_t seed, uint64_t first,
                        uint64_t count, uint32_t *d_pairs) {
  if (count == 0) return SST_OK;
  sst_status st = ensure_leaf_dir(g);
  if (st != SST_OK) return st;
  LeafDir &D = g->dir;
  SST_LAUNCH_PDL(k_sample, blocks_for(count), kTB, 0, g->stream, g->d_slots, D.owner,
             D.slot, D.pre, D.nleaves, g->m, seed, first, count, d_pairs);
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

sst_status touch_all_sum(sst_graph *g, uint64_t *out) {
  sst_status st = ensure_leaf_dir(g);
  if (st != SST_OK) return st;
  cudaStream_t s = g->stream;
  LeafDir &D = g->dir;
  g->arena.reset();
  SST_CUDA_TRY(g->arena.reserve(4096));
  unsigned long long *acc = g->arena.take<unsigned long long>(1);
  SST_CUDA_TRY(cudaMemsetAsync(acc, 0, 8, s));
  if (D.nleaves)
    SST_LAUNCH_PDL(k_sum_leaves, warp_blocks(D.nleaves), kTB, 0, s, g->d_slots,
               D.slot, D.cnt, D.nleaves, acc);
  SST_CUDA_TRY(cudaMemcpyAsync(out, acc, 8, cudaMemcpyDeviceToHost, s));
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  return SST_OK;
}

}  // namespace sst

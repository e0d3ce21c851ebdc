// Serving runtime: a request loop over one device-resident graph.
//
//  - Updates (insert / remove requests) are applied by one writer thread.
//    Every pass takes all pending update requests in submission order (up to
//    max_coalesce) and applies them as one batched pipeline pass
//    (update_batches), so requests that arrive while a pass runs join the
//    next one.  The epoch counts update requests applied.
//  - Queries (BFS, PageRank, per-vertex triangle counts) run on query slots.
//    Each slot owns a device snapshot of the graph: before a query, a stale
//    snapshot is refreshed by copying the live graph between writer passes
//    (under the writer's lock), so a query sees the graph after a prefix of
//    the update requests -- its epoch -- and then runs on its own stream
//    while the writer keeps updating the live graph.
//  - Admission: a slot exists only while the HBM budget holds the live graph
//    plus the slot's snapshot and traversal buffers; queries wait for a free
//    slot in arrival order.
//  - Every request records queue, run and total latency.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "graph.cuh"
#include "traverse.cuh"

using Clock = std::chrono::steady_clock;

namespace sst {

// copy src's current contents into dst (same shape); both quiescent
sst_status graph_copy_into(sst_graph *dst, sst_graph *src) {
  SST_CUDA_TRY(cudaStreamSynchronize(src->stream));
  uint64_t used = (src->bump + kLeaf - 1) & ~uint64_t(kLeaf - 1);
  if (dst->nslots < used) {
    cudaStreamSynchronize(dst->stream);
    cudaFree(dst->d_slots);
    cudaFree(dst->d_lcnt);
    cudaFree(dst->d_vals);
    dst->d_slots = nullptr;
    dst->d_lcnt = nullptr;
    dst->d_vals = nullptr;
    uint64_t want = std::max(used + used / 4, src->nslots);
    want = (want + kLeaf - 1) & ~uint64_t(kLeaf - 1);
    SST_CUDA_TRY(cudaMalloc(&dst->d_slots, want * 4));
    SST_CUDA_TRY(cudaMalloc(&dst->d_lcnt, want / kLeaf + 1));
    if (dst->weighted) SST_CUDA_TRY(cudaMalloc(&dst->d_vals, want * 4));
    dst->nslots = want;
  }
  uint64_t n = std::max<uint64_t>(src->n, 1);
  cudaStream_t s = dst->stream;
  SST_CUDA_TRY(cudaMemcpyAsync(dst->d_base, src->d_base, n * 8, cudaMemcpyDeviceToDevice, s));
  SST_CUDA_TRY(cudaMemcpyAsync(dst->d_cap, src->d_cap, n * 4, cudaMemcpyDeviceToDevice, s));
  SST_CUDA_TRY(cudaMemcpyAsync(dst->d_deg, src->d_deg, n * 4, cudaMemcpyDeviceToDevice, s));
  if (used) {
    SST_CUDA_TRY(cudaMemcpyAsync(dst->d_slots, src->d_slots, used * 4, cudaMemcpyDeviceToDevice, s));
    SST_CUDA_TRY(cudaMemcpyAsync(dst->d_lcnt, src->d_lcnt, used / kLeaf, cudaMemcpyDeviceToDevice, s));
    if (src->d_vals)
      SST_CUDA_TRY(cudaMemcpyAsync(dst->d_vals, src->d_vals, used * 4, cudaMemcpyDeviceToDevice, s));
  }
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  dst->bump = src->bump;
  dst->m = src->m;
  dst->version += 1;  // invalidates the snapshot's traversal work lists
  return SST_OK;
}

// per-vertex triangle counts of the listed vertices:
// t(u) = (1/2) * sum over w in N(u) of |N(u) n N(w)| (symmetric graph).
// Three passes over work items:
//  1. leaf items (query, leaf of N(u)); each item and lane is a pair slot
//     holding the neighbour w in that slot of the leaf (or nothing);
//  2. each pair's cost: the shorter of N(u) and N(w), in chunks of 32
//     leaves;
//  3. a warp per chunk: lanes take the chunk's leaves of the shorter list one
//     at a time and probe each id in the longer list (binary search over its
//     leaf heads, then within the leaf).
// A pair of two long lists spreads over as many warps as the shorter one has
// 32-leaf chunks, so no warp walks a long list alone.
namespace {
constexpr uint32_t kTcvChunkLeaves = 32;

__device__ __forceinline__ bool probe(const DGraph &g, uint64_t base,
                                      uint32_t cap, uint32_t deg, uint32_t x) {
  uint32_t l = find_leaf(g.slots, base, cap, x);
  uint32_t c = leaf_count(g, base, cap, deg, l);
  const uint32_t *p = g.slots + base + ((uint64_t)l << kLeafLog);
  uint32_t pos = leaf_lower_bound(p, c, x);
  return pos < c && p[pos] == x;
}

__device__ __forceinline__ uint32_t leaves_of(uint32_t cap) {
  return cap == 0 ? 0 : (cap <= kLeaf ? 1 : cap >> kLeafLog);
}

__global__ void k_tcv_leaves(DGraph g, const uint32_t *__restrict__ vs,
                             uint64_t k, uint64_t *__restrict__ nl,
                             unsigned long long *__restrict__ out) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  uint32_t u = vs[i];
  nl[i] = u < g.n ? leaves_of(g.cap[u]) : 0;
  out[i] = 0;
}

// pass 2: warp per leaf item; lane = pair slot
__global__ void k_tcv_pairs(DGraph g, const uint32_t *__restrict__ vs, uint64_t k,
                            const uint64_t *__restrict__ loff, uint64_t items,
                            uint32_t *__restrict__ pq, uint32_t *__restrict__ pw,
                            uint32_t *__restrict__ cost) {
  const int lane = threadIdx.x & 31;
  const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t wi = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       wi < items; wi += warps) {
    // query q with loff[q] <= wi < loff[q + 1]
    uint64_t lo = 0, hi = k;
    while (hi - lo > 1) {
      const uint64_t mid = (lo + hi) >> 1;
      if (loff[mid] <= wi) lo = mid; else hi = mid;
    }
    const uint32_t u = vs[lo];
    const uint32_t l = (uint32_t)(wi - loff[lo]);
    const uint64_t base = g.base[u];
    const uint32_t cap = g.cap[u], deg = g.deg[u];
    const uint32_t c = leaf_count(g, base, cap, deg, l);
    const uint32_t w = (uint32_t)lane < c ? g.slots[base + ((uint64_t)l << kLeafLog) + lane]
                                          : kEmpty;
    uint32_t chunks = 0;
    if (w != kEmpty) {
      const uint32_t s = deg <= g.deg[w] ? u : w;  // the shorter list
      chunks = (leaves_of(g.cap[s]) + kTcvChunkLeaves - 1) / kTcvChunkLeaves;
    }
    pw[wi * 32 + lane] = w;
    cost[wi * 32 + lane] = chunks;
    if (lane == 0) pq[wi] = (uint32_t)lo;
  }
}

// pass 3: warp per chunk of a pair
__global__ void k_tcv_count(DGraph g, const uint32_t *__restrict__ vs,
                            const uint32_t *__restrict__ pq,
                            const uint32_t *__restrict__ pw,
                            const uint32_t *__restrict__ coff, uint64_t nslots,
                            uint64_t nchunks, unsigned long long *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t ci = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       ci < nchunks; ci += warps) {
    // pair slot p: the last with coff[p] <= ci (slots of cost 0 share their
    // offset with the next slot, so the last one is the pair that owns ci)
    uint64_t lo = 0, hi = nslots;
    while (hi - lo > 1) {
      const uint64_t mid = (lo + hi) >> 1;
      if (coff[mid] <= ci) lo = mid; else hi = mid;
    }
    const uint32_t q = pq[lo >> 5], w = pw[lo], u = vs[q];
    const uint32_t j = (uint32_t)(ci - coff[lo]);  // chunk of the pair
    const uint32_t s = g.deg[u] <= g.deg[w] ? u : w, o = s == u ? w : u;
    const uint64_t sbase = g.base[s], obase = g.base[o];
    const uint32_t scap = g.cap[s], sdeg = g.deg[s];
    const uint32_t ocap = g.cap[o], odeg = g.deg[o];
    const uint32_t l0 = j * kTcvChunkLeaves;
    const uint32_t l1 = min(l0 + kTcvChunkLeaves, leaves_of(scap));
    uint32_t hits = 0;
    for (uint32_t l = l0; l < l1; l++) {
      const uint32_t c = leaf_count(g, sbase, scap, sdeg, l);
      if ((uint32_t)lane < c)
        hits += probe(g, obase, ocap, odeg, g.slots[sbase + ((uint64_t)l << kLeafLog) + lane]);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) hits += __shfl_down_sync(0xffffffffu, hits, d);
    if (lane == 0 && hits) atomicAdd(&out[q], (unsigned long long)hits);
  }
}

__global__ void k_tcv_half(unsigned long long *__restrict__ out, uint64_t k) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) out[i] >>= 1;
}
}  // namespace

sst_status tc_vertices(sst_graph *g, const uint32_t *d_vs, uint64_t k,
                       uint64_t *d_out) {
  if (k == 0) return SST_OK;
  cudaStream_t s = g->stream;
  unsigned long long *out = reinterpret_cast<unsigned long long *>(d_out);
  const unsigned tb = 256;
  const uint64_t cap_blocks = (uint64_t)g->sms * 16;
  // pass 1: leaf items per query
  uint64_t *loff = nullptr;
  SST_CUDA_TRY(cudaMallocAsync(&loff, (k + 1) * 8, s));
  g->arena.reset();
  cudaError_t e = g->arena.reserve(scan_scratch_bytes(k, 8) + 4096);
  uint64_t *tot = e == cudaSuccess ? g->arena.take<uint64_t>(1) : nullptr;
  if (e == cudaSuccess && !tot) e = cudaErrorMemoryAllocation;
  uint64_t items = 0;
  if (e == cudaSuccess) {
    SST_LAUNCH(k_tcv_leaves, (unsigned)((k + tb - 1) / tb), tb, 0, s, g->view(),
               d_vs, k, loff, out);
    e = scan<uint64_t, OpAdd>(loff, loff, k, 0ull, OpAdd{}, true, false, tot,
                              g->arena, s);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&items, tot, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  // pass 2: pair slots and their chunk counts
  uint32_t *pq = nullptr, *pw = nullptr, *cost = nullptr, *coff = nullptr;
  const uint64_t nslots = items * 32;
  uint32_t nchunks = 0;
  if (e == cudaSuccess && items) {
    e = cudaMallocAsync(&pq, items * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&pw, nslots * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&cost, nslots * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&coff, nslots * 4, s);
    if (e == cudaSuccess) {
      g->arena.reset();
      e = g->arena.reserve(scan_scratch_bytes(nslots, 4) + 4096);
    }
    uint32_t *ctot = e == cudaSuccess ? g->arena.take<uint32_t>(1) : nullptr;
    if (e == cudaSuccess && !ctot) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess) {
      SST_LAUNCH(k_tcv_pairs, (unsigned)std::min<uint64_t>((items * 32 + tb - 1) / tb, cap_blocks),
                 tb, 0, s, g->view(), d_vs, k, loff, items, pq, pw, cost);
      e = scan<uint32_t, OpAdd>(cost, coff, nslots, 0u, OpAdd{}, true, false, ctot,
                                g->arena, s);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nchunks, ctot, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    // pass 3
    if (e == cudaSuccess && nchunks) {
      SST_LAUNCH(k_tcv_count,
                 (unsigned)std::min<uint64_t>(((uint64_t)nchunks * 32 + tb - 1) / tb, cap_blocks),
                 tb, 0, s, g->view(), d_vs, pq, pw, coff, nslots, nchunks, out);
      SST_LAUNCH(k_tcv_half, (unsigned)((k + tb - 1) / tb), tb, 0, s, out, k);
      e = cudaGetLastError();
    }
  }
  for (void *p : {(void *)loff, (void *)pq, (void *)pw, (void *)cost, (void *)coff})
    if (p) cudaFreeAsync(p, s);
  SST_CUDA_TRY(e);
  return SST_OK;
}

}  // namespace sst

// ======================================================================
struct SrvRequest {
  sst_request req;
  std::vector<uint32_t> data;  // copied pairs / vertices
  uint64_t ticket = 0;
  Clock::time_point submitted, started, finished;
  bool done = false;
  sst_request_info info{};
};

struct SrvSlot {
  sst_graph *snap = nullptr;
  uint64_t epoch = ~0ull;
  std::thread th;
};

struct sst_server {
  sst_graph *g = nullptr;
  sst_server_config cfg{};
  std::mutex mu;                  // queues, results, counters
  std::condition_variable cv_work, cv_done;
  std::mutex write_mu;            // held by the writer pass and snapshot copies
  std::deque<SrvRequest *> updates, queries;
  std::map<uint64_t, SrvRequest *> all;
  uint64_t next_ticket = 1;
  uint64_t epoch = 0;             // update requests applied to the live graph
  bool stop = false;
  std::thread writer;
  std::vector<SrvSlot *> slots;
  uint64_t updates_applied = 0, update_edges = 0, passes = 0;
};

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

void finish(sst_server *s, SrvRequest *r, sst_status st, uint64_t epoch) {
  r->finished = Clock::now();
  r->info.status = st;
  r->info.epoch = epoch;
  r->info.queue_ms = ms_between(r->submitted, r->started);
  r->info.run_ms = ms_between(r->started, r->finished);
  r->info.total_ms = ms_between(r->submitted, r->finished);
  r->done = true;
}

void writer_loop(sst_server *s) {
  cudaSetDevice(s->g->device);
  std::vector<uint32_t> pairs;
  std::vector<uint64_t> offs;
  std::vector<uint8_t> ops;
  for (;;) {
    std::vector<SrvRequest *> take;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->updates.empty(); });
      if (s->updates.empty() && s->stop) return;
      uint32_t lim = s->cfg.max_coalesce ? s->cfg.max_coalesce : 1u << 20;
      while (!s->updates.empty() && take.size() < lim) {
        take.push_back(s->updates.front());
        s->updates.pop_front();
      }
    }
    Clock::time_point t0 = Clock::now();
    pairs.clear();
    offs.assign(1, 0);
    ops.clear();
    for (SrvRequest *r : take) {
      r->started = t0;
      pairs.insert(pairs.end(), r->data.begin(), r->data.end());
      offs.push_back(pairs.size() / 2);
      ops.push_back(r->req.kind == SST_REQ_INSERT ? 1 : 0);
    }
    sst_status st;
    uint64_t epoch_after;
    {
      std::lock_guard<std::mutex> wl(s->write_mu);
      st = sst_update_batches(s->g, pairs.data(), offs.data(), ops.data(),
                              (uint32_t)take.size(), SST_HOST_PTR, nullptr);
      std::lock_guard<std::mutex> lk(s->mu);
      s->epoch += take.size();
      epoch_after = s->epoch;
      s->updates_applied += take.size();
      s->update_edges += pairs.size() / 2;
      s->passes++;
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (SrvRequest *r : take) finish(s, r, st, epoch_after);
    }
    s->cv_done.notify_all();
  }
}

sst_status run_query(sst_server *s, SrvSlot *slot, SrvRequest *r) {
  sst_graph *q = slot->snap;
  const uint32_t n = q->n;
  switch (r->req.kind) {
    case SST_REQ_BFS: {
      if (r->req.src >= n) return SST_EINVAL;
      return sst_bfs(q, r->req.src, nullptr, static_cast<int32_t *>(r->req.out),
                     SST_HOST_PTR);
    }
    case SST_REQ_PAGERANK:
      return sst_pagerank(q, r->req.iters, r->req.damping,
                          static_cast<double *>(r->req.out), SST_HOST_PTR);
    case SST_REQ_TC_VERTICES: {
      uint64_t k = r->data.size();
      uint32_t *dv = nullptr;
      uint64_t *dout = nullptr;
      SST_CUDA_TRY(cudaMallocAsync(&dv, std::max<uint64_t>(k, 1) * 4, q->stream));
      SST_CUDA_TRY(cudaMallocAsync(&dout, std::max<uint64_t>(k, 1) * 8, q->stream));
      if (k) SST_CUDA_TRY(cudaMemcpyAsync(dv, r->data.data(), k * 4, cudaMemcpyHostToDevice, q->stream));
      sst_status st = sst::tc_vertices(q, dv, k, dout);
      if (st == SST_OK && k)
        SST_CUDA_TRY(cudaMemcpyAsync(r->req.out, dout, k * 8, cudaMemcpyDeviceToHost, q->stream));
      cudaFreeAsync(dv, q->stream);
      cudaFreeAsync(dout, q->stream);
      SST_CUDA_TRY(cudaStreamSynchronize(q->stream));
      return st;
    }
  }
  return SST_EINVAL;
}

void slot_loop(sst_server *s, SrvSlot *slot) {
  cudaSetDevice(s->g->device);
  for (;;) {
    SrvRequest *r;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->queries.empty(); });
      if (s->queries.empty() && s->stop) return;
      r = s->queries.front();
      s->queries.pop_front();
    }
    r->started = Clock::now();
    sst_status st = SST_OK;
    uint64_t ep;
    {
      // refresh the snapshot between writer passes
      std::lock_guard<std::mutex> wl(s->write_mu);
      {
        std::lock_guard<std::mutex> lk(s->mu);
        ep = s->epoch;
      }
      if (slot->epoch != ep) {
        st = sst::graph_copy_into(slot->snap, s->g);
        if (st == SST_OK) slot->epoch = ep;
      }
    }
    if (st == SST_OK) st = run_query(s, slot, r);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      finish(s, r, st, slot->epoch);
    }
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

sst_status sst_server_create(sst_graph *g, const sst_server_config *cfg,
                             sst_server **out) {
  if (!g || !out) {
    sst::set_error_message("null argument");
    return SST_EINVAL;
  }
  *out = nullptr;
  if (g->n != g->width) {  // queries are traversals: square graphs only
    sst::set_error_message("a server needs a graph with as many rows as columns");
    return SST_EINVAL;
  }
  sst_server *s = new (std::nothrow) sst_server();
  if (!s) return SST_ENOMEM;
  s->g = g;
  if (cfg) s->cfg = *cfg;
  uint32_t want = s->cfg.query_slots ? s->cfg.query_slots : 2;
  // admission: the live graph (with its update scratch) plus, per slot, a
  // snapshot -- vertex table, slab and leaf counts, no update scratch -- and
  // its traversal buffers (~40 B per vertex)
  uint64_t graph_bytes = sst::graph_device_bytes(g);
  uint64_t per_slot = (uint64_t)g->n * 16 + g->nslots * (g->weighted ? 8 : 4) +
                      g->nslots / sst::kLeaf +
                      (uint64_t)g->n * 40;
  if (s->cfg.hbm_budget_bytes) {
    uint64_t room = s->cfg.hbm_budget_bytes > graph_bytes ? s->cfg.hbm_budget_bytes - graph_bytes : 0;
    uint64_t fit = room / std::max<uint64_t>(per_slot, 1);
    if (fit == 0) {
      delete s;
      sst::set_error_message("HBM budget too small for one query slot");
      return SST_EBUDGET;
    }
    want = (uint32_t)std::min<uint64_t>(want, fit);
  }
  for (uint32_t i = 0; i < want; i++) {
    SrvSlot *slot = new SrvSlot();
    sst_status st = sst_graph_clone(g, &slot->snap);
    if (st != SST_OK) {
      delete slot;
      if (i == 0) {
        delete s;
        return st;
      }
      break;  // memory for fewer slots only
    }
    slot->epoch = 0;
    s->slots.push_back(slot);
  }
  s->writer = std::thread(writer_loop, s);
  for (SrvSlot *slot : s->slots) slot->th = std::thread(slot_loop, s, slot);
  *out = s;
  return SST_OK;
}

sst_status sst_server_slots(sst_server *s, uint32_t *out) {
  if (!s || !out) return SST_EINVAL;
  *out = (uint32_t)s->slots.size();
  return SST_OK;
}

sst_status sst_server_submit(sst_server *s, const sst_request *req,
                             uint64_t *ticket) {
  if (!s || !req || !ticket) return SST_EINVAL;
  SrvRequest *r = new (std::nothrow) SrvRequest();
  if (!r) return SST_ENOMEM;
  r->req = *req;
  r->submitted = Clock::now();
  switch (req->kind) {
    case SST_REQ_INSERT:
    case SST_REQ_REMOVE:
      if (req->n && !req->pairs) {
        delete r;
        return SST_EINVAL;
      }
      r->data.assign(req->pairs, req->pairs + 2 * req->n);
      break;
    case SST_REQ_TC_VERTICES:
      if (req->n && (!req->pairs || !req->out)) {
        delete r;
        return SST_EINVAL;
      }
      r->data.assign(req->pairs, req->pairs + req->n);
      break;
    case SST_REQ_BFS:
    case SST_REQ_PAGERANK:
      if (!req->out) {
        delete r;
        return SST_EINVAL;
      }
      break;
    default:
      delete r;
      sst::set_error_message("unknown request kind %d", req->kind);
      return SST_EINVAL;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    s->all[r->ticket] = r;
    if (req->kind == SST_REQ_INSERT || req->kind == SST_REQ_REMOVE)
      s->updates.push_back(r);
    else
      s->queries.push_back(r);
    *ticket = r->ticket;
  }
  s->cv_work.notify_all();
  return SST_OK;
}

sst_status sst_server_wait(sst_server *s, uint64_t ticket, uint32_t timeout_ms,
                           sst_request_info *info) {
  if (!s) return SST_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) {
    sst::set_error_message("unknown ticket");
    return SST_EINVAL;
  }
  SrvRequest *r = it->second;
  bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                [&] { return r->done; });
  if (!ok) {
    sst::set_error_message("request %llu still running", (unsigned long long)ticket);
    return SST_ETIMEDOUT;
  }
  if (info) *info = r->info;
  sst_status st = r->info.status;
  s->all.erase(it);
  delete r;
  return st;
}

sst_status sst_server_stats(sst_server *s, uint64_t *epoch, uint64_t *passes,
                            uint64_t *update_edges) {
  if (!s) return SST_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  if (epoch) *epoch = s->epoch;
  if (passes) *passes = s->passes;
  if (update_edges) *update_edges = s->update_edges;
  return SST_OK;
}

sst_status sst_server_destroy(sst_server *s) {
  if (!s) return SST_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->writer.joinable()) s->writer.join();
  for (SrvSlot *slot : s->slots) {
    if (slot->th.joinable()) slot->th.join();
    sst_graph_destroy(slot->snap);
    delete slot;
  }
  for (auto &kv : s->all) delete kv.second;
  delete s;
  return SST_OK;
}

}  // extern "C"

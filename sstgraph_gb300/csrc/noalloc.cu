// PageRank that allocates nothing during the call.
//
// Some callers cannot let a library call allocate device memory: a serving
// loop that holds a fixed HBM budget must not have a request fail half-way
// on an allocation, and a host program that shares the GPU with other
// streams cannot afford cudaMalloc / cudaFree, which synchronise the whole
// device.  This entry point runs a pull PageRank with sst_pagerank's
// definition (results within 1e-9 relative: it sums FP64 values in warp
// order, where sst_pagerank sums exact fixed-point integers) with its
// scratch -- the two vectors of per-vertex contributions rank/deg -- in one
// file-scope device array of fixed size, so the call itself issues kernels
// and nothing else.  The graph handle and the output vector are the
// caller's, allocated beforehand.
//
// Limits and sharing: square graphs (column ids index the contribution
// vectors) of up to kNoAllocMaxVertices rows.  Every call in
// the process uses the same array, on whatever stream the graph is bound to:
// two calls that overlap on the GPU (different streams, or different graphs
// on the same device at once) race on it.  Each call initialises the part
// it reads, so nothing carries over from the previous call.
#include <map>
#include <mutex>

#include "graph.cuh"

namespace sst {
namespace {

constexpr uint32_t kNoAllocMaxVertices = 1u << 18;  // 262,144 rows: 4 MiB

// contribution vectors, ping-ponged between iterations
static __device__ __align__(256) double g_pr_scratch[2 * kNoAllocMaxVertices];

std::mutex g_sym_mu;
std::map<int, double *> g_sym_ptr;  // device ordinal -> address of the array

// Device address of the scratch array on the current device (set-up, once
// per device).  In host code the array's name is only a stand-in for it.
sst_status scratch_on_current_device(double **out) {
  int dev = 0;
  SST_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_sym_mu);
  auto it = g_sym_ptr.find(dev);
  if (it != g_sym_ptr.end()) {
    *out = it->second;
    return SST_OK;
  }
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_pr_scratch);
  if (e != cudaSuccess) {
    set_cuda_error(e, "cudaGetSymbolAddress(g_pr_scratch)", __FILE__, __LINE__);
    return SST_EDEVICE;
  }
  g_sym_ptr[dev] = static_cast<double *>(p);
  *out = static_cast<double *>(p);
  return SST_OK;
}

__global__ void k_pr_na_init(const uint32_t *__restrict__ deg, uint32_t n,
                             double r0, double *__restrict__ contrib,
                             double *__restrict__ rank) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  uint32_t d = deg[v];
  contrib[v] = d ? r0 / (double)d : 0.0;
  rank[v] = r0;
}

// warp per vertex: the same pull sum as sst_pagerank, one warp walking all
// leaves of the vertex
__global__ void k_pr_na_iter(DGraph g, const double *__restrict__ cin,
                             double *__restrict__ cout, double *__restrict__ rank,
                             double base, double damp) {
  uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (v >= g.n) return;
  uint32_t cap = g.cap[v], deg = g.deg[v];
  uint64_t sb = g.base[v];
  double acc = 0.0;
  if (cap > 0) {
    uint32_t nl = nleaves_of(cap);
    for (uint32_t l = 0; l < nl; l++) {
      uint32_t c = leaf_count(g, sb, cap, deg, l);
      if ((uint32_t)lane < c) acc += cin[g.slots[sb + ((uint64_t)l << kLeafLog) + lane]];
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
  if (lane == 0) {
    double r = base + damp * acc;
    rank[v] = r;
    cout[v] = deg ? r / (double)deg : 0.0;
  }
}

}  // namespace
}  // namespace sst

extern "C" {

// Declared in include/sstgraph.h.  The first call on a device resolves the
// scratch array's device address (cudaGetSymbolAddress); make that first
// call before capturing any stream.
sst_status sst_pagerank_noalloc(sst_graph *g, uint32_t iters, double damping,
                                double *d_rank) {
  using namespace sst;
  if (!g || !d_rank) {
    set_error_message("sst_pagerank_noalloc: null graph or output");
    return SST_EINVAL;
  }
  // column ids index the contribution vectors, which hold one entry per row
  if (g->n != g->width) {
    set_error_message("sst_pagerank_noalloc needs as many rows as columns (%u x %u)",
                      g->n, g->width);
    return SST_EINVAL;
  }
  if (g->n > kNoAllocMaxVertices) {
    set_error_message(
        "sst_pagerank_noalloc: %u rows exceed the fixed scratch of %u rows; "
        "use sst_pagerank",
        g->n, kNoAllocMaxVertices);
    return SST_EINVAL;
  }
  SST_CUDA_TRY(cudaSetDevice(g->device));
  double *scratch = nullptr;
  sst_status st = scratch_on_current_device(&scratch);
  if (st != SST_OK) return st;
  uint32_t n = g->n;
  if (n == 0) return SST_OK;
  cudaStream_t s = g->stream;
  double *ca = scratch, *cb = scratch + kNoAllocMaxVertices;
  double r0 = 1.0 / (double)n, base = (1.0 - damping) / (double)n;
  unsigned blocks = (n + 255) / 256;
  SST_LAUNCH(k_pr_na_init, blocks, 256, 0, s, g->d_deg, n, r0, ca, d_rank);
  DGraph dg = g->view();
  unsigned wblocks = (unsigned)(((uint64_t)n * 32 + 255) / 256);
  for (uint32_t it = 0; it < iters; it++) {
    SST_LAUNCH(k_pr_na_iter, wblocks, 256, 0, s, dg, ca, cb, d_rank, base, damping);
    double *t = ca;
    ca = cb;
    cb = t;
  }
  SST_CUDA_TRY(cudaGetLastError());
  return SST_OK;
}

}  // extern "C"

// The extern "C" boundary (include/sstgraph.h): argument checks, host
// staging of host-pointer arguments, and dispatch to the device paths.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "graph.cuh"
#include "traverse.cuh"

namespace sst {
const char *error_message();
void profile_start(const char *filter);
std::string profile_collect();
cudaError_t gen_rmat(uint32_t scale, double a, double b, double c, uint64_t seed,
                     uint64_t first, uint64_t count, uint32_t *d_pairs,
                     cudaStream_t s);
cudaError_t gen_er(uint32_t n, uint64_t seed, uint64_t first, uint64_t count,
                   uint32_t *d_pairs, cudaStream_t s);
cudaError_t gen_ref_rmat(uint32_t nn, double a, double b, double c,
                         uint64_t first, uint64_t count, uint32_t *d_pairs,
                         cudaStream_t s);
}  // namespace sst

using sst::set_error_message;

#define CHECK_G(g)                                                            \
  do {                                                                        \
    if (!(g)) {                                                               \
      set_error_message("null graph handle");                                 \
      return SST_EINVAL;                                                      \
    }                                                                         \
    if (cudaSetDevice((g)->device) != cudaSuccess) {                          \
      set_error_message("cannot select device %d", (g)->device);              \
      return SST_EDEVICE;                                                     \
    }                                                                         \
  } while (0)

// Traversals index per-vertex arrays of `rows` entries by column id, so a
// graph with more columns than rows would send them past those arrays: they
// take square graphs only (the reference's drivers build square, symmetric
// graphs, internal/test.hpp:407-450).
#define CHECK_SQUARE(g, what)                                                 \
  do {                                                                        \
    if ((g)->n != (g)->width) {                                               \
      set_error_message("%s needs as many rows as columns (%u x %u)", what,  \
                        (g)->n, (g)->width);                                  \
      return SST_EINVAL;                                                      \
    }                                                                         \
  } while (0)

namespace {

bool is_dev(uint32_t flags) { return (flags & SST_DEVICE_PTR) != 0; }

// Host-pointer calls stage their arrays in the graph's io arena: io_begin
// sizes it for the whole call, then stage_in / stage_out carve from it.
sst_status io_begin(sst_graph *g, size_t bytes) {
  g->io.reset();
  SST_CUDA_TRY(g->io.reserve(bytes + 8192));
  return SST_OK;
}

// device copy of a host input array (or the device pointer itself).  With
// `mapped`, for an input the kernels read once: pinned host memory is read
// by the kernel in place (over the host link, no separate copy).
template <typename T>
sst_status stage_in(sst_graph *g, const T *p, uint64_t count, uint32_t flags,
                    const T **out, bool mapped = false) {
  if (is_dev(flags) || count == 0) {
    *out = p;
    return SST_OK;
  }
  if (mapped) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost &&
        a.devicePointer) {
      *out = static_cast<const T *>(a.devicePointer);
      return SST_OK;
    }
    cudaGetLastError();  // pageable memory: copy it below
  }
  T *d = g->io.take<T>(count);
  if (!d) {
    set_error_message("staging buffer sizing error");
    return SST_ENOMEM;
  }
  SST_CUDA_TRY(cudaMemcpyAsync(d, p, count * sizeof(T), cudaMemcpyHostToDevice,
                               g->stream));
  *out = d;
  return SST_OK;
}

// device output buffer for a host output
template <typename T>
sst_status stage_out(sst_graph *g, T *p, uint64_t count, uint32_t flags,
                     T **dev) {
  if (is_dev(flags)) {
    *dev = p;
    return SST_OK;
  }
  *dev = g->io.take<T>(count ? count : 1);
  if (!*dev) {
    set_error_message("staging buffer sizing error");
    return SST_ENOMEM;
  }
  return SST_OK;
}

template <typename T>
sst_status finish_out(sst_graph *g, T *host, const T *dev, uint64_t count,
                      uint32_t flags) {
  if (is_dev(flags)) return SST_OK;
  if (count)
    SST_CUDA_TRY(cudaMemcpyAsync(host, dev, count * sizeof(T),
                                 cudaMemcpyDeviceToHost, g->stream));
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  return SST_OK;
}

}  // namespace

extern "C" {

const char *sst_last_error_message(void) { return sst::error_message(); }

const char *sst_status_string(sst_status s) {
  switch (s) {
    case SST_OK: return "ok";
    case SST_EINVAL: return "invalid argument";
    case SST_ENOMEM: return "out of device memory";
    case SST_EBUDGET: return "HBM budget exceeded";
    case SST_ETIMEDOUT: return "device wait timed out";
    case SST_EDEVICE: return "CUDA device error";
    case SST_ESTATE: return "invalid state";
  }
  return "unknown status";
}

uint64_t sst_kernel_launches(void) { return sst::launches(); }

sst_status sst_set_scan_lookback_polls(uint32_t polls, uint32_t *old) {
  if (old) *old = (uint32_t)sst::lookback_polls();
  sst::set_lookback_polls(polls > (1u << 30) ? (1 << 30) : (int)polls);
  return SST_OK;
}

sst_status sst_profile_start(const char *kernel_filter) {
  sst::profile_start(kernel_filter);
  return SST_OK;
}

sst_status sst_profile_collect(char *buf, uint64_t cap) {
  if (!buf || cap == 0) return SST_EINVAL;
  std::string s = sst::profile_collect();
  size_t k = std::min<size_t>(s.size(), cap - 1);
  memcpy(buf, s.data(), k);
  buf[k] = 0;
  return SST_OK;
}

sst_status sst_raw_state(sst_graph *g, uint64_t *base, uint32_t *cap,
                         uint32_t *deg, uint32_t *slots, uint8_t *lcnt,
                         uint64_t *nslots) {
  CHECK_G(g);
  if (!nslots) return SST_EINVAL;
  cudaStream_t s = g->stream;
  SST_CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t n = g->n;
  if (base) SST_CUDA_TRY(cudaMemcpy(base, g->d_base, n * 8, cudaMemcpyDeviceToHost));
  if (cap) SST_CUDA_TRY(cudaMemcpy(cap, g->d_cap, n * 4, cudaMemcpyDeviceToHost));
  if (deg) SST_CUDA_TRY(cudaMemcpy(deg, g->d_deg, n * 4, cudaMemcpyDeviceToHost));
  uint64_t used = (g->bump + 31) & ~uint64_t(31);
  if (slots) SST_CUDA_TRY(cudaMemcpy(slots, g->d_slots, std::min(*nslots, used) * 4, cudaMemcpyDeviceToHost));
  if (lcnt) SST_CUDA_TRY(cudaMemcpy(lcnt, g->d_lcnt, std::min(*nslots, used) / 32, cudaMemcpyDeviceToHost));
  *nslots = used;
  return SST_OK;
}

sst_status sst_graph_create(uint32_t height, uint32_t width,
                            const sst_config *cfg, sst_graph **out) {
  if (!out) {
    set_error_message("null output handle");
    return SST_EINVAL;
  }
  *out = nullptr;
  if (width == 0xFFFFFFFFu) {
    set_error_message("width must be below 2^32-1 (0xFFFFFFFF marks a gap)");
    return SST_EINVAL;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error_message("no CUDA device available");
    return SST_EDEVICE;
  }
  sst_graph *g = new (std::nothrow) sst_graph();
  if (!g) return SST_ENOMEM;
  sst_status st = sst::graph_init(g, height, width, cfg);
  if (st != SST_OK) {
    sst::graph_release(g);
    delete g;
    return st;
  }
  *out = g;
  return SST_OK;
}

sst_status sst_graph_destroy(sst_graph *g) {
  if (!g) return SST_OK;
  sst::graph_release(g);
  delete g;
  return SST_OK;
}

sst_status sst_graph_clone(const sst_graph *src, sst_graph **out) {
  if (!src || !out) {
    set_error_message("null argument");
    return SST_EINVAL;
  }
  SST_CUDA_TRY(cudaSetDevice(src->device));
  sst_graph *g = new (std::nothrow) sst_graph();
  if (!g) return SST_ENOMEM;
  sst_status st = sst::graph_clone(src, g);
  if (st != SST_OK) {
    sst::graph_release(g);
    delete g;
    return st;
  }
  *out = g;
  return SST_OK;
}

sst_status sst_set_stream(sst_graph *g, void *stream) {
  CHECK_G(g);
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  g->stream = stream ? static_cast<cudaStream_t>(stream) : g->own_stream;
  return SST_OK;
}

sst_status sst_set_plan_graphs(sst_graph *g, int enable) {
  CHECK_G(g);
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  if (enable < 0 || enable > 2) {
    set_error_message("plan graph mode must be 0, 1 or 2");
    return SST_EINVAL;
  }
  g->plan_graphs = enable != 0;
  g->plan_direct = enable == 2;
  if (!enable) sst::plan_cache_release(g);
  return SST_OK;
}

sst_status sst_sync(sst_graph *g) {
  CHECK_G(g);
  return sst::sync_checked(g);
}

static sst_status do_update(sst_graph *g, const uint32_t *pairs, uint64_t n,
                            uint32_t flags, uint64_t *n_invalid, bool insert,
                            const uint32_t *values = nullptr) {
  CHECK_G(g);
  if (n && !pairs) {
    set_error_message("null pairs");
    return SST_EINVAL;
  }
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, n * 12 + 512);
  if (st != SST_OK) return st;
  // the key build reads each pair (and value) once: pinned host inputs are
  // read in place; the plan readback inside the update comes after it
  const uint32_t *d = nullptr, *dv = nullptr;
  st = stage_in(g, pairs, 2 * n, flags, &d, true);
  if (st != SST_OK) return st;
  if (values) st = stage_in(g, values, n, flags, &dv, true);
  if (st != SST_OK) return st;
  st = sst::update_batch(g, d, n, insert, n_invalid, dv);
  if (st == SST_OK && !is_dev(flags)) st = sst::sync_checked(g);
  return st;
}

sst_status sst_insert_batch(sst_graph *g, const uint32_t *pairs, uint64_t n,
                            uint32_t flags, uint64_t *n_invalid) {
  return do_update(g, pairs, n, flags, n_invalid, true);
}

sst_status sst_remove_batch(sst_graph *g, const uint32_t *pairs, uint64_t n,
                            uint32_t flags, uint64_t *n_invalid) {
  return do_update(g, pairs, n, flags, n_invalid, false);
}

sst_status sst_insert_batch_weighted(sst_graph *g, const uint32_t *pairs,
                                     const uint32_t *values, uint64_t n,
                                     uint32_t flags, uint64_t *n_invalid) {
  CHECK_G(g);
  if (!g->weighted) {
    set_error_message("the graph was not created weighted (sst_config.weighted)");
    return SST_ESTATE;
  }
  if (n && !values) {
    set_error_message("null values");
    return SST_EINVAL;
  }
  return do_update(g, pairs, n, flags, n_invalid, true, values);
}

sst_status sst_values_batch(sst_graph *g, const uint32_t *pairs, uint64_t n,
                            uint32_t *values, uint8_t *found, uint32_t flags) {
  CHECK_G(g);
  if (!g->weighted) {
    set_error_message("the graph was not created weighted (sst_config.weighted)");
    return SST_ESTATE;
  }
  if (n && (!pairs || !values)) {
    set_error_message("null argument");
    return SST_EINVAL;
  }
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, n * 13 + 1024);
  if (st != SST_OK) return st;
  const uint32_t *d = nullptr;
  st = stage_in(g, pairs, 2 * n, flags, &d);
  if (st != SST_OK) return st;
  uint32_t *dval = nullptr;
  uint8_t *dfound = nullptr;
  st = stage_out(g, values, n, flags, &dval);
  if (st == SST_OK && found) st = stage_out(g, found, n, flags, &dfound);
  if (st != SST_OK) return st;
  st = sst::has_batch(g, d, n, dfound, dval);
  if (st != SST_OK) return st;
  if (found) st = finish_out(g, found, dfound, n, flags);
  if (st != SST_OK) return st;
  return finish_out(g, values, dval, n, flags);
}

sst_status sst_update_batches(sst_graph *g, const uint32_t *pairs,
                              const uint64_t *offsets, const uint8_t *ops,
                              uint32_t nbatches, uint32_t flags,
                              uint64_t *n_invalid) {
  CHECK_G(g);
  if (g->weighted) {
    set_error_message("the batched form takes unweighted graphs only");
    return SST_ESTATE;
  }
  if (n_invalid) *n_invalid = 0;
  if (nbatches == 0) return SST_OK;
  if (!offsets || !ops) {
    set_error_message("null offsets or ops");
    return SST_EINVAL;
  }
  uint64_t N = 0;
  if (is_dev(flags)) {
    SST_CUDA_TRY(cudaMemcpyAsync(&N, offsets + nbatches, 8, cudaMemcpyDeviceToHost, g->stream));
    SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  } else {
    N = offsets[nbatches];
  }
  if (N && !pairs) {
    set_error_message("null pairs");
    return SST_EINVAL;
  }
  sst_status st = is_dev(flags) ? SST_OK
                                : io_begin(g, N * 8 + (nbatches + 1) * 9 + 1024);
  if (st != SST_OK) return st;
  const uint32_t *dp = nullptr;
  const uint64_t *doff = nullptr;
  const uint8_t *dops = nullptr;
  st = stage_in(g, pairs, 2 * N, flags, &dp);
  if (st == SST_OK) st = stage_in(g, offsets, (uint64_t)nbatches + 1, flags, &doff);
  if (st == SST_OK) st = stage_in(g, ops, (uint64_t)nbatches, flags, &dops);
  if (st != SST_OK) return st;
  st = sst::update_batches(g, dp, doff, dops, nbatches, N, n_invalid);
  if (st == SST_OK && !is_dev(flags)) st = sst::sync_checked(g);
  return st;
}

sst_status sst_insert(sst_graph *g, uint32_t row, uint32_t col) {
  uint32_t p[2] = {row, col};
  uint64_t bad = 0;
  sst_status st = sst_insert_batch(g, p, 1, SST_HOST_PTR, &bad);
  if (st == SST_OK && bad) {
    set_error_message("id out of range");
    return SST_EINVAL;
  }
  return st;
}

sst_status sst_remove(sst_graph *g, uint32_t row, uint32_t col) {
  uint32_t p[2] = {row, col};
  uint64_t bad = 0;
  sst_status st = sst_remove_batch(g, p, 1, SST_HOST_PTR, &bad);
  if (st == SST_OK && bad) {
    set_error_message("id out of range");
    return SST_EINVAL;
  }
  return st;
}

sst_status sst_build_from_csr(sst_graph *g, const uint64_t *offsets,
                              const uint32_t *cols, uint32_t flags) {
  CHECK_G(g);
  if (g->weighted) {
    set_error_message("building from a CSR takes unweighted graphs only");
    return SST_ESTATE;
  }
  if (!offsets) {
    set_error_message("null offsets");
    return SST_EINVAL;
  }
  if (is_dev(flags)) return sst::build_from_csr(g, offsets, cols);
  uint64_t m = offsets[g->n];
  uint64_t *doff = nullptr;
  uint32_t *dcols = nullptr;
  SST_CUDA_TRY(cudaMalloc(&doff, ((uint64_t)g->n + 1) * 8));
  SST_CUDA_TRY(cudaMalloc(&dcols, std::max<uint64_t>(m, 1) * 4));
  SST_CUDA_TRY(cudaMemcpyAsync(doff, offsets, ((uint64_t)g->n + 1) * 8,
                               cudaMemcpyHostToDevice, g->stream));
  if (m) SST_CUDA_TRY(cudaMemcpyAsync(dcols, cols, m * 4, cudaMemcpyHostToDevice, g->stream));
  sst_status st = sst::build_from_csr(g, doff, dcols);
  cudaStreamSynchronize(g->stream);
  cudaFree(doff);
  cudaFree(dcols);
  return st;
}

sst_status sst_has_batch(sst_graph *g, const uint32_t *pairs, uint64_t n,
                         uint8_t *out, uint32_t flags) {
  CHECK_G(g);
  if (n && (!pairs || !out)) {
    set_error_message("null argument");
    return SST_EINVAL;
  }
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, n * 9 + 512);
  if (st != SST_OK) return st;
  const uint32_t *d = nullptr;
  st = stage_in(g, pairs, 2 * n, flags, &d);
  if (st != SST_OK) return st;
  uint8_t *dout = nullptr;
  st = stage_out(g, out, n, flags, &dout);
  if (st != SST_OK) return st;
  st = sst::has_batch(g, d, n, dout);
  if (st != SST_OK) return st;
  return finish_out(g, out, dout, n, flags);
}

sst_status sst_has(sst_graph *g, uint32_t row, uint32_t col, int *out) {
  if (!out) {
    set_error_message("null argument");
    return SST_EINVAL;
  }
  uint32_t p[2] = {row, col};
  uint8_t r = 0;
  sst_status st = sst_has_batch(g, p, 1, &r, SST_HOST_PTR);
  *out = r;
  return st;
}

sst_status sst_num_nodes(const sst_graph *g, uint64_t *out) {
  if (!g || !out) return SST_EINVAL;
  *out = g->n;
  return SST_OK;
}
sst_status sst_get_rows(const sst_graph *g, uint32_t *out) {
  if (!g || !out) return SST_EINVAL;
  *out = g->n;
  return SST_OK;
}
sst_status sst_get_cols(const sst_graph *g, uint32_t *out) {
  if (!g || !out) return SST_EINVAL;
  *out = g->width;
  return SST_OK;
}

sst_status sst_M(sst_graph *g, uint64_t *out) {
  if (!g || !out) return SST_EINVAL;
  *out = g->m;
  return SST_OK;
}

sst_status sst_degrees(sst_graph *g, uint32_t *out, uint32_t flags) {
  CHECK_G(g);
  if (!out) return SST_EINVAL;
  if (is_dev(flags)) {
    SST_CUDA_TRY(cudaMemcpyAsync(out, g->d_deg, (uint64_t)g->n * 4,
                                 cudaMemcpyDeviceToDevice, g->stream));
    return SST_OK;
  }
  SST_CUDA_TRY(cudaMemcpyAsync(out, g->d_deg, (uint64_t)g->n * 4,
                               cudaMemcpyDeviceToHost, g->stream));
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  return SST_OK;
}

sst_status sst_get_degree(sst_graph *g, uint32_t v, uint32_t *out) {
  CHECK_G(g);
  if (!out || v >= g->n) {
    set_error_message("vertex out of range");
    return SST_EINVAL;
  }
  SST_CUDA_TRY(cudaMemcpyAsync(out, g->d_deg + v, 4, cudaMemcpyDeviceToHost, g->stream));
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  return SST_OK;
}

sst_status sst_neighbors(sst_graph *g, uint32_t v, uint32_t *out, uint64_t cap,
                         uint64_t *deg) {
  CHECK_G(g);
  if (!deg || v >= g->n || (cap && !out)) {
    set_error_message("bad argument to sst_neighbors");
    return SST_EINVAL;
  }
  uint32_t d = 0;
  SST_CUDA_TRY(cudaMemcpyAsync(&d, g->d_deg + v, 4, cudaMemcpyDeviceToHost, g->stream));
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  uint64_t take = std::min<uint64_t>(cap, d);
  sst_status st0 = io_begin(g, (uint64_t)d * 4 + 256);
  if (st0 != SST_OK) return st0;
  uint32_t *dout = g->io.take<uint32_t>(std::max<uint32_t>(d, 1));
  uint64_t full = 0;
  sst_status st = sst::neighbors(g, v, dout, d, &full);
  if (st != SST_OK) return st;
  *deg = full;
  if (take)
    SST_CUDA_TRY(cudaMemcpyAsync(out, dout, take * 4, cudaMemcpyDeviceToHost, g->stream));
  SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  return SST_OK;
}

static sst_status csr_out(sst_graph *g, uint64_t *offsets, uint32_t *cols,
                          uint32_t *vals, uint32_t flags) {
  CHECK_G(g);
  if (!offsets || (g->m && !cols)) return SST_EINVAL;
  if (is_dev(flags)) return sst::to_csr(g, offsets, cols, vals);
  uint64_t *doff = nullptr;
  uint32_t *dcols = nullptr, *dvals = nullptr;
  SST_CUDA_TRY(cudaMalloc(&doff, ((uint64_t)g->n + 1) * 8));
  SST_CUDA_TRY(cudaMalloc(&dcols, std::max<uint64_t>(g->m, 1) * 4));
  if (vals) SST_CUDA_TRY(cudaMalloc(&dvals, std::max<uint64_t>(g->m, 1) * 4));
  sst_status st = sst::to_csr(g, doff, dcols, dvals);
  if (st == SST_OK) {
    cudaMemcpyAsync(offsets, doff, ((uint64_t)g->n + 1) * 8, cudaMemcpyDeviceToHost, g->stream);
    if (g->m) cudaMemcpyAsync(cols, dcols, g->m * 4, cudaMemcpyDeviceToHost, g->stream);
    if (g->m && vals) cudaMemcpyAsync(vals, dvals, g->m * 4, cudaMemcpyDeviceToHost, g->stream);
    if (cudaStreamSynchronize(g->stream) != cudaSuccess) st = SST_EDEVICE;
  }
  cudaFree(doff);
  cudaFree(dcols);
  if (dvals) cudaFree(dvals);
  return st;
}

sst_status sst_to_csr(sst_graph *g, uint64_t *offsets, uint32_t *cols,
                      uint32_t flags) {
  return csr_out(g, offsets, cols, nullptr, flags);
}

sst_status sst_to_csr_values(sst_graph *g, uint64_t *offsets, uint32_t *cols,
                             uint32_t *values, uint32_t flags) {
  if (g && !g->weighted) {
    set_error_message("the graph was not created weighted (sst_config.weighted)");
    return SST_ESTATE;
  }
  if (g && g->m && !values) return SST_EINVAL;
  return csr_out(g, offsets, cols, values, flags);
}

sst_status sst_touch_all_sum(sst_graph *g, uint64_t *out) {
  CHECK_G(g);
  if (!out) return SST_EINVAL;
  return sst::touch_all_sum(g, out);
}

sst_status sst_touch_all(sst_graph *g, uint64_t *out) {
  return sst_touch_all_sum(g, out);
}

sst_status sst_release_scratch(sst_graph *g) {
  CHECK_G(g);
  return sst::release_scratch(g);
}

sst_status sst_memory_size(sst_graph *g, uint64_t *out) {
  if (!g || !out) return SST_EINVAL;
  *out = sst::graph_device_bytes(g);
  return SST_OK;
}

sst_status sst_sample_edges(sst_graph *g, uint64_t seed, uint64_t first,
                            uint64_t count, uint32_t *pairs, uint32_t flags) {
  CHECK_G(g);
  if (count && !pairs) return SST_EINVAL;
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, count * 8 + 256);
  if (st != SST_OK) return st;
  uint32_t *d = nullptr;
  st = stage_out(g, pairs, 2 * count, flags, &d);
  if (st != SST_OK) return st;
  st = sst::sample_edges(g, seed, first, count, d);
  if (st != SST_OK) return st;
  return finish_out(g, pairs, d, 2 * count, flags);
}

sst_status sst_tc_vertices(sst_graph *g, const uint32_t *vertices, uint64_t k,
                           uint64_t *out, uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_tc_vertices");
  if (k && (!vertices || !out)) return SST_EINVAL;
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, k * 12 + 512);
  if (st != SST_OK) return st;
  const uint32_t *dv = nullptr;
  st = stage_in(g, vertices, k, flags, &dv);
  if (st != SST_OK) return st;
  uint64_t *dout = nullptr;
  st = stage_out(g, out, k, flags, &dout);
  if (st != SST_OK) return st;
  st = sst::tc_vertices(g, dv, k, dout);
  if (st != SST_OK) return st;
  return finish_out(g, out, dout, k, flags);
}

sst_status sst_degree_order_map(sst_graph *g, uint32_t *map, uint32_t flags) {
  CHECK_G(g);
  if (!map) return SST_EINVAL;
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, (uint64_t)g->n * 4 + 256);
  if (st != SST_OK) return st;
  uint32_t *d = nullptr;
  st = stage_out(g, map, g->n, flags, &d);
  if (st != SST_OK) return st;
  st = sst::degree_order_map(g, d);
  if (st != SST_OK) return st;
  return finish_out(g, map, d, g->n, flags);
}

sst_status sst_rewrite_graph(sst_graph *g, const uint32_t *map, uint32_t flags,
                             sst_graph **out) {
  CHECK_G(g);
  if (g->weighted) {
    set_error_message("relabelling takes unweighted graphs only");
    return SST_ESTATE;
  }
  if (!map || !out) return SST_EINVAL;
  *out = nullptr;
  if (g->n != g->width) {
    set_error_message("rewrite_graph needs as many rows as columns");
    return SST_EINVAL;
  }
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, (uint64_t)g->n * 4 + 256);
  if (st != SST_OK) return st;
  const uint32_t *d = nullptr;
  st = stage_in(g, map, g->n, flags, &d);
  if (st != SST_OK) return st;
  sst_config cfg{};
  cfg.device = g->device;
  cfg.hbm_budget_bytes = g->budget;
  cfg.initial_slots = g->nslots;
  cfg.upper_root = g->params.upper_root;
  cfg.lower_root = g->params.lower_root;
  cfg.grow_fill = g->params.grow_fill;
  sst_graph *ng = new (std::nothrow) sst_graph();
  if (!ng) return SST_ENOMEM;
  st = sst::graph_init(ng, g->n, g->width, &cfg);
  if (st == SST_OK) st = sst::rewrite_graph(g, d, ng);
  if (st != SST_OK) {
    sst::graph_release(ng);
    delete ng;
    return st;
  }
  *out = ng;
  return SST_OK;
}

sst_status sst_common_neighbors_batch(sst_graph *g, const uint32_t *pairs,
                                      uint64_t n, int early_end, uint64_t *out,
                                      uint32_t flags) {
  CHECK_G(g);
  if (n && (!pairs || !out)) return SST_EINVAL;
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, n * 16 + 512);
  if (st != SST_OK) return st;
  const uint32_t *d = nullptr;
  st = stage_in(g, pairs, 2 * n, flags, &d);
  if (st != SST_OK) return st;
  uint64_t *dout = nullptr;
  st = stage_out(g, out, n, flags, &dout);
  if (st != SST_OK) return st;
  st = sst::common_neighbors_batch(g, d, n, early_end != 0, dout);
  if (st != SST_OK) return st;
  return finish_out(g, out, dout, n, flags);
}

sst_status sst_bfs(sst_graph *g, uint32_t src, int32_t *parents,
                   int32_t *depths, uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_bfs");
  if (src >= g->n) {
    set_error_message("source out of range");
    return SST_EINVAL;
  }
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, (uint64_t)g->n * 8 + 512);
  if (st != SST_OK) return st;
  int32_t *dp = nullptr, *dd = nullptr;
  if (parents) st = stage_out(g, parents, g->n, flags, &dp);
  if (st == SST_OK && depths) st = stage_out(g, depths, g->n, flags, &dd);
  if (st != SST_OK) return st;
  st = sst::bfs(g, src, dp, dd);
  if (st != SST_OK) return st;
  if (parents) st = finish_out(g, parents, dp, g->n, flags);
  if (st == SST_OK && depths) st = finish_out(g, depths, dd, g->n, flags);
  return st;
}

// sources come to the host for validation and the source table
static sst_status sources_to_host(sst_graph *g, const uint32_t *srcs,
                                  uint32_t k, uint32_t flags,
                                  std::vector<uint32_t> *out) {
  out->resize(k);
  if (!k) return SST_OK;
  if (is_dev(flags)) {
    SST_CUDA_TRY(cudaMemcpyAsync(out->data(), srcs, (uint64_t)k * 4,
                                 cudaMemcpyDeviceToHost, g->stream));
    SST_CUDA_TRY(cudaStreamSynchronize(g->stream));
  } else {
    memcpy(out->data(), srcs, (uint64_t)k * 4);
  }
  for (uint32_t i = 0; i < k; i++)
    if ((*out)[i] >= g->n) {
      set_error_message("source %u out of range", (*out)[i]);
      return SST_EINVAL;
    }
  return SST_OK;
}

sst_status sst_bfs_multi(sst_graph *g, const uint32_t *srcs, uint32_t k,
                         int32_t *depths, uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_bfs_multi");
  if (k > 64 || (k && (!srcs || !depths))) {
    set_error_message(k > 64 ? "at most 64 sources" : "null argument");
    return SST_EINVAL;
  }
  if (!k) return SST_OK;
  std::vector<uint32_t> hs;
  sst_status st = sources_to_host(g, srcs, k, flags, &hs);
  if (st != SST_OK) return st;
  const uint64_t cnt = (uint64_t)k * g->n;
  st = is_dev(flags) ? SST_OK : io_begin(g, cnt * 4 + 512);
  if (st != SST_OK) return st;
  int32_t *d = nullptr;
  st = stage_out(g, depths, cnt, flags, &d);
  if (st != SST_OK) return st;
  st = sst::bfs_multi(g, hs.data(), k, d);
  if (st != SST_OK) return st;
  return finish_out(g, depths, d, cnt, flags);
}

sst_status sst_bc_multi(sst_graph *g, const uint32_t *srcs, uint32_t k,
                        double *out, uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_bc_multi");
  if (k > 64 || (k && (!srcs || !out))) {
    set_error_message(k > 64 ? "at most 64 sources" : "null argument");
    return SST_EINVAL;
  }
  if (!k) return SST_OK;
  std::vector<uint32_t> hs;
  sst_status st = sources_to_host(g, srcs, k, flags, &hs);
  if (st != SST_OK) return st;
  const uint64_t cnt = (uint64_t)k * g->n;
  st = is_dev(flags) ? SST_OK : io_begin(g, cnt * 8 + 512);
  if (st != SST_OK) return st;
  double *d = nullptr;
  st = stage_out(g, out, cnt, flags, &d);
  if (st != SST_OK) return st;
  st = sst::bc_multi(g, hs.data(), k, d);
  if (st != SST_OK) return st;
  return finish_out(g, out, d, cnt, flags);
}

sst_status sst_bf(sst_graph *g, uint32_t src, int32_t *dist, uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_bf");
  if (!dist) return SST_EINVAL;
  if (src >= g->n) {
    set_error_message("source out of range");
    return SST_EINVAL;
  }
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, (uint64_t)g->n * 4 + 256);
  if (st != SST_OK) return st;
  int32_t *d = nullptr;
  st = stage_out(g, dist, g->n, flags, &d);
  if (st != SST_OK) return st;
  st = sst::bellman_ford(g, src, d);
  if (st != SST_OK) return st;
  return finish_out(g, dist, d, g->n, flags);
}

sst_status sst_autotune(sst_graph *g, sst_tuning *out) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_autotune");
  if (!out) return SST_EINVAL;
  return sst::autotune(g, out);
}

sst_status sst_get_tuning(sst_graph *g, sst_tuning *out) {
  CHECK_G(g);
  if (!out) return SST_EINVAL;
  return sst::get_tuning(g, out);
}

sst_status sst_set_tuning(sst_graph *g, const sst_tuning *in) {
  CHECK_G(g);
  if (!in) return SST_EINVAL;
  return sst::set_tuning(g, in);
}

sst_status sst_pagerank(sst_graph *g, uint32_t iters, double damping,
                        double *out, uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_pagerank");
  if (!out) return SST_EINVAL;
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, (uint64_t)g->n * 8 + 256);
  if (st != SST_OK) return st;
  double *d = nullptr;
  st = stage_out(g, out, g->n, flags, &d);
  if (st != SST_OK) return st;
  st = sst::pagerank(g, iters, damping, d);
  if (st != SST_OK) return st;
  return finish_out(g, out, d, g->n, flags);
}

sst_status sst_cc(sst_graph *g, uint32_t *labels, uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_cc");
  if (!labels) return SST_EINVAL;
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, (uint64_t)g->n * 4 + 256);
  if (st != SST_OK) return st;
  uint32_t *d = nullptr;
  st = stage_out(g, labels, g->n, flags, &d);
  if (st != SST_OK) return st;
  st = sst::cc(g, d);
  if (st != SST_OK) return st;
  return finish_out(g, labels, d, g->n, flags);
}

sst_status sst_bc(sst_graph *g, uint32_t src, double *out, uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_bc");
  if (!out || src >= g->n) {
    set_error_message("bad argument to sst_bc");
    return SST_EINVAL;
  }
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, (uint64_t)g->n * 8 + 256);
  if (st != SST_OK) return st;
  double *d = nullptr;
  st = stage_out(g, out, g->n, flags, &d);
  if (st != SST_OK) return st;
  st = sst::bc(g, src, d);
  if (st != SST_OK) return st;
  return finish_out(g, out, d, g->n, flags);
}

sst_status sst_tc(sst_graph *g, uint64_t *total, uint64_t *per_vertex,
                  uint32_t flags) {
  CHECK_G(g);
  CHECK_SQUARE(g, "sst_tc");
  if (!total) return SST_EINVAL;
  sst_status st = is_dev(flags) ? SST_OK : io_begin(g, (uint64_t)g->n * 8 + 256);
  if (st != SST_OK) return st;
  uint64_t *dpv = nullptr;
  if (per_vertex) st = stage_out(g, per_vertex, g->n, flags, &dpv);
  if (st != SST_OK) return st;
  st = sst::tc(g, total, dpv);
  if (st != SST_OK) return st;
  if (per_vertex) return finish_out(g, per_vertex, dpv, g->n, flags);
  return SST_OK;
}

// ---- generators: no graph handle; host outputs go through a temporary
static sst_status gen_common(uint64_t count, uint32_t *pairs, uint32_t flags,
                             cudaError_t (*fn)(uint32_t *, cudaStream_t, void *),
                             void *ctx) {
  if (count && !pairs) return SST_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error_message("no CUDA device available");
    return SST_EDEVICE;
  }
  if (is_dev(flags)) {
    SST_CUDA_TRY(fn(pairs, 0, ctx));
    SST_CUDA_TRY(cudaStreamSynchronize(0));
    return SST_OK;
  }
  uint32_t *d = nullptr;
  SST_CUDA_TRY(cudaMalloc(&d, std::max<uint64_t>(count, 1) * 8));
  cudaError_t e = fn(d, 0, ctx);
  if (e == cudaSuccess)
    e = cudaMemcpy(pairs, d, count * 8, cudaMemcpyDeviceToHost);
  cudaFree(d);
  SST_CUDA_TRY(e);
  return SST_OK;
}

struct RmatCtx {
  uint32_t scale;
  double a, b, c;
  uint64_t seed, first, count;
};

sst_status sst_gen_rmat(uint32_t scale, double a, double b, double c,
                        uint64_t seed, uint64_t first, uint64_t count,
                        uint32_t *pairs, uint32_t flags) {
  if (scale == 0 || scale > 32 || a + b + c > 1.0) {
    set_error_message("bad RMAT parameters");
    return SST_EINVAL;
  }
  RmatCtx ctx{scale, a, b, c, seed, first, count};
  return gen_common(count, pairs, flags,
                    [](uint32_t *d, cudaStream_t s, void *p) {
                      RmatCtx *x = static_cast<RmatCtx *>(p);
                      return sst::gen_rmat(x->scale, x->a, x->b, x->c, x->seed,
                                           x->first, x->count, d, s);
                    },
                    &ctx);
}

sst_status sst_gen_er(uint32_t n, uint64_t seed, uint64_t first, uint64_t count,
                      uint32_t *pairs, uint32_t flags) {
  if (n == 0) return SST_EINVAL;
  RmatCtx ctx{n, 0, 0, 0, seed, first, count};
  return gen_common(count, pairs, flags,
                    [](uint32_t *d, cudaStream_t s, void *p) {
                      RmatCtx *x = static_cast<RmatCtx *>(p);
                      return sst::gen_er(x->scale, x->seed, x->first, x->count,
                                         d, s);
                    },
                    &ctx);
}

sst_status sst_gen_ref_rmat(uint32_t nn, double a, double b, double c,
                            uint64_t first, uint64_t count, uint32_t *pairs,
                            uint32_t flags) {
  if (nn == 0 || (nn & (nn - 1)) != 0 || a + b + c > 1.0) {
    set_error_message("nn must be a power of two and a+b+c <= 1");
    return SST_EINVAL;
  }
  RmatCtx ctx{nn, a, b, c, 0, first, count};
  return gen_common(count, pairs, flags,
                    [](uint32_t *d, cudaStream_t s, void *p) {
                      RmatCtx *x = static_cast<RmatCtx *>(p);
                      return sst::gen_ref_rmat(x->scale, x->a, x->b, x->c,
                                               x->first, x->count, d, s);
                    },
                    &ctx);
}

}  // extern "C"

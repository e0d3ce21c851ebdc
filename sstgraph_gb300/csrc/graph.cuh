// Host-side graph object shared by the C ABI, the update path and the
// traversal path.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sstgraph.h"
#include "common.cuh"
#include "primitives.cuh"

namespace sst {
struct PlanCache;  // captured planning launches of update batches (graph.cu)

// Summary of a planned batch, copied to the host once per batch: it sizes
// the apply launches, the window scratch and the slab allocation.
struct PlanSummary {
  uint32_t n_items;      // unique valid keys that change the graph
  uint32_t n_groups;     // (row, leaf) groups among them
  uint32_t n_merge;      // leaf-local merge tasks
  uint32_t n_tasks;      // window / resize tasks
  uint32_t n_climb;      // groups whose leaf over- or underflowed
  uint64_t task_elems;   // elements staged by window / resize tasks
  uint64_t src_leaves;   // leaves read by those tasks
  uint64_t dst_leaves;   // leaves written by those tasks
  uint64_t invalid;      // pairs with an id out of range
  uint32_t class_cnt[kNumClasses];  // new segments per capacity class
  unsigned long long apply_err;     // staged ranks out of range (must be 0)
  uint32_t n_keys;                  // keys kept by a compacting key build
  uint32_t n_hard;                  // tasks set up a warp each (k_task_setup_hard)
};

// Flattened list of all leaves in vertex order: the iteration space of the
// copy-out, sampling and traversal kernels.  Rebuilt when the graph version
// changes.
struct TravState;

struct LeafDir {
  uint64_t version = ~0ull;
  uint64_t nleaves = 0;
  uint64_t cap = 0;
  uint32_t *owner = nullptr;  // vertex of each leaf
  uint64_t *slot = nullptr;   // first slot of each leaf
  uint32_t *cnt = nullptr;    // elements in each leaf
  uint64_t *pre = nullptr;    // exclusive prefix of cnt = CSR position
  uint64_t *vleaf = nullptr;  // per vertex: index of its first leaf (n+1)
  void release();
};

}  // namespace sst

struct sst_graph {
  int device = 0;
  int sms = 148;  // multiprocessors of the device
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaEvent_t plan_ready = nullptr;  // an update's plan has reached the host
  cudaStream_t side = nullptr;  // an update's leaf merges, beside its tasks;
                                // its planning launches are captured here
  cudaEvent_t fork_ev = nullptr, merge_done = nullptr;
  // independent scans of an update's planning sequence run here, forked
  // from its stream and joined back (inside a captured plan: parallel
  // branches of the graph)
  cudaStream_t aux[2] = {nullptr, nullptr};
  cudaEvent_t aux_fork = nullptr, aux_join[2] = {nullptr, nullptr};
  sst::PlanCache *plans = nullptr;  // captured planning launches
  bool plan_graphs = true;  // replay planning launches (off: launch directly)
  bool plan_direct = false; // with plan_graphs: launch them directly, in the
                            // kernel forms of a replay (per-kernel timing)
  uint32_t n = 0, width = 0;
  int rbits = 0, dbits = 0;
  sst::PmaParams params;
  uint64_t budget = 0;
  bool keep_loops = false;  // inserts keep (v, v) (per-row sets)

  uint64_t *d_base = nullptr;
  uint32_t *d_cap = nullptr;
  uint32_t *d_deg = nullptr;
  uint32_t *d_slots = nullptr;
  uint8_t *d_lcnt = nullptr;
  uint32_t *d_vals = nullptr;  // weighted graphs: one value per slot
  bool weighted = false;
  uint64_t nslots = 0;
  uint64_t bump = 0;
  uint64_t m = 0;
  uint64_t version = 0;

  sst::Arena arena;  // per-operation scratch
  sst::Arena work;   // window / resize staging
  sst::Arena io;     // device copies of host-pointer arguments
  sst::PlanSummary *h_plan = nullptr;  // pinned
  sst::PlanSummary *h_plan_dev = nullptr;  // h_plan's address for kernels (mapped)
  sst::PlanSummary *d_plan = nullptr;
  unsigned long long *d_err = nullptr;  // staging-rank check, read lazily
  uint64_t *d_bounds = nullptr;  // window density bounds (sst::window_bounds_table)
  unsigned long long *d_scan_epoch = nullptr;  // tags of captured scans
  sst::LeafDir dir;
  sst::TravState *trav = nullptr;  // traversal work lists and buffers
  void *h_pinned = nullptr;  // pinned staging for host-pointer calls
  size_t h_pinned_cap = 0;

  sst::DGraph view() const {
    return sst::DGraph{n, width, d_base, d_cap, d_deg, d_slots, d_lcnt, d_vals};
  }
};

namespace sst {

sst_status graph_init(sst_graph *g, uint32_t height, uint32_t width,
                      const sst_config *cfg);
void graph_release(sst_graph *g);
void plan_cache_release(sst_graph *g);
sst_status graph_clone(const sst_graph *src, sst_graph *dst);
uint64_t graph_device_bytes(const sst_graph *g);

// pairs are device pointers here; the C ABI stages host buffers
// d_w: per-pair values for a weighted graph (null: value 1)
sst_status update_batch(sst_graph *g, const uint32_t *d_pairs, uint64_t n,
                        bool insert, uint64_t *n_invalid,
                        const uint32_t *d_w = nullptr);
// nb batches: pairs[boff[i]..boff[i+1]) with ops[i] (1 insert, 0 remove),
// applied as if in order; N = boff[nb]
sst_status update_batches(sst_graph *g, const uint32_t *d_pairs,
                          const uint64_t *d_boff, const uint8_t *d_ops,
                          uint32_t nb, uint64_t N, uint64_t *n_invalid);
sst_status degree_order_map(sst_graph *g, uint32_t *d_map);
sst_status rewrite_graph(sst_graph *g, const uint32_t *d_map, sst_graph *out);
sst_status build_from_csr(sst_graph *g, const uint64_t *d_off,
                          const uint32_t *d_cols);
// d_out (membership) and d_vals (values, weighted graphs) may each be null
sst_status has_batch(sst_graph *g, const uint32_t *d_pairs, uint64_t n,
                     uint8_t *d_out, uint32_t *d_vals = nullptr);
sst_status ensure_leaf_dir(sst_graph *g);
sst_status to_csr(sst_graph *g, uint64_t *d_off, uint32_t *d_cols,
                  uint32_t *d_vals = nullptr);
sst_status neighbors(sst_graph *g, uint32_t v, uint32_t *d_out, uint64_t cap,
                     uint64_t *deg);
sst_status sample_edges(sst_graph *g, uint64_t seed, uint64_t first,
                        uint64_t count, uint32_t *d_pairs);
sst_status touch_all_sum(sst_graph *g, uint64_t *out);
sst_status repack(sst_graph *g, uint64_t extra_slots);
sst_status sync_checked(sst_graph *g);

// host staging buffer (pinned) of at least `bytes`
void *pinned(sst_graph *g, size_t bytes);
void trav_release(sst_graph *g);
// frees the traversal buffers and work lists (kept: the tuning)
void trav_trim(sst_graph *g);
uint64_t trav_device_bytes(const sst_graph *g);
// frees every buffer the graph rebuilds on demand: update scratch, task
// staging, host-call staging, captured planning graphs, the leaf directory
// and the traversal buffers
sst_status release_scratch(sst_graph *g);

}  // namespace sst

// Source-level drop-in for the reference's graph interface on this path:
// SSTGraph::SparseMatrixV<true> (include/SSTGraph/SparseMatrix.hpp) and the
// EdgeMapVertexMap entry points its drivers call (internal/test.hpp:476-618),
// implemented over the C ABI in sstgraph.h (the graph lives in GPU memory).
//
// Differences a caller sees:
//  - errors throw SSTGraph::sst_error instead of asserting or exiting;
//  - insert_batch / remove_batch leave the caller's buffer as it was (the
//    reference sorts it in place, SparseMatrix.hpp:578,664);
//  - map_neighbors / map_range call host functors on copied-out neighbour
//    lists (same order and early-exit rules, SparseMatrix.hpp:179-315);
//  - the binary CSR form (SparseMatrixV<true>) and the uint32-weighted one
//    (SparseMatrixV<true, uint32_t>, test.hpp:699-846) exist; on the
//    weighted form the batched update, relabel and CSR build are refused.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../sstgraph.h"

namespace SSTGraph {

using el_t = uint32_t;

class sst_error : public std::runtime_error {
 public:
  sst_error(sst_status s, const char *what)
      : std::runtime_error(std::string(sst_status_string(s)) + ": " + what),
        status(s) {}
  sst_status status;
};

inline void check(sst_status s) {
  if (s != SST_OK) throw sst_error(s, sst_last_error_message());
}

template <bool is_csr_ = true, typename... Ts> class SparseMatrixV {
  static_assert(is_csr_, "the device graph is stored by rows (CSR) only");
  static constexpr bool weighted = sizeof...(Ts) == 1;
  static_assert(sizeof...(Ts) == 0 ||
                    (weighted && std::is_same_v<std::tuple<Ts...>, std::tuple<uint32_t>>),
                "edge values are uint32_t (or none)");
  using edge_t = std::tuple<el_t, el_t, Ts...>;
  sst_graph *g_ = nullptr;

  static std::vector<uint32_t> flatten(const edge_t *edges, uint64_t n) {
    std::vector<uint32_t> p(2 * n);
    for (uint64_t i = 0; i < n; i++) {
      p[2 * i] = std::get<0>(edges[i]);
      p[2 * i + 1] = std::get<1>(edges[i]);
    }
    return p;
  }
  static std::vector<uint32_t> values_of(const edge_t *edges, uint64_t n) {
    std::vector<uint32_t> v(n);
    if constexpr (weighted)
      for (uint64_t i = 0; i < n; i++) v[i] = std::get<2>(edges[i]);
    return v;
  }
  static const sst_config *config() {
    static sst_config cfg = [] {
      sst_config c{};
      c.weighted = weighted ? 1u : 0u;
      return c;
    }();
    return &cfg;
  }

  std::vector<uint32_t> neighbours(uint64_t i) const {
    uint32_t d = getDegree((uint32_t)i);
    std::vector<uint32_t> out(d);
    uint64_t full = 0;
    check(sst_neighbors(g_, (uint32_t)i, out.data(), d, &full));
    return out;
  }

 public:
  SparseMatrixV(el_t height, el_t width, const sst_config *cfg = nullptr) {
    check(sst_graph_create(height, width, cfg ? cfg : config(), &g_));
  }
  explicit SparseMatrixV(sst_graph *adopt) : g_(adopt) {}
  SparseMatrixV(const SparseMatrixV &o) { check(sst_graph_clone(o.g_, &g_)); }
  SparseMatrixV(SparseMatrixV &&o) noexcept : g_(o.g_) { o.g_ = nullptr; }
  SparseMatrixV &operator=(const SparseMatrixV &o) {
    if (this != &o) {
      sst_graph *c = nullptr;
      check(sst_graph_clone(o.g_, &c));
      sst_graph_destroy(g_);
      g_ = c;
    }
    return *this;
  }
  SparseMatrixV &operator=(SparseMatrixV &&o) noexcept {
    if (this != &o) {
      sst_graph_destroy(g_);
      g_ = o.g_;
      o.g_ = nullptr;
    }
    return *this;
  }
  ~SparseMatrixV() { sst_graph_destroy(g_); }

  sst_graph *handle() const { return g_; }
  static constexpr bool is_csr() { return true; }
  static constexpr bool is_csc() { return false; }
  static constexpr bool is_binary() { return true; }

  uint32_t get_rows() const {
    uint32_t r = 0;
    check(sst_get_rows(g_, &r));
    return r;
  }
  uint32_t get_cols() const {
    uint32_t c = 0;
    check(sst_get_cols(g_, &c));
    return c;
  }
  uint32_t get_line_count() const { return get_rows(); }
  uint32_t get_line_width() const { return get_cols(); }
  size_t num_nodes() const { return get_rows(); }
  uint32_t getDegree(uint32_t node) const {
    uint32_t d = 0;
    check(sst_get_degree(g_, node, &d));
    return d;
  }
  uint64_t M() const {
    uint64_t m = 0;
    check(sst_M(g_, &m));
    return m;
  }
  uint64_t get_memory_size() const {
    uint64_t b = 0;
    check(sst_memory_size(g_, &b));
    return b;
  }

  bool has(el_t row, el_t col) const {
    int r = 0;
    check(sst_has(g_, row, col, &r));
    return r != 0;
  }
  // binary: membership; weighted: the edge's value (0 where absent)
  auto value(el_t row, el_t col) const {
    if constexpr (weighted) {
      uint32_t p[2] = {row, col}, v = 0;
      check(sst_values_batch(g_, p, 1, &v, nullptr, 0u));
      return v;
    } else {
      return has(row, col);
    }
  }
  void insert(el_t row, el_t col) { check(sst_insert(g_, row, col)); }
  void insert(std::tuple<el_t, el_t> e) { insert(std::get<0>(e), std::get<1>(e)); }
  void remove(el_t row, el_t col) { check(sst_remove(g_, row, col)); }

  void insert_batch(edge_t *edges, uint64_t n, bool semi_sorted = false) {
    std::vector<uint32_t> p = flatten(edges, n);
    if constexpr (weighted) {
      std::vector<uint32_t> v = values_of(edges, n);
      check(sst_insert_batch_weighted(g_, p.data(), v.data(), n,
                                      semi_sorted ? SST_SEMI_SORTED : 0u, nullptr));
    } else {
      check(sst_insert_batch(g_, p.data(), n, semi_sorted ? SST_SEMI_SORTED : 0u,
                             nullptr));
    }
  }
  void remove_batch(edge_t *edges, uint64_t n, bool semi_sorted = false) {
    std::vector<uint32_t> p = flatten(edges, n);
    check(sst_remove_batch(g_, p.data(), n, semi_sorted ? SST_SEMI_SORTED : 0u,
                           nullptr));
  }

  uint64_t common_neighbors(uint32_t a, uint32_t b, bool early_end = false) const {
    uint32_t p[2] = {a, b};
    uint64_t out = 0;
    check(sst_common_neighbors_batch(g_, p, 1, early_end ? 1 : 0, &out, 0));
    return out;
  }
  uint64_t touch_all_sum() const {
    uint64_t s = 0;
    check(sst_touch_all_sum(g_, &s));
    return s;
  }

  // f(src, dst) in ascending dst order; with early exit a true return stops
  template <bool no_early_exit, class F>
  void map_neighbors_impl(uint64_t i, F &&f) const {
    for (uint32_t x : neighbours(i)) {
      if constexpr (no_early_exit) {
        f(i, (uint64_t)x);
      } else {
        if (f(i, (uint64_t)x)) return;
      }
    }
  }
  template <class F>
  void map_neighbors(uint64_t i, F &f, void * /*d*/, bool /*parallel*/) const {
    map_neighbors_impl<std::remove_reference_t<F>::no_early_exit>(i, f);
  }
  template <class F>
  void map_neighbors_early_exit(uint64_t i, F &&f, void *, bool) const {
    map_neighbors_impl<false>(i, f);
  }
  template <class F>
  void map_neighbors_no_early_exit(uint64_t i, F &&f, void *, bool) const {
    map_neighbors_impl<true>(i, f);
  }
  // every row in [start, end): one copy-out of the whole graph
  template <class F>
  void map_range(F &f, uint64_t start, uint64_t end, void * /*d*/) const {
    std::vector<uint64_t> off(get_rows() + 1);
    std::vector<uint32_t> cols(M());
    check(sst_to_csr(g_, off.data(), cols.data(), 0));
    for (uint64_t i = start; i < end; i++)
      for (uint64_t k = off[i]; k < off[i + 1]; k++) f(i, (uint64_t)cols[k]);
  }

  std::vector<uint64_t> degree_order_map() const {
    std::vector<uint32_t> m(get_rows());
    check(sst_degree_order_map(g_, m.data(), 0));
    return std::vector<uint64_t>(m.begin(), m.end());
  }
  SparseMatrixV rewrite_graph(std::vector<uint64_t> new_label_map) const {
    std::vector<uint32_t> m(new_label_map.begin(), new_label_map.end());
    sst_graph *out = nullptr;
    check(sst_rewrite_graph(g_, m.data(), 0, &out));
    return SparseMatrixV(out);
  }
};

}  // namespace SSTGraph

// The algorithm entry points the reference drivers call
// (internal/test.hpp:476-618); arrays are malloc'd, the caller frees them.
namespace EdgeMapVertexMap {

template <class G> int32_t *BFS(const G &g, uint32_t src) {
  int32_t *out = static_cast<int32_t *>(std::malloc(g.num_nodes() * sizeof(int32_t)));
  SSTGraph::check(sst_bfs(g.handle(), src, out, nullptr, 0));
  return out;
}
template <class T, class G> T *PR_S(const G &g, long iters) {
  static_assert(std::is_same_v<T, double>, "PageRank is computed in FP64");
  double *out = static_cast<double *>(std::malloc(g.num_nodes() * sizeof(double)));
  SSTGraph::check(sst_pagerank(g.handle(), (uint32_t)iters, 0.85, out, 0));
  return out;
}
template <class G> double *BC(const G &g, uint32_t src) {
  double *out = static_cast<double *>(std::malloc(g.num_nodes() * sizeof(double)));
  SSTGraph::check(sst_bc(g.handle(), src, out, 0));
  return out;
}
template <class G> int32_t *BF(const G &g, uint32_t src) {
  int32_t *out = static_cast<int32_t *>(std::malloc(g.num_nodes() * sizeof(int32_t)));
  SSTGraph::check(sst_bf(g.handle(), src, out, 0));
  return out;
}
template <class G> uint32_t *CC(const G &g) {
  uint32_t *out = static_cast<uint32_t *>(std::malloc(g.num_nodes() * sizeof(uint32_t)));
  SSTGraph::check(sst_cc(g.handle(), out, 0));
  return out;
}
template <class G> uint64_t TC(const G &g) {
  uint64_t t = 0;
  SSTGraph::check(sst_tc(g.handle(), &t, nullptr, 0));
  return t;
}
template <class G> uint64_t TouchAll(const G &g) {
  uint64_t s = 0;
  SSTGraph::check(sst_touch_all(g.handle(), &s));
  return s;
}

}  // namespace EdgeMapVertexMap

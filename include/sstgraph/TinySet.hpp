// Source-level drop-in for the reference's binary set type,
// SSTGraph::TinySetV<> (include/SSTGraph/TinySet.hpp:27-73): one sorted set
// of uint32 elements in [0, max_el), kept on the GPU as the single row of a
// device graph that keeps (0, 0) (sst_config.keep_self_loops), over the C ABI
// in sstgraph.h.
//
// Differences a caller sees:
//  - errors throw SSTGraph::sst_error (an element >= max_el among them);
//  - map calls the host functor on a copied-out element list, in ascending
//    order, stopping on a true return unless no_early_exit
//    (TinySet_small.hpp:303-319);
//  - value-carrying sets (TinySetV<Ts...> with Ts non-empty) do not exist.
#pragma once

#include <cstdint>
#include <tuple>
#include <vector>

#include "SparseMatrix.hpp"

namespace SSTGraph {

template <typename... Ts> class TinySetV {
  static_assert(sizeof...(Ts) == 0, "only the binary (key-only) set exists");
  sst_graph *g_ = nullptr;
  uint32_t max_el_ = 1;

  static sst_graph *make(uint32_t max_el) {
    sst_config cfg{};
    cfg.keep_self_loops = 1;
    sst_graph *g = nullptr;
    check(sst_graph_create(1, max_el ? max_el : 1, &cfg, &g));
    return g;
  }
  void in_range(el_t e) const {
    if (e >= max_el_)
      throw sst_error(SST_EINVAL, "element out of range for this set");
  }

 public:
  explicit TinySetV(uint32_t max_el) : g_(make(max_el)), max_el_(max_el ? max_el : 1) {}
  TinySetV(const TinySetV &o) : max_el_(o.max_el_) { check(sst_graph_clone(o.g_, &g_)); }
  TinySetV(TinySetV &&o) noexcept : g_(o.g_), max_el_(o.max_el_) { o.g_ = nullptr; }
  TinySetV &operator=(const TinySetV &o) {
    if (this != &o) {
      sst_graph *c = nullptr;
      check(sst_graph_clone(o.g_, &c));
      sst_graph_destroy(g_);
      g_ = c;
      max_el_ = o.max_el_;
    }
    return *this;
  }
  TinySetV &operator=(TinySetV &&o) noexcept {
    if (this != &o) {
      sst_graph_destroy(g_);
      g_ = o.g_;
      max_el_ = o.max_el_;
      o.g_ = nullptr;
    }
    return *this;
  }
  ~TinySetV() { sst_graph_destroy(g_); }

  bool has(el_t e) const {
    if (e >= max_el_) return false;
    int r = 0;
    check(sst_has(g_, 0, e, &r));
    return r != 0;
  }
  bool value(el_t e) const { return has(e); }
  void insert(el_t e) {
    in_range(e);
    check(sst_insert(g_, 0, e));
  }
  void insert(std::tuple<el_t> e) { insert(std::get<0>(e)); }
  void remove(el_t e) {
    if (e < max_el_) check(sst_remove(g_, 0, e));
  }
  void insert_batch(const el_t *els, uint64_t n) {
    std::vector<uint32_t> p(2 * n);
    for (uint64_t i = 0; i < n; i++) {
      in_range(els[i]);
      p[2 * i] = 0;
      p[2 * i + 1] = els[i];
    }
    check(sst_insert_batch(g_, p.data(), n, 0u, nullptr));
  }
  void insert_batch(const std::tuple<el_t> *els, uint64_t n) {
    std::vector<el_t> e(n);
    for (uint64_t i = 0; i < n; i++) e[i] = std::get<0>(els[i]);
    insert_batch(e.data(), n);
  }
  uint64_t get_n() const {
    uint64_t m = 0;
    check(sst_M(g_, &m));
    return m;
  }
  uint64_t get_size() const {
    uint64_t b = 0;
    check(sst_memory_size(g_, &b));
    return b;
  }
  std::vector<el_t> elements() const {
    uint32_t d = 0;
    check(sst_get_degree(g_, 0, &d));
    std::vector<el_t> out(d);
    uint64_t full = 0;
    check(sst_neighbors(g_, 0, out.data(), d, &full));
    return out;
  }
  // f(element) in ascending order; with early exit a true return stops
  template <bool no_early_exit, class F> void map(F f, bool /*parallel*/ = false) const {
    for (el_t x : elements()) {
      if constexpr (no_early_exit) {
        f(x);
      } else {
        if (f(x)) return;
      }
    }
  }
  template <bool no_early_exit, class F> void parallel_map(F f) const {
    map<no_early_exit>(f);
  }
};

}  // namespace SSTGraph

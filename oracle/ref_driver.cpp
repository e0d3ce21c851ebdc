// C-ABI driver over the reference's own storage code (SparseMatrixV<true>,
// TinySetV, rMat, create_random_data, the .mtx loader), compiled from the
// reference headers where they lie plus the stand-in headers in shim/.
//
// Test infrastructure only: it pins the oracle restatement (sst_oracle.c) and
// generates the golden fixtures under tests/golden/.  Nothing in the product
// links it.
//
// Reference interfaces driven here:
//   SparseMatrixV(el_t,el_t)              include/SSTGraph/SparseMatrix.hpp:73
//   insert_batch / remove_batch           include/SSTGraph/SparseMatrix.hpp:556,645
//   insert / remove / has                 include/SSTGraph/SparseMatrix.hpp:527,537,721
//   getDegree / M / common_neighbors      include/SSTGraph/SparseMatrix.hpp:57,518,61
//   map_neighbors_no_early_exit           include/SSTGraph/SparseMatrix.hpp:243
//   touch_all_sum                         include/SSTGraph/SparseMatrix.hpp:436
//   SparseMatrixV<true, uint32_t>         include/SSTGraph/SparseMatrix.hpp:167,179-216,727
//   TinySetV                              include/SSTGraph/TinySet.hpp:8-73
//   TinySetV_small get_thresholds, get_b  include/SSTGraph/TinySet_small.hpp:129-135,227-263
//   rMat / random_aspen / hash64 / hash32 include/SSTGraph/internal/rmat_util.h:29-131
//   create_random_data                    include/SSTGraph/internal/helpers.hpp:752
//   get_edges_from_file_mtx               include/SSTGraph/internal/helpers.hpp:379
#include <cstdint>
#include <functional>
#include <cstdlib>
#include <tuple>
#include <vector>

#include "SSTGraph/SparseMatrix.hpp"
#include "SSTGraph/TinySet.hpp"
#include "SSTGraph/internal/helpers.hpp"
#include "SSTGraph/internal/rmat_util.h"

using namespace SSTGraph;
using Graph = SparseMatrixV<true>;

extern "C" {

void *ref_graph_new(uint32_t n) { return new Graph(n, n); }
void ref_graph_free(void *g) { delete static_cast<Graph *>(g); }

static std::vector<std::tuple<el_t, el_t>> to_tuples(const uint32_t *pairs,
                                                     uint64_t b) {
  std::vector<std::tuple<el_t, el_t>> es(b);
  for (uint64_t i = 0; i < b; i++) es[i] = {pairs[2 * i], pairs[2 * i + 1]};
  return es;
}

// insert_batch sorts the caller's buffer in place; a copy keeps the caller's
// pairs untouched
void ref_insert_batch(void *g, const uint32_t *pairs, uint64_t b) {
  auto es = to_tuples(pairs, b);
  static_cast<Graph *>(g)->insert_batch(es.data(), b);
}
void ref_remove_batch(void *g, const uint32_t *pairs, uint64_t b) {
  auto es = to_tuples(pairs, b);
  static_cast<Graph *>(g)->remove_batch(es.data(), b);
}
void ref_insert(void *g, uint32_t r, uint32_t c) {
  static_cast<Graph *>(g)->insert(r, c);
}
void ref_remove(void *g, uint32_t r, uint32_t c) {
  static_cast<Graph *>(g)->remove(r, c);
}
int ref_has(void *g, uint32_t r, uint32_t c) {
  return static_cast<Graph *>(g)->has(r, c) ? 1 : 0;
}
uint32_t ref_degree(void *g, uint32_t v) {
  return static_cast<Graph *>(g)->getDegree(v);
}
uint64_t ref_M(void *g) { return static_cast<Graph *>(g)->M(); }
uint64_t ref_common_neighbors(void *g, uint32_t a, uint32_t b, int early) {
  return static_cast<Graph *>(g)->common_neighbors(a, b, early != 0);
}
uint64_t ref_touch_all_sum(void *g) {
  return static_cast<Graph *>(g)->touch_all_sum();
}

struct collect_f {
  static constexpr bool no_early_exit = true;
  std::vector<uint32_t> *out;
  bool operator()(uint64_t, uint64_t dst) {
    out->push_back(static_cast<uint32_t>(dst));
    return false;
  }
};

// neighbour sets in map order as a CSR: offsets[n+1], cols[M]
void ref_to_csr(void *gp, uint64_t *offsets, uint32_t *cols) {
  Graph *g = static_cast<Graph *>(gp);
  uint64_t pos = 0;
  std::vector<uint32_t> tmp;
  for (uint64_t v = 0; v < g->num_nodes(); v++) {
    offsets[v] = pos;
    tmp.clear();
    collect_f f{&tmp};
    g->map_neighbors(v, f, nullptr, false);
    for (uint32_t x : tmp) cols[pos++] = x;
  }
  offsets[g->num_nodes()] = pos;
}

// degree_order_map / rewrite_graph  SparseMatrix.hpp:737-766
void ref_degree_order_map(void *gp, uint32_t *out) {
  Graph *g = static_cast<Graph *>(gp);
  std::vector<uint64_t> m = g->degree_order_map();
  for (size_t i = 0; i < m.size(); i++) out[i] = static_cast<uint32_t>(m[i]);
}
void *ref_rewrite_graph(void *gp, const uint32_t *map) {
  Graph *g = static_cast<Graph *>(gp);
  std::vector<uint64_t> m(map, map + g->num_nodes());
  return new Graph(g->rewrite_graph(m));
}

// ---- weighted graph: SparseMatrixV<true, uint32_t>  (internal/test.hpp:714)
// insert_batch takes (row, col, value) tuples (SparseMatrix.hpp:167,558);
// a present edge takes the new value (PMA.hpp:1137-1145)
using WGraph = SparseMatrixV<true, uint32_t>;
void *ref_wgraph_new(uint32_t n) { return new WGraph(n, n); }
void ref_wgraph_free(void *g) { delete static_cast<WGraph *>(g); }
void ref_winsert_batch(void *g, const uint32_t *pairs, const uint32_t *vals,
                       uint64_t b) {
  std::vector<std::tuple<el_t, el_t, uint32_t>> es(b);
  for (uint64_t i = 0; i < b; i++) es[i] = {pairs[2 * i], pairs[2 * i + 1], vals[i]};
  static_cast<WGraph *>(g)->insert_batch(es.data(), b);
}
// The weighted remove_batch does not compile in the reference (its sort
// comparator takes the (row, col, value) element while remove_batch passes
// (row, col) pairs, SparseMatrix.hpp:489-494,647), so removes go through the
// single-edge remove (SparseMatrix.hpp:537) one pair at a time.
void ref_wremove_each(void *g, const uint32_t *pairs, uint64_t b) {
  for (uint64_t i = 0; i < b; i++)
    static_cast<WGraph *>(g)->remove(pairs[2 * i], pairs[2 * i + 1]);
}
uint64_t ref_wM(void *g) { return static_cast<WGraph *>(g)->M(); }
// value(row, col)  SparseMatrix.hpp:727 (0 where absent)
uint32_t ref_wvalue(void *g, uint32_t r, uint32_t c) {
  return std::get<0>(static_cast<WGraph *>(g)->value(r, c));
}

struct collect_wf {
  static constexpr bool no_early_exit = true;
  std::vector<uint32_t> *out, *vout;
  bool operator()(uint64_t, uint64_t dst, uint32_t val) {
    out->push_back(static_cast<uint32_t>(dst));
    vout->push_back(val);
    return false;
  }
};

// neighbour sets with their values in map order: offsets[n+1], cols[M],
// vals[M]  (the value-carrying map_neighbors, SparseMatrix.hpp:179-216)
void ref_wto_csr(void *gp, uint64_t *offsets, uint32_t *cols, uint32_t *vals) {
  WGraph *g = static_cast<WGraph *>(gp);
  uint64_t pos = 0;
  std::vector<uint32_t> tmp, vtmp;
  for (uint64_t v = 0; v < g->num_nodes(); v++) {
    offsets[v] = pos;
    tmp.clear();
    vtmp.clear();
    collect_wf f{&tmp, &vtmp};
    g->map_neighbors(v, f, nullptr, false);
    for (size_t k = 0; k < tmp.size(); k++) {
      cols[pos] = tmp[k];
      vals[pos] = vtmp[k];
      pos++;
    }
  }
  offsets[g->num_nodes()] = pos;
}

// ---- standalone set (TinySetV) ----
using Set = TinySetV<>;
void *ref_set_new(uint32_t max_el) { return new Set(max_el); }
void ref_set_free(void *s) { delete static_cast<Set *>(s); }
void ref_set_insert(void *s, uint32_t e) {
  static_cast<Set *>(s)->insert(std::tuple<el_t>(e));
}
void ref_set_remove(void *s, uint32_t e) { static_cast<Set *>(s)->remove(e); }
int ref_set_has(void *s, uint32_t e) {
  return static_cast<Set *>(s)->has(e) ? 1 : 0;
}
uint64_t ref_set_n(void *s) { return static_cast<Set *>(s)->get_n(); }
uint64_t ref_set_to_array(void *s, uint32_t *out) {
  uint64_t k = 0;
  static_cast<Set *>(s)->map<true>([&](el_t e) { out[k++] = e; });
  return k;
}

// ---- byte-width rows: TinySetV_small's key width ----
// get_thresholds  TinySet_small.hpp:227-263
void ref_tinyset_thresholds(uint64_t max_el, uint32_t *out) {
  auto d = TinySetV_small<>::get_thresholds(max_el);
  out[0] = d.thresh_24;
  out[1] = d.thresh_16;
  out[2] = d.thresh_8;
}
// get_b() of a TinySetV_small over max_el after inserting els[0..k)
// (TinySet_small.hpp:129-130; the width follows the count, :204-214)
uint32_t ref_tinyset_width(uint64_t max_el, const uint32_t *els, uint64_t k) {
  auto d = TinySetV_small<>::get_thresholds(max_el);
  TinySetV_small<> ts;
  for (uint64_t i = 0; i < k; i++) ts.insert(std::tuple<el_t>(els[i]), d);
  uint32_t b = ts.get_b();
  ts.destroy(d);
  return b;
}

// ---- generators ----
uint64_t ref_hash64(uint64_t u) { return hash64(u); }
uint32_t ref_hash32(uint32_t u) { return hash32(u); }

// the batch stream of the reference's update benchmark
// (internal/test.hpp:636-654): rMat<uint32_t>(nn, random_aspen().ith_rand(0),
// a, b, c), edge i = rmat(i)
void ref_rmat_stream(uint32_t nn, double a, double b, double c, uint64_t count,
                     uint32_t *out) {
  auto r = random_aspen();
  auto rmat = rMat<uint32_t>(nn, r.ith_rand(0), a, b, c);
  for (uint64_t i = 0; i < count; i++) {
    auto e = rmat(static_cast<uint32_t>(i));
    out[2 * i] = e.first;
    out[2 * i + 1] = e.second;
  }
}

// create_random_data<uint32_t>(n, max, seed): the known-answer inputs of
// PMA_test.cpp / Tinyset_test.cpp
void ref_random_data(uint64_t n, uint32_t max_val, uint32_t seed,
                     uint32_t *out) {
  auto v = create_random_data<uint32_t>(n, max_val, seed);
  for (uint64_t i = 0; i < n; i++) out[i] = v[i];
}

// the reference .mtx loader (1-indexed, always symmetrised)
uint64_t ref_load_mtx(const char *path, uint32_t *rows, uint32_t **pairs_out) {
  uint64_t m = 0;
  el_t r = 0, c = 0;
  auto *edges = get_edges_from_file_mtx<bool>(path, &m, &r, &c, false);
  uint32_t *out = static_cast<uint32_t *>(std::malloc(2 * m * sizeof(uint32_t)));
  for (uint64_t i = 0; i < m; i++) {
    out[2 * i] = std::get<0>(edges[i]);
    out[2 * i + 1] = std::get<1>(edges[i]);
  }
  std::free(edges);
  *rows = r;
  *pairs_out = out;
  return m;
}
void ref_free(void *p) { std::free(p); }

} // extern "C"

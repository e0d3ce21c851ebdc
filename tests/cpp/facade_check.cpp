// Drives the C++ drop-in header the way the reference's drivers drive
// SparseMatrixV<true> (internal/test.hpp): batch inserts and removes, then
// the EdgeMapVertexMap entry points, checked against a std::set model.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <set>
#include <tuple>
#include <vector>

#include "sstgraph/SparseMatrix.hpp"
#include "sstgraph/TinySet.hpp"

using namespace SSTGraph;

// the reference's TinySet tests in miniature (Tinyset_test.cpp: insert
// random elements below max, check membership; remove, check absence)
// the weighted form: values, overwrite on re-insert, Bellman-Ford on a
// small chain with a shortcut
static int weighted_check() {
  SparseMatrixV<true, uint32_t> w(6, 6);
  std::vector<std::tuple<el_t, el_t, uint32_t>> es = {
      {0, 1, 4}, {1, 2, 3}, {2, 3, 2}, {0, 3, 20}, {3, 4, 1}, {0, 1, 5}};
  w.insert_batch(es.data(), es.size());
  if (w.value(0, 1) != 5 || w.value(0, 3) != 20 || w.value(4, 3) != 0) {
    std::printf("weighted values differ\n");
    return 1;
  }
  std::vector<std::tuple<el_t, el_t, uint32_t>> upd = {{0, 3, 7}};
  w.insert_batch(upd.data(), upd.size());
  int32_t *d = EdgeMapVertexMap::BF(w, 0);
  // 0->3 costs 7 directly (was 20), 0->1->2->3 costs 10; 0->3->4 costs 8
  const int32_t exp[6] = {0, 5, 8, 7, 8, 0x7FFFFFFF};
  for (int v = 0; v < 6; v++)
    if (d[v] != exp[v]) {
      std::printf("BF[%d] = %d, expected %d\n", v, d[v], exp[v]);
      std::free(d);
      return 1;
    }
  std::free(d);
  return 0;
}

static int tinyset_check() {
  const uint32_t max = 5000;
  TinySetV<> ts(max);
  std::mt19937 rng(7);
  std::set<uint32_t> model;
  for (int i = 0; i < 3000; i++) {
    uint32_t e = rng() % max;
    ts.insert(e);
    model.insert(e);
  }
  std::vector<uint32_t> batch;
  for (int i = 0; i < 2000; i++) batch.push_back(rng() % max);
  ts.insert_batch(batch.data(), batch.size());
  model.insert(batch.begin(), batch.end());
  ts.insert(0);  // element 0 of row 0 stays (the set keeps (0, 0))
  model.insert(0);
  for (uint32_t e = 0; e < max; e++)
    if (ts.has(e) != (model.count(e) == 1)) {
      std::printf("tinyset has(%u) differs\n", e);
      return 1;
    }
  for (int i = 0; i < 1500; i++) {
    uint32_t e = rng() % max;
    ts.remove(e);
    model.erase(e);
  }
  if (ts.get_n() != model.size()) {
    std::printf("tinyset n %llu != %zu\n", (unsigned long long)ts.get_n(), model.size());
    return 1;
  }
  std::vector<uint32_t> seen;
  ts.map<true>([&](uint32_t e) { seen.push_back(e); });
  if (seen != std::vector<uint32_t>(model.begin(), model.end())) {
    std::printf("tinyset map order differs\n");
    return 1;
  }
  bool threw = false;
  try {
    ts.insert(max);
  } catch (const sst_error &) {
    threw = true;
  }
  return threw ? 0 : 1;
}

struct collect {
  static constexpr bool no_early_exit = true;
  std::vector<uint32_t> *out;
  bool operator()(uint64_t, uint64_t d) {
    out->push_back((uint32_t)d);
    return false;
  }
};

int main() {
  const uint32_t n = 2000;
  std::mt19937 rng(7);
  std::uniform_int_distribution<uint32_t> pick(0, n - 1);
  std::set<std::pair<uint32_t, uint32_t>> model;
  SparseMatrixV<true> g(n, n);
  for (int round = 0; round < 6; round++) {
    std::vector<std::tuple<el_t, el_t>> es(5000);
    for (auto &e : es) {
      uint32_t a = pick(rng) % (round + 3), b = pick(rng);
      e = {a, b};
    }
    if (round % 3 == 2) {
      g.remove_batch(es.data(), es.size());
      for (auto &e : es) model.erase({std::get<0>(e), std::get<1>(e)});
    } else {
      g.insert_batch(es.data(), es.size());
      for (auto &e : es)
        if (std::get<0>(e) != std::get<1>(e)) model.insert({std::get<0>(e), std::get<1>(e)});
    }
  }
  if (g.M() != model.size()) {
    std::printf("M %llu != %zu\n", (unsigned long long)g.M(), model.size());
    return 1;
  }
  for (uint32_t v = 0; v < 8; v++) {
    std::vector<uint32_t> got;
    collect f{&got};
    g.map_neighbors(v, f, nullptr, false);
    std::vector<uint32_t> exp;
    for (auto it = model.lower_bound({v, 0}); it != model.end() && it->first == v; ++it)
      exp.push_back(it->second);
    if (got != exp || g.getDegree(v) != exp.size()) {
      std::printf("row %u differs\n", v);
      return 1;
    }
  }
  if (!g.has(model.begin()->first, model.begin()->second)) return 1;
  SparseMatrixV<true> copy = g;  // deep copy on the device
  int32_t *par = EdgeMapVertexMap::BFS(copy, 0);
  double *pr = EdgeMapVertexMap::PR_S<double>(copy, 10);
  uint32_t *cc = EdgeMapVertexMap::CC(copy);
  uint64_t tc = EdgeMapVertexMap::TC(copy);
  if (par[0] != 0 || pr[0] <= 0.0) return 1;
  std::free(par);
  std::free(pr);
  std::free(cc);
  if (tinyset_check()) return 1;
  if (weighted_check()) return 1;
  std::printf("facade ok: M=%llu tc=%llu\n", (unsigned long long)g.M(),
              (unsigned long long)tc);
  return 0;
}

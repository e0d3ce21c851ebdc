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

using namespace SSTGraph;

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
  std::printf("facade ok: M=%llu tc=%llu\n", (unsigned long long)g.M(),
              (unsigned long long)tc);
  return 0;
}

// Stand-in for the absent ParallelTools reducers (per-thread slots combined on
// get()).  Written for this project from the reference call sites.
#pragma once
#include <cstdint>
#include <vector>
#include "ParallelTools/parallel.h"

namespace ParallelTools {

template <typename T> class Reducer_sum {
  struct alignas(64) slot { T v{}; };
  std::vector<slot> slots;

public:
  Reducer_sum() : slots(omp_get_max_threads()) {}
  explicit Reducer_sum(T init) : slots(omp_get_max_threads()) { slots[0].v = init; }
  void add(T x) { slots[omp_get_thread_num()].v += x; }
  void inc() { slots[omp_get_thread_num()].v += 1; }
  T get() const {
    T r{};
    for (const auto &s : slots) r += s.v;
    return r;
  }
};

template <typename T> class Reducer {
  struct alignas(64) slot { T v{}; };
  std::vector<slot> slots;

public:
  Reducer() : slots(omp_get_max_threads()) {}
  void update(const T &x) { slots[omp_get_thread_num()].v.update(x); }
  T get() const {
    T r{};
    for (const auto &s : slots) r.update(s.v);
    return r;
  }
};

} // namespace ParallelTools

// Stand-in for the absent ParallelTools submodule, written for this project
// from the call sites in the reference headers (parallel_for over an index
// range, getWorkers, sort).  Backed by OpenMP.  Test infrastructure only.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <type_traits>
#include <omp.h>

namespace ParallelTools {

inline int getWorkers() { return omp_get_max_threads(); }
inline int getWorkerNum() { return omp_get_thread_num(); }

template <typename A, typename B, typename F>
inline void parallel_for(A start, B end, F &&f) {
  using I = std::common_type_t<A, B>;
  const int64_t s = static_cast<int64_t>(start);
  const int64_t e = static_cast<int64_t>(static_cast<I>(end));
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = s; i < e; i++) {
    f(static_cast<I>(i));
  }
}

template <typename A, typename B, typename F>
inline void parallel_for(A start, B end, F &&f, size_t /*grain*/) {
  parallel_for(start, end, std::forward<F>(f));
}

template <typename It, typename Cmp> inline void sort(It b, It e, Cmp cmp) {
  std::sort(b, e, cmp);
}
template <typename It> inline void sort(It b, It e) { std::sort(b, e); }

} // namespace ParallelTools

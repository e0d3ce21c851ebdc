// Stand-in for the one parlaylib routine the reference graph uses
// (integer_sort_inplace keyed on the row id).  A stable sort gives the same
// row order; order inside a row never reaches the stored sets.
#pragma once
#include <algorithm>
#include <vector>

namespace parlay {
template <typename Vec, typename Key>
inline void integer_sort_inplace(Vec &v, Key &&key) {
  std::stable_sort(v.begin(), v.end(), [&](const auto &a, const auto &b) {
    return key(a) < key(b);
  });
}
} // namespace parlay

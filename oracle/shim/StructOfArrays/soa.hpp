// Stand-in for the absent StructOfArrays submodule, written for this project
// from the calls PMA.hpp makes on SOA<key> (the binary, key-only layout the
// graph path instantiates): a packed array of one element type, accessed as
// tuples of references.  Multi-field layouts are not provided.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <tuple>

template <typename... Ts> class SOA;

template <typename T> class SOA<T> {
  void *data_ = nullptr;
  size_t n_ = 0;

  static T *at(const void *base, size_t i) {
    return reinterpret_cast<T *>(const_cast<uint8_t *>(
               static_cast<const uint8_t *>(base))) + i;
  }

public:
  static constexpr size_t get_size_static(size_t n) { return n * sizeof(T); }

  template <size_t... Is>
  static std::tuple<T &> get_static(const void *base, size_t /*n*/, size_t i) {
    return std::tuple<T &>(*at(base, i));
  }

  static T get_element_static(const void *base, size_t /*n*/, size_t i) {
    return *at(base, i);
  }

  // new buffer of new_n elements: the first min(old_n, new_n) copied, the
  // rest zero (a zero key is the PMA's empty slot)
  static void *resize_static(const void *base, size_t old_n, size_t new_n) {
    void *p = std::malloc(get_size_static(new_n));
    size_t keep = old_n < new_n ? old_n : new_n;
    std::memcpy(p, base, get_size_static(keep));
    std::memset(static_cast<uint8_t *>(p) + get_size_static(keep), 0,
                get_size_static(new_n - keep));
    return p;
  }

  template <class F>
  static void map_range_static(const void *base, size_t n, F &&f,
                               size_t start = 0, size_t end = SIZE_MAX) {
    if (end > n) end = n;
    for (size_t i = start; i < end; i++) f(*at(base, i));
  }

  template <class F>
  static void map_range_with_index_static(const void *base, size_t n, F &&f,
                                          size_t start = 0,
                                          size_t end = SIZE_MAX) {
    if (end > n) end = n;
    for (size_t i = start; i < end; i++) f(i, *at(base, i));
  }

  static void print_type_details() {
    std::cout << "SOA<" << sizeof(T) << " bytes>\n";
  }

  explicit SOA(size_t n) : data_(std::calloc(n ? n : 1, sizeof(T))), n_(n) {}
  SOA(const SOA &) = delete;
  SOA &operator=(const SOA &) = delete;
  ~SOA() { std::free(data_); }
  std::tuple<T &> get(size_t i) { return std::tuple<T &>(*at(data_, i)); }
};

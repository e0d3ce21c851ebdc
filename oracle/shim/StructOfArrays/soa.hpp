// Stand-in for the absent StructOfArrays submodule, written for this project
// from the calls PMA.hpp makes on SOA<key> (the binary, key-only layout of
// the unweighted graph) and SOA<key, value...> (weighted graphs): a packed
// struct of arrays -- n keys, then n of each value type -- accessed as
// tuples of references.  Also leftshift_tuple, which PMA.hpp and
// TinySet_small.hpp call (a tuple without its first element).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <tuple>
#include <type_traits>
#include <utility>

template <typename... Ts> class SOA;

namespace soa_shim {
template <typename Tup, size_t... Is>
auto drop_first(const Tup &t, std::index_sequence<Is...>) {
  return std::make_tuple(std::get<Is + 1>(t)...);
}
}  // namespace soa_shim

// (a, b, c...) -> (b, c...) as values
template <typename... Ts>
auto leftshift_tuple(const std::tuple<Ts...> &t) {
  static_assert(sizeof...(Ts) >= 1, "leftshift of an empty tuple");
  return soa_shim::drop_first(t, std::make_index_sequence<sizeof...(Ts) - 1>{});
}

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

// Two or more fields: field I of element i lives at
// base + n * (sizeof(T0) + ... + sizeof(T_{I-1})) + i * sizeof(T_I).
template <typename T0, typename T1, typename... Rest> class SOA<T0, T1, Rest...> {
  using Tup = std::tuple<T0, T1, Rest...>;
  static constexpr size_t NF = 2 + sizeof...(Rest);
  template <size_t I> using F = std::tuple_element_t<I, Tup>;
  void *data_ = nullptr;
  size_t n_ = 0;

  template <size_t I> static constexpr size_t before() {
    if constexpr (I == 0) {
      return 0;
    } else {
      return before<I - 1>() + sizeof(F<I - 1>);
    }
  }
  template <size_t I> static F<I> *field(const void *base, size_t n) {
    return reinterpret_cast<F<I> *>(const_cast<uint8_t *>(
        static_cast<const uint8_t *>(base) + n * before<I>()));
  }
  template <size_t... Is>
  static std::tuple<F<Is> &...> refs(const void *base, size_t n, size_t i,
                                     std::index_sequence<Is...>) {
    return std::tuple<F<Is> &...>(field<Is>(base, n)[i]...);
  }
  template <class Fn, size_t... Is>
  static void call(const void *base, size_t n, size_t i, Fn &f,
                   std::index_sequence<Is...>) {
    f(field<Is>(base, n)[i]...);
  }
  template <class Fn, size_t... Is>
  static void call_i(const void *base, size_t n, size_t i, Fn &f,
                     std::index_sequence<Is...>) {
    f(i, field<Is>(base, n)[i]...);
  }
  template <size_t... Is>
  static void copy_fields(const void *src, size_t sn, void *dst, size_t dn,
                          size_t keep, std::index_sequence<Is...>) {
    (std::memcpy(field<Is>(dst, dn), field<Is>(src, sn), keep * sizeof(F<Is>)), ...);
  }

public:
  static constexpr size_t get_size_static(size_t n) { return n * before<NF>(); }

  template <size_t... Is>
  static auto get_static(const void *base, size_t n, size_t i) {
    if constexpr (sizeof...(Is) == 0)
      return refs(base, n, i, std::make_index_sequence<NF>{});
    else
      return std::tuple<F<Is> &...>(field<Is>(base, n)[i]...);
  }

  // the key of element i
  static T0 get_element_static(const void *base, size_t n, size_t i) {
    return field<0>(base, n)[i];
  }

  // new buffer of new_n elements: each field's first min(old_n, new_n)
  // entries copied, the rest zero (a zero key is the PMA's empty slot)
  static void *resize_static(const void *base, size_t old_n, size_t new_n) {
    void *p = std::calloc(new_n ? new_n : 1, before<NF>());
    const size_t keep = old_n < new_n ? old_n : new_n;
    copy_fields(base, old_n, p, new_n, keep, std::make_index_sequence<NF>{});
    return p;
  }

  template <class Fn>
  static void map_range_static(const void *base, size_t n, Fn &&f,
                               size_t start = 0, size_t end = SIZE_MAX) {
    if (end > n) end = n;
    for (size_t i = start; i < end; i++)
      call(base, n, i, f, std::make_index_sequence<NF>{});
  }

  template <class Fn>
  static void map_range_with_index_static(const void *base, size_t n, Fn &&f,
                                          size_t start = 0,
                                          size_t end = SIZE_MAX) {
    if (end > n) end = n;
    for (size_t i = start; i < end; i++)
      call_i(base, n, i, f, std::make_index_sequence<NF>{});
  }

  static void print_type_details() {
    std::cout << "SOA<" << before<NF>() << " bytes per element>\n";
  }

  explicit SOA(size_t n) : data_(std::calloc(n ? n : 1, before<NF>())), n_(n) {}
  SOA(const SOA &) = delete;
  SOA &operator=(const SOA &) = delete;
  ~SOA() { std::free(data_); }
  auto get(size_t i) { return refs(data_, n_, i, std::make_index_sequence<NF>{}); }
};

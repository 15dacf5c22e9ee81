// Minimal host-only (OpenMP) implementation of the subset of the Kokkos 4.x API
// that the reference library's synchrotron path uses.  It exists so that the
// reference's own, unmodified C++ sources compile on this machine (Kokkos itself
// is not installed and cannot be fetched) and serve as a CPU pin for the oracle.
//
// Semantics mirrored from the Kokkos API (not from its source):
//   * View<T*> / View<T*[N]>: reference-counted, zero-initialised, LayoutRight
//     (the Kokkos default for host memory spaces); subviews alias the parent.
//   * create_mirror_view of a host view returns the view itself.
//   * parallel_for over RangePolicy / MDRangePolicy<Rank<2|3>> runs an OpenMP
//     static schedule; parallel_reduce with MinMax<T> starts from (+max, lowest).
//   * math functions follow Kokkos' overload set: float in -> float out,
//     double in -> double out, mixed/integral arguments promote to double.
//
// This header is test infrastructure for the oracle only.
#pragma once

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]

namespace Kokkos {

  namespace shim_detail {
    inline bool& initialized_flag() {
      static bool flag = false;
      return flag;
    }

    template <class D>
    struct data_traits;

    template <class T>
    struct data_traits<T*> {
      using value_type                 = T;
      static constexpr int         rank = 1;
      static constexpr std::size_t N1   = 1;
    };

    template <class T, std::size_t N>
    struct data_traits<T* [N]> {
      using value_type                 = T;
      static constexpr int         rank = 2;
      static constexpr std::size_t N1   = N;
    };
  } // namespace shim_detail

  inline void initialize() {
    shim_detail::initialized_flag() = true;
  }

  inline void finalize() {
    shim_detail::initialized_flag() = false;
  }

  inline bool is_initialized() {
    return shim_detail::initialized_flag();
  }

  inline void fence() {}

  struct ALL_t {};
  constexpr ALL_t ALL {};

  // A strided view of rank 1 or 2.  Element (i, j) lives at
  // ptr[i * stride0 + j * stride1].
  template <class DataType>
  class View {
  public:
    using traits     = shim_detail::data_traits<DataType>;
    using value_type = typename traits::value_type;

    View() = default;

    View(const std::string& label, std::size_t n0) : m_label { label } {
      m_ext[0] = n0;
      m_ext[1] = traits::N1;
      const std::size_t total = n0 * traits::N1;
      m_owner = std::shared_ptr<value_type[]>(new value_type[total > 0 ? total : 1]());
      m_ptr    = m_owner.get();
      m_str[0] = traits::N1;
      m_str[1] = 1;
    }

    View(const char* label, std::size_t n0) : View(std::string(label), n0) {}

    static constexpr auto rank() -> int {
      return traits::rank;
    }

    auto extent(int d) const -> std::size_t {
      return d < traits::rank ? m_ext[d] : 1;
    }

    auto extent_int(int d) const -> int {
      return static_cast<int>(extent(d));
    }

    auto size() const -> std::size_t {
      return traits::rank == 1 ? m_ext[0] : m_ext[0] * m_ext[1];
    }

    auto span() const -> std::size_t {
      return size();
    }

    auto data() const -> value_type* {
      return m_ptr;
    }

    auto label() const -> std::string {
      return m_label;
    }

    auto stride(int d) const -> std::size_t {
      return m_str[d];
    }

    auto operator()(std::size_t i) const -> value_type& {
      return m_ptr[i * m_str[0]];
    }

    auto operator()(std::size_t i, std::size_t j) const -> value_type& {
      return m_ptr[i * m_str[0] + j * m_str[1]];
    }

    // internal constructor used by subview
    View(std::shared_ptr<value_type[]> owner,
         value_type*                   ptr,
         std::array<std::size_t, 2>    ext,
         std::array<std::size_t, 2>    str,
         std::string                   label)
      : m_owner { std::move(owner) }
      , m_ptr { ptr }
      , m_ext { ext }
      , m_str { str }
      , m_label { std::move(label) } {}

    auto owner() const -> const std::shared_ptr<value_type[]>& {
      return m_owner;
    }

  private:
    std::shared_ptr<value_type[]> m_owner {};
    value_type*                   m_ptr { nullptr };
    std::array<std::size_t, 2>    m_ext { 0, traits::N1 };
    std::array<std::size_t, 2>    m_str { traits::N1, 1 };
    std::string                   m_label {};
  };

  // ---- subviews -----------------------------------------------------------
  template <class T>
  auto subview(const View<T*>& v, std::pair<std::size_t, std::size_t> r) -> View<T*> {
    return View<T*>(v.owner(),
                    v.data() + r.first * v.stride(0),
                    { r.second - r.first, 1 },
                    { v.stride(0), 1 },
                    v.label());
  }

  template <class T, std::size_t N>
  auto subview(const View<T* [N]>& v, std::pair<std::size_t, std::size_t> r, ALL_t)
    -> View<T* [N]> {
    return View<T* [N]>(v.owner(),
                        v.data() + r.first * v.stride(0),
                        { r.second - r.first, N },
                        { v.stride(0), v.stride(1) },
                        v.label());
  }

  template <class T, std::size_t N, class I>
  auto subview(const View<T* [N]>& v, std::pair<std::size_t, std::size_t> r, I comp)
    -> std::enable_if_t<std::is_integral_v<I>, View<T*>> {
    return View<T*>(v.owner(),
                    v.data() + r.first * v.stride(0) + static_cast<std::size_t>(comp) * v.stride(1),
                    { r.second - r.first, 1 },
                    { v.stride(0), 1 },
                    v.label());
  }

  template <class T, std::size_t N, class I>
  auto subview(const View<T* [N]>& v, ALL_t, I comp)
    -> std::enable_if_t<std::is_integral_v<I>, View<T*>> {
    return subview(v, std::pair<std::size_t, std::size_t> { 0, v.extent(0) }, comp);
  }

  template <class V>
  auto create_mirror_view(const V& v) -> V {
    return v;
  }

  template <class D, class S>
  void deep_copy(const View<D>& dst, const View<S>& src) {
    if (dst.data() == src.data() && dst.stride(0) == src.stride(0)) {
      return;
    }
    if constexpr (View<D>::rank() == 1) {
      const std::size_t n = std::min(dst.extent(0), src.extent(0));
      for (std::size_t i = 0; i < n; ++i) {
        dst(i) = src(i);
      }
    } else {
      const std::size_t n0 = std::min(dst.extent(0), src.extent(0));
      const std::size_t n1 = std::min(dst.extent(1), src.extent(1));
      for (std::size_t i = 0; i < n0; ++i) {
        for (std::size_t j = 0; j < n1; ++j) {
          dst(i, j) = src(i, j);
        }
      }
    }
  }

  template <class D>
  void deep_copy(const View<D>& dst, const typename View<D>::value_type& value) {
    if constexpr (View<D>::rank() == 1) {
      for (std::size_t i = 0; i < dst.extent(0); ++i) {
        dst(i) = value;
      }
    } else {
      for (std::size_t i = 0; i < dst.extent(0); ++i) {
        for (std::size_t j = 0; j < dst.extent(1); ++j) {
          dst(i, j) = value;
        }
      }
    }
  }

  // ---- execution policies ---------------------------------------------------
  template <class... Args>
  struct RangePolicy {
    std::size_t begin { 0 }, end { 0 };

    RangePolicy() = default;

    RangePolicy(std::size_t b, std::size_t e) : begin { b }, end { e } {}
  };

  template <unsigned R>
  struct Rank {
    static constexpr unsigned rank = R;
  };

  template <class RankT>
  struct MDRangePolicy {
    static constexpr unsigned R = RankT::rank;
    std::array<std::size_t, R> lo {}, hi {};

    MDRangePolicy(std::initializer_list<std::size_t> l,
                  std::initializer_list<std::size_t> h) {
      std::copy(l.begin(), l.end(), lo.begin());
      std::copy(h.begin(), h.end(), hi.begin());
    }
  };

  template <class F>
  void parallel_for(const std::string&, std::size_t n, const F& f) {
#pragma omp parallel for schedule(static)
    for (std::size_t i = 0; i < n; ++i) {
      f(i);
    }
  }

  template <class F, class... A>
  void parallel_for(const std::string&, const RangePolicy<A...>& p, const F& f) {
#pragma omp parallel for schedule(static)
    for (std::size_t i = p.begin; i < p.end; ++i) {
      f(i);
    }
  }

  template <class F>
  void parallel_for(const std::string&, const MDRangePolicy<Rank<2>>& p, const F& f) {
#pragma omp parallel for collapse(2) schedule(static)
    for (std::size_t i = p.lo[0]; i < p.hi[0]; ++i) {
      for (std::size_t j = p.lo[1]; j < p.hi[1]; ++j) {
        f(i, j);
      }
    }
  }

  template <class F>
  void parallel_for(const std::string&, const MDRangePolicy<Rank<3>>& p, const F& f) {
#pragma omp parallel for collapse(3) schedule(static)
    for (std::size_t i = p.lo[0]; i < p.hi[0]; ++i) {
      for (std::size_t j = p.lo[1]; j < p.hi[1]; ++j) {
        for (std::size_t k = p.lo[2]; k < p.hi[2]; ++k) {
          f(i, j, k);
        }
      }
    }
  }

  // ---- reductions -------------------------------------------------------------
  template <class T>
  struct MinMaxScalar {
    T min_val { std::numeric_limits<T>::max() };
    T max_val { std::numeric_limits<T>::lowest() };
  };

  template <class T>
  struct MinMax {
    MinMaxScalar<T>& result;

    explicit MinMax(MinMaxScalar<T>& r) : result { r } {}
  };

  template <class F, class T>
  void parallel_reduce(const std::string&, std::size_t n, const F& f, MinMax<T> red) {
    MinMaxScalar<T> acc {};
    for (std::size_t i = 0; i < n; ++i) {
      f(i, acc);
    }
    red.result = acc;
  }

  // ---- math (Kokkos overload set) ---------------------------------------------
  inline auto sqrt(float x) -> float {
    return std::sqrt(x);
  }

  inline auto sqrt(double x) -> double {
    return std::sqrt(x);
  }

  inline auto log10(float x) -> float {
    return std::log10(x);
  }

  inline auto log10(double x) -> double {
    return std::log10(x);
  }

  inline auto log(float x) -> float {
    return std::log(x);
  }

  inline auto log(double x) -> double {
    return std::log(x);
  }

  inline auto abs(float x) -> float {
    return std::fabs(x);
  }

  inline auto abs(double x) -> double {
    return std::fabs(x);
  }

  inline auto pow(float x, float y) -> float {
    return std::pow(x, y);
  }

  inline auto pow(double x, double y) -> double {
    return std::pow(x, y);
  }

  template <class A, class B>
  inline auto pow(A x, B y)
    -> std::enable_if_t<!(std::is_same_v<A, B> && std::is_floating_point_v<A>), double> {
    return std::pow(static_cast<double>(x), static_cast<double>(y));
  }

} // namespace Kokkos

// Host-side containers of the drop-in module.  They mirror the reference's
// containers (src/containers/*.hpp) and own device memory through the C ABI
// (include/ragnar_gb300.h); no CUDA headers are needed here.
#pragma once

#include "ragnar_gb300.h"

#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace rgh {

  // Status -> exception, with the reference's exception classes: RG_ERR_RANGE maps
  // to std::range_error (Python ValueError), the rest to std::runtime_error.
  inline void check(int status) {
    if (status == RG_OK) {
      return;
    }
    const std::string msg = rg_last_error();
    if (status == RG_ERR_RANGE) {
      throw std::range_error(msg);
    }
    throw std::runtime_error(msg);
  }

  // Owning device allocation.
  class DeviceBuffer {
  public:
    explicit DeviceBuffer(std::size_t bytes) : m_bytes { bytes } {
      check(rg_malloc(&m_ptr, bytes));
      if (bytes) {
        check(rg_memset(m_ptr, 0, bytes, nullptr));
      }
    }

    ~DeviceBuffer() {
      if (m_ptr) {
        rg_free(m_ptr);
      }
    }

    DeviceBuffer(const DeviceBuffer&)            = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;

    auto get() const -> void* {
      return m_ptr;
    }

    auto bytes() const -> std::size_t {
      return m_bytes;
    }

  private:
    void*       m_ptr { nullptr };
    std::size_t m_bytes { 0 };
  };

  // Array1D<T> (array.hpp:15-42): a reference-counted 1-D device array.
  template <class T>
  struct Array1D {
    std::shared_ptr<DeviceBuffer> buf;
    std::size_t                   n { 0 };

    Array1D() = default;

    explicit Array1D(std::size_t count)
      : buf { std::make_shared<DeviceBuffer>(count * sizeof(T)) }
      , n { count } {}

    static auto from_host(const T* data, std::size_t count) -> Array1D {
      Array1D a(count);
      if (count) {
        check(rg_memcpy_htod(a.buf->get(), data, count * sizeof(T), nullptr));
        check(rg_stream_synchronize(nullptr));
      }
      return a;
    }

    auto data() const -> T* {
      return buf ? static_cast<T*>(buf->get()) : nullptr;
    }

    auto extent(unsigned short d = 0) const -> std::size_t {
      return d == 0 ? n : 1;
    }

    auto to_host() const -> std::vector<T> {
      std::vector<T> h(n);
      if (n) {
        check(rg_memcpy_dtoh(h.data(), data(), n * sizeof(T), nullptr));
        check(rg_stream_synchronize(nullptr));
      }
      return h;
    }
  };

  // Bins (bins.hpp:17-30): an Array1D<float> plus the log_spaced flag and unit.
  struct Bins : Array1D<float> {
    bool        log_spaced { false };
    std::string unit;

    Bins() = default;

    Bins(const Array1D<float>& arr, const std::string& u) : Array1D<float> { arr }, unit { u } {}
  };

  // TabulatedDistribution (distributions.hpp:59-78): energy bins and f.
  struct TabulatedDistribution {
    Bins           bins;
    Array1D<float> f;

    TabulatedDistribution(const Bins& b, const Array1D<float>& fv) : bins { b }, f { fv } {
      if (bins.extent() != f.extent()) {
        throw std::runtime_error("e_bins.extent() != f.extent()");
      }
    }
  };

  // Particles<D> (particles.hpp:18-72) as device SoA arrays.  Components never
  // set by fromArrays are known to be zero and are passed to kernels as null.
  template <unsigned short D>
  class Particles {
  public:
    explicit Particles(const std::string& label) : m_label { label } {}

    // components: 0..2 U, 3..5 E, 6..8 B, 9 W (weights), 10.. X1..XD
    static constexpr int kU = 0, kE = 3, kB = 6, kW = 9, kX = 10, kN = 10 + D;

    void allocate(std::size_t nalloc);
    void reallocate(std::size_t nalloc);
    void setNactive(std::size_t n);

    void setIgnoreCoords(bool ig) {
      m_coords_ignored = ig;
    }

    auto is_allocated() const -> bool {
      return m_is_allocated;
    }

    auto nalloc() const -> std::size_t {
      return m_nalloc;
    }

    auto nactive() const -> std::size_t {
      return m_nactive;
    }

    auto label() const -> const std::string& {
      return m_label;
    }

    auto coords_ignored() const -> bool {
      return m_coords_ignored;
    }

    // Device pointer of component c (allocating zeros on demand).
    auto comp(int c) -> float*;

    // Device pointer or null when the component is known to be zero.
    auto comp_or_null(int c) const -> const float* {
      return m_written[c] ? static_cast<const float*>(m_comp[c]->get()) : nullptr;
    }

    auto written(int c) const -> bool {
      return m_written[c];
    }

    void mark_written(int c) {
      m_written[c] = true;
    }

    auto view() const -> rg_particles;

  private:
    bool                                       m_is_allocated { false };
    bool                                       m_coords_ignored { false };
    std::size_t                                m_nactive { 0 };
    std::size_t                                m_nalloc { 0 };
    std::string                                m_label;
    std::shared_ptr<DeviceBuffer>              m_comp[kN] {};
    bool                                       m_written[kN] {};
  };

  template <unsigned short D>
  void Particles<D>::allocate(std::size_t nalloc) {
    if (m_is_allocated) {
      throw std::runtime_error("Particles already allocated");
    }
    for (int c = 0; c < kN; ++c) {
      m_comp[c].reset();
      m_written[c] = false;
    }
    m_is_allocated = true;
    m_nalloc       = nalloc;
  }

  template <unsigned short D>
  auto Particles<D>::comp(int c) -> float* {
    if (!m_comp[c]) {
      // round the allocation up so every stream keeps 16-byte granularity
      m_comp[c] = std::make_shared<DeviceBuffer>(((m_nalloc + 3) / 4) * 4 * sizeof(float));
    }
    return static_cast<float*>(m_comp[c]->get());
  }

  template <unsigned short D>
  void Particles<D>::reallocate(std::size_t nalloc) {
    if (!m_is_allocated) {
      throw std::runtime_error("Particles not allocated, if you want to allocate, call `allocate` instead");
    }
    if (nalloc <= m_nalloc) {
      throw std::runtime_error("New allocation size must be greater than the current one");
    }
    for (int c = 0; c < kN; ++c) {
      if (!m_comp[c]) {
        continue;
      }
      auto fresh = std::make_shared<DeviceBuffer>(((nalloc + 3) / 4) * 4 * sizeof(float));
      check(rg_memcpy_dtod(fresh->get(), m_comp[c]->get(), m_nalloc * sizeof(float), nullptr));
      m_comp[c] = fresh;
    }
    check(rg_stream_synchronize(nullptr));
    m_nalloc = nalloc;
  }

  template <unsigned short D>
  void Particles<D>::setNactive(std::size_t n) {
    if (!m_is_allocated) {
      throw std::runtime_error("Particles not allocated");
    }
    m_nactive = n;
  }

  template <unsigned short D>
  auto Particles<D>::view() const -> rg_particles {
    rg_particles v {};
    for (int d = 0; d < 3; ++d) {
      // U is always present (zeros when never written) so kernels read it
      v.u[d] = m_comp[kU + d] ? static_cast<const float*>(m_comp[kU + d]->get()) : nullptr;
      v.e[d] = comp_or_null(kE + d);
      v.b[d] = comp_or_null(kB + d);
    }
    v.w = comp_or_null(kW);
    v.n = static_cast<int64_t>(m_nactive);
    return v;
  }

} // namespace rgh

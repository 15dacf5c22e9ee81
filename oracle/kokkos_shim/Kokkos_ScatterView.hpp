// Host-only ScatterView for the Kokkos-API shim (see Kokkos_Core.hpp).
// Mirrors the Kokkos "ScatterDuplicated" strategy used by the OpenMP backend:
// every OpenMP thread adds into its own zero-initialised copy of the target,
// and contribute() sums the copies into the target view.  An access
// "acc(i) += v" converts v to the view's value type before adding, as the
// Kokkos ScatterSum accessor does.
//
// This header is test infrastructure for the oracle only.
#pragma once

#include "Kokkos_Core.hpp"

#include <omp.h>

#include <memory>
#include <vector>

namespace Kokkos {
  namespace Experimental {

    template <class DataType>
    class ScatterView;

    template <class T>
    class ScatterView<T*> {
    public:
      struct Proxy {
        T* slot;

        void operator+=(const T& v) const {
          *slot += v;
        }
      };

      struct Access {
        T* base;

        auto operator()(std::size_t i) const -> Proxy {
          return Proxy { base + i };
        }
      };

      ScatterView() = default;

      explicit ScatterView(const View<T*>& v)
        : m_n { v.extent(0) }
        , m_nthreads { static_cast<std::size_t>(omp_get_max_threads()) }
        , m_dup { std::make_shared<std::vector<T>>(m_n * m_nthreads, T {}) } {}

      auto access() const -> Access {
        return Access { m_dup->data() + m_n * static_cast<std::size_t>(omp_get_thread_num()) };
      }

      void contribute_into(const View<T*>& v) const {
        for (std::size_t t = 0; t < m_nthreads; ++t) {
          for (std::size_t i = 0; i < m_n; ++i) {
            v(i) += (*m_dup)[t * m_n + i];
          }
        }
      }

    private:
      std::size_t                     m_n { 0 };
      std::size_t                     m_nthreads { 1 };
      std::shared_ptr<std::vector<T>> m_dup {};
    };

    template <class T>
    auto create_scatter_view(const View<T*>& v) -> ScatterView<T*> {
      return ScatterView<T*>(v);
    }

    template <class T>
    void contribute(const View<T*>& v, const ScatterView<T*>& s) {
      s.contribute_into(v);
    }

  } // namespace Experimental
} // namespace Kokkos

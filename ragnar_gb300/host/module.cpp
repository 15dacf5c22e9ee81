// pybind11 module `ragnar_gb300._ragnar`: the drop-in for the reference's
// `ragnar` module (pyinterface.cpp:26-91) on the synchrotron path.  Names,
// argument names, defaults, return types and error classes follow the
// reference's pyDefine* functions; compute goes through the C ABI.
#include "containers.hpp"

#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace py = pybind11;
using namespace pybind11::literals;

namespace rgh {

  bool g_verbose = true; // progress lines as the reference prints them

  // global.h:21-27
  struct EnergyUnits {
    inline static const std::string eV   = "eV";
    inline static const std::string MeV  = "MeV";
    inline static const std::string GeV  = "GeV";
    inline static const std::string mec2 = "mec2";
    inline static const std::string mpc2 = "mpc2";
  };

  // snippets.cpp:92-110 (ToHumanReadable without suffixes), for the progress lines
  std::string human(double v) {
    int p = 0;
    if (v > 0) {
      while (v < 0.1 || v >= 10) {
        if (v < 0.1) {
          v *= 10;
          --p;
        } else {
          v /= 10;
          ++p;
        }
      }
    }
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.2f", v);
    return std::string(buf) + "·10^" + std::to_string(p);
  }

  template <class T>
  Array1D<T> array_from_numpy(const py::array_t<T>& arr) {
    auto a = py::array_t<T, py::array::c_style | py::array::forcecast>::ensure(arr);
    if (!a) {
      throw std::runtime_error("could not convert array");
    }
    return Array1D<T>::from_host(a.data(), static_cast<std::size_t>(a.size()));
  }

  template <class T>
  py::array_t<T> as_array(const Array1D<T>& a) {
    py::array_t<T> out(static_cast<py::ssize_t>(a.n));
    if (a.n) {
      check(rg_memcpy_dtoh(out.mutable_data(), a.data(), a.n * sizeof(T), nullptr));
      check(rg_stream_synchronize(nullptr));
    }
    return out;
  }

  Array1D<float> make_logspace(float start, float stop, std::size_t num) {
    std::vector<float> h(num);
    check(rg_logspace(start, stop, static_cast<int64_t>(num), h.data()));
    return Array1D<float>::from_host(h.data(), num);
  }

  Array1D<float> make_linspace(float start, float stop, std::size_t num) {
    std::vector<float> h(num);
    check(rg_linspace(start, stop, static_cast<int64_t>(num), h.data()));
    return Array1D<float>::from_host(h.data(), num);
  }

  // ---- distribution generators (distributions.cpp:37-136), host float math ----
  struct DistGenerator {
    float m_norm { 1.0f };

    virtual ~DistGenerator() = default;
    virtual float f(float energy) const = 0;

    Array1D<float> compute(const Bins& bins) const {
      const auto         e = bins.to_host();
      std::vector<float> v(e.size());
      for (std::size_t i = 0; i < e.size(); ++i) {
        v[i] = f(e[i]);
      }
      return Array1D<float>::from_host(v.data(), v.size());
    }
  };

  struct PlawGenerator : DistGenerator {
    const float p, emin, emax;

    PlawGenerator(float p_, float emin_, float emax_) : p { p_ }, emin { emin_ }, emax { emax_ } {
      if (emin < 0.0) {
        throw std::runtime_error("emin < 0.0");
      } else if (emin > emax and emax > 0.0) {
        throw std::runtime_error("emin > emax");
      } else if (emin == 0.0 and p <= -1.0) {
        throw std::runtime_error("p <= -1 and emin = 0.0 : normalization diverges");
      } else if (emax == 0.0 and p >= -1.0) {
        throw std::runtime_error("p >= -1 and emax = 0.0 (infinity) : normalization diverges");
      } else if (emax == 0.0) {
        m_norm = -std::pow(emin, p + 1) / (p + 1);
      } else if (p != -1.0) {
        m_norm = (std::pow(emax, p + 1) - std::pow(emin, p + 1)) / (p + 1);
      } else {
        m_norm = std::log(emax / emin);
      }
    }

    float f(float energy) const override {
      if (energy < emin or (emax > 0.0 and energy >= emax)) {
        return 0.0f;
      }
      return std::pow(energy, p) / m_norm;
    }
  };

  struct BrokenPlawGenerator : DistGenerator {
    const float e_break, emin, emax;
    const float p1, p2;

    BrokenPlawGenerator(float eb, float p1_, float p2_, float emin_, float emax_)
      : e_break { eb }
      , emin { emin_ }
      , emax { emax_ }
      , p1 { p1_ }
      , p2 { p2_ } {
      if (e_break <= 0.0) {
        throw std::runtime_error("e_break <= 0.0");
      }
      if (emin < 0.0) {
        throw std::runtime_error("emin < 0.0");
      }
      if (emin > emax and emax > 0.0) {
        throw std::runtime_error("emin > emax");
      }
      float pre_break, post_break;
      if (emin == 0.0 and p1 <= -1.0) {
        throw std::runtime_error("p1 <= -1 and emin = 0.0 : normalization diverges");
      } else if (e_break <= emin) {
        pre_break = 0.0;
      } else {
        pre_break = (1 - std::pow(emin / e_break, p1 + 1)) / (p1 + 1);
      }
      if (emax == 0.0 and p2 >= -1.0) {
        throw std::runtime_error("p2 >= -1 and emax = 0.0 (infinity) : normalization diverges");
      } else if (emax == 0.0) {
        post_break = 1 / (-p2 - 1);
      } else if (p2 == -1.0) {
        post_break = std::log(emax / e_break);
      } else {
        post_break = (std::pow(emax / e_break, p2 + 1) - 1) / (p2 + 1);
      }
      m_norm = (pre_break + post_break) * e_break;
    }

    float f(float energy) const override {
      if (energy < emin or (emax > 0.0 and energy >= emax)) {
        return 0.0f;
      }
      if (energy < e_break) {
        return std::pow(energy / e_break, p1) / m_norm;
      }
      return std::pow(energy / e_break, p2) / m_norm;
    }
  };

  struct DeltaGenerator : DistGenerator {
    const float energy0, denergy;

    DeltaGenerator(float e0, float de) : energy0 { e0 }, denergy { de } {
      m_norm = 1.0 / denergy;
    }

    float f(float energy) const override {
      if (std::abs(energy - energy0) < denergy * 0.5) {
        return 1.0 * m_norm;
      }
      return 0.0f;
    }
  };

  // ---- TabulatedFunction<LG> (tabulation.hpp:55-116, tabulation.cpp:17-117) -----
  template <bool LG>
  struct TabulatedFunction {
    Array1D<float> x, y;
    float          yfill;
    std::size_t    n;
    float          xmin { 0 }, xmax { 0 };

    TabulatedFunction(const Array1D<float>& xa, const Array1D<float>& ya, float fill)
      : x { xa }
      , y { ya }
      , yfill { fill }
      , n { xa.extent() } {
      const auto hx = x.to_host();
      xmin          = std::numeric_limits<float>::max();
      xmax          = std::numeric_limits<float>::lowest();
      for (float v : hx) {
        xmin = std::min(xmin, v);
        xmax = std::max(xmax, v);
      }
      if (y.extent() != n) {
        throw std::range_error("y.size != x.size in TabulatedFunction");
      }
      if (xmin >= xmax) {
        throw std::range_error("xmin >= xmax in TabulatedFunction");
      }
      if (LG && xmin <= 0.0) {
        throw std::range_error("xmin <= 0.0 in Logspace TabulatedFunction");
      }
    }
  };

  // ---- particles -------------------------------------------------------------------

  template <unsigned short D>
  void from_arrays(Particles<D>& P, const std::map<std::string, py::array_t<float>>& arrays,
                   bool append) {
    if ((not append) and P.is_allocated()) {
      throw std::runtime_error(
        "Particles already allocated, if you want to append, specify `append = True`");
    }
    std::size_t nprtls = 0;
    for (const auto& kv : arrays) {
      const std::size_t len = static_cast<std::size_t>(kv.second.shape(0));
      if (nprtls == 0) {
        nprtls = len;
      } else if (nprtls != len) {
        throw std::runtime_error("Inconsistent number of particles");
      }
    }
    if (nprtls == 0) {
      throw std::runtime_error("No particles provided");
    }
    std::size_t start = 0;
    if (P.is_allocated()) {
      start = P.nactive();
      if (start + nprtls > P.nalloc()) {
        P.reallocate(P.nactive() + nprtls);
      }
    } else {
      P.allocate(nprtls);
    }
    // coordinates are kept unless ignored (particles.cpp:53-69)
    bool has_coords = not P.coords_ignored();
    std::map<std::string, int> keys;
    for (int d = 0; d < 3; ++d) {
      keys["U" + std::to_string(d + 1)] = Particles<D>::kU + d;
      keys["E" + std::to_string(d + 1)] = Particles<D>::kE + d;
      keys["B" + std::to_string(d + 1)] = Particles<D>::kB + d;
    }
    keys["W"] = Particles<D>::kW; // extension: per-particle weights
    for (int d = 0; d < D; ++d) {
      const std::string k = "X" + std::to_string(d + 1);
      if (arrays.count(k)) {
        has_coords = true;
      }
      keys[k] = Particles<D>::kX + d;
    }
    P.setIgnoreCoords(not has_coords);
    for (const auto& kv : keys) {
      auto it = arrays.find(kv.first);
      if (it == arrays.end()) {
        continue;
      }
      const int c = kv.second;
      if (c >= Particles<D>::kX && !has_coords) {
        continue;
      }
      auto a = py::array_t<float, py::array::c_style | py::array::forcecast>::ensure(it->second);
      float* dst = P.comp(c);
      check(rg_memcpy_htod(dst + start, a.data(), nprtls * sizeof(float), nullptr));
      P.mark_written(c);
    }
    for (int d = 0; d < 3; ++d) {
      P.comp(Particles<D>::kU + d); // U always exists on the device
    }
    check(rg_stream_synchronize(nullptr));
    P.setNactive(start + nprtls);
  }

  template <unsigned short D>
  Array1D<float> component(Particles<D>& P, int c, const char* name) {
    Array1D<float> out(P.nactive());
    if (P.nactive()) {
      check(rg_memcpy_dtod(out.data(), P.comp(c), P.nactive() * sizeof(float), nullptr));
      check(rg_stream_synchronize(nullptr));
    }
    (void)name;
    return out;
  }

  template <unsigned short D>
  TabulatedDistribution energy_distribution(Particles<D>& P, const Bins& bins, bool fourvel) {
    if (g_verbose) {
      py::print("Computing energy distribution for", P.label(), "...", "end"_a = "", "flush"_a = true);
    }
    const auto     hb = bins.to_host();
    Array1D<float> hist(bins.extent());
    if (!hb.empty()) {
      const auto v = P.view();
      for (int d = 0; d < 3; ++d) {
        P.comp(Particles<D>::kU + d);
      }
      const auto v2 = P.view();
      {
        py::gil_scoped_release nogil;
        check(rg_energy_distribution(v2.u[0], v2.u[1], v2.u[2], v.n, hb.data(),
                                     static_cast<int32_t>(hb.size()), bins.log_spaced ? 1 : 0,
                                     fourvel ? 1 : 0, hist.data(), nullptr, nullptr));
        // the reference fences before returning (particles.cpp:256)
        check(rg_stream_synchronize(nullptr));
      }
    }
    if (g_verbose) {
      py::print(": OK", "flush"_a = true);
    }
    return TabulatedDistribution(bins, hist);
  }

  template <unsigned short D>
  Array1D<float> synchrotron_spectrum(Particles<D>& P, const Bins& bins, float B0, float g_syn,
                                      float eps) {
    if (g_verbose) {
      py::print("Computing synchrotron spectrum for", P.label(), "flush"_a = true);
      py::print(" Launching", human(static_cast<double>(P.nactive()) * bins.extent()), "threads",
                "end"_a = "", "flush"_a = true);
    }
    // sync::Kernel constructor (synchrotron.hpp:139-142)
    if (bins.unit != EnergyUnits::mec2 and bins.unit != EnergyUnits::mpc2) {
      throw std::runtime_error("bins_e_syn must be in units of mc^2");
    }
    const auto     hb = bins.to_host();
    Array1D<float> out(bins.extent());
    if (P.is_allocated()) {
      for (int d = 0; d < 3; ++d) {
        P.comp(Particles<D>::kU + d);
      }
    }
    const rg_particles v = P.view();
    if (!hb.empty() && v.n > 0) {
      py::gil_scoped_release nogil;
      check(rg_synchrotron_spectrum(&v, hb.data(), static_cast<int32_t>(hb.size()), B0, g_syn, eps,
                                    out.data(), nullptr));
      check(rg_stream_synchronize(nullptr));
    }
    if (g_verbose) {
      py::print(": OK", "flush"_a = true);
    }
    return out;
  }

  // Extension: spectra of consecutive particle ranges [offsets[s], offsets[s+1]) in
  // one launch; returns a [nseg, nbins] float32 numpy array.
  template <unsigned short D>
  py::array_t<float> synchrotron_spectrum_batched(Particles<D>& P, const std::vector<int64_t>& offsets,
                                                  const Bins& bins, float B0, float g_syn,
                                                  float eps) {
    if (bins.unit != EnergyUnits::mec2 and bins.unit != EnergyUnits::mpc2) {
      throw std::runtime_error("bins_e_syn must be in units of mc^2");
    }
    if (offsets.size() < 1) {
      throw std::runtime_error("offsets must hold nseg + 1 values");
    }
    const int  nseg = static_cast<int>(offsets.size()) - 1;
    const auto hb   = bins.to_host();
    py::array_t<float> res({ static_cast<py::ssize_t>(nseg), static_cast<py::ssize_t>(hb.size()) });
    if (nseg == 0 || hb.empty()) {
      return res;
    }
    for (std::size_t i = 0; i + 1 < offsets.size(); ++i) {
      if (offsets[i + 1] < offsets[i] || offsets[i] < 0) {
        throw std::runtime_error("offsets must be non-decreasing and >= 0");
      }
    }
    if (offsets.back() > static_cast<int64_t>(P.nactive())) {
      throw std::runtime_error("offsets exceed the number of active particles");
    }
    for (int d = 0; d < 3; ++d) {
      P.comp(Particles<D>::kU + d);
    }
    const rg_particles v = P.view();
    Array1D<int64_t>   doff = Array1D<int64_t>::from_host(offsets.data(), offsets.size());
    Array1D<float>     out(static_cast<std::size_t>(nseg) * hb.size());
    {
      py::gil_scoped_release nogil;
      rg_spectrum_plan*      plan = nullptr;
      check(rg_spectrum_plan_create(hb.data(), static_cast<int32_t>(hb.size()), B0, g_syn, eps,
                                    RG_TABLE_REFERENCE, &plan));
      int st = rg_spectrum_run_batched(plan, &v, doff.data(), nseg, out.data(), nullptr);
      if (st == RG_OK) {
        st = rg_spectrum_plan_check(plan, nullptr);
      }
      rg_spectrum_plan_destroy(plan);
      check(st);
    }
    check(rg_memcpy_dtoh(res.mutable_data(), out.data(), out.n * sizeof(float), nullptr));
    check(rg_stream_synchronize(nullptr));
    return res;
  }

  Array1D<float> synchrotron_spectrum_from_dist(const TabulatedDistribution& dist, const Bins& bins,
                                                float g_syn, float eps) {
    if (g_verbose) {
      py::print("Computing synchrotron spectrum from a distribution", "flush"_a = true);
      py::print(" Launching", human(static_cast<double>(dist.f.extent()) * bins.extent()),
                "threads", "end"_a = "", "flush"_a = true);
    }
    const auto     hb = bins.to_host();
    Array1D<float> out(bins.extent());
    if (!hb.empty()) {
      py::gil_scoped_release nogil;
      check(rg_synchrotron_spectrum_from_dist(
        dist.bins.data(), dist.f.data(), static_cast<int32_t>(dist.f.extent()),
        dist.bins.log_spaced ? 1 : 0, hb.data(), static_cast<int32_t>(hb.size()), g_syn, eps,
        out.data(), nullptr));
    }
    if (g_verbose) {
      py::print(": OK", "flush"_a = true);
    }
    return out;
  }

  // ICSpectrum (ic.cpp:15-46) with the unit checks of ic::Kernel (ic.hpp:57-63).
  Array1D<float> ic_spectrum(const TabulatedDistribution& dist_prtls, const TabulatedDistribution& dist_soft,
                             const Bins& bins_e_ic) {
    if (dist_soft.bins.unit != EnergyUnits::mec2) {
      throw std::runtime_error("Soft photons energy bins must be in units of mec^2");
    }
    if (bins_e_ic.unit != EnergyUnits::mec2) {
      throw std::runtime_error("E_ic must be in units of mec^2");
    }
    if (g_verbose) {
      py::print("Computing IC spectrum ...", "flush"_a = true);
      py::print(" Launching",
                human(static_cast<double>(dist_prtls.f.extent()) * dist_soft.f.extent() * bins_e_ic.extent()),
                "threads", "end"_a = "", "flush"_a = true);
    }
    Array1D<float> out(bins_e_ic.extent());
    if (out.n > 0) {
      py::gil_scoped_release nogil;
      check(rg_ic_spectrum(dist_prtls.bins.data(), dist_prtls.f.data(), static_cast<int32_t>(dist_prtls.f.extent()),
                           dist_prtls.bins.log_spaced ? 1 : 0, dist_soft.bins.data(), dist_soft.f.data(),
                           static_cast<int32_t>(dist_soft.f.extent()), bins_e_ic.data(),
                           static_cast<int32_t>(bins_e_ic.extent()), out.data(), nullptr));
      check(rg_stream_synchronize(nullptr));
    }
    if (g_verbose) {
      py::print(": OK", "flush"_a = true);
    }
    return out;
  }

  float ffunc_integrand(float x) {
    Array1D<float> dx = Array1D<float>::from_host(&x, 1);
    Array1D<float> dy(1);
    check(rg_ffunc_integrand(dx.data(), 1, dy.data(), nullptr));
    return dy.to_host()[0];
  }

  template <class T>
  void define_array(py::module& m, const char* name) {
    py::class_<Array1D<T>>(m, name)
      .def(py::init<>())
      .def(py::init([](const py::array_t<T>& arr) { return array_from_numpy<T>(arr); }), "arr"_a)
      .def(
        "head",
        [](const Array1D<T>& a, std::size_t n, std::size_t start) {
          if (start + n > a.n) {
            throw std::range_error("Array::head: n > data.extent(0)");
          }
          const auto h = a.to_host();
          for (std::size_t i = start; i < start + n; ++i) {
            py::print(h[i], " ", "end"_a = "");
          }
          py::print();
        },
        "n"_a = 10, "start"_a = 0)
      .def("__repr__",
           [](const Array1D<T>& a) {
             return "1D Array [ size: " + std::to_string(a.n) + " ]";
           })
      .def("as_array", [](const Array1D<T>& a) { return as_array<T>(a); })
      .def("extent", &Array1D<T>::extent, "d"_a = 0);
  }

  template <bool LG>
  void define_tabulated_function(py::module& m) {
    using TF = TabulatedFunction<LG>;
    py::class_<TF>(m, LG ? "TabulatedFunction_log" : "TabulatedFunction")
      .def(py::init<const Array1D<float>&, const Array1D<float>&, float>(), "x"_a, "y"_a,
           "yfill"_a = 0.0)
      .def(py::init([](const py::array_t<float>& x, const py::array_t<float>& y, float fill) {
             return TF(array_from_numpy<float>(x), array_from_numpy<float>(y), fill);
           }),
           "x"_a, "y"_a, "yfill"_a = 0.0)
      .def("xArr", [](const TF& t) { return t.x; })
      .def("yArr", [](const TF& t) { return t.y; })
      .def("nPoints", [](const TF& t) { return t.n; })
      .def("yFill", [](const TF& t) { return t.yfill; })
      .def("xMin", [](const TF& t) { return t.xmin; })
      .def("xMax", [](const TF& t) { return t.xmax; });
  }

  template <class Gen>
  void define_generator_compute(py::class_<Gen>& c) {
    c.def("compute", [](const Gen& g, const Bins& b) { return g.compute(b); }, "energy_bins"_a);
  }

  template <unsigned short D>
  void define_particles(py::module& m) {
    using P = Particles<D>;
    const std::string name = "Particles_" + std::to_string(D) + "D";
    py::class_<P>(m, name.c_str())
      .def(py::init<const std::string&>())
      .def("__repr__",
           [](const P& p) {
             return "Particles<" + std::to_string(D) + "D> (" + p.label() + ") : " +
                    (p.is_allocated() ? human(static_cast<double>(p.nactive())) : "not allocated");
           })
      .def("__len__", &P::nactive)
      .def("fromArrays", &from_arrays<D>, "arrays"_a, "append"_a = false)
      .def("setNactive", &P::setNactive)
      .def("setIgnoreCoords", &P::setIgnoreCoords)
      .def("allocate", &P::allocate)
      .def(
        "printHead",
        [](P& p, std::size_t number, std::size_t start) {
          py::print("Particles:", p.label());
          if (!p.is_allocated()) {
            py::print(" [ not allocated ]");
            return;
          }
          if (start + number > p.nalloc()) {
            throw std::runtime_error("Number of particles to print exceeds allocated space");
          }
          py::print(" [", p.nactive(), "/", p.nalloc(), "]");
          py::print(" showing", start, "to", start + number);
          const char* qs[3] = { "U", "E", "B" };
          for (int q = 0; q < 3; ++q) {
            for (int d = 0; d < 3; ++d) {
              std::vector<float> h(number);
              if (number) {
                check(rg_memcpy_dtoh(h.data(), p.comp(3 * q + d) + start, number * sizeof(float), nullptr));
                check(rg_stream_synchronize(nullptr));
              }
              py::print(" ", std::string(qs[q]) + "_" + std::to_string(d + 1), ":", "end"_a = "");
              if (start > 0) {
                py::print("...", "end"_a = "");
              }
              for (float v : h) {
                py::print(v, " ", "end"_a = "");
              }
              if (p.nalloc() > start + number) {
                py::print("...");
              } else {
                py::print();
              }
            }
          }
        },
        "number"_a = 5, "start"_a = 0)
      .def("is_allocated", &P::is_allocated)
      .def("nactive", &P::nactive)
      .def("nalloc", &P::nalloc)
      .def("label", &P::label)
      .def("energyDistribution", &energy_distribution<D>, "energy_bins"_a, "fourvel"_a = true)
      .def(
        "X",
        [](P& p, std::size_t d) {
          if (p.coords_ignored()) {
            throw std::runtime_error("Particle coordinates ignored");
          }
          if (d < 1 || d > D) {
            throw std::out_of_range("Invalid component");
          }
          return component<D>(p, P::kX + static_cast<int>(d) - 1, "X");
        },
        "d"_a)
      .def(
        "U",
        [](P& p, std::size_t d) {
          if (d < 1 || d > 3) {
            throw std::out_of_range("Invalid component");
          }
          return component<D>(p, P::kU + static_cast<int>(d) - 1, "U");
        },
        "d"_a)
      .def(
        "E",
        [](P& p, std::size_t d) {
          if (d < 1 || d > 3) {
            throw std::out_of_range("Invalid component");
          }
          return component<D>(p, P::kE + static_cast<int>(d) - 1, "E");
        },
        "d"_a)
      .def(
        "B",
        [](P& p, std::size_t d) {
          if (d < 1 || d > 3) {
            throw std::out_of_range("Invalid component");
          }
          return component<D>(p, P::kB + static_cast<int>(d) - 1, "B");
        },
        "d"_a)
      .def("W", [](P& p) { return component<D>(p, P::kW, "W"); })
      .def("device_view",
           [](P& p) {
             // extension: device pointers of the SoA streams (0 = known zero)
             for (int d = 0; d < 3; ++d) {
               p.comp(P::kU + d);
             }
             const rg_particles v = p.view();
             py::dict           out;
             const char*        un[3] = { "U1", "U2", "U3" };
             const char*        en[3] = { "E1", "E2", "E3" };
             const char*        bn[3] = { "B1", "B2", "B3" };
             for (int d = 0; d < 3; ++d) {
               out[un[d]] = reinterpret_cast<uintptr_t>(v.u[d]);
               out[en[d]] = reinterpret_cast<uintptr_t>(v.e[d]);
               out[bn[d]] = reinterpret_cast<uintptr_t>(v.b[d]);
             }
             out["W"] = reinterpret_cast<uintptr_t>(v.w);
             out["n"] = v.n;
             return out;
           });
    m.def(("SynchrotronSpectrum_" + std::to_string(D) + "D").c_str(), &synchrotron_spectrum<D>,
          "prtls"_a, "bins_e_syn"_a, "B0"_a, "g_syn"_a, "e_syn_at_g_syn"_a,
          "Compute the synchrotron spectrum E^2 dN/dE for a set of particles");
    m.def(("SynchrotronSpectrumBatched_" + std::to_string(D) + "D").c_str(),
          &synchrotron_spectrum_batched<D>, "prtls"_a, "offsets"_a, "bins_e_syn"_a, "B0"_a,
          "g_syn"_a, "e_syn_at_g_syn"_a,
          "Spectra of the particle ranges [offsets[s], offsets[s+1]) in one launch; "
          "returns a [nseg, nbins] float32 array");
  }

} // namespace rgh

PYBIND11_MODULE(_ragnar, m) {
  using namespace rgh;
  m.doc() = "ragnar_gb300: GB300-native synchrotron path of the ragnar radiative post-processing library";

  m.def(
    "Initialize",
    []() {
      check(rg_init(0));
    },
    "Initialize the GPU context (device 0) and build the F table");
  m.def(
    "Finalize", []() { check(rg_finalize()); }, "Release cached GPU tables");
  m.def(
    "SetVerbose", [](bool v) { g_verbose = v; }, "v"_a,
    "Print the reference's progress lines (default True)");

  py::class_<EnergyUnits>(m, "EnergyUnits")
    .def_readonly_static("eV", &EnergyUnits::eV)
    .def_readonly_static("MeV", &EnergyUnits::MeV)
    .def_readonly_static("GeV", &EnergyUnits::GeV)
    .def_readonly_static("mec2", &EnergyUnits::mec2)
    .def_readonly_static("mpc2", &EnergyUnits::mpc2);

  m.def("Linspace", &make_linspace, "start"_a, "stop"_a, "num"_a);
  m.def("Logspace", &make_logspace, "start"_a, "stop"_a, "num"_a);

  define_array<int>(m, "Array1D_i");
  define_array<float>(m, "Array1D_f");
  define_array<double>(m, "Array1D_d");

  py::class_<Bins, Array1D<float>>(m, "Bins")
    .def(py::init<const Array1D<float>&, const std::string&>(), "arr"_a, "unit"_a = "")
    .def(py::init([](const std::string& u) { return Bins(Array1D<float>(), u); }), "unit"_a = "")
    .def(py::init([](const py::array_t<float>& a, const std::string& u) {
           return Bins(array_from_numpy<float>(a), u);
         }),
         "arr"_a, "unit"_a = "")
    .def_readwrite("log_spaced", &Bins::log_spaced)
    .def_readwrite("unit", &Bins::unit);

  m.def(
    "Linbins",
    [](float a, float b, std::size_t n, const std::string& u) {
      Bins r(make_linspace(a, b, n), u);
      r.log_spaced = false;
      return r;
    },
    "start"_a, "stop"_a, "num"_a, "unit"_a = "");
  m.def(
    "Logbins",
    [](float a, float b, std::size_t n, const std::string& u) {
      Bins r(make_logspace(a, b, n), u);
      r.log_spaced = true;
      return r;
    },
    "start"_a, "stop"_a, "num"_a, "unit"_a = "");

  define_tabulated_function<true>(m);
  define_tabulated_function<false>(m);

  py::class_<PlawGenerator> plaw(m, "PlawGenerator");
  plaw.def(py::init<float, float, float>(), "p"_a, "emin"_a = 0.0, "emax"_a = 0.0)
    .def_readonly("p", &PlawGenerator::p)
    .def_readonly("emin", &PlawGenerator::emin)
    .def_readonly("emax", &PlawGenerator::emax);
  define_generator_compute(plaw);
  py::class_<BrokenPlawGenerator> bplaw(m, "BrokenPlawGenerator");
  bplaw
    .def(py::init<float, float, float, float, float>(), "e_break"_a, "p1"_a, "p2"_a,
         "emin"_a = 0.0, "emax"_a = 0.0)
    .def_readonly("e_break", &BrokenPlawGenerator::e_break)
    .def_readonly("p1", &BrokenPlawGenerator::p1)
    .def_readonly("p2", &BrokenPlawGenerator::p2)
    .def_readonly("emin", &BrokenPlawGenerator::emin)
    .def_readonly("emax", &BrokenPlawGenerator::emax);
  define_generator_compute(bplaw);
  py::class_<DeltaGenerator> delta(m, "DeltaGenerator");
  delta.def(py::init<float, float>(), "energy0"_a, "denergy"_a)
    .def_readonly("energy0", &DeltaGenerator::energy0)
    .def_readonly("denergy", &DeltaGenerator::denergy);
  define_generator_compute(delta);

  py::class_<TabulatedDistribution>(m, "TabulatedDistribution")
    .def(py::init<const Bins&, const Array1D<float>&>(), "bins_energy"_a, "f"_a)
    .def(py::init([](const Bins& b, const PlawGenerator& g) { return TabulatedDistribution(b, g.compute(b)); }),
         "bins_energy"_a, "generator"_a)
    .def(py::init([](const Bins& b, const BrokenPlawGenerator& g) {
           return TabulatedDistribution(b, g.compute(b));
         }),
         "bins_energy"_a, "generator"_a)
    .def(py::init([](const Bins& b, const DeltaGenerator& g) { return TabulatedDistribution(b, g.compute(b)); }),
         "bins_energy"_a, "generator"_a)
    .def("extent", [](const TabulatedDistribution& d) { return d.f.extent(); })
    .def("log_spaced", [](const TabulatedDistribution& d) { return d.bins.log_spaced; })
    .def("EnergyBins", [](const TabulatedDistribution& d) { return d.bins; })
    .def("F", [](const TabulatedDistribution& d) { return d.f; });

  define_particles<1>(m);
  define_particles<2>(m);
  define_particles<3>(m);

  m.def("Ffunc_integrand", &ffunc_integrand, "x"_a);
  m.def("ICSpectrum", &ic_spectrum, "dist_prtls"_a, "dist_soft_photons"_a, "bins_e_ic"_a,
        "Compute the IC spectrum E^2 dN/dE of a particle distribution on a soft-photon distribution");
  m.def("SynchrotronSpectrumFromDist", &synchrotron_spectrum_from_dist, "dist_prtls"_a,
        "bins_e_syn"_a, "g_syn"_a, "e_syn_at_g_syn"_a,
        "Compute the synchrotron spectrum E^2 dN/dE from a distribution of particles");
}

// ragnar oracle -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of the reference library's synchrotron hot path, used by the
// tests, by smoke() and by bench.py's cpu_baseline / reference arm as the checker
// and the CPU baseline.  The product never links or calls this file.
//
// Two kinds of entry points:
//   *_ref32  follow the reference's arithmetic step by step (float storage,
//            the FP64 kinematics that `auto gamma = sqrt(1.0 + ...)` deduces,
//            log10f interpolation, per-thread float accumulation as Kokkos'
//            OpenMP ScatterView does).  They are the "port" CPU baseline and
//            reproduce the reference's results to its own rounding noise.
//   *_f64    the same mathematical function with every intermediate in double
//            (the float table nodes, float bins and float particle data are the
//            data; kinematics, interpolation and accumulation are double).  They
//            are the ground truth for the relative-error checks.
//
// Citations are file:line in the reference tree (paths under src/).
// Built by oracle/Makefile with -ffp-contract=off so that float expressions are
// evaluated exactly as written, as g++ -std=c++20 does for the reference.

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace {

  constexpr double kOneThird  = 0.3333333333333333;
  constexpr double kFiveThird = 1.6666666666666667;

  int threads_or_default(int nthreads) {
    return nthreads > 0 ? nthreads : omp_get_max_threads();
  }

  // snippets.cpp:39-62 (Logspace): pow(10, log10f(a) + float(i) * log10f(b/a) / float(n-1))
  // with Kokkos' pow(int, float) promoting to double, stored as float.
  float logspace_point(float start, float stop, std::size_t num, std::size_t i) {
    if (num == 1) {
      return start;
    }
    const float e = std::log10(start) +
                    static_cast<float>(i) * (std::log10(stop / start)) /
                      static_cast<float>(num - 1);
    return static_cast<float>(std::pow(10.0, static_cast<double>(e)));
  }

  // tabulation.hpp:19-53 with LG = true, evaluated in float as the reference does.
  float interp_log_f32(float x0, const float* x, const float* y, std::size_t n,
                       float xmin, float xmax, float yfill) {
    if (x0 < xmin or x0 >= xmax) {
      return yfill;
    }
    const auto xi = static_cast<std::size_t>(static_cast<float>(n - 1) *
                                             std::fabs(std::log10(x0 / xmin)) /
                                             std::log10(xmax / xmin));
    if (xi >= n - 1) {
      return y[n - 1];
    }
    return (y[xi + 1] * std::log10(x0 / x[xi]) + y[xi] * std::log10(x[xi + 1] / x0)) /
           std::log10(x[xi + 1] / x[xi]);
  }

  // The same selection rule and two-node lerp, in double.  The segment index is
  // the reference's ideal-grid floor; the lerp uses the actual float nodes.
  double interp_log_f64(double x0, const float* x, const float* y, std::size_t n,
                        double xmin, double xmax) {
    if (x0 < xmin or x0 >= xmax) {
      return 0.0;
    }
    const double t  = static_cast<double>(n - 1) * std::fabs(std::log10(x0 / xmin)) /
                     std::log10(xmax / xmin);
    const auto   xi = static_cast<std::size_t>(t);
    if (xi >= n - 1) {
      return y[n - 1];
    }
    const double xa = x[xi], xb = x[xi + 1];
    return (static_cast<double>(y[xi + 1]) * std::log10(x0 / xa) +
            static_cast<double>(y[xi]) * std::log10(xb / x0)) /
           std::log10(xb / xa);
  }

  // synchrotron.hpp:181-232 (OmegaSync_ChiR) in double; the dead eprime lines
  // (:201-217) are omitted because nothing reads them.
  inline void omega_chi_f64(double ux, double uy, double uz, double ex, double ey, double ez,
                            double bx, double by, double bz, double B0, double g_syn,
                            double eps, double& e_peak, double& chiR) {
    const double gamma  = std::sqrt(1.0 + ux * ux + uy * uy + uz * uz);
    const double beta_x = ux / gamma, beta_y = uy / gamma, beta_z = uz / gamma;
    const double bde    = beta_x * ex + beta_y * ey + beta_z * ez;
    const double cx     = beta_y * bz - beta_z * by;
    const double cy     = beta_z * bx - beta_x * bz;
    const double cz     = beta_x * by - beta_y * bx;
    const double vx = ex + cx, vy = ey + cy, vz = ez + cz;
    const double v2 = vx * vx + vy * vy + vz * vz;
    chiR            = std::sqrt(v2 - bde * bde) / B0;
    e_peak          = eps * gamma * gamma * chiR / (g_syn * g_syn);
  }

  // The reference's own rounding of the same (synchrotron.hpp:230-231): chiR is a
  // float output parameter, so e_peak is formed from the float chiR, and
  // g_syn * g_syn is a float product; e_peak is stored as float.
  inline void omega_chi_ref(float ux, float uy, float uz, float ex, float ey, float ez, float bx,
                            float by, float bz, float B0, float g_syn, float eps, float& e_peak,
                            float& chiR) {
    const double gamma  = std::sqrt(1.0 + ux * ux + uy * uy + uz * uz);
    const double beta_x = ux / gamma, beta_y = uy / gamma, beta_z = uz / gamma;
    const double bde    = beta_x * ex + beta_y * ey + beta_z * ez;
    const double cx     = beta_y * bz - beta_z * by;
    const double cy     = beta_z * bx - beta_x * bz;
    const double cz     = beta_x * by - beta_y * bx;
    const double vx = ex + cx, vy = ey + cy, vz = ez + cz;
    const double v2 = vx * vx + vy * vy + vz * vz;
    chiR            = static_cast<float>(std::sqrt(v2 - bde * bde) / B0);
    e_peak          = static_cast<float>(eps * gamma * gamma * chiR / (g_syn * g_syn));
  }

  struct Particles {
    const float *ux, *uy, *uz, *ex, *ey, *ez, *bx, *by, *bz, *w;
  };

  inline float comp(const float* p, std::int64_t i) {
    return p ? p[i] : 0.0f;
  }

} // namespace

extern "C" {

// snippets.cpp:21-37 (Linspace): start + i * (stop - start) / (num - 1), with i a
// size_t promoted to float.
void orc_linspace(float start, float stop, std::int64_t num, float* out) {
  for (std::int64_t i = 0; i < num; ++i) {
    out[i] = (num == 1) ? start
                        : start + static_cast<std::size_t>(i) * (stop - start) /
                                    static_cast<std::size_t>(num - 1);
  }
}

void orc_logspace(float start, float stop, std::int64_t num, float* out) {
  for (std::int64_t i = 0; i < num; ++i) {
    out[i] = logspace_point(start, stop, static_cast<std::size_t>(num), static_cast<std::size_t>(i));
  }
}

// synchrotron.cpp:28-46 (Ffunc_integrand): asymptotic below 1e-5, zero above 20,
// else x * trapezoid of K_{5/3} on a 100-point log grid from x to 20 accumulated
// in float (each step promoted through double by the 0.5 literal).
float orc_ffunc_integrand(float x) {
  if (x < 1e-5) {
    return static_cast<float>(4.0 * M_PI / (std::sqrt(3.0) * std::tgamma(kOneThird)) *
                              std::pow(0.5 * x, 1.0 / 3.0));
  } else if (x > 20) {
    return 0.0f;
  }
  float xs[100], ys[100];
  for (int i = 0; i < 100; ++i) {
    xs[i] = logspace_point(x, 20.0f, 100, i);
    ys[i] = static_cast<float>(std::cyl_bessel_k(kFiveThird, static_cast<double>(xs[i])));
  }
  float integrand = 0.0f;
  for (int i = 0; i < 99; ++i) {
    integrand += 0.5 * (ys[i] + ys[i + 1]) * (xs[i + 1] - xs[i]);
  }
  return x * integrand;
}

// synchrotron.cpp:48-65 (TabulateFfunc).  `ys[i] > 100.0` reads a zeroed slot and is
// always false; `xs[i] < 1e-6` compares float against double, so the first node
// (float(1e-6) < 1e-6) gets y = 0.
void orc_tabulate_ffunc(std::int64_t npoints, float xmin, float xmax, float* xs, float* ys) {
  for (std::int64_t i = 0; i < npoints; ++i) {
    xs[i] = logspace_point(xmin, xmax, static_cast<std::size_t>(npoints), static_cast<std::size_t>(i));
    ys[i] = 0.0f;
  }
  for (std::int64_t i = 0; i < npoints; ++i) {
    if (xs[i] < 1e-6 or ys[i] > 100.0) {
      ys[i] = 0.0f;
    } else {
      ys[i] = orc_ffunc_integrand(xs[i]);
    }
  }
}

float orc_interp_log_f32(float x0, const float* x, const float* y, std::int64_t n,
                         float xmin, float xmax, float yfill) {
  return interp_log_f32(x0, x, y, static_cast<std::size_t>(n), xmin, xmax, yfill);
}

double orc_interp_log_f64(double x0, const float* x, const float* y, std::int64_t n,
                          float xmin, float xmax) {
  return interp_log_f64(x0, x, y, static_cast<std::size_t>(n), xmin, xmax);
}

// synchrotron.cpp:107-145 + synchrotron.hpp:145-172: MDRange over (particle, bin);
// every eval recomputes the kinematics (FP64, rounded to float), forms
// x0 = e/e_peak in float, interpolates in float and adds e*chiR*F into a per-thread
// float duplicate; duplicates are summed at the end.  w (optional) multiplies
// the term; the reference has no weight (w = 1).
void orc_sync_spectrum_ref32(const float* ux, const float* uy, const float* uz,
                             const float* ex, const float* ey, const float* ez,
                             const float* bx, const float* by, const float* bz,
                             const float* w, std::int64_t n,
                             const float* bins, std::int64_t nbins,
                             float B0, float g_syn, float eps,
                             const float* tx, const float* ty, std::int64_t nt,
                             float* out, int nthreads) {
  const int   nth  = threads_or_default(nthreads);
  const float xmin = *std::min_element(tx, tx + nt);
  const float xmax = *std::max_element(tx, tx + nt);
  std::vector<float> dup(static_cast<std::size_t>(nth) * nbins, 0.0f);
#pragma omp parallel for collapse(2) schedule(static) num_threads(nth)
  for (std::int64_t p = 0; p < n; ++p) {
    for (std::int64_t e = 0; e < nbins; ++e) {
      const float e_syn = bins[e];
      float       e_peak, chiR;
      omega_chi_ref(ux[p], uy[p], uz[p], comp(ex, p), comp(ey, p), comp(ez, p),
                    bx[p], by[p], bz[p], B0, g_syn, eps, e_peak, chiR);
      if (e_peak > 0.0) {
        const float F = interp_log_f32(e_syn / e_peak, tx, ty, nt, xmin, xmax, 0.0f);
        float       v = e_syn * chiR * F;
        if (w) {
          v *= w[p];
        }
        dup[static_cast<std::size_t>(omp_get_thread_num()) * nbins + e] += v;
      }
    }
  }
  for (std::int64_t e = 0; e < nbins; ++e) {
    out[e] = 0.0f;
  }
  for (int t = 0; t < nth; ++t) {
    for (std::int64_t e = 0; e < nbins; ++e) {
      out[e] += dup[static_cast<std::size_t>(t) * nbins + e];
    }
  }
}

// FP64 ground truth of the same spectrum: kinematics, x = e/e_peak, the lerp and
// the accumulation in double (per particle hoisted; the math is per eval).
void orc_sync_spectrum_f64(const float* ux, const float* uy, const float* uz,
                           const float* ex, const float* ey, const float* ez,
                           const float* bx, const float* by, const float* bz,
                           const float* w, std::int64_t n,
                           const float* bins, std::int64_t nbins,
                           float B0, float g_syn, float eps,
                           const float* tx, const float* ty, std::int64_t nt,
                           double* out, int nthreads) {
  const int    nth  = threads_or_default(nthreads);
  const double xmin = *std::min_element(tx, tx + nt);
  const double xmax = *std::max_element(tx, tx + nt);
  std::vector<double> dup(static_cast<std::size_t>(nth) * nbins, 0.0);
#pragma omp parallel num_threads(nth)
  {
    double* acc = dup.data() + static_cast<std::size_t>(omp_get_thread_num()) * nbins;
#pragma omp for schedule(static)
    for (std::int64_t p = 0; p < n; ++p) {
      double ep, ch;
      omega_chi_f64(ux[p], uy[p], uz[p], comp(ex, p), comp(ey, p), comp(ez, p),
                    bx[p], by[p], bz[p], B0, g_syn, eps, ep, ch);
      if (!(ep > 0.0)) {
        continue;
      }
      const double amp = ch * (w ? static_cast<double>(w[p]) : 1.0);
      for (std::int64_t e = 0; e < nbins; ++e) {
        const double es = bins[e];
        acc[e] += es * amp * interp_log_f64(es / ep, tx, ty, nt, xmin, xmax);
      }
    }
  }
  for (std::int64_t e = 0; e < nbins; ++e) {
    double s = 0.0;
    for (int t = 0; t < nth; ++t) {
      s += dup[static_cast<std::size_t>(t) * nbins + e];
    }
    out[e] = s;
  }
}

// Batched spectra over segments [off[s], off[s+1]) of one particle set, FP64.
void orc_sync_spectrum_batched_f64(const float* ux, const float* uy, const float* uz,
                                   const float* ex, const float* ey, const float* ez,
                                   const float* bx, const float* by, const float* bz,
                                   const float* w, const std::int64_t* off, std::int64_t nseg,
                                   const float* bins, std::int64_t nbins,
                                   float B0, float g_syn, float eps,
                                   const float* tx, const float* ty, std::int64_t nt,
                                   double* out, int nthreads) {
  for (std::int64_t s = 0; s < nseg; ++s) {
    const std::int64_t a = off[s];
    auto               sh = [a](const float* q) { return q ? q + a : nullptr; };
    orc_sync_spectrum_f64(sh(ux), sh(uy), sh(uz), sh(ex), sh(ey), sh(ez), sh(bx), sh(by),
                          sh(bz), sh(w), off[s + 1] - a, bins, nbins, B0, g_syn, eps, tx,
                          ty, nt, out + s * nbins, nthreads);
  }
}

// particles.cpp:189-260 (energyDistribution).  Index math in double except
// log10(emax/emin), which is float; out-of-range energies clamp into bins 0 and
// n-1; log-spaced bins add float(1.0/energy), linear bins add 1.  hist_ref32 uses
// per-thread float duplicates like the reference; hist_f64 sums in double; counts
// are exact.  Any output pointer may be null.
static std::size_t energy_bin_index_usqr(float Usqr, bool fourvel, float emin, float emax,
                                         std::size_t n, double& energy) {
  energy = fourvel ? static_cast<double>(std::sqrt(Usqr)) : std::sqrt(1.0 + Usqr);
  if (energy < emin) {
    return 0;
  } else if (energy >= emax) {
    return n - 1;
  }
  const auto ei = static_cast<std::size_t>(static_cast<float>(n - 1) *
                                           std::fabs(std::log10(energy / emin)) /
                                           std::log10(emax / emin));
  return ei > n - 1 ? n - 1 : ei;
}

static std::size_t energy_bin_index(float ux, float uy, float uz, bool fourvel, float emin,
                                    float emax, std::size_t n, double& energy) {
  const float Usqr = ux * ux + uy * uy + uz * uz;
  return energy_bin_index_usqr(Usqr, fourvel, emin, emax, n, energy);
}

std::int64_t orc_energy_bin_index_usqr(float Usqr, int fourvel, float emin, float emax,
                                       std::int64_t n) {
  double energy;
  return static_cast<std::int64_t>(
    energy_bin_index_usqr(Usqr, fourvel != 0, emin, emax, static_cast<std::size_t>(n), energy));
}

std::int64_t orc_energy_bin_index(float ux, float uy, float uz, int fourvel, float emin,
                                  float emax, std::int64_t n) {
  double energy;
  return static_cast<std::int64_t>(
    energy_bin_index(ux, uy, uz, fourvel != 0, emin, emax, static_cast<std::size_t>(n), energy));
}

void orc_energy_distribution(const float* ux, const float* uy, const float* uz, std::int64_t n,
                             const float* bins, std::int64_t nbins, int log_spaced, int fourvel,
                             float* hist_ref32, double* hist_f64, std::int64_t* counts,
                             int nthreads) {
  const int   nth  = threads_or_default(nthreads);
  float       emin = std::numeric_limits<float>::max();
  float       emax = std::numeric_limits<float>::lowest();
  for (std::int64_t i = 0; i < nbins; ++i) {
    emin = std::min(emin, bins[i]);
    emax = std::max(emax, bins[i]);
  }
  std::vector<float>        d32(static_cast<std::size_t>(nth) * nbins, 0.0f);
  std::vector<double>       d64(static_cast<std::size_t>(nth) * nbins, 0.0);
  std::vector<std::int64_t> dct(static_cast<std::size_t>(nth) * nbins, 0);
#pragma omp parallel num_threads(nth)
  {
    const std::size_t t = static_cast<std::size_t>(omp_get_thread_num()) * nbins;
#pragma omp for schedule(static)
    for (std::int64_t p = 0; p < n; ++p) {
      double      energy;
      std::size_t idx = energy_bin_index(ux[p], uy[p], uz[p], fourvel != 0, emin, emax,
                                         static_cast<std::size_t>(nbins), energy);
      if (log_spaced) {
        d32[t + idx] += static_cast<float>(1.0 / energy);
        d64[t + idx] += static_cast<double>(static_cast<float>(1.0 / energy));
      } else {
        d32[t + idx] += 1.0f;
        d64[t + idx] += 1.0;
      }
      dct[t + idx] += 1;
    }
  }
  for (std::int64_t e = 0; e < nbins; ++e) {
    float        s32 = 0.0f;
    double       s64 = 0.0;
    std::int64_t c   = 0;
    for (int t = 0; t < nth; ++t) {
      s32 += d32[static_cast<std::size_t>(t) * nbins + e];
      s64 += d64[static_cast<std::size_t>(t) * nbins + e];
      c += dct[static_cast<std::size_t>(t) * nbins + e];
    }
    if (hist_ref32) hist_ref32[e] = s32;
    if (hist_f64) hist_f64[e] = s64;
    if (counts) counts[e] = c;
  }
}

// synchrotron.cpp:69-105 + synchrotron.hpp:72-95 (FromDist): per (gamma bin,
// photon bin): e_peak = eps*gb*gb/(g*g) in float; S[e] += f*e*gb*F (log-spaced
// gamma bins) or f*e*F (linear).  ndist distributions share the gamma bins: f is
// [ndist x ng] row-major, out is [ndist x nbins].
void orc_sync_from_dist_ref32(const float* gb, const float* f, std::int64_t ng,
                              std::int64_t ndist, int log_spaced, const float* bins,
                              std::int64_t nbins, float g_syn, float eps, const float* tx,
                              const float* ty, std::int64_t nt, float* out, int nthreads) {
  const int   nth  = threads_or_default(nthreads);
  const float xmin = *std::min_element(tx, tx + nt);
  const float xmax = *std::max_element(tx, tx + nt);
  for (std::int64_t d = 0; d < ndist; ++d) {
    const float*       fd = f + d * ng;
    std::vector<float> dup(static_cast<std::size_t>(nth) * nbins, 0.0f);
#pragma omp parallel for collapse(2) schedule(static) num_threads(nth)
    for (std::int64_t g = 0; g < ng; ++g) {
      for (std::int64_t e = 0; e < nbins; ++e) {
        const float e_syn  = bins[e];
        const float gbeta  = gb[g];
        const float fp     = fd[g];
        const float e_peak = eps * gbeta * gbeta / (g_syn * g_syn);
        if (e_peak > 0.0) {
          const float F   = interp_log_f32(e_syn / e_peak, tx, ty, nt, xmin, xmax, 0.0f);
          float&      acc = dup[static_cast<std::size_t>(omp_get_thread_num()) * nbins + e];
          if (log_spaced) {
            acc += fp * e_syn * gbeta * F;
          } else {
            acc += fp * e_syn * F;
          }
        }
      }
    }
    for (std::int64_t e = 0; e < nbins; ++e) {
      float s = 0.0f;
      for (int t = 0; t < nth; ++t) {
        s += dup[static_cast<std::size_t>(t) * nbins + e];
      }
      out[d * nbins + e] = s;
    }
  }
}

void orc_sync_from_dist_f64(const float* gb, const float* f, std::int64_t ng,
                            std::int64_t ndist, int log_spaced, const float* bins,
                            std::int64_t nbins, float g_syn, float eps, const float* tx,
                            const float* ty, std::int64_t nt, double* out, int nthreads) {
  const int    nth  = threads_or_default(nthreads);
  const double xmin = *std::min_element(tx, tx + nt);
  const double xmax = *std::max_element(tx, tx + nt);
  // K[e][g] = e * J_g * F(e / e_peak(g)), shared by all distributions
  std::vector<double> K(static_cast<std::size_t>(nbins) * ng, 0.0);
#pragma omp parallel for schedule(static) num_threads(nth)
  for (std::int64_t e = 0; e < nbins; ++e) {
    for (std::int64_t g = 0; g < ng; ++g) {
      const double gbeta  = gb[g];
      const double e_peak = static_cast<double>(eps) * gbeta * gbeta /
                            (static_cast<double>(g_syn) * g_syn);
      if (e_peak > 0.0) {
        const double es = bins[e];
        K[e * ng + g]   = es * (log_spaced ? gbeta : 1.0) *
                        interp_log_f64(es / e_peak, tx, ty, nt, xmin, xmax);
      }
    }
  }
#pragma omp parallel for schedule(static) num_threads(nth)
  for (std::int64_t d = 0; d < ndist; ++d) {
    for (std::int64_t e = 0; e < nbins; ++e) {
      double s = 0.0;
      for (std::int64_t g = 0; g < ng; ++g) {
        s += K[e * ng + g] * static_cast<double>(f[d * ng + g]);
      }
      out[d * nbins + e] = s;
    }
  }
}

// ---------------------------------------------------------------------------------
// Differentiable ("smooth") mode.  F on [xmin, xmax) is the C1 cubic Hermite
// interpolant in t = (ln x - ln xmin)/dln through nodes x_j = xmin e^{j dln} with
// values F(x_j) = x_j int_{x_j}^inf K_{5/3} and slopes dF/dln x = F - x^2 K_{5/3}(x)
// (so F'(x) = F/x - x K_{5/3}); zero outside, like the reference table's support.
// Segment j in tau = t - j: F = c0 + tau (c1 + tau (c2 + tau c3)).
// ---------------------------------------------------------------------------------

namespace {

  // Gauss-Legendre nodes/weights on [-1, 1] (Newton on P_n).
  void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
      double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; ++k) {
          const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0              = p1;
          p1              = p2;
        }
        const double dp = n * (z * p1 - p0) / (z * z - 1.0);
        const double dz = p1 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-16) {
          break;
        }
      }
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0              = p1;
        p1              = p2;
      }
      const double dp = n * (z * p1 - p0) / (z * z - 1.0);
      x[i]            = z;
      w[i]            = 2.0 / ((1.0 - z * z) * dp * dp);
    }
  }

  // F(x) = x int_x^inf K_{5/3}(t) dt with t = x e^v (dt = t dv), v in [0, ln(60/x)],
  // 96 panels x 16-point Gauss-Legendre, K from std::cyl_bessel_k.
  struct GaussLegendre16 {
    std::vector<double> x, w;

    GaussLegendre16() {
      gauss_legendre(16, x, w);
    }
  };

  double exact_F_oracle(double x) {
    // function-local static: initialised once, thread-safely, before first use
    static const GaussLegendre16 gl;
    const std::vector<double>&   gx = gl.x;
    const std::vector<double>&   gw = gl.w;
    const double V = std::log(std::max(60.0, 2.0 * x) / x) + 1.0;
    const int    P = 96;
    double       s = 0.0;
    for (int p = 0; p < P; ++p) {
      const double a = V * p / P, b = V * (p + 1) / P, h = 0.5 * (b - a), c = 0.5 * (a + b);
      for (int i = 0; i < 16; ++i) {
        const double v = c + h * gx[i];
        const double t = x * std::exp(v);
        s += gw[i] * h * t * std::cyl_bessel_k(kFiveThird, t);
      }
    }
    return x * s;
  }

  struct SmoothTable {
    const float* c; // nseg x 4
    int64_t      nseg;
    double       ln_xmin, dln;
  };

  // F and dF/dln x of the Hermite interpolant at ln x (0 outside the support).
  inline void smooth_eval(const SmoothTable& T, double lnx, double& F, double& dF) {
    const double t = (lnx - T.ln_xmin) / T.dln;
    F = dF = 0.0;
    if (!(t >= 0.0) || !(t < static_cast<double>(T.nseg))) {
      return;
    }
    const int64_t j   = static_cast<int64_t>(t);
    const double  tau = t - static_cast<double>(j);
    const double  c0 = T.c[4 * j], c1 = T.c[4 * j + 1], c2 = T.c[4 * j + 2], c3 = T.c[4 * j + 3];
    F  = c0 + tau * (c1 + tau * (c2 + tau * c3));
    dF = (c1 + tau * (2.0 * c2 + 3.0 * tau * c3)) / T.dln;
  }

  // chi_R, e_peak and their u-gradients (d ln chi / du, d ln e_peak / du) in double.
  struct Kin {
    double chi, lneps;
    double dlnchi[3], dlneps[3];
  };

  inline bool kinematics(const double u[3], const double E[3], const double B[3], double B0,
                         double g_syn, double eps, Kin& k) {
    const double G     = 1.0 + u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const double gamma = std::sqrt(G);
    const double c[3]  = { u[1] * B[2] - u[2] * B[1], u[2] * B[0] - u[0] * B[2],
                           u[0] * B[1] - u[1] * B[0] };
    const double V[3]  = { gamma * E[0] + c[0], gamma * E[1] + c[1], gamma * E[2] + c[2] };
    const double uE    = u[0] * E[0] + u[1] * E[1] + u[2] * E[2];
    const double W     = V[0] * V[0] + V[1] * V[1] + V[2] * V[2] - uE * uE;
    const double K0    = eps / (g_syn * g_syn * B0);
    if (!(W > 0.0) || !(K0 > 0.0)) {
      return false;
    }
    k.chi   = std::sqrt(W) / (gamma * B0);
    k.lneps = std::log(K0) + 0.5 * std::log(G) + 0.5 * std::log(W);
    // dW/du = (2 V.E / gamma) u + 2 B x V - 2 (u.E) E
    const double VE     = V[0] * E[0] + V[1] * E[1] + V[2] * E[2];
    const double BxV[3] = { B[1] * V[2] - B[2] * V[1], B[2] * V[0] - B[0] * V[2],
                            B[0] * V[1] - B[1] * V[0] };
    for (int d = 0; d < 3; ++d) {
      const double gW  = 2.0 * VE / gamma * u[d] + 2.0 * BxV[d] - 2.0 * uE * E[d];
      const double glG = 2.0 * u[d] / G;
      k.dlnchi[d]      = 0.5 * gW / W - 0.5 * glG;
      k.dlneps[d]      = 0.5 * glG + 0.5 * gW / W;
    }
    return true;
  }

  inline double dcomp(const double* p, std::int64_t i) {
    return p ? p[i] : 0.0;
  }

} // namespace

// Coefficients of the smooth table (nseg segments on [xmin, xmax)) in FP64 from
// std::cyl_bessel_k; coef is [nseg x 4].
void orc_smooth_coefficients(std::int64_t nseg, double xmin, double xmax, double* coef,
                             int nthreads) {
  const double        ln_xmin = std::log(xmin), dln = std::log(xmax / xmin) / nseg;
  std::vector<double> F(nseg + 1), D(nseg + 1);
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads_or_default(nthreads))
  for (std::int64_t j = 0; j <= nseg; ++j) {
    const double x = std::exp(ln_xmin + j * dln);
    F[j]           = exact_F_oracle(x);
    D[j]           = F[j] - x * x * std::cyl_bessel_k(kFiveThird, x);
  }
  for (std::int64_t j = 0; j < nseg; ++j) {
    coef[4 * j]     = F[j];
    coef[4 * j + 1] = D[j] * dln;
    coef[4 * j + 2] = 3.0 * (F[j + 1] - F[j]) - dln * (2.0 * D[j] + D[j + 1]);
    coef[4 * j + 3] = 2.0 * (F[j] - F[j + 1]) + dln * (D[j] + D[j + 1]);
  }
}

double orc_exact_F(double x) {
  return exact_F_oracle(x);
}

// Smooth-mode spectrum S[b] = e_b sum_p w_p chi_p F(e_b / e_peak_p) in FP64 for
// double particle data (any component pointer may be null = 0; w null = 1).
void orc_sync_smooth_f64(const double* ux, const double* uy, const double* uz, const double* ex,
                         const double* ey, const double* ez, const double* bx, const double* by,
                         const double* bz, const double* w, std::int64_t n, const float* bins,
                         std::int64_t nbins, double B0, double g_syn, double eps, const float* coef,
                         std::int64_t nseg, double ln_xmin, double dln, double* out, int nthreads) {
  const int           nth = threads_or_default(nthreads);
  const SmoothTable   T { coef, nseg, ln_xmin, dln };
  std::vector<double> dup(static_cast<std::size_t>(nth) * nbins, 0.0);
#pragma omp parallel num_threads(nth)
  {
    double* acc = dup.data() + static_cast<std::size_t>(omp_get_thread_num()) * nbins;
#pragma omp for schedule(static)
    for (std::int64_t p = 0; p < n; ++p) {
      const double u[3] = { ux[p], uy[p], uz[p] };
      const double E[3] = { dcomp(ex, p), dcomp(ey, p), dcomp(ez, p) };
      const double B[3] = { dcomp(bx, p), dcomp(by, p), dcomp(bz, p) };
      Kin          k;
      if (!kinematics(u, E, B, B0, g_syn, eps, k)) {
        continue;
      }
      const double amp = k.chi * (w ? w[p] : 1.0);
      for (std::int64_t b = 0; b < nbins; ++b) {
        double F, dF;
        smooth_eval(T, std::log(static_cast<double>(bins[b])) - k.lneps, F, dF);
        acc[b] += static_cast<double>(bins[b]) * amp * F;
      }
    }
  }
  for (std::int64_t b = 0; b < nbins; ++b) {
    double s = 0.0;
    for (int t = 0; t < nth; ++t) {
      s += dup[static_cast<std::size_t>(t) * nbins + b];
    }
    out[b] = s;
  }
}

// Analytic gradient of L(S) given gS = dL/dS (nbins): dL/dw_p and dL/du_p of the
// smooth-mode spectrum, in FP64.  gw / gu* may be null.
void orc_sync_smooth_grad_f64(const double* ux, const double* uy, const double* uz,
                              const double* ex, const double* ey, const double* ez,
                              const double* bx, const double* by, const double* bz,
                              const double* w, std::int64_t n, const float* bins,
                              std::int64_t nbins, double B0, double g_syn, double eps,
                              const float* coef, std::int64_t nseg, double ln_xmin, double dln,
                              const double* gS, double* gw, double* gux, double* guy, double* guz,
                              int nthreads) {
  const SmoothTable T { coef, nseg, ln_xmin, dln };
#pragma omp parallel for schedule(static) num_threads(threads_or_default(nthreads))
  for (std::int64_t p = 0; p < n; ++p) {
    const double u[3] = { ux[p], uy[p], uz[p] };
    const double E[3] = { dcomp(ex, p), dcomp(ey, p), dcomp(ez, p) };
    const double B[3] = { dcomp(bx, p), dcomp(by, p), dcomp(bz, p) };
    Kin          k;
    double       g[3] = { 0.0, 0.0, 0.0 }, gwp = 0.0;
    if (kinematics(u, E, B, B0, g_syn, eps, k)) {
      double R1 = 0.0, R2 = 0.0;
      for (std::int64_t b = 0; b < nbins; ++b) {
        double F, dF;
        smooth_eval(T, std::log(static_cast<double>(bins[b])) - k.lneps, F, dF);
        const double ge = gS[b] * static_cast<double>(bins[b]);
        R1 += ge * F;
        R2 += ge * dF;
      }
      const double wp  = w ? w[p] : 1.0;
      const double amp = k.chi * wp;
      gwp              = k.chi * R1;
      for (int d = 0; d < 3; ++d) {
        g[d] = amp * (R1 * k.dlnchi[d] - R2 * k.dlneps[d]);
      }
    }
    if (gw) gw[p] = gwp;
    if (gux) gux[p] = g[0];
    if (guy) guy[p] = g[1];
    if (guz) guz[p] = g[2];
  }
}

} // extern "C"

// ---- inverse Compton (physics/ic.hpp:20-95, physics/ic.cpp:15-46) ----------------------

namespace {

  // ic.hpp:20-25 (KNfunc) with the reference's type promotions: 2 q log(q) in float
  // (logf), 0.5 Gq Gq / (1 + Gq) in double (0.5 is a double literal), the whole
  // expression in double, returned as float.
  float ic_kn_ref32(float Gamma, float q) {
    const float  Gq    = Gamma * q;
    const float  a     = 2 * q * std::log(q);
    const double inner = static_cast<double>(1 + 2 * q) + 0.5 * Gq * Gq / static_cast<double>(1 + Gq);
    return static_cast<float>(static_cast<double>(a) + static_cast<double>(1 - q) * inner);
  }

  double ic_kn_f64(double Gamma, double q) {
    const double Gq = Gamma * q;
    return 2.0 * q * std::log(q) + (1.0 - q) * ((1.0 + 2.0 * q) + 0.5 * Gq * Gq / (1.0 + Gq));
  }

} // namespace

extern "C" {

// ic.cpp:15-46: MDRange (gamma bin, soft-photon bin, IC bin) running ic::Kernel
// (ic.hpp:67-94) into a ScatterView; float arithmetic as the reference writes it,
// OpenMP static schedule over the collapsed index space with per-thread copies
// summed in thread order (the Kokkos-API shim's ScatterDuplicated behaviour).
void orc_ic_spectrum_ref32(const float* gb, const float* fp, std::int64_t ng, int log_spaced,
                           const float* es, const float* fs, std::int64_t ns, const float* eic,
                           std::int64_t ne, float* out, int nthreads) {
  const int          nth = threads_or_default(nthreads);
  std::vector<float> dup(static_cast<std::size_t>(nth) * ne, 0.0f);
#pragma omp parallel for collapse(3) schedule(static) num_threads(nth)
  for (std::int64_t g = 0; g < ng; ++g) {
    for (std::int64_t s = 0; s < ns; ++s) {
      for (std::int64_t e = 0; e < ne; ++e) {
        const float g_prtls = gb[g], f_prtls = fp[g];
        const float e_soft = es[s], f_soft = fs[s];
        const float e_ic   = eic[e];
        const float Gamma  = 4 * g_prtls * e_soft;
        if (e_ic > g_prtls * Gamma / (1 + Gamma)) {
          continue;
        }
        const float q  = (e_ic / g_prtls) / (Gamma * (1 - (e_ic / g_prtls)));
        const float kn = ic_kn_ref32(Gamma, q);
        const float v  = log_spaced ? f_prtls * (f_soft / e_soft) * e_ic * e_ic * kn / g_prtls
                                    : f_prtls * (f_soft / e_soft) * e_ic * e_ic * kn / (g_prtls * g_prtls);
        dup[static_cast<std::size_t>(omp_get_thread_num()) * ne + e] += v;
      }
    }
  }
  for (std::int64_t e = 0; e < ne; ++e) {
    float acc = 0.0f;
    for (int t = 0; t < nth; ++t) {
      acc += dup[static_cast<std::size_t>(t) * ne + e];
    }
    out[e] = acc;
  }
}

// FP64 ground truth of the same sum (inputs are the float arrays).
void orc_ic_spectrum_f64(const float* gb, const float* fp, std::int64_t ng, int log_spaced,
                         const float* es, const float* fs, std::int64_t ns, const float* eic,
                         std::int64_t ne, double* out, int nthreads) {
  const int nth = threads_or_default(nthreads);
#pragma omp parallel for schedule(static) num_threads(nth)
  for (std::int64_t e = 0; e < ne; ++e) {
    const double e_ic = eic[e];
    double       acc  = 0.0;
    for (std::int64_t g = 0; g < ng; ++g) {
      const double g_prtls = gb[g], f_prtls = fp[g];
      for (std::int64_t s = 0; s < ns; ++s) {
        const double e_soft = es[s], f_soft = fs[s];
        const double Gamma  = 4.0 * g_prtls * e_soft;
        if (e_ic > g_prtls * Gamma / (1.0 + Gamma)) {
          continue;
        }
        const double r  = e_ic / g_prtls;
        const double q  = r / (Gamma * (1.0 - r));
        const double kn = ic_kn_f64(Gamma, q);
        acc += f_prtls * (f_soft / e_soft) * e_ic * e_ic * kn / (log_spaced ? g_prtls : g_prtls * g_prtls);
      }
    }
    out[e] = acc;
  }
}

} // extern "C"

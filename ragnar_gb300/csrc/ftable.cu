// Synchrotron kernel tables, built on the GPU in FP64.
//
// K_{5/3}(x) uses the integral representation
//     K_nu(x) = int_0^inf exp(-x cosh s) cosh(nu s) ds
// and F(x) = x int_x^inf K_{5/3}(t) dt the (exchanged-order) representation
//     F(x) = x int_0^inf exp(-x cosh s) cosh(5 s / 3) / cosh(s) ds,
// both evaluated with the trapezoidal rule after factoring out exp(-x):
//     int_0^inf g(s) ds,  g(s) = exp(-x (cosh s - 1)) cosh(5 s / 3) [/ cosh s].
// g is even and entire; on the strip |Im s| <= y it is bounded by
// exp(x y^2 / 2) times its real-axis size, so the trapezoidal error is about
// exp(x y^2/2 - 2 pi y / h).  With h = min(1/8, 1/(2 sqrt x)) the best y gives an
// error below exp(-79) relative, far under double rounding, for every x > 0.
#include "rg_common.cuh"
#include "rg_internal.hpp"

#include <algorithm>
#include <cmath>
#include <vector>

namespace rg {

  namespace {

    constexpr double kFiveThird = 1.6666666666666667;

    // Shared quadrature: exp(-x) * h * sum_k' g(k h), p = 1 adds the 1/cosh s
    // factor.  Stops once x (cosh s - 1) - 5 s / 3 > 45: later terms are below
    // e^-45 of g(0) = 1 and decay doubly exponentially.
    __host__ __device__ double cosh_quad(double x, int p) {
      const double h   = fmin(0.125, 0.5 / sqrt(x));
      double       sum = 0.5; // g(0) with the trapezoid end weight 1/2
      for (int k = 1; k < 100000; ++k) {
        const double s  = k * h;
        const double sh = sinh(0.5 * s);
        const double a  = 2.0 * x * sh * sh; // x (cosh s - 1) without cancellation
        double       term = exp(-a) * cosh(kFiveThird * s);
        if (p == 1) {
          term /= cosh(s);
        }
        sum += term;
        if (a - kFiveThird * s > 45.0 || s > 400.0) {
          break;
        }
      }
      return exp(-x) * sum * h;
    }

  } // namespace

  __host__ __device__ double bessel_k53(double x) {
    return cosh_quad(x, 0);
  }

  __host__ __device__ double exact_F(double x) {
    return x * cosh_quad(x, 1);
  }

  namespace {

    constexpr int kInner = 100; // inner grid points of Ffunc_integrand (synchrotron.cpp:35)

    // Inner grids Logspace(x, 20, 100) of every x in [1e-5, 20], computed on the
    // host: they are float results of the platform's log10f and pow, exactly as
    // the reference computes them (log10f is not correctly rounded, so a GPU
    // evaluation would move some grid points by one ulp).
    std::vector<float> inner_grids(const std::vector<float>& xs) {
      std::vector<float> g(xs.size() * kInner, 0.0f);
      for (std::size_t i = 0; i < xs.size(); ++i) {
        const float x = xs[i];
        if (static_cast<double>(x) >= 1e-5 && !(x > 20.0f)) {
          for (int j = 0; j < kInner; ++j) {
            g[i * kInner + j] = logspace_point(x, 20.0f, kInner, j);
          }
        }
      }
      return g;
    }

    // Ffunc_integrand (synchrotron.cpp:28-46), one warp per x: the lanes evaluate
    // K_{5/3} in FP64 on the 100-point inner grid, lane 0 accumulates the
    // trapezoid in the reference's order (float accumulator, each step through
    // double).
    __global__ void ffunc_integrand_kernel(const float* __restrict__ x,
                                           const float* __restrict__ grids, int64_t n,
                                           float* __restrict__ y, int zero_below_1em6) {
      __shared__ float xs_s[4][kInner];
      __shared__ float ys_s[4][kInner];
      const int     wib  = threadIdx.x >> 5;
      const int     lane = threadIdx.x & 31;
      const int64_t i    = static_cast<int64_t>(blockIdx.x) * 4 + wib;
      if (i >= n) {
        return;
      }
      const float xi = x[i];
      float       out;
      if (zero_below_1em6 && static_cast<double>(xi) < 1e-6) {
        out = 0.0f; // TabulateFfunc (synchrotron.cpp:58): xs[i] < 1e-6 -> 0
      } else if (static_cast<double>(xi) < 1e-5) {
        out = __double2float_rn(4.0 * M_PI / (sqrt(3.0) * tgamma(0.3333333333333333)) *
                                pow(0.5 * static_cast<double>(xi), 1.0 / 3.0));
      } else if (xi > 20.0f) {
        out = 0.0f;
      } else {
        for (int j = lane; j < kInner; j += 32) {
          const float xj = grids[i * kInner + j];
          xs_s[wib][j]   = xj;
          ys_s[wib][j]   = __double2float_rn(bessel_k53(static_cast<double>(xj)));
        }
        __syncwarp();
        float integrand = 0.0f;
        if (lane == 0) {
          for (int j = 0; j < 99; ++j) {
            const float  ysum = __fadd_rn(ys_s[wib][j], ys_s[wib][j + 1]);
            const float  dx   = __fsub_rn(xs_s[wib][j + 1], xs_s[wib][j]);
            const double term = 0.5 * static_cast<double>(ysum) * static_cast<double>(dx);
            integrand = __double2float_rn(__dadd_rn(static_cast<double>(integrand), term));
          }
        }
        out = __fmul_rn(xi, integrand);
      }
      if (lane == 0) {
        y[i] = out;
      }
    }

    // Segment coefficients of the reference table.  For segment i the reference
    // interpolates linearly in log10 x between its actual float nodes
    // (tabulation.hpp:39-41); written in the ideal coordinate t = (ln x - ln xmin)/dln
    // that is F = c0 + (t - i) c1 with
    //   beta = (y[i+1] - y[i]) / log10(x[i+1]/x[i]),
    //   c0   = y[i] + beta * (log10 xmin + i dln/ln10 - log10 x[i]),  c1 = beta dln/ln10.
    __global__ void ref_coef_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                    int n, double ln_xmin, double dln, float2* __restrict__ coef) {
      const int i = blockIdx.x * blockDim.x + threadIdx.x;
      if (i >= kRefEntries) {
        return;
      }
      float2 c = make_float2(0.0f, 0.0f);
      if (i < n - 1) {
        const double xa = x[i], xb = x[i + 1], ya = y[i], yb = y[i + 1];
        const double d10  = dln / M_LN10;
        const double beta = (yb - ya) / log10(xb / xa);
        const double c0   = ya + beta * (ln_xmin / M_LN10 + i * d10 - log10(xa));
        const double c1   = beta * d10;
        c                 = make_float2(__double2float_rn(c0), __double2float_rn(c1 * kSlopeScale));
      }
      coef[i] = c;
    }

    // Smooth table: nodes s_j = ln xmin + j*dln (j = 0..N), F_j = exact F and
    // D_j = dF/dln x = F_j - x_j^2 K_{5/3}(x_j); cubic Hermite on each segment in
    // tau = t - j: c0 = F_j, c1 = D_j dln, c2 = 3(F_{j+1}-F_j) - dln(2D_j + D_{j+1}),
    // c3 = 2(F_j - F_{j+1}) + dln(D_j + D_{j+1}).
    __global__ void smooth_nodes_kernel(int nnodes, double ln_xmin, double dln,
                                        double2* __restrict__ nodes) {
      const int j = blockIdx.x * blockDim.x + threadIdx.x;
      if (j >= nnodes) {
        return;
      }
      const double xj = exp(ln_xmin + j * dln);
      const double F  = exact_F(xj);
      const double D  = F - xj * xj * bessel_k53(xj);
      nodes[j]        = make_double2(F, D);
    }

    __global__ void smooth_coef_kernel(const double2* __restrict__ nodes, int nseg, double dln,
                                       float4* __restrict__ coef) {
      const int j = blockIdx.x * blockDim.x + threadIdx.x;
      if (j >= nseg) {
        return;
      }
      const double F0 = nodes[j].x, D0 = nodes[j].y, F1 = nodes[j + 1].x, D1 = nodes[j + 1].y;
      const double c0 = F0, c1 = D0 * dln;
      const double c2 = 3.0 * (F1 - F0) - dln * (2.0 * D0 + D1);
      const double c3 = 2.0 * (F0 - F1) + dln * (D0 + D1);
      coef[j] = make_float4(__double2float_rn(c0), __double2float_rn(c1), __double2float_rn(c2),
                            __double2float_rn(c3));
    }

  } // namespace

  int build_reference_table(int n, float xmin, float xmax, RefTable& t, cudaStream_t s) {
    if (n < 2) {
      return set_error(RG_ERR_ARGUMENT, "TabulateFfunc needs at least 2 points");
    }
    t.n = n;
    t.h_x.resize(n);
    for (int i = 0; i < n; ++i) {
      t.h_x[i] = logspace_point(xmin, xmax, static_cast<std::size_t>(n), static_cast<std::size_t>(i));
    }
    // TabulatedFunction::findMinMax (tabulation.cpp:84-102)
    t.xmin = t.h_x[0];
    t.xmax = t.h_x[0];
    for (float v : t.h_x) {
      t.xmin = std::min(t.xmin, v);
      t.xmax = std::max(t.xmax, v);
    }
    t.ln_xmin = std::log(static_cast<double>(t.xmin));
    t.dln     = std::log(static_cast<double>(t.xmax) / static_cast<double>(t.xmin)) / (n - 1);
    RG_CUDA_TRY(cudaMalloc(&t.d_x, sizeof(float) * n));
    RG_CUDA_TRY(cudaMalloc(&t.d_y, sizeof(float) * n));
    RG_CUDA_TRY(cudaMalloc(&t.d_coef, sizeof(float2) * kRefEntries));
    RG_CUDA_TRY(cudaMemcpyAsync(t.d_x, t.h_x.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    const std::vector<float> grids = inner_grids(t.h_x);
    ScratchBuffer<float>     d_grids;
    RG_CUDA_TRY(cudaMalloc(&d_grids.p, sizeof(float) * grids.size()));
    RG_CUDA_TRY(cudaMemcpyAsync(d_grids.p, grids.data(), sizeof(float) * grids.size(),
                                cudaMemcpyHostToDevice, s));
    ffunc_integrand_kernel<<<(n + 3) / 4, 128, 0, s>>>(t.d_x, d_grids.p, n, t.d_y, 1);
    RG_CUDA_TRY(cudaGetLastError());
    RG_CUDA_TRY(cudaStreamSynchronize(s));
    ref_coef_kernel<<<kRefEntries / 256, 256, 0, s>>>(t.d_x, t.d_y, n, t.ln_xmin, t.dln, t.d_coef);
    RG_CUDA_TRY(cudaGetLastError());
    t.h_y.resize(n);
    RG_CUDA_TRY(cudaMemcpyAsync(t.h_y.data(), t.d_y, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    RG_CUDA_TRY(cudaStreamSynchronize(s));
    return RG_OK;
  }

  // The reference table built into caller-supplied device buffers (x, y: n floats;
  // coef: kRefEntries float2; grids: n * 100 floats) without allocating; used by
  // the allocation-free spectrum.  Synchronises `s`.
  int build_reference_table_into(int n, float xmin, float xmax, float* d_x, float* d_y, float2* d_coef,
                                 float* d_grids, double& ln_xmin, double& dln, cudaStream_t s) {
    if (n < 2) {
      return set_error(RG_ERR_ARGUMENT, "TabulateFfunc needs at least 2 points");
    }
    std::vector<float> hx(n);
    for (int i = 0; i < n; ++i) {
      hx[i] = logspace_point(xmin, xmax, static_cast<std::size_t>(n), static_cast<std::size_t>(i));
    }
    const float lo = *std::min_element(hx.begin(), hx.end());
    const float hi = *std::max_element(hx.begin(), hx.end());
    ln_xmin        = std::log(static_cast<double>(lo));
    dln            = std::log(static_cast<double>(hi) / static_cast<double>(lo)) / (n - 1);
    const std::vector<float> grids = inner_grids(hx);
    RG_CUDA_TRY(cudaMemcpyAsync(d_x, hx.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    RG_CUDA_TRY(cudaMemcpyAsync(d_grids, grids.data(), sizeof(float) * grids.size(), cudaMemcpyHostToDevice, s));
    ffunc_integrand_kernel<<<(n + 3) / 4, 128, 0, s>>>(d_x, d_grids, n, d_y, 1);
    RG_CUDA_TRY(cudaGetLastError());
    ref_coef_kernel<<<kRefEntries / 256, 256, 0, s>>>(d_x, d_y, n, ln_xmin, dln, d_coef);
    RG_CUDA_TRY(cudaGetLastError());
    RG_CUDA_TRY(cudaStreamSynchronize(s));
    return RG_OK;
  }

  int build_smooth_table(SmoothTable& t, cudaStream_t s) {
    return build_smooth_table_geom(t, std::log(kSmoothXmin), std::log(kSmoothXmax / kSmoothXmin) / kSmoothSegments,
                                   kSmoothSegments, s);
  }

  int build_smooth_table_geom(SmoothTable& t, double ln_xmin, double dln, int nseg, cudaStream_t s) {
    if (nseg < 1 || nseg > kSmoothMaxSegments || !(dln > 0.0)) {
      return set_error(RG_ERR_ARGUMENT, "smooth table: bad geometry");
    }
    t.ln_xmin = ln_xmin;
    t.dln     = dln;
    t.nseg    = nseg;
    ScratchBuffer<double2> nodes;
    RG_CUDA_TRY(cudaMalloc(&nodes.p, sizeof(double2) * (nseg + 1)));
    RG_CUDA_TRY(cudaMalloc(&t.d_coef, sizeof(float4) * (nseg + 1)));
    RG_CUDA_TRY(cudaMemsetAsync(t.d_coef + nseg, 0, sizeof(float4), s));
    smooth_nodes_kernel<<<(nseg + 1 + 127) / 128, 128, 0, s>>>(nseg + 1, t.ln_xmin, t.dln, nodes.p);
    RG_CUDA_TRY(cudaGetLastError());
    smooth_coef_kernel<<<(nseg + 127) / 128, 128, 0, s>>>(nodes.p, nseg, t.dln, t.d_coef);
    RG_CUDA_TRY(cudaGetLastError());
    RG_CUDA_TRY(cudaStreamSynchronize(s));
    return RG_OK;
  }

} // namespace rg

extern "C" {

namespace rg {
  namespace {
    // x (device, n) -> y (device, n); `zero_first` applies TabulateFfunc's
    // x < 1e-6 rule.  Synchronises `s`.
    int ffunc_eval(const float* x, int64_t n, float* y, int zero_first, cudaStream_t s) {
      std::vector<float> hx(static_cast<std::size_t>(n));
      RG_CUDA_TRY(cudaMemcpyAsync(hx.data(), x, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
      RG_CUDA_TRY(cudaStreamSynchronize(s));
      const std::vector<float> grids = inner_grids(hx);
      ScratchBuffer<float>     d_grids;
      RG_CUDA_TRY(cudaMalloc(&d_grids.p, sizeof(float) * grids.size()));
      RG_CUDA_TRY(cudaMemcpyAsync(d_grids.p, grids.data(), sizeof(float) * grids.size(),
                                  cudaMemcpyHostToDevice, s));
      ffunc_integrand_kernel<<<static_cast<unsigned>((n + 3) / 4), 128, 0, s>>>(x, d_grids.p, n, y,
                                                                               zero_first);
      RG_CUDA_TRY(cudaGetLastError());
      // the host grids and the scratch must outlive the kernel
      RG_CUDA_TRY(cudaStreamSynchronize(s));
      return RG_OK;
    }
  } // namespace
} // namespace rg

int rg_ffunc_integrand(const float* x, int64_t n, float* y, void* stream) {
  if (n <= 0) {
    return RG_OK;
  }
  if ((n + 3) / 4 > 0x7fffffff) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_ffunc_integrand: n too large");
  }
  return rg::ffunc_eval(x, n, y, 0, static_cast<cudaStream_t>(stream));
}

int rg_ffunc_table(int64_t n, float xmin, float xmax, float* x, float* y, void* stream) {
  if (n < 1) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_ffunc_table: n must be >= 1");
  }
  std::vector<float> hx(static_cast<std::size_t>(n));
  RG_TRY(rg_logspace(xmin, xmax, n, hx.data()));
  auto s = static_cast<cudaStream_t>(stream);
  RG_CUDA_TRY(cudaMemcpyAsync(x, hx.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
  return rg::ffunc_eval(x, n, y, 1, s);
}

// Diagnostics: the FP64 quadratures evaluated on the host (same code as on the GPU).
double rg_debug_bessel_k53(double x) {
  return rg::bessel_k53(x);
}

double rg_debug_exact_F(double x) {
  return rg::exact_F(x);
}

} // extern "C"

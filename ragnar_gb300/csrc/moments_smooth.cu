// Differentiable (smooth-table) particle spectrum and its adjoint by cell moments.
//
// Reference path: SynchrotronSpectrum<D> (synchrotron.cpp:107-145) over
// sync::Kernel<D>::operator() (synchrotron.hpp:145-172); the smooth table is this
// library's own differentiable F (exact x int K_{5/3} at the nodes, C1 cubic
// Hermite in between; ftable.cu).
//
// For photon bins that are log-uniform (Logbins), a plan builds its own smooth
// table on a grid aligned to the bins: node spacing dln = (bin spacing) / m for an
// integer m, and nodes placed so that every bin's table coordinate t_b is an
// integer up to a tiny residual eps_b (float rounding of the bins; |eps_b| < 1e-3
// segments).  With x = e_b / e_peak, t = t_b - q_p, q_p = ln e_peak_p / dln, every
// bin then sees a particle at the same position inside a segment,
//   tau_p = frac(-q_p),   segment s = t_b - ceil(q_p),
// so with R = Pmax - Q (Q = q 2^F in fixed point, Pmax the largest bin coordinate)
// a particle's cell Rc = R >> F and tau = (R mod 2^F) 2^-F are the same for every
// bin, and bin b reads segment Rc - Dc_b (Dc_b = (Pmax >> F) - t_b).  The forward is
//   S_b / e_b = sum_cells sum_j c'_j(Rc - Dc_b) M_j(Rc),  M_j = sum_p A_p tau_p^j,
//   c'_j = c_j + eps_b (j + 1) c_{j+1}   (first order in eps_b: F(tau + eps)),
// four FP64 moments per cell (deposited into 32 slots per cell, which spreads the
// atomics of crowded cells, then folded), and the adjoint of a loss L with
// G_b = dL/dS_b is, per particle, the cubic of its cell
//   R1(tau) = sum_b G_b e_b F_b(tau) = sum_j alpha_j(Rc) tau^j,
//   alpha_j(c) = sum_b G_b e_b c'_j(c - Dc_b),   R2 = (dR1/dtau) / dln,
// from which particle_gradient forms dL/dw and dL/du.  Work: one particle stage per
// particle plus (cells x bins) in the forward and the adjoint, instead of
// (particles x bins) in each.
#include "moments_common.cuh"
#include "spectrum_plan.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

namespace rg {

  namespace {

    // Slots per cell: a particle adds its moments (which are absolute within the cell) to
    // the slot of its lane, shifted by its position in the cell, so the lanes of a warp
    // whose particles crowd one cell hit different addresses.
    constexpr int    kSub         = 32;
    constexpr int    kSubBits     = 5;
    constexpr int    kSmThreads   = 256;
    constexpr int    kSmSharedSeg = 1024;      // segment offsets staged in shared memory
    constexpr int    kSmRows      = 16;        // segment groups of the reduce kernel
    constexpr double kTargetDln   = 0.0089954; // ln(1e8) / 2048: the device-wide table's spacing
    constexpr size_t kSmSharedMax = 200 * 1024; // shared-memory cell table of the block-aggregated deposit
    // Largest bin residual |eps_b|, in table segments.  Logbins-style bins carry ~2e-6 in
    // ln e (their exponent is rounded to float before the power); the first-order
    // correction leaves eps^2 |F''| / 2 < 1e-6 F at this bound.
    constexpr double kUniformTol  = 1e-3;

    struct SmoothMomParams {
      FusedParams    fp;        // streams, kinematics constants (plan's frac), status
      int64_t        Pmin, Pmax, L;
      int            F;         // fraction bits of the coordinate (plan frac + 8)
      float          tau_scale; // 2^-F
      const int64_t* seg_off;   // nseg + 1 particle offsets (device), or null: particles [0, n)
      int            nseg;
      int64_t        n;
      int            nc;        // cells
      double*        hist;      // [nseg][nc][kSub][4]
    };

    // Stages and checks the segment offsets (as the interval-moment deposit does); false
    // for the whole block if they are bad or the status word is set.
    __device__ __forceinline__ bool stage_offsets(const SmoothMomParams& m, int64_t* soff) {
      bool bad = false;
      if (m.seg_off) {
        for (int i = threadIdx.x; i <= m.nseg; i += blockDim.x) {
          soff[i] = m.seg_off[i];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < m.nseg; i += blockDim.x) {
          bad = bad || soff[i + 1] < soff[i] || soff[i] < 0 || soff[i + 1] > m.n;
        }
      }
      if (__syncthreads_or(bad)) {
        if (threadIdx.x == 0 && blockIdx.x == 0) {
          atomicOr(m.fp.status, kDevBadOffsets);
        }
        return false;
      }
      return !__syncthreads_or(*m.fp.status != kDevOk);
    }

    __global__ void __launch_bounds__(kSmThreads) smooth_deposit_kernel(const __grid_constant__ SmoothMomParams m) {
      __shared__ int64_t soff[kSmSharedSeg + 1];
      if (!stage_offsets(m, soff)) {
        return;
      }
      const int64_t  first  = m.seg_off ? soff[0] : 0;
      const int64_t  last   = m.seg_off ? soff[m.nseg] : m.n;
      const int64_t  stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
      const uint32_t mask   = (1u << m.F) - 1u;
      const int64_t  i0     = first + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      // this thread's segment, advanced as its particle index grows
      int seg = m.seg_off ? segment_of(soff, m.nseg, i0) : 0;
      for (int64_t i = i0; i < last; i += stride) {
        if (m.seg_off) {
          while (seg < m.nseg && soff[seg + 1] <= i) {
            ++seg;
          }
        }
        float v[kComps];
#pragma unroll
        for (int c = 0; c < kComps; ++c) {
          v[c] = m.fp.comp[c] ? __ldg(m.fp.comp[c] + i) : 0.0f;
        }
        int64_t Q = 0;
        float   A = 0.0f;
        if (!moment_particle_stage(v, m.fp, m.Pmin, m.Pmax, m.L, Q, A)) {
          continue;
        }
        const uint64_t R   = static_cast<uint64_t>(m.Pmax - Q);
        const uint32_t Rc  = static_cast<uint32_t>(R >> m.F);
        const uint32_t Rl  = static_cast<uint32_t>(R) & mask;
        const int      sub = static_cast<int>(((Rl >> (m.F - kSubBits)) + threadIdx.x) & (kSub - 1));
        if (Rc >= static_cast<uint32_t>(m.nc) || seg >= m.nseg) { // self-check: never taken for live particles
          atomicOr(m.fp.status, kDevBadIndex);
          continue;
        }
        const float tau = __uint2float_rn(Rl) * m.tau_scale;
        const float a1  = A * tau, a2 = a1 * tau, a3 = a2 * tau;
        double*     h   = m.hist + ((static_cast<int64_t>(seg) * m.nc + Rc) * kSub + sub) * 4;
        red_add_float(h + 0, A);
        red_add_float(h + 1, a1);
        red_add_float(h + 2, a2);
        red_add_float(h + 3, a3);
      }
    }

    // Single-segment runs whose cell table fits in shared memory: one 1024-thread block per
    // SM accumulates the four moments of every cell in shared memory (FP64 atomics on the
    // block's own copy) and adds its copy to slot 0 of the global table once at the end, so
    // the global atomics are per (block, cell), not per particle.
    constexpr int kSmSharedThreads = 1024;

    __global__ void __launch_bounds__(kSmSharedThreads, 1)
      smooth_deposit_shared_kernel(const __grid_constant__ SmoothMomParams m) {
      extern __shared__ __align__(16) double cellm[]; // nc x 4
      for (int i = threadIdx.x; i < m.nc * 4; i += blockDim.x) {
        cellm[i] = 0.0;
      }
      if (__syncthreads_or(*m.fp.status != kDevOk)) {
        return;
      }
      const int64_t  stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
      const uint32_t mask   = (1u << m.F) - 1u;
      for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < m.n; i += stride) {
        float v[kComps];
#pragma unroll
        for (int c = 0; c < kComps; ++c) {
          v[c] = m.fp.comp[c] ? __ldg(m.fp.comp[c] + i) : 0.0f;
        }
        int64_t Q = 0;
        float   A = 0.0f;
        if (!moment_particle_stage(v, m.fp, m.Pmin, m.Pmax, m.L, Q, A)) {
          continue;
        }
        const uint64_t R  = static_cast<uint64_t>(m.Pmax - Q);
        const uint32_t Rc = static_cast<uint32_t>(R >> m.F);
        if (Rc >= static_cast<uint32_t>(m.nc)) { // self-check: never taken for live particles
          atomicOr(m.fp.status, kDevBadIndex);
          continue;
        }
        const float tau = __uint2float_rn(static_cast<uint32_t>(R) & mask) * m.tau_scale;
        const float a1  = A * tau, a2 = a1 * tau, a3 = a2 * tau;
        double*     h   = cellm + Rc * 4;
        atomicAdd(h + 0, static_cast<double>(A));
        atomicAdd(h + 1, static_cast<double>(a1));
        atomicAdd(h + 2, static_cast<double>(a2));
        atomicAdd(h + 3, static_cast<double>(a3));
      }
      __syncthreads();
      for (int i = threadIdx.x; i < m.nc * 4; i += blockDim.x) {
        const double x = cellm[i];
        if (x != 0.0) {
          atomicAdd(m.hist + (static_cast<int64_t>(i >> 2) * kSub) * 4 + (i & 3), x);
        }
      }
    }

    // Sums each cell's sub-cells into sub-cell 0 (thread per (segment, cell, moment)).
    __global__ void smooth_fold_kernel(double* hist, int64_t cells_total) {
      const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= cells_total * 4) {
        return;
      }
      const int64_t cell = t >> 2;
      const int     j    = static_cast<int>(t & 3);
      double*       h    = hist + cell * kSub * 4 + j;
      double        s    = 0.0;
#pragma unroll
      for (int k = 0; k < kSub; ++k) {
        s += h[k * 4];
      }
      h[0] = s;
    }

    struct SmoothReduceParams {
      const double*   hist; // folded: cell moments at sub-cell 0
      int             nc;
      const int4*     binfo; // per bin: (Dc, eps bits, 0, valid)
      const float4*   coef;  // the plan's table, nseg segments
      int             nseg_tab;
      int             nbins;
      const float*    ebins;
      const unsigned* status;
      float*          out; // nseg x nbins
    };

    __global__ void __launch_bounds__(32 * kSmRows) smooth_reduce_kernel(const __grid_constant__ SmoothReduceParams r) {
      __shared__ double part[kSmRows][33];
      const int  bin    = blockIdx.x * 32 + threadIdx.x;
      const int  seg    = blockIdx.y;
      const bool failed = *r.status != kDevOk;
      int4       bi     = make_int4(0, 0, 0, 0);
      if (bin < r.nbins && !failed) {
        bi = r.binfo[bin];
      }
      double sum = 0.0;
      if (bi.w) {
        const double  eps = static_cast<double>(__int_as_float(bi.y));
        const double* h   = r.hist + static_cast<int64_t>(seg) * r.nc * kSub * 4;
        for (int s = threadIdx.y; s < r.nseg_tab; s += kSmRows) {
          const int c = bi.x + s;
          if (c >= r.nc) {
            break;
          }
          const float4  k  = __ldg(r.coef + s);
          const double* M  = h + static_cast<int64_t>(c) * kSub * 4;
          const double  c0 = k.x, c1 = k.y, c2 = k.z, c3 = k.w;
          sum += (c0 + eps * c1) * M[0] + (c1 + 2.0 * eps * c2) * M[1] + (c2 + 3.0 * eps * c3) * M[2] + c3 * M[3];
        }
      }
      part[threadIdx.y][threadIdx.x] = sum;
      __syncthreads();
      if (threadIdx.y != 0 || bin >= r.nbins) {
        return;
      }
      double result = 0.0;
      if (failed) {
        result = __longlong_as_double(0x7ff8000000000000LL);
      } else if (bi.w) {
        double t = 0.0;
#pragma unroll
        for (int y = 0; y < kSmRows; ++y) {
          t += part[y][threadIdx.x];
        }
        result = t * static_cast<double>(r.ebins[bin]);
      }
      r.out[static_cast<int64_t>(seg) * r.nbins + bin] = __double2float_rn(result);
    }

    // alpha_j(c) = sum_b G_b e_b c'_j(c - Dc_b) for every (segment, cell): FP32 products,
    // compensated (Kahan) sums.  Thread per (segment, cell).
    struct SmoothAlphaParams {
      const float*  grad_out; // nseg x nbins
      const int4*   binfo;
      const float4* coef;
      int           nseg_tab;
      int           nbins;
      const float*  ebins;
      int           nc;
      int           nseg;
      float4*       alpha; // nseg x nc
    };

    __device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
      const float y = __fsub_rn(x, c);
      const float t = __fadd_rn(s, y);
      c             = __fsub_rn(__fsub_rn(t, s), y);
      s             = t;
    }

    __global__ void smooth_alpha_kernel(const __grid_constant__ SmoothAlphaParams a) {
      const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= static_cast<int64_t>(a.nseg) * a.nc) {
        return;
      }
      const int seg = static_cast<int>(t / a.nc), c = static_cast<int>(t % a.nc);
      float     s[4] = { 0.f, 0.f, 0.f, 0.f }, e[4] = { 0.f, 0.f, 0.f, 0.f };
      for (int b = 0; b < a.nbins; ++b) {
        const int4 bi = __ldg(a.binfo + b);
        const int  sg = c - bi.x;
        if (!bi.w || sg < 0 || sg >= a.nseg_tab) {
          continue;
        }
        const float  g   = __ldg(a.grad_out + static_cast<int64_t>(seg) * a.nbins + b) * __ldg(a.ebins + b);
        const float  eps = __int_as_float(bi.y);
        const float4 k   = __ldg(a.coef + sg);
        kahan_add(s[0], e[0], g * fmaf(eps, k.y, k.x));
        kahan_add(s[1], e[1], g * fmaf(2.0f * eps, k.z, k.y));
        kahan_add(s[2], e[2], g * fmaf(3.0f * eps, k.w, k.z));
        kahan_add(s[3], e[3], g * k.w);
      }
      a.alpha[t] = make_float4(s[0], s[1], s[2], s[3]);
    }

    struct SmoothAdjParams {
      SmoothMomParams m;
      const float4*   alpha; // nseg x nc
      float           inv_dln;
      float*          gw;
      float*          gu[3];
    };

    __global__ void __launch_bounds__(kSmThreads) smooth_adjoint_kernel(const __grid_constant__ SmoothAdjParams a) {
      __shared__ int64_t     soff[kSmSharedSeg + 1];
      const SmoothMomParams& m = a.m;
      if (!stage_offsets(m, soff)) {
        return;
      }
      const int64_t  first  = m.seg_off ? soff[0] : 0;
      const int64_t  last   = m.seg_off ? soff[m.nseg] : m.n;
      const int64_t  stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
      const uint32_t mask   = (1u << m.F) - 1u;
      const int64_t  i0     = first + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      // this thread's segment, advanced as its particle index grows
      int seg = m.seg_off ? segment_of(soff, m.nseg, i0) : 0;
      for (int64_t i = i0; i < last; i += stride) {
        if (m.seg_off) {
          while (seg < m.nseg && soff[seg + 1] <= i) {
            ++seg;
          }
        }
        float v[kComps];
#pragma unroll
        for (int c = 0; c < kComps; ++c) {
          v[c] = m.fp.comp[c] ? __ldg(m.fp.comp[c] + i) : 0.0f;
        }
        float   gw = 0.0f, gu[3] = { 0.0f, 0.0f, 0.0f };
        int64_t Q = 0;
        float   A = 0.0f;
        if (moment_particle_stage(v, m.fp, m.Pmin, m.Pmax, m.L, Q, A)) {
          const uint64_t R   = static_cast<uint64_t>(m.Pmax - Q);
          const uint32_t Rc  = static_cast<uint32_t>(R >> m.F);
          const uint32_t Rl  = static_cast<uint32_t>(R) & mask;
          if (Rc < static_cast<uint32_t>(m.nc) && seg < m.nseg) {
            const float  tau = __uint2float_rn(Rl) * m.tau_scale;
            const float4 al  = __ldg(a.alpha + static_cast<int64_t>(seg) * m.nc + Rc);
            const float  R1  = fmaf(tau, fmaf(tau, fmaf(tau, al.w, al.z), al.y), al.x);
            const float  dR1 = fmaf(tau, fmaf(tau, 3.0f * al.w, 2.0f * al.z), al.y);
            particle_gradient(v, m.fp, R1, dR1 * a.inv_dln, gw, gu);
          } else { // self-check: never taken for live particles
            atomicOr(m.fp.status, kDevBadIndex);
          }
        }
        if (a.gw) {
          a.gw[i] = gw;
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          if (a.gu[d]) {
            a.gu[d][i] = gu[d];
          }
        }
      }
    }

    void fill_smooth_params(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off, int64_t n,
                            int nseg, SmoothMomParams& m) {
      m = SmoothMomParams {};
      fill_params(pl, comp, nullptr, nullptr, n, 1, m.fp);
      m.Pmin      = pl->sm_pmin;
      m.Pmax      = pl->sm_pmax;
      m.L         = pl->mom_L;
      m.F         = pl->frac + 8;
      m.tau_scale = std::ldexp(1.0f, -m.F);
      m.seg_off   = d_off;
      m.nseg      = d_off ? nseg : 1;
      m.n         = n;
      m.nc        = pl->sm_cells;
      m.hist      = reinterpret_cast<double*>(pl->d_hist);
    }

    int particle_grid(int64_t n, int& grid) {
      DeviceContext* ctx = nullptr;
      RG_TRY(context(&ctx));
      const int64_t need = (n + kSmThreads - 1) / kSmThreads;
      grid               = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(need, ctx->sms * 8)));
      return RG_OK;
    }

  } // namespace

  // A plan's own smooth table aligned to log-uniform bins (see the file comment); leaves
  // the plan on the device-wide table when the bins are not log-uniform or the table
  // would need more than kSmoothMaxSegments segments.  ln_k0 = ln(eps / (g^2 B0)).
  int smooth_align_plan(rg_spectrum_plan* pl, double ln_k0) {
    const int n = pl->nbins;
    if (n < 2) {
      return RG_OK;
    }
    std::vector<double> le(n);
    for (int b = 0; b < n; ++b) {
      const double e = pl->h_bins[b];
      if (!(e > 0.0) || !std::isfinite(e)) {
        return RG_OK;
      }
      le[b] = std::log(e);
    }
    const double step = (le[n - 1] - le[0]) / (n - 1);
    if (!(step > 0.0)) {
      return RG_OK;
    }
    const int    m   = static_cast<int>(std::ceil(step / kTargetDln));
    const double dln = step / m;
    for (int b = 0; b < n; ++b) {
      if (std::fabs(le[b] - le[0] - b * step) > kUniformTol * dln) {
        return RG_OK;
      }
    }
    // nodes at ln e_0 - ln K0 - k dln, with the first node at or below x = 1e-6 and the
    // last at or above x = 100 (the device-wide table's range)
    const double base  = le[0] - ln_k0;
    const double k     = std::ceil((base - std::log(kSmoothXmin)) / dln);
    const double ln_x0 = base - k * dln;
    const double nseg  = std::ceil((std::log(kSmoothXmax) - ln_x0) / dln);
    if (!(nseg >= 1.0) || nseg > kSmoothMaxSegments) {
      return RG_OK;
    }
    RG_TRY(build_smooth_table_geom(pl->own_smooth, ln_x0, dln, static_cast<int>(nseg), nullptr));
    pl->smooth  = &pl->own_smooth;
    pl->aligned = true;
    return RG_OK;
  }

  // Cell tables of an aligned smooth plan (after its bins' fixed-point preparation).
  int smooth_moments_prepare(rg_spectrum_plan* pl, double ln_k0) {
    pl->moments_ok       = false;
    const SmoothTable* t = pl->smooth;
    const int          F = pl->frac + 8;
    if (pl->nbins < 1 || F > 30) {
      return RG_OK;
    }
    std::vector<int64_t> tb(pl->nbins);
    std::vector<double>  eps(pl->nbins);
    std::vector<int4>    binfo(pl->nbins, make_int4(0, 0, 0, 0));
    int64_t tmin = std::numeric_limits<int64_t>::max(), tmax = std::numeric_limits<int64_t>::min();
    for (int b = 0; b < pl->nbins; ++b) {
      const double tt = (std::log(static_cast<double>(pl->h_bins[b])) - ln_k0 - t->ln_xmin) / t->dln;
      tb[b]           = std::llround(tt);
      eps[b]          = tt - static_cast<double>(tb[b]);
      tmin            = std::min(tmin, tb[b]);
      tmax            = std::max(tmax, tb[b]);
    }
    for (int b = 0; b < pl->nbins; ++b) {
      const float e32 = static_cast<float>(eps[b]);
      int         ebits;
      std::memcpy(&ebits, &e32, sizeof(ebits));
      binfo[b] = make_int4(static_cast<int>(tmax - tb[b]), ebits, 0, 1);
    }
    const int64_t cells = (tmax - tmin) + t->nseg;
    if (cells > (int64_t(1) << 24)) {
      return RG_OK;
    }
    pl->sm_pmin      = tmin << F;
    pl->sm_pmax      = tmax << F;
    pl->mom_L        = static_cast<int64_t>(t->nseg) << F;
    pl->sm_cells     = static_cast<int>(cells);
    pl->hist_per_seg = cells * kSub * 2; // double2 entries: kSub x 4 doubles per cell
    RG_CUDA_TRY(cudaMalloc(&pl->d_binfo, sizeof(int4) * binfo.size()));
    RG_CUDA_TRY(cudaMemcpy(pl->d_binfo, binfo.data(), sizeof(int4) * binfo.size(), cudaMemcpyHostToDevice));
    pl->moments_ok = true;
    return RG_OK;
  }

  int smooth_moments_deposit(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off, int64_t n,
                             int nseg, cudaStream_t s) {
    if (n == 0 && !d_off) {
      return RG_OK;
    }
    SmoothMomParams m;
    fill_smooth_params(pl, comp, d_off, n, nseg, m);
    int grid = 1;
    RG_TRY(particle_grid(n, grid));
    std::pair<cudaEvent_t, cudaEvent_t> ev { nullptr, nullptr };
    if (pl->timing) {
      if (pl->ev_free.empty()) {
        RG_CUDA_TRY(cudaEventCreate(&ev.first));
        RG_CUDA_TRY(cudaEventCreate(&ev.second));
      } else {
        ev = pl->ev_free.back();
        pl->ev_free.pop_back();
      }
      RG_CUDA_TRY(cudaEventRecord(ev.first, s));
    }
    const size_t cell_bytes = sizeof(double) * 4 * static_cast<size_t>(pl->sm_cells);
    if (!d_off && cell_bytes <= kSmSharedMax) {
      static std::atomic<uint64_t> configured { 0 };
      RG_CUDA_TRY(ensure_max_dynamic_smem(smooth_deposit_shared_kernel, static_cast<int>(kSmSharedMax), configured));
      DeviceContext* ctx = nullptr;
      RG_TRY(context(&ctx));
      const int64_t need = (n + kSmSharedThreads - 1) / kSmSharedThreads;
      const int     g1   = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(need, ctx->sms)));
      smooth_deposit_shared_kernel<<<g1, kSmSharedThreads, cell_bytes, s>>>(m);
    } else {
      smooth_deposit_kernel<<<grid, kSmThreads, 0, s>>>(m);
    }
    RG_CUDA_TRY(cudaGetLastError());
    if (pl->timing) {
      RG_CUDA_TRY(cudaEventRecord(ev.second, s));
      pl->ev_used.push_back(ev);
    }
    return RG_OK;
  }

  int smooth_moments_finish(rg_spectrum_plan* pl, int nseg, float* out, cudaStream_t s) {
    const int64_t cells_total = static_cast<int64_t>(nseg) * pl->sm_cells;
    smooth_fold_kernel<<<static_cast<int>((cells_total * 4 + 255) / 256), 256, 0, s>>>(
      reinterpret_cast<double*>(pl->d_hist), cells_total);
    RG_CUDA_TRY(cudaGetLastError());
    SmoothReduceParams r {};
    r.hist     = reinterpret_cast<const double*>(pl->d_hist);
    r.nc       = pl->sm_cells;
    r.binfo    = pl->d_binfo;
    r.coef     = pl->smooth->d_coef;
    r.nseg_tab = pl->smooth->nseg;
    r.nbins    = pl->nbins;
    r.ebins    = pl->d_ebins;
    r.status   = pl->d_status;
    r.out      = out;
    smooth_reduce_kernel<<<dim3((pl->nbins + 31) / 32, nseg), dim3(32, kSmRows), 0, s>>>(r);
    RG_CUDA_TRY(cudaGetLastError());
    return RG_OK;
  }

  // The adjoint through cell cubics: grad_out is nseg x nbins; gradients of the particles
  // [0, n) (one segment) or of the segments of d_off.
  int smooth_moments_adjoint(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off, int64_t n,
                             int nseg, const float* grad_out, float* gw, float* const gu[3], cudaStream_t s) {
    const int    nsg  = d_off ? nseg : 1;
    const size_t need = static_cast<size_t>(nsg) * pl->sm_cells;
    if (need > pl->alpha_cap) {
      cudaFree(pl->d_alpha);
      pl->d_alpha = nullptr;
      RG_CUDA_TRY(cudaMalloc(&pl->d_alpha, sizeof(float4) * need));
      pl->alpha_cap = need;
    }
    SmoothAlphaParams a {};
    a.grad_out = grad_out;
    a.binfo    = pl->d_binfo;
    a.coef     = pl->smooth->d_coef;
    a.nseg_tab = pl->smooth->nseg;
    a.nbins    = pl->nbins;
    a.ebins    = pl->d_ebins;
    a.nc       = pl->sm_cells;
    a.nseg     = nsg;
    a.alpha    = pl->d_alpha;
    smooth_alpha_kernel<<<static_cast<int>((need + 127) / 128), 128, 0, s>>>(a);
    RG_CUDA_TRY(cudaGetLastError());
    if (n == 0 && !d_off) {
      return RG_OK;
    }
    SmoothAdjParams x {};
    fill_smooth_params(pl, comp, d_off, n, nseg, x.m);
    x.alpha   = pl->d_alpha;
    x.inv_dln = static_cast<float>(1.0 / pl->smooth->dln);
    x.gw      = gw;
    for (int d = 0; d < 3; ++d) {
      x.gu[d] = gu[d];
    }
    int grid = 1;
    RG_TRY(particle_grid(n, grid));
    smooth_adjoint_kernel<<<grid, kSmThreads, 0, s>>>(x);
    RG_CUDA_TRY(cudaGetLastError());
    return RG_OK;
  }

} // namespace rg

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
// four FP64 moments per cell (deposited into 64 slots per cell, which spreads the
// atomics of crowded cells, then folded into a compact cell table), and the adjoint of a loss L with
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
#include <type_traits>
#include <vector>

namespace rg {

  namespace {

    // Slots per cell: a particle adds its moments (which are absolute within the cell) to
    // the slot of its lane, shifted by its position in the cell, so the lanes of a warp
    // whose particles crowd one cell hit different addresses.
    constexpr int    kSub         = 64;
    constexpr int    kSubBits     = 6;
    constexpr int    kSmThreads   = 256;
    constexpr int    kSmSharedSeg = 1024;      // segment offsets staged in shared memory
    constexpr double kTargetDln   = 0.0089954; // ln(1e8) / 2048: the device-wide table's spacing
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
      uint2*         place;     // single-segment runs: per particle (cell, fraction bits) or
                                // (kNoCell, 0) for a particle that adds nothing; null: not kept
    };

    constexpr uint32_t kNoCell = 0xffffffffu;

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

    template <bool kI32>
    __global__ void __launch_bounds__(kSmThreads) smooth_deposit_kernel(const __grid_constant__ SmoothMomParams m) {
      __shared__ int64_t soff[kSmSharedSeg + 1];
      if (!stage_offsets(m, soff)) {
        return;
      }
      const int64_t  first  = m.seg_off ? soff[0] : 0;
      const int64_t  last   = m.seg_off ? soff[m.nseg] : m.n;
      // 32-bit particle indices when the stream allows it (the host checks last + stride < 2^32)
      using Idx            = std::conditional_t<kI32, uint32_t, int64_t>;
      const Idx      stride = static_cast<Idx>(gridDim.x) * blockDim.x;
      const uint32_t mask   = (1u << m.F) - 1u;
      const Idx      i0     = static_cast<Idx>(first + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x);
      const Idx      iend   = static_cast<Idx>(last);
      // this thread's segment, advanced as its particle index grows
      int seg = m.seg_off ? segment_of(soff, m.nseg, static_cast<int64_t>(i0)) : 0;
      for (Idx i = i0; i < iend; i += stride) {
        if (m.seg_off) {
          while (seg < m.nseg && soff[seg + 1] <= static_cast<int64_t>(i)) {
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
          if (m.place) {
            m.place[i] = make_uint2(kNoCell, 0u);
          }
          continue;
        }
        const uint64_t R   = static_cast<uint64_t>(m.Pmax - Q);
        const uint32_t Rc  = static_cast<uint32_t>(R >> m.F);
        const uint32_t Rl  = static_cast<uint32_t>(R) & mask;
        const int      sub = static_cast<int>(((Rl >> (m.F - kSubBits)) + threadIdx.x) & (kSub - 1));
        if (Rc >= static_cast<uint32_t>(m.nc) || seg >= m.nseg) { // self-check: never taken for live particles
          atomicOr(m.fp.status, kDevBadIndex);
          if (m.place) {
            m.place[i] = make_uint2(kNoCell, 0u);
          }
          continue;
        }
        if (m.place) {
          m.place[i] = make_uint2(Rc, Rl);
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

    // Sums each cell's sub-cells into the compact cell table cells[seg][cell][4] (thread per
    // (segment, cell, moment)).
    __global__ void smooth_fold_kernel(const double* __restrict__ hist, int64_t cells_total, double* __restrict__ cells) {
      const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= cells_total * 4) {
        return;
      }
      const double* h = hist + (t >> 2) * kSub * 4 + (t & 3);
      double        s = 0.0;
#pragma unroll
      for (int k = 0; k < kSub; ++k) {
        s += h[k * 4];
      }
      cells[t] = s;
    }

    // The table's coefficients as doubles for the reduce: (c0, c1), (c2, c3), and the
    // coefficients of the first-order bin-residual term (c1, 2 c2), (3 c3, 0).
    __global__ void smooth_coef64_kernel(const float4* __restrict__ coef, int nseg, double2* __restrict__ out) {
      const int s = blockIdx.x * blockDim.x + threadIdx.x;
      if (s < nseg) {
        const float4 k = coef[s];
        out[4 * s + 0] = make_double2(k.x, k.y);
        out[4 * s + 1] = make_double2(k.z, k.w);
        out[4 * s + 2] = make_double2(k.y, 2.0 * static_cast<double>(k.z));
        out[4 * s + 3] = make_double2(3.0 * static_cast<double>(k.w), 0.0);
      }
    }

    struct SmoothReduceParams {
      const double*   cells;  // nseg x nc x 4 folded cell moments
      int             nc;
      const int4*     binfo;  // per bin: (Dc, eps bits, 0, valid)
      const double2*  coef64; // per table segment: 4 double2 (smooth_coef64_kernel)
      int             nseg_tab;
      int             nbins;
      const float*    ebins;
      const unsigned* status;
      float*          out; // nseg x nbins
    };

    // S_b / e_b = sum_s sum_j c'_j(s) M_j(Dc_b + s) = A + eps_b B with A = sum c_j M_j and
    // B = sum (j + 1) c_{j+1} M_j: one 256-thread block per (bin, segment), its threads taking
    // every 256th table segment (consecutive cells: coalesced), FP64, summed in a fixed order.
    constexpr int kSmRedThreads = 256;

    __global__ void __launch_bounds__(kSmRedThreads) smooth_reduce_kernel(const __grid_constant__ SmoothReduceParams r) {
      __shared__ double wsum[kSmRedThreads / 32];
      const int  bin    = blockIdx.x;
      const int  seg    = blockIdx.y;
      const bool failed = *r.status != kDevOk;
      const int4 bi     = r.binfo[bin];
      double     t      = 0.0;
      if (bi.w && !failed) {
        const double2* M    = reinterpret_cast<const double2*>(r.cells + (static_cast<int64_t>(seg) * r.nc + bi.x) * 4);
        const int      smax = min(r.nseg_tab, r.nc - bi.x);
        double         a = 0.0, b = 0.0;
        for (int s = threadIdx.x; s < smax; s += kSmRedThreads) {
          const double2 m01 = M[2 * s], m23 = M[2 * s + 1];
          const double2 c01 = __ldg(r.coef64 + 4 * s), c23 = __ldg(r.coef64 + 4 * s + 1);
          const double2 d01 = __ldg(r.coef64 + 4 * s + 2), d23 = __ldg(r.coef64 + 4 * s + 3);
          a = fma(c01.x, m01.x, a);
          a = fma(c01.y, m01.y, a);
          a = fma(c23.x, m23.x, a);
          a = fma(c23.y, m23.y, a);
          b = fma(d01.x, m01.x, b);
          b = fma(d01.y, m01.y, b);
          b = fma(d23.x, m23.x, b);
        }
        t = fma(static_cast<double>(__int_as_float(bi.y)), b, a);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        t += __shfl_down_sync(0xffffffffu, t, o);
      }
      if ((threadIdx.x & 31) == 0) {
        wsum[threadIdx.x >> 5] = t;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double result = 0.0;
        if (failed) {
          result = __longlong_as_double(0x7ff8000000000000LL);
        } else if (bi.w) {
          double u = 0.0;
#pragma unroll
          for (int w = 0; w < kSmRedThreads / 32; ++w) {
            u += wsum[w];
          }
          result = u * static_cast<double>(r.ebins[bin]);
        }
        r.out[static_cast<int64_t>(seg) * r.nbins + bin] = __double2float_rn(result);
      }
    }

    // alpha_j(c) = sum_b G_b e_b c'_j(c - Dc_b) for every (segment, cell): one warp per
    // (segment, cell), its lanes taking every 32nd bin with FP32 products and compensated
    // (Kahan) sums, then a double-float sum over the lanes in a fixed order.
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

    constexpr int kSmAlphaThreads = 256;

    __global__ void __launch_bounds__(kSmAlphaThreads) smooth_alpha_kernel(const __grid_constant__ SmoothAlphaParams a) {
      const int64_t t    = (static_cast<int64_t>(blockIdx.x) * kSmAlphaThreads + threadIdx.x) >> 5;
      const int     lane = threadIdx.x & 31;
      if (t >= static_cast<int64_t>(a.nseg) * a.nc) { // warp-uniform
        return;
      }
      const int seg = static_cast<int>(t / a.nc), c = static_cast<int>(t % a.nc);
      float     s[4] = { 0.f, 0.f, 0.f, 0.f }, e[4] = { 0.f, 0.f, 0.f, 0.f };
      for (int b = lane; b < a.nbins; b += 32) {
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
      float out[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        // the lane's sum is s - e; add the lanes' double-floats pairwise
        ff v = fast_two_sum(s[j], -e[j]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float oh = __shfl_xor_sync(0xffffffffu, v.hi, o);
          const float ol = __shfl_xor_sync(0xffffffffu, v.lo, o);
          // every lane forms the same sum in the same order: the lower lane's value first
          const bool lower = (lane & o) == 0;
          const ff   x = lower ? v : ff { oh, ol }, y = lower ? ff { oh, ol } : v;
          const ff   h = two_sum(x.hi, y.hi);
          v          = fast_two_sum(h.hi, __fadd_rn(h.lo, __fadd_rn(x.lo, y.lo)));
        }
        out[j] = __fadd_rn(v.hi, v.lo);
      }
      if (lane == 0) {
        a.alpha[t] = make_float4(out[0], out[1], out[2], out[3]);
      }
    }

    struct SmoothAdjParams {
      SmoothMomParams m;
      const uint2*    place; // a forward's placement record (single segment), or null: recompute
      const float4*   alpha; // nseg x nc
      float           inv_dln;
      float*          gw;
      float*          gu[3];
    };

    template <bool kI32>
    __global__ void __launch_bounds__(kSmThreads) smooth_adjoint_kernel(const __grid_constant__ SmoothAdjParams a) {
      __shared__ int64_t     soff[kSmSharedSeg + 1];
      const SmoothMomParams& m = a.m;
      if (!stage_offsets(m, soff)) {
        return;
      }
      const int64_t  first  = m.seg_off ? soff[0] : 0;
      const int64_t  last   = m.seg_off ? soff[m.nseg] : m.n;
      // 32-bit particle indices when the stream allows it (the host checks last + stride < 2^32)
      using Idx            = std::conditional_t<kI32, uint32_t, int64_t>;
      const Idx      stride = static_cast<Idx>(gridDim.x) * blockDim.x;
      const uint32_t mask   = (1u << m.F) - 1u;
      const Idx      i0     = static_cast<Idx>(first + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x);
      const Idx      iend   = static_cast<Idx>(last);
      // this thread's segment, advanced as its particle index grows
      int seg = m.seg_off ? segment_of(soff, m.nseg, static_cast<int64_t>(i0)) : 0;
      for (Idx i = i0; i < iend; i += stride) {
        if (m.seg_off) {
          while (seg < m.nseg && soff[seg + 1] <= static_cast<int64_t>(i)) {
            ++seg;
          }
        }
        float v[kComps];
#pragma unroll
        for (int c = 0; c < kComps; ++c) {
          v[c] = m.fp.comp[c] ? __ldg(m.fp.comp[c] + i) : 0.0f;
        }
        float    gw = 0.0f, gu[3] = { 0.0f, 0.0f, 0.0f };
        bool     live = false;
        uint32_t Rc = 0, Rl = 0;
        if (a.place) { // the forward placed this particle already
          const uint2 pc = a.place[i];
          live           = pc.x != kNoCell;
          Rc             = pc.x;
          Rl             = pc.y;
        } else {
          int64_t Q = 0;
          float   A = 0.0f;
          live      = moment_particle_stage(v, m.fp, m.Pmin, m.Pmax, m.L, Q, A);
          if (live) {
            const uint64_t R = static_cast<uint64_t>(m.Pmax - Q);
            Rc               = static_cast<uint32_t>(R >> m.F);
            Rl               = static_cast<uint32_t>(R) & mask;
          }
        }
        if (live) {
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
      // 32 blocks per SM (more than fit at once) even out the SMs: measured against 8 and 16
      grid               = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(need, ctx->sms * 32)));
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
    RG_CUDA_TRY(cudaMalloc(&pl->d_coef64, sizeof(double2) * 4 * static_cast<size_t>(t->nseg)));
    smooth_coef64_kernel<<<(t->nseg + 127) / 128, 128>>>(t->d_coef, t->nseg, pl->d_coef64);
    RG_CUDA_TRY(cudaGetLastError());
    RG_CUDA_TRY(cudaDeviceSynchronize());
    pl->moments_ok = true;
    return RG_OK;
  }

  // Per-(segment, cell) scratch for at least `entries` (segment, cell) pairs.
  int smooth_reserve_cells(rg_spectrum_plan* pl, size_t entries) {
    if (entries > pl->cells_cap) {
      cudaFree(pl->d_cells);
      pl->d_cells   = nullptr;
      pl->cells_cap = 0;
      RG_CUDA_TRY(cudaMalloc(&pl->d_cells, sizeof(double) * 4 * entries));
      pl->cells_cap = entries;
    }
    return RG_OK;
  }

  int smooth_moments_deposit(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off, int64_t n,
                             int nseg, cudaStream_t s, uint2* place) {
    if (n == 0 && !d_off) {
      return RG_OK;
    }
    SmoothMomParams m;
    fill_smooth_params(pl, comp, d_off, n, nseg, m);
    m.place = d_off ? nullptr : place;
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
    if (n + static_cast<int64_t>(grid) * kSmThreads < (int64_t(1) << 32)) {
      smooth_deposit_kernel<true><<<grid, kSmThreads, 0, s>>>(m);
    } else {
      smooth_deposit_kernel<false><<<grid, kSmThreads, 0, s>>>(m);
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
    RG_TRY(smooth_reserve_cells(pl, static_cast<size_t>(cells_total)));
    smooth_fold_kernel<<<static_cast<int>((cells_total * 4 + 255) / 256), 256, 0, s>>>(
      reinterpret_cast<const double*>(pl->d_hist), cells_total, pl->d_cells);
    RG_CUDA_TRY(cudaGetLastError());
    SmoothReduceParams r {};
    r.cells    = pl->d_cells;
    r.nc       = pl->sm_cells;
    r.binfo    = pl->d_binfo;
    r.coef64   = pl->d_coef64;
    r.nseg_tab = pl->smooth->nseg;
    r.nbins    = pl->nbins;
    r.ebins    = pl->d_ebins;
    r.status   = pl->d_status;
    r.out      = out;
    smooth_reduce_kernel<<<dim3(pl->nbins, nseg), kSmRedThreads, 0, s>>>(r);
    RG_CUDA_TRY(cudaGetLastError());
    return RG_OK;
  }

  // The adjoint through cell cubics: grad_out is nseg x nbins; gradients of the particles
  // [0, n) (one segment) or of the segments of d_off.
  int smooth_moments_adjoint(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off, int64_t n,
                             int nseg, const float* grad_out, float* gw, float* const gu[3], cudaStream_t s,
                             const uint2* place) {
    const int    nsg  = d_off ? nseg : 1;
    const size_t need = static_cast<size_t>(nsg) * pl->sm_cells;
    RG_TRY(smooth_reserve_cells(pl, need));
    SmoothAlphaParams a {};
    a.grad_out = grad_out;
    a.binfo    = pl->d_binfo;
    a.coef     = pl->smooth->d_coef;
    a.nseg_tab = pl->smooth->nseg;
    a.nbins    = pl->nbins;
    a.ebins    = pl->d_ebins;
    a.nc       = pl->sm_cells;
    a.nseg     = nsg;
    a.alpha    = reinterpret_cast<float4*>(pl->d_cells);
    smooth_alpha_kernel<<<static_cast<int>((need * 32 + kSmAlphaThreads - 1) / kSmAlphaThreads), kSmAlphaThreads, 0, s>>>(a);
    RG_CUDA_TRY(cudaGetLastError());
    if (n == 0 && !d_off) {
      return RG_OK;
    }
    SmoothAdjParams x {};
    fill_smooth_params(pl, comp, d_off, n, nseg, x.m);
    x.place   = d_off ? nullptr : place;
    x.alpha   = reinterpret_cast<const float4*>(pl->d_cells);
    x.inv_dln = static_cast<float>(1.0 / pl->smooth->dln);
    x.gw      = gw;
    for (int d = 0; d < 3; ++d) {
      x.gu[d] = gu[d];
    }
    int grid = 1;
    RG_TRY(particle_grid(n, grid));
    if (n + static_cast<int64_t>(grid) * kSmThreads < (int64_t(1) << 32)) {
      smooth_adjoint_kernel<true><<<grid, kSmThreads, 0, s>>>(x);
    } else {
      smooth_adjoint_kernel<false><<<grid, kSmThreads, 0, s>>>(x);
    }
    RG_CUDA_TRY(cudaGetLastError());
    return RG_OK;
  }

} // namespace rg

// Adjoint of the synchrotron spectrum on sm_103a.
//
// Forward (spectrum.cu):  S_b = e_b sum_p A_p F(x_pb),  x_pb = e_b / e_peak_p,
//   A_p = w_p chiR_p (particles) or f_g J_g (distribution, J_g = gbeta_g for
//   log-spaced gamma bins).  Given G_b = dL/dS_b, with R1_p = sum_b G_b e_b F(x_pb)
//   and R2_p = sum_b G_b e_b dF/dln x (x_pb):
//     dL/dw_p = chiR_p R1_p,
//     dL/du_p = A_p (R1_p d ln chiR / du - R2_p d ln e_peak / du),
//     dL/df_g = J_g R1_g,
//   with ln chiR = ln W / 2 - ln G / 2 - ln B0, ln e_peak = ln K0 + ln G / 2 + ln W / 2,
//   G = 1 + u^2, W = |gamma E + u x B|^2 - (u.E)^2,
//   dW/du = (2 V.E / gamma) u + 2 B x V - 2 (u.E) E,  V = gamma E + u x B.
// dF/dln x is the derivative of the table the forward evaluates: for the smooth
// table the C1 Hermite interpolant of exact F with node slopes
// F(x) - x^2 K_{5/3}(x), i.e. x F'(x) with F'(x) = F(x)/x - x K_{5/3}(x); for the
// reference table the slope of its log-linear segments.  e_peak is recomputed
// here, not stored by the forward.
//
// Layout: the forward's work items and TMA staging; lanes own photon bins (G_b e_b
// in registers), warps own particles.  Each lane sums its bins for a particle;
// the 32 lane sums of 8 particles at a time are transposed through shared memory
// and reduced by 8 lanes; then one thread per particle forms the gradient from
// the recomputed kinematics.  Every particle is written by exactly one thread, so
// no atomics and a deterministic result.
#include "spectrum_common.cuh"
#include "spectrum_plan.hpp"

#include <algorithm>
#include <cmath>
#include <memory>

namespace rg {

  namespace {

    constexpr int kBatch = 8; // particles per shared-memory transpose

    struct AdjExtra {
      const float*   grad_out; // nseg x nbins
      const float*   ebins;
      const uint8_t* valid;
      int            nbins;
      float          dscale;   // dF/dt -> dF/dln x (and 2^-127 for the reference slopes)
      float*         gw;       // dL/dw (particles) or dL/df (distribution); nullable
      float*         gu[3];    // nullable
    };

    template <int K, int MODE>
    __global__ void __launch_bounds__(kThreads, kBlocksPerSM)
      adjoint_kernel(const __grid_constant__ FusedParams p, const __grid_constant__ AdjExtra x) {
      extern __shared__ __align__(128) unsigned char smem[];
      float2*   tab      = reinterpret_cast<float2*>(smem);
      float4*   htab     = reinterpret_cast<float4*>(smem);
      const int tab_size = (MODE == kModeRef) ? static_cast<int>(sizeof(float2)) * kRefEntries
                                              : static_cast<int>(sizeof(float4)) * (p.hseg + 1);
      int2*   qa    = reinterpret_cast<int2*>(smem + tab_size);
      float2* R     = reinterpret_cast<float2*>(qa + kChunk);
      float2* xbuf  = R + kChunk;                                   // [kWarps][kBatch][32]
      float*  stage = reinterpret_cast<float*>(xbuf + kWarps * kBatch * 32);
      __shared__ uint64_t mbar[2];
      __shared__ ItemInfo info[2];

      const int     tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
      const int     G        = gridDim.x, b = blockIdx.x;
      const int64_t n_items  = total_items(p.item_prefix, p.nseg, p.n_single);
      const int64_t it_begin = static_cast<int64_t>(b) * n_items / G;
      const int64_t it_end   = static_cast<int64_t>(b + 1) * n_items / G;
      if (it_begin >= it_end) {
        return;
      }
      if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        fence_mbar_init();
      }
      // one block-wide decision on the status word, and the barriers are
      // initialised before any thread waits on them
      if (__syncthreads_or(*p.status != kDevOk)) {
        return;
      }
      if (MODE == kModeRef) {
        for (int i = tid; i < kRefEntries; i += kThreads) {
          tab[i] = p.table[i];
        }
      } else {
        stage_smooth_table(p, htab, tid, kThreads);
      }
      int32_t P[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        P[k] = p.P[k * 32 + lane];
      }
      const int64_t  Pmin = p.Prange[0], Pmax = p.Prange[1];
      const int      stage_floats = p.nslots * kChunkPad;
      const uint32_t dead         = dead_coordinate(Pmin, p.L);
      const int      frac         = (MODE == kModeRef) ? kFrac : p.frac;
      const uint32_t hseg         = static_cast<uint32_t>(p.hseg);
      // fraction bits = T - seg * 2^frac as an IMAD, opaque to the compiler
      const uint32_t seg_neg      = (~p.opaque_zero) << frac;

      int seg_hint = 0;
      if (tid == 0) {
        info[0] = item_info(p, it_begin, seg_hint);
        if (p.use_tma) {
          issue_stage(p, info[0], stage, &mbar[0]);
        }
      }
      float Gk[K];
      int   cur_seg = -1;
      for (int64_t i = it_begin, it = 0; i < it_end; ++i, ++it) {
        const int st = static_cast<int>(it & 1);
        if (tid == 0 && i + 1 < it_end) {
          info[st ^ 1] = item_info(p, i + 1, seg_hint);
          if (p.use_tma) {
            fence_proxy_async_smem();
            issue_stage(p, info[st ^ 1], stage + (st ^ 1) * stage_floats, &mbar[st ^ 1]);
          }
        }
        bool ok = true;
        if (p.use_tma) {
          ok = mbar_wait_bounded(&mbar[st], static_cast<uint32_t>((it >> 1) & 1));
        }
        if (!__syncthreads_and(ok)) {
          if (tid == 0) {
            atomicOr(p.status, kDevTimeoutStage);
            if (i + 1 < it_end &&
                !mbar_wait_bounded(&mbar[st ^ 1], static_cast<uint32_t>(((it + 1) >> 1) & 1))) {
              atomicOr(p.status, kDevTimeoutDrain);
            }
          }
          return;
        }
        const ItemInfo I = info[st];
        if (I.seg != cur_seg) {
          cur_seg = I.seg;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const int bin = k * 32 + lane;
            Gk[k]         = (bin < x.nbins && x.valid[bin])
                              ? x.grad_out[static_cast<int64_t>(cur_seg) * x.nbins + bin] * x.ebins[bin]
                              : 0.0f;
          }
        }
        const float* sbuf = stage + st * stage_floats;
        // ---- per-particle stage (as the forward) ----------------------------------
        for (int j = tid; j < I.np; j += kThreads) {
          float v[kComps];
          load_comps(p, I, sbuf, I.pstart + j, v);
          uint32_t   q    = 0;
          float      A    = 0.0f;
          const bool live = (p.source == kSrcParticles) ? particle_stage(v, p, Pmin, Pmax, q, A)
                                                        : dist_stage(v[0], v[1], p, Pmin, Pmax, q, A);
          qa[j] = make_int2(static_cast<int>(live ? q : dead), __float_as_int(A));
        }
        __syncthreads();

        // ---- per-particle sums over bins ----------------------------------------------
        const int per = (I.np + kWarps - 1) / kWarps;
        const int j0  = warp * per;
        const int j1  = min(I.np, j0 + per);
        float2*   xb  = xbuf + warp * kBatch * 32;
        for (int jb = j0; jb < j1; jb += kBatch) {
#pragma unroll 1
          for (int jj = 0; jj < kBatch; ++jj) {
            const int j  = jb + jj;
            float     r1 = 0.0f, r2 = 0.0f;
            if (j < j1) {
              const uint32_t q = static_cast<uint32_t>(qa[j].x);
#pragma unroll
              for (int k = 0; k < K; ++k) {
                const uint32_t T = static_cast<uint32_t>(P[k]) - q;
                const uint32_t sg = T >> frac;
                if (MODE == kModeRef) {
                  const float2 c = tab[sg];
                  const float  m = __uint_as_float(sg * seg_neg + T);
                  r1             = __fmaf_rn(Gk[k], __fmaf_rn(m, c.y, c.x), r1);
                  r2             = __fmaf_rn(Gk[k], c.y, r2);
                } else {
                  const float4 c   = htab[min(sg, hseg)];
                  const float  tau = smooth_tau(sg * seg_neg + T);
                  const float  p2  = __fmaf_rn(tau, c.w, c.z);
                  const float  F   = __fmaf_rn(tau, __fmaf_rn(tau, p2, c.y), c.x);
                  const float  dF  = __fmaf_rn(tau, __fmaf_rn(tau, c.w, p2 + p2), c.y);
                  r1               = __fmaf_rn(Gk[k], F, r1);
                  r2               = __fmaf_rn(Gk[k], dF, r2);
                }
              }
            }
            xb[jj * 32 + lane] = make_float2(r1, r2);
          }
          __syncwarp();
          if (lane < kBatch && jb + lane < j1) {
            float s1 = 0.0f, s2 = 0.0f;
            for (int l = 0; l < 32; ++l) {
              const float2 t = xb[lane * 32 + l];
              s1 += t.x;
              s2 += t.y;
            }
            R[jb + lane] = make_float2(s1, s2 * x.dscale);
          }
          __syncwarp();
        }
        __syncthreads();

        // ---- gradients, one thread per particle -----------------------------------------
        for (int j = tid; j < I.np; j += kThreads) {
          const int64_t gp = I.pstart + j;
          float         v[kComps];
          load_comps(p, I, sbuf, gp, v);
          const float2 r = R[j];
          if (p.source == kSrcParticles) {
            float gw, gu[3];
            particle_gradient(v, p, r.x, r.y, gw, gu);
            if (x.gw) {
              x.gw[gp] = gw;
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              if (x.gu[d]) {
                x.gu[d][gp] = gu[d];
              }
            }
          } else if (x.gw) {
            x.gw[gp] = (p.log_spaced ? v[0] : 1.0f) * r.x;
          }
        }
        __syncthreads(); // staging buffer and R are reused by the next item
      }
    }

    size_t adjoint_smem(int mode, int hseg, int nslots) {
      const size_t tab = (mode == kModeRef) ? sizeof(float2) * kRefEntries : sizeof(float4) * (hseg + 1);
      return tab + sizeof(int2) * kChunk + sizeof(float2) * kChunk + sizeof(float2) * kWarps * kBatch * 32 +
             sizeof(float) * 2 * nslots * kChunkPad;
    }

    template <int K, int MODE>
    cudaError_t launch_adjoint_k(const FusedParams& fp, const AdjExtra& x, int grid, size_t smem,
                                 cudaStream_t s) {
      static std::atomic<uint64_t> configured { 0 };
      const cudaError_t            e = ensure_max_dynamic_smem(
        adjoint_kernel<K, MODE>, static_cast<int>(adjoint_smem(MODE, kSmoothMaxSegments, kComps)), configured);
      if (e != cudaSuccess) {
        return e;
      }
      adjoint_kernel<K, MODE><<<grid, kThreads, smem, s>>>(fp, x);
      return cudaGetLastError();
    }

    template <int MODE>
    cudaError_t launch_adjoint_mode(int K, const FusedParams& fp, const AdjExtra& x, int grid, size_t smem,
                                    cudaStream_t s) {
      switch (K) {
#define RG_K_CASE(k)                                                                         \
  case k:                                                                                    \
    return launch_adjoint_k<k, MODE>(fp, x, grid, smem, s);
        RG_K_CASE(1) RG_K_CASE(2) RG_K_CASE(3) RG_K_CASE(4) RG_K_CASE(5) RG_K_CASE(6)
        RG_K_CASE(7) RG_K_CASE(8) RG_K_CASE(9) RG_K_CASE(10) RG_K_CASE(11) RG_K_CASE(12)
        RG_K_CASE(13) RG_K_CASE(14) RG_K_CASE(15) RG_K_CASE(16)
#undef RG_K_CASE
        default:
          return cudaErrorInvalidValue;
      }
    }

    int run_adjoint(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off,
                    int64_t n_single, int nseg, const float* grad_out, float* gw, float* const gu[3],
                    cudaStream_t s) {
      if (nseg <= 0) {
        return RG_OK;
      }
      if (!pl->zero && pl->nbins > 0 && pl->aligned && moments_selected(pl, nseg)) {
        return smooth_moments_adjoint(pl, comp, d_off, n_single, nseg, grad_out, gw, gu, s);
      }
      if (pl->algo == RG_ALGO_MOMENTS && pl->table_mode == kModeSmooth) {
        return set_error(RG_ERR_UNSUPPORTED, "this plan or run cannot use the moment adjoint");
      }
      if (pl->nslices != 1) {
        return set_error(RG_ERR_UNSUPPORTED, "the adjoint supports up to 512 photon bins");
      }
      const bool any_out = gw || gu[0] || gu[1] || gu[2];
      if (!any_out) {
        return RG_OK;
      }
      const int64_t n_total = n_single; // gradients cover every particle of the set
      if (pl->zero || pl->nbins == 0) {
        // no particle contributes: every gradient is zero
        if (gw) {
          RG_CUDA_TRY(cudaMemsetAsync(gw, 0, sizeof(float) * n_total, s));
        }
        for (int d = 0; d < 3; ++d) {
          if (gu[d]) {
            RG_CUDA_TRY(cudaMemsetAsync(gu[d], 0, sizeof(float) * n_total, s));
          }
        }
        return RG_OK;
      }
      RG_TRY(plan_reserve(pl, nseg));
      const int64_t* d_prefix = nullptr;
      if (d_off) {
        RG_TRY(item_prefix(pl, d_off, nseg, n_single, s));
        d_prefix = pl->d_prefix;
      }
      FusedParams  fp;
      const int    nslots = fill_params(pl, comp, d_off, d_prefix, n_single, nseg, fp);
      const double dln    = (pl->table_mode == kModeRef) ? pl->ref->dln : pl->smooth->dln;
      AdjExtra     x {};
      x.grad_out = grad_out;
      x.ebins    = pl->d_ebins;
      x.valid    = pl->d_valid;
      x.nbins    = pl->nbins;
      // reference slopes carry 2^127; smooth slopes are per tau' = tau 2^(frac - 23)
      x.dscale   = static_cast<float>((pl->table_mode == kModeRef ? 1.0 / kSlopeScale
                                                                  : std::ldexp(1.0, pl->frac - 23)) / dln);
      x.gw       = gw;
      for (int d = 0; d < 3; ++d) {
        x.gu[d] = gu[d];
      }
      int G = pl->grid;
      if (!d_off) {
        const int64_t items = (n_single + kChunk - 1) / kChunk;
        G = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(items, pl->grid)));
        if (n_single == 0) {
          return RG_OK;
        }
      }
      const size_t smem = adjoint_smem(pl->table_mode, fp.hseg, nslots);
      const cudaError_t e = (pl->table_mode == kModeRef)
                              ? launch_adjoint_mode<kModeRef>(pl->K, fp, x, G, smem, s)
                              : launch_adjoint_mode<kModeSmooth>(pl->K, fp, x, G, smem, s);
      RG_CUDA_TRY(e);
      return RG_OK;
    }

  } // namespace

} // namespace rg

extern "C" {

int rg_spectrum_adjoint(const rg_spectrum_plan* cplan, const rg_particles* p, const float* grad_out,
                        float* grad_w, float* grad_ux, float* grad_uy, float* grad_uz, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrumAdjoint");
  auto* plan = const_cast<rg_spectrum_plan*>(cplan);
  if (!plan || !grad_out || plan->source != rg::kSrcParticles) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_adjoint: bad arguments");
  }
  RG_TRY(rg::check_particles(p));
  const float* comp[rg::kComps];
  rg::particle_comps(p, comp);
  float* gu[3] = { grad_ux, grad_uy, grad_uz };
  return rg::run_adjoint(plan, comp, nullptr, p->n, 1, grad_out, grad_w, gu,
                         static_cast<cudaStream_t>(stream));
}

int rg_spectrum_adjoint_placed(rg_spectrum_plan* plan, const rg_particles* p, const void* placement,
                               const float* grad_out, float* grad_w, float* grad_ux, float* grad_uy, float* grad_uz,
                               void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrumAdjoint");
  if (!plan || !placement || !grad_out || plan->source != rg::kSrcParticles) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_adjoint_placed: bad arguments");
  }
  RG_TRY(rg::check_particles(p));
  if (plan->zero || plan->nbins == 0 || !plan->aligned || !rg::moments_selected(plan, 1)) {
    return rg::set_error(RG_ERR_UNSUPPORTED,
                         "rg_spectrum_adjoint_placed: needs a plan that runs cell moments on its bin-aligned smooth table");
  }
  const float* comp[rg::kComps];
  rg::particle_comps(p, comp);
  float* gu[3] = { grad_ux, grad_uy, grad_uz };
  return rg::smooth_moments_adjoint(plan, comp, nullptr, p->n, 1, grad_out, grad_w, gu,
                                    static_cast<cudaStream_t>(stream), static_cast<const uint2*>(placement));
}

int rg_spectrum_adjoint_batched(rg_spectrum_plan* plan, const rg_particles* p, const int64_t* offsets,
                                int32_t nseg, const float* grad_out, float* grad_w, float* grad_ux,
                                float* grad_uy, float* grad_uz, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrumAdjoint");
  if (!plan || !offsets || nseg < 0 || !grad_out || plan->source != rg::kSrcParticles) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_adjoint_batched: bad arguments");
  }
  RG_TRY(rg::check_particles(p));
  const float* comp[rg::kComps];
  rg::particle_comps(p, comp);
  float* gu[3] = { grad_ux, grad_uy, grad_uz };
  return rg::run_adjoint(plan, comp, offsets, p->n, nseg, grad_out, grad_w, gu,
                         static_cast<cudaStream_t>(stream));
}

int rg_dist_plan_create(const float* bins, int32_t nbins, float g_syn, float e_syn_at_g_syn,
                        int32_t log_spaced, int32_t table_mode, rg_spectrum_plan** plan) {
  // a particle plan with B0 = 1 has K0 = eps / g^2, the distribution's constant
  RG_TRY(rg::create_plan(bins, nbins, 1.0f, g_syn, e_syn_at_g_syn, table_mode, rg::kSrcDist, plan));
  (*plan)->log_spaced = log_spaced ? 1 : 0;
  (*plan)->amp        = 1.0f;
  return RG_OK;
}

int rg_dist_adjoint(const rg_spectrum_plan* plan, const float* gbeta, const float* f, int32_t ng,
                    const float* grad_out, float* grad_f, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrumFromDistAdjoint");
  if (!plan || plan->source != rg::kSrcDist || ng < 0 || !grad_out || (ng > 0 && (!gbeta || !f))) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_dist_adjoint: bad arguments");
  }
  const float* comp[rg::kComps] = {};
  comp[0]                       = gbeta;
  comp[1]                       = f;
  float* gu[3]                  = { nullptr, nullptr, nullptr };
  return rg::run_adjoint(const_cast<rg_spectrum_plan*>(plan), comp, nullptr, ng, 1, grad_out, grad_f, gu,
                         static_cast<cudaStream_t>(stream));
}

} // extern "C"

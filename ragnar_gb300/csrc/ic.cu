// Inverse-Compton spectrum on sm_103a: ICSpectrum (ic.cpp:15-46), ic::Kernel
// (ic.hpp:67-94) and KNfunc (ic.hpp:20-25).
//
//   S[e] = sum_g sum_s f_g (f_s / e_s) e^2 KN(Gamma, q) / g^k      (k = 1 for log-spaced
//          gamma bins, 2 for linear ones), over the (g, s) pairs with e <= g Gamma / (1 + Gamma),
//   Gamma = 4 g e_s,  q = (e / g) / (Gamma (1 - e / g)),
//   KN(Gamma, q) = 2 q ln q + (1 - q) (1 + 2 q + (Gamma q)^2 / (2 (1 + Gamma q))).
//
// Rewritten so that the per-(g, s, e) work is one multiply and one logarithm:
//   t = Gamma q = e / (g - e) depends on (e, g) only; g - e is exact in FP32 where it
//     matters (e in [g/2, g]), so t avoids the reference's 1 - e/g cancellation;
//   q = t / Gamma = (t / g) (1 / (4 e_s));  e <= g Gamma / (1 + Gamma)  <=>  q <= 1 (e < g);
//   KN = q (2 ln 2) log2 q + ((1 + h) + (1 - h) q - 2 q^2),  h = t^2 / (2 (1 + t)).
// With L = 2 ln 2 and p = L q (so 2 q ln q = p log2 q = p (log2 p - log2 L)) this is
//   KN = p log2 p + ((1 + h) + ((1 - h) / L - log2 L) p - (2 / L^2) p^2),
// whose quadratic's coefficients depend on (e, g) only and are set once per item.
// Per eval: FMUL (p = (L t / g) (1 / (4 e_s))), MUFU.LG2, two FFMA (quadratic), FFMA (log
// term), max(KN, 0), FFMA into the FP32 accumulator.  max(KN, 0) is KN [q <= 1]: at fixed
// h, KN(1) = 0, KN'(1) = -1 - h < 0 and KN'' = 2/q - 4 < 0 for q > 1/2, so KN < 0 for every
// q > 1, while KN >= 0 on (0, 1] (the Klein-Nishina kernel).  Evals with p = inf (masked
// soft photons; (e, g) pairs that no soft photon reaches, e >= g or an invalid e, which get
// pg = inf) evaluate to NaN, which max(., 0) also maps to 0.  q >= 1e-30 is guaranteed by a
// floor on t/g set per (e, g) from the smallest 1 / (4 e_s), so the log's argument is a
// normal float or inf.  (A form without the per-eval logarithm, log2 p split into
// log2 (t/g) + log2 (1/(4 e_s)) per item and per photon, takes five FP32 instructions per
// eval but leaves absolute errors of a few ulp of those logarithms' magnitudes in KN: 2.4e-5
// to 8.6e-5 from FP64 on the reference's delta-function soft-photon cases, where a single
// (g, s) pair at 1 - q = 3.5e-3 feeds an IC bin.)
//
// Layout: lanes own IC bins (K rows of 32 per lane, 512-bin slices in blockIdx.y); warps take
// (gamma bin, 64-soft-photon chunk) items; per item the FP32 sums are scaled by
// e^2 f_g / g^k and folded into a double-float; per-warp FP64 partials are reduced in a
// fixed order: the block's warps in FP64 at its end, then the blocks by a second kernel
// (deterministic).  Non-positive or non-finite IC bins give
// 0 (the reference produces NaN there).
#include "rg_common.cuh"
#include "rg_internal.hpp"

#include <algorithm>
#include <cmath>

namespace rg {

  namespace {

    constexpr int kIcThreads = 256;
    constexpr int kIcWarps   = kIcThreads / 32;
    constexpr int kIcSlice   = 512; // the widest slice of IC bins (K = 16 rows of 32 per lane)
    constexpr int kIcSChunk  = 64; // soft photons per work item
    constexpr int kIcMaxRows = 16; // rows of 32 IC bins per lane (the slice width is rows x 32)

    struct IcParams {
      const float* gb;      // ng gamma (gamma beta) bins
      const float* fp;      // ng particle distribution
      int          ng;
      int          log_spaced;
      const float* inv4es;  // ns: 1 / (4 e_s)
      const float* inv4es_min; // min over s of 1 / (4 e_s) (positive values), one float
      const float* ws;      // ns: f_s / e_s
      const float4* setup;  // ng x ne_pad per (gamma bin, IC bin): (pg, 1 + h, B1, 0), or null
      int          ne_pad;  // nslices x slice_w
      int          ns;
      const float* eic;     // ne IC photon energies
      int          ne;
      int          nslices;
      int          slice_w;  // IC bins per slice: K x 32
      double*      partials; // [grid][nslices][slice_w]: one row per block
    };

    // inv4es, ws and the smallest positive inv4es (positive floats order like their bit
    // patterns, so an unsigned atomicMin finds it; the slot starts at +inf)
    __global__ void ic_prep_kernel(const float* __restrict__ es, const float* __restrict__ fs, int ns,
                                   float* __restrict__ inv4es, float* __restrict__ ws, unsigned* min_bits) {
      const int s = blockIdx.x * blockDim.x + threadIdx.x;
      if (s < ns) {
        const float e  = es[s];
        const bool  ok = e > 0.0f && isfinite(e); // non-positive soft-photon bins contribute nothing
        const float i4 = ok ? __frcp_rn(__fmul_rn(4.0f, e)) : __int_as_float(0x7f800000); // q = inf: masked
        inv4es[s]      = i4;
        ws[s]          = ok ? __fdiv_rn(fs[s], e) : 0.0f;
        if (ok && i4 > 0.0f) {
          atomicMin(min_bits, __float_as_uint(i4));
        }
      }
    }

    // L = 2 ln 2 rounded to FP32; log2 L and -2 / L^2 of that FP32 value
    constexpr float kIcL     = 1.3862943649291992f;
    constexpr float kIcLog2L = 0.47123363101939075f;

    // What an (IC bin, gamma bin) pair contributes to every eval: pg = L t / g (p = pg / (4 e_s)),
    // 1 + h, and the linear coefficient (1 - h) / L - log2 L; pg = inf for a pair that no soft
    // photon reaches (e >= g or an invalid e).  e: the bin's energy, 0 if invalid.
    __device__ __forceinline__ float4 ic_pair_setup(float e, float gv, float inv_g, float tg_floor) {
      const float d     = __fsub_rn(gv, e);
      const bool  reach = e > 0.0f && d > 0.0f;
      float       t = 0.0f, h = 0.0f;
      if (reach) {
        t = __fdiv_rn(e, d);
        h = __fdiv_rn(__fmul_rn(0.5f, __fmul_rn(t, t)), __fadd_rn(1.0f, t));
      }
      const float pg = reach ? __fmul_rn(kIcL, fmaxf(__fmul_rn(t, inv_g), tg_floor)) : __int_as_float(0x7f800000);
      return make_float4(pg, __fadd_rn(1.0f, h), __fsub_rn(__fdiv_rn(__fsub_rn(1.0f, h), kIcL), kIcLog2L), 0.0f);
    }

    __device__ __forceinline__ float ic_bin_energy(const IcParams& p, int bin) {
      const float e = bin < p.ne ? __ldg(p.eic + bin) : 0.0f;
      return (e > 0.0f && isfinite(e)) ? e : 0.0f;
    }

    // t/g >= this keeps q = (t/g) / (4 e_s) >= 1e-30 for every soft photon with e_s > 0: the
    // log's argument stays a normal float without a per-eval clamp
    __device__ __forceinline__ float ic_tg_floor(const IcParams& p) {
      return __fdiv_rn(1e-30f, *p.inv4es_min);
    }

    // The pair setups of every (gamma bin, padded IC bin), once per call: the main kernel's
    // items (gamma bin, 64 soft photons) would otherwise repeat them for every chunk.
    __global__ void ic_setup_kernel(const __grid_constant__ IcParams p, float4* __restrict__ setup) {
      const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= static_cast<int64_t>(p.ng) * p.ne_pad) {
        return;
      }
      const int   g   = static_cast<int>(t / p.ne_pad), bin = static_cast<int>(t % p.ne_pad);
      const float gv  = __ldg(p.gb + g);
      // invalid gamma bins are skipped by the main kernel before it reads their row
      setup[t] = (gv > 0.0f && isfinite(gv)) ? ic_pair_setup(ic_bin_energy(p, bin), gv, __frcp_rn(gv), ic_tg_floor(p))
                                             : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }

    template <int K>
    __global__ void __launch_bounds__(kIcThreads, 2) ic_kernel(const __grid_constant__ IcParams p) {
      const int     lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      const int     slice = blockIdx.y;
      const int     nsc   = (p.ns + kIcSChunk - 1) / kIcSChunk;
      const int64_t items = static_cast<int64_t>(p.ng) * nsc;
      const int64_t G = gridDim.x, b = blockIdx.x;
      const int64_t i0 = b * items / G, i1 = (b + 1) * items / G;

      // this lane's IC energy of row k (0 for padding and for invalid bins); reloaded
      // where needed (per item) instead of held in registers
      auto energy = [&](int k) -> float { return ic_bin_energy(p, slice * (K * 32) + k * 32 + lane); };
      float hi[K], lo[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        hi[k] = 0.0f;
        lo[k] = 0.0f;
      }
      const float kC2      = -1.0406844847835448f; // -2 / L^2
      const float tg_floor = ic_tg_floor(p);

      for (int64_t it = i0 + warp; it < i1; it += kIcWarps) {
        const int   g     = static_cast<int>(it / nsc);
        const int   s0    = static_cast<int>(it - static_cast<int64_t>(g) * nsc) * kIcSChunk;
        const int   s1    = min(p.ns, s0 + kIcSChunk);
        const float gv    = __ldg(p.gb + g);
        const float fv    = __ldg(p.fp + g);
        if (!(gv > 0.0f) || !isfinite(gv)) {
          continue; // non-positive or non-finite gamma bins contribute nothing (warp-uniform)
        }
        const float inv_g = __frcp_rn(gv);
        // per (e, g): pg, 1 + h and the linear coefficient (ic_pair_setup), from the call's
        // setup table when there is one; q = (t / g) / (4 e_s) > 1 marks no contribution
        float pg[K], A0[K], B1[K], acc[K];
        const float4* su = p.setup ? p.setup + static_cast<int64_t>(g) * p.ne_pad + slice * (K * 32) + lane : nullptr;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const float4 v = su ? __ldg(su + k * 32) : ic_pair_setup(energy(k), gv, inv_g, tg_floor);
          pg[k]  = v.x;
          A0[k]  = v.y;
          B1[k]  = v.z;
          acc[k] = 0.0f;
        }
        for (int s = s0; s < s1; ++s) {
          const float i4 = __ldg(p.inv4es + s);
          const float w  = __ldg(p.ws + s);
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const float pq = __fmul_rn(pg[k], i4);
            // p >= L 1e-30 by the floor on t/g, so the log's argument is a normal float or
            // inf; max(KN, 0) is KN [q <= 1] and maps NaN to 0
            const float lp   = lg2_normal(pq);
            const float poly = __fmaf_rn(__fmaf_rn(kC2, pq, B1[k]), pq, A0[k]);
            const float kn   = __fmaf_rn(pq, lp, poly);
            acc[k]           = __fmaf_rn(w, fmaxf(kn, 0.0f), acc[k]);
          }
        }
        // scale by e^2 f_g / g^k and fold into the double-float sums
        const float fg = p.log_spaced ? __fmul_rn(fv, inv_g) : __fmul_rn(__fmul_rn(fv, inv_g), inv_g);
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const float e    = energy(k);
          const float term = __fmul_rn(__fmul_rn(acc[k], fg), __fmul_rn(e, e));
          const ff    sm   = two_sum(hi[k], term);
          hi[k]            = sm.hi;
          lo[k]            = __fadd_rn(lo[k], sm.lo);
        }
      }
      // the block's warps summed in FP64 in warp order: one partial row per block
      __shared__ double red[kIcWarps * kIcSlice];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        red[warp * (K * 32) + k * 32 + lane] = static_cast<double>(hi[k]) + static_cast<double>(lo[k]);
      }
      __syncthreads();
      double* dst = p.partials + (b * p.nslices + slice) * (K * 32);
      for (int j = threadIdx.x; j < K * 32; j += kIcThreads) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < kIcWarps; ++w) {
          t += red[w * (K * 32) + j];
        }
        dst[j] = t;
      }
    }

    // out[e] = sum over blocks (fixed order) of the partial rows; 32 bins x 32 row groups.
    __global__ void __launch_bounds__(1024)
      ic_reduce_kernel(const double* __restrict__ partials, int grid, int nslices, int slice_w, int ne,
                       float* __restrict__ out) {
      __shared__ double part[32][33];
      const int bin = blockIdx.x * 32 + threadIdx.x, ty = threadIdx.y;
      double    sum = 0.0;
      if (bin < ne) {
        const int slice = bin / slice_w, j = bin % slice_w;
        // unrolled so that several rows' loads are in flight (the adds stay in row order)
#pragma unroll 8
        for (int r = ty; r < grid; r += 32) {
          sum += partials[(static_cast<int64_t>(r) * nslices + slice) * slice_w + j];
        }
      }
      part[ty][threadIdx.x] = sum;
      __syncthreads();
      if (ty == 0 && bin < ne) {
        double t = 0.0;
        for (int y = 0; y < 32; ++y) {
          t += part[y][threadIdx.x];
        }
        out[bin] = __double2float_rn(t);
      }
    }

    template <int K>
    cudaError_t launch_ic_k(const IcParams& p, dim3 grid, cudaStream_t s) {
      ic_kernel<K><<<grid, kIcThreads, 0, s>>>(p);
      return cudaGetLastError();
    }

    cudaError_t launch_ic(int K, const IcParams& p, dim3 grid, cudaStream_t s) {
      switch (K) {
#define RG_IC_K(k)                                                                                   \
  case k:                                                                                            \
    return launch_ic_k<k>(p, grid, s);
        RG_IC_K(1) RG_IC_K(2) RG_IC_K(3) RG_IC_K(4) RG_IC_K(5) RG_IC_K(6) RG_IC_K(7) RG_IC_K(8)
        RG_IC_K(9) RG_IC_K(10) RG_IC_K(11) RG_IC_K(12) RG_IC_K(13) RG_IC_K(14) RG_IC_K(15) RG_IC_K(16)
#undef RG_IC_K
        default:
          return cudaErrorInvalidValue;
      }
    }

  } // namespace

} // namespace rg

extern "C" {

int rg_ic_spectrum(const float* gbins, const float* f, int32_t ng, int32_t log_spaced, const float* es,
                   const float* fs, int32_t ns, const float* eic, int32_t ne, float* out, void* stream) {
  rg::NvtxRange nvtx_range("ICSpectrum");
  rg::clear_error();
  if (ng < 0 || ns < 0 || ne < 0 || (ng > 0 && (!gbins || !f)) || (ns > 0 && (!es || !fs)) ||
      (ne > 0 && (!eic || !out))) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_ic_spectrum: bad arguments");
  }
  auto s = static_cast<cudaStream_t>(stream);
  if (ne == 0) {
    return RG_OK;
  }
  if (ng == 0 || ns == 0) {
    RG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * ne, s));
    return RG_OK;
  }
  rg::DeviceContext* ctx = nullptr;
  RG_TRY(rg::context(&ctx));
  const int     K       = std::min(rg::kIcMaxRows, (std::min(ne, rg::kIcSlice) + 31) / 32);
  const int     slice_w = K * 32;
  const int     nslices = (ne + slice_w - 1) / slice_w;
  const int64_t items   = static_cast<int64_t>(ng) * ((ns + rg::kIcSChunk - 1) / rg::kIcSChunk);
  const int     grid    = static_cast<int>(std::max<int64_t>(
    1, std::min<int64_t>(2 * ctx->sms, (items + rg::kIcWarps - 1) / rg::kIcWarps)));
  // one stream-ordered scratch allocation: inv4es, ws, partials
  const size_t off_ws   = 256 * ((sizeof(float) * ns + 255) / 256);
  const size_t off_min  = off_ws + 256 * ((sizeof(float) * ns + 255) / 256);
  const size_t off_part = off_min + 256;
  // the (gamma bin, IC bin) setup table when it is small (it is 16 bytes per pair)
  const int64_t ne_pad    = static_cast<int64_t>(nslices) * slice_w;
  const size_t  set_bytes = sizeof(float4) * static_cast<size_t>(ng) * static_cast<size_t>(ne_pad);
  const bool    use_setup = set_bytes <= (size_t(64) << 20);
  const size_t  off_set   = 256 * ((off_part + sizeof(double) * static_cast<size_t>(grid) * nslices * slice_w + 255) / 256);
  const size_t  bytes     = off_set + (use_setup ? set_bytes : 0);
  unsigned char* buf    = nullptr;
  RG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&buf), bytes, s));
  rg::IcParams p {};
  p.gb         = gbins;
  p.fp         = f;
  p.ng         = ng;
  p.log_spaced = log_spaced ? 1 : 0;
  p.inv4es     = reinterpret_cast<float*>(buf);
  p.ws         = reinterpret_cast<float*>(buf + off_ws);
  p.ns         = ns;
  p.eic        = eic;
  p.ne         = ne;
  p.nslices    = nslices;
  p.slice_w    = slice_w;
  p.partials   = reinterpret_cast<double*>(buf + off_part);
  p.ne_pad     = static_cast<int>(ne_pad);
  p.setup      = nullptr;
  p.inv4es_min = reinterpret_cast<float*>(buf + off_min);
  // the minimum slot starts at 0x7f7f7f7f (3.4e38, above any 1 / (4 e_s) of a positive float)
  cudaError_t e = cudaMemsetAsync(buf + off_min, 0x7f, sizeof(unsigned), s);
  if (e == cudaSuccess) {
    rg::ic_prep_kernel<<<(ns + 255) / 256, 256, 0, s>>>(es, fs, ns, reinterpret_cast<float*>(buf),
                                                         reinterpret_cast<float*>(buf + off_ws),
                                                         reinterpret_cast<unsigned*>(buf + off_min));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && use_setup) {
    auto* setup  = reinterpret_cast<float4*>(buf + off_set);
    const int64_t pairs = static_cast<int64_t>(ng) * ne_pad;
    rg::ic_setup_kernel<<<static_cast<unsigned>((pairs + 255) / 256), 256, 0, s>>>(p, setup);
    e       = cudaGetLastError();
    p.setup = setup;
  }
  if (e == cudaSuccess) e = rg::launch_ic(K, p, dim3(grid, nslices), s);
  if (e == cudaSuccess) {
    rg::ic_reduce_kernel<<<dim3((ne + 31) / 32), dim3(32, 32), 0, s>>>(p.partials, grid, nslices, slice_w, ne,
                                                                        out);
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(buf, s);
  if (e != cudaSuccess) {
    return rg::cuda_error(e, "rg_ic_spectrum launch");
  }
  RG_CUDA_TRY(ef);
  return RG_OK;
}

} // extern "C"

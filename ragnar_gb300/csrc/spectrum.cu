// Particle and distribution synchrotron spectra on sm_103a.
//
// Reference path: sync::Kernel<D>::operator() (synchrotron.hpp:145-172) and
// sync::KernelFromDist::operator() (synchrotron.hpp:72-95), reduced over
// particles as SynchrotronSpectrum<D> / SynchrotronSpectrumFromDist do
// (synchrotron.cpp:69-145).
//
// Design (the "fused" kernel):
//  * Per-particle stage, once per particle: gamma^2 = 1 + u^2 and
//    W = |gamma E + u x B|^2 - (u.E)^2 as double-floats, then
//      chiR = sqrt(W) / (gamma B0),  e_peak = K0 gamma sqrt(W),  K0 = eps / (g^2 B0),
//    and the particle's table coordinate Q = 2^22 (ln gamma + ln W / 2) / dln as a
//    fixed-point integer (ln of a double-float to ~1e-10 absolute).
//  * Photon bin b carries P_b = 2^22 (ln e_b - ln xmin - ln K0) / dln (host, FP64),
//    so T = P_b - Q (one 32-bit integer add, exact) is the fixed-point table
//    coordinate of x = e_b / e_peak.  Its top 10 bits index a 1024-entry segment
//    table in shared memory (entries past the last segment are zero, so an
//    out-of-range x reads zero without a branch); its low 22 bits, read as a
//    denormal, times the stored slope (pre-scaled by 2^127) give frac * slope in
//    one FFMA.  Per eval: IADD, SHF, LOP, LDS.64, FFMA (F), FFMA (accumulate).
//  * Lanes own photon bins (32 consecutive bins per row, K rows per lane), warps
//    own particles; per-warp FP32 register accumulators are folded into
//    double-float accumulators after every chunk, combined across warps in FP64
//    in a fixed order and written per block; a second kernel sums the blocks in
//    FP64 in a fixed order, so results are bit-reproducible.
//  * Particle streams (SoA FP32) are staged chunk by chunk into shared memory
//    with 1-D TMA bulk copies (cp.async.bulk + mbarrier), double buffered.
//  * Work items are (segment, chunk) pairs in particle order; each block of the
//    persistent grid takes a contiguous range of items, so one spectrum and a
//    batch of uneven segments run through the same launch, and every block
//    touches each segment in one contiguous run (one partial per (block, seg)).
#include "rg_common.cuh"
#include "rg_internal.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

namespace rg {

  namespace {

    constexpr int kThreads   = 256;
    constexpr int kWarps     = kThreads / 32;
    constexpr int kSliceBins = 512; // bins per block slice (K <= 16 rows of 32)
    constexpr int kChunk     = 512; // particles per work item
    constexpr int kChunkPad  = kChunk + 4;
    constexpr int kComps     = 10;  // u0 u1 u2 e0 e1 e2 b0 b1 b2 w
    constexpr int kBlocksPerSM = 2;

    // extra status bit: segment offsets were not non-decreasing
    constexpr unsigned kDevBadOffsets = 4u;

    enum Source : int { kSrcParticles = 0, kSrcDist = 1 };

    struct FusedParams {
      const float*   comp[kComps]; // particle streams (dist: comp[0] = gbeta, comp[1] = f)
      int            slot[kComps]; // shared-memory stream slot, -1 if not staged
      int            nslots;
      int            source;
      int            has_e;
      int            has_w;
      int            use_tma;
      int            log_spaced;   // dist: J_g = gbeta when set
      const int64_t* seg_off;      // nseg + 1 particle offsets (device), or null: one segment
      const int64_t* item_prefix;  // nseg + 1 cumulative item counts (device), or null
      int64_t        n_single;     // particle count when seg_off is null
      int            nseg;
      const int32_t* P;            // nslices * kSliceBins fixed-point bin coordinates
      const int64_t* Prange;       // per slice: (Pmin, Pmax) over valid bins
      int64_t        L;            // (n_nodes - 1) << kFrac
      float          Sh, Sl;       // 2^kFrac / (2 dln) as a double-float
      int64_t        Cfx;          // round(S ln2 2^16)
      float          amp;          // 1 / B0 (particles) or 1 (dist)
      const float2*  table;        // kRefEntries segments
      double*        partials;     // [(grid + nseg) * nslices * kSliceBins]
      int            nslices;
      unsigned*      status;
    };

    struct ItemInfo {
      int     seg;
      int     np;
      int64_t pstart, pend, a0, a1;
    };

    __device__ __forceinline__ int64_t seg_begin(const FusedParams& p, int s) {
      return p.seg_off ? p.seg_off[s] : 0;
    }

    __device__ __forceinline__ int64_t seg_end(const FusedParams& p, int s) {
      return p.seg_off ? p.seg_off[s + 1] : p.n_single;
    }

    __device__ __forceinline__ int64_t items_before(const int64_t* prefix, int s) {
      return prefix ? prefix[s] : 0;
    }

    __device__ __forceinline__ int64_t total_items(const int64_t* prefix, int nseg,
                                                   int64_t n_single) {
      return prefix ? prefix[nseg] : (n_single + kChunk - 1) / kChunk;
    }

    // ---- accurate logarithm of a positive double-float ---------------------------
    struct LnParts {
      int   e; // ln x = e ln2 + h + l
      float h, l;
    };

    __device__ __forceinline__ LnParts ln_parts(ff x) {
      int   e;
      float m = frexpf(x.hi, &e); // x.hi = m 2^e, m in [0.5, 1)
      if (m < 0.70710678f) {
        m = __fmul_rn(m, 2.0f);
        e -= 1;
      }
      // ln m = 2 atanh(z), z = (m - 1)/(m + 1), |z| < 0.1716
      const float f  = __fsub_rn(m, 1.0f); // exact
      const ff    d  = two_sum(m, 1.0f);
      const float q  = __fdiv_rn(f, d.hi);
      const float r  = __fmaf_rn(-q, d.hi, f); // exact remainder
      const float zl = __fdiv_rn(__fmaf_rn(-q, d.lo, r), d.hi);
      const float w  = __fmul_rn(q, q);
      const float poly =
        w * (0.33333334f + w * (0.2f + w * (0.14285715f + w * (0.11111111f + w * 0.09090909f))));
      LnParts o;
      o.e = e;
      o.h = __fmul_rn(2.0f, q);
      o.l = __fadd_rn(__fmaf_rn(o.h, poly, __fmul_rn(2.0f, zl)), __fdiv_rn(x.lo, x.hi));
      return o;
    }

    // round(S (ln X1 + ln X2)), S = Sh + Sl; the exponent part goes through the
    // integer constant Cfx = round(S ln2 2^16).
    __device__ __forceinline__ int64_t fixed_log_sum(ff X1, ff X2, float Sh, float Sl,
                                                     int64_t Cfx) {
      const LnParts a = ln_parts(X1);
      const LnParts b = ln_parts(X2);
      ff            s = two_sum(a.h, b.h);
      s.lo            = __fadd_rn(s.lo, __fadd_rn(a.l, b.l));
      const float ph  = __fmul_rn(s.hi, Sh);
      const float pe  = __fmaf_rn(s.hi, Sh, -ph);
      const float pl  = __fadd_rn(pe, __fmaf_rn(s.hi, Sl, __fmul_rn(s.lo, Sh)));
      const int64_t q = static_cast<int64_t>(a.e + b.e) * Cfx +
                        __float2ll_rn(__fmul_rn(ph, 65536.0f)) +
                        __float2ll_rn(__fmul_rn(pl, 65536.0f));
      return (q + 32768) >> 16;
    }

    // Per-particle stage for particle data.  Returns false if the particle adds
    // nothing (e_peak <= 0 or not finite, or x outside the table for every bin).
    __device__ __forceinline__ bool particle_stage(const float (&v)[kComps], const FusedParams& p,
                                                   int64_t Pmin, int64_t Pmax, uint32_t& q32,
                                                   float& A) {
      const float ux = v[0], uy = v[1], uz = v[2];
      const float bx = v[6], by = v[7], bz = v[8];
      ff          u2 = two_prod(ux, ux);
      u2             = ff_add(u2, two_prod(uy, uy));
      u2             = ff_add(u2, two_prod(uz, uz));
      const ff G     = ff_add(ff { 1.0f, 0.0f }, u2);
      const ff cx    = ff_diff_of_products(uy, bz, uz, by);
      const ff cy    = ff_diff_of_products(uz, bx, ux, bz);
      const ff cz    = ff_diff_of_products(ux, by, uy, bx);
      ff       W;
      if (!p.has_e) {
        W = ff_add(ff_add(ff_sqr(cx), ff_sqr(cy)), ff_sqr(cz));
      } else {
        const float ex = v[3], ey = v[4], ez = v[5];
        // gamma as a double-float: g = sqrt(G.hi), correction (G - g^2) / (2 g)
        const float gh = sqrtf(G.hi);
        const float gl = __fdiv_rn(__fadd_rn(__fmaf_rn(-gh, gh, G.hi), G.lo), __fmul_rn(2.0f, gh));
        const ff    gm { gh, gl };
        const ff    Vx = ff_add(ff_mul(gm, ff { ex, 0.0f }), cx);
        const ff    Vy = ff_add(ff_mul(gm, ff { ey, 0.0f }), cy);
        const ff    Vz = ff_add(ff_mul(gm, ff { ez, 0.0f }), cz);
        ff          uE = two_prod(ux, ex);
        uE             = ff_add(uE, two_prod(uy, ey));
        uE             = ff_add(uE, two_prod(uz, ez));
        W = ff_add(ff_add(ff_add(ff_sqr(Vx), ff_sqr(Vy)), ff_sqr(Vz)), ff_neg(ff_sqr(uE)));
      }
      if (!(W.hi > 0.0f) || !isfinite(W.hi) || !isfinite(G.hi)) {
        return false;
      }
      const int64_t Q = fixed_log_sum(G, W, p.Sh, p.Sl, p.Cfx);
      if (Q <= Pmin - p.L || Q > Pmax) {
        return false;
      }
      q32 = static_cast<uint32_t>(Q);
      A   = p.amp * sqrtf(__fdiv_rn(W.hi, G.hi));
      if (p.has_w) {
        A *= v[9];
      }
      return isfinite(A);
    }

    // Per-"particle" stage of a tabulated distribution (synchrotron.hpp:76-94):
    // e_peak = K0 gbeta^2, amplitude f * (gbeta if the gamma bins are log-spaced).
    __device__ __forceinline__ bool dist_stage(float gb, float f, const FusedParams& p,
                                               int64_t Pmin, int64_t Pmax, uint32_t& q32,
                                               float& A) {
      const ff X = two_prod(gb, gb);
      if (!(X.hi > 0.0f) || !isfinite(X.hi)) {
        return false;
      }
      const int64_t Q = fixed_log_sum(X, X, p.Sh, p.Sl, p.Cfx);
      if (Q <= Pmin - p.L || Q > Pmax) {
        return false;
      }
      q32 = static_cast<uint32_t>(Q);
      A   = p.log_spaced ? __fmul_rn(f, gb) : f;
      return isfinite(A);
    }

    __device__ __forceinline__ ItemInfo item_info(const FusedParams& p, int64_t i, int& seg_hint) {
      int s = seg_hint;
      while (s + 1 < p.nseg && items_before(p.item_prefix, s + 1) <= i) {
        ++s;
      }
      seg_hint        = s;
      const int64_t c = i - items_before(p.item_prefix, s);
      ItemInfo      I;
      I.seg    = s;
      I.pstart = seg_begin(p, s) + c * kChunk;
      I.pend   = min(I.pstart + kChunk, seg_end(p, s));
      I.np     = static_cast<int>(I.pend - I.pstart);
      I.a0     = I.pstart & ~int64_t(3);
      I.a1     = I.pend & ~int64_t(3);
      if (I.a1 < I.a0) {
        I.a1 = I.a0;
      }
      return I;
    }

    __device__ __forceinline__ void issue_stage(const FusedParams& p, const ItemInfo& I,
                                                float* buf, uint64_t* bar) {
      const uint32_t bytes = static_cast<uint32_t>(I.a1 - I.a0) * 4u;
      mbar_arrive_expect_tx(bar, bytes * static_cast<uint32_t>(p.nslots));
      if (bytes) {
        for (int c = 0; c < kComps; ++c) {
          if (p.slot[c] >= 0) {
            bulk_g2s(buf + p.slot[c] * kChunkPad, p.comp[c] + I.a0, bytes, bar);
          }
        }
      }
    }

    // Block b of G owns items [b n / G, (b+1) n / G); the block holding item i:
    __device__ __forceinline__ int block_of_item(int64_t i, int64_t n_items, int G) {
      return static_cast<int>(((i + 1) * G - 1) / n_items);
    }

    template <int K>
    __device__ __forceinline__ void flush_block(float (&hi)[K], float (&lo)[K], double* red,
                                                double* dst, int warp, int lane, int tid) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        red[warp * kSliceBins + k * 32 + lane] =
          static_cast<double>(hi[k]) + static_cast<double>(lo[k]);
        hi[k] = 0.0f;
        lo[k] = 0.0f;
      }
      __syncthreads();
      for (int j = tid; j < K * 32; j += kThreads) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
          s += red[w * kSliceBins + j];
        }
        dst[j] = s;
      }
      __syncthreads();
    }

    template <int K>
    __global__ void __launch_bounds__(kThreads, kBlocksPerSM)
      fused_spectrum_kernel(const __grid_constant__ FusedParams p) {
      extern __shared__ __align__(128) unsigned char smem[];
      float2* tab   = reinterpret_cast<float2*>(smem);
      int2*   qa    = reinterpret_cast<int2*>(smem + sizeof(float2) * kRefEntries);
      double* red   = reinterpret_cast<double*>(qa + 2 * kChunk);
      float*  stage = reinterpret_cast<float*>(red + kWarps * kSliceBins);
      __shared__ uint64_t mbar[2];
      __shared__ ItemInfo info[2];

      const int     tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
      const int     slice    = blockIdx.y;
      const int     G        = gridDim.x, b = blockIdx.x;
      const int64_t n_items  = total_items(p.item_prefix, p.nseg, p.n_single);
      const int64_t it_begin = static_cast<int64_t>(b) * n_items / G;
      const int64_t it_end   = static_cast<int64_t>(b + 1) * n_items / G;
      if (it_begin >= it_end || *p.status != kDevOk) {
        return;
      }
      for (int i = tid; i < kRefEntries; i += kThreads) {
        tab[i] = p.table[i];
      }
      int32_t P[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        P[k] = p.P[slice * kSliceBins + k * 32 + lane];
      }
      const int64_t Pmin = p.Prange[2 * slice], Pmax = p.Prange[2 * slice + 1];
      const int     stage_floats = p.nslots * kChunkPad;

      int seg_hint = 0;
      if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        fence_mbar_init();
        info[0] = item_info(p, it_begin, seg_hint);
        if (p.use_tma) {
          issue_stage(p, info[0], stage, &mbar[0]);
        }
      }

      float acc[K], hi[K], lo[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        acc[k] = 0.0f;
        hi[k]  = 0.0f;
        lo[k]  = 0.0f;
      }

      int cur_seg = -1;
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
          if (cur_seg >= 0) {
            flush_block<K>(hi, lo, red,
                           p.partials + (static_cast<int64_t>(b + cur_seg) * p.nslices + slice) *
                                          kSliceBins,
                           warp, lane, tid);
          }
          cur_seg = I.seg;
        }

        // ---- per-particle stage ------------------------------------------------
        const float* sbuf = stage + st * stage_floats;
        int2*        qdst = qa + st * kChunk;
        for (int j = tid; j < I.np; j += kThreads) {
          const int64_t gp      = I.pstart + j;
          const bool    in_smem = p.use_tma && gp < I.a1;
          float         v[kComps];
#pragma unroll
          for (int c = 0; c < kComps; ++c) {
            const float* src = p.comp[c];
            v[c]             = 0.0f;
            if (src) {
              v[c] = in_smem ? sbuf[p.slot[c] * kChunkPad + (gp - I.a0)] : __ldg(src + gp);
            }
          }
          uint32_t q = 0;
          float    A = 0.0f;
          const bool live = (p.source == kSrcParticles) ? particle_stage(v, p, Pmin, Pmax, q, A)
                                                        : dist_stage(v[0], v[1], p, Pmin, Pmax, q, A);
          if (!live) {
            q = 0;
            A = 0.0f;
          }
          qdst[j] = make_int2(static_cast<int>(q), __float_as_int(A));
        }
        __syncthreads();

        // ---- evaluation: lanes over bins, warps over particles -------------------
        const int per = (I.np + kWarps - 1) / kWarps;
        const int j0  = warp * per;
        const int j1  = min(I.np, j0 + per);
        for (int j = j0; j < j1; ++j) {
          const int2     e = qdst[j];
          const uint32_t q = static_cast<uint32_t>(e.x);
          const float    A = __int_as_float(e.y);
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const uint32_t T = static_cast<uint32_t>(P[k]) - q;
            const float2   c = tab[T >> kFrac];
            const float    m = __uint_as_float(T & kFracMask);
            const float    F = __fmaf_rn(m, c.y, c.x);
            acc[k]           = __fmaf_rn(A, F, acc[k]);
          }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const ff s = two_sum(hi[k], acc[k]);
          hi[k]      = s.hi;
          lo[k]      = __fadd_rn(lo[k], s.lo);
          acc[k]     = 0.0f;
        }
      }
      if (cur_seg >= 0) {
        flush_block<K>(hi, lo, red,
                       p.partials + (static_cast<int64_t>(b + cur_seg) * p.nslices + slice) *
                                      kSliceBins,
                       warp, lane, tid);
      }
    }

    // Cumulative chunk counts of the segments (one block), with a check that the
    // offsets never decrease and stay within [0, n]; on failure the status word
    // is set and the fused kernel that follows does no work.
    __global__ void item_prefix_kernel(const int64_t* __restrict__ off, int nseg, int64_t n,
                                       int64_t* __restrict__ prefix, unsigned* status) {
      __shared__ int64_t carry;
      __shared__ int64_t warp_sums[32];
      if (threadIdx.x == 0) {
        carry     = 0;
        prefix[0] = 0;
      }
      __syncthreads();
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      for (int base = 0; base < nseg; base += blockDim.x) {
        const int s = base + threadIdx.x;
        int64_t   v = 0;
        if (s < nseg) {
          const int64_t a = off[s], e = off[s + 1];
          if (e < a || a < 0 || e > n) {
            atomicOr(status, kDevBadOffsets);
          } else {
            v = (e - a + kChunk - 1) / kChunk;
          }
        }
        // inclusive scan within the warp, then across warps
        for (int o = 1; o < 32; o <<= 1) {
          const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
          if (lane >= o) {
            v += t;
          }
        }
        if (lane == 31) {
          warp_sums[wid] = v;
        }
        __syncthreads();
        if (wid == 0) {
          int64_t w = lane < static_cast<int>(blockDim.x >> 5) ? warp_sums[lane] : 0;
          for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) {
              w += t;
            }
          }
          warp_sums[lane] = w;
        }
        __syncthreads();
        const int64_t excl = (wid > 0 ? warp_sums[wid - 1] : 0) + carry;
        if (s < nseg) {
          prefix[s + 1] = excl + v;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) {
          carry = excl + v;
        }
        __syncthreads();
      }
    }

    // Sums the per-block partials of every (segment, bin) in block order and
    // applies the photon-energy factor; masked bins are zero, and every output is
    // NaN if the device status reports a failure.
    struct ReduceParams {
      const double*   partials;
      const int64_t*  item_prefix; // or null: one segment
      int64_t         n_single;
      int             grid;
      int             nslices;
      int             nseg;
      int             nbins;
      const float*    ebins;
      const uint8_t*  valid;
      const unsigned* status;
      float*          out;   // nseg x nbins
      double*         acc64; // when set: acc64 += result in FP64 instead of writing out
    };

    __global__ void reduce_partials_kernel(const __grid_constant__ ReduceParams r) {
      const int bin = blockIdx.x * blockDim.x + threadIdx.x;
      const int s   = blockIdx.y;
      if (bin >= r.nbins) {
        return;
      }
      double result = 0.0;
      if (*r.status != kDevOk) {
        result = __longlong_as_double(0x7ff8000000000000LL);
      } else {
        const int64_t n_items = total_items(r.item_prefix, r.nseg, r.n_single);
        const int64_t i0      = items_before(r.item_prefix, s);
        const int64_t i1      = r.item_prefix ? r.item_prefix[s + 1] : n_items;
        if (i1 > i0 && r.valid[bin]) {
          const int b0    = block_of_item(i0, n_items, r.grid);
          const int b1    = block_of_item(i1 - 1, n_items, r.grid);
          const int slice = bin / kSliceBins, j = bin % kSliceBins;
          double    sum   = 0.0;
          for (int b = b0; b <= b1; ++b) {
            sum += r.partials[(static_cast<int64_t>(b + s) * r.nslices + slice) * kSliceBins + j];
          }
          result = sum * static_cast<double>(r.ebins[bin]);
        }
      }
      const int64_t o = static_cast<int64_t>(s) * r.nbins + bin;
      if (r.acc64) {
        r.acc64[o] += result;
      } else {
        r.out[o] = __double2float_rn(result);
      }
    }

    __global__ void finalize_acc_kernel(const double* __restrict__ acc, int n,
                                        const unsigned* status, float* __restrict__ out) {
      const int i = blockIdx.x * blockDim.x + threadIdx.x;
      if (i < n) {
        out[i] = (*status != kDevOk) ? __int_as_float(0x7fc00000) : __double2float_rn(acc[i]);
      }
    }

    // ---- plain baseline kernel ------------------------------------------------------
    // Thread per particle, kinematics hoisted per thread in FP32, per-eval
    // interpolation as tabulation.hpp:19-53 writes it (log10f and divisions),
    // warp-shuffle sum per bin into shared-memory accumulators, FP64 atomics per
    // block into the global result.
    struct PlainParams {
      const float* comp[kComps];
      int64_t      n;
      const float* bins;
      int          nbins;
      float        B0, g_syn, eps;
      const float* tx;
      const float* ty;
      int          nt;
      float        xmin, xmax;
      double*      acc; // nbins
    };

    __device__ __forceinline__ float interp_ref(float x0, const float* x, const float* y, int n,
                                                float xmin, float xmax) {
      if (x0 < xmin || x0 >= xmax) {
        return 0.0f;
      }
      const int xi = static_cast<int>(static_cast<float>(n - 1) * fabsf(log10f(x0 / xmin)) /
                                      log10f(xmax / xmin));
      if (xi >= n - 1) {
        return y[n - 1];
      }
      return (y[xi + 1] * log10f(x0 / x[xi]) + y[xi] * log10f(x[xi + 1] / x0)) /
             log10f(x[xi + 1] / x[xi]);
    }

    __global__ void __launch_bounds__(256) plain_spectrum_kernel(const __grid_constant__ PlainParams p) {
      extern __shared__ float sm[];
      float* sx  = sm;
      float* sy  = sx + p.nt;
      float* sb  = sy + p.nt;
      float* acc = sb + p.nbins;
      for (int i = threadIdx.x; i < p.nt; i += blockDim.x) {
        sx[i] = p.tx[i];
        sy[i] = p.ty[i];
      }
      for (int i = threadIdx.x; i < p.nbins; i += blockDim.x) {
        sb[i]  = p.bins[i];
        acc[i] = 0.0f;
      }
      __syncthreads();
      const int lane = threadIdx.x & 31;
      for (int64_t base = static_cast<int64_t>(blockIdx.x) * blockDim.x; base < p.n;
           base += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t i      = base + threadIdx.x;
        float         e_peak = 0.0f, chiR = 0.0f, w = 0.0f;
        if (i < p.n) {
          const float ux = p.comp[0][i], uy = p.comp[1][i], uz = p.comp[2][i];
          const float ex = p.comp[3] ? p.comp[3][i] : 0.0f;
          const float ey = p.comp[4] ? p.comp[4][i] : 0.0f;
          const float ez = p.comp[5] ? p.comp[5][i] : 0.0f;
          const float bx = p.comp[6] ? p.comp[6][i] : 0.0f;
          const float by = p.comp[7] ? p.comp[7][i] : 0.0f;
          const float bz = p.comp[8] ? p.comp[8][i] : 0.0f;
          w                 = p.comp[9] ? p.comp[9][i] : 1.0f;
          const float gamma = sqrtf(1.0f + ux * ux + uy * uy + uz * uz);
          const float btx = ux / gamma, bty = uy / gamma, btz = uz / gamma;
          const float bde = btx * ex + bty * ey + btz * ez;
          const float vx  = ex + (bty * bz - btz * by);
          const float vy  = ey + (btz * bx - btx * bz);
          const float vz  = ez + (btx * by - bty * bx);
          chiR            = sqrtf(vx * vx + vy * vy + vz * vz - bde * bde) / p.B0;
          e_peak          = p.eps * gamma * gamma * chiR / (p.g_syn * p.g_syn);
        }
        for (int e = 0; e < p.nbins; ++e) {
          float v = 0.0f;
          if (e_peak > 0.0f) {
            const float es = sb[e];
            v = es * chiR * interp_ref(es / e_peak, sx, sy, p.nt, p.xmin, p.xmax) * w;
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            v += __shfl_down_sync(0xffffffffu, v, o);
          }
          if (lane == 0) {
            atomicAdd(&acc[e], v);
          }
        }
      }
      __syncthreads();
      for (int e = threadIdx.x; e < p.nbins; e += blockDim.x) {
        atomicAdd(&p.acc[e], static_cast<double>(acc[e]));
      }
    }

    __global__ void f64_to_f32_kernel(const double* in, float* out, int n) {
      const int i = blockIdx.x * blockDim.x + threadIdx.x;
      if (i < n) {
        out[i] = __double2float_rn(in[i]);
      }
    }

    size_t fused_smem(int nslots) {
      return sizeof(float2) * kRefEntries + sizeof(int2) * 2 * kChunk +
             sizeof(double) * kWarps * kSliceBins + sizeof(float) * 2 * nslots * kChunkPad;
    }

    template <int K>
    cudaError_t launch_fused_k(const FusedParams& fp, dim3 grid, size_t smem, cudaStream_t s) {
      static bool configured = false;
      if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(fused_spectrum_kernel<K>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(fused_smem(kComps)));
        if (e != cudaSuccess) {
          return e;
        }
        configured = true;
      }
      fused_spectrum_kernel<K><<<grid, kThreads, smem, s>>>(fp);
      return cudaGetLastError();
    }

    cudaError_t launch_fused(int K, const FusedParams& fp, dim3 grid, size_t smem, cudaStream_t s) {
      switch (K) {
#define RG_K_CASE(k)                                                                         \
  case k:                                                                                    \
    return launch_fused_k<k>(fp, grid, smem, s);
        RG_K_CASE(1) RG_K_CASE(2) RG_K_CASE(3) RG_K_CASE(4) RG_K_CASE(5) RG_K_CASE(6)
        RG_K_CASE(7) RG_K_CASE(8) RG_K_CASE(9) RG_K_CASE(10) RG_K_CASE(11) RG_K_CASE(12)
        RG_K_CASE(13) RG_K_CASE(14) RG_K_CASE(15) RG_K_CASE(16)
#undef RG_K_CASE
        default:
          return cudaErrorInvalidValue;
      }
    }

  } // namespace

} // namespace rg

// ---------------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------------

struct rg_spectrum_plan {
  int                 device     = 0;
  int                 table_mode = RG_TABLE_REFERENCE;
  int                 source     = rg::kSrcParticles;
  int                 nbins      = 0;
  int                 nslices    = 0;
  int                 K          = 0;
  bool                zero       = false; // every contribution is zero (K0 <= 0 ...)
  float               B0 = 1, g_syn = 1, eps = 1;
  int                 log_spaced = 0; // dist source
  int64_t             L          = 0;
  float               Sh = 0, Sl = 0;
  int64_t             Cfx        = 0;
  float               amp        = 1;
  int                 grid       = 0; // blocks per slice of the fused kernel
  std::vector<float>  h_bins;
  int32_t*            d_P         = nullptr;
  int64_t*            d_Prange    = nullptr;
  float*              d_ebins     = nullptr;
  uint8_t*            d_valid     = nullptr;
  unsigned*           d_status    = nullptr;
  double*             d_partials  = nullptr;
  size_t              partial_cap = 0; // doubles
  int64_t*            d_prefix    = nullptr;
  int                 prefix_cap  = 0; // segments
  double*             d_plain_acc = nullptr;
  const rg::RefTable* ref         = nullptr;
  // kernel timing (events bracketing each fused launch)
  bool                                             timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_used, ev_free;
  // host-resident streaming: device staging for two chunks, a copy stream
  float*       d_stage[2]     = { nullptr, nullptr };
  int64_t      stage_chunk    = 0;
  cudaStream_t copy_stream    = nullptr;
  cudaEvent_t  copied[2]      = { nullptr, nullptr };
  cudaEvent_t  consumed[2]    = { nullptr, nullptr };
  double*      d_acc64        = nullptr;
};

namespace rg {

  namespace {

    int plan_reserve(rg_spectrum_plan* pl, int max_seg) {
      const size_t need = static_cast<size_t>(pl->grid + max_seg) * pl->nslices * kSliceBins;
      if (need > pl->partial_cap) {
        cudaFree(pl->d_partials);
        pl->d_partials = nullptr;
        RG_CUDA_TRY(cudaMalloc(&pl->d_partials, sizeof(double) * need));
        pl->partial_cap = need;
      }
      if (max_seg > pl->prefix_cap) {
        cudaFree(pl->d_prefix);
        pl->d_prefix = nullptr;
        RG_CUDA_TRY(cudaMalloc(&pl->d_prefix, sizeof(int64_t) * (max_seg + 1)));
        pl->prefix_cap = max_seg;
      }
      return RG_OK;
    }

    // Fixed-point coordinates of the photon bins (FP64 on the host).  Fails if one
    // 512-bin slice spans more than the 32-bit window allows (about 33 decades).
    int plan_prepare_bins(rg_spectrum_plan* pl, double ln_xmin, double dln, int n_nodes,
                          double ln_k0) {
      const double scale = std::ldexp(1.0, kFrac) / dln;
      pl->L              = static_cast<int64_t>(n_nodes - 1) << kFrac;
      const double S     = std::ldexp(1.0, kFrac) / (2.0 * dln);
      pl->Sh             = static_cast<float>(S);
      pl->Sl             = static_cast<float>(S - static_cast<double>(pl->Sh));
      pl->Cfx            = std::llround(S * M_LN2 * 65536.0);
      const size_t         nsb = static_cast<size_t>(pl->nslices) * kSliceBins;
      std::vector<int32_t> hP(nsb, 0);
      std::vector<int64_t> hR(2 * pl->nslices, 0);
      std::vector<uint8_t> hV(std::max(pl->nbins, 1), 0);
      for (int s = 0; s < pl->nslices; ++s) {
        int64_t              pmin = std::numeric_limits<int64_t>::max();
        int64_t              pmax = std::numeric_limits<int64_t>::min();
        std::vector<int64_t> Ps(kSliceBins, 0);
        for (int j = 0; j < kSliceBins; ++j) {
          const int bidx = s * kSliceBins + j;
          if (bidx >= pl->nbins) {
            continue;
          }
          const double e = pl->h_bins[bidx];
          if (!(e > 0.0) || !std::isfinite(e)) {
            continue;
          }
          const double t = (std::log(e) - ln_xmin - ln_k0) * scale;
          if (!(std::fabs(t) < 1e18)) {
            return set_error(RG_ERR_UNSUPPORTED, "photon bin energy out of the supported range");
          }
          Ps[j]    = std::llround(t);
          hV[bidx] = 1;
          pmin     = std::min(pmin, Ps[j]);
          pmax     = std::max(pmax, Ps[j]);
        }
        if (pmin > pmax) { // no valid bin in this slice
          pmin = 0;
          pmax = 0;
        }
        if (static_cast<double>(pmax - pmin) + static_cast<double>(pl->L) > 4294967296.0) {
          return set_error(RG_ERR_UNSUPPORTED,
                           "photon bins of one 512-bin slice span more than the 32-bit table "
                           "window (about 33 decades)");
        }
        for (int j = 0; j < kSliceBins; ++j) {
          const int     bidx = s * kSliceBins + j;
          const int64_t v    = (bidx < pl->nbins && hV[bidx]) ? Ps[j] : pmin;
          hP[s * kSliceBins + j] = static_cast<int32_t>(static_cast<uint32_t>(v & 0xffffffffLL));
        }
        hR[2 * s]     = pmin;
        hR[2 * s + 1] = pmax;
      }
      RG_CUDA_TRY(cudaMemcpy(pl->d_P, hP.data(), sizeof(int32_t) * nsb, cudaMemcpyHostToDevice));
      RG_CUDA_TRY(cudaMemcpy(pl->d_Prange, hR.data(), sizeof(int64_t) * hR.size(),
                             cudaMemcpyHostToDevice));
      RG_CUDA_TRY(cudaMemcpy(pl->d_valid, hV.data(), hV.size(), cudaMemcpyHostToDevice));
      if (pl->nbins) {
        RG_CUDA_TRY(cudaMemcpy(pl->d_ebins, pl->h_bins.data(), sizeof(float) * pl->nbins,
                               cudaMemcpyHostToDevice));
      }
      return RG_OK;
    }

    int create_plan_common(rg_spectrum_plan* pl, const float* bins, int32_t nbins) {
      if (nbins < 0 || (nbins > 0 && !bins)) {
        return set_error(RG_ERR_ARGUMENT, "bins: need nbins >= 0 host values");
      }
      RG_CUDA_TRY(cudaGetDevice(&pl->device));
      pl->nbins = nbins;
      pl->h_bins.assign(bins, bins + nbins);
      pl->nslices = std::max(1, (nbins + kSliceBins - 1) / kSliceBins);
      pl->K       = nbins > kSliceBins ? 16 : std::max(1, (nbins + 31) / 32);
      DeviceContext* ctx = nullptr;
      RG_TRY(context(&ctx));
      pl->grid = ctx->sms * kBlocksPerSM;
      const size_t nsb = static_cast<size_t>(pl->nslices) * kSliceBins;
      RG_CUDA_TRY(cudaMalloc(&pl->d_P, sizeof(int32_t) * nsb));
      RG_CUDA_TRY(cudaMalloc(&pl->d_Prange, sizeof(int64_t) * 2 * pl->nslices));
      RG_CUDA_TRY(cudaMalloc(&pl->d_ebins, sizeof(float) * std::max(nbins, 1)));
      RG_CUDA_TRY(cudaMalloc(&pl->d_valid, std::max(nbins, 1)));
      RG_CUDA_TRY(cudaMalloc(&pl->d_status, sizeof(unsigned)));
      RG_CUDA_TRY(cudaMemset(pl->d_status, 0, sizeof(unsigned)));
      RG_TRY(reference_table(&pl->ref));
      return RG_OK;
    }

    int timed_launch(rg_spectrum_plan* pl, const FusedParams& fp, dim3 grid, size_t smem,
                     cudaStream_t s) {
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
      RG_CUDA_TRY(launch_fused(pl->K, fp, grid, smem, s));
      if (pl->timing) {
        RG_CUDA_TRY(cudaEventRecord(ev.second, s));
        pl->ev_used.push_back(ev);
      }
      return RG_OK;
    }

    // Launches fused + reduce.  `d_off` (device, nseg + 1) may be null for a
    // single segment [0, n_single).  With `acc64` the spectra are added in FP64
    // to acc64 (nseg x nbins) instead of being written to `out`.
    int run_fused(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off,
                  int64_t n_single, int nseg, float* out, cudaStream_t s,
                  double* acc64 = nullptr) {
      if (nseg <= 0 || pl->nbins == 0) {
        return RG_OK;
      }
      if (pl->zero) {
        if (!acc64) {
          RG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * pl->nbins * nseg, s));
        }
        return RG_OK;
      }
      RG_TRY(plan_reserve(pl, nseg));
      const int64_t* d_prefix = nullptr;
      if (d_off) {
        item_prefix_kernel<<<1, 1024, 0, s>>>(d_off, nseg, n_single, pl->d_prefix, pl->d_status);
        RG_CUDA_TRY(cudaGetLastError());
        d_prefix = pl->d_prefix;
      }
      FusedParams fp {};
      int         nslots  = 0;
      bool        aligned = true;
      for (int c = 0; c < kComps; ++c) {
        fp.comp[c] = comp[c];
        fp.slot[c] = -1;
        if (comp[c]) {
          fp.slot[c] = nslots++;
          aligned    = aligned && (reinterpret_cast<uintptr_t>(comp[c]) % 16 == 0);
        }
      }
      fp.nslots      = nslots;
      fp.use_tma     = aligned ? 1 : 0;
      fp.source      = pl->source;
      fp.has_e       = (comp[3] || comp[4] || comp[5]) ? 1 : 0;
      fp.has_w       = comp[9] ? 1 : 0;
      fp.log_spaced  = pl->log_spaced;
      fp.seg_off     = d_off;
      fp.item_prefix = d_prefix;
      fp.n_single    = n_single;
      fp.nseg        = nseg;
      fp.P           = pl->d_P;
      fp.Prange      = pl->d_Prange;
      fp.L           = pl->L;
      fp.Sh          = pl->Sh;
      fp.Sl          = pl->Sl;
      fp.Cfx         = pl->Cfx;
      fp.amp         = pl->amp;
      fp.table       = pl->ref->d_coef;
      fp.partials    = pl->d_partials;
      fp.nslices     = pl->nslices;
      fp.status      = pl->d_status;
      // a single segment with fewer items than blocks uses fewer blocks
      int G = pl->grid;
      if (!d_off) {
        const int64_t items = (n_single + kChunk - 1) / kChunk;
        G = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(items, pl->grid)));
      }
      const bool any = d_off ? true : n_single > 0;
      if (any) {
        RG_TRY(timed_launch(pl, fp, dim3(G, pl->nslices), fused_smem(nslots), s));
      }
      ReduceParams rp {};
      rp.partials    = pl->d_partials;
      rp.item_prefix = d_prefix;
      rp.n_single    = n_single;
      rp.grid        = G;
      rp.nslices     = pl->nslices;
      rp.nseg        = nseg;
      rp.nbins       = pl->nbins;
      rp.ebins       = pl->d_ebins;
      rp.valid       = pl->d_valid;
      rp.status      = pl->d_status;
      rp.out         = out;
      rp.acc64       = acc64;
      dim3 rgrid((pl->nbins + 127) / 128, nseg);
      reduce_partials_kernel<<<rgrid, 128, 0, s>>>(rp);
      RG_CUDA_TRY(cudaGetLastError());
      return RG_OK;
    }

    void particle_comps(const rg_particles* p, const float* out[kComps]) {
      for (int d = 0; d < 3; ++d) {
        out[d]     = p->u[d];
        out[3 + d] = p->e[d];
        out[6 + d] = p->b[d];
      }
      out[9] = p->w;
    }

    int check_particles(const rg_particles* p) {
      if (!p || p->n < 0 || (p->n > 0 && (!p->u[0] || !p->u[1] || !p->u[2]))) {
        return set_error(RG_ERR_ARGUMENT, "particles need U1..U3 device arrays and n >= 0");
      }
      return RG_OK;
    }

    std::mutex& oneshot_mutex() {
      static std::mutex m;
      return m;
    }

  } // namespace

} // namespace rg

extern "C" {

int rg_spectrum_plan_create(const float* bins, int32_t nbins, float B0, float g_syn,
                            float e_syn_at_g_syn, int32_t table_mode, rg_spectrum_plan** plan) {
  rg::clear_error();
  if (!plan) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan pointer");
  }
  *plan = nullptr;
  if (table_mode != RG_TABLE_REFERENCE) {
    return rg::set_error(RG_ERR_UNSUPPORTED, "table mode not available for this entry point");
  }
  if (B0 == 0.0f) {
    return rg::set_error(RG_ERR_ARGUMENT, "B0 must be non-zero");
  }
  auto pl        = std::make_unique<rg_spectrum_plan>();
  pl->table_mode = table_mode;
  pl->source     = rg::kSrcParticles;
  pl->B0         = B0;
  pl->g_syn      = g_syn;
  pl->eps        = e_syn_at_g_syn;
  int st         = rg::create_plan_common(pl.get(), bins, nbins);
  if (st != RG_OK) {
    rg_spectrum_plan_destroy(pl.release());
    return st;
  }
  // e_peak = K0 gamma sqrt(W) with K0 = eps / (g^2 B0); the reference keeps only
  // e_peak > 0, so K0 <= 0 (or not finite) gives an all-zero spectrum.
  const double K0 = static_cast<double>(e_syn_at_g_syn) /
                    (static_cast<double>(g_syn) * g_syn * static_cast<double>(B0));
  pl->zero = !(K0 > 0.0) || !std::isfinite(K0);
  pl->amp  = static_cast<float>(1.0 / static_cast<double>(B0));
  st       = rg::plan_prepare_bins(pl.get(), pl->ref->ln_xmin, pl->ref->dln, pl->ref->n,
                                   pl->zero ? 0.0 : std::log(K0));
  if (st == RG_OK) {
    st = rg::plan_reserve(pl.get(), 1);
  }
  if (st != RG_OK) {
    rg_spectrum_plan_destroy(pl.release());
    return st;
  }
  *plan = pl.release();
  return RG_OK;
}

int rg_spectrum_plan_destroy(rg_spectrum_plan* pl) {
  if (!pl) {
    return RG_OK;
  }
  cudaFree(pl->d_P);
  cudaFree(pl->d_Prange);
  cudaFree(pl->d_ebins);
  cudaFree(pl->d_valid);
  cudaFree(pl->d_status);
  cudaFree(pl->d_partials);
  cudaFree(pl->d_prefix);
  cudaFree(pl->d_plain_acc);
  cudaFree(pl->d_stage[0]);
  cudaFree(pl->d_stage[1]);
  cudaFree(pl->d_acc64);
  for (int b = 0; b < 2; ++b) {
    if (pl->copied[b]) cudaEventDestroy(pl->copied[b]);
    if (pl->consumed[b]) cudaEventDestroy(pl->consumed[b]);
  }
  if (pl->copy_stream) cudaStreamDestroy(pl->copy_stream);
  for (auto* v : { &pl->ev_used, &pl->ev_free }) {
    for (auto& e : *v) {
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
  }
  delete pl;
  return RG_OK;
}

int rg_spectrum_plan_enable_timing(rg_spectrum_plan* pl, int32_t enable) {
  if (!pl) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan");
  }
  pl->timing = enable != 0;
  return RG_OK;
}

int rg_spectrum_plan_kernel_time(rg_spectrum_plan* pl, double* ms, int64_t* launches) {
  if (!pl || !ms) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_plan_kernel_time: bad arguments");
  }
  double total = 0.0;
  if (!pl->ev_used.empty()) {
    RG_CUDA_TRY(cudaEventSynchronize(pl->ev_used.back().second));
  }
  for (auto& e : pl->ev_used) {
    float t = 0.0f;
    RG_CUDA_TRY(cudaEventElapsedTime(&t, e.first, e.second));
    total += t;
  }
  if (launches) {
    *launches = static_cast<int64_t>(pl->ev_used.size());
  }
  pl->ev_free.insert(pl->ev_free.end(), pl->ev_used.begin(), pl->ev_used.end());
  pl->ev_used.clear();
  *ms = total;
  return RG_OK;
}

int rg_spectrum_run_host(rg_spectrum_plan* pl, const rg_particles* p, float* out, void* stream) {
  if (!pl || (!out && pl->nbins > 0) || pl->source != rg::kSrcParticles) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_run_host: bad arguments");
  }
  RG_TRY(rg::check_particles(p));
  if (pl->nbins == 0) {
    return RG_OK;
  }
  auto s = static_cast<cudaStream_t>(stream);
  constexpr int64_t kStageChunk = int64_t(1) << 22; // particles per staged chunk
  if (!pl->d_stage[0]) {
    for (int b = 0; b < 2; ++b) {
      RG_CUDA_TRY(cudaMalloc(&pl->d_stage[b], sizeof(float) * rg::kComps * kStageChunk));
      RG_CUDA_TRY(cudaEventCreateWithFlags(&pl->copied[b], cudaEventDisableTiming));
      RG_CUDA_TRY(cudaEventCreateWithFlags(&pl->consumed[b], cudaEventDisableTiming));
    }
    RG_CUDA_TRY(cudaStreamCreateWithFlags(&pl->copy_stream, cudaStreamNonBlocking));
    RG_CUDA_TRY(cudaMalloc(&pl->d_acc64, sizeof(double) * pl->nbins));
    pl->stage_chunk = kStageChunk;
  }
  const float* host[rg::kComps];
  rg::particle_comps(p, host);
  RG_CUDA_TRY(cudaMemsetAsync(pl->d_acc64, 0, sizeof(double) * pl->nbins, s));
  // staging may still be read by earlier work on `s`
  RG_CUDA_TRY(cudaEventRecord(pl->consumed[0], s));
  RG_CUDA_TRY(cudaEventRecord(pl->consumed[1], s));
  const int64_t n = p->n;
  for (int64_t c = 0, a = 0; a < n; ++c, a += kStageChunk) {
    const int     b = static_cast<int>(c & 1);
    const int64_t m = std::min(kStageChunk, n - a);
    RG_CUDA_TRY(cudaStreamWaitEvent(pl->copy_stream, pl->consumed[b], 0));
    const float* dev[rg::kComps] = {};
    for (int k = 0; k < rg::kComps; ++k) {
      if (host[k]) {
        float* dst = pl->d_stage[b] + k * kStageChunk;
        RG_CUDA_TRY(cudaMemcpyAsync(dst, host[k] + a, sizeof(float) * m, cudaMemcpyHostToDevice,
                                    pl->copy_stream));
        dev[k] = dst;
      }
    }
    RG_CUDA_TRY(cudaEventRecord(pl->copied[b], pl->copy_stream));
    RG_CUDA_TRY(cudaStreamWaitEvent(s, pl->copied[b], 0));
    RG_TRY(rg::run_fused(pl, dev, nullptr, m, 1, out, s, pl->d_acc64));
    RG_CUDA_TRY(cudaEventRecord(pl->consumed[b], s));
  }
  rg::finalize_acc_kernel<<<(pl->nbins + 255) / 256, 256, 0, s>>>(pl->d_acc64, pl->nbins,
                                                                  pl->d_status, out);
  RG_CUDA_TRY(cudaGetLastError());
  return RG_OK;
}

int rg_spectrum_plan_reserve(rg_spectrum_plan* pl, int32_t max_segments) {
  if (!pl || max_segments < 1) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_plan_reserve: bad arguments");
  }
  return rg::plan_reserve(pl, max_segments);
}

int rg_spectrum_plan_check(rg_spectrum_plan* pl, void* stream) {
  if (!pl) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan");
  }
  auto     s  = static_cast<cudaStream_t>(stream);
  unsigned st = 0;
  RG_CUDA_TRY(cudaMemcpyAsync(&st, pl->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  RG_CUDA_TRY(cudaStreamSynchronize(s));
  if (st != rg::kDevOk) {
    RG_CUDA_TRY(cudaMemsetAsync(pl->d_status, 0, sizeof(unsigned), s));
    RG_CUDA_TRY(cudaStreamSynchronize(s));
    if (st & rg::kDevBadOffsets) {
      return rg::set_error(RG_ERR_ARGUMENT,
                           "segment offsets must be non-decreasing, >= 0 and <= the particle count");
    }
    return rg::set_error(RG_ERR_TIMEOUT, "a bounded wait on the GPU gave up (status " +
                                           std::to_string(st) + "); results are invalid");
  }
  return RG_OK;
}

int rg_spectrum_run(const rg_spectrum_plan* plan, const rg_particles* p, float* out,
                    void* stream) {
  if (!plan || (!out && plan->nbins > 0)) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_run: null argument");
  }
  if (plan->source != rg::kSrcParticles) {
    return rg::set_error(RG_ERR_ARGUMENT, "plan was not made for particles");
  }
  RG_TRY(rg::check_particles(p));
  const float* comp[rg::kComps];
  rg::particle_comps(p, comp);
  return rg::run_fused(const_cast<rg_spectrum_plan*>(plan), comp, nullptr, p->n, 1, out,
                       static_cast<cudaStream_t>(stream));
}

int rg_spectrum_run_batched(rg_spectrum_plan* plan, const rg_particles* p,
                            const int64_t* offsets, int32_t nseg, float* out, void* stream) {
  if (!plan || !offsets || nseg < 0 || (!out && nseg > 0 && plan->nbins > 0)) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_run_batched: null argument");
  }
  RG_TRY(rg::check_particles(p));
  const float* comp[rg::kComps];
  rg::particle_comps(p, comp);
  return rg::run_fused(plan, comp, offsets, p->n, nseg, out, static_cast<cudaStream_t>(stream));
}

int rg_spectrum_run_plain(const rg_spectrum_plan* cplan, const rg_particles* p, float* out,
                          void* stream) {
  auto* plan = const_cast<rg_spectrum_plan*>(cplan);
  if (!plan || plan->source != rg::kSrcParticles) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_run_plain: bad arguments");
  }
  RG_TRY(rg::check_particles(p));
  auto s = static_cast<cudaStream_t>(stream);
  if (plan->nbins == 0) {
    return RG_OK;
  }
  if (!plan->d_plain_acc) {
    RG_CUDA_TRY(cudaMalloc(&plan->d_plain_acc, sizeof(double) * plan->nbins));
  }
  RG_CUDA_TRY(cudaMemsetAsync(plan->d_plain_acc, 0, sizeof(double) * plan->nbins, s));
  rg::PlainParams pp {};
  const float*    comp[rg::kComps];
  rg::particle_comps(p, comp);
  for (int c = 0; c < rg::kComps; ++c) {
    pp.comp[c] = comp[c];
  }
  pp.n     = p->n;
  pp.bins  = plan->d_ebins;
  pp.nbins = plan->nbins;
  pp.B0    = plan->B0;
  pp.g_syn = plan->g_syn;
  pp.eps   = plan->eps;
  pp.tx    = plan->ref->d_x;
  pp.ty    = plan->ref->d_y;
  pp.nt    = plan->ref->n;
  pp.xmin  = plan->ref->xmin;
  pp.xmax  = plan->ref->xmax;
  pp.acc   = plan->d_plain_acc;
  rg::DeviceContext* ctx = nullptr;
  RG_TRY(rg::context(&ctx));
  const size_t smem = sizeof(float) * (2 * pp.nt + 2 * pp.nbins);
  if (smem > 200 * 1024) {
    return rg::set_error(RG_ERR_UNSUPPORTED, "plain kernel: too many bins");
  }
  if (smem > 48 * 1024) {
    RG_CUDA_TRY(cudaFuncSetAttribute(rg::plain_spectrum_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
  }
  if (p->n > 0) {
    const int64_t need   = (p->n + 255) / 256;
    const int     blocks = static_cast<int>(std::min<int64_t>(need, ctx->sms * 8));
    rg::plain_spectrum_kernel<<<blocks, 256, smem, s>>>(pp);
    RG_CUDA_TRY(cudaGetLastError());
  }
  rg::f64_to_f32_kernel<<<(plan->nbins + 255) / 256, 256, 0, s>>>(plan->d_plain_acc, out,
                                                                   plan->nbins);
  RG_CUDA_TRY(cudaGetLastError());
  return RG_OK;
}

int rg_synchrotron_spectrum(const rg_particles* p, const float* bins, int32_t nbins, float B0,
                            float g_syn, float e_syn_at_g_syn, float* out, void* stream) {
  // plans are cached by (device, bins, scalars)
  using Key = std::tuple<int, std::vector<float>, float, float, float>;
  static std::map<Key, rg_spectrum_plan*> cache;
  if (nbins < 0 || (nbins > 0 && !bins)) {
    return rg::set_error(RG_ERR_ARGUMENT, "bins: need nbins >= 0 host values");
  }
  int dev = 0;
  RG_CUDA_TRY(cudaGetDevice(&dev));
  Key               key { dev, std::vector<float>(bins, bins + nbins), B0, g_syn, e_syn_at_g_syn };
  rg_spectrum_plan* pl = nullptr;
  {
    std::lock_guard<std::mutex> lock(rg::oneshot_mutex());
    auto                        it = cache.find(key);
    if (it == cache.end()) {
      RG_TRY(rg_spectrum_plan_create(bins, nbins, B0, g_syn, e_syn_at_g_syn, RG_TABLE_REFERENCE,
                                     &pl));
      if (cache.size() >= 32) {
        RG_CUDA_TRY(cudaDeviceSynchronize());
        for (auto& kv : cache) {
          rg_spectrum_plan_destroy(kv.second);
        }
        cache.clear();
      }
      cache.emplace(key, pl);
    } else {
      pl = it->second;
    }
  }
  return rg_spectrum_run(pl, p, out, stream);
}

int rg_synchrotron_spectrum_from_dist(const float* gbeta, const float* f, int32_t ng,
                                      int32_t log_spaced, const float* bins, int32_t nbins,
                                      float g_syn, float e_syn_at_g_syn, float* out,
                                      void* stream) {
  rg::clear_error();
  if (ng < 0 || nbins < 0 || (ng > 0 && (!gbeta || !f)) || (nbins > 0 && !out)) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_synchrotron_spectrum_from_dist: bad arguments");
  }
  auto pl        = std::make_unique<rg_spectrum_plan>();
  pl->source     = rg::kSrcDist;
  pl->log_spaced = log_spaced ? 1 : 0;
  pl->g_syn      = g_syn;
  pl->eps        = e_syn_at_g_syn;
  int st         = rg::create_plan_common(pl.get(), bins, nbins);
  // e_peak(g) = K0 gbeta^2 with K0 = eps / g^2 (synchrotron.hpp:78-79)
  const double K0 = static_cast<double>(e_syn_at_g_syn) / (static_cast<double>(g_syn) * g_syn);
  pl->zero        = !(K0 > 0.0) || !std::isfinite(K0);
  pl->amp         = 1.0f;
  if (st == RG_OK) {
    st = rg::plan_prepare_bins(pl.get(), pl->ref->ln_xmin, pl->ref->dln, pl->ref->n,
                               pl->zero ? 0.0 : std::log(K0));
  }
  auto s = static_cast<cudaStream_t>(stream);
  if (st == RG_OK) {
    const float* comp[rg::kComps] = {};
    comp[0]                       = gbeta;
    comp[1]                       = f;
    st = rg::run_fused(pl.get(), comp, nullptr, ng, 1, out, s);
  }
  if (st == RG_OK) {
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      st = rg::cuda_error(e, "rg_synchrotron_spectrum_from_dist");
    }
  }
  if (st == RG_OK) {
    st = rg_spectrum_plan_check(pl.get(), stream);
  }
  rg_spectrum_plan_destroy(pl.release());
  return st;
}

} // extern "C"

// Device pieces shared by the spectrum forward (spectrum.cu) and adjoint
// (adjoint.cu) kernels: launch geometry, parameters, the per-particle stage
// (kinematics to a fixed-point table coordinate), work items and TMA staging.
//
// Reference: sync::Kernel<D>::OmegaSync_ChiR (synchrotron.hpp:181-232) for the
// kinematics, InterpolateTabulatedFunction<true> (tabulation.hpp:19-53) for the
// table coordinate, sync::KernelFromDist (synchrotron.hpp:72-95) for the
// distribution source.
#pragma once

#include "rg_common.cuh"
#include "rg_internal.hpp"

namespace rg {

  constexpr int kThreads     = 256;
  constexpr int kWarps       = kThreads / 32;
  constexpr int kSliceBins   = 512; // bins per block slice (K <= 16 rows of 32)
  constexpr int kChunk       = 512; // particles per work item
  constexpr int kChunkPad    = kChunk + 4;
  constexpr int kBlocksPerSM = 2;

  // extra status bit: segment offsets were not non-decreasing / within [0, n]
  constexpr unsigned kDevBadOffsets = 4u;
  constexpr unsigned kDevBadIndex   = 8u; // a staging self-check found an out-of-range span; access skipped

  enum Source : int { kSrcParticles = 0, kSrcDist = 1 };
  enum Mode : int { kModeRef = RG_TABLE_REFERENCE, kModeSmooth = RG_TABLE_SMOOTH };

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
    int64_t        L;            // table segments << frac
    float          Sh, Sl;       // 2^frac / (2 dln) as a double-float
    int64_t        Cfx;          // round(S ln2 2^16)
    float          amp;          // 1 / B0 (particles) or 1 (dist)
    // reference mode: 1024 (c0, c1 * 2^127) segments, frac = kFrac
    const float2*  table;
    // smooth mode: hseg Hermite segments + one zero entry, runtime frac
    const float4*  htable;
    int            hseg;
    int            frac;
    double*        partials;     // [(grid + nseg) * nslices * kSliceBins]
    int            accumulate;   // 1: a block adds its sums to its partial row (chunked runs)
    int            nslices;
    unsigned*      status;
    // Always 0 (zero-initialised with the struct).  The kernel builds an integer
    // multiplier from it, so the compiler cannot fold the multiply into a mask:
    // part of the per-eval coordinate arithmetic then runs as IMAD on the FMA
    // pipe instead of on the half-rate integer ALU pipe.
    uint32_t       opaque_zero;
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

  __device__ __forceinline__ int64_t total_items(const int64_t* prefix, int nseg, int64_t n_single) {
    return prefix ? prefix[nseg] : (n_single + kChunk - 1) / kChunk;
  }

  // Block b of G owns items [b n / G, (b+1) n / G); the block holding item i:
  __device__ __forceinline__ int block_of_item(int64_t i, int64_t n_items, int G) {
    return static_cast<int>(((i + 1) * G - 1) / n_items);
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

  // round(S (ln X1 + ln X2) 2^(16 - kShift)), S = Sh + Sl; the exponent part goes
  // through the integer constant Cfx = round(S ln2 2^16).  kShift = 16 gives the
  // coordinate in units of S; smaller shifts keep 16 - kShift more fraction bits.
  template <int kShift = 16>
  __device__ __forceinline__ int64_t fixed_log_sum(ff X1, ff X2, float Sh, float Sl, int64_t Cfx) {
    const LnParts a = ln_parts(X1);
    const LnParts b = ln_parts(X2);
    ff            s = two_sum(a.h, b.h);
    s.lo            = __fadd_rn(s.lo, __fadd_rn(a.l, b.l));
    const float ph  = __fmul_rn(s.hi, Sh);
    const float pe  = __fmaf_rn(s.hi, Sh, -ph);
    const float pl  = __fadd_rn(pe, __fmaf_rn(s.hi, Sl, __fmul_rn(s.lo, Sh)));
    const int64_t q = static_cast<int64_t>(a.e + b.e) * Cfx + __float2ll_rn(__fmul_rn(ph, 65536.0f)) +
                      __float2ll_rn(__fmul_rn(pl, 65536.0f));
    return (q + (int64_t(1) << (kShift - 1))) >> kShift;
  }

  // gamma^2 = 1 + u^2 and W = |gamma E + u x B|^2 - (u.E)^2 as double-floats, so
  // that chiR = sqrt(W) / (gamma B0) and e_peak = K0 gamma sqrt(W).
  __device__ __forceinline__ void kinematics_ff(const float (&v)[kComps], bool has_e, ff& G, ff& W) {
    const float ux = v[0], uy = v[1], uz = v[2];
    const float bx = v[6], by = v[7], bz = v[8];
    ff          u2 = two_prod(ux, ux);
    u2             = ff_add(u2, two_prod(uy, uy));
    u2             = ff_add(u2, two_prod(uz, uz));
    G              = ff_add(ff { 1.0f, 0.0f }, u2);
    const ff cx    = ff_diff_of_products(uy, bz, uz, by);
    const ff cy    = ff_diff_of_products(uz, bx, ux, bz);
    const ff cz    = ff_diff_of_products(ux, by, uy, bx);
    if (!has_e) {
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
  }

  // Per-particle stage for particle data.  Returns false if the particle adds
  // nothing (e_peak <= 0 or not finite, or x outside the table for every bin).
  __device__ __forceinline__ bool particle_stage(const float (&v)[kComps], const FusedParams& p,
                                                 int64_t Pmin, int64_t Pmax, uint32_t& q32,
                                                 float& A) {
    ff G, W;
    kinematics_ff(v, p.has_e != 0, G, W);
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
  __device__ __forceinline__ bool dist_stage(float gb, float f, const FusedParams& p, int64_t Pmin,
                                             int64_t Pmax, uint32_t& q32, float& A) {
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

  // Coordinate given to a particle that adds nothing: every bin lands past the
  // last table segment (T - L in [0, R] for all bins), so it reads a zero entry.
  __device__ __forceinline__ uint32_t dead_coordinate(int64_t Pmin, int64_t L) {
    return static_cast<uint32_t>(Pmin - L);
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

  // One elected thread: 1-D TMA bulk copies of the item's 16-byte-aligned span
  // [a0, a1) of every staged stream into `buf`, completing on `bar`.
  __device__ __forceinline__ void issue_stage(const FusedParams& p, const ItemInfo& I, float* buf,
                                              uint64_t* bar) {
    // self-check: the span lies inside the streams (n_single is the stream length),
    // fits the staging slot, and every source address is 16-byte aligned
    bool ok = I.a0 >= 0 && I.a0 <= I.a1 && I.a1 <= p.n_single && I.a1 - I.a0 <= kChunkPad;
    for (int c = 0; c < kComps && ok; ++c) {
      if (p.slot[c] >= 0) {
        ok = (reinterpret_cast<uintptr_t>(p.comp[c] + I.a0) & 15u) == 0;
      }
    }
    if (!ok) {
      atomicOr(p.status, kDevBadIndex);
    }
    const uint32_t bytes = ok ? static_cast<uint32_t>(I.a1 - I.a0) * 4u : 0u;
    mbar_arrive_expect_tx(bar, bytes * static_cast<uint32_t>(p.nslots));
    if (bytes) {
      for (int c = 0; c < kComps; ++c) {
        if (p.slot[c] >= 0) {
          bulk_g2s(buf + p.slot[c] * kChunkPad, p.comp[c] + I.a0, bytes, bar);
        }
      }
    }
  }

  // Particle gp's components: from the staged span when present, else global.
  __device__ __forceinline__ void load_comps(const FusedParams& p, const ItemInfo& I,
                                             const float* sbuf, int64_t gp, float (&v)[kComps]) {
    const bool in_smem = p.use_tma && gp < I.a1;
    // self-check of the direct loads: gp inside the streams
    const bool in_range = gp >= 0 && gp < p.n_single;
    if (!in_smem && !in_range) {
      atomicOr(p.status, kDevBadIndex);
    }
#pragma unroll
    for (int c = 0; c < kComps; ++c) {
      const float* src = p.comp[c];
      v[c]             = 0.0f;
      if (src) {
        if (in_smem) {
          v[c] = sbuf[p.slot[c] * kChunkPad + (gp - I.a0)];
        } else if (in_range) {
          v[c] = __ldg(src + gp);
        }
      }
    }
  }

  // dL/dw and dL/du of one particle from R1 = sum_b G_b e_b F(x_pb) and
  // R2 = sum_b G_b e_b dF/dln x (x_pb), G_b = dL/dS_b (FP32, recomputed kinematics):
  //   dL/dw = chiR R1,  dL/du = A (R1 d ln chiR / du - R2 d ln e_peak / du).
  __device__ __forceinline__ void particle_gradient(const float (&v)[kComps], const FusedParams& p,
                                                    float R1, float R2, float& gw, float (&gu)[3]) {
    gw = 0.0f;
    gu[0] = gu[1] = gu[2] = 0.0f;
    const float u[3] = { v[0], v[1], v[2] };
    const float E[3] = { v[3], v[4], v[5] };
    const float B[3] = { v[6], v[7], v[8] };
    const float G    = fmaf(u[0], u[0], fmaf(u[1], u[1], fmaf(u[2], u[2], 1.0f)));
    const float c[3] = { ff_diff_of_products(u[1], B[2], u[2], B[1]).hi,
                         ff_diff_of_products(u[2], B[0], u[0], B[2]).hi,
                         ff_diff_of_products(u[0], B[1], u[1], B[0]).hi };
    float       V[3], gW[3], W;
    if (p.has_e) {
      const float gamma = sqrtf(G);
      const float uE    = u[0] * E[0] + u[1] * E[1] + u[2] * E[2];
      for (int d = 0; d < 3; ++d) {
        V[d] = fmaf(gamma, E[d], c[d]);
      }
      W              = V[0] * V[0] + V[1] * V[1] + V[2] * V[2] - uE * uE;
      const float VE = V[0] * E[0] + V[1] * E[1] + V[2] * E[2];
      const float BxV[3] = { B[1] * V[2] - B[2] * V[1], B[2] * V[0] - B[0] * V[2],
                             B[0] * V[1] - B[1] * V[0] };
      for (int d = 0; d < 3; ++d) {
        gW[d] = 2.0f * VE / gamma * u[d] + 2.0f * BxV[d] - 2.0f * uE * E[d];
      }
    } else {
      W = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
      const float Bxc[3] = { B[1] * c[2] - B[2] * c[1], B[2] * c[0] - B[0] * c[2],
                             B[0] * c[1] - B[1] * c[0] };
      for (int d = 0; d < 3; ++d) {
        gW[d] = 2.0f * Bxc[d];
      }
    }
    if (!(W > 0.0f) || !isfinite(W)) {
      return;
    }
    const float chi = p.amp * sqrtf(W / G);
    const float w   = p.has_w ? v[9] : 1.0f;
    const float A   = chi * w;
    const float iW = 0.5f / W, iG = 1.0f / G;
    for (int d = 0; d < 3; ++d) {
      const float dlnchi = gW[d] * iW - u[d] * iG;
      const float dlneps = u[d] * iG + gW[d] * iW;
      gu[d]              = A * (R1 * dlnchi - R2 * dlneps);
    }
    gw = chi * R1;
  }

  // Smooth-table segments staged in shared memory with the cubic's coefficients
  // rescaled to the variable tau' = fraction bits * 2^-23 (tau = tau' 2^(23 - frac),
  // frac in [12, 22]): c1 s, c2 s^2, c3 s^3 with s = 2^(23 - frac), all exact.
  __device__ __forceinline__ void stage_smooth_table(const FusedParams& p, float4* htab, int tid,
                                                     int nthreads) {
    const float s1 = ldexpf(1.0f, 23 - p.frac), s2 = s1 * s1, s3 = s2 * s1;
    for (int i = tid; i <= p.hseg; i += nthreads) {
      const float4 c = p.htable[i];
      htab[i]        = make_float4(c.x, c.y * s1, c.z * s2, c.w * s3);
    }
  }

  // tau' from the fraction bits fb < 2^22: fb read as a denormal float is fb 2^-149
  // exactly, and 2^126 times that is fb 2^-23, exactly (one FMUL, no conversion).
  __device__ __forceinline__ float smooth_tau(uint32_t fb) {
    return __uint_as_float(fb) * 0x1p126f;
  }

  // The FP64 partial row of block b for segment seg (kSliceBins per slice).
  __device__ __forceinline__ double* block_partial(const FusedParams& p, int b, int seg, int slice) {
    return p.partials + (static_cast<int64_t>(b + seg) * p.nslices + slice) * kSliceBins;
  }

} // namespace rg

// Device pieces of the moment spectra (moments.cu, moments_smooth.cu): the particle
// stage with a finer 64-bit table coordinate and the FP64 operands of the moment
// atomics, built with integer instructions (GB300 issues FP64 arithmetic and 64-bit
// conversions at a small fraction of the FP32 rate).
#pragma once

#include "spectrum_common.cuh"

namespace rg {

  __device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }

  // ln x = e ln2 + h + l of a positive finite double-float, as ln_parts computes it
  // (2 atanh((m - 1)/(m + 1)) of the mantissa m in [0.71, 1.42)), with the quotient
  // taken through one approximate reciprocal: its low part comes from the residual
  // f - q d, so an approximate q costs nothing in the double-float result (the
  // residual's own rounding is below 2^-48 absolute).
  __device__ __forceinline__ LnParts ln_parts_rcp(ff x) {
    int adj = 0;
    if (x.hi < 1.17549435e-38f) { // subnormal: scale into the normal range (exact)
      x.hi = __fmul_rn(x.hi, 0x1p64f);
      x.lo = __fmul_rn(x.lo, 0x1p64f);
      adj  = -64;
    }
    const uint32_t bits = __float_as_uint(x.hi);
    int            e    = static_cast<int>(bits >> 23) - 126 + adj; // x.hi = m 2^e, m in [0.5, 1)
    float          m    = __uint_as_float((bits & 0x007fffffu) | 0x3f000000u);
    if (m < 0.70710678f) {
      m = __fmul_rn(m, 2.0f);
      e -= 1;
    }
    const float f  = __fsub_rn(m, 1.0f); // exact
    const ff    d  = two_sum(m, 1.0f);
    const float ri = rcp_approx(d.hi);
    const float q  = __fmul_rn(f, ri);
    const float r  = __fmaf_rn(-q, d.hi, f);
    const float zl = __fmul_rn(__fmaf_rn(-q, d.lo, r), ri);
    const float w  = __fmul_rn(q, q);
    const float poly =
      w * (0.33333334f + w * (0.2f + w * (0.14285715f + w * (0.11111111f + w * 0.09090909f))));
    LnParts o;
    o.e = e;
    o.h = __fmul_rn(2.0f, q);
    o.l = __fadd_rn(__fmaf_rn(o.h, poly, __fmul_rn(2.0f, zl)), __fmul_rn(x.lo, rcp_approx(x.hi)));
    return o;
  }

  // GB300 issues FP64 arithmetic and 64-bit conversions at a small fraction of the FP32
  // rate, so the deposit builds its FP64 values and 64-bit integers with integer
  // instructions only.

  // round(x) as a 64-bit integer for a finite float x with |x| < 2^62.
  __device__ __forceinline__ int64_t float_to_ll_rn(float x) {
    if (fabsf(x) < 4194304.0f) { // |x| < 2^22: round through the 1.5 2^23 shifter
      return static_cast<int64_t>(__float_as_int(__fadd_rn(x, 12582912.0f)) - 0x4B400000);
    }
    const uint32_t b = __float_as_uint(x); // |x| >= 2^22: a multiple of 1/2 ... integral from 2^23
    const int      E = static_cast<int>((b >> 23) & 0xffu);
    const uint64_t m = static_cast<uint64_t>((b & 0x7fffffu) | 0x800000u);
    int64_t        v;
    if (E >= 150) {
      v = static_cast<int64_t>(m << (E - 150));
    } else { // 2^22 <= |x| < 2^23: one fraction bit, round half away from zero
      v = static_cast<int64_t>((m + 1) >> 1);
    }
    return (b >> 31) ? -v : v;
  }

  // The double equal to a float of normal magnitude (either sign), from its bits.
  __device__ __forceinline__ double float_to_double_bits(float a) {
    const uint32_t b = __float_as_uint(a);
    const uint64_t d = (static_cast<uint64_t>(b >> 31) << 63) |
                       (static_cast<uint64_t>(((b >> 23) & 0xffu) + 896u) << 52) |
                       (static_cast<uint64_t>(b & 0x7fffffu) << 29);
    return __longlong_as_double(static_cast<long long>(d));
  }

  // a r as a double for a float a of normal magnitude (either sign) and an integer
  // 0 <= r < 2^30: the 24-bit mantissa times r is an exact integer below 2^54,
  // rounded to 53 bits.
  __device__ __forceinline__ double product_to_double_bits(float a, uint32_t r) {
    if (r == 0) {
      return 0.0;
    }
    const uint32_t b   = __float_as_uint(a);
    const uint64_t P   = static_cast<uint64_t>((b & 0x7fffffu) | 0x800000u) * r;
    int            top = 63 - __clzll(static_cast<long long>(P)); // leading bit position, <= 53
    uint64_t       mant;
    if (top <= 52) {
      mant = P << (52 - top);
    } else { // 54 significant bits: round to nearest (ties up)
      mant = (P + 1) >> 1;
      if (mant >> 53) {
        mant >>= 1;
        ++top;
      }
    }
    // |value| = P 2^(E - 150) with E the float's biased exponent
    const int64_t  e = static_cast<int64_t>(top) + static_cast<int64_t>((b >> 23) & 0xffu) - 150 + 1023;
    const uint64_t d = (static_cast<uint64_t>(b >> 31) << 63) | (static_cast<uint64_t>(e) << 52) |
                       (mant & ((uint64_t(1) << 52) - 1));
    return __longlong_as_double(static_cast<long long>(d));
  }

  // FP64 atomic add of a float: values of normal magnitude take the integer-built
  // operand, subnormals the FP64 pipe, zeros nothing.
  __device__ __forceinline__ void red_add_float(double* dst, float v) {
    const float m = fabsf(v);
    if (m >= 1.17549435e-38f) {
      atomicAdd(dst, float_to_double_bits(v));
    } else if (m > 0.0f) {
      atomicAdd(dst, static_cast<double>(v));
    }
  }

  // G = 1 + u^2 and W = |u x B|^2 (no E field) as double-floats (relative error ~2^-46; a
  // host emulation over 2e6 random and nearly parallel u, B: 1e-14 and 2e-13), in
  // fewer operations than kinematics_ff: squares and products are exact pairs, sums of
  // positive terms run two_sum on the high parts only with the low parts added plainly, and
  // the pairs are normalised once at the end.
  __device__ __forceinline__ ff diff_of_products_pair(float a, float b, float c, float d) {
    const float p  = __fmul_rn(a, b), q = __fmul_rn(c, d);
    const float ep = __fmaf_rn(a, b, -p), eq = __fmaf_rn(c, d, -q);
    const ff    r  = two_sum(p, -q);
    // normalised: when p and q nearly cancel, the remainders carry the whole value
    return fast_two_sum(r.hi, __fadd_rn(r.lo, __fsub_rn(ep, eq)));
  }

  __device__ __forceinline__ void kinematics_noe_ff(const float (&v)[kComps], ff& G, ff& W) {
    const float ux = v[0], uy = v[1], uz = v[2];
    const float x2 = __fmul_rn(ux, ux), y2 = __fmul_rn(uy, uy), z2 = __fmul_rn(uz, uz);
    const ff    s  = two_sum(x2, y2);
    const ff    t  = two_sum(s.hi, z2);
    const float lo = __fadd_rn(__fadd_rn(__fadd_rn(__fmaf_rn(ux, ux, -x2), __fmaf_rn(uy, uy, -y2)),
                                         __fadd_rn(__fmaf_rn(uz, uz, -z2), s.lo)),
                               t.lo);
    const ff g = two_sum(1.0f, t.hi);
    G          = fast_two_sum(g.hi, __fadd_rn(g.lo, lo));
    const float bx = v[6], by = v[7], bz = v[8];
    const ff    cx = diff_of_products_pair(uy, bz, uz, by);
    const ff    cy = diff_of_products_pair(uz, bx, ux, bz);
    const ff    cz = diff_of_products_pair(ux, by, uy, bx);
    // c^2 = hi^2 + (error of hi^2 + 2 hi lo)
    const float hx = __fmul_rn(cx.hi, cx.hi), hy = __fmul_rn(cy.hi, cy.hi), hz = __fmul_rn(cz.hi, cz.hi);
    const float lx = __fmaf_rn(2.0f * cx.hi, cx.lo, __fmaf_rn(cx.hi, cx.hi, -hx));
    const float ly = __fmaf_rn(2.0f * cy.hi, cy.lo, __fmaf_rn(cy.hi, cy.hi, -hy));
    const float lz = __fmaf_rn(2.0f * cz.hi, cz.lo, __fmaf_rn(cz.hi, cz.hi, -hz));
    const ff    sw = two_sum(hx, hy);
    const ff    tw = two_sum(sw.hi, hz);
    W              = fast_two_sum(tw.hi, __fadd_rn(__fadd_rn(__fadd_rn(lx, ly), __fadd_rn(lz, sw.lo)), tw.lo));
  }

  // The particle stage of this path: the kinematics and amplitude of particle_stage,
  // with the table coordinate Q = round(2^(kFrac + 8) (ln gamma + ln sqrt W) / dln)
  // as a 64-bit integer (8 more fraction bits than the fused kernel's).  ln G + ln W
  // is one logarithm of the product G W wherever that is a normal float.  The particle
  // adds nothing unless Pmin - L < Q <= Pmax.
  __device__ __forceinline__ bool moment_particle_stage(const float (&v)[kComps], const FusedParams& p,
                                                        int64_t Pmin, int64_t Pmax, int64_t L, int64_t& Q,
                                                        float& A) {
    ff G, W;
    if (p.has_e) {
      kinematics_ff(v, true, G, W);
    } else {
      kinematics_noe_ff(v, G, W);
    }
    if (!(W.hi > 0.0f) || !isfinite(W.hi) || !isfinite(G.hi)) {
      return false;
    }
    const ff X = ff_mul(G, W);
    int      e;
    ff       s;
    if (X.hi >= 1.17549435e-38f && X.hi <= 3.0e38f) {
      const LnParts a = ln_parts_rcp(X);
      e               = a.e;
      s               = ff { a.h, a.l };
    } else {
      const LnParts a = ln_parts_rcp(G);
      const LnParts b = ln_parts_rcp(W);
      e               = a.e + b.e;
      s               = two_sum(a.h, b.h);
      s.lo            = __fadd_rn(s.lo, __fadd_rn(a.l, b.l));
    }
    const float   ph = __fmul_rn(s.hi, p.Sh);
    const float   pe = __fmaf_rn(s.hi, p.Sh, -ph);
    const float   pl = __fadd_rn(pe, __fmaf_rn(s.hi, p.Sl, __fmul_rn(s.lo, p.Sh)));
    const int64_t q  = static_cast<int64_t>(e) * p.Cfx + float_to_ll_rn(__fmul_rn(ph, 65536.0f)) +
                      float_to_ll_rn(__fmul_rn(pl, 65536.0f));
    Q = (q + 128) >> 8;
    if (Q <= Pmin - L || Q > Pmax) {
      return false;
    }
    // W / G within an ulp (approximate reciprocal and one correction), then sqrt
    const float rg = rcp_approx(G.hi);
    float       t  = __fmul_rn(W.hi, rg);
    t              = __fmaf_rn(__fmaf_rn(-t, G.hi, W.hi), rg, t);
    A              = p.amp * sqrtf(t);
    if (p.has_w) {
      A *= v[9];
    }
    return isfinite(A);
  }

  // Largest s in [0, nseg] with off[s] <= i (off non-decreasing).
  __device__ __forceinline__ int segment_of(const int64_t* off, int nseg, int64_t i) {
    int lo = 0, hi = nseg;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= i) {
        lo = mid;
      } else {
        hi = mid - 1;
      }
    }
    return lo;
  }

} // namespace rg

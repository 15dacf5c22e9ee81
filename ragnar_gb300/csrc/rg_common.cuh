// Shared device-side helpers for the ragnar_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace rg {

  // Bit flags written to a plan's device status word.
  enum DeviceStatus : unsigned {
    kDevOk            = 0u,
    kDevTimeoutStage  = 1u, // an mbarrier wait on a particle-stream copy gave up
    kDevTimeoutDrain  = 2u, // the drain wait after a timeout gave up as well
  };

  // Upper bound on mbarrier polls before a wait is abandoned (each poll is a
  // try_wait with a hardware time hint, so this is on the order of seconds).
  constexpr unsigned kWaitLimit = 1u << 22;

  // ---- shared-memory barrier + bulk copy (Blackwell async proxy) -----------

  __device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
  }

  __device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
  }

  __device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  __device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }

  __device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile(
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
  }

  __device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
  }

  // 1-D bulk copy global -> shared, completion signalled on `bar` (transaction
  // bytes).  dst, src and bytes must be multiples of 16.
  __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                           uint64_t* bar) {
    asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
        "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
  }

  __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
    return ok != 0;
  }

  // Bounded wait for phase `parity` of `bar`.  Returns false if it gave up.
  __device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                    unsigned limit = kWaitLimit) {
    for (unsigned it = 0; it < limit; ++it) {
      if (mbar_try_wait(bar, parity)) {
        return true;
      }
    }
    return false;
  }

  // Hardware base-2 logarithm (PTX lg2.approx.ftz.f32) for arguments known to be
  // normal floats: no denormal-input handling around the MUFU operation.
  __device__ __forceinline__ float lg2_normal(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
  }

  // ---- error-free transformations (double-float arithmetic) ----------------

  struct ff {
    float hi, lo;
  };

  __device__ __forceinline__ ff two_sum(float a, float b) {
    const float s  = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e  = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return { s, e };
  }

  __device__ __forceinline__ ff fast_two_sum(float a, float b) { // |a| >= |b|
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return { s, e };
  }

  __device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return { p, __fmaf_rn(a, b, -p) };
  }

  __device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, s.lo);
  }

  __device__ __forceinline__ ff ff_neg(ff a) {
    return { -a.hi, -a.lo };
  }

  __device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
  }

  __device__ __forceinline__ ff ff_sqr(ff a) {
    return ff_mul(a, a);
  }

  // a*b - c*d as a double-float; the products are exact pairs.
  __device__ __forceinline__ ff ff_diff_of_products(float a, float b, float c, float d) {
    return ff_add(two_prod(a, b), ff_neg(two_prod(c, d)));
  }

} // namespace rg

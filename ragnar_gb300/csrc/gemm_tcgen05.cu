// Batched SynchrotronSpectrumFromDist on the Blackwell tensor cores (sm_103a).
//
// Reference: SynchrotronSpectrumFromDist (synchrotron.cpp:69-105) evaluates, per
// distribution, S[e] = sum_g f_g e J_g F(e / e_peak(g)) (synchrotron.hpp:72-95),
// J_g = gbeta_g for log-spaced gamma bins, e_peak(g) = eps gbeta_g^2 / g_syn^2.
// The kernel matrix K[e, g] = J_g F(e / e_peak(g)) depends only on the bins, so
// many distributions f[d, g] give one GEMM:  S[d, e] = e * sum_g f[d, g] K[e, g].
//
// Precision: FP32 operands are split into BF16 terms (x = h + m + l, each the
// BF16 rounding of the remainder; for FP32 input every step is exact in FP32) and
// the products are summed in one GEMM, accumulated in FP32 in tensor memory:
//   6 products  (h.h + h.m + m.h + h.l + l.h + m.m): ~1e-8 relative per product (default)
//   3 products  (h.h + h.m + m.h):                  ~1e-5 relative per product (fast)
// The dominant h.h product accumulates in its own TMEM accumulator and the
// correction products in a second one; the epilogue adds the two.  The FP32
// accumulator is rounded once per MMA, so keeping the small corrections out of
// the large running sum bounds the accumulation error by the h.h steps alone
// (4 per 64 gamma bins) instead of by all of them.
//
// GEMM: C[M x N] = A[M x K] . B[N x K]^T.  The right operand (the kernel matrix,
// split once per plan) is stored as BF16 terms [h | m | l] per row and streamed
// by TMA (cp.async.bulk.tensor, 128-byte swizzle) through a ring of k blocks.  The
// left operand (the distributions, FP32) is read by eight converter warps, split
// exactly into its BF16 terms and written straight into 128-byte-swizzled shared
// tiles, double-buffered per 64-gamma block: no split kernel and no BF16 copy in
// HBM.  The k loop runs gamma block outer, right term inner, and every product of
// a resident right term runs before its ring stage is released, so each converted
// left tile and each streamed right tile serves every product that uses it.  One
// thread issues tcgen05.mma (M 128, N = tile width, K 16) and commits each ring
// stage back to the producer and each left buffer back to the converters; after
// the last commit warps 0..7 read both accumulators with tcgen05.ld (warp w owns
// TMEM lanes 32(w%4)..+31, half w/4 of the columns), scale them by col_scale,
// write them into 128-byte-swizzled 32 x 128 boxes in the ring's shared memory,
// and one thread stores the boxes with TMA tensor stores (direct stores when the
// output is not 16-byte aligned).  Every mbarrier wait is bounded; a wait that
// gives up records the status word, and the CTA still frees its tensor memory.
#include "rg_common.cuh"
#include "rg_internal.hpp"

#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

namespace rg {

  namespace {

    constexpr int kBM       = 128;
    constexpr int kBK       = 64; // bf16 elements = 128 bytes: one swizzle row
    constexpr int kUmmaK    = 16;
    constexpr int kGemmThreads = 320; // warp 0 TMA, warp 1 MMA, warps 2..9 convert the left operand

    // Tile shapes the autotuner chooses from: N width of the CTA tile (M is 128)
    // and the depth of the TMA ring.  Two FP32 accumulators of `bn` TMEM columns.
    struct GemmConfig {
      int bn, stages;
    };
    constexpr GemmConfig kConfigs[] = { { 256, 4 }, { 128, 6 }, { 128, 4 } };
    constexpr int        kNumConfigs = 3;
    constexpr unsigned kDevGemmTimeout = 8u;
    // Products of stored terms (0 h, 1 m, 2 l): every (left L, right R) with L + R < nstore,
    // i.e. h.h, m.h, l.h, h.m, m.m, h.l for 3 stored terms and h.h, m.h, h.m for 2.  The
    // ring streams each right term of a gamma block once, and every product that uses it
    // runs while it is resident.

    __device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y,
                                                uint64_t* bar) {
      asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
    }

    // Tensor store of one 32-column x 128-row FP32 box (128-byte swizzled in shared memory)
    // at (x, y, z) of a 3-D map; out-of-range rows and columns are not written.
    __device__ __forceinline__ void tma_store_3d(const CUtensorMap* tm, const void* src, int x, int y, int z) {
      asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     reinterpret_cast<uint64_t>(tm)),
                   "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
                   : "memory");
    }

    // Commits the issued tensor stores and waits until they have completed.
    __device__ __forceinline__ void tma_store_commit_and_wait() {
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }

    // Shared-memory matrix descriptor, K-major operand in the 128-byte swizzle
    // layout: 8-row atoms of 128-byte rows, atoms 1024 bytes apart (SBO), the
    // leading offset unused for swizzled K-major layouts (encoded 1).
    __device__ __forceinline__ uint64_t smem_desc_sw128(const void* p) {
      const uint64_t addr = smem_u32(p);
      uint64_t       d    = (addr & 0x3FFFFull) >> 4;
      d |= uint64_t(1) << 16;           // leading byte offset (unused), encoded 16 >> 4
      d |= uint64_t(1024 >> 4) << 32;   // stride byte offset: 8 rows x 128 B
      d |= uint64_t(1) << 46;           // descriptor version for tcgen05
      d |= uint64_t(2) << 61;           // swizzle: 128 B
      return d;
    }

    // Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major,
    // N = bn, M = 128.
    template <int BN>
    constexpr uint32_t idesc() {
      return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(BN >> 3) << 17) | (uint32_t(kBM >> 4) << 24);
    }

    __device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                             uint32_t accumulate) {
      asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
    }

    __device__ __forceinline__ void mma_commit(uint64_t* bar) {
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                   : "memory");
    }

    __device__ __forceinline__ void tc_fence_after() {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }

    __device__ __forceinline__ void tc_fence_before() {
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }

    // 32 consecutive FP32 columns of this thread's TMEM lane.
    __device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
      uint32_t r[32];
      asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
        "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
        "[%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        v[i] = __uint_as_float(r[i]);
      }
    }

    // Both accumulators' 32 columns at once: two loads, one wait.
    __device__ __forceinline__ void tmem_ld32x2(uint32_t ta, uint32_t tb, float (&v)[32], float (&w)[32]) {
      uint32_t r[32], q[32];
      asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
        "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
        "[%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(ta));
      asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
        "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
        "[%32];"
        : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]), "=r"(q[4]), "=r"(q[5]), "=r"(q[6]), "=r"(q[7]),
          "=r"(q[8]), "=r"(q[9]), "=r"(q[10]), "=r"(q[11]), "=r"(q[12]), "=r"(q[13]), "=r"(q[14]),
          "=r"(q[15]), "=r"(q[16]), "=r"(q[17]), "=r"(q[18]), "=r"(q[19]), "=r"(q[20]), "=r"(q[21]),
          "=r"(q[22]), "=r"(q[23]), "=r"(q[24]), "=r"(q[25]), "=r"(q[26]), "=r"(q[27]), "=r"(q[28]),
          "=r"(q[29]), "=r"(q[30]), "=r"(q[31])
        : "r"(tb));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        v[i] = __uint_as_float(r[i]);
        w[i] = __uint_as_float(q[i]);
      }
    }

    // Splits v into BF16 terms h, m, l (each the rounding of the remainder).
    __device__ __forceinline__ void split3(double v, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
      h         = __double2bfloat16(v);
      double r  = v - static_cast<double>(__bfloat162float(h));
      m         = __double2bfloat16(r);
      r        -= static_cast<double>(__bfloat162float(m));
      l         = __double2bfloat16(r);
    }

    // The same for an FP32 value: h is within a binade of v, so v - h and the next
    // remainder are exact in FP32 (at most 17 significant bits).
    __device__ __forceinline__ void split3f(float v, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
      h       = __float2bfloat16_rn(v);
      float r = __fsub_rn(v, __bfloat162float(h));
      m       = __float2bfloat16_rn(r);
      r       = __fsub_rn(r, __bfloat162float(m));
      l       = __float2bfloat16_rn(r);
    }

    __device__ __forceinline__ uint32_t pack_bf16x2(__nv_bfloat16 a, __nv_bfloat16 b) {
      return static_cast<uint32_t>(__bfloat16_as_ushort(a)) | (static_cast<uint32_t>(__bfloat16_as_ushort(b)) << 16);
    }

    struct GemmArgs {
      int          M, N;
      int          kpt;        // k blocks of 64 (padded K / kBK)
      int          nprod;      // products: 6 or 3 (the first is h.h, accumulator 0)
      int          nstore;     // BF16 terms of each operand: 3 (h, m, l) or 2 (h, m)
      const float* left;       // M x cols FP32 left operand, row stride ld
      int          cols, ld;
      const float* left_scale; // per left column (nullable)
      float*       C;
      int          ldc;
      const float* col_scale;  // per output column (nullable)
      unsigned*    status;
      int          splits;       // K split into this many gamma-block ranges (blockIdx.z); 1: none
      int64_t      split_stride; // elements between the C slices of consecutive ranges
      int          c_tma;        // 1: the epilogue stores C tiles with TMA through tmC
    };

    // Warps 2..9 turn the FP32 left operand into BF16 terms in shared memory.
    constexpr int      kConvWarps  = 8;
    constexpr int      kConvThreads = 32 * kConvWarps;
    constexpr uint32_t kBytesTerm  = kBM * kBK * 2; // one 128 x 64 BF16 term tile (16 KB)

    template <int kBN, int kStages>
    __global__ void __launch_bounds__(kGemmThreads, 1)
      gemm_bf16_tn_kernel(const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmC,
                          const __grid_constant__ GemmArgs g) {
      constexpr uint32_t kBytesB   = kBN * kBK * 2;
      constexpr uint32_t kTmemCols = 2 * kBN; // two accumulators
      constexpr uint32_t kIdesc    = idesc<kBN>();
      extern __shared__ __align__(1024) unsigned char smem_raw[];
      // 1024-byte alignment of the swizzled tiles
      unsigned char* smem = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
      unsigned char* sB = smem;                      // kStages right-operand tiles (TMA)
      unsigned char* sA = smem + kStages * kBytesB;  // 2 buffers x nstore left-operand term tiles
      __shared__ uint64_t b_full[kStages], b_empty[kStages], a_full[2], a_empty[2], done_bar;
      __shared__ uint32_t tmem_slot;

      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      const int n0 = blockIdx.x * kBN, m0 = blockIdx.y * kBM;
      // this CTA's gamma blocks [gb0, gb0 + nloc) (all of them unless K is split)
      const int gb0  = static_cast<int>(static_cast<int64_t>(blockIdx.z) * g.kpt / g.splits);
      const int nloc = static_cast<int>(static_cast<int64_t>(blockIdx.z + 1) * g.kpt / g.splits) - gb0;
      const int nk   = g.nstore * nloc; // ring: gamma block outer, right term inner

      if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
          mbar_init(&b_full[s], 1);
          mbar_init(&b_empty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
          mbar_init(&a_full[s], kConvWarps);
          mbar_init(&a_empty[s], 1);
        }
        mbar_init(&done_bar, 1);
        fence_mbar_init();
      }
      if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
      }
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      const uint32_t tmem_d = tmem_slot;

      int issued = 0; // right-operand k blocks handed to TMA
      if (warp == 0 && lane == 0) {
        // ---- producer: TMA of the right operand into the ring ---------------------------
        for (int kb = 0; kb < nk; ++kb, ++issued) {
          const int      s  = kb % kStages;
          const uint32_t ph = static_cast<uint32_t>(kb / kStages) & 1u;
          if (kb >= kStages && !mbar_wait_bounded(&b_empty[s], ph ^ 1u)) {
            atomicOr(g.status, kDevGemmTimeout);
            break;
          }
          // right term r of gamma block gb0 + i
          const int i = kb / g.nstore, r = kb - i * g.nstore;
          mbar_arrive_expect_tx(&b_full[s], kBytesB);
          tma_load_2d(sB + s * kBytesB, &tmB, (r * g.kpt + gb0 + i) * kBK, n0, &b_full[s]);
        }
      } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer -------------------------------------------------------------------
        bool     ok      = true;
        uint32_t started = 0; // bit a: accumulator a holds a partial sum
        for (int i = 0; i < nloc && ok; ++i) {
          const int ab = i & 1;
          if (!mbar_wait_bounded(&a_full[ab], static_cast<uint32_t>(i >> 1) & 1u)) {
            atomicOr(g.status, kDevGemmTimeout);
            break;
          }
          for (int r = 0; r < g.nstore; ++r) {
            const int      kb = i * g.nstore + r;
            const int      s  = kb % kStages;
            const uint32_t ph = static_cast<uint32_t>(kb / kStages) & 1u;
            if (!mbar_wait_bounded(&b_full[s], ph)) {
              atomicOr(g.status, kDevGemmTimeout);
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t db = smem_desc_sw128(sB + s * kBytesB);
            for (int L = 0; L + r < g.nstore; ++L) {
              const uint64_t da  = smem_desc_sw128(sA + (ab * g.nstore + L) * kBytesTerm);
              const uint32_t acc = (L == 0 && r == 0) ? 0u : 1u; // h.h alone in accumulator 0
#pragma unroll
              for (int k = 0; k < kBK / kUmmaK; ++k) {
                // advance along K inside the 128-byte swizzle row: 32 bytes = 2 in the >> 4 field
                mma_bf16(tmem_d + acc * kBN, da + uint64_t(2 * k), db + uint64_t(2 * k), kIdesc,
                         ((started >> acc) & 1u) | (k > 0 ? 1u : 0u));
              }
              started |= 1u << acc;
            }
            mma_commit(&b_empty[s]); // the stage is free once every product using it completes
          }
          mma_commit(&a_empty[ab]); // the left tiles of gamma block gb are free once these MMAs complete
        }
        mma_commit(&done_bar);
      } else if (warp >= 2) {
        // ---- converters: FP32 left operand -> BF16 terms, 128-byte swizzled -----------------
        const int  ct  = threadIdx.x - 64;
        const bool vec = (g.ld & 3) == 0 && (reinterpret_cast<uintptr_t>(g.left) & 15) == 0;
        for (int i = 0; i < nloc; ++i) {
          const int gb = gb0 + i, ab = i & 1;
          if (i >= 2 &&
              !__all_sync(0xffffffffu, mbar_wait_bounded(&a_empty[ab], static_cast<uint32_t>((i - 2) >> 1) & 1u))) {
            if (lane == 0) {
              atomicOr(g.status, kDevGemmTimeout);
            }
            break;
          }
          unsigned char* tile = sA + ab * g.nstore * kBytesTerm;
          // unit = 8 consecutive k of one row (a 16-byte chunk of each term tile); all of
          // this thread's loads are issued before any is used, to keep them in flight together
          constexpr int kUnits = (kBM * kBK / 8) / kConvThreads;
          float         v[kUnits][8];
#pragma unroll
          for (int i = 0; i < kUnits; ++i) {
            const int    u = ct + kConvThreads * i;
            const int    row = m0 + (u >> 3), k0 = gb * kBK + (u & 7) * 8;
            const float* src = g.left + static_cast<int64_t>(row) * g.ld + k0;
            if (row < g.M && vec && k0 + 8 <= g.cols) {
              const float4 p0 = __ldg(reinterpret_cast<const float4*>(src));
              const float4 p1 = __ldg(reinterpret_cast<const float4*>(src) + 1);
              v[i][0] = p0.x; v[i][1] = p0.y; v[i][2] = p0.z; v[i][3] = p0.w;
              v[i][4] = p1.x; v[i][5] = p1.y; v[i][6] = p1.z; v[i][7] = p1.w;
            } else {
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                v[i][j] = (row < g.M && k0 + j < g.cols) ? __ldg(src + j) : 0.0f;
              }
            }
          }
#pragma unroll
          for (int i = 0; i < kUnits; ++i) {
            const int u = ct + kConvThreads * i;
            const int r = u >> 3, c = u & 7, k0 = gb * kBK + c * 8;
            __nv_bfloat16 h[8], m[8], l[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              float x = v[i][j];
              if (g.left_scale && k0 + j < g.cols) {
                x = __fmul_rn(x, __ldg(g.left_scale + k0 + j));
              }
              split3f(x, h[j], m[j], l[j]);
            }
            // 128-byte swizzle: 16-byte chunk c of row r sits at chunk c ^ (r % 8)
            const uint32_t off = static_cast<uint32_t>((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
            *reinterpret_cast<uint4*>(tile + off) =
              make_uint4(pack_bf16x2(h[0], h[1]), pack_bf16x2(h[2], h[3]), pack_bf16x2(h[4], h[5]), pack_bf16x2(h[6], h[7]));
            *reinterpret_cast<uint4*>(tile + kBytesTerm + off) =
              make_uint4(pack_bf16x2(m[0], m[1]), pack_bf16x2(m[2], m[3]), pack_bf16x2(m[4], m[5]), pack_bf16x2(m[6], m[7]));
            if (g.nstore > 2) {
              *reinterpret_cast<uint4*>(tile + 2 * kBytesTerm + off) =
                make_uint4(pack_bf16x2(l[0], l[1]), pack_bf16x2(l[2], l[3]), pack_bf16x2(l[4], l[5]), pack_bf16x2(l[6], l[7]));
            }
          }
          // generic-proxy stores -> visible to the tensor core's async-proxy reads
          fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(&a_full[ab]);
          }
        }
      }
      __syncwarp();

      // ---- epilogue: TMEM -> registers -> global (warps 0..3 own TMEM lanes 0..127) -----------
      // tcgen05.ld is warp-collective: every thread takes the same branch
      const bool done = __syncthreads_and(mbar_wait_bounded(&done_bar, 0)) != 0;
      if (!done && threadIdx.x == 0) {
        atomicOr(g.status, kDevGemmTimeout);
        // a wait gave up: let the copies still in flight land before the CTA exits
        for (int s = 0; s < kStages && s < issued; ++s) {
          const int last = s + ((issued - 1 - s) / kStages) * kStages;
          mbar_wait_bounded(&b_full[s], static_cast<uint32_t>(last / kStages) & 1u);
        }
      }
      tc_fence_after();
      // the tile's output column scales (1 when there are none), staged in the left operand's
      // shared memory, which no MMA reads any more
      float* s_scale = reinterpret_cast<float*>(sA);
      if (done) {
        for (int i = threadIdx.x; i < kBN; i += kGemmThreads) {
          const int col = n0 + i;
          s_scale[i]    = !g.col_scale ? 1.0f : (col < g.N ? __ldg(g.col_scale + col) : 0.0f);
        }
      }
      __syncthreads();
      // warps 0..7: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows) for half w / 4 of the columns
      if (done && warp < 8) {
        const int      q         = warp & 3, half = warp >> 2;
        const int      r         = q * 32 + lane; // row within the tile
        const int      row       = m0 + r;
        const bool     two       = g.nprod > 1;   // accumulator 1 was written
        const uint32_t lane_base = static_cast<uint32_t>(q * 32) << 16;
        constexpr int  kHalf     = kBN / 64;      // 32-column chunks per half
#pragma unroll 1
        for (int c = half * kHalf; c < (half + 1) * kHalf; ++c) {
          float v[32];
          if (nk == 0) { // an empty gamma range (more ranges than gamma blocks) adds zero
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              v[j] = 0.0f;
            }
          } else if (two) {
            float w[32];
            tmem_ld32x2(tmem_d + lane_base + static_cast<uint32_t>(c * 32),
                        tmem_d + lane_base + static_cast<uint32_t>(kBN + c * 32), v, w);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              v[j] += w[j];
            }
          } else {
            tmem_ld32(tmem_d + lane_base + static_cast<uint32_t>(c * 32), v);
          }
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            v[j] *= s_scale[c * 32 + j];
          }
          const int col0 = n0 + c * 32;
          if (g.c_tma) {
            // box c of the ring's shared memory: 128 rows of 128 bytes, 16-byte piece p of
            // row r at piece p ^ (r % 8) (the map's 128-byte swizzle; conflict-free stores)
            unsigned char* box = sB + c * (kBM * 128);
#pragma unroll
            for (int p4 = 0; p4 < 8; ++p4) {
              *reinterpret_cast<float4*>(box + r * 128 + ((p4 ^ (r & 7)) << 4)) =
                make_float4(v[4 * p4], v[4 * p4 + 1], v[4 * p4 + 2], v[4 * p4 + 3]);
            }
          } else if (row < g.M && col0 < g.N) {
            float* dst = g.C + blockIdx.z * g.split_stride + static_cast<int64_t>(row) * g.ldc + col0;
            if (col0 + 32 <= g.N && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
#pragma unroll
              for (int j = 0; j < 32; j += 4) {
                *reinterpret_cast<float4*>(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
              }
            } else {
#pragma unroll
              for (int j = 0; j < 32; ++j) {
                if (col0 + j < g.N) {
                  dst[j] = v[j];
                }
              }
            }
          }
        }
      }
      if (g.c_tma) {
        // generic-proxy writes of the boxes -> visible to the tensor store; one thread stores
        fence_proxy_async_smem();
        __syncthreads();
        if (done && threadIdx.x == 0) {
          for (int c = 0; c < kBN / 32; ++c) {
            if (n0 + c * 32 < g.N) {
              tma_store_3d(&tmC, sB + c * (kBM * 128), n0 + c * 32, m0, static_cast<int>(blockIdx.z));
            }
          }
          tma_store_commit_and_wait(); // the boxes are read and C written before the CTA exits
        }
      }
      tc_fence_before();
      __syncthreads();
      if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(kTmemCols)
                     : "memory");
      }
    }

    // Split-K reduction: C[r, c] = sum over ranges z = 0, 1, ... (in that order) of the
    // range's slice; deterministic.
    __global__ void splitk_reduce_kernel(const float* __restrict__ ws, int splits, int64_t stride, int M, int N,
                                         float* __restrict__ C, int ldc) {
      const int64_t n = static_cast<int64_t>(M) * N;
      for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
           i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float t = ws[i];
        for (int z = 1; z < splits; ++z) {
          t = __fadd_rn(t, ws[z * stride + i]);
        }
        const int64_t r = i / N, c = i - r * N;
        C[r * ldc + c] = t;
      }
    }

    // ---- operand preparation -------------------------------------------------------------

    // Kernel matrix in FP64: K[e][g] = J_g F(e_b / e_peak(g)) with the plan's table,
    // written as the right operand (rows e) and its transpose (rows g).
    struct KParams {
      const float*   gbeta; // ng
      const float*   ebins; // nbins
      int            ng, nbins, log_spaced;
      double         ln_k0, ln_xmin, dln;
      int            mode, nseg;
      const float2*  ref;   // reference segments (c0, c1 * 2^127)
      const float4*  hcoef; // smooth segments
      double*        K;     // nbins x ng
    };

    __global__ void kernel_matrix_kernel(const __grid_constant__ KParams p) {
      const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= static_cast<int64_t>(p.nbins) * p.ng) {
        return;
      }
      const int    e = static_cast<int>(i / p.ng), g = static_cast<int>(i % p.ng);
      const double gb = p.gbeta[g], eb = p.ebins[e];
      double       K  = 0.0;
      if (gb != 0.0 && eb > 0.0 && isfinite(gb) && isfinite(eb)) {
        const double t = (log(eb) - p.ln_k0 - 2.0 * log(fabs(gb)) - p.ln_xmin) / p.dln;
        if (t >= 0.0 && t < static_cast<double>(p.nseg)) {
          const int    j   = static_cast<int>(t);
          const double tau = t - j;
          double       F;
          if (p.mode == RG_TABLE_REFERENCE) {
            const float2 c = p.ref[j];
            F              = static_cast<double>(c.x) + tau * static_cast<double>(c.y) / kSlopeScale;
          } else {
            const float4 c = p.hcoef[j];
            F = c.x + tau * (c.y + tau * (c.z + tau * static_cast<double>(c.w)));
          }
          K = F * (p.log_spaced ? gb : 1.0);
        }
      }
      p.K[i] = K;
    }

    __global__ void split_matrix_kernel(const double* __restrict__ K, int nbins, int ng, int transpose,
                                        __nv_bfloat16* __restrict__ dst, int cpad, int nstore) {
      // rows: e (cols g) or, transposed, g (cols e)
      const int     rows = transpose ? ng : nbins, cols = transpose ? nbins : ng;
      const int64_t i    = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= static_cast<int64_t>(rows) * cpad) {
        return;
      }
      const int r = static_cast<int>(i / cpad), c = static_cast<int>(i % cpad);
      __nv_bfloat16 t[3];
      if (c < cols) {
        const double v = transpose ? K[static_cast<int64_t>(c) * ng + r] : K[static_cast<int64_t>(r) * ng + c];
        split3(v, t[0], t[1], t[2]);
      } else {
        t[0] = t[1] = t[2] = __float2bfloat16(0.0f);
      }
      __nv_bfloat16* row = dst + static_cast<int64_t>(r) * nstore * cpad;
      for (int k = 0; k < nstore; ++k) {
        row[k * cpad + c] = t[k];
      }
    }

    // ---- tensor maps -------------------------------------------------------------------------
    using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                       const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                       CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                       CUtensorMapFloatOOBfill);

    // cuTensorMapEncodeTiled from the driver (looked up once, thread-safe), or null.
    EncodeTiledFn encode_fn() {
      static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void*                           p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
              cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
          cudaGetLastError();
          return nullptr;
        }
        return reinterpret_cast<EncodeTiledFn>(p);
      }();
      return fn;
    }

    int encode_tiled(CUtensorMap* tm, void* base, uint64_t cols, uint64_t rows, uint32_t box_rows) {
      const EncodeTiledFn fn = encode_fn();
      if (!fn) {
        return set_error(RG_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
      }
      const cuuint64_t dims[2]    = { cols, rows };
      const cuuint64_t strides[1] = { cols * 2 };
      const cuuint32_t box[2]     = { static_cast<cuuint32_t>(kBK), box_rows };
      const cuuint32_t estr[2]    = { 1, 1 };
      const CUresult   r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) {
        return set_error(RG_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(static_cast<int>(r)) + ")");
      }
      return RG_OK;
    }

    // Tensor map of the output for the epilogue's tensor stores: FP32 [ranges][M][N] with row
    // stride ldc and range stride `stride` (elements), boxes of 32 columns x 128 rows in the
    // 128-byte swizzle.  Returns false (the epilogue then stores directly) when the base or
    // the strides are not 16-byte multiples or the driver refuses the map.
    bool encode_c_map(CUtensorMap* tm, float* base, int N, int M, int ranges, int ldc, int64_t stride) {
      const EncodeTiledFn fn = encode_fn();
      if (!fn) {
        return false;
      }
      if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || (ldc & 3) != 0 || (stride & 3) != 0) {
        return false;
      }
      const cuuint64_t dims[3]    = { static_cast<cuuint64_t>(N), static_cast<cuuint64_t>(M),
                                      static_cast<cuuint64_t>(ranges) };
      const cuuint64_t strides[2] = { static_cast<cuuint64_t>(ldc) * 4, static_cast<cuuint64_t>(stride) * 4 };
      const cuuint32_t box[3]     = { 32, static_cast<cuuint32_t>(kBM), 1 };
      const cuuint32_t estr[3]    = { 1, 1, 1 };
      return fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    }

    // right-operand ring + two buffers of the left operand's BF16 term tiles + alignment slack
    size_t gemm_smem(int cfg, int nstore) {
      return static_cast<size_t>(kConfigs[cfg].stages) * kConfigs[cfg].bn * kBK * 2 +
             static_cast<size_t>(2 * nstore) * kBytesTerm + 1024;
    }

    template <int BN, int STAGES>
    int launch_gemm_t(int cfg, const CUtensorMap& tB, const CUtensorMap& tC, const GemmArgs& g, cudaStream_t s) {
      static std::atomic<uint64_t> configured { 0 };
      RG_CUDA_TRY(ensure_max_dynamic_smem(gemm_bf16_tn_kernel<BN, STAGES>, static_cast<int>(gemm_smem(cfg, 3)),
                                          configured));
      const dim3 grid((g.N + BN - 1) / BN, (g.M + kBM - 1) / kBM, g.splits);
      gemm_bf16_tn_kernel<BN, STAGES><<<grid, kGemmThreads, gemm_smem(cfg, g.nstore), s>>>(tB, tC, g);
      RG_CUDA_TRY(cudaGetLastError());
      return RG_OK;
    }

    // tB is the right operand's tensor map whose box height is the config's bn; the output's
    // map is made here (g.C, g.ldc, g.splits ranges g.split_stride apart).
    int launch_gemm(int cfg, const CUtensorMap& tB, GemmArgs g, cudaStream_t s) {
      if (g.M <= 0 || g.N <= 0) {
        return RG_OK;
      }
      CUtensorMap tC {};
      const int64_t stride = g.splits > 1 ? g.split_stride : static_cast<int64_t>(g.M) * g.ldc;
      g.c_tma = encode_c_map(&tC, g.C, g.N, g.M, g.splits, g.ldc, stride) ? 1 : 0;
      switch (cfg) {
        case 0:
          return launch_gemm_t<kConfigs[0].bn, kConfigs[0].stages>(0, tB, tC, g, s);
        case 1:
          return launch_gemm_t<kConfigs[1].bn, kConfigs[1].stages>(1, tB, tC, g, s);
        case 2:
          return launch_gemm_t<kConfigs[2].bn, kConfigs[2].stages>(2, tB, tC, g, s);
        default:
          return set_error(RG_ERR_ARGUMENT, "unknown GEMM configuration");
      }
    }

    // Box height index of a config's right-operand tensor map: 0 for bn 256, 1 for 128.
    int box_index(int cfg) {
      return kConfigs[cfg].bn == 256 ? 0 : 1;
    }

    int round_up(int v, int m) {
      return (v + m - 1) / m * m;
    }

  } // namespace

} // namespace rg

struct rg_fromdist_plan {
  int            ng = 0, nbins = 0, nprod = 6, nstore = 3, max_dist = 0, log_spaced = 1, mode = RG_TABLE_REFERENCE;
  int            gpad = 0, epad = 0; // padded K extents of the forward / adjoint GEMMs
  float          g_syn = 1, eps = 1;
  bool           zero  = false;
  float*         d_gbeta = nullptr;
  float*         d_ebins = nullptr; // photon energies with invalid bins set to 0
  double*        d_K     = nullptr; // nbins x ng kernel matrix (FP64)
  // right operands as BF16 terms [h | m | l] (the first nstore) per row; the left operand
  // (distributions, or dL/dS) is split inside the GEMM
  __nv_bfloat16* d_B     = nullptr; // forward right operand  [nbins x nstore*gpad]
  __nv_bfloat16* d_BT    = nullptr; // adjoint right operand  [ng x nstore*epad]
  unsigned*      d_status = nullptr;
  CUtensorMap    tB[2], tBT[2]; // right operands with box height 256 and 128
  int            cfg_fwd = 0, cfg_adj = 0; // autotuned tile shapes
  int            split_fwd = 1, split_adj = 1; // autotuned split-K range counts
  float*         d_ws   = nullptr; // split-K slices (split x max_dist x N floats)
  size_t         ws_cap = 0;       // floats
};

namespace rg {

  namespace {

    constexpr int kSplits[]   = { 1, 2, 4, 8 }; // split-K range counts the autotuner tries
    constexpr int kNumSplits  = 4;

    // A split-K range count is usable if every range holds a gamma block.
    bool split_ok(int split, int kpt) {
      return split >= 1 && split <= kpt;
    }

    int ensure_workspace(rg_fromdist_plan* pl, size_t floats) {
      if (floats <= pl->ws_cap) {
        return RG_OK;
      }
      RG_CUDA_TRY(cudaDeviceSynchronize()); // the old slices may still be read
      cudaFree(pl->d_ws);
      pl->d_ws   = nullptr;
      pl->ws_cap = 0;
      RG_CUDA_TRY(cudaMalloc(&pl->d_ws, sizeof(float) * floats));
      pl->ws_cap = floats;
      return RG_OK;
    }

    // One GEMM: C = g.C (row stride g.ldc).  With split > 1 the gamma blocks are cut into
    // `split` ranges (blockIdx.z) whose products land in the plan's workspace slices, then
    // summed in range order into C.  The workspace must already hold split x M x N floats.
    int run_gemm(rg_fromdist_plan* pl, int cfg, int split, const CUtensorMap& tB, GemmArgs g, cudaStream_t s) {
      g.splits       = 1;
      g.split_stride = 0;
      if (split <= 1 || g.M <= 0 || g.N <= 0) {
        return launch_gemm(cfg, tB, g, s);
      }
      if (!split_ok(split, g.kpt)) {
        return set_error(RG_ERR_ARGUMENT, "split-K range count above the number of gamma blocks");
      }
      const int64_t n = static_cast<int64_t>(g.M) * g.N;
      if (static_cast<size_t>(split) * static_cast<size_t>(n) > pl->ws_cap) {
        return set_error(RG_ERR_ARGUMENT, "split-K workspace smaller than the request (ndist above max_dist?)");
      }
      float*    out = g.C;
      const int ldc = g.ldc;
      g.C            = pl->d_ws;
      g.ldc          = g.N;
      g.splits       = split;
      g.split_stride = n;
      RG_TRY(launch_gemm(cfg, tB, g, s));
      DeviceContext* ctx = nullptr;
      RG_TRY(context(&ctx));
      const int blocks = static_cast<int>(std::min<int64_t>((n + 255) / 256, static_cast<int64_t>(ctx->sms) * 8));
      splitk_reduce_kernel<<<blocks, 256, 0, s>>>(pl->d_ws, split, n, g.M, g.N, out, ldc);
      RG_CUDA_TRY(cudaGetLastError());
      return RG_OK;
    }

    // Times every tile shape and split-K range count on the plan's own GEMM (max_dist
    // rows, zero left operand) and returns the fastest; results are cached per device
    // and shape.
    int tune_gemm(rg_fromdist_plan* pl, bool adjoint, int* best_cfg, int* best_split) {
      static std::mutex                                   mu;
      static std::map<std::vector<int>, std::pair<int, int>> cache;
      int dev = 0;
      RG_CUDA_TRY(cudaGetDevice(&dev));
      GemmArgs g {};
      g.M         = pl->max_dist;
      g.N         = adjoint ? pl->ng : pl->nbins;
      g.kpt       = (adjoint ? pl->epad : pl->gpad) / kBK;
      g.nprod     = pl->nprod;
      g.nstore    = pl->nstore;
      g.cols      = adjoint ? pl->nbins : pl->ng;
      g.ld        = g.cols;
      g.left_scale = adjoint ? pl->d_ebins : nullptr;
      g.ldc       = g.N;
      g.col_scale = adjoint ? nullptr : pl->d_ebins;
      g.status    = pl->d_status;
      const std::vector<int> key { dev, adjoint ? 1 : 0, g.M, g.N, g.kpt, g.nprod };
      {
        std::lock_guard<std::mutex> lock(mu);
        const auto it = cache.find(key);
        if (it != cache.end()) {
          *best_cfg   = it->second.first;
          *best_split = it->second.second;
          return ensure_workspace(pl, static_cast<size_t>(*best_split) * g.M * g.N);
        }
      }
      float*      C  = nullptr;
      float*      L  = nullptr; // zero left operand for the timing runs
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      auto cleanup = [&]() {
        cudaFree(C);
        cudaFree(L);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
      };
      auto fail = [&](int st) {
        cleanup();
        return st;
      };
      cudaError_t e = cudaMalloc(&C, sizeof(float) * static_cast<size_t>(g.M) * g.N);
      if (e == cudaSuccess) e = cudaEventCreate(&e0);
      if (e == cudaSuccess) e = cudaEventCreate(&e1);
      const size_t lbytes = sizeof(float) * static_cast<size_t>(g.M) * g.cols;
      if (e == cudaSuccess) e = cudaMalloc(&L, lbytes);
      if (e == cudaSuccess) e = cudaMemset(L, 0, lbytes);
      if (e != cudaSuccess) {
        return fail(cuda_error(e, "GEMM autotuning setup"));
      }
      g.C        = C;
      g.left     = L;
      int maxsplit = 1;
      for (int si = 0; si < kNumSplits; ++si) {
        if (split_ok(kSplits[si], g.kpt)) {
          maxsplit = std::max(maxsplit, kSplits[si]);
        }
      }
      {
        const int st = ensure_workspace(pl, static_cast<size_t>(maxsplit) * g.M * g.N);
        if (st != RG_OK) {
          return fail(st);
        }
      }
      int   best = 0, best_sp = 1;
      float best_ms = 0.0f;
      bool  first   = true;
      for (int cfg = 0; cfg < kNumConfigs; ++cfg) {
        const CUtensorMap& tB = adjoint ? pl->tBT[box_index(cfg)] : pl->tB[box_index(cfg)];
        for (int si = 0; si < kNumSplits; ++si) {
          const int split = kSplits[si];
          if (!split_ok(split, g.kpt)) {
            continue;
          }
          for (int r = 0; r < 2; ++r) {
            const int st = run_gemm(pl, cfg, split, tB, g, nullptr);
            if (st != RG_OK) {
              return fail(st);
            }
          }
          e = cudaEventRecord(e0, nullptr);
          for (int r = 0; r < 5 && e == cudaSuccess; ++r) {
            const int st = run_gemm(pl, cfg, split, tB, g, nullptr);
            if (st != RG_OK) {
              return fail(st);
            }
          }
          if (e == cudaSuccess) e = cudaEventRecord(e1, nullptr);
          if (e == cudaSuccess) e = cudaEventSynchronize(e1);
          float ms = 0.0f;
          if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
          if (e != cudaSuccess) {
            return fail(cuda_error(e, "GEMM autotuning"));
          }
          if (first || ms < best_ms) {
            best    = cfg;
            best_sp = split;
            best_ms = ms;
            first   = false;
          }
        }
      }
      unsigned st = 0;
      e = cudaMemcpy(&st, pl->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        return fail(cuda_error(e, "GEMM autotuning status"));
      }
      cleanup();
      if (st != 0) {
        return set_error(RG_ERR_TIMEOUT, "a bounded wait in the tensor-core GEMM gave up during autotuning");
      }
      std::lock_guard<std::mutex> lock(mu);
      cache[key]  = { best, best_sp };
      *best_cfg   = best;
      *best_split = best_sp;
      return RG_OK;
    }

  } // namespace

} // namespace rg

extern "C" {

int rg_fromdist_plan_create(const float* gbeta, int32_t ng, int32_t log_spaced, const float* bins, int32_t nbins,
                            float g_syn, float e_syn_at_g_syn, int32_t table_mode, int32_t split_products,
                            int32_t max_dist, rg_fromdist_plan** plan) {
  rg::clear_error();
  if (!plan || ng < 1 || nbins < 1 || max_dist < 1 || !gbeta || !bins) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_fromdist_plan_create: bad arguments");
  }
  if (split_products != 3 && split_products != 6) {
    return rg::set_error(RG_ERR_ARGUMENT, "split_products must be 3 or 6");
  }
  if (table_mode != RG_TABLE_REFERENCE && table_mode != RG_TABLE_SMOOTH) {
    return rg::set_error(RG_ERR_ARGUMENT, "unknown table mode");
  }
  *plan          = nullptr;
  auto pl        = std::make_unique<rg_fromdist_plan>();
  pl->ng         = ng;
  pl->nbins      = nbins;
  pl->nprod      = split_products;
  pl->nstore     = split_products == 6 ? 3 : 2; // 3 products use h and m only
  pl->max_dist   = max_dist;
  pl->log_spaced = log_spaced ? 1 : 0;
  pl->mode       = table_mode;
  pl->g_syn      = g_syn;
  pl->eps        = e_syn_at_g_syn;
  pl->gpad       = rg::round_up(ng, rg::kBK);
  pl->epad       = rg::round_up(nbins, rg::kBK);
  const double K0 = static_cast<double>(e_syn_at_g_syn) / (static_cast<double>(g_syn) * g_syn);
  pl->zero        = !(K0 > 0.0) || !std::isfinite(K0);

  const rg::RefTable*    ref = nullptr;
  const rg::SmoothTable* sm  = nullptr;
  RG_TRY(rg::reference_table(&ref));
  if (table_mode == RG_TABLE_SMOOTH) {
    RG_TRY(rg::smooth_table(&sm));
  }
  std::vector<float> eb(bins, bins + nbins);
  for (float& v : eb) {
    if (!(v > 0.0f) || !std::isfinite(v)) {
      v = 0.0f; // non-positive bins yield 0, as in the particle path
    }
  }
  auto fail = [&](int st) {
    rg_fromdist_plan_destroy(pl.release());
    return st;
  };
#define RG_PLAN_CUDA(expr)                                                                  \
  do {                                                                                      \
    cudaError_t e_ = (expr);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      return fail(rg::cuda_error(e_, #expr));                                               \
    }                                                                                       \
  } while (0)
  const size_t kf = static_cast<size_t>(pl->nstore) * pl->gpad, ka = static_cast<size_t>(pl->nstore) * pl->epad;
  RG_PLAN_CUDA(cudaMalloc(&pl->d_gbeta, sizeof(float) * ng));
  RG_PLAN_CUDA(cudaMalloc(&pl->d_ebins, sizeof(float) * nbins));
  RG_PLAN_CUDA(cudaMalloc(&pl->d_K, sizeof(double) * nbins * ng));
  RG_PLAN_CUDA(cudaMalloc(&pl->d_B, sizeof(__nv_bfloat16) * nbins * kf));
  RG_PLAN_CUDA(cudaMalloc(&pl->d_BT, sizeof(__nv_bfloat16) * ng * ka));
  RG_PLAN_CUDA(cudaMalloc(&pl->d_status, sizeof(unsigned)));
  RG_PLAN_CUDA(cudaMemset(pl->d_status, 0, sizeof(unsigned)));
  RG_PLAN_CUDA(cudaMemcpy(pl->d_gbeta, gbeta, sizeof(float) * ng, cudaMemcpyHostToDevice));
  RG_PLAN_CUDA(cudaMemcpy(pl->d_ebins, eb.data(), sizeof(float) * nbins, cudaMemcpyHostToDevice));

  rg::KParams kp {};
  kp.gbeta      = pl->d_gbeta;
  kp.ebins      = pl->d_ebins;
  kp.ng         = ng;
  kp.nbins      = nbins;
  kp.log_spaced = pl->log_spaced;
  kp.ln_k0      = pl->zero ? 0.0 : std::log(K0);
  kp.mode       = table_mode;
  if (table_mode == RG_TABLE_REFERENCE) {
    kp.ln_xmin = ref->ln_xmin;
    kp.dln     = ref->dln;
    kp.nseg    = ref->n - 1;
  } else {
    kp.ln_xmin = sm->ln_xmin;
    kp.dln     = sm->dln;
    kp.nseg    = rg::kSmoothSegments;
  }
  kp.ref   = ref->d_coef;
  kp.hcoef = sm ? sm->d_coef : nullptr;
  kp.K     = pl->d_K;
  const int64_t nk = static_cast<int64_t>(nbins) * ng;
  rg::kernel_matrix_kernel<<<static_cast<unsigned>((nk + 255) / 256), 256>>>(kp);
  RG_PLAN_CUDA(cudaGetLastError());
  if (pl->zero) {
    RG_PLAN_CUDA(cudaMemset(pl->d_K, 0, sizeof(double) * nk));
  }
  const int64_t nb = static_cast<int64_t>(nbins) * pl->gpad, nt = static_cast<int64_t>(ng) * pl->epad;
  rg::split_matrix_kernel<<<static_cast<unsigned>((nb + 255) / 256), 256>>>(pl->d_K, nbins, ng, 0, pl->d_B,
                                                                            pl->gpad, pl->nstore);
  RG_PLAN_CUDA(cudaGetLastError());
  rg::split_matrix_kernel<<<static_cast<unsigned>((nt + 255) / 256), 256>>>(pl->d_K, nbins, ng, 1, pl->d_BT,
                                                                            pl->epad, pl->nstore);
  RG_PLAN_CUDA(cudaGetLastError());
  RG_PLAN_CUDA(cudaDeviceSynchronize());
  int st = RG_OK;
  for (int b = 0; b < 2 && st == RG_OK; ++b) {
    const uint32_t box = b == 0 ? 256u : 128u;
    st = rg::encode_tiled(&pl->tB[b], pl->d_B, kf, nbins, box);
    if (st == RG_OK) st = rg::encode_tiled(&pl->tBT[b], pl->d_BT, ka, ng, box);
  }
  if (st == RG_OK) st = rg::tune_gemm(pl.get(), false, &pl->cfg_fwd, &pl->split_fwd);
  if (st == RG_OK) st = rg::tune_gemm(pl.get(), true, &pl->cfg_adj, &pl->split_adj);
  if (st != RG_OK) {
    return fail(st);
  }
#undef RG_PLAN_CUDA
  *plan = pl.release();
  return RG_OK;
}

int rg_fromdist_plan_destroy(rg_fromdist_plan* pl) {
  if (!pl) {
    return RG_OK;
  }
  cudaFree(pl->d_gbeta);
  cudaFree(pl->d_ebins);
  cudaFree(pl->d_K);
  cudaFree(pl->d_B);
  cudaFree(pl->d_BT);
  cudaFree(pl->d_status);
  cudaFree(pl->d_ws);
  delete pl;
  return RG_OK;
}

int rg_fromdist_run(rg_fromdist_plan* pl, const float* f, int32_t ndist, float* out, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrumFromDist");
  if (!pl || ndist < 0 || ndist > pl->max_dist || (ndist > 0 && (!f || !out))) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_fromdist_run: bad arguments (ndist above the plan's max_dist?)");
  }
  if (ndist == 0) {
    return RG_OK;
  }
  rg::GemmArgs g {};
  g.M          = ndist;
  g.N          = pl->nbins;
  g.kpt        = pl->gpad / rg::kBK;
  g.nprod      = pl->nprod;
  g.nstore     = pl->nstore;
  g.left       = f;
  g.cols       = pl->ng;
  g.ld         = pl->ng;
  g.left_scale = nullptr;
  g.C          = out;
  g.ldc        = pl->nbins;
  g.col_scale  = pl->d_ebins;
  g.status     = pl->d_status;
  return rg::run_gemm(pl, pl->cfg_fwd, pl->split_fwd, pl->tB[rg::box_index(pl->cfg_fwd)], g,
                      static_cast<cudaStream_t>(stream));
}

int rg_fromdist_adjoint(rg_fromdist_plan* pl, const float* grad_out, int32_t ndist, float* grad_f, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrumFromDistAdjoint");
  if (!pl || ndist < 0 || ndist > pl->max_dist || (ndist > 0 && (!grad_out || !grad_f))) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_fromdist_adjoint: bad arguments (ndist above the plan's max_dist?)");
  }
  if (ndist == 0) {
    return RG_OK;
  }
  // left operand: dL/dS[d][e] * e_e (scaled while it is split)
  rg::GemmArgs g {};
  g.M          = ndist;
  g.N          = pl->ng;
  g.kpt        = pl->epad / rg::kBK;
  g.nprod      = pl->nprod;
  g.nstore     = pl->nstore;
  g.left       = grad_out;
  g.cols       = pl->nbins;
  g.ld         = pl->nbins;
  g.left_scale = pl->d_ebins;
  g.C          = grad_f;
  g.ldc        = pl->ng;
  g.col_scale  = nullptr;
  g.status     = pl->d_status;
  return rg::run_gemm(pl, pl->cfg_adj, pl->split_adj, pl->tBT[rg::box_index(pl->cfg_adj)], g,
                      static_cast<cudaStream_t>(stream));
}

int rg_fromdist_plan_check(rg_fromdist_plan* pl, void* stream) {
  if (!pl) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan");
  }
  auto     s  = static_cast<cudaStream_t>(stream);
  unsigned st = 0;
  RG_CUDA_TRY(cudaMemcpyAsync(&st, pl->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  RG_CUDA_TRY(cudaStreamSynchronize(s));
  if (st != 0) {
    RG_CUDA_TRY(cudaMemset(pl->d_status, 0, sizeof(unsigned)));
    return rg::set_error(RG_ERR_TIMEOUT, "a bounded wait in the tensor-core GEMM gave up; results are invalid");
  }
  return RG_OK;
}

int rg_fromdist_plan_config(const rg_fromdist_plan* pl, int32_t* fwd_bn, int32_t* fwd_stages, int32_t* adj_bn,
                            int32_t* adj_stages) {
  if (!pl) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan");
  }
  if (fwd_bn) *fwd_bn = rg::kConfigs[pl->cfg_fwd].bn;
  if (fwd_stages) *fwd_stages = rg::kConfigs[pl->cfg_fwd].stages;
  if (adj_bn) *adj_bn = rg::kConfigs[pl->cfg_adj].bn;
  if (adj_stages) *adj_stages = rg::kConfigs[pl->cfg_adj].stages;
  return RG_OK;
}

int rg_fromdist_plan_set_config(rg_fromdist_plan* pl, int32_t fwd_cfg, int32_t adj_cfg) {
  if (!pl || fwd_cfg >= rg::kNumConfigs || adj_cfg >= rg::kNumConfigs) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_fromdist_plan_set_config: configuration index out of range");
  }
  if (fwd_cfg >= 0) pl->cfg_fwd = fwd_cfg;
  if (adj_cfg >= 0) pl->cfg_adj = adj_cfg;
  return RG_OK;
}

int rg_fromdist_plan_split_k(const rg_fromdist_plan* pl, int32_t* fwd_split, int32_t* adj_split) {
  if (!pl) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan");
  }
  if (fwd_split) *fwd_split = pl->split_fwd;
  if (adj_split) *adj_split = pl->split_adj;
  return RG_OK;
}

int rg_fromdist_plan_set_split_k(rg_fromdist_plan* pl, int32_t fwd_split, int32_t adj_split) {
  if (!pl) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan");
  }
  const int kf = pl->gpad / rg::kBK, ka = pl->epad / rg::kBK;
  auto listed  = [](int v) {
    for (int si = 0; si < rg::kNumSplits; ++si) {
      if (rg::kSplits[si] == v) return true;
    }
    return false;
  };
  if ((fwd_split >= 0 && (!listed(fwd_split) || !rg::split_ok(fwd_split, kf))) ||
      (adj_split >= 0 && (!listed(adj_split) || !rg::split_ok(adj_split, ka)))) {
    return rg::set_error(RG_ERR_ARGUMENT,
                         "rg_fromdist_plan_set_split_k: counts are 1, 2, 4 or 8 and at most the gamma blocks");
  }
  const int    f    = fwd_split >= 0 ? fwd_split : pl->split_fwd;
  const int    a    = adj_split >= 0 ? adj_split : pl->split_adj;
  const size_t need = std::max(static_cast<size_t>(f) * pl->max_dist * pl->nbins,
                               static_cast<size_t>(a) * pl->max_dist * pl->ng);
  RG_TRY(rg::ensure_workspace(pl, need));
  pl->split_fwd = f;
  pl->split_adj = a;
  return RG_OK;
}

int rg_fromdist_kernel_matrix(rg_fromdist_plan* pl, double* K_host) {
  if (!pl || !K_host) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_fromdist_kernel_matrix: bad arguments");
  }
  RG_CUDA_TRY(cudaMemcpy(K_host, pl->d_K, sizeof(double) * pl->nbins * pl->ng, cudaMemcpyDeviceToHost));
  return RG_OK;
}

} // extern "C"

// Particle and distribution synchrotron spectra on sm_103a (forward).
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
//    and the particle's table coordinate Q = 2^frac (ln gamma + ln W / 2) / dln
//    as a fixed-point integer (ln of a double-float to ~1e-10 absolute).
//  * Photon bin b carries P_b = 2^frac (ln e_b - ln xmin - ln K0) / dln (host,
//    FP64), so T = P_b - Q (one 32-bit integer add, exact) is the fixed-point
//    table coordinate of x = e_b / e_peak.
//      reference table (frac = 22): the top 10 bits of T index a 1024-entry
//      segment table in shared memory whose entries past the last segment are
//      zero, so an out-of-range x reads zero without a branch; the low 22 bits,
//      read as a denormal, times the stored slope (pre-scaled by 2^127) give
//      frac * slope in one FFMA.  Per eval: IADD (T), SHF (segment, ALU pipe),
//      IMAD (fraction bits = T - segment 2^22, FMA pipe), LDS.64, FFMA (F),
//      FFMA (accumulate).
//      smooth table: T >> frac (clamped to a zero entry) indexes cubic Hermite
//      segments; the fraction bits read as a denormal times 2^126 give
//      tau' = bits 2^-23 exactly (the coefficients are rescaled to tau' when
//      staged), and three FFMAs evaluate the cubic.
//  * Lanes own photon bins (32 consecutive bins per row, K rows per lane), warps
//    own particles; per-warp FP32 register accumulators are folded into
//    double-float accumulators after every chunk; at a segment's end the block sums
//    its warps in FP64 (warp order) into one partial row per block, and a second
//    kernel sums the blocks' rows in FP64 in a fixed order, so results are
//    bit-reproducible.
//  * Particle streams (SoA FP32) are staged chunk by chunk into shared memory
//    with 1-D TMA bulk copies (cp.async.bulk + mbarrier), double buffered.
//  * Work items are (segment, chunk) pairs in particle order; each block of the
//    persistent grid takes a contiguous range of items, so one spectrum and a
//    batch of uneven segments run through the same launch, and every block
//    touches each segment in one contiguous run (one partial per (block, seg)).
#include "spectrum_common.cuh"
#include "spectrum_plan.hpp"

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

    // Rows of 32 bins combined per pass of flush_block: the pass's scratch, kFlushRows x
    // kWarps x 32 doubles, is the 8 KB of the two (q, A) buffers.
    constexpr int kFlushRows = 4;
    static_assert(kFlushRows * kWarps * 32 * sizeof(double) <= 2 * kChunk * sizeof(int2),
                  "flush scratch must fit the (q, A) buffers");

    // Sums the warps' double-float accumulators of one segment in warp order (FP64) and
    // writes the block's partial row; the accumulators are cleared.  Called by the whole
    // block at a point where no warp reads the (q, A) buffers that serve as scratch.
    template <int K>
    __device__ __forceinline__ void flush_block(float (&hi)[K], float (&lo)[K], double* scratch, double* dst,
                                                int tid, bool accumulate) {
      const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
      for (int k0 = 0; k0 < K; k0 += kFlushRows) {
#pragma unroll
        for (int r = 0; r < kFlushRows; ++r) {
          if (k0 + r < K) {
            scratch[(r * kWarps + warp) * 32 + lane] =
              static_cast<double>(hi[k0 + r]) + static_cast<double>(lo[k0 + r]);
          }
        }
        __syncthreads();
        const int r = tid >> 5;
        if (r < kFlushRows && k0 + r < K) {
          double t = 0.0;
#pragma unroll
          for (int w = 0; w < kWarps; ++w) {
            t += scratch[(r * kWarps + w) * 32 + lane];
          }
          double* d = dst + (k0 + r) * 32 + lane;
          *d        = accumulate ? *d + t : t;
        }
        __syncthreads();
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        hi[k] = 0.0f;
        lo[k] = 0.0f;
      }
    }

    template <int K, int MODE>
    __global__ void __launch_bounds__(kThreads, kBlocksPerSM)
      fused_spectrum_kernel(const __grid_constant__ FusedParams p) {
      extern __shared__ __align__(128) unsigned char smem[];
      float2* tab  = reinterpret_cast<float2*>(smem);
      float4* htab = reinterpret_cast<float4*>(smem);
      const int tab_size = (MODE == kModeRef) ? static_cast<int>(sizeof(float2)) * kRefEntries
                                              : static_cast<int>(sizeof(float4)) * (p.hseg + 1);
      int2*  qa    = reinterpret_cast<int2*>(smem + tab_size);
      float* stage = reinterpret_cast<float*>(qa + 2 * kChunk);
      __shared__ uint64_t mbar[2];
      __shared__ ItemInfo info[2];

      const int     tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
      const int     slice    = blockIdx.y;
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
        P[k] = p.P[slice * kSliceBins + k * 32 + lane];
      }
      const int64_t  Pmin = p.Prange[2 * slice], Pmax = p.Prange[2 * slice + 1];
      const int      stage_floats = p.nslots * kChunkPad;
      const uint32_t dead         = dead_coordinate(Pmin, p.L);
      const int      frac         = (MODE == kModeRef) ? kFrac : p.frac;
      const uint32_t hseg         = static_cast<uint32_t>(p.hseg);
      // fraction bits = T - seg * 2^frac as an IMAD (FMA pipe) next to the segment
      // shift (ALU pipe): the two integer pipes share the per-eval work
      const uint32_t seg_neg = (~p.opaque_zero) << frac;

      int seg_hint = 0;
      if (tid == 0) {
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
          // block-uniform (info[st] is shared); every warp is past the previous item's
          // evaluation (the barrier above), so the (q, A) buffers are free
          if (cur_seg >= 0) {
            flush_block<K>(hi, lo, reinterpret_cast<double*>(qa), block_partial(p, b, cur_seg, slice), tid,
                           p.accumulate != 0);
          }
          cur_seg = I.seg;
        }

        // ---- per-particle stage ------------------------------------------------
        const float* sbuf = stage + st * stage_floats;
        int2*        qdst = qa + st * kChunk;
        for (int j = tid; j < I.np; j += kThreads) {
          float v[kComps];
          load_comps(p, I, sbuf, I.pstart + j, v);
          uint32_t   q    = 0;
          float      A    = 0.0f;
          const bool live = (p.source == kSrcParticles) ? particle_stage(v, p, Pmin, Pmax, q, A)
                                                        : dist_stage(v[0], v[1], p, Pmin, Pmax, q, A);
          if (!live) {
            q = dead;
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
            if (MODE == kModeRef) {
              const uint32_t sg = T >> kFrac;
              const float2   c  = tab[sg];
              const float    m  = __uint_as_float(sg * seg_neg + T);
              const float    F  = __fmaf_rn(m, c.y, c.x);
              acc[k]         = __fmaf_rn(A, F, acc[k]);
            } else {
              const uint32_t sg  = T >> frac;
              const float4   c   = htab[min(sg, hseg)];
              const float    tau = smooth_tau(sg * seg_neg + T);
              const float    F   = __fmaf_rn(tau, __fmaf_rn(tau, __fmaf_rn(tau, c.w, c.z), c.y), c.x);
              acc[k]           = __fmaf_rn(A, F, acc[k]);
            }
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
        __syncthreads(); // every warp is done reading the last item's (q, A)
        flush_block<K>(hi, lo, reinterpret_cast<double*>(qa), block_partial(p, b, cur_seg, slice), tid,
                       p.accumulate != 0);
      }
    }

    // Cumulative chunk counts of the segments (one block), with a check that the
    // offsets never decrease and stay within [0, n]; on failure the status word
    // is set and the kernels that follow do no work.
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
    };

    // Block (32 bins x kReduceRows row groups): row group y sums the block partial
    // rows y, y + kReduceRows, ... of its segment, then the row groups are
    // combined in order through shared memory.  The summation order depends only
    // on the launch geometry, so results are deterministic.
    constexpr int kReduceRows  = 32;
    constexpr int kReduceLoads = 8;

    __global__ void __launch_bounds__(32 * kReduceRows)
      reduce_partials_kernel(const __grid_constant__ ReduceParams r) {
      __shared__ double part[kReduceRows][33];
      const int bin = blockIdx.x * 32 + threadIdx.x;
      const int s   = blockIdx.y;
      const int ty  = threadIdx.y;
      const bool failed = *r.status != kDevOk;
      bool       active = false;
      double     sum    = 0.0;
      if (bin < r.nbins && !failed) {
        const int64_t n_items = total_items(r.item_prefix, r.nseg, r.n_single);
        const int64_t i0      = items_before(r.item_prefix, s);
        const int64_t i1      = r.item_prefix ? r.item_prefix[s + 1] : n_items;
        if (i1 > i0 && r.valid[bin]) {
          active          = true;
          const int b0    = block_of_item(i0, n_items, r.grid);
          const int b1    = block_of_item(i1 - 1, n_items, r.grid);
          const int slice = bin / kSliceBins, j = bin % kSliceBins;
          const int rows  = b1 - b0 + 1; // one partial row per block
          const double* base =
            r.partials + (static_cast<int64_t>(b0 + s) * r.nslices + slice) * kSliceBins + j;
          const int64_t block_stride = static_cast<int64_t>(r.nslices) * kSliceBins;
          // a block that owns no item (more blocks than items) wrote no partials; with at
          // least one item per block every block owns one, and the per-row ownership test
          // (two 64-bit divisions) is skipped
          const bool every_block_owns = n_items >= r.grid;
          // kReduceLoads rows loaded before they are added (in row order, as one at a
          // time would): the loop is bound by load latency, not by the adds
          for (int row0 = ty; row0 < rows; row0 += kReduceRows * kReduceLoads) {
            double v[kReduceLoads];
#pragma unroll
            for (int u = 0; u < kReduceLoads; ++u) {
              const int row = row0 + u * kReduceRows;
              v[u]          = 0.0;
              if (row < rows) {
                const int64_t b = b0 + row;
                if (every_block_owns || b * n_items / r.grid < (b + 1) * n_items / r.grid) {
                  v[u] = base[row * block_stride];
                }
              }
            }
#pragma unroll
            for (int u = 0; u < kReduceLoads; ++u) {
              sum += v[u];
            }
          }
        }
      }
      part[ty][threadIdx.x] = sum;
      __syncthreads();
      if (ty != 0 || bin >= r.nbins) {
        return;
      }
      double result = 0.0;
      if (failed) {
        result = __longlong_as_double(0x7ff8000000000000LL);
      } else if (active) {
        double t = 0.0;
#pragma unroll
        for (int y = 0; y < kReduceRows; ++y) {
          t += part[y][threadIdx.x];
        }
        result = t * static_cast<double>(r.ebins[bin]);
      }
      r.out[static_cast<int64_t>(s) * r.nbins + bin] = __double2float_rn(result);
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

    // The failure path of the stage wait, taken on purpose without a fault: the
    // barrier expects two arrivals and gets one, so its phase never completes, every
    // thread's wait gives up after `polls` polls and the block records the status the
    // fused kernel records when a particle-stream copy does not land.  No copy is in
    // flight, so nothing is left to drain.
    __global__ void __launch_bounds__(64) stage_wait_probe_kernel(unsigned* status, unsigned polls) {
      __shared__ __align__(8) uint64_t bar;
      if (threadIdx.x == 0) {
        mbar_init(&bar, 2);
        fence_mbar_init();
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        mbar_arrive(&bar);
      }
      const bool ok = mbar_wait_bounded(&bar, 0u, polls);
      if (!__syncthreads_and(ok) && threadIdx.x == 0) {
        atomicOr(status, kDevTimeoutStage);
      }
    }

    size_t fused_smem(int mode, int hseg, int nslots) {
      const size_t tab = (mode == kModeRef) ? sizeof(float2) * kRefEntries : sizeof(float4) * (hseg + 1);
      return tab + sizeof(int2) * 2 * kChunk + sizeof(float) * 2 * nslots * kChunkPad;
    }

    // Sets the kernel's shared-memory limit once per device (which also loads it).
    template <int K, int MODE>
    cudaError_t configure_fused_k() {
      static std::atomic<uint64_t> configured { 0 };
      return ensure_max_dynamic_smem(fused_spectrum_kernel<K, MODE>,
                                     static_cast<int>(fused_smem(MODE, kSmoothMaxSegments, kComps)), configured);
    }

    template <int K, int MODE>
    cudaError_t launch_fused_k(const FusedParams& fp, dim3 grid, size_t smem, cudaStream_t s) {
      const cudaError_t e = configure_fused_k<K, MODE>();
      if (e != cudaSuccess) {
        return e;
      }
      fused_spectrum_kernel<K, MODE><<<grid, kThreads, smem, s>>>(fp);
      return cudaGetLastError();
    }

    template <int MODE>
    cudaError_t launch_fused_mode(int K, const FusedParams& fp, dim3 grid, size_t smem, cudaStream_t s) {
      switch (K) {
#define RG_K_CASE(k)                                                                         \
  case k:                                                                                    \
    return launch_fused_k<k, MODE>(fp, grid, smem, s);
        RG_K_CASE(1) RG_K_CASE(2) RG_K_CASE(3) RG_K_CASE(4) RG_K_CASE(5) RG_K_CASE(6)
        RG_K_CASE(7) RG_K_CASE(8) RG_K_CASE(9) RG_K_CASE(10) RG_K_CASE(11) RG_K_CASE(12)
        RG_K_CASE(13) RG_K_CASE(14) RG_K_CASE(15) RG_K_CASE(16)
#undef RG_K_CASE
        default:
          return cudaErrorInvalidValue;
      }
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
      const cudaError_t e = (pl->table_mode == kModeRef)
                              ? launch_fused_mode<kModeRef>(pl->K, fp, grid, smem, s)
                              : launch_fused_mode<kModeSmooth>(pl->K, fp, grid, smem, s);
      RG_CUDA_TRY(e);
      if (pl->timing) {
        RG_CUDA_TRY(cudaEventRecord(ev.second, s));
        pl->ev_used.push_back(ev);
      }
      return RG_OK;
    }

    // Fixed-point coordinates of the photon bins (FP64 on the host).  For the
    // smooth table the fraction bits are chosen so that every slice's bin span
    // plus the table fits the 32-bit window; the reference table uses kFrac and
    // fails if a 512-bin slice spans more than about 33 decades.
    int plan_prepare_bins(rg_spectrum_plan* pl, double ln_xmin, double dln, int nseg_table,
                          double ln_k0) {
      // span of the valid bins of each slice, in table segments
      double max_span = 0.0;
      for (int s = 0; s < pl->nslices; ++s) {
        double lo = std::numeric_limits<double>::max(), hi = -lo;
        for (int j = 0; j < kSliceBins && s * kSliceBins + j < pl->nbins; ++j) {
          const double e = pl->h_bins[s * kSliceBins + j];
          if (e > 0.0 && std::isfinite(e)) {
            lo = std::min(lo, std::log(e));
            hi = std::max(hi, std::log(e));
          }
        }
        if (hi >= lo) {
          max_span = std::max(max_span, (hi - lo) / dln);
        }
      }
      if (pl->table_mode == kModeRef) {
        pl->frac = kFrac;
      } else {
        const double room = 4294967296.0 / (max_span + nseg_table + 2.0);
        pl->frac          = std::min(kFrac, static_cast<int>(std::floor(std::log2(room))));
        if (pl->frac < 12) {
          return set_error(RG_ERR_UNSUPPORTED, "photon bins span too many decades for the smooth table");
        }
      }
      const double scale = std::ldexp(1.0, pl->frac) / dln;
      pl->L              = static_cast<int64_t>(nseg_table) << pl->frac;
      const double S     = std::ldexp(1.0, pl->frac) / (2.0 * dln);
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
          const int     bidx     = s * kSliceBins + j;
          const int64_t v        = (bidx < pl->nbins && hV[bidx]) ? Ps[j] : pmin;
          hP[s * kSliceBins + j] = static_cast<int32_t>(static_cast<uint32_t>(v & 0xffffffffLL));
        }
        hR[2 * s]     = pmin;
        hR[2 * s + 1] = pmax;
      }
      RG_CUDA_TRY(cudaMemcpy(pl->d_P, hP.data(), sizeof(int32_t) * nsb, cudaMemcpyHostToDevice));
      RG_CUDA_TRY(cudaMemcpy(pl->d_Prange, hR.data(), sizeof(int64_t) * hR.size(), cudaMemcpyHostToDevice));
      RG_CUDA_TRY(cudaMemcpy(pl->d_valid, hV.data(), hV.size(), cudaMemcpyHostToDevice));
      if (pl->nbins) {
        RG_CUDA_TRY(cudaMemcpy(pl->d_ebins, pl->h_bins.data(), sizeof(float) * pl->nbins,
                               cudaMemcpyHostToDevice));
      }
      return moments_prepare(pl, hV, ln_xmin, dln, ln_k0);
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
      pl->grid         = ctx->sms * kBlocksPerSM;
      const size_t nsb = static_cast<size_t>(pl->nslices) * kSliceBins;
      RG_CUDA_TRY(cudaMalloc(&pl->d_P, sizeof(int32_t) * nsb));
      RG_CUDA_TRY(cudaMalloc(&pl->d_Prange, sizeof(int64_t) * 2 * pl->nslices));
      RG_CUDA_TRY(cudaMalloc(&pl->d_ebins, sizeof(float) * std::max(nbins, 1)));
      RG_CUDA_TRY(cudaMalloc(&pl->d_valid, std::max(nbins, 1)));
      RG_CUDA_TRY(cudaMalloc(&pl->d_status, sizeof(unsigned)));
      RG_CUDA_TRY(cudaMemset(pl->d_status, 0, sizeof(unsigned)));
      RG_TRY(reference_table(&pl->ref));
      if (pl->table_mode == kModeSmooth) {
        RG_TRY(smooth_table(&pl->smooth));
      }
      return RG_OK;
    }

    // Table geometry of the plan: (ln xmin, dln, segments).
    void table_geometry(const rg_spectrum_plan* pl, double& ln_xmin, double& dln, int& nseg) {
      if (pl->table_mode == kModeRef) {
        ln_xmin = pl->ref->ln_xmin;
        dln     = pl->ref->dln;
        nseg    = pl->ref->n - 1;
      } else {
        ln_xmin = pl->smooth->ln_xmin;
        dln     = pl->smooth->dln;
        nseg    = pl->smooth->nseg;
      }
    }

  } // namespace

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
    // the interval moments of max_seg segments, so that runs allocate nothing (and can be
    // captured in a CUDA graph)
    if (moments_selected(pl, max_seg)) {
      const size_t need = static_cast<size_t>(max_seg) * static_cast<size_t>(pl->hist_per_seg);
      if (need > pl->hist_cap) {
        cudaFree(pl->d_hist);
        pl->d_hist = nullptr;
        RG_CUDA_TRY(cudaMalloc(&pl->d_hist, sizeof(double2) * need));
        pl->hist_cap = need;
      }
      // the smooth moment path's per-cell scratch (folded moments, adjoint cubics)
      if (pl->aligned) {
        RG_TRY(smooth_reserve_cells(pl, static_cast<size_t>(max_seg) * pl->sm_cells));
      }
    }
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

  int fill_params(const rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off,
                  const int64_t* d_prefix, int64_t n_single, int nseg, FusedParams& fp) {
    fp          = FusedParams {};
    int  nslots = 0;
    bool aligned = true;
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
    fp.htable      = pl->smooth ? pl->smooth->d_coef : nullptr;
    fp.hseg        = pl->smooth ? pl->smooth->nseg : kSmoothSegments;
    fp.frac        = pl->frac;
    fp.partials    = pl->d_partials;
    fp.nslices     = pl->nslices;
    fp.status      = pl->d_status;
    return nslots;
  }

  // Launch entry points for callers that supply every device buffer themselves
  // (the allocation-free spectrum in noalloc.cu): the reference-table fused
  // kernel over one segment, and the block/warp reduction into `out`.
  int launch_fused_reference(int K, const FusedParams& fp, int grid, cudaStream_t s) {
    RG_CUDA_TRY(launch_fused_mode<kModeRef>(K, fp, dim3(grid, 1), fused_smem(kModeRef, 0, fp.nslots), s));
    return RG_OK;
  }

  // Loads the reference-table fused kernels (every row count K) and the reduction on the
  // current device, so that a later launch needs no module load (a load reserves device
  // memory for the code under CUDA's lazy loading).
  int preload_reference_kernels() {
#define RG_K_LOAD(k) RG_CUDA_TRY((configure_fused_k<k, kModeRef>()));
    RG_K_LOAD(1) RG_K_LOAD(2) RG_K_LOAD(3) RG_K_LOAD(4) RG_K_LOAD(5) RG_K_LOAD(6) RG_K_LOAD(7) RG_K_LOAD(8)
    RG_K_LOAD(9) RG_K_LOAD(10) RG_K_LOAD(11) RG_K_LOAD(12) RG_K_LOAD(13) RG_K_LOAD(14) RG_K_LOAD(15)
    RG_K_LOAD(16)
#undef RG_K_LOAD
    cudaFuncAttributes attr {};
    RG_CUDA_TRY(cudaFuncGetAttributes(&attr, reduce_partials_kernel));
    return RG_OK;
  }

  int launch_reduce_single(const double* partials, int grid, int64_t n, int nbins, const float* ebins,
                           const uint8_t* valid, const unsigned* status, float* out, cudaStream_t s) {
    ReduceParams rp {};
    rp.partials    = partials;
    rp.item_prefix = nullptr;
    rp.n_single    = n;
    rp.grid        = grid;
    rp.nslices     = 1;
    rp.nseg        = 1;
    rp.nbins       = nbins;
    rp.ebins       = ebins;
    rp.valid       = valid;
    rp.status      = status;
    rp.out         = out;
    reduce_partials_kernel<<<dim3((nbins + 31) / 32, 1), dim3(32, kReduceRows), 0, s>>>(rp);
    RG_CUDA_TRY(cudaGetLastError());
    return RG_OK;
  }

  int item_prefix(rg_spectrum_plan* pl, const int64_t* d_off, int nseg, int64_t n, cudaStream_t s) {
    item_prefix_kernel<<<1, 1024, 0, s>>>(d_off, nseg, n, pl->d_prefix, pl->d_status);
    RG_CUDA_TRY(cudaGetLastError());
    return RG_OK;
  }

  namespace {

    // The reduction of a launch's partial rows into `out` (nseg x nbins): `grid` blocks over
    // the items of n_single particles (or of the segments of d_prefix).
    int reduce_rows(rg_spectrum_plan* pl, const int64_t* d_prefix, int64_t n_single, int grid, int nseg,
                    float* out, cudaStream_t s) {
      ReduceParams rp {};
      rp.partials    = pl->d_partials;
      rp.item_prefix = d_prefix;
      rp.n_single    = n_single;
      rp.grid        = grid;
      rp.nslices     = pl->nslices;
      rp.nseg        = nseg;
      rp.nbins       = pl->nbins;
      rp.ebins       = pl->d_ebins;
      rp.valid       = pl->d_valid;
      rp.status      = pl->d_status;
      rp.out         = out;
      dim3 rgrid((pl->nbins + 31) / 32, nseg);
      reduce_partials_kernel<<<rgrid, dim3(32, kReduceRows), 0, s>>>(rp);
      RG_CUDA_TRY(cudaGetLastError());
      return RG_OK;
    }

    // Blocks of the fused kernel over a single segment of n particles.
    int single_segment_grid(const rg_spectrum_plan* pl, int64_t n) {
      const int64_t items = (n + kChunk - 1) / kChunk;
      return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(items, pl->grid)));
    }

    // Launches fused + reduce.  `d_off` (device, nseg + 1) may be null for a
    // single segment [0, n_single).
    int run_fused(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off,
                  int64_t n_single, int nseg, float* out, cudaStream_t s) {
      if (nseg <= 0 || pl->nbins == 0) {
        return RG_OK;
      }
      if (pl->zero) {
        RG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * pl->nbins * nseg, s));
        return RG_OK;
      }
      if (moments_selected(pl, nseg)) {
        RG_TRY(moments_begin(pl, nseg, s));
        RG_TRY(moments_deposit(pl, comp, d_off, n_single, nseg, s));
        return moments_finish(pl, nseg, out, s);
      }
      if (pl->algo == RG_ALGO_MOMENTS) {
        return set_error(RG_ERR_UNSUPPORTED, "this plan or run cannot use the interval-moment algorithm");
      }
      RG_TRY(plan_reserve(pl, nseg));
      const int64_t* d_prefix = nullptr;
      if (d_off) {
        RG_TRY(item_prefix(pl, d_off, nseg, n_single, s));
        d_prefix = pl->d_prefix;
      }
      FusedParams fp;
      const int   nslots = fill_params(pl, comp, d_off, d_prefix, n_single, nseg, fp);
      // a single segment with fewer items than blocks uses fewer blocks
      const int G = d_off ? pl->grid : single_segment_grid(pl, n_single);
      const bool any = d_off ? true : n_single > 0;
      if (any) {
        RG_TRY(timed_launch(pl, fp, dim3(G, pl->nslices), fused_smem(pl->table_mode, fp.hseg, nslots), s));
      }
      return reduce_rows(pl, d_prefix, n_single, G, nseg, out, s);
    }

    // One chunk of a host-resident run (a single segment of n particles): the blocks write
    // their partial rows (first chunk) or add to them (later chunks, no larger than the
    // first); the rows are reduced once after the last chunk.
    int run_fused_chunk(rg_spectrum_plan* pl, const float* const comp[kComps], int64_t n, bool accumulate,
                        cudaStream_t s) {
      RG_TRY(plan_reserve(pl, 1));
      FusedParams fp;
      const int   nslots = fill_params(pl, comp, nullptr, nullptr, n, 1, fp);
      fp.accumulate      = accumulate ? 1 : 0;
      if (n > 0) {
        RG_TRY(timed_launch(pl, fp, dim3(single_segment_grid(pl, n), pl->nslices),
                            fused_smem(pl->table_mode, fp.hseg, nslots), s));
      }
      return RG_OK;
    }

    std::mutex& oneshot_mutex() {
      static std::mutex m;
      return m;
    }

  } // namespace

  // A plan for particles or (source kSrcDist) for one tabulated distribution; only particle
  // plans over log-uniform bins take a bin-aligned smooth table.
  int create_plan(const float* bins, int32_t nbins, float B0, float g_syn, float e_syn_at_g_syn,
                  int32_t table_mode, int source, rg_spectrum_plan** plan) {
  rg::clear_error();
  if (!plan) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan pointer");
  }
  *plan = nullptr;
  if (table_mode != RG_TABLE_REFERENCE && table_mode != RG_TABLE_SMOOTH) {
    return rg::set_error(RG_ERR_ARGUMENT, "unknown table mode");
  }
  if (B0 == 0.0f) {
    return rg::set_error(RG_ERR_ARGUMENT, "B0 must be non-zero");
  }
  auto pl        = std::make_unique<rg_spectrum_plan>();
  pl->table_mode = table_mode;
  pl->source     = source;
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
  if (table_mode == RG_TABLE_SMOOTH && !pl->zero && source == rg::kSrcParticles) {
    // log-uniform bins: the plan's own smooth table aligned to them (moments_smooth.cu)
    st = rg::smooth_align_plan(pl.get(), std::log(K0));
    if (st != RG_OK) {
      rg_spectrum_plan_destroy(pl.release());
      return st;
    }
  }
  double ln_xmin, dln;
  int    nseg;
  rg::table_geometry(pl.get(), ln_xmin, dln, nseg);
  st = rg::plan_prepare_bins(pl.get(), ln_xmin, dln, nseg, pl->zero ? 0.0 : std::log(K0));
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

} // namespace rg

extern "C" {

int rg_spectrum_plan_create(const float* bins, int32_t nbins, float B0, float g_syn,
                            float e_syn_at_g_syn, int32_t table_mode, rg_spectrum_plan** plan) {
  return rg::create_plan(bins, nbins, B0, g_syn, e_syn_at_g_syn, table_mode, rg::kSrcParticles, plan);
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
  rg::moments_free(pl);
  for (auto* v : { &pl->ev_used, &pl->ev_free }) {
    for (auto& e : *v) {
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
  }
  delete pl;
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
    if (st & rg::kDevBadIndex) {
      return rg::set_error(RG_ERR_CUDA, "a particle-stream index self-check failed on the GPU (status " +
                                          std::to_string(st) + "); results are invalid");
    }
    return rg::set_error(RG_ERR_TIMEOUT, "a bounded wait on the GPU gave up (status " + std::to_string(st) +
                                           "); results are invalid");
  }
  return RG_OK;
}

int rg_spectrum_plan_probe_stage_timeout(rg_spectrum_plan* pl, uint32_t polls, void* stream) {
  if (!pl) {
    return rg::set_error(RG_ERR_ARGUMENT, "null plan");
  }
  if (polls == 0 || polls > rg::kWaitLimit) {
    return rg::set_error(RG_ERR_ARGUMENT, "polls must be in [1, " + std::to_string(rg::kWaitLimit) + "]");
  }
  rg::stage_wait_probe_kernel<<<1, 64, 0, static_cast<cudaStream_t>(stream)>>>(pl->d_status, polls);
  RG_CUDA_TRY(cudaGetLastError());
  return RG_OK;
}

int rg_spectrum_plan_smooth_table(const rg_spectrum_plan* pl, float* coef, int32_t* nseg, double* ln_xmin,
                                  double* dln) {
  if (!pl || pl->table_mode != RG_TABLE_SMOOTH || !pl->smooth) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_plan_smooth_table: needs a smooth-table plan");
  }
  const rg::SmoothTable* t = pl->smooth;
  if (nseg) {
    *nseg = t->nseg;
  }
  if (ln_xmin) {
    *ln_xmin = t->ln_xmin;
  }
  if (dln) {
    *dln = t->dln;
  }
  if (coef) {
    RG_CUDA_TRY(cudaMemcpy(coef, t->d_coef, sizeof(float4) * t->nseg, cudaMemcpyDeviceToHost));
  }
  return RG_OK;
}

int rg_spectrum_plan_set_algorithm(rg_spectrum_plan* pl, int32_t algo) {
  if (!pl || (algo != RG_ALGO_AUTO && algo != RG_ALGO_DIRECT && algo != RG_ALGO_MOMENTS)) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_plan_set_algorithm: bad arguments");
  }
  pl->algo = algo;
  return RG_OK;
}

int rg_spectrum_plan_algorithm(const rg_spectrum_plan* pl, int32_t nseg, int32_t* algo) {
  if (!pl || !algo || nseg < 1) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_plan_algorithm: bad arguments");
  }
  *algo = rg::moments_selected(pl, nseg) ? RG_ALGO_MOMENTS : RG_ALGO_DIRECT;
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

int rg_spectrum_run(const rg_spectrum_plan* plan, const rg_particles* p, float* out, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrum");
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

int rg_spectrum_run_placed(rg_spectrum_plan* plan, const rg_particles* p, float* out, void* placement,
                           void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrum");
  if (!plan || !placement || (!out && plan->nbins > 0) || plan->source != rg::kSrcParticles) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_run_placed: bad arguments");
  }
  RG_TRY(rg::check_particles(p));
  if (plan->zero || plan->nbins == 0 || !plan->aligned || !rg::moments_selected(plan, 1)) {
    return rg::set_error(RG_ERR_UNSUPPORTED,
                         "rg_spectrum_run_placed: needs a plan that runs cell moments on its bin-aligned smooth table");
  }
  const float* comp[rg::kComps];
  rg::particle_comps(p, comp);
  auto s = static_cast<cudaStream_t>(stream);
  RG_TRY(rg::moments_begin(plan, 1, s));
  RG_TRY(rg::smooth_moments_deposit(plan, comp, nullptr, p->n, 1, s, static_cast<uint2*>(placement)));
  return rg::moments_finish(plan, 1, out, s);
}

int rg_spectrum_run_batched(rg_spectrum_plan* plan, const rg_particles* p, const int64_t* offsets,
                            int32_t nseg, float* out, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrum");
  if (!plan || !offsets || nseg < 0 || (!out && nseg > 0 && plan->nbins > 0)) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_run_batched: null argument");
  }
  RG_TRY(rg::check_particles(p));
  const float* comp[rg::kComps];
  rg::particle_comps(p, comp);
  return rg::run_fused(plan, comp, offsets, p->n, nseg, out, static_cast<cudaStream_t>(stream));
}

int rg_spectrum_run_host(rg_spectrum_plan* pl, const rg_particles* p, float* out, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrum");
  if (!pl || (!out && pl->nbins > 0) || pl->source != rg::kSrcParticles) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_run_host: bad arguments");
  }
  RG_TRY(rg::check_particles(p));
  if (pl->nbins == 0) {
    return RG_OK;
  }
  auto s = static_cast<cudaStream_t>(stream);
  if (pl->zero) {
    RG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * pl->nbins, s));
    return RG_OK;
  }
  // 2^22-particle chunks, double-buffered (each chunk costs a kernel launch and tail, so
  // chunks are kept large; 2^21-particle chunks and a third buffer were measured slower or
  // no faster).  The chunks' blocks accumulate into their partial rows and one reduction
  // at the end writes the spectrum.
  rg::HostStaging* st = nullptr;
  RG_TRY(rg::host_staging(&st));
  constexpr int64_t kStageChunk = rg::HostStaging::kChunk;
  constexpr int     kBuffers    = rg::HostStaging::kBuffers;
  const float*      host[rg::kComps];
  rg::particle_comps(p, host);
  // consumed[b] was last recorded after the kernel that read staging buffer b (in an
  // earlier call on this device, by any plan, or never): the first copies of this call
  // wait for exactly that, so they overlap the tail of the previous call's kernels
  std::lock_guard<std::mutex> lock(st->mu);
  const int64_t               n       = p->n;
  const bool                  moments = rg::moments_selected(pl, 1);
  if (!moments && pl->algo == RG_ALGO_MOMENTS) {
    return rg::set_error(RG_ERR_UNSUPPORTED, "this plan cannot use the interval-moment algorithm");
  }
  if (moments) {
    RG_TRY(rg::moments_begin(pl, 1, s));
  }
  for (int64_t a = 0; a < n; a += kStageChunk) {
    const int     b = static_cast<int>(st->issued++ % kBuffers);
    const int64_t m = std::min(kStageChunk, n - a);
    RG_CUDA_TRY(cudaStreamWaitEvent(st->copy_stream, st->consumed[b], 0));
    const float* dev[rg::kComps] = {};
    for (int k = 0; k < rg::kComps; ++k) {
      if (host[k]) {
        float* dst = st->d_stage[b] + k * kStageChunk;
        RG_CUDA_TRY(cudaMemcpyAsync(dst, host[k] + a, sizeof(float) * m, cudaMemcpyHostToDevice,
                                    st->copy_stream));
        dev[k] = dst;
      }
    }
    RG_CUDA_TRY(cudaEventRecord(st->copied[b], st->copy_stream));
    RG_CUDA_TRY(cudaStreamWaitEvent(s, st->copied[b], 0));
    if (moments) {
      RG_TRY(rg::moments_deposit(pl, dev, nullptr, m, 1, s));
    } else {
      RG_TRY(rg::run_fused_chunk(pl, dev, m, a > 0, s));
    }
    RG_CUDA_TRY(cudaEventRecord(st->consumed[b], s));
  }
  if (moments) {
    return rg::moments_finish(pl, 1, out, s);
  }
  // the rows the chunks accumulated: as many blocks as the first (largest) chunk used
  const int64_t first = std::min(kStageChunk, n);
  return rg::reduce_rows(pl, nullptr, first, rg::single_segment_grid(pl, first), 1, out, s);
}

int rg_spectrum_run_plain(const rg_spectrum_plan* cplan, const rg_particles* p, float* out,
                          void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrum");
  auto* plan = const_cast<rg_spectrum_plan*>(cplan);
  if (!plan || plan->source != rg::kSrcParticles || plan->table_mode != RG_TABLE_REFERENCE) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_spectrum_run_plain: needs a reference-table particle plan");
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
    RG_CUDA_TRY(cudaFuncSetAttribute(rg::plain_spectrum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
  }
  if (p->n > 0) {
    const int64_t need   = (p->n + 255) / 256;
    const int     blocks = static_cast<int>(std::min<int64_t>(need, ctx->sms * 8));
    rg::plain_spectrum_kernel<<<blocks, 256, smem, s>>>(pp);
    RG_CUDA_TRY(cudaGetLastError());
  }
  rg::f64_to_f32_kernel<<<(plan->nbins + 255) / 256, 256, 0, s>>>(plan->d_plain_acc, out, plan->nbins);
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
      RG_TRY(rg_spectrum_plan_create(bins, nbins, B0, g_syn, e_syn_at_g_syn, RG_TABLE_REFERENCE, &pl));
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

int rg_dist_run(const rg_spectrum_plan* plan, const float* gbeta, const float* f, int32_t ng, float* out,
                void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrumFromDist");
  if (!plan || plan->source != rg::kSrcDist || ng < 0 || (ng > 0 && (!gbeta || !f)) ||
      (!out && plan->nbins > 0)) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_dist_run: bad arguments");
  }
  // the distribution source reads comp[0] = gbeta and comp[1] = f
  const float* comp[rg::kComps] = {};
  comp[0]                       = gbeta;
  comp[1]                       = f;
  return rg::run_fused(const_cast<rg_spectrum_plan*>(plan), comp, nullptr, ng, 1, out,
                       static_cast<cudaStream_t>(stream));
}

int rg_synchrotron_spectrum_from_dist(const float* gbeta, const float* f, int32_t ng,
                                      int32_t log_spaced, const float* bins, int32_t nbins,
                                      float g_syn, float e_syn_at_g_syn, float* out, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrumFromDist");
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
    double ln_xmin, dln;
    int    nseg;
    rg::table_geometry(pl.get(), ln_xmin, dln, nseg);
    st = rg::plan_prepare_bins(pl.get(), ln_xmin, dln, nseg, pl->zero ? 0.0 : std::log(K0));
  }
  auto s = static_cast<cudaStream_t>(stream);
  if (st == RG_OK) {
    const float* comp[rg::kComps] = {};
    comp[0]                       = gbeta;
    comp[1]                       = f;
    st                            = rg::run_fused(pl.get(), comp, nullptr, ng, 1, out, s);
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

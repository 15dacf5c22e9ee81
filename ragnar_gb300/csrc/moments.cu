// Particle synchrotron spectrum by interval moments (reference table).
//
// Reference path: SynchrotronSpectrum<D> (synchrotron.cpp:107-145) summing
// sync::Kernel<D>::operator() (synchrotron.hpp:145-172) over every (particle,
// photon bin) pair, with F from the 200-point table interpolated linearly in
// log x (InterpolateTabulatedFunction<true>, tabulation.hpp:19-53).
//
// The spectrum is the same sum, S_b = e_b sum_p A_p f(P_b - Q_p), of the same
// function f of the same fixed-point table coordinate as the fused kernel
// (spectrum.cu): Q_p is the particle's coordinate, P_b the bin's, and
// f(T) = c0[T >> F] + c1[T >> F] (T mod 2^F) is piecewise linear with its
// kinks where T is a multiple of 2^F (F fraction bits per table segment: 30 here,
// 8 more than the fused kernel's 32-bit coordinate, because the log-linear
// lerp of the steep high-x tail of F magnifies a coordinate's rounding up to a
// thousandfold).  Write R = Pmax - Q (Pmax: the largest bin coordinate of the
// slice) and D_b = Pmax - P_b, so T = R - D_b, and split both into a cell (bits F
// and up) and a low part: R = (Rc, Rl), D_b = (Dc_b, Dl_b).  Then the segment of
// (p, b) is Rc - Dc_b when Rl >= Dl_b and Rc - Dc_b - 1 otherwise, and the
// position inside it is Rl - Dl_b (+ 2^F).  So within an
// interval of R that lies in one cell and between two consecutive low parts
// Dl of the slice's bins, every bin's f is one linear function of Rl, and the
// sums over the particles in that interval need only
//     M0 = sum A_p,   M1 = sum A_p Rl_p.
// The deposit kernel computes each particle's (Q, A) once, with the fused
// kernel's double-float kinematics and the same atanh-series logarithm, finds
// its interval (cell, rank of Rl among the sorted Dl) and adds (A, A Rl) to
// that interval's FP64 moments; a scan turns each cell's row of
// interval moments into prefix sums, and the reduce kernel sums, for every bin,
// over the at most 200 cells its table segments reach:
//     S_b / e_b = sum_cells c0[s] U0 + c1[s] (U1 - Dl_b U0)
//                         + c0[s-1] L0 + c1[s-1] (L1 - (Dl_b - 2^F) L0),
// s = Rc - Dc_b, L = moments of the cell's intervals below Dl_b, U = the rest.
// The work is one particle stage per particle plus (cells x bins), not
// (particles x bins), and the per-(particle, bin) value of f is summed exactly
// (FP64 moments and coefficients) instead of being rounded to FP32 per eval.
// The FP64 atomic sums make the result independent of the particle order up to
// FP64 rounding, not bit for bit.
#include "moments_common.cuh"
#include "spectrum_plan.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>
#include <type_traits>
#include <vector>

namespace rg {

  namespace {

    constexpr int kMomFrac       = kFrac + 8;        // fraction bits of the coordinate
    constexpr int kMomBuckets    = 4096;             // buckets over the low kMomFrac bits
    constexpr int kMomBucketBits = kMomFrac - 12;
    constexpr int kMomSharedSeg  = 1024;             // segment offsets staged in shared memory
    constexpr int kMomThreads    = 256;
    constexpr int kMomMaxTable   = 256;              // largest reference table (segments) this path takes
    constexpr size_t kMomMaxBytes = size_t(8) << 30; // histogram memory above which the fused kernel runs

    struct MomentParams {
      FusedParams     fp;      // streams, kinematics constants, status
      const int64_t*  range;   // per slice: (Pmin, Pmax) in kMomFrac units
      int64_t         L;       // table segments << kMomFrac
      const int64_t*  seg_off; // nseg + 1 particle offsets (device), or null: particles [0, n)
      int             nseg;
      int64_t         n;       // stream length
      const int4*     mslice;  // per slice: (valid bins, cells, histogram offset, 0)
      const int32_t*  thr;     // per slice: kSliceBins sorted low parts
      const uint16_t* bucket;  // per slice: kMomBuckets + 1 threshold starts
      double2*        hist;    // nseg x per_seg interval moments (M0, M1)
      int64_t         per_seg;
    };

    template <bool kI32>
    __global__ void __launch_bounds__(kMomThreads) moments_deposit_kernel(const __grid_constant__ MomentParams m) {
      __shared__ int32_t  thr[kSliceBins];
      __shared__ uint16_t bucket[kMomBuckets + 1];
      __shared__ int64_t  soff[kMomSharedSeg + 1];
      const int  slice = blockIdx.y;
      const int4 ms    = m.mslice[slice];
      const int  nv = ms.x, nc = ms.y;
      for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        thr[i] = m.thr[slice * kSliceBins + i];
      }
      for (int i = threadIdx.x; i <= kMomBuckets; i += blockDim.x) {
        bucket[i] = m.bucket[slice * (kMomBuckets + 1) + i];
      }
      bool bad = false;
      if (m.seg_off) {
        for (int i = threadIdx.x; i <= m.nseg; i += blockDim.x) {
          soff[i] = m.seg_off[i];
        }
        __syncthreads();
        // offsets must not decrease and must lie in [0, n]
        for (int i = threadIdx.x; i < m.nseg; i += blockDim.x) {
          bad = bad || soff[i + 1] < soff[i] || soff[i] < 0 || soff[i + 1] > m.n;
        }
      }
      if (__syncthreads_or(bad)) {
        if (threadIdx.x == 0 && blockIdx.x == 0 && slice == 0) {
          atomicOr(m.fp.status, kDevBadOffsets);
        }
        return;
      }
      if (__syncthreads_or(*m.fp.status != kDevOk)) {
        return;
      }
      const int64_t  Pmin = m.range[2 * slice], Pmax = m.range[2 * slice + 1];
      const int      row    = nv + 1;
      double2*       base   = m.hist + ms.z;
      const int64_t  first  = m.seg_off ? soff[0] : 0;
      const int64_t  last   = m.seg_off ? soff[m.nseg] : m.n;
      // 32-bit particle indices when the stream allows it (the host checks last + stride < 2^32)
      using Idx          = std::conditional_t<kI32, uint32_t, int64_t>;
      const Idx  stride  = static_cast<Idx>(gridDim.x) * blockDim.x;
      const Idx  i0      = static_cast<Idx>(first + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x);
      const Idx  iend    = static_cast<Idx>(last);
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
        if (!moment_particle_stage(v, m.fp, Pmin, Pmax, m.L, Q, A)) {
          continue;
        }
        // live particles have 0 <= Pmax - Q < Pmax - Pmin + L
        const uint64_t R  = static_cast<uint64_t>(Pmax - Q);
        const uint32_t Rc = static_cast<uint32_t>(R >> kMomFrac);
        const uint32_t Rl = static_cast<uint32_t>(R) & ((1u << kMomFrac) - 1u);
        // rank of Rl among the slice's sorted low parts: its bucket, then a binary
        // search over the thresholds inside the bucket
        const uint32_t k  = Rl >> kMomBucketBits;
        int            lo = bucket[k], hi = bucket[k + 1];
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (static_cast<uint32_t>(thr[mid]) <= Rl) {
            lo = mid + 1;
          } else {
            hi = mid;
          }
        }
        if (Rc >= static_cast<uint32_t>(nc) || seg >= m.nseg) { // self-check: never taken for live particles
          atomicOr(m.fp.status, kDevBadIndex);
          continue;
        }
        double2* h = base + seg * m.per_seg + static_cast<int64_t>(Rc) * row + lo;
        if (fabsf(A) >= 1.17549435e-38f) { // amplitudes may be negative (negative weights or B0)
          atomicAdd(&h->x, float_to_double_bits(A));
          atomicAdd(&h->y, product_to_double_bits(A, Rl));
        } else if (A != 0.0f) { // subnormal amplitude (rare): the FP64 pipe
          atomicAdd(&h->x, static_cast<double>(A));
          atomicAdd(&h->y, static_cast<double>(A) * static_cast<double>(Rl));
        }
      }
    }

    // In-place inclusive prefix sums along each cell's row of interval moments: one warp
    // per row (cell), rows of (segment, slice) blockIdx.y.  Each lane takes a contiguous
    // chunk of the row (its loads independent, all in flight at once), sums it, and adds
    // the exclusive warp scan of the chunk totals.
    constexpr int kScanChunk = (kSliceBins + 1 + 31) / 32; // entries per lane for the longest row

    __global__ void __launch_bounds__(256) moments_scan_kernel(double2* hist, const int4* mslice, int nslices,
                                                               int64_t per_seg) {
      const int  seg = blockIdx.y / nslices, slice = blockIdx.y % nslices;
      const int4 ms  = mslice[slice];
      const int  lane = threadIdx.x & 31;
      const int  cell = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
      if (cell >= ms.y) {
        return;
      }
      const int row = ms.x + 1;
      const int C   = (row + 31) >> 5;
      const int j0  = lane * C;
      double2*  r   = hist + seg * per_seg + ms.z + static_cast<int64_t>(cell) * row;
      double2   v[kScanChunk];
#pragma unroll
      for (int k = 0; k < kScanChunk; ++k) {
        v[k] = (k < C && j0 + k < row) ? r[j0 + k] : make_double2(0.0, 0.0);
      }
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int k = 0; k < kScanChunk; ++k) {
        s0 += v[k].x;
        s1 += v[k].y;
        v[k] = make_double2(s0, s1);
      }
      // inclusive scan of the chunk totals, shifted by one lane: the exclusive offsets
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double a = __shfl_up_sync(0xffffffffu, s0, o);
        const double b = __shfl_up_sync(0xffffffffu, s1, o);
        if (lane >= o) {
          s0 += a;
          s1 += b;
        }
      }
      double e0 = __shfl_up_sync(0xffffffffu, s0, 1), e1 = __shfl_up_sync(0xffffffffu, s1, 1);
      if (lane == 0) {
        e0 = 0.0;
        e1 = 0.0;
      }
#pragma unroll
      for (int k = 0; k < kScanChunk; ++k) {
        if (k < C && j0 + k < row) {
          r[j0 + k] = make_double2(v[k].x + e0, v[k].y + e1);
        }
      }
    }

    struct MomentReduceParams {
      const double2*  hist;
      int64_t         per_seg;
      const int4*     mslice;
      const int4*     binfo;    // per bin: (sorted position, cell offset Dc, low part Dl, valid)
      const double2*  coef;     // per table segment: (c0, c1 per fraction bit), FP64
      int             nseg_tab; // table segments
      int             nbins;
      const float*    ebins;
      const unsigned* status;
      float*          out;      // nseg x nbins
    };

    // One 256-thread block per (bin, segment): each thread takes every 256th cell the bin's
    // table segments reach (at most nseg_tab + 1 cells), then the block sums in a fixed order.
    constexpr int kMomRedThreads = 256;

    __global__ void __launch_bounds__(kMomRedThreads) moments_reduce_kernel(const __grid_constant__ MomentReduceParams r) {
      __shared__ double wsum[kMomRedThreads / 32];
      const int  bin    = blockIdx.x;
      const int  seg    = blockIdx.y;
      const bool failed = *r.status != kDevOk;
      const int4 bi     = r.binfo[bin];
      double     sum    = 0.0;
      if (bi.w && !failed) {
        const int4     ms  = r.mslice[bin / kSliceBins];
        const int      row = ms.x + 1;
        const double2* h   = r.hist + seg * r.per_seg + ms.z;
        const int      pos = bi.x, Dc = bi.y;
        const double   Dl = static_cast<double>(bi.z), Dlw = Dl - static_cast<double>(1u << kMomFrac);
        const int      c_end = min(ms.y, Dc + r.nseg_tab + 1);
        for (int c = Dc + threadIdx.x; c < c_end; c += kMomRedThreads) {
          const double2 Lm = h[static_cast<int64_t>(c) * row + pos];
          const double2 Tm = h[static_cast<int64_t>(c) * row + ms.x];
          const int     s  = c - Dc;
          if (s < r.nseg_tab) { // intervals at or above Dl: segment s
            const double2 k  = __ldg(r.coef + s);
            const double  U0 = Tm.x - Lm.x, U1 = Tm.y - Lm.y;
            sum += k.x * U0 + k.y * (U1 - Dl * U0);
          }
          if (s >= 1) { // intervals below Dl: segment s - 1, position Rl - Dl + 2^F
            const double2 k = __ldg(r.coef + s - 1);
            sum += k.x * Lm.x + k.y * (Lm.y - Dlw * Lm.x);
          }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
      }
      if ((threadIdx.x & 31) == 0) {
        wsum[threadIdx.x >> 5] = sum;
      }
      __syncthreads();
      if (threadIdx.x != 0) {
        return;
      }
      double result = 0.0;
      if (failed) {
        result = __longlong_as_double(0x7ff8000000000000LL);
      } else if (bi.w) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < kMomRedThreads / 32; ++w) {
          t += wsum[w];
        }
        result = t * static_cast<double>(r.ebins[bin]);
      }
      r.out[static_cast<int64_t>(seg) * r.nbins + bin] = __double2float_rn(result);
    }

    int max_cells(const rg_spectrum_plan* pl) {
      int m = 1;
      for (int s = 0; s < pl->nslices; ++s) {
        m = std::max(m, pl->h_mslice[4 * s + 1]);
      }
      return m;
    }

  } // namespace

  // Interval tables of a reference-table particle plan: the bins' coordinates in
  // kMomFrac units (FP64 on the host, as the fused kernel's in kFrac units), their
  // validity, and the table geometry (ln xmin, dln) and ln K0 the coordinates use.
  int moments_prepare(rg_spectrum_plan* pl, const std::vector<uint8_t>& valid, double ln_xmin, double dln,
                      double ln_k0) {
    pl->moments_ok = false;
    if (pl->table_mode == kModeSmooth && pl->aligned) {
      return smooth_moments_prepare(pl, ln_k0);
    }
    if (pl->table_mode != kModeRef || pl->source != kSrcParticles || pl->ref->n - 1 > kMomMaxTable) {
      return RG_OK;
    }
    const int            ns    = pl->nslices;
    const double         scale = std::ldexp(1.0, kMomFrac) / dln;
    const int64_t        L     = static_cast<int64_t>(pl->ref->n - 1) << kMomFrac;
    const int64_t        mask  = (int64_t(1) << kMomFrac) - 1;
    std::vector<int64_t> Ps(std::max(pl->nbins, 1), 0);
    std::vector<int64_t> range(2 * static_cast<size_t>(ns), 0);
    std::vector<int32_t> thr(static_cast<size_t>(ns) * kSliceBins, 0);
    std::vector<uint16_t> bucket(static_cast<size_t>(ns) * (kMomBuckets + 1), 0);
    std::vector<int4>    binfo(std::max(pl->nbins, 1), make_int4(0, 0, 0, 0));
    pl->h_mslice.assign(4 * static_cast<size_t>(ns), 0);
    int64_t off = 0;
    for (int s = 0; s < ns; ++s) {
      std::vector<int> idx;
      int64_t          Pmin = std::numeric_limits<int64_t>::max(), Pmax = std::numeric_limits<int64_t>::min();
      for (int j = 0; j < kSliceBins; ++j) {
        const int b = s * kSliceBins + j;
        if (b < pl->nbins && valid[b]) {
          Ps[b] = std::llround((std::log(static_cast<double>(pl->h_bins[b])) - ln_xmin - ln_k0) * scale);
          Pmin  = std::min(Pmin, Ps[b]);
          Pmax  = std::max(Pmax, Ps[b]);
          idx.push_back(b);
        }
      }
      if (idx.empty()) {
        Pmin = Pmax = 0;
      }
      range[2 * s]     = Pmin;
      range[2 * s + 1] = Pmax;
      const auto low = [&](int b) { return static_cast<int32_t>((Pmax - Ps[b]) & mask); };
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return low(a) < low(b); });
      const int nv = static_cast<int>(idx.size());
      for (int k = 0; k < nv; ++k) {
        const int b = idx[k];
        thr[static_cast<size_t>(s) * kSliceBins + k] = low(b);
        binfo[b] = make_int4(k, static_cast<int>((Pmax - Ps[b]) >> kMomFrac), low(b), 1);
      }
      for (int k = 0; k <= kMomBuckets; ++k) {
        const int64_t edge = static_cast<int64_t>(k) << kMomBucketBits;
        int           c    = 0;
        while (c < nv && thr[static_cast<size_t>(s) * kSliceBins + c] < edge) {
          ++c;
        }
        bucket[static_cast<size_t>(s) * (kMomBuckets + 1) + k] = static_cast<uint16_t>(c);
      }
      // live particles have Pmax - Q in [0, Pmax - Pmin + L)
      const int64_t cells = nv ? ((Pmax - Pmin + L - 1) >> kMomFrac) + 1 : 1;
      if (off + cells * (nv + 1) > std::numeric_limits<int32_t>::max()) {
        return RG_OK; // too large for this path; the fused kernel serves the plan
      }
      pl->h_mslice[4 * s + 0] = nv;
      pl->h_mslice[4 * s + 1] = static_cast<int32_t>(cells);
      pl->h_mslice[4 * s + 2] = static_cast<int32_t>(off);
      off += cells * (nv + 1);
    }
    pl->hist_per_seg = off;
    pl->mom_L        = L;
    // FP64 segment coefficients of the reference's log-linear lerp (tabulation.hpp:39-41)
    // in the ideal coordinate, per coordinate unit: F = c0 + c1 (T mod 2^kMomFrac)
    const int            nt = pl->ref->n - 1;
    std::vector<double2> coef(nt);
    const double         d10 = pl->ref->dln / M_LN10;
    for (int i = 0; i < nt; ++i) {
      const double xa = pl->ref->h_x[i], xb = pl->ref->h_x[i + 1], ya = pl->ref->h_y[i], yb = pl->ref->h_y[i + 1];
      const double beta = (yb - ya) / std::log10(xb / xa);
      const double c0   = ya + beta * (pl->ref->ln_xmin / M_LN10 + i * d10 - std::log10(xa));
      coef[i]           = make_double2(c0, beta * d10 / std::ldexp(1.0, kMomFrac));
    }
    RG_CUDA_TRY(cudaMalloc(&pl->d_mslice, sizeof(int32_t) * pl->h_mslice.size()));
    RG_CUDA_TRY(cudaMalloc(&pl->d_mrange, sizeof(int64_t) * range.size()));
    RG_CUDA_TRY(cudaMalloc(&pl->d_thr, sizeof(int32_t) * thr.size()));
    RG_CUDA_TRY(cudaMalloc(&pl->d_bucket, sizeof(uint16_t) * bucket.size()));
    RG_CUDA_TRY(cudaMalloc(&pl->d_binfo, sizeof(int4) * binfo.size()));
    RG_CUDA_TRY(cudaMalloc(&pl->d_mcoef, sizeof(double2) * std::max(nt, 1)));
    RG_CUDA_TRY(cudaMemcpy(pl->d_mslice, pl->h_mslice.data(), sizeof(int32_t) * pl->h_mslice.size(),
                           cudaMemcpyHostToDevice));
    RG_CUDA_TRY(cudaMemcpy(pl->d_mrange, range.data(), sizeof(int64_t) * range.size(), cudaMemcpyHostToDevice));
    RG_CUDA_TRY(cudaMemcpy(pl->d_thr, thr.data(), sizeof(int32_t) * thr.size(), cudaMemcpyHostToDevice));
    RG_CUDA_TRY(cudaMemcpy(pl->d_bucket, bucket.data(), sizeof(uint16_t) * bucket.size(), cudaMemcpyHostToDevice));
    RG_CUDA_TRY(cudaMemcpy(pl->d_binfo, binfo.data(), sizeof(int4) * binfo.size(), cudaMemcpyHostToDevice));
    RG_CUDA_TRY(cudaMemcpy(pl->d_mcoef, coef.data(), sizeof(double2) * nt, cudaMemcpyHostToDevice));
    pl->moments_ok = true;
    return RG_OK;
  }

  // Whether a run over nseg segments takes the interval-moment path.
  bool moments_selected(const rg_spectrum_plan* pl, int nseg) {
    if (!pl->moments_ok || pl->algo == RG_ALGO_DIRECT || nseg > kMomSharedSeg) {
      return false;
    }
    return static_cast<size_t>(nseg) * static_cast<size_t>(pl->hist_per_seg) * sizeof(double2) <= kMomMaxBytes;
  }

  // Zeroes the interval moments of nseg segments (allocating them on first use).
  int moments_begin(rg_spectrum_plan* pl, int nseg, cudaStream_t s) {
    const size_t need = static_cast<size_t>(nseg) * static_cast<size_t>(pl->hist_per_seg);
    if (need > pl->hist_cap) {
      cudaFree(pl->d_hist);
      pl->d_hist = nullptr;
      RG_CUDA_TRY(cudaMalloc(&pl->d_hist, sizeof(double2) * need));
      pl->hist_cap = need;
    }
    RG_CUDA_TRY(cudaMemsetAsync(pl->d_hist, 0, sizeof(double2) * need, s));
    return RG_OK;
  }

  // Adds the particles [0, n) (one segment, d_off null) or the nseg segments of d_off to
  // the interval moments.
  int moments_deposit(rg_spectrum_plan* pl, const float* const comp[kComps], const int64_t* d_off, int64_t n,
                      int nseg, cudaStream_t s) {
    if (pl->aligned) {
      return smooth_moments_deposit(pl, comp, d_off, n, nseg, s);
    }
    MomentParams m {};
    fill_params(pl, comp, nullptr, nullptr, n, 1, m.fp);
    m.range   = pl->d_mrange;
    m.L       = pl->mom_L;
    m.seg_off = d_off;
    m.nseg    = d_off ? nseg : 1;
    m.n       = n;
    m.mslice  = reinterpret_cast<const int4*>(pl->d_mslice);
    m.thr     = pl->d_thr;
    m.bucket  = pl->d_bucket;
    m.hist    = pl->d_hist;
    m.per_seg = pl->hist_per_seg;
    DeviceContext* ctx = nullptr;
    RG_TRY(context(&ctx));
    const int64_t blocks_needed = (n + kMomThreads - 1) / kMomThreads;
    // many more blocks than fit at once (32 per SM, ~6 resident): the blocks that finish early
    // take new ones, which evens out the SMs (measured against 6, 8, 12, 16, 24 and 48 per SM)
    const int     grid          = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(blocks_needed, ctx->sms * 32)));
    if (n == 0 && !d_off) {
      return RG_OK;
    }
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
    if (n + static_cast<int64_t>(grid) * kMomThreads < (int64_t(1) << 32)) {
      moments_deposit_kernel<true><<<dim3(grid, pl->nslices), kMomThreads, 0, s>>>(m);
    } else {
      moments_deposit_kernel<false><<<dim3(grid, pl->nslices), kMomThreads, 0, s>>>(m);
    }
    RG_CUDA_TRY(cudaGetLastError());
    if (pl->timing) {
      RG_CUDA_TRY(cudaEventRecord(ev.second, s));
      pl->ev_used.push_back(ev);
    }
    return RG_OK;
  }

  // Prefix sums of the moments and the per-bin sums into out (nseg x nbins).
  int moments_finish(rg_spectrum_plan* pl, int nseg, float* out, cudaStream_t s) {
    if (pl->aligned) {
      return smooth_moments_finish(pl, nseg, out, s);
    }
    const int warps = 8;
    moments_scan_kernel<<<dim3((max_cells(pl) + warps - 1) / warps, nseg * pl->nslices), 32 * warps, 0, s>>>(
      pl->d_hist, reinterpret_cast<const int4*>(pl->d_mslice), pl->nslices, pl->hist_per_seg);
    RG_CUDA_TRY(cudaGetLastError());
    MomentReduceParams r {};
    r.hist     = pl->d_hist;
    r.per_seg  = pl->hist_per_seg;
    r.mslice   = reinterpret_cast<const int4*>(pl->d_mslice);
    r.binfo    = pl->d_binfo;
    r.coef     = pl->d_mcoef;
    r.nseg_tab = pl->ref->n - 1;
    r.nbins    = pl->nbins;
    r.ebins    = pl->d_ebins;
    r.status   = pl->d_status;
    r.out      = out;
    moments_reduce_kernel<<<dim3(pl->nbins, nseg), kMomRedThreads, 0, s>>>(r);
    RG_CUDA_TRY(cudaGetLastError());
    return RG_OK;
  }

  void moments_free(rg_spectrum_plan* pl) {
    cudaFree(pl->d_mslice);
    cudaFree(pl->d_mrange);
    cudaFree(pl->d_thr);
    cudaFree(pl->d_bucket);
    cudaFree(pl->d_binfo);
    cudaFree(pl->d_mcoef);
    cudaFree(pl->d_hist);
    cudaFree(pl->d_cells);
    cudaFree(pl->d_coef64);
    cudaFree(pl->own_smooth.d_coef);
    pl->d_cells           = nullptr;
    pl->cells_cap         = 0;
    pl->d_coef64          = nullptr;
    pl->own_smooth.d_coef = nullptr;
    pl->d_mslice = nullptr;
    pl->d_mrange = nullptr;
    pl->d_thr    = nullptr;
    pl->d_bucket = nullptr;
    pl->d_binfo  = nullptr;
    pl->d_mcoef  = nullptr;
    pl->d_hist   = nullptr;
    pl->hist_cap = 0;
  }

} // namespace rg

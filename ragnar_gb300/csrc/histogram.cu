// Particles<D>::energyDistribution (particles.cpp:189-260) on sm_103a.
//
// The reference computes Usqr = ux*ux + uy*uy + uz*uz in float, then the bin
// index through a double expression (double log10 of energy/emin, float log10
// of emax/emin), clamping out-of-range energies into bins 0 and n-1.  Because that
// index is a non-decreasing function of the float Usqr alone, the host finds,
// for every k, the smallest float Usqr whose index is >= k (binary search over
// float bit patterns with the reference's own expression).  The GPU computes
// Usqr with the same rounding steps, reads a lower bound of its bin from a table
// over cells of float bit patterns (the bin of each cell's smallest float) and
// steps over the thresholds inside the cell, so every particle lands in exactly
// the bin the reference picks and the counts are bit-exact.
//
// Log-spaced bins add float(1.0 / energy): for |u| energies that is the
// correctly rounded reciprocal of sqrtf(Usqr) (double rounding of one division
// of floats through double is innocuous); for sqrt(1 + Usqr) energies it is a
// double-float Newton step of rsqrt rounded to float.  Sums are accumulated in
// FP32 shared-memory bins (kSumCopies lane-indexed copies) flushed to FP64 every
// chunk, then across blocks in FP64 in a fixed order.
#include "rg_common.cuh"
#include "rg_internal.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <mutex>
#include <vector>

namespace rg {

  namespace {

    constexpr int kHistThreads   = 256;
    // Copies of the FP32 sum bins, lane l adding into copy l mod kSumCopies: the float
    // shared-memory add retries while lanes of a warp hit the same bin, and energies
    // of a power law crowd a few bins (4 copies: 0.155 ms against 0.179 ms per call on
    // 3.3e7 particles; 16 copies were slower).
    constexpr int kSumCopies     = 4;
    constexpr int kHistMaxBins   = 4096;
    constexpr int kFlushParticles = 4096; // per block between FP32 -> FP64 flushes
    // Cells of the bin lookup: the finest cells of float bit patterns (bits >> shift)
    // such that [thr[1], the largest finite threshold] spans at most kMaxCells of them
    // (64 cells per octave for 200 log bins over five decades: at most one threshold
    // per cell).  Against an FP32 log2 estimate corrected both ways: 97.5 M against
    // 113.5 M warp instructions, 121.8 us against 130.8 us for 3.3e7 particles x 200 bins.
    constexpr int kMaxCells = 4096;

    // particles.cpp:224-253, the index of one particle given its float Usqr.
    std::size_t ref_energy_index(float Usqr, bool fourvel, float emin, float emax, std::size_t n) {
      const double energy = fourvel ? static_cast<double>(std::sqrt(Usqr)) : std::sqrt(1.0 + Usqr);
      if (energy < emin) {
        return 0;
      } else if (energy >= emax) {
        return n - 1;
      }
      const auto ei = static_cast<std::size_t>(static_cast<float>(n - 1) *
                                               std::fabs(std::log10(energy / emin)) /
                                               std::log10(emax / emin));
      return ei > n - 1 ? n - 1 : ei;
    }

    float bits_to_float(uint32_t b) {
      float f;
      std::memcpy(&f, &b, 4);
      return f;
    }

    struct HistParams {
      const float*    ux;
      const float*    uy;
      const float*    uz;
      int64_t         n;
      int             nbins;
      int             fourvel;
      int             log_spaced;
      const float*    thr;      // nbins thresholds: thr[k] = smallest Usqr with index >= k (thr[0] = 0)
      int             nan_index;
      const uint16_t* start;        // [ncells + 1]: 0, then the bin of each cell's smallest float
      int             cell_shift;   // cell of a float = its bit pattern >> cell_shift
      int             cell_base;    // cell of thr[1]
      int             ncells;
      unsigned long long* part_counts; // [grid][nbins]
      double*         part_sums;       // [grid][nbins]
    };

    // Bin of one particle: start[ci] is the bin of the smallest float of its cell (entry
    // 0 for cells below thr[1], the last entry for cells above the table), a lower bound
    // because the index is non-decreasing in Usqr; the thresholds between it and U are
    // stepped over (bounded).  Usqr >= 0, so its bit pattern orders like its value.
    __device__ __forceinline__ int bin_of(float U, const HistParams& p, const float* thr,
                                          const uint16_t* start) {
      if (U != U) {
        return p.nan_index;
      }
      int ci = static_cast<int>(__float_as_uint(U) >> p.cell_shift) - p.cell_base + 1;
      ci     = max(0, min(ci, p.ncells));
      int       g   = start[ci];
      const int nm1 = p.nbins - 1;
      for (int it = 0; it < p.nbins && g < nm1 && thr[g + 1] <= U; ++it) {
        ++g;
      }
      return g;
    }

    // float(1.0 / sqrt(1.0 + U)) without FP64: one Newton step in double-float.
    __device__ __forceinline__ float inv_sqrt_one_plus(float U) {
      if (!(U < 3.0e38f)) {
        return U == U ? 0.0f : U; // 1/sqrt(1 + inf) = 0; NaN stays NaN
      }
      const ff    s  = two_sum(1.0f, U);
      const float r0 = rsqrtf(s.hi);
      // e = 1 - s r0^2 in double-float, r = r0 + r0 e / 2
      const ff r2 = two_prod(r0, r0);
      const ff sr = ff_mul(s, r2);
      const float e = __fadd_rn(__fsub_rn(1.0f, sr.hi), -sr.lo);
      return __fmaf_rn(__fmul_rn(0.5f, r0), e, r0);
    }

    __global__ void __launch_bounds__(kHistThreads)
      histogram_kernel(const __grid_constant__ HistParams p) {
      extern __shared__ __align__(16) unsigned char smem[];
      const int nb      = p.nbins;
      float*    thr     = reinterpret_cast<float*>(smem);
      unsigned* cnt     = reinterpret_cast<unsigned*>(thr + nb);
      constexpr int kC = kSumCopies;
      float*    sum32   = reinterpret_cast<float*>(cnt + nb); // [kC][nb]
      double*   sum64   = reinterpret_cast<double*>(smem + (((2 + kC) * sizeof(float) * nb + 15) & ~size_t(15)));
      uint16_t* start   = reinterpret_cast<uint16_t*>(sum64 + nb);
      for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        thr[i]   = p.thr[i];
        cnt[i]   = 0u;
        sum64[i] = 0.0;
      }
      for (int i = threadIdx.x; i < kC * nb; i += blockDim.x) {
        sum32[i] = 0.0f;
      }
      for (int i = threadIdx.x; i <= p.ncells; i += blockDim.x) {
        start[i] = p.start[i];
      }
      __syncthreads();
      float* sum_l = sum32 + (threadIdx.x & (kC - 1)) * nb;

      // contiguous range of particles per block, in rounds of kFlushParticles
      const int64_t G       = gridDim.x;
      const int64_t per     = ((p.n + G - 1) / G + 3) & ~int64_t(3);
      const int64_t begin   = min(p.n, per * blockIdx.x);
      const int64_t end     = min(p.n, begin + per);
      const bool    vec_ok  = ((reinterpret_cast<uintptr_t>(p.ux) | reinterpret_cast<uintptr_t>(p.uy) |
                            reinterpret_cast<uintptr_t>(p.uz)) & 15) == 0;

      for (int64_t r0 = begin; r0 < end; r0 += kFlushParticles) {
        const int64_t r1 = min(end, r0 + kFlushParticles);
        auto          one = [&](float x, float y, float z) {
          const float U = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
          const int   k = bin_of(U, p, thr, start);
          atomicAdd(&cnt[k], 1u);
          if (p.log_spaced) {
            // 1/|u|: rsqrt and one Newton step (within an ulp; the reference rounds this
            // value through double, so the sums are compared with a tolerance anyway)
            float v;
            if (!p.fourvel) {
              v = inv_sqrt_one_plus(U);
            } else if (U > 0.0f && U < 3.0e38f) {
              const float r = rsqrtf(U);
              v             = __fmul_rn(r, __fmaf_rn(__fmul_rn(-0.5f * U, r), r, 1.5f));
            } else {
              v = __frcp_rn(sqrtf(U)); // 0 -> inf, inf -> 0, NaN -> NaN
            }
            atomicAdd(&sum_l[k], v);
          }
        };
        if (vec_ok) {
          // 4 particles per thread with 128-bit loads (begin and per are multiples of 4)
          const int64_t nv = (r1 - r0) / 4;
          for (int64_t v = threadIdx.x; v < nv; v += blockDim.x) {
            const int64_t i  = r0 + 4 * v;
            const float4  X  = __ldcs(reinterpret_cast<const float4*>(p.ux + i));
            const float4  Y  = __ldcs(reinterpret_cast<const float4*>(p.uy + i));
            const float4  Z  = __ldcs(reinterpret_cast<const float4*>(p.uz + i));
            one(X.x, Y.x, Z.x);
            one(X.y, Y.y, Z.y);
            one(X.z, Y.z, Z.z);
            one(X.w, Y.w, Z.w);
          }
          for (int64_t i = r0 + 4 * nv + threadIdx.x; i < r1; i += blockDim.x) {
            one(p.ux[i], p.uy[i], p.uz[i]);
          }
        } else {
          for (int64_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            one(p.ux[i], p.uy[i], p.uz[i]);
          }
        }
        if (p.log_spaced) {
          __syncthreads();
          for (int i = threadIdx.x; i < nb; i += blockDim.x) {
            double t = sum64[i];
            for (int c = 0; c < kC; ++c) {
              t += static_cast<double>(sum32[c * nb + i]);
              sum32[c * nb + i] = 0.0f;
            }
            sum64[i] = t;
          }
        }
        __syncthreads();
      }
      for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        p.part_counts[static_cast<int64_t>(blockIdx.x) * nb + i] = cnt[i];
        p.part_sums[static_cast<int64_t>(blockIdx.x) * nb + i]   = sum64[i];
      }
    }

    // Block (32 bins x 32 row groups): row group y sums block partials y, y + 32, ...
    // then the groups are combined in order (deterministic).
    constexpr int kHistReduceRows = 32;

    __global__ void __launch_bounds__(32 * kHistReduceRows)
      histogram_reduce_kernel(const unsigned long long* __restrict__ pc, const double* __restrict__ ps,
                              int grid, int nbins, int log_spaced, float* __restrict__ hist,
                              unsigned long long* __restrict__ counts) {
      __shared__ unsigned long long c_part[kHistReduceRows][33];
      __shared__ double             s_part[kHistReduceRows][33];
      const int k  = blockIdx.x * 32 + threadIdx.x;
      const int ty = threadIdx.y;
      unsigned long long c = 0;
      double             s = 0.0;
      if (k < nbins) {
        // unrolled so that several rows' loads are in flight (the adds stay in row order)
#pragma unroll 8
        for (int b = ty; b < grid; b += kHistReduceRows) {
          c += pc[static_cast<int64_t>(b) * nbins + k];
          s += ps[static_cast<int64_t>(b) * nbins + k];
        }
      }
      c_part[ty][threadIdx.x] = c;
      s_part[ty][threadIdx.x] = s;
      __syncthreads();
      if (ty != 0 || k >= nbins) {
        return;
      }
      for (int y = 1; y < kHistReduceRows; ++y) {
        c += c_part[y][threadIdx.x];
        s += s_part[y][threadIdx.x];
      }
      hist[k] = log_spaced ? __double2float_rn(s) : static_cast<float>(c);
      if (counts) {
        counts[k] = c;
      }
    }

  } // namespace

  // Thresholds thr[k] (k = 1..n-1): the smallest non-negative float Usqr whose
  // reference index is >= k (+inf if none); thr[0] = 0.  Exposed for tests.
  void energy_thresholds(const float* bins, int n, bool fourvel, std::vector<float>& thr,
                         int& nan_index, float& emin, float& emax) {
    emin = std::numeric_limits<float>::max();
    emax = std::numeric_limits<float>::lowest();
    for (int i = 0; i < n; ++i) {
      emin = std::min(emin, bins[i]);
      emax = std::max(emax, bins[i]);
    }
    thr.assign(n, 0.0f);
    const uint32_t inf_bits = 0x7f800000u;
    for (int k = 1; k < n; ++k) {
      // smallest bit pattern b in [0, inf] with index(b) >= k
      uint32_t lo = 0, hi = inf_bits;
      if (ref_energy_index(bits_to_float(hi), fourvel, emin, emax, n) < static_cast<std::size_t>(k)) {
        thr[k] = std::numeric_limits<float>::infinity();
        continue;
      }
      while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (ref_energy_index(bits_to_float(mid), fourvel, emin, emax, n) >= static_cast<std::size_t>(k)) {
          hi = mid;
        } else {
          lo = mid + 1;
        }
      }
      thr[k] = bits_to_float(lo);
    }
    nan_index = static_cast<int>(
      ref_energy_index(std::numeric_limits<float>::quiet_NaN(), fourvel, emin, emax, n));
  }

  namespace {

    // Thresholds of recently used bin sets (the host binary search costs far more
    // than the histogram kernel for small particle counts), with one device copy per
    // GPU that used them, so a call copies nothing to the device and need not wait
    // for a host buffer; keyed on the bin values and the energy definition, at most
    // kThrCacheEntries kept.
    struct ThrEntry {
      std::vector<float>                  bins, thr;
      bool                                fourvel   = true;
      int                                 nan_index = 0;
      float                               emin = 0, emax = 0;
      std::vector<uint16_t>               start; // cell table (see bin_of)
      int                                 cell_shift = 0, cell_base = 0, ncells = 0;
      std::vector<std::pair<int, float*>> dev; // (device, thresholds then cell table on that device)
    };

    uint32_t float_bits(float f) {
      uint32_t b;
      std::memcpy(&b, &f, 4);
      return b;
    }

    // The cell table over [thr[1], the largest finite threshold]: the smallest shift
    // that keeps at most kMaxCells cells; start[0] = 0 (cells below thr[1]) and
    // start[i] = the number of thresholds thr[1..n-1] <= the smallest float of cell
    // cell_base + i - 1, i.e. that float's bin.  No finite thr[1]: no cells, every
    // particle starts from bin 0.
    void make_cells(ThrEntry& e) {
      const int n = static_cast<int>(e.thr.size());
      e.start.assign(1, 0);
      e.cell_shift = 0;
      e.cell_base  = 0;
      e.ncells     = 0;
      if (n < 2 || !std::isfinite(e.thr[1])) {
        return;
      }
      const uint32_t lo = float_bits(e.thr[1]);
      uint32_t       hi = lo;
      for (int k = 1; k < n; ++k) {
        if (std::isfinite(e.thr[k])) {
          hi = float_bits(e.thr[k]);
        }
      }
      int sh = 0;
      while (sh < 31 && (hi >> sh) - (lo >> sh) + 1 > static_cast<uint32_t>(kMaxCells)) {
        ++sh;
      }
      e.cell_shift = sh;
      e.cell_base  = static_cast<int>(lo >> sh);
      e.ncells     = static_cast<int>((hi >> sh) - (lo >> sh) + 1);
      e.start.resize(static_cast<std::size_t>(e.ncells) + 1);
      int k = 1; // thr[1..k-1] <= the current cell's smallest float
      for (int i = 1; i <= e.ncells; ++i) {
        const float low = bits_to_float(static_cast<uint32_t>(e.cell_base + i - 1) << sh);
        while (k < n && e.thr[k] <= low) {
          ++k;
        }
        e.start[i] = static_cast<uint16_t>(k - 1);
      }
    }

    constexpr std::size_t kThrCacheEntries = 16;

    std::mutex& thr_mutex() {
      static std::mutex m;
      return m;
    }

    std::vector<ThrEntry>& thr_cache() { // most recent last
      static std::vector<ThrEntry> c;
      return c;
    }

    // Frees the device copies of an entry; a kernel of any stream may still read them,
    // so each device is synchronised first (entries are evicted rarely).
    void free_entry(ThrEntry& e) {
      int cur = 0;
      cudaGetDevice(&cur);
      for (auto& d : e.dev) {
        cudaSetDevice(d.first);
        cudaDeviceSynchronize();
        cudaFree(d.second);
      }
      cudaSetDevice(cur);
      e.dev.clear();
    }

  } // namespace

  // What the histogram kernel needs of a bin set, on the current device.
  struct DeviceBins {
    const float*    thr   = nullptr;
    const uint16_t* start = nullptr;
    int             nan_index = 0, cell_shift = 0, cell_base = 0, ncells = 0;
  };

  // Thresholds and cell table of a bin set on the current device.
  int device_thresholds(const float* bins, int n, bool fourvel, DeviceBins& out) {
    int device = 0;
    RG_CUDA_TRY(cudaGetDevice(&device));
    std::lock_guard<std::mutex> lock(thr_mutex());
    auto&                       cache = thr_cache();
    auto                        it    = cache.begin();
    for (; it != cache.end(); ++it) {
      if (it->fourvel == fourvel && static_cast<int>(it->bins.size()) == n &&
          std::memcmp(it->bins.data(), bins, sizeof(float) * n) == 0) {
        break;
      }
    }
    if (it == cache.end()) {
      ThrEntry e;
      energy_thresholds(bins, n, fourvel, e.thr, e.nan_index, e.emin, e.emax);
      make_cells(e);
      e.bins.assign(bins, bins + n);
      e.fourvel = fourvel;
      if (cache.size() >= kThrCacheEntries) {
        free_entry(cache.front());
        cache.erase(cache.begin());
      }
      cache.push_back(std::move(e));
      it = cache.end() - 1;
    } else {
      std::rotate(it, it + 1, cache.end());
      it = cache.end() - 1;
    }
    ThrEntry& e = *it;
    float*    p = nullptr;
    for (auto& d : e.dev) {
      if (d.first == device) {
        p = d.second;
      }
    }
    if (!p) {
      RG_CUDA_TRY(cudaMalloc(&p, sizeof(float) * n + sizeof(uint16_t) * e.start.size()));
      cudaError_t err = cudaMemcpy(p, e.thr.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
      if (err == cudaSuccess) {
        err = cudaMemcpy(p + n, e.start.data(), sizeof(uint16_t) * e.start.size(), cudaMemcpyHostToDevice);
      }
      if (err != cudaSuccess) {
        cudaFree(p);
        return cuda_error(err, "threshold copy");
      }
      e.dev.emplace_back(device, p);
    }
    out.thr        = p;
    out.start      = reinterpret_cast<const uint16_t*>(p + n);
    out.nan_index  = e.nan_index;
    out.cell_shift = e.cell_shift;
    out.cell_base  = e.cell_base;
    out.ncells     = e.ncells;
    return RG_OK;
  }

  void free_threshold_cache() {
    std::lock_guard<std::mutex> lock(thr_mutex());
    for (auto& e : thr_cache()) {
      free_entry(e);
    }
    thr_cache().clear();
  }

} // namespace rg

extern "C" {

int rg_energy_thresholds(const float* bins, int32_t nbins, int32_t fourvel, float* thr,
                         int32_t* nan_index) {
  if (nbins < 1 || !bins || !thr) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_energy_thresholds: bad arguments");
  }
  std::vector<float> t;
  int                ni = 0;
  float              emin, emax;
  rg::energy_thresholds(bins, nbins, fourvel != 0, t, ni, emin, emax);
  std::copy(t.begin(), t.end(), thr);
  if (nan_index) {
    *nan_index = ni;
  }
  return RG_OK;
}

int rg_energy_distribution(const float* ux, const float* uy, const float* uz, int64_t n,
                           const float* bins, int32_t nbins, int32_t log_spaced, int32_t fourvel,
                           float* hist, uint64_t* counts, void* stream) {
  rg::NvtxRange nvtx_range("ComputeEnergyDistribution");
  rg::clear_error();
  if (nbins < 1 || !bins || !hist || n < 0 || (n > 0 && (!ux || !uy || !uz))) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_energy_distribution: bad arguments");
  }
  if (nbins > rg::kHistMaxBins) {
    return rg::set_error(RG_ERR_UNSUPPORTED, "energyDistribution supports at most 4096 bins");
  }
  auto           s = static_cast<cudaStream_t>(stream);
  rg::DeviceBins db;
  RG_TRY(rg::device_thresholds(bins, nbins, fourvel != 0, db));

  rg::DeviceContext* ctx = nullptr;
  RG_TRY(rg::context(&ctx));
  const size_t smem = (((2 + rg::kSumCopies) * sizeof(float) * nbins + 15) & ~size_t(15)) +
                      sizeof(double) * nbins + sizeof(uint16_t) * (db.ncells + 1);
  if (smem > 48 * 1024) {
    RG_CUDA_TRY(cudaFuncSetAttribute(rg::histogram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
  }
  int per_sm = 0;
  RG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rg::histogram_kernel,
                                                            rg::kHistThreads, smem));
  per_sm = std::max(1, std::min(per_sm, 8));
  const int64_t want = std::max<int64_t>(1, (n + 4095) / 4096);
  const int     G    = static_cast<int>(std::min<int64_t>(want, static_cast<int64_t>(ctx->sms) * per_sm));

  // one stream-ordered allocation for the per-block partials
  const size_t   off_ps = sizeof(unsigned long long) * static_cast<size_t>(G) * nbins;
  const size_t   bytes  = off_ps + sizeof(double) * static_cast<size_t>(G) * nbins;
  unsigned char* buf    = nullptr;
  RG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&buf), bytes, s));

  rg::HistParams p {};
  p.ux         = ux;
  p.uy         = uy;
  p.uz         = uz;
  p.n          = n;
  p.nbins      = nbins;
  p.fourvel    = fourvel ? 1 : 0;
  p.log_spaced = log_spaced ? 1 : 0;
  p.thr        = db.thr;
  p.nan_index  = db.nan_index;
  p.start      = db.start;
  p.cell_shift = db.cell_shift;
  p.cell_base  = db.cell_base;
  p.ncells     = db.ncells;
  p.part_counts = reinterpret_cast<unsigned long long*>(buf);
  p.part_sums   = reinterpret_cast<double*>(buf + off_ps);
  rg::histogram_kernel<<<G, rg::kHistThreads, smem, s>>>(p);
  RG_CUDA_TRY(cudaGetLastError());
  rg::histogram_reduce_kernel<<<(nbins + 31) / 32, dim3(32, rg::kHistReduceRows), 0, s>>>(
    p.part_counts, p.part_sums, G, nbins, p.log_spaced, hist,
    reinterpret_cast<unsigned long long*>(counts));
  RG_CUDA_TRY(cudaGetLastError());
  RG_CUDA_TRY(cudaFreeAsync(buf, s));
  return RG_OK;
}

} // extern "C"

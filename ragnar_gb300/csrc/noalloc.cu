// Allocation-free particle spectrum: rg_synchrotron_spectrum_noalloc.
//
// Some callers cannot allocate device memory once they are running: codes that
// hand a fixed device-memory budget out at start-up (a simulation that reserves
// the whole GPU for its fields and particles, or a plugin loaded into such a
// process) and callers whose own rules forbid allocation after initialisation.
// This entry point computes the same spectrum as rg_synchrotron_spectrum with
// the same fused and reduction kernels, but takes every byte of scratch -- the
// per-block FP64 partial sums, the photon bins' fixed-point coordinates, the
// status word and the reference F table -- from one file-scope device array of
// fixed size, so it calls no cudaMalloc, cudaFree or allocating library routine.
//
// Limits and sharing:
//  * at most kNoAllocMaxBins (512) photon bins, reference table only; the
//    array is kNoAllocBytes (about 1.4 MB) and every GPU that loads the
//    library holds it until the process exits;
//  * the array and the kernels this entry point launches come into existence
//    on a device when their code is loaded there, which CUDA's lazy module
//    loading does on first use; rg_init(device) does it up front: it looks up
//    the array's device address with cudaGetSymbolAddress, loads the kernels and
//    builds the F table into the array (synchronising the device's default
//    stream).  Call rg_init for every device before handing the device memory
//    budget out; without it, the first call on a device does this set-up
//    itself, needs device memory for the code and the array at that moment, and
//    should come before any stream capture;
//  * every call shares the array and it keeps the last call's contents; each
//    call rewrites what it reads and clears the status word itself, but calls
//    whose GPU work overlaps (on different streams or threads) race on it;
//  * a failure found on the device (a bounded wait that gave up) shows up as
//    NaN outputs; there is no separate status query.
#include "spectrum_common.cuh"

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>
#include <mutex>
#include <vector>

namespace rg {

  int launch_fused_reference(int K, const FusedParams& fp, int grid, cudaStream_t s);
  int preload_reference_kernels();
  int launch_reduce_single(const double* partials, int grid, int64_t n, int nbins, const float* ebins,
                           const uint8_t* valid, const unsigned* status, float* out, cudaStream_t s);
  int build_reference_table_into(int n, float xmin, float xmax, float* d_x, float* d_y, float2* d_coef,
                                 float* d_grids, double& ln_xmin, double& dln, cudaStream_t s);

  namespace {

    constexpr int    kNoAllocMaxBins = kSliceBins; // one slice of the fused kernel
    constexpr int    kNoAllocMaxGrid = 320;        // blocks (2 per SM up to 160 SMs)
    constexpr int    kTableNodes     = 200;        // TabulateFfunc() defaults (synchrotron.hpp:26-29)
    constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }

    // Layout of the scratch array.
    constexpr size_t kOffStatus   = 0;
    constexpr size_t kOffP        = 256;
    constexpr size_t kOffRange    = align256(kOffP + sizeof(int32_t) * kSliceBins);
    constexpr size_t kOffEbins    = align256(kOffRange + 2 * sizeof(int64_t));
    constexpr size_t kOffValid    = align256(kOffEbins + sizeof(float) * kNoAllocMaxBins);
    constexpr size_t kOffTabX     = align256(kOffValid + kNoAllocMaxBins);
    constexpr size_t kOffTabY     = align256(kOffTabX + sizeof(float) * kTableNodes);
    constexpr size_t kOffCoef     = align256(kOffTabY + sizeof(float) * kTableNodes);
    constexpr size_t kOffGrids    = align256(kOffCoef + sizeof(float2) * kRefEntries);
    constexpr size_t kOffPartials = align256(kOffGrids + sizeof(float) * kTableNodes * 100);
    constexpr size_t kNoAllocBytes =
      kOffPartials + sizeof(double) * static_cast<size_t>(kNoAllocMaxGrid) * kSliceBins;

  } // namespace

  static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

  namespace {

    struct NoAllocDevice {
      unsigned char* base = nullptr; // device address of g_noalloc_scratch
      double         ln_xmin = 0, dln = 0;
      int            sms     = 0;
    };

    std::mutex& noalloc_mutex() {
      static std::mutex m;
      return m;
    }

    std::map<int, NoAllocDevice>& noalloc_devices() {
      static std::map<int, NoAllocDevice> m;
      return m;
    }

    // Once per device, with that device current: the array's device address (looking
    // it up loads this file's module, which holds the array), the kernels, the F table.
    int noalloc_setup(int dev, NoAllocDevice& d) {
      void* ptr = nullptr;
      RG_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
      d.base = static_cast<unsigned char*>(ptr);
      RG_CUDA_TRY(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
      RG_TRY(preload_reference_kernels());
      RG_TRY(build_reference_table_into(kTableNodes, 1e-6f, 100.0f, reinterpret_cast<float*>(d.base + kOffTabX),
                                        reinterpret_cast<float*>(d.base + kOffTabY),
                                        reinterpret_cast<float2*>(d.base + kOffCoef),
                                        reinterpret_cast<float*>(d.base + kOffGrids), d.ln_xmin, d.dln, nullptr));
      return RG_OK;
    }

    // The device's set-up record, made on first use (under the mutex).
    int noalloc_device(int dev, NoAllocDevice& out) {
      std::lock_guard<std::mutex> lock(noalloc_mutex());
      auto                        it = noalloc_devices().find(dev);
      if (it == noalloc_devices().end()) {
        NoAllocDevice fresh;
        RG_TRY(noalloc_setup(dev, fresh));
        it = noalloc_devices().emplace(dev, fresh).first;
      }
      out = it->second;
      return RG_OK;
    }

  } // namespace

  // Called by rg_init with `dev` current, so that the array and the kernels are resident
  // before a caller hands its device memory out.
  int noalloc_prepare(int dev) {
    NoAllocDevice d;
    return noalloc_device(dev, d);
  }

} // namespace rg

extern "C" {

int rg_synchrotron_spectrum_noalloc(const rg_particles* p, const float* bins, int32_t nbins, float B0,
                                    float g_syn, float e_syn_at_g_syn, float* out, void* stream) {
  rg::NvtxRange nvtx_range("SynchrotronSpectrum");
  using namespace rg;
  clear_error();
  if (!p || p->n < 0 || (p->n > 0 && (!p->u[0] || !p->u[1] || !p->u[2]))) {
    return set_error(RG_ERR_ARGUMENT, "particles need U1..U3 device arrays and n >= 0");
  }
  if (nbins < 0 || nbins > kNoAllocMaxBins || (nbins > 0 && (!bins || !out))) {
    return set_error(RG_ERR_ARGUMENT, "rg_synchrotron_spectrum_noalloc: needs 0 to " +
                                        std::to_string(kNoAllocMaxBins) + " photon bins (got " +
                                        std::to_string(nbins) + ") and an output array");
  }
  if (B0 == 0.0f) {
    return set_error(RG_ERR_ARGUMENT, "B0 must be non-zero");
  }
  if (nbins == 0) { // as rg_synchrotron_spectrum: nothing to compute
    return RG_OK;
  }
  int dev = 0;
  RG_CUDA_TRY(cudaGetDevice(&dev));
  NoAllocDevice d;
  RG_TRY(noalloc_device(dev, d));
  auto s = static_cast<cudaStream_t>(stream);
  // the caller may change or free `bins` once this returns, even if it is pinned
  // memory (whose copy would otherwise still be in flight): copy from a host vector
  const std::vector<float> hB(bins, bins + nbins);

  // e_peak = K0 gamma sqrt(W), K0 = eps / (g^2 B0): K0 <= 0 means no emission
  const double K0 = static_cast<double>(e_syn_at_g_syn) /
                    (static_cast<double>(g_syn) * g_syn * static_cast<double>(B0));
  if (!(K0 > 0.0) || !std::isfinite(K0) || p->n == 0) {
    RG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * nbins, s));
    return RG_OK;
  }

  // photon bins in fixed-point table coordinates (reference table, kFrac bits)
  const double scale = std::ldexp(1.0, kFrac) / d.dln;
  const double S     = std::ldexp(1.0, kFrac) / (2.0 * d.dln);
  const int64_t L    = static_cast<int64_t>(kTableNodes - 1) << kFrac;
  std::vector<int64_t> Ps(kSliceBins, 0);
  std::vector<int32_t> hP(kSliceBins, 0);
  std::vector<uint8_t> hV(kNoAllocMaxBins, 0);
  int64_t              pmin = std::numeric_limits<int64_t>::max(), pmax = std::numeric_limits<int64_t>::min();
  for (int j = 0; j < nbins; ++j) {
    const double e = hB[j];
    if (!(e > 0.0) || !std::isfinite(e)) {
      continue;
    }
    const double t = (std::log(e) - d.ln_xmin - std::log(K0)) * scale;
    if (!(std::fabs(t) < 1e18)) {
      return set_error(RG_ERR_UNSUPPORTED, "photon bin energy out of the supported range");
    }
    Ps[j] = std::llround(t);
    hV[j] = 1;
    pmin  = std::min(pmin, Ps[j]);
    pmax  = std::max(pmax, Ps[j]);
  }
  if (pmin > pmax) {
    pmin = pmax = 0;
  }
  if (static_cast<double>(pmax - pmin) + static_cast<double>(L) > 4294967296.0) {
    return set_error(RG_ERR_UNSUPPORTED, "photon bins span more than the 32-bit table window (about 33 decades)");
  }
  for (int j = 0; j < kSliceBins; ++j) {
    const int64_t v = (j < nbins && hV[j]) ? Ps[j] : pmin;
    hP[j]           = static_cast<int32_t>(static_cast<uint32_t>(v & 0xffffffffLL));
  }
  const int64_t hR[2] = { pmin, pmax };
  unsigned char* b    = d.base;
  // pageable sources: each copy has left the host buffer when the call returns
  RG_CUDA_TRY(cudaMemsetAsync(b + kOffStatus, 0, sizeof(unsigned), s));
  RG_CUDA_TRY(cudaMemcpyAsync(b + kOffP, hP.data(), sizeof(int32_t) * kSliceBins, cudaMemcpyHostToDevice, s));
  RG_CUDA_TRY(cudaMemcpyAsync(b + kOffRange, hR, sizeof(hR), cudaMemcpyHostToDevice, s));
  RG_CUDA_TRY(cudaMemcpyAsync(b + kOffEbins, hB.data(), sizeof(float) * nbins, cudaMemcpyHostToDevice, s));
  RG_CUDA_TRY(cudaMemcpyAsync(b + kOffValid, hV.data(), nbins, cudaMemcpyHostToDevice, s));

  FusedParams fp {};
  const float* comp[kComps] = { p->u[0], p->u[1], p->u[2], p->e[0], p->e[1], p->e[2],
                                p->b[0], p->b[1], p->b[2], p->w };
  int          nslots       = 0;
  bool         aligned      = true;
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
  fp.source      = kSrcParticles;
  fp.has_e       = (comp[3] || comp[4] || comp[5]) ? 1 : 0;
  fp.has_w       = comp[9] ? 1 : 0;
  fp.seg_off     = nullptr;
  fp.item_prefix = nullptr;
  fp.n_single    = p->n;
  fp.nseg        = 1;
  fp.P           = reinterpret_cast<const int32_t*>(b + kOffP);
  fp.Prange      = reinterpret_cast<const int64_t*>(b + kOffRange);
  fp.L           = L;
  fp.Sh          = static_cast<float>(S);
  fp.Sl          = static_cast<float>(S - static_cast<double>(fp.Sh));
  fp.Cfx         = std::llround(S * M_LN2 * 65536.0);
  fp.amp         = static_cast<float>(1.0 / static_cast<double>(B0));
  fp.table       = reinterpret_cast<const float2*>(b + kOffCoef);
  fp.htable      = nullptr;
  fp.hseg        = 0;
  fp.frac        = kFrac;
  fp.partials    = reinterpret_cast<double*>(b + kOffPartials);
  fp.nslices     = 1;
  fp.status      = reinterpret_cast<unsigned*>(b + kOffStatus);
  const int64_t items = (p->n + kChunk - 1) / kChunk;
  const int     grid  = static_cast<int>(
    std::max<int64_t>(1, std::min<int64_t>(items, std::min(kNoAllocMaxGrid, d.sms * kBlocksPerSM))));
  const int K = std::max(1, (nbins + 31) / 32);
  RG_TRY(launch_fused_reference(K, fp, grid, s));
  RG_TRY(launch_reduce_single(fp.partials, grid, p->n, nbins, reinterpret_cast<const float*>(b + kOffEbins),
                              reinterpret_cast<const uint8_t*>(b + kOffValid), fp.status, out, s));
  return RG_OK;
}

} // extern "C"

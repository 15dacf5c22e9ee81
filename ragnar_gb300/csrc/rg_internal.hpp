// Internal host-side declarations of the ragnar_gb300 library.
#pragma once

#include "ragnar_gb300.h"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

namespace rg {

  // ---- errors ---------------------------------------------------------------
  int  set_error(int status, const std::string& msg);
  int  cuda_error(cudaError_t e, const char* what);
  void clear_error();

#define RG_CUDA_TRY(expr)                                                               \
  do {                                                                                  \
    cudaError_t rg_e_ = (expr);                                                         \
    if (rg_e_ != cudaSuccess) {                                                         \
      return ::rg::cuda_error(rg_e_, #expr);                                            \
    }                                                                                   \
  } while (0)

#define RG_TRY(expr)                                                                    \
  do {                                                                                  \
    int rg_s_ = (expr);                                                                 \
    if (rg_s_ != RG_OK) {                                                               \
      return rg_s_;                                                                     \
    }                                                                                   \
  } while (0)

  // Raises a kernel's dynamic shared-memory limit to `bytes` once per device (the
  // attribute is per device; `done` keeps one bit per device ordinal below 64).
  template <typename Kernel>
  cudaError_t ensure_max_dynamic_smem(Kernel* kernel, int bytes, std::atomic<uint64_t>& done) {
    int               dev = 0;
    const cudaError_t e0  = cudaGetDevice(&dev);
    if (e0 != cudaSuccess) {
      return e0;
    }
    const uint64_t bit = dev < 64 ? (uint64_t(1) << dev) : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit)) {
      return cudaSuccess;
    }
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && bit) {
      done.fetch_or(bit, std::memory_order_release);
    }
    return e;
  }

  // NVTX range around one C-ABI call, named after the Kokkos label the reference gives the
  // same work (synchrotron.cpp:92,131 "SynchrotronSpectrum", particles.cpp:225
  // "ComputeEnergyDistribution", ic.cpp:38 "ICSpectrum"), so a profiler shows the stages
  // under the reference's names.  NVTX v3 is header-only: without an attached tool each
  // push and pop is a test of a null function pointer.
  struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&)            = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
  };

  // Scratch device buffer freed when it leaves scope (also on an early error return).
  template <typename T>
  struct ScratchBuffer {
    T* p = nullptr;
    ScratchBuffer() = default;
    ScratchBuffer(const ScratchBuffer&) = delete;
    ScratchBuffer& operator=(const ScratchBuffer&) = delete;
    ~ScratchBuffer() { cudaFree(p); }
  };

  // Particle streams of a spectrum input: u0 u1 u2 e0 e1 e2 b0 b1 b2 w.
  constexpr int kComps = 10;

  // ---- F tables ---------------------------------------------------------------

  // Fixed-point table coordinate: T = t * 2^kFrac with t the (fractional) node
  // index.  The reference table's segments occupy entries [0, n-2] of a
  // 1024-entry table whose other entries are zero, so any 32-bit T maps to a
  // valid entry (T >> kFrac < 1024).
  constexpr int      kFrac        = 22;
  constexpr int      kRefEntries  = 1024;
  // c1 is stored pre-multiplied by 2^127: a denormal built from the fraction
  // bits (bits * 2^-149) times c1 * 2^127 equals frac * c1.
  constexpr double   kSlopeScale  = 1.7014118346046923e38; // 2^127

  // Smooth (differentiable) table: exact F on a log grid, cubic Hermite segments.
  constexpr int    kSmoothSegments = 2048;
  // Upper bound on the segments of any smooth table (the device-wide one above or a
  // plan's own table aligned to its bins); sizes the kernels' shared-memory limit.
  constexpr int    kSmoothMaxSegments = 4096;
  constexpr double kSmoothXmin     = 1e-6;
  constexpr double kSmoothXmax     = 100.0;

  struct RefTable {
    int     n      = 0;       // nodes
    float   xmin   = 0, xmax = 0;
    float*  d_x    = nullptr; // n nodes
    float*  d_y    = nullptr; // n values
    float2* d_coef = nullptr; // kRefEntries (c0, c1 * 2^127) per segment
    double  ln_xmin = 0, dln = 0; // ideal grid: t = (ln x - ln_xmin) / dln
    std::vector<float> h_x, h_y;
  };

  struct SmoothTable {
    float4* d_coef  = nullptr; // nseg (c0, c1, c2, c3) in tau, then one zero entry
    double  ln_xmin = 0, dln = 0;
    int     nseg    = kSmoothSegments;
  };

  // Device staging for host-resident particle streams.  Every host-input call on a
  // device, whatever its plan, streams through the same buffers and copy stream, so
  // consecutive calls form one pipeline: the first copies of a call overlap the last
  // kernels of the previous one, and two plans never compete for the host link.
  struct HostStaging {
    static constexpr int     kBuffers = 2;
    static constexpr int64_t kChunk   = int64_t(1) << 22; // particles per buffer (all components)
    std::mutex   mu;                                       // held while a call enqueues its chunks
    float*       d_stage[kBuffers]  = {};
    cudaEvent_t  copied[kBuffers]   = {};
    cudaEvent_t  consumed[kBuffers] = {};
    cudaStream_t copy_stream        = nullptr;
    uint64_t     issued             = 0; // chunks issued so far; chunk c uses buffer c % kBuffers
    HostStaging() = default;
    HostStaging(const HostStaging&) = delete;
    HostStaging& operator=(const HostStaging&) = delete;
    ~HostStaging(); // waits for its copies and kernels, then releases everything it holds
  };

  struct DeviceContext {
    int         device = -1;
    int         sms    = 0;
    RefTable    ref;
    SmoothTable smooth;
    bool        ref_ready = false, smooth_ready = false;
    std::unique_ptr<HostStaging> staging;
  };

  // Context of the current device (created on first use; builds tables lazily).
  int context(DeviceContext** ctx);
  // The current device's host staging (allocated on first use).
  int host_staging(HostStaging** out);
  int reference_table(const RefTable** t);
  int smooth_table(const SmoothTable** t);

  // Builds the reference table on `n` nodes of Logspace(xmin, xmax) (FP64 on the GPU).
  int build_reference_table(int n, float xmin, float xmax, RefTable& t, cudaStream_t s);
  int build_smooth_table(SmoothTable& t, cudaStream_t s);
  // A smooth table of nseg segments of width dln (in ln x) from ln_xmin.
  int build_smooth_table_geom(SmoothTable& t, double ln_xmin, double dln, int nseg, cudaStream_t s);
  // Makes the allocation-free entry point's scratch array and kernels resident on `dev`
  // (the current device) and builds its F table; noalloc.cu.
  int noalloc_prepare(int dev);
  void free_tables(DeviceContext& c);
  void free_staging(DeviceContext& c);
  // Device copies of the histogram's bin thresholds (histogram.cu).
  void free_threshold_cache();

  // Host grids with the reference's float/double arithmetic.
  float logspace_point(float start, float stop, std::size_t num, std::size_t i);

} // namespace rg

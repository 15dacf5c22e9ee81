// Runtime pieces of the C ABI: errors, device context, memory helpers, grids.
#include "rg_internal.hpp"

#include <cmath>
#include <cstring>
#include <map>
#include <memory>

namespace rg {

  namespace {
    thread_local std::string g_last_error;

    std::mutex&                                  ctx_mutex() {
      static std::mutex m;
      return m;
    }

    // Never destroyed: releasing device resources from a static destructor at process exit
    // would call the CUDA runtime while it unloads (rg_finalize releases them explicitly).
    std::map<int, std::unique_ptr<DeviceContext>>& contexts() {
      static auto* m = new std::map<int, std::unique_ptr<DeviceContext>>();
      return *m;
    }
  } // namespace

  int set_error(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
  }

  int cuda_error(cudaError_t e, const char* what) {
    return set_error(RG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                                    cudaGetErrorString(e) + ")");
  }

  void clear_error() {
    g_last_error.clear();
  }

  int context(DeviceContext** out) {
    int dev = 0;
    RG_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(ctx_mutex());
    auto&                       m = contexts();
    auto                        it = m.find(dev);
    if (it == m.end()) {
      auto c    = std::make_unique<DeviceContext>();
      c->device = dev;
      RG_CUDA_TRY(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev));
      it = m.emplace(dev, std::move(c)).first;
    }
    *out = it->second.get();
    return RG_OK;
  }

  int reference_table(const RefTable** t) {
    DeviceContext* c = nullptr;
    RG_TRY(context(&c));
    std::lock_guard<std::mutex> lock(ctx_mutex());
    if (!c->ref_ready) {
      // TabulateFfunc() defaults (synchrotron.hpp:26-29): 200 nodes on [1e-6, 100].
      RG_TRY(build_reference_table(200, 1e-6f, 100.0f, c->ref, nullptr));
      RG_CUDA_TRY(cudaStreamSynchronize(nullptr));
      c->ref_ready = true;
    }
    *t = &c->ref;
    return RG_OK;
  }

  int smooth_table(const SmoothTable** t) {
    DeviceContext* c = nullptr;
    RG_TRY(context(&c));
    std::lock_guard<std::mutex> lock(ctx_mutex());
    if (!c->smooth_ready) {
      RG_TRY(build_smooth_table(c->smooth, nullptr));
      RG_CUDA_TRY(cudaStreamSynchronize(nullptr));
      c->smooth_ready = true;
    }
    *t = &c->smooth;
    return RG_OK;
  }

  int host_staging(HostStaging** out) {
    DeviceContext* c = nullptr;
    RG_TRY(context(&c));
    std::lock_guard<std::mutex> lock(ctx_mutex());
    if (!c->staging) {
      // on a failed allocation st's destructor releases what was made
      auto st = std::make_unique<HostStaging>();
      for (int b = 0; b < HostStaging::kBuffers; ++b) {
        RG_CUDA_TRY(cudaMalloc(&st->d_stage[b], sizeof(float) * kComps * HostStaging::kChunk));
        RG_CUDA_TRY(cudaEventCreateWithFlags(&st->copied[b], cudaEventDisableTiming));
        RG_CUDA_TRY(cudaEventCreateWithFlags(&st->consumed[b], cudaEventDisableTiming));
      }
      RG_CUDA_TRY(cudaStreamCreateWithFlags(&st->copy_stream, cudaStreamNonBlocking));
      c->staging = std::move(st);
    }
    *out = c->staging.get();
    return RG_OK;
  }

  HostStaging::~HostStaging() {
    if (copy_stream) {
      cudaStreamSynchronize(copy_stream);
      cudaStreamDestroy(copy_stream);
    }
    for (int b = 0; b < kBuffers; ++b) {
      if (consumed[b]) {
        cudaEventSynchronize(consumed[b]);
        cudaEventDestroy(consumed[b]);
      }
      if (copied[b]) {
        cudaEventDestroy(copied[b]);
      }
      cudaFree(d_stage[b]); // null for a buffer never allocated
    }
  }

  void free_staging(DeviceContext& c) {
    c.staging.reset();
  }

  void free_tables(DeviceContext& c) {
    cudaFree(c.ref.d_x);
    cudaFree(c.ref.d_y);
    cudaFree(c.ref.d_coef);
    cudaFree(c.smooth.d_coef);
    c.ref          = RefTable {};
    c.smooth       = SmoothTable {};
    c.ref_ready    = false;
    c.smooth_ready = false;
  }

  // snippets.cpp:48-60: pow(10, log10f(start) + float(i) * log10f(stop/start) / float(num-1)),
  // Kokkos' pow(int, float) promoting to double; the result is stored as float.
  float logspace_point(float start, float stop, std::size_t num, std::size_t i) {
    if (num == 1) {
      return start;
    }
    const float e = std::log10(start) +
                    static_cast<float>(i) * (std::log10(stop / start)) / static_cast<float>(num - 1);
    return static_cast<float>(std::pow(10.0, static_cast<double>(e)));
  }

} // namespace rg

extern "C" {

const char* rg_last_error(void) {
  return rg::g_last_error.c_str();
}

int rg_init(int device) {
  rg::clear_error();
  int count = 0;
  RG_CUDA_TRY(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) {
    return rg::set_error(RG_ERR_ARGUMENT, "rg_init: device " + std::to_string(device) +
                                            " out of range (" + std::to_string(count) +
                                            " devices)");
  }
  RG_CUDA_TRY(cudaSetDevice(device));
  RG_CUDA_TRY(cudaFree(nullptr)); // create the primary context
  const rg::RefTable* t = nullptr;
  RG_TRY(rg::reference_table(&t));
  // the allocation-free entry point's array and kernels, made resident now
  return rg::noalloc_prepare(device);
}

int rg_finalize(void) {
  rg::free_threshold_cache();
  std::lock_guard<std::mutex> lock(rg::ctx_mutex());
  for (auto& kv : rg::contexts()) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(kv.first);
    rg::free_staging(*kv.second);
    rg::free_tables(*kv.second);
    cudaSetDevice(cur);
  }
  rg::contexts().clear();
  return RG_OK;
}

int rg_smooth_table(float* coef, int32_t* nseg, double* ln_xmin, double* dln) {
  const rg::SmoothTable* t = nullptr;
  RG_TRY(rg::smooth_table(&t));
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

int rg_device_sm_count(int* sms) {
  rg::DeviceContext* c = nullptr;
  RG_TRY(rg::context(&c));
  *sms = c->sms;
  return RG_OK;
}

int rg_malloc(void** ptr, size_t bytes) {
  *ptr = nullptr;
  if (bytes == 0) {
    return RG_OK;
  }
  RG_CUDA_TRY(cudaMalloc(ptr, bytes));
  return RG_OK;
}

int rg_free(void* ptr) {
  if (ptr) {
    RG_CUDA_TRY(cudaFree(ptr));
  }
  return RG_OK;
}

int rg_memcpy_htod(void* dst, const void* src, size_t bytes, void* stream) {
  if (bytes) {
    RG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice,
                                static_cast<cudaStream_t>(stream)));
  }
  return RG_OK;
}

int rg_memcpy_dtoh(void* dst, const void* src, size_t bytes, void* stream) {
  if (bytes) {
    RG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost,
                                static_cast<cudaStream_t>(stream)));
  }
  return RG_OK;
}

int rg_memcpy_dtod(void* dst, const void* src, size_t bytes, void* stream) {
  if (bytes) {
    RG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice,
                                static_cast<cudaStream_t>(stream)));
  }
  return RG_OK;
}

int rg_memset(void* dst, int value, size_t bytes, void* stream) {
  if (bytes) {
    RG_CUDA_TRY(cudaMemsetAsync(dst, value, bytes, static_cast<cudaStream_t>(stream)));
  }
  return RG_OK;
}

int rg_stream_synchronize(void* stream) {
  RG_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  return RG_OK;
}

int rg_logspace(float start, float stop, int64_t num, float* out) {
  if (num < 0) {
    return rg::set_error(RG_ERR_ARGUMENT, "Logspace num must be >= 0");
  }
  if (start <= 0.0 or stop <= 0.0) {
    return rg::set_error(RG_ERR_ARGUMENT, "Logspace start and stop must be strictly positive");
  }
  if (start >= stop) {
    return rg::set_error(RG_ERR_ARGUMENT, "Logspace start must be < stop");
  }
  for (int64_t i = 0; i < num; ++i) {
    out[i] = rg::logspace_point(start, stop, static_cast<std::size_t>(num),
                                static_cast<std::size_t>(i));
  }
  return RG_OK;
}

// snippets.cpp:21-37: start + i * (stop - start) / (num - 1) with the size_t
// operands converted to float.
int rg_linspace(float start, float stop, int64_t num, float* out) {
  if (num < 0) {
    return rg::set_error(RG_ERR_ARGUMENT, "Linspace num must be >= 0");
  }
  if (start >= stop) {
    return rg::set_error(RG_ERR_ARGUMENT, "Linspace start must be < stop");
  }
  for (int64_t i = 0; i < num; ++i) {
    out[i] = (num == 1) ? start
                        : start + static_cast<std::size_t>(i) * (stop - start) /
                                    static_cast<std::size_t>(num - 1);
  }
  return RG_OK;
}

} // extern "C"

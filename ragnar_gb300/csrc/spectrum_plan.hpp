// rg_spectrum_plan: the host-side state of a prepared spectrum (photon bins in
// fixed-point table coordinates, scalars, scratch).  Shared by spectrum.cu and adjoint.cu.
#pragma once

#include "rg_internal.hpp"

#include <cuda_runtime.h>

#include <cstdint>
#include <utility>
#include <vector>

struct rg_spectrum_plan {
  int                   device     = 0;
  int                   table_mode = RG_TABLE_REFERENCE;
  int                   source     = 0; // rg::Source
  int                   nbins      = 0;
  int                   nslices    = 0;
  int                   K          = 0;
  bool                  zero       = false; // every contribution is zero (K0 <= 0 ...)
  float                 B0 = 1, g_syn = 1, eps = 1;
  int                   log_spaced = 0; // dist source
  int                   frac       = 0; // fixed-point fraction bits of the table coordinate
  int64_t               L          = 0;
  float                 Sh = 0, Sl = 0;
  int64_t               Cfx        = 0;
  float                 amp        = 1;
  int                   grid       = 0; // blocks per slice of the fused kernel
  std::vector<float>    h_bins;
  int32_t*              d_P         = nullptr;
  int64_t*              d_Prange    = nullptr;
  float*                d_ebins     = nullptr;
  uint8_t*              d_valid     = nullptr;
  unsigned*             d_status    = nullptr;
  double*               d_partials  = nullptr;
  size_t                partial_cap = 0; // doubles
  int64_t*              d_prefix    = nullptr;
  int                   prefix_cap  = 0; // segments
  double*               d_plain_acc = nullptr;
  const rg::RefTable*   ref         = nullptr;
  const rg::SmoothTable* smooth     = nullptr;
  // kernel timing (events bracketing each fused launch)
  bool                                             timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_used, ev_free;
};

namespace rg {

  // Shared plan helpers (spectrum.cu).
  int  plan_reserve(rg_spectrum_plan* pl, int max_seg);
  int  check_particles(const rg_particles* p);
  void particle_comps(const rg_particles* p, const float* out[10]);
  // Fills the launch parameters common to the forward and adjoint kernels;
  // returns the number of staged streams.
  struct FusedParams;
  int fill_params(const rg_spectrum_plan* pl, const float* const comp[10], const int64_t* d_off,
                  const int64_t* d_prefix, int64_t n_single, int nseg, FusedParams& fp);
  int item_prefix(rg_spectrum_plan* pl, const int64_t* d_off, int nseg, int64_t n, cudaStream_t s);

} // namespace rg

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
  // interval-moment path (reference table, particle source; moments.cu)
  int                   algo        = RG_ALGO_AUTO;
  bool                  moments_ok  = false;  // the plan's bins were prepared for it
  std::vector<int32_t>  h_mslice;             // per slice: (valid bins, cells, histogram offset lo, hi)
  int32_t*              d_mslice    = nullptr;
  int64_t*              d_mrange    = nullptr; // per slice: (Pmin, Pmax) in the finer coordinate
  int64_t               mom_L       = 0;       // table segments in the finer coordinate
  int32_t*              d_thr       = nullptr; // per slice: sorted low parts of Pmax - P_b (kSliceBins)
  uint16_t*             d_bucket    = nullptr; // per slice: first threshold of each bucket (kMomBuckets + 1)
  int4*                 d_binfo     = nullptr; // per bin: (sorted position, cell offset, low part, valid)
  double2*              d_mcoef     = nullptr; // per table segment: FP64 (c0, c1 per fraction bit)
  int64_t               hist_per_seg = 0;      // double2 entries of one segment's histograms
  double2*              d_hist      = nullptr;
  size_t                hist_cap    = 0;       // double2 entries
  // smooth table aligned to log-uniform bins (moments_smooth.cu)
  rg::SmoothTable       own_smooth;            // the plan's own table when `aligned`
  bool                  aligned     = false;
  int64_t               sm_pmin = 0, sm_pmax = 0; // smallest / largest bin coordinate, fine units
  int                   sm_cells    = 0;
  double*               d_cells     = nullptr; // nseg x cells x 4 doubles: the forward's folded cell
                                               // moments, or (as float4) the adjoint's cell cubics
  size_t                cells_cap   = 0;       // (segment, cell) entries
  double2*              d_coef64    = nullptr; // per table segment: (c0, c1), (c2, c3), (c1, 2 c2), (3 c3, 0)
  // kernel timing (events bracketing each fused launch)
  bool                                             timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_used, ev_free;
};

namespace rg {

  // Shared plan helpers (spectrum.cu).
  int  create_plan(const float* bins, int32_t nbins, float B0, float g_syn, float e_syn_at_g_syn,
                   int32_t table_mode, int source, rg_spectrum_plan** plan);
  int  plan_reserve(rg_spectrum_plan* pl, int max_seg);
  int  check_particles(const rg_particles* p);
  void particle_comps(const rg_particles* p, const float* out[10]);
  // Fills the launch parameters common to the forward and adjoint kernels;
  // returns the number of staged streams.
  struct FusedParams;
  int fill_params(const rg_spectrum_plan* pl, const float* const comp[10], const int64_t* d_off,
                  const int64_t* d_prefix, int64_t n_single, int nseg, FusedParams& fp);
  int item_prefix(rg_spectrum_plan* pl, const int64_t* d_off, int nseg, int64_t n, cudaStream_t s);

  // Interval-moment path of reference-table particle plans (moments.cu).
  int  moments_prepare(rg_spectrum_plan* pl, const std::vector<uint8_t>& valid, double ln_xmin, double dln,
                       double ln_k0);
  bool moments_selected(const rg_spectrum_plan* pl, int nseg);
  int  moments_begin(rg_spectrum_plan* pl, int nseg, cudaStream_t s);
  int  moments_deposit(rg_spectrum_plan* pl, const float* const comp[10], const int64_t* d_off, int64_t n,
                       int nseg, cudaStream_t s);
  int  moments_finish(rg_spectrum_plan* pl, int nseg, float* out, cudaStream_t s);
  void moments_free(rg_spectrum_plan* pl);
  // The smooth-table variant (moments_smooth.cu).
  int  smooth_align_plan(rg_spectrum_plan* pl, double ln_k0);
  int  smooth_moments_prepare(rg_spectrum_plan* pl, double ln_k0);
  int  smooth_reserve_cells(rg_spectrum_plan* pl, size_t entries);
  // place: optional per-particle placement record (single-segment runs; see rg_spectrum_run_placed)
  int  smooth_moments_deposit(rg_spectrum_plan* pl, const float* const comp[10], const int64_t* d_off, int64_t n,
                              int nseg, cudaStream_t s, uint2* place = nullptr);
  int  smooth_moments_finish(rg_spectrum_plan* pl, int nseg, float* out, cudaStream_t s);
  int  smooth_moments_adjoint(rg_spectrum_plan* pl, const float* const comp[10], const int64_t* d_off, int64_t n,
                              int nseg, const float* grad_out, float* gw, float* const gu[3], cudaStream_t s,
                              const uint2* place = nullptr);

} // namespace rg

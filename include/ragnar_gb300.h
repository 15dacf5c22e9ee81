/*
 * ragnar_gb300 -- C ABI of the GB300 (sm_103a) synchrotron hot path.
 *
 * Plain pointers and sizes only.  "device" pointers are CUDA device memory on
 * the current device; "host" pointers are ordinary host memory.  `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).  Every entry
 * point returns an rg_status; rg_last_error() gives the message of the last
 * failure on the calling thread.  Unless stated otherwise, a call only enqueues
 * work on `stream` and returns without synchronising.
 *
 * Threads: the library's own state (device contexts, tables, the host staging
 * pipeline, caches) is guarded and may be used from several threads.  A plan
 * (rg_spectrum_plan, rg_fromdist_plan) holds scratch that its runs reuse: calls on
 * one plan must be ordered on one stream (or externally synchronised), and two
 * plans are needed for work that overlaps.
 *
 * Each declaration cites the reference interface it replaces (file:line in the
 * reference tree, paths under src/).
 */
#ifndef RAGNAR_GB300_H
#define RAGNAR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rg_status {
  RG_OK              = 0,
  RG_ERR_ARGUMENT    = 1, /* invalid argument; the reference throws std::runtime_error */
  RG_ERR_CUDA        = 2, /* a CUDA runtime/driver call failed */
  RG_ERR_TIMEOUT     = 3, /* a bounded on-device wait gave up; results are invalid */
  RG_ERR_UNSUPPORTED = 4, /* configuration outside what this build supports */
  RG_ERR_RANGE       = 5  /* the reference throws std::range_error / out_of_range */
} rg_status;

/* Table modes for the spectrum plans. */
enum {
  RG_TABLE_REFERENCE = 0, /* the reference's 200-point F table, piecewise linear in log10 x */
  RG_TABLE_SMOOTH    = 1  /* exact F on a fine log grid, C1 cubic Hermite (differentiable) */
};

/* How a particle plan sums its spectrum (rg_spectrum_plan_set_algorithm). */
enum {
  RG_ALGO_AUTO    = 0, /* moments where the plan supports them, else the fused kernels */
  RG_ALGO_DIRECT  = 1, /* the fused kernels: every (particle, bin) pair evaluated in FP32 */
  RG_ALGO_MOMENTS = 2  /* FP64 moments per table cell (and bin interval) */
};

/* --------------------------------------------------------------------------
 * Runtime
 * ------------------------------------------------------------------------ */

/* rg.Initialize (pyinterface.cpp:30-38): select `device`, create the context,
 * build the default F table and make rg_synchrotron_spectrum_noalloc's fixed
 * device array and kernels resident.  Idempotent. */
int rg_init(int device);

/* rg.Finalize (pyinterface.cpp:40-49): release cached plans and tables. */
int rg_finalize(void);

/* Message of the last failed call on this thread ("" if none). */
const char* rg_last_error(void);

/* Number of streaming multiprocessors of the current device (grid sizing). */
int rg_device_sm_count(int* sms);

/* Device memory helpers standing in for Kokkos::View allocation and
 * deep_copy (array.hpp:21-30, array.cpp:46-51). */
int rg_malloc(void** ptr, size_t bytes);
int rg_free(void* ptr);
int rg_memcpy_htod(void* dst, const void* src, size_t bytes, void* stream);
int rg_memcpy_dtoh(void* dst, const void* src, size_t bytes, void* stream);
int rg_memcpy_dtod(void* dst, const void* src, size_t bytes, void* stream);
int rg_memset(void* dst, int value, size_t bytes, void* stream);
int rg_stream_synchronize(void* stream);

/* --------------------------------------------------------------------------
 * Grids (host)
 * ------------------------------------------------------------------------ */

/* Logspace (snippets.cpp:39-62): pow(10, log10f(a) + i*log10f(b/a)/(n-1)) in the
 * reference's float/double mix; writes `num` floats to host `out`.  Errors as the
 * reference: start/stop must be > 0 and start < stop. */
int rg_logspace(float start, float stop, int64_t num, float* out);

/* Linspace (snippets.cpp:21-37): start + i*(stop-start)/(num-1); start < stop. */
int rg_linspace(float start, float stop, int64_t num, float* out);

/* --------------------------------------------------------------------------
 * Synchrotron kernel function F(x) = x * int_x^inf K_{5/3}
 * ------------------------------------------------------------------------ */

/* Ffunc_integrand (synchrotron.cpp:28-46) for n device values x -> device y:
 * K_{5/3} on the GPU in FP64 (own quadrature), the trapezoid with the reference's
 * float rounding steps; the 100-point inner grids Logspace(x, 20, 100) are
 * computed on the host with the platform's log10f/pow as the reference does.
 * Synchronises `stream`. */
int rg_ffunc_integrand(const float* x, int64_t n, float* y, void* stream);

/* TabulateFfunc (synchrotron.cpp:48-65): the n-node table on Logspace(xmin, xmax, n)
 * (x nodes on the host exactly as Logspace does, y as rg_ffunc_integrand with the
 * x < 1e-6 -> 0 rule).  x and y are device arrays of n floats.  Synchronises
 * `stream`. */
int rg_ffunc_table(int64_t n, float xmin, float xmax, float* x, float* y, void* stream);

/* The smooth (differentiable) table: exact F(x) = x int_x^inf K_{5/3} at nodes
 * x_j = e^{ln_xmin + j dln}, j = 0..nseg, built on the GPU in FP64, as C1 cubic
 * Hermite segments with node slopes dF/dln x = F - x^2 K_{5/3}; coef (host,
 * nullable) receives nseg x 4 floats (c0..c3 in tau = t - j).  Extension: the
 * reference has only the 200-point table. */
int rg_smooth_table(float* coef, int32_t* nseg, double* ln_xmin, double* dln);

/* --------------------------------------------------------------------------
 * Particle synchrotron spectrum
 * ------------------------------------------------------------------------ */

/* Device SoA view of Particles<D> (particles.hpp:18-72): U, E, B as three
 * components each (NULL E or B component = 0, as unset components of the
 * reference are zero), optional per-particle weight (NULL = 1; the reference has
 * no weight). */
typedef struct rg_particles {
  const float* u[3];
  const float* e[3];
  const float* b[3];
  const float* w;
  int64_t      n;
} rg_particles;

typedef struct rg_spectrum_plan rg_spectrum_plan;

/* Prepares a spectrum over `nbins` host photon energies (any positive values;
 * non-positive bins yield 0) for the scalars of SynchrotronSpectrum<D>
 * (synchrotron.cpp:107-145): B0, g_syn, e_syn_at_g_syn.  `table_mode` is one of
 * RG_TABLE_*.  Allocates the plan's device state.  A plan may be run on one
 * stream at a time. */
int rg_spectrum_plan_create(const float* bins, int32_t nbins, float B0, float g_syn,
                            float e_syn_at_g_syn, int32_t table_mode,
                            rg_spectrum_plan** plan);
int rg_spectrum_plan_destroy(rg_spectrum_plan* plan);

/* Reserves scratch for batched runs of up to `max_segments` segments (call before
 * capturing a batched run into a CUDA graph). */
int rg_spectrum_plan_reserve(rg_spectrum_plan* plan, int32_t max_segments);

/* Synchronises `stream` and reports a failure recorded on the device by earlier
 * runs of `plan` (bad segment offsets: RG_ERR_ARGUMENT; a bounded wait that gave
 * up: RG_ERR_TIMEOUT, outputs are NaN).  Clears the record.  The reference has no
 * device-side failure path; this replaces the synchronous Kokkos::fence()
 * (synchrotron.cpp:142) as the point where errors surface. */
int rg_spectrum_plan_check(rg_spectrum_plan* plan, void* stream);

/* Failure-path self-test (no reference counterpart).  Enqueues one block that
 * waits on a shared-memory barrier phase that nothing completes, bounded by
 * `polls` polls (1 .. 2^22); the wait gives up and records the status a fused run
 * records when a particle-stream copy never lands, so the next
 * rg_spectrum_plan_check returns RG_ERR_TIMEOUT.  No fault, trap or unbounded
 * wait is involved and the context stays usable. */
int rg_spectrum_plan_probe_stage_timeout(rg_spectrum_plan* plan, uint32_t polls, void* stream);

/* The fused forward: out[b] = e_b * sum_p w_p chiR_p F(e_b / e_peak_p) for the
 * particles in `p` (sync::Kernel<D>::operator(), synchrotron.hpp:145-172, summed
 * as SynchrotronSpectrum<D> does).  `out` is nbins device floats. */
int rg_spectrum_run(const rg_spectrum_plan* plan, const rg_particles* p, float* out,
                    void* stream);

/* Batched form: segment s covers particles [offsets[s], offsets[s+1]) of `p`
 * (device array of nseg+1 non-decreasing offsets); out is [nseg x nbins] device
 * floats.  One persistent launch for all segments; no host synchronisation, so
 * the call can be captured into a CUDA graph after rg_spectrum_plan_reserve.
 * Extension: the reference computes one spectrum per call. */
int rg_spectrum_run_batched(rg_spectrum_plan* plan, const rg_particles* p,
                            const int64_t* offsets, int32_t nseg, float* out, void* stream);

/* Host-resident form of rg_spectrum_run: the particle streams in `p` are HOST
 * pointers (pinned memory gives full copy bandwidth).  They are copied to the
 * device in chunks on a second stream, overlapped with the fused kernel on
 * `stream`; the chunk partials are summed in FP64.  `out` is nbins DEVICE
 * floats.  Replaces the reference's host-mirror + deep_copy ingest followed by
 * the spectrum (particles.cpp:55-99 then synchrotron.cpp:107-145).  Returns
 * after enqueueing; the host buffers must stay valid until `stream` completes. */
int rg_spectrum_run_host(rg_spectrum_plan* plan, const rg_particles* p, float* out,
                         void* stream);

/* Chooses how a particle plan sums its spectrum (and, for the smooth table, its
 * adjoint): RG_ALGO_AUTO (the default: moments when the plan supports them, the
 * fused kernels otherwise), RG_ALGO_DIRECT (the fused kernels, which evaluate
 * every (particle, bin) pair in FP32 and are bit-reproducible) or
 * RG_ALGO_MOMENTS (fails with RG_ERR_UNSUPPORTED at run time where the plan
 * cannot take it: smooth table over bins that are not log-uniform, distribution
 * source, more than 1024 segments).  All compute the reference's sum over
 * particles and bins of synchrotron.hpp:145-172.  Reference table: interval
 * moments sum the piecewise-linear F exactly in FP64 per (table cell, bin
 * interval).  Smooth table over log-uniform bins: four FP64 moments per cell of
 * the plan's bin-aligned table, and the adjoint as one cubic per cell.  Moments
 * use FP64 atomics (independent of particle order to FP64 rounding).  No
 * reference counterpart. */
int rg_spectrum_plan_set_algorithm(rg_spectrum_plan* plan, int32_t algo);
/* The smooth table a RG_TABLE_SMOOTH plan evaluates: its segment count, ln of its
 * first node and segment width in ln x, and (coef: 4 floats per segment, may be
 * NULL) the cubic Hermite coefficients (c0, c1, c2, c3) in the position tau inside
 * a segment.  For log-uniform photon bins a plan builds its own table, with nodes
 * aligned to the bins and a segment width of (bin spacing) / m, m a whole number,
 * near the device-wide table's ln(1e8) / 2048, covering at least [1e-6, 100];
 * otherwise it shares the device-wide table (rg_smooth_table).  Extension: the
 * reference has no differentiable table. */
int rg_spectrum_plan_smooth_table(const rg_spectrum_plan* plan, float* coef, int32_t* nseg, double* ln_xmin,
                                  double* dln);
/* The algorithm a run over `nseg` segments would use (RG_ALGO_DIRECT or RG_ALGO_MOMENTS). */
int rg_spectrum_plan_algorithm(const rg_spectrum_plan* plan, int32_t nseg, int32_t* algo);

/* Kernel timing: when enabled, every fused-kernel launch of `plan` is bracketed
 * by CUDA events on its stream.  rg_spectrum_plan_kernel_time synchronises those
 * events and returns the summed kernel time (ms) and the launch count since the
 * last query.  No reference counterpart (the reference has only Kokkos labels,
 * synchrotron.cpp:131). */
int rg_spectrum_plan_enable_timing(rg_spectrum_plan* plan, int32_t enable);
int rg_spectrum_plan_kernel_time(rg_spectrum_plan* plan, double* ms, int64_t* launches);

/* The plain one-spectrum-per-launch kernel (thread per particle, per-eval
 * interpolation as the reference writes it); the baseline the fused kernel is
 * measured against.  Reference table mode only. */
int rg_spectrum_run_plain(const rg_spectrum_plan* plan, const rg_particles* p, float* out,
                          void* stream);

/* One-shot drop-in for SynchrotronSpectrum<D> (synchrotron.cpp:107-145): plan
 * (cached by arguments) + run, reference table mode. */
int rg_synchrotron_spectrum(const rg_particles* p, const float* bins, int32_t nbins, float B0,
                            float g_syn, float e_syn_at_g_syn, float* out, void* stream);

/* Allocation-free form of rg_synchrotron_spectrum, for callers that cannot
 * allocate device memory once they run (a process that hands its whole device
 * memory budget out at start-up, or a plugin inside one).  No counterpart in the
 * reference.  Same arguments and result (reference table); every byte of scratch
 * comes from one fixed file-scope device array of about 1.4 MB that each GPU
 * loading the library keeps until exit, and the call makes no cudaMalloc,
 * cudaFree or other allocating call.  At most 512 photon bins (larger counts are
 * rejected with RG_ERR_ARGUMENT; nbins = 0 does nothing).  The array and the
 * kernels exist on a device once their code is loaded there (CUDA loads modules
 * lazily, on first use): rg_init(device) loads them, looks up the array's
 * address and builds the F table into it, so call rg_init on every device
 * before handing its memory out.  Without it, the first call on a device does
 * that set-up itself, needs device memory for it at that moment and
 * synchronises the device's default stream: it must then come before any
 * stream capture.  All calls share the array: calls whose GPU work overlaps
 * race on it.  A device-side failure shows as NaN outputs. */
int rg_synchrotron_spectrum_noalloc(const rg_particles* p, const float* bins, int32_t nbins, float B0,
                                    float g_syn, float e_syn_at_g_syn, float* out, void* stream);

/* --------------------------------------------------------------------------
 * Adjoint (differentiation)
 * ------------------------------------------------------------------------ */

/* Gradient of a loss L through rg_spectrum_run: given grad_out = dL/dS (nbins
 * device floats), writes dL/dw and dL/du (device, n floats each; any may be
 * NULL) for every particle of `p`.  The derivative is that of the table the plan
 * evaluates: with RG_TABLE_SMOOTH, F'(x) = F(x)/x - x K_{5/3}(x) at the table
 * nodes and the derivative of its C1 cubic Hermite interpolant in between; with
 * RG_TABLE_REFERENCE, the slope of the reference's log-linear segments
 * (tabulation.hpp:39-41).  e_peak is recomputed, not stored.  Up to 512 bins.
 * Extension: the reference has no derivative. */
int rg_spectrum_adjoint(const rg_spectrum_plan* plan, const rg_particles* p, const float* grad_out,
                        float* grad_w, float* grad_ux, float* grad_uy, float* grad_uz, void* stream);

/* Forward and adjoint with a placement record (extension): rg_spectrum_run_placed is
 * rg_spectrum_run that also writes, for every particle of `p`, the table cell and the
 * position inside it that place the particle on the plan's bin-aligned smooth table
 * (`placement`: device memory of 8 bytes per particle, p->n entries); given that record,
 * rg_spectrum_adjoint_placed skips the double-float particle stage that the adjoint
 * otherwise repeats.  The adjoint's arguments must be the plan and particles of the forward
 * that wrote the record (as for a tensor saved for a backward pass); results equal those of
 * rg_spectrum_adjoint bit for bit.  Both need a plan that runs cell moments on its
 * bin-aligned smooth table (RG_TABLE_SMOOTH over log-uniform bins, rg_spectrum_plan_algorithm
 * reporting RG_ALGO_MOMENTS for one segment); otherwise RG_ERR_UNSUPPORTED. */
int rg_spectrum_run_placed(rg_spectrum_plan* plan, const rg_particles* p, float* out, void* placement,
                           void* stream);
int rg_spectrum_adjoint_placed(rg_spectrum_plan* plan, const rg_particles* p, const void* placement,
                               const float* grad_out, float* grad_w, float* grad_ux, float* grad_uy, float* grad_uz,
                               void* stream);

/* Batched adjoint: grad_out is [nseg x nbins], segments as rg_spectrum_run_batched. */
int rg_spectrum_adjoint_batched(rg_spectrum_plan* plan, const rg_particles* p, const int64_t* offsets,
                                int32_t nseg, const float* grad_out, float* grad_w, float* grad_ux,
                                float* grad_uy, float* grad_uz, void* stream);

/* --------------------------------------------------------------------------
 * Spectrum from a tabulated distribution
 * ------------------------------------------------------------------------ */

/* A plan for sync::KernelFromDist (synchrotron.hpp:72-95): e_peak(g) =
 * e_syn_at_g_syn gbeta^2 / g_syn^2, amplitude f_g (times gbeta_g when the gamma
 * bins are log-spaced).  bins is host (nbins).  Either table mode. */
int rg_dist_plan_create(const float* bins, int32_t nbins, float g_syn, float e_syn_at_g_syn,
                        int32_t log_spaced, int32_t table_mode, rg_spectrum_plan** plan);

/* Spectrum of one distribution (gbeta, f: device, ng) into out (device, nbins). */
int rg_dist_run(const rg_spectrum_plan* plan, const float* gbeta, const float* f, int32_t ng, float* out,
                void* stream);

/* dL/df (device, ng) given dL/dS (device, nbins). */
int rg_dist_adjoint(const rg_spectrum_plan* plan, const float* gbeta, const float* f, int32_t ng,
                    const float* grad_out, float* grad_f, void* stream);

/* SynchrotronSpectrumFromDist (synchrotron.cpp:69-105, sync::KernelFromDist
 * synchrotron.hpp:72-95): gbeta (device, ng) and f (device, ng) describe the
 * distribution; J_g = gbeta_g if log_spaced else 1; bins is host (nbins);
 * out is nbins device floats. */
int rg_synchrotron_spectrum_from_dist(const float* gbeta, const float* f, int32_t ng,
                                      int32_t log_spaced, const float* bins, int32_t nbins,
                                      float g_syn, float e_syn_at_g_syn, float* out,
                                      void* stream);

/* --------------------------------------------------------------------------
 * Many distributions at once on the tensor cores
 * ------------------------------------------------------------------------ */

typedef struct rg_fromdist_plan rg_fromdist_plan;

/* Batched SynchrotronSpectrumFromDist (synchrotron.cpp:69-105 once per
 * distribution): up to max_dist distributions f[d][g] on the shared gamma bins
 * gbeta (host, ng) give S[d][e] = e * sum_g K[e][g] f[d][g] with the kernel
 * matrix K[e][g] = J_g F(e / e_peak(g)) (built once here, FP64).  The product
 * runs as one BF16 tensor-core GEMM (tcgen05) over split-precision operands:
 * split_products = 6 (three BF16 terms per operand, ~1e-8 relative per product)
 * or 3 (two terms, ~1e-5 relative).  bins is host (nbins).  Either table mode.
 * Creation builds K, splits it and autotunes the GEMM tile shape and split-K count
 * (synchronous).
 * Extension: the reference handles one distribution per call. */
int rg_fromdist_plan_create(const float* gbeta, int32_t ng, int32_t log_spaced, const float* bins, int32_t nbins,
                            float g_syn, float e_syn_at_g_syn, int32_t table_mode, int32_t split_products,
                            int32_t max_dist, rg_fromdist_plan** plan);
int rg_fromdist_plan_destroy(rg_fromdist_plan* plan);

/* f: device [ndist x ng] row-major; out: device [ndist x nbins]. */
int rg_fromdist_run(rg_fromdist_plan* plan, const float* f, int32_t ndist, float* out, void* stream);

/* Transpose GEMM: grad_f[d][g] = sum_e grad_out[d][e] e K[e][g] (device arrays). */
int rg_fromdist_adjoint(rg_fromdist_plan* plan, const float* grad_out, int32_t ndist, float* grad_f,
                        void* stream);

/* Synchronises `stream`; RG_ERR_TIMEOUT if a bounded wait in the GEMM gave up. */
int rg_fromdist_plan_check(rg_fromdist_plan* plan, void* stream);

/* Tile shape of the forward and adjoint GEMMs: chosen at plan creation by timing
 * every supported shape (CTA tile 128 x bn, a TMA ring of `stages` k blocks) on
 * the plan's own sizes, cached per device and shape.  No reference counterpart. */
int rg_fromdist_plan_config(const rg_fromdist_plan* plan, int32_t* fwd_bn, int32_t* fwd_stages,
                            int32_t* adj_bn, int32_t* adj_stages);

/* Overrides the tuned shapes with entries 0..2 of the supported list
 * ((256, 4), (128, 6), (128, 4)); -1 keeps the current choice. */
int rg_fromdist_plan_set_config(rg_fromdist_plan* plan, int32_t fwd_cfg, int32_t adj_cfg);

/* Split-K range counts of the forward and adjoint GEMMs (1: none): the gamma (or
 * photon) blocks are cut into that many ranges computed by separate CTAs and
 * summed in range order (deterministic), which fills the GPU when there are few
 * output tiles.  Tuned with the tile shape at plan creation.  No reference
 * counterpart. */
int rg_fromdist_plan_split_k(const rg_fromdist_plan* plan, int32_t* fwd_split, int32_t* adj_split);

/* Overrides the tuned counts: 1, 2, 4 or 8 and at most the direction's number of
 * 64-wide k blocks; -1 keeps the current choice.  May allocate the plan's workspace
 * (synchronous). */
int rg_fromdist_plan_set_split_k(rg_fromdist_plan* plan, int32_t fwd_split, int32_t adj_split);

/* Copies the FP64 kernel matrix K (nbins x ng) to host memory. */
int rg_fromdist_kernel_matrix(rg_fromdist_plan* plan, double* K_host);

/* --------------------------------------------------------------------------
 * Inverse-Compton spectrum
 * ------------------------------------------------------------------------ */

/* ICSpectrum (ic.cpp:15-46; ic::Kernel ic.hpp:67-94, KNfunc ic.hpp:20-25):
 * out[e] = sum_g sum_s f[g] (fs[s] / es[s]) eic[e]^2 KN(4 g es[s], q) / g^k over the pairs
 * with eic[e] <= g Gamma / (1 + Gamma), k = 1 for log-spaced gamma bins (log_spaced != 0)
 * and 2 otherwise.  All arrays are device arrays: gbins, f (ng), es, fs (ns), eic, out
 * (ne).  Non-positive IC bins give 0 (the reference yields NaN there).  Units are the
 * caller's to check (the reference requires mec^2 for es and eic). */
int rg_ic_spectrum(const float* gbins, const float* f, int32_t ng, int32_t log_spaced, const float* es,
                   const float* fs, int32_t ns, const float* eic, int32_t ne, float* out, void* stream);

/* --------------------------------------------------------------------------
 * Energy distribution (histogram)
 * ------------------------------------------------------------------------ */

/* Bin thresholds used by rg_energy_distribution: thr[k] (k >= 1) is the smallest
 * non-negative float |u|^2 whose reference bin index (particles.cpp:231-243) is
 * >= k; thr[0] = 0; nan_index receives the index the host's build of that
 * expression gives a NaN energy.  bins is host (nbins); thr is host (nbins). */
int rg_energy_thresholds(const float* bins, int32_t nbins, int32_t fourvel, float* thr,
                         int32_t* nan_index);

/* Particles<D>::energyDistribution (particles.cpp:189-260): energy = |u| (fourvel)
 * or sqrt(1+u^2); bin index always from log10 (even for linear bins), clamped
 * into [0, n-1]; hist[k] = sum 1/energy (log_spaced) or the count.  bins is host
 * (nbins); hist is nbins device floats; counts (nullable) receives exact
 * uint64 counts per bin.  Stream-ordered: returns once the work is enqueued (the
 * bin thresholds are cached on the device per bin set, so no host buffer is read
 * after the call returns). */
int rg_energy_distribution(const float* ux, const float* uy, const float* uz, int64_t n,
                           const float* bins, int32_t nbins, int32_t log_spaced,
                           int32_t fourvel, float* hist, uint64_t* counts, void* stream);

/* --------------------------------------------------------------------------
 * Diagnostics: the FP64 quadratures of the table builders evaluated on the
 * host (same code as on the GPU); K_{5/3}(x) and F(x) = x int_x^inf K_{5/3}.
 * The reference evaluates K_{5/3} with std::cyl_bessel_k (synchrotron.cpp:38).
 * ------------------------------------------------------------------------ */
double rg_debug_bessel_k53(double x);
double rg_debug_exact_F(double x);

#ifdef __cplusplus
}
#endif

#endif /* RAGNAR_GB300_H */

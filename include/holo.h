/*
 * holo.h -- C ABI of the GB300 (sm_103a) Huygens superposition library.
 *
 * One hot path: for every target m,
 *     y_m = sum_n a_n * exp(i (phi_n + s k r_nm)) / r_nm,   k = 2 pi / lambda,
 * chained object x -> projector y -> projection z.  s = +1 is the reference's
 * Direction::Forwards (y -> z), s = -1 is Direction::Backwards (x -> y).
 *
 * Conventions (all entry points):
 *   - return an int status: HOLO_OK (0) or a negative holo_status; the library
 *     never exits the process.  holo_last_error_string() describes the last
 *     failure of the calling thread.
 *   - the caller owns every buffer.  Positions are xyz-interleaved FP64 (N*3),
 *     amplitudes and phases are FP64 arrays, fields are interleaved (re, im)
 *     FP64 pairs (the reference's cuDoubleComplex / WAVE layout).
 *   - pointers are either all device pointers (the call is asynchronous on
 *     `stream`) or all host pointers (the call copies in and out and returns
 *     when the results are in host memory).  Mixing the two is rejected.
 *     Host buffers in page-locked memory (cudaHostAlloc / cudaHostRegister)
 *     are copied at the host link's rate; pageable ones go through the CUDA
 *     driver's staging buffer (1.1 ms more per 63 MB on GB300).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - calls on one handle are serialised internally; use one handle per host
 *     thread for concurrency.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   holo_transform        transform_full<dir, alg, smem>()  cuda/transform.cu:147-340
 *                         + superposition::per_block         cuda/superposition.cu:59-154
 *                         + kernel::sum_rows (cublasZgemv)   cuda/kernel.cu:179-195
 *   holo_normalize_polar  normalize_amp + polar output       cuda/transform.cu:106-139, 376, 402-405
 *   holo_project          main() file-mode chain x->y->z     cuda/main.cu:77-97, 213-221
 *   holo_transform_mc     transform() (Monte Carlo), named at README.md:127 and
 *                         driven by py/experiment.py:61-73, 147; absent from the
 *                         reference snapshot -- defined here, see the function.
 */
#ifndef HOLO_GB300_H
#define HOLO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HOLO_ABI_VERSION 1

typedef enum {
  HOLO_OK = 0,
  HOLO_ERR_INVALID = -1,     /* bad argument: null pointer, size, sign, lambda, mixed pointers */
  HOLO_ERR_CUDA = -2,        /* a CUDA runtime call failed */
  HOLO_ERR_ALLOC = -3,       /* device or host allocation failed */
  HOLO_ERR_NONFINITE = -4,   /* non-finite input or output (the reference exits with 4) */
  HOLO_ERR_TIMEOUT = -5,     /* a bounded device-side wait ran out */
  HOLO_ERR_UNSUPPORTED = -6, /* geometry outside the precision mode's validity range */
  HOLO_ERR_NO_DEVICE = -7    /* no usable CUDA device */
} holo_status;

typedef enum {
  HOLO_FP64 = 0,    /* the reference's FP64 brute force, term for term */
  HOLO_SPLIT32 = 1  /* FP64 tile frames + FP32 pair arithmetic (rel-L2 <= 1e-5) */
} holo_precision;

typedef enum { HOLO_FORWARDS = 1, HOLO_BACKWARDS = -1 } holo_direction;

/* debug flag for holo_plan_execute_flags: replace every term by 1+0i, so every
 * target sum equals N exactly (the reference's TEST_CONST_PHASE mode,
 * cuda/superposition.cu:113-116, cuda/transform.cu:325-328). */
#define HOLO_FLAG_CONST_PHASE 0x1

typedef struct holo_handle_s *holo_handle;
typedef struct holo_plan_s *holo_plan;
typedef struct holo_batch_s *holo_batch;
typedef void *holo_stream_t;

/* ---- handle -------------------------------------------------------------- */
int holo_create(int device, holo_handle *out);
int holo_destroy(holo_handle h);
const char *holo_last_error_string(void);
int holo_abi_version(void);
/* Synchronise `stream` and report (then clear) a device-side error word: a
 * kernel whose bounded wait ran out sets it (HOLO_ERR_TIMEOUT).  Calls with
 * host pointers check it themselves. */
int holo_device_status(holo_handle h, holo_stream_t stream);

/* ---- one-shot transform (transform_full, cuda/transform.cu:147-340) -----
 * y_re_im[2m], y_re_im[2m+1] = raw (unnormalised) sum for target m. */
int holo_transform(holo_handle h, int sign, double lambda,
                   const double *amp, const double *phase, const double *u_xyz, size_t N,
                   const double *v_xyz, size_t M, double *y_re_im,
                   int precision, holo_stream_t stream);

/* Same as holo_transform with an explicit kernel variant (see holo_variant_*). */
int holo_transform_variant(holo_handle h, int sign, double lambda,
                           const double *amp, const double *phase, const double *u_xyz,
                           size_t N, const double *v_xyz, size_t M, double *y_re_im,
                           int precision, int variant, holo_stream_t stream);

/* ---- plans: positions fixed, amplitudes/phases vary per call -------------
 * A plan holds the spatial tiling of sources and targets (HOLO_SPLIT32) or the
 * packed FP64 layout (HOLO_FP64).  Positions must be device pointers or host
 * pointers; they are copied into the plan. */
int holo_plan_create(holo_handle h, const double *u_xyz, size_t N, const double *v_xyz,
                     size_t M, int precision, holo_stream_t stream, holo_plan *out);
int holo_plan_destroy(holo_plan p);
int holo_plan_execute(holo_plan p, int sign, double lambda, const double *amp,
                      const double *phase, double *y_re_im, holo_stream_t stream);
int holo_plan_execute_flags(holo_plan p, int sign, double lambda, const double *amp,
                            const double *phase, double *y_re_im, int flags,
                            holo_stream_t stream);
/* Sorted visiting order of the plan's points (which = 0: sources, 1: targets):
 * out[i] = original index of the i-th point in tile order.  Host pointer. */
int holo_plan_get_order(holo_plan p, int which, int32_t *out);
/* Selected kernel variant and split factor (for the autotuner and tests). */
int holo_plan_info(holo_plan p, int *variant, int *splits, int *target_tile,
                   int *source_tile);
/* HOLO_SPLIT32: bound (metres) on the path-length error of any term, from the
 * tile extents and the gap between the point sets; the phase error bound is
 * k times it.  The planner picks tiles small enough to keep it under 3.2e-13 m
 * (5e-6 rad at 400 nm) when it can; 0 for HOLO_FP64.  Infinite when the two
 * point sets' bounding boxes touch (near field: use HOLO_FP64). */
int holo_plan_error_bound(holo_plan p, double *metres);

/* ---- tilings (no counterpart in the reference: it keeps points in file order;
 * its square-tile reorder, cuda/reorder.cu:1-92, is never called) ------------
 * HOLO_TILE_HILBERT: one stable sort by the Hilbert index of a 64 x 64 cell grid
 * over the two widest axes (cheap; exact squares on power-of-two grids).
 * HOLO_TILE_PACKED: super tiles of 8192 points in strips, each bisected so that
 * every tile of 256, 512 or 1024 consecutive points is nearly square (about twice
 * the planning time; narrower tiles for most other point counts).
 * A HOLO_SPLIT32 plan tiles with HOLO_TILE_HILBERT and tries HOLO_TILE_PACKED
 * where the Hilbert tiles' error bound rules out the fastest kernel. */
#define HOLO_TILE_HILBERT 0
#define HOLO_TILE_PACKED 1
/* Tile order of n points (xyz triples, device or host pointer): order[i] = input
 * index of the i-th point in tile order (order: n entries, host or device pointer;
 * the call returns when it is written).  No reference counterpart. */
int holo_tile_order(holo_handle h, const double *xyz, size_t n, int tiling, int32_t *order,
                    holo_stream_t stream);
/* The tiling a HOLO_SPLIT32 plan used for its sources and for its targets (-1 for a
 * HOLO_FP64 plan, which keeps the caller's order). */
int holo_plan_tiling(holo_plan p, int *tiling_sources, int *tiling_targets);

/* ---- Monte Carlo estimator (transform(), README.md:127; not in the snapshot)
 * Sources in tile order are cut into strata of `subsample` entries, targets in
 * tile order into blocks of `targets_per_block`.  Every block sums one source
 * per stratum, picked by Philox4x32-10 with counter (stratum, block, 0, 0) and
 * key (seed_lo, seed_hi), weighted by the stratum size; unbiased for the full
 * sum.  subsample = 1 reproduces the brute-force sum.  HOLO_SPLIT32 only. */
int holo_transform_mc(holo_handle h, int sign, double lambda,
                      const double *amp, const double *phase, const double *u_xyz, size_t N,
                      const double *v_xyz, size_t M, double *y_re_im,
                      uint64_t seed, int subsample, int targets_per_block,
                      holo_stream_t stream);
int holo_plan_execute_mc(holo_plan p, int sign, double lambda, const double *amp,
                         const double *phase, double *y_re_im, uint64_t seed, int subsample,
                         int targets_per_block, holo_stream_t stream);

/* ---- adjoint: gradients of a real loss L through y = transform(x) ----------
 * grad_y[2m], grad_y[2m+1] = dL/dRe y_m, dL/dIm y_m.  Computes the
 * conjugate-transposed sum w_n = e^{i phi_n} conj(sum_m G_m e^{-i s k r}/r) and
 * writes grad_amp[n] = Re w_n, grad_phase[n] = -a_n Im w_n.  The N x M phasor
 * matrix is never stored.  (No reference counterpart: the reference has no
 * gradients; e.g. 1024^2 projector phases against a 512^2 target.) */
int holo_plan_adjoint(holo_plan p, int sign, double lambda, const double *amp,
                      const double *phase, const double *grad_y, double *grad_amp,
                      double *grad_phase, holo_stream_t stream);
int holo_adjoint(holo_handle h, int sign, double lambda,
                 const double *amp, const double *phase, const double *u_xyz, size_t N,
                 const double *v_xyz, size_t M, const double *grad_y,
                 double *grad_amp, double *grad_phase, int precision, holo_stream_t stream);

/* ---- output semantics (normalize_amp + polar, cuda/transform.cu:106-139, 376,
 * 402-405): divide by max |y| unless it is below 1e-6, then write
 * amp = |y|, phase = atan2(im, re).  max_amp_out (host, may be NULL) receives
 * max |y|; with device pointers the call synchronises `stream` only when
 * max_amp_out is given. */
int holo_normalize_polar(holo_handle h, const double *y_re_im, size_t M, double *amp_out,
                         double *phase_out, double *max_amp_out, holo_stream_t stream);

/* ---- the x -> y -> z chain of the reference's file mode (cuda/main.cu:186,
 * 213-216), with the correct y -> z pass: y = Backwards(x, u -> v) normalised
 * to polar, then z = Forwards(y, v -> w) normalised to polar.  P may be 0 (no
 * z pass).  reference_wave != 0 adds the amplitude-only projector's reference
 * wave (PROJECT_PHASE = 0, cuda/transform.cu:379-395) at distance
 * reference_distance behind the projector plane. */
int holo_project(holo_handle h, double lambda,
                 const double *x_amp, const double *x_phase, const double *u_xyz, size_t N,
                 const double *v_xyz, size_t M, const double *w_xyz, size_t P,
                 double *y_amp, double *y_phase, double *z_amp, double *z_phase,
                 int precision, int reference_wave, double reference_distance,
                 holo_stream_t stream);

/* ---- batched uneven problems in one persistent launch --------------------
 * Every problem owns device buffers; a batch captures one CUDA graph (gathers,
 * persistent work-queue kernel, reductions) that holo_batch_execute replays.
 * Pointers are baked into the graph: update inputs in place between replays. */
typedef struct {
  const double *amp, *phase, *u_xyz;
  size_t N;
  const double *v_xyz;
  size_t M;
  int sign;
  double lambda;
  double *y_re_im;
} holo_problem;

int holo_batch_create(holo_handle h, const holo_problem *problems, int n_problems,
                      int precision, holo_stream_t stream, holo_batch *out);
int holo_batch_execute(holo_batch b, holo_stream_t stream);
int holo_batch_destroy(holo_batch b);
/* Total pair evaluations (sum of N * M) of one execute of the batch. */
int holo_batch_pairs(holo_batch b, long long *pairs);
int holo_transform_batched(holo_handle h, const holo_problem *problems, int n_problems,
                           int precision, holo_stream_t stream);

/* ---- kernel variants and the autotuner -----------------------------------
 * Variants are (threads per CTA, targets per thread, sources per tile, targets
 * per thread whose sin/cos run on the FMA pipe, pair model).  The pair model of
 * a HOLO_SPLIT32 variant says how the curvature term and 1/r are formed per
 * pair: 0 = with the curvature correction c^2/8r^3, 1 = without it, 2 = without
 * it and with 1/r replaced by a first-order series of 1/q (no rsqrt), 3 = model
 * 2 with the phase computed on the tensor cores (tcgen05 TF32 MMAs); it is 0
 * for every HOLO_FP64 variant.  The pair loop is 0 for scalar FP32, 1 for
 * packed FP32 pairs (f32x2, two sources per instruction), 2 for packed pairs
 * with warp-specialised sin/cos (a quarter of the warps on the FMA-pipe
 * polynomial for all their targets; fma_sincos_targets is then 0), 3 for the
 * tensor-core kernel (fma_sincos_targets then counts source pairs of every
 * 16 on the polynomial).  The planner takes the first of a speed-ordered list
 * of variants whose error bound holds for the point
 * sets; holo_autotune times every variant on a synthetic problem of the given
 * size and records the fastest for its bucket.  The Python layer persists the
 * table as JSON. */
int holo_variant_count(int precision);
int holo_variant_describe(int precision, int variant, int *threads, int *targets_per_thread,
                          int *source_tile, int *fma_sincos_targets, int *pair_model,
                          int *pair_loop);
int holo_set_variant(holo_handle h, int precision, int bucket, int variant);
int holo_get_variant(holo_handle h, int precision, int bucket, int *variant);
int holo_size_bucket(size_t N, size_t M);
int holo_autotune(holo_handle h, int precision, size_t N, size_t M, int repeats,
                  holo_stream_t stream, int *best_variant, double *best_pairs_per_s);

/* ---- measurement (the reference timed whole transforms with clock_gettime,
 * cuda/transform.cu:355, 397-398, and reported 29 FLOP per pair,
 * cuda/macros.h:71-80) ------------------------------------------------------
 * holo_kernel_launches: kernels this library has launched in the process.
 * holo_profile_begin/end: CUDA-event time of every pair-evaluation kernel
 * launched on the handle in between (end synchronises those events).
 * holo_probe_peak: measured issue rate of this GPU's pipes, kind 0 = MUFU
 * (sin.approx.f32, the XU pipe), kind 1 = FP32 FMA, kind 2 = packed FP32 pair
 * FMA (fma.rn.f32x2, two FMAs each), kind 3 = FP64 FMA (the FP64 pipe), in
 * lane-instructions per second. */
int holo_kernel_launches(long long *out);
int holo_profile_begin(holo_handle h);
int holo_profile_end(holo_handle h, double *total_ms, int *launches);
int holo_probe_peak(holo_handle h, int kind, double *ops_per_s);
/* No counterpart in the reference: a test of the failure path.  Launches one
 * thread that waits on a barrier phase nothing completes, giving up after
 * `max_cycles` (at most ~2 s of SM clock) exactly as the pipelined kernels do:
 * the handle's device error word is raised, so the next holo_device_status on
 * `stream` returns HOLO_ERR_TIMEOUT (and clears it) while the context stays
 * usable.  No GPU fault is involved. */
int holo_selftest_bounded_wait(holo_handle h, long long max_cycles, holo_stream_t stream);

/* ---- transform without any device allocation ------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate GPU memory -- hosts that own the whole device memory budget,
 * plugins running inside another framework's allocator, or real-time loops
 * that must not hit cudaMalloc/cudaFree and their implicit synchronisation.
 * Same result as holo_transform(..., HOLO_SPLIT32, ...) on device pointers
 * (amp, phase, u_xyz, v_xyz, y_re_im must all be device memory; there is no
 * handle, the device is given by index).  All scratch comes from one fixed
 * 64 MiB array in the library's device code, held on every GPU that loads the
 * library until the process exits; problems that do not fit are rejected with
 * HOLO_ERR_INVALID.  Every call shares that array and overwrites it, so calls
 * that overlap on the GPU race: calls in one process are serialised by a lock
 * and each returns only after its work on `stream` has finished.  The first
 * call on a device looks up the array's address (cudaGetSymbolAddress) and keeps
 * it for the life of the process: after a cudaDeviceReset, which may move the
 * array, this entry point must not be called again in that process.  A
 * call waits for `stream` partway (it reads the tile statistics back), so a
 * stream being captured into a graph is refused with HOLO_ERR_INVALID. */
int holo_transform_noalloc(int device, int sign, double lambda, const double *amp,
                           const double *phase, const double *u_xyz, size_t N,
                           const double *v_xyz, size_t M, double *y_re_im,
                           holo_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif

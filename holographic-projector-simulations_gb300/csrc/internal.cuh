// internal.cuh -- shared declarations of the GB300 Huygens superposition library.
//
// Layout in HBM (per point set, after planning):
//   pos     FP64 xyz, absolute positions in tile order, padded with zeros to a
//           multiple of the source tile (bulk-copy granularity)
//   ap      FP64 (phase, amp) pairs of the sources in tile order (per execute)
//   tiles   per tile of `tile` consecutive points: FP64 centre xyz + half-extent xyz
//   order   int32, tile-order position -> original index
//   partial FP64 complex [splits][M] cross-CTA partial sums (scratch)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "holo.h"

namespace holo {

// ---- constants -----------------------------------------------------------
constexpr double kTwoPi = 6.283185307179586476925286766559;
// Two-constant Cody-Waite split of 2 pi for FP64 range reduction:
// kTwoPiHi = fl64(2 pi), kTwoPiLo = 2 pi - kTwoPiHi.
constexpr double kTwoPiHi = 6.283185307179586232;
constexpr double kTwoPiLo = 2.4492935982947064e-16;
constexpr double kInvTwoPi = 0.15915494309189533577;

constexpr int kCells = 4096;                     // bins of the tiler's counting sorts
constexpr int kSuperTile = 8192;                 // points bisected together in shared memory
constexpr int kLeafTile = 256;                   // smallest tile of the bisection
constexpr int kSortBlock = 4096;                 // points per block of the counting sort
constexpr long long kWaitCycles = 4000000000LL;  // bounded device wait (~2 s at 2 GHz)

// device error word values (written by kernels, read by holo_device_status)
constexpr int kDevErrTimeout = 1;

// ---- error reporting ---------------------------------------------------------
void set_error(const char *fmt, ...);
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define HOLO_CUDA(expr)                                                  \
  do {                                                                   \
    cudaError_t _e = (expr);                                             \
    if (_e != cudaSuccess) return ::holo::cuda_fail(_e, #expr, __FILE__, __LINE__); \
  } while (0)

#define HOLO_TRY(expr)            \
  do {                            \
    int _rc = (expr);             \
    if (_rc != HOLO_OK) return _rc; \
  } while (0)

// ---- kernel variants -----------------------------------------------------------
struct Variant {
  int threads;  // threads per CTA
  int r;        // targets per thread (register blocking)
  int cs;       // sources per tile (one bulk copy per tile)
  int poly = 0; // targets per thread whose sin/cos run on the FMA pipe
  int model = 0; // per-pair model of the curvature term rho and of 1/r:
                 //   0: c / 2r (1 + c / 4r^2) with r from rsqrt (12 FP32 + 3 MUFU)
                 //   1: c / 2r, rsqrt                             (10 FP32 + 3 MUFU)
                 //   2: c / 2q with 1/q to first order in Ps / Qt  (8 FP32 + 2 MUFU)
                 //   3: model 2 with the phase from tcgen05 TF32 MMAs (3 FP32 + 2 MUFU)
                 // the planner takes models 1-3 only where their error bound holds
  int packed = 0; // 1: pair loop on packed FP32 pairs (two sources per instruction)
  int ws = 0;     // 1: warp-specialised sin/cos (`poly` is then the average per thread)
  int tc = 0;     // 1: phase on the tensor cores (kernel_tc.cu; `poly` of 16 source pairs)
  int sc = 0;     // tc only, build flags: 1 MUFU pairs accumulated in scalar FP32, 4 chunk
                 // loop half unrolled, 8 one reciprocal for the target row's 1/Qt, 1/Qt^2,
                 // 16 next block's first TMEM load early, 32 / 64 the MMA warp's /
                 // consumers' waits sleep between polls
  int tt() const { return threads * r; }
};

int split_variant_count();
Variant split_variant(int i);
// Split variants in the planner's order of preference (fastest first) for N x M.
std::vector<int> split_preferences(size_t N, size_t M);

// Largest tile boxes of a source and a target tiling: per set the bounding box
// of all tiles (lo, hi), the largest tile half-diagonal h and the largest
// half-extent along each axis hd.
struct TileStats {
  double lo_s[3], hi_s[3], h_s, hd_s[3];
  double lo_t[3], hi_t[3], h_t, hd_t[3];
};

// Error model of the split path (metres of path length) for one tiling:
//   base: FP32 rounding of the curvature term and of the in-tile offsets, and the
//         series truncation of pair model 0;
//   curv: the curvature term c^2 / 8r^3 that pair models 1 and 2 drop;
//   lin:  the extra error of pair model 2 (1/q to first order in Ps / Qt, and
//         1/q for the amplitude 1/r), its amplitude part as the phase (radians at
//         400 nm) of the same size;
//   gemm: the extra rounding of pair model 3 (3xTF32 products accumulated by the
//         tensor core, taken as 4 FP32 ulps of the curvature term).
// Infinite when the two point sets' boxes touch.
void split_error_model(const TileStats &st, double *base, double *curv, double *lin,
                       double *gemm);
// Path-length error budget of the split path: 5e-6 rad at lambda = 400 nm.
constexpr double kSplitBoundMetres = 5e-6 * 400e-9 / (2.0 * 3.14159265358979323846);
int fp64_variant_count();
Variant fp64_variant(int i);

// ---- device-side problem descriptor (one plan execute) ------------------------
struct SplitProblem {
  const float *geo_s;      // sources, tile order: offset from own tile centre, float-float
                           // (hi xyz, lo xyz) x Ns_pad
  const float2 *apf_s;     // sources, tile order, (phase mod 2 pi, amp) floats (Ns_pad)
  const float *geo_t;      // targets, tile order: offset from own tile centre, float-float (M)
  const double *pos_s;     // sources, tile order, absolute xyz (3 * Ns_pad); Monte Carlo
  const double2 *ap_s;     // sources, tile order, (phase, amp) (Ns_pad); Monte Carlo
  const double *tiles_s;   // source tiles of `cs` points: centre xyz, half xyz
  const double *pos_t;     // targets, tile order, absolute xyz (3 * M)
  const double *tiles_t;   // target tiles of `tt` points
  const int32_t *order_t;  // target tile order -> original index
  double2 *partial;        // [splits][M] (tile order) when splits > 1
  double2 *y;              // output, original target order, when splits == 1
  int N, M;
  int n_stiles, n_ttiles, splits;
  int sign;
  double sk;               // sign * k
  // Monte Carlo
  uint32_t seed_lo, seed_hi;
  int sub;                 // sources per stratum
};

struct Fp64Problem {
  const double *pos_s;     // original order, absolute xyz (3 * Ns_pad)
  const double2 *ap_s;     // (phase, amp) (Ns_pad)
  const double *pos_t;     // original order xyz (3 * M)
  double2 *partial;        // [splits][M]
  double2 *y;              // output when splits == 1
  int N, M;
  int n_stiles, n_ttiles, splits;
  int sign;
  double k;
};

// batched work item: problem index, target tile, [s_begin, s_end) source tiles, split slot
struct WorkItem {
  int problem, ttile, s_begin, s_end, split, pad0, pad1, pad2;
};

// ---- per-device kernel set-up ------------------------------------------------------
// Raise Kern's dynamic shared-memory limit to `smem_bytes` and query its CTAs per SM,
// once per device (the host API calls cost microseconds per launch); the result is
// cached per kernel and device.  `ctas_per_sm` may be null.
template <auto Kern>
int kernel_setup(int threads, int smem_bytes, int *ctas_per_sm) {
  static std::atomic<int> cache[64];  // CTAs per SM + 1 per device; 0: not set up yet
  int dev = 0;
  HOLO_CUDA(cudaGetDevice(&dev));
  const bool cached = dev >= 0 && dev < 64;
  if (cached) {
    const int c = cache[dev].load(std::memory_order_acquire);
    if (c > 0) {
      if (ctas_per_sm) *ctas_per_sm = c - 1;
      return HOLO_OK;
    }
  }
  HOLO_CUDA(cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  int occ = 0;
  HOLO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, Kern, threads, smem_bytes));
  if (cached) cache[dev].store(occ + 1, std::memory_order_release);
  if (ctas_per_sm) *ctas_per_sm = occ;
  return HOLO_OK;
}

// ---- launchers (defined in the .cu files) --------------------------------------
// probe.cu: count of kernels this library launched (reported by the benchmark)
void note_launches(int n);

// tiler.cu
int launch_bbox(const double *pos, int n, double *bbox6, double *scratch, int scratch_blocks,
                cudaStream_t s);
size_t sort_hist_entries(int n);
// Device scratch of tile_order for n points: bbox[6], bbox_scratch[6 * 1024],
// keys and keys2[n], hist[sort_hist_entries(n)], scan[that + 4096 + 16], tmp_a and
// tmp_b[n].
struct TileScratch {
  double *bbox, *bbox_scratch;
  uint16_t *keys, *keys2;
  uint32_t *hist, *scan;
  int32_t *tmp_a, *tmp_b;
};
// Tile order of a point set (pos: n xyz triples): order[r] = input index of the
// r-th point; tiles of 256, 512 and 1024 consecutive points are spatially compact.
// tiling: kTileHilbert (needs bbox, bbox_scratch, keys, hist, scan of the scratch)
// or kTilePacked (all of it; none for n <= kSuperTile).
constexpr int kTileHilbert = 0, kTilePacked = 1;
int tile_order(const double *pos, int n, int32_t *order, const TileScratch &t, cudaStream_t s,
               int tiling);
int launch_gather_pos(const double *pos, const int32_t *order, int n, int n_pad, double *out,
                      cudaStream_t s);
int launch_tile_bbox(const double *pos_sorted, int n, int tile, double *tiles, cudaStream_t s);
int launch_gather_ap(const double *amp, const double *phase, const int32_t *order, int n,
                     int n_pad, double2 *out, cudaStream_t s);
int launch_pack_ap(const double *amp, const double *phase, int n, int n_pad, double2 *out,
                   cudaStream_t s);
int launch_pack_pos(const double *pos, int n, int n_pad, double *out, cudaStream_t s);
int launch_iota(int32_t *order, int n, cudaStream_t s);
// Load the kernels of the Hilbert tiling, the tile boxes and the gathers (CUDA maps a
// kernel's code on its first use; callers that must not allocate later call this first).
int tiler_preload_hilbert();
int launch_rel_hilo(const double *pos_sorted, int n, int n_out, const double *tiles, int tile,
                    float *out, cudaStream_t s);
int launch_gather_apf(const double *amp, const double *phase, const int32_t *order, int n,
                      int n_pad, float2 *out, cudaStream_t s);

// kernel_split.cu
// kernel_tc.cu: the tensor-core split kernel (pair model 3) on source tiles of `cs`
// (1024, 512 or 256: 4 consumer warps per TMEM lane group and MMA blocks of 256
// sources; 768: 6 consumer warps, blocks of 192), `poly16` of every 16 source pairs
// on the FMA-pipe sin/cos, `flags` (Variant.sc): 1 MUFU pairs accumulated unpacked, 4
// chunk loop half unrolled, 8 one reciprocal for the target row's 1/Qt and 1/Qt^2
int launch_split_tc(const SplitProblem &p, int cs, int poly16, int flags, int grid, int *err,
                    cudaStream_t s);
int split_tc_occupancy(int cs, int poly16, int flags, int *ctas_per_sm);
// Whether a tensor-core build exists for (cs, poly16, flags) (host only, no CUDA call).
bool split_tc_has_build(int cs, int poly16, int flags);
int launch_split_tc_batched(const SplitProblem *probs, const WorkItem *items, int n_items,
                            int *queue, int cs, int poly16, int flags, int grid, int *err,
                            cudaStream_t s);
int launch_split(const SplitProblem &p, int variant, int grid, bool const_phase, bool mc,
                 int *err, cudaStream_t s);
int launch_split_batched(const SplitProblem *probs_dev, const WorkItem *items, int n_items,
                         int *queue, int variant, int grid, int *err, cudaStream_t s);
int split_occupancy(int variant, bool mc, int *ctas_per_sm);

// kernel_fp64.cu
int launch_fp64(const Fp64Problem &p, int variant, int grid, bool const_phase, int *err,
                cudaStream_t s);
int fp64_occupancy(int variant, int *ctas_per_sm);

// epilogue.cu
int epilogue_preload();  // as tiler_preload_hilbert, for the split reduction
int launch_reduce(const double2 *partial, int splits, int M, const int32_t *order,
                  double2 *y, cudaStream_t s);
int launch_reduce_batched(const SplitProblem *probs_dev, const int *prob_offsets, int n_probs,
                          int total_targets, cudaStream_t s);
int launch_max_abs(const double2 *y, int M, double *partials, int n_partials, double *max_out,
                   cudaStream_t s);
int launch_normalize_polar(const double2 *y, int M, const double *max_abs, double *amp,
                           double *phase, cudaStream_t s);
int launch_complex_to_polar(const double2 *g, int M, double *amp, double *phase,
                            cudaStream_t s);
int launch_adjoint_epilogue(const double2 *h, const double *amp, const double *phase, int N,
                            double *grad_amp, double *grad_phase, cudaStream_t s);
int launch_reference_wave(double2 *y, const double2 *y_ref, int M, const double *max_y,
                          const double *max_ref, double *amp_out, double *phase_out,
                          cudaStream_t s);

}  // namespace holo

// ---- handle, plan, batch -----------------------------------------------------------
struct holo_handle_s {
  int device = 0;
  int sm_count = 0;
  cudaMemPool_t pool = nullptr;
  int *dev_err = nullptr;  // device error word
  std::mutex mu;
  // CUDA-event pairs around each pair-evaluation kernel while profiling is on
  bool profiling = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof;
  // variant table per precision x size bucket (-1 = built-in choice)
  int variant_table[2][8] = {{-1, -1, -1, -1, -1, -1, -1, -1}, {-1, -1, -1, -1, -1, -1, -1, -1}};
};

struct holo_plan_s {
  holo_handle h = nullptr;
  int precision = HOLO_SPLIT32;
  int N = 0, M = 0;
  int n_pad = 0;                 // padded source count
  int variant = 0;
  int splits = 1;
  int grid = 0;
  int n_stiles = 0, n_ttiles = 0;
  double err_bound = 0.0;        // split path: bound on the path-length error (m)
  double model_bounds[4] = {0.0, 0.0, 0.0, 0.0};  // the same for pair models 0-3 (same tiles)
  int tiling_s = holo::kTileHilbert, tiling_t = holo::kTileHilbert;  // split: each set's tiling
  cudaStream_t last_stream = nullptr;
  // device buffers
  double *pos_s = nullptr;       // 3 * n_pad
  double *pos_t = nullptr;       // 3 * M
  double *tiles_s = nullptr;     // 6 * n_stiles
  double *tiles_t = nullptr;     // 6 * n_ttiles
  int32_t *order_s = nullptr;    // N (split only)
  int32_t *order_t = nullptr;    // M (split only)
  float *geo_s = nullptr;        // split: float-float offsets from the tile centres
  float *geo_t = nullptr;
  double *u_orig = nullptr;      // original-order positions (for the adjoint)
  double *v_orig = nullptr;
  std::vector<void *> owned;     // everything allocated for the plan
  // adjoint: the transposed plan (targets become sources), built on first use
  holo_plan_s *transposed = nullptr;
};

struct holo_batch_s {
  holo_handle h = nullptr;
  std::vector<holo_plan_s *> plans;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void *> owned;
  long long total_pairs = 0;
};

namespace holo {
// abi.cu helpers shared with the autotuner
void *pool_alloc(holo_handle h, size_t bytes, cudaStream_t s);
void pool_free(void *p, cudaStream_t s);
int size_bucket(size_t N, size_t M);
// known_order_s / known_order_t: the tile order of the same source / target array
// from another split plan (copied instead of recomputed), of tiling known_tiling_s/t
int plan_create_impl(holo_handle h, const double *u_dev, size_t N, const double *v_dev,
                     size_t M, int precision, int forced_variant, cudaStream_t s,
                     holo_plan_s **out, const int32_t *known_order_s = nullptr,
                     const int32_t *known_order_t = nullptr, int known_tiling_s = kTileHilbert,
                     int known_tiling_t = kTileHilbert);
int plan_execute_impl(holo_plan_s *p, int sign, double lambda, const double *amp_dev,
                      const double *phase_dev, double2 *y_dev, int flags, cudaStream_t s);
void plan_release(holo_plan_s *p, cudaStream_t s);
// probe.cu: bracket a pair-evaluation kernel with events while profiling
int profile_mark(holo_handle h, cudaStream_t s, bool begin);
}  // namespace holo

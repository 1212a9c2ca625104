// tiler.cu -- spatial tiling of a point set on the device.
//
// The split-precision kernel needs every tile of consecutive points to be
// spatially compact (its FP32 arithmetic is relative to the tile centre).  The
// reference keeps points in file order (its square-tile reorder,
// cuda/reorder.cu:1-92, is never called); here points are sorted by the
// Hilbert index of a 64 x 64 cell grid over the two widest axes of the
// bounding box, with a stable counting sort (deterministic: equal keys keep
// their input order).  Tiles are then fixed-size ranges of the sorted order.
#include <float.h>

#include "internal.cuh"

namespace holo {
namespace {

__device__ __forceinline__ void minmax3(double *lo, double *hi, const double *p) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = fmin(lo[d], p[d]);
    hi[d] = fmax(hi[d], p[d]);
  }
}

// Block-wide min/max of 3 coordinates; result valid in thread 0.
template <int T>
__device__ void block_minmax(double *lo, double *hi) {
  __shared__ double s_lo[T][3], s_hi[T][3];
  for (int d = 0; d < 3; ++d) {
    s_lo[threadIdx.x][d] = lo[d];
    s_hi[threadIdx.x][d] = hi[d];
  }
  __syncthreads();
  for (int w = T / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      for (int d = 0; d < 3; ++d) {
        s_lo[threadIdx.x][d] = fmin(s_lo[threadIdx.x][d], s_lo[threadIdx.x + w][d]);
        s_hi[threadIdx.x][d] = fmax(s_hi[threadIdx.x][d], s_hi[threadIdx.x + w][d]);
      }
    }
    __syncthreads();
  }
  for (int d = 0; d < 3; ++d) {
    lo[d] = s_lo[0][d];
    hi[d] = s_hi[0][d];
  }
}

__global__ void __launch_bounds__(256) k_bbox_partial(const double *__restrict__ pos, int n,
                                                      double *__restrict__ partial) {
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    minmax3(lo, hi, pos + 3 * (size_t)i);
  block_minmax<256>(lo, hi);
  if (threadIdx.x == 0)
    for (int d = 0; d < 3; ++d) {
      partial[6 * blockIdx.x + d] = lo[d];
      partial[6 * blockIdx.x + 3 + d] = hi[d];
    }
}

__global__ void __launch_bounds__(256) k_bbox_final(const double *__restrict__ partial, int nb,
                                                    double *__restrict__ bbox) {
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int d = 0; d < 3; ++d) {
      lo[d] = fmin(lo[d], partial[6 * b + d]);
      hi[d] = fmax(hi[d], partial[6 * b + 3 + d]);
    }
  block_minmax<256>(lo, hi);
  if (threadIdx.x == 0)
    for (int d = 0; d < 3; ++d) {
      bbox[d] = lo[d];
      bbox[3 + d] = hi[d];
    }
}

// Hilbert index of cell (x, y) on an n x n grid (n a power of two): the
// classic quadrant-rotation construction of the curve.
__device__ __forceinline__ uint32_t hilbert_xy2d(int n, int x, int y) {
  uint32_t d = 0;
  for (int s = n / 2; s > 0; s /= 2) {
    const int rx = (x & s) > 0;
    const int ry = (y & s) > 0;
    d += (uint32_t)s * (uint32_t)s * (uint32_t)((3 * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = n - 1 - x;
        y = n - 1 - y;
      }
      const int t = x;
      x = y;
      y = t;
    }
  }
  return d;
}

__global__ void __launch_bounds__(256) k_cell_keys(const double *__restrict__ pos, int n,
                                                   const double *__restrict__ bbox,
                                                   uint16_t *__restrict__ keys) {
  // the two widest axes of the bounding box span the cell grid
  double ext[3];
  for (int d = 0; d < 3; ++d) ext[d] = bbox[3 + d] - bbox[d];
  int a0 = 0, a1 = 1, a2 = 2;  // sort axes by extent, descending
  if (ext[a1] > ext[a0]) { int t = a0; a0 = a1; a1 = t; }
  if (ext[a2] > ext[a1]) { int t = a1; a1 = a2; a2 = t; }
  if (ext[a1] > ext[a0]) { int t = a0; a0 = a1; a1 = t; }
  const double s0 = ext[a0] > 0 ? kHilbertGrid / ext[a0] : 0.0;
  const double s1 = ext[a1] > 0 ? kHilbertGrid / ext[a1] : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double *p = pos + 3 * (size_t)i;
    int cx = (int)((p[a0] - bbox[a0]) * s0);
    int cy = (int)((p[a1] - bbox[a1]) * s1);
    cx = min(max(cx, 0), kHilbertGrid - 1);
    cy = min(max(cy, 0), kHilbertGrid - 1);
    keys[i] = (uint16_t)hilbert_xy2d(kHilbertGrid, cx, cy);
  }
}

// Per-block histogram of cell keys, stored cell-major: hist[cell * nblk + blk].
__global__ void __launch_bounds__(256) k_hist(const uint16_t *__restrict__ keys, int n,
                                              uint32_t *__restrict__ hist, int nblk) {
  __shared__ uint32_t h[kCells];
  for (int c = threadIdx.x; c < kCells; c += blockDim.x) h[c] = 0;
  __syncthreads();
  const int i0 = blockIdx.x * kSortBlock;
  const int i1 = min(n, i0 + kSortBlock);
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) atomicAdd(&h[keys[i]], 1u);
  __syncthreads();
  for (int c = threadIdx.x; c < kCells; c += blockDim.x)
    hist[(size_t)c * nblk + blockIdx.x] = h[c];
}

// Exclusive scan, three passes over blocks of 4096 entries.
__device__ uint32_t block_exclusive_scan_1024(uint32_t v, uint32_t *total) {
  __shared__ uint32_t warp_sums[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sums[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    warp_sums[lane] = w;
  }
  __syncthreads();
  const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
  *total = warp_sums[31];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(1024) k_scan_blocks(const uint32_t *__restrict__ in,
                                                      size_t count, uint32_t *__restrict__ out,
                                                      uint32_t *__restrict__ sums) {
  const size_t base = (size_t)blockIdx.x * 4096 + 4 * threadIdx.x;
  uint32_t v[4], s = 0;
  for (int j = 0; j < 4; ++j) {
    v[j] = base + j < count ? in[base + j] : 0u;
    s += v[j];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan_1024(s, &total);
  for (int j = 0; j < 4; ++j) {
    if (base + j < count) out[base + j] = run;
    run += v[j];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t *__restrict__ sums, int nb) {
  // nb <= 4096
  uint32_t v[4], s = 0;
  for (int j = 0; j < 4; ++j) {
    const int i = 4 * threadIdx.x + j;
    v[j] = i < nb ? sums[i] : 0u;
    s += v[j];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan_1024(s, &total);
  for (int j = 0; j < 4; ++j) {
    const int i = 4 * threadIdx.x + j;
    if (i < nb) sums[i] = run;
    run += v[j];
  }
}

__global__ void __launch_bounds__(1024) k_scan_add(uint32_t *__restrict__ out, size_t count,
                                                   const uint32_t *__restrict__ sums) {
  const size_t base = (size_t)blockIdx.x * 4096;
  const uint32_t add = sums[blockIdx.x];
  for (int j = threadIdx.x; j < 4096; j += blockDim.x)
    if (base + j < count) out[base + j] += add;
}

// Stable scatter: one warp walks its block's points in input order, 32 at a
// time; equal keys within a step are ranked by lane (match.any + popc), so the
// sorted order preserves input order among equal keys.
__global__ void __launch_bounds__(32) k_scatter(const uint16_t *__restrict__ keys, int n,
                                                const uint32_t *__restrict__ offsets, int nblk,
                                                int32_t *__restrict__ order) {
  __shared__ uint32_t base[kCells];
  const int lane = threadIdx.x;
  for (int c = lane; c < kCells; c += 32) base[c] = offsets[(size_t)c * nblk + blockIdx.x];
  __syncwarp();
  const int i0 = blockIdx.x * kSortBlock;
  const int i1 = min(n, i0 + kSortBlock);
  const uint32_t lt = (1u << lane) - 1u;
  for (int s = i0; s < i1; s += 32) {
    const int i = s + lane;
    const bool valid = i < i1;
    const int key = valid ? (int)keys[i] : kCells;  // kCells: sentinel, never stored
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const uint32_t rank = __popc(peers & lt);
    uint32_t dst = 0;
    if (valid) dst = base[key] + rank;
    __syncwarp();
    // the highest lane of each key group advances the running offset
    const bool last = (peers >> lane) == 1u;
    if (valid && last) base[key] += __popc(peers);
    __syncwarp();
    if (valid) order[dst] = i;
  }
}

__global__ void __launch_bounds__(256) k_gather_pos(const double *__restrict__ pos,
                                                    const int32_t *__restrict__ order, int n,
                                                    int n_pad, double *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += gridDim.x * blockDim.x) {
    if (i < n) {
      const size_t j = 3 * (size_t)(order ? order[i] : i);
      out[3 * (size_t)i] = pos[j];
      out[3 * (size_t)i + 1] = pos[j + 1];
      out[3 * (size_t)i + 2] = pos[j + 2];
    } else {
      out[3 * (size_t)i] = 0.0;
      out[3 * (size_t)i + 1] = 0.0;
      out[3 * (size_t)i + 2] = 0.0;
    }
  }
}

__global__ void __launch_bounds__(256) k_tile_bbox(const double *__restrict__ pos, int n,
                                                   int tile, double *__restrict__ tiles) {
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  const int i0 = blockIdx.x * tile;
  const int i1 = min(n, i0 + tile);
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) minmax3(lo, hi, pos + 3 * (size_t)i);
  block_minmax<256>(lo, hi);
  if (threadIdx.x == 0)
    for (int d = 0; d < 3; ++d) {
      tiles[6 * blockIdx.x + d] = 0.5 * (lo[d] + hi[d]);
      tiles[6 * blockIdx.x + 3 + d] = 0.5 * (hi[d] - lo[d]);
    }
}

__global__ void __launch_bounds__(256) k_gather_ap(const double *__restrict__ amp,
                                                   const double *__restrict__ phase,
                                                   const int32_t *__restrict__ order, int n,
                                                   int n_pad, double2 *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += gridDim.x * blockDim.x) {
    if (i < n) {
      const int j = order ? order[i] : i;
      out[i] = make_double2(phase[j], amp[j]);
    } else {
      out[i] = make_double2(0.0, 0.0);
    }
  }
}

// Offsets of tile-ordered points from their tile's centre as float-float pairs:
// out[6 i .. 6 i + 2] = hi = fl32(p - c), out[6 i + 3 .. 6 i + 5] = lo =
// fl32((p - c) - hi); zeros for the padding i >= n.
__global__ void __launch_bounds__(256) k_rel_hilo(const double *__restrict__ pos, int n,
                                                  int n_out, const double *__restrict__ tiles,
                                                  int tile, float *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_out; i += gridDim.x * blockDim.x) {
    float *o = out + 6 * (size_t)i;
    if (i < n) {
      const double *c = tiles + 6 * (size_t)(i / tile);
      for (int d = 0; d < 3; ++d) {
        const double r = pos[3 * (size_t)i + d] - c[d];
        const float hi = (float)r;
        o[d] = hi;
        o[3 + d] = (float)(r - (double)hi);
      }
    } else {
      for (int d = 0; d < 6; ++d) o[d] = 0.f;
    }
  }
}

// (phase reduced to [-pi, pi], amplitude) in float, tile order.
__global__ void __launch_bounds__(256) k_gather_apf(const double *__restrict__ amp,
                                                    const double *__restrict__ phase,
                                                    const int32_t *__restrict__ order, int n,
                                                    int n_pad, float2 *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += gridDim.x * blockDim.x) {
    if (i < n) {
      const int j = order ? order[i] : i;
      const double p = phase[j];
      const double q = rint(p * kInvTwoPi);  // two-constant Cody-Waite reduction
      const double r = fma(-q, kTwoPiLo, fma(-q, kTwoPiHi, p));
      out[i] = make_float2((float)r, (float)amp[j]);
    } else {
      out[i] = make_float2(0.f, 0.f);
    }
  }
}

__global__ void __launch_bounds__(256) k_iota(int32_t *__restrict__ order, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    order[i] = i;
}

int grid_for(int n, int per_block, int cap) {
  int g = (n + per_block - 1) / per_block;
  return g < 1 ? 1 : (g > cap ? cap : g);
}

}  // namespace

int launch_bbox(const double *pos, int n, double *bbox6, double *scratch, int scratch_blocks,
                cudaStream_t s) {
  const int nb = grid_for(n, 256 * 8, scratch_blocks);
  k_bbox_partial<<<nb, 256, 0, s>>>(pos, n, scratch); note_launches(1);
  k_bbox_final<<<1, 256, 0, s>>>(scratch, nb, bbox6); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

size_t sort_hist_entries(int n) {
  const size_t nblk = (size_t)((n + kSortBlock - 1) / kSortBlock);
  return (nblk ? nblk : 1) * kCells;
}

int sort_points(const double *pos, int n, const double *bbox6, int32_t *order, uint16_t *keys,
                uint32_t *hist, uint32_t *scan_tmp, cudaStream_t s) {
  if (n <= 0) return HOLO_OK;
  const int nblk = (n + kSortBlock - 1) / kSortBlock;
  if (nblk > 4096) return fail(HOLO_ERR_INVALID, "point set too large for the tiler (%d)", n);
  k_cell_keys<<<grid_for(n, 256, 4096), 256, 0, s>>>(pos, n, bbox6, keys); note_launches(1);
  k_hist<<<nblk, 256, 0, s>>>(keys, n, hist, nblk); note_launches(1);
  const size_t count = (size_t)nblk * kCells;
  const int nb = (int)((count + 4095) / 4096);  // == nblk
  uint32_t *offsets = scan_tmp;
  uint32_t *sums = scan_tmp + count;
  k_scan_blocks<<<nb, 1024, 0, s>>>(hist, count, offsets, sums); note_launches(1);
  k_scan_sums<<<1, 1024, 0, s>>>(sums, nb); note_launches(1);
  k_scan_add<<<nb, 1024, 0, s>>>(offsets, count, sums); note_launches(1);
  k_scatter<<<nblk, 32, 0, s>>>(keys, n, offsets, nblk, order); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_gather_pos(const double *pos, const int32_t *order, int n, int n_pad, double *out,
                      cudaStream_t s) {
  if (n_pad <= 0) return HOLO_OK;
  k_gather_pos<<<grid_for(n_pad, 256, 8192), 256, 0, s>>>(pos, order, n, n_pad, out); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_pack_pos(const double *pos, int n, int n_pad, double *out, cudaStream_t s) {
  return launch_gather_pos(pos, nullptr, n, n_pad, out, s);
}

int launch_tile_bbox(const double *pos_sorted, int n, int tile, double *tiles, cudaStream_t s) {
  if (n <= 0) return HOLO_OK;
  const int nt = (n + tile - 1) / tile;
  k_tile_bbox<<<nt, 256, 0, s>>>(pos_sorted, n, tile, tiles); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_gather_ap(const double *amp, const double *phase, const int32_t *order, int n,
                     int n_pad, double2 *out, cudaStream_t s) {
  if (n_pad <= 0) return HOLO_OK;
  k_gather_ap<<<grid_for(n_pad, 256, 8192), 256, 0, s>>>(amp, phase, order, n, n_pad, out); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_pack_ap(const double *amp, const double *phase, int n, int n_pad, double2 *out,
                   cudaStream_t s) {
  return launch_gather_ap(amp, phase, nullptr, n, n_pad, out, s);
}

int launch_rel_hilo(const double *pos_sorted, int n, int n_out, const double *tiles, int tile,
                    float *out, cudaStream_t s) {
  if (n_out <= 0) return HOLO_OK;
  k_rel_hilo<<<grid_for(n_out, 256, 8192), 256, 0, s>>>(pos_sorted, n, n_out, tiles, tile, out); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_gather_apf(const double *amp, const double *phase, const int32_t *order, int n,
                      int n_pad, float2 *out, cudaStream_t s) {
  if (n_pad <= 0) return HOLO_OK;
  k_gather_apf<<<grid_for(n_pad, 256, 8192), 256, 0, s>>>(amp, phase, order, n, n_pad, out); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_iota(int32_t *order, int n, cudaStream_t s) {
  if (n <= 0) return HOLO_OK;
  k_iota<<<grid_for(n, 256, 8192), 256, 0, s>>>(order, n); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

}  // namespace holo

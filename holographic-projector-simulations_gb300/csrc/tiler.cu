// tiler.cu -- spatial tiling of a point set on the device.
//
// The split-precision kernels need every tile of consecutive points to be
// spatially compact: their FP32 arithmetic is relative to the tile centre, and
// the planner's error bound grows with the square of the widest tile.  The
// reference keeps points in file order (its square-tile reorder,
// cuda/reorder.cu:1-92, is never called).  Two tilings:
//   Hilbert: one stable counting sort by the Hilbert index of a 64 x 64 cell grid
//     over the two widest axes -- cheap, and exact squares on power-of-two grids,
//     but runs of the curve can be L-shaped or long for other point counts;
//   packed: super tiles of 8192 by sort-tile-recursive strips (stable counting
//     sorts by the quantised widest axis, then the second axis, then the strip),
//     each bisected in shared memory down to tiles of 256 by splitting off
//     power-of-two prefixes, so every tile of 256, 512 or 1024 points is one
//     bisection segment of nearly square extent -- about twice the planning
//     time, used where the Hilbert tiles' error bound rules out the fastest kernel.
// All sorts are stable and ties keep input order: each order is deterministic
// and does not depend on the tile size.
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

constexpr int kHilbertCells = 64;  // cells per axis of the Hilbert tiling (kCells in all)
static_assert(kHilbertCells * kHilbertCells == kCells, "Hilbert cells fill the sort's bins");

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
  const double s0 = ext[a0] > 0 ? kHilbertCells / ext[a0] : 0.0;
  const double s1 = ext[a1] > 0 ? kHilbertCells / ext[a1] : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double *p = pos + 3 * (size_t)i;
    int cx = (int)((p[a0] - bbox[a0]) * s0);
    int cy = (int)((p[a1] - bbox[a1]) * s1);
    cx = min(max(cx, 0), kHilbertCells - 1);
    cy = min(max(cy, 0), kHilbertCells - 1);
    keys[i] = (uint16_t)hilbert_xy2d(kHilbertCells, cx, cy);
  }
}

// The two widest axes of a bounding box (lo[3], hi[3]), widest first.
__device__ __forceinline__ void widest_axes(const double *bbox, int *a0, int *a1) {
  double ext[3];
  for (int d = 0; d < 3; ++d) ext[d] = bbox[3 + d] - bbox[d];
  int x = 0, y = 1, z = 2;  // sort axes by extent, descending
  if (ext[y] > ext[x]) { int t = x; x = y; y = t; }
  if (ext[z] > ext[y]) { int t = y; y = z; z = t; }
  if (ext[y] > ext[x]) { int t = x; x = y; y = t; }
  *a0 = x;
  *a1 = y;
}

// Points per strip: about sqrt(#super tiles / aspect) strips make the super tiles
// square; the count is a multiple of the super tile so strips end on super-tile
// boundaries.  Every thread computes the same value from the box.
__device__ __forceinline__ long long strip_points(const double *bbox, int n) {
  int a0, a1;
  widest_axes(bbox, &a0, &a1);
  const double e0 = bbox[3 + a0] - bbox[a0], e1 = bbox[3 + a1] - bbox[a1];
  const long long nsup = (n + kSuperTile - 1) / kSuperTile;
  const double aspect = e0 > 0.0 ? fmax(e1 / e0, 1e-9) : 1.0;
  long long strips = llround(sqrt((double)nsup / aspect));
  strips = max(1LL, min(strips, min(nsup, (long long)kCells)));
  return (nsup + strips - 1) / strips * kSuperTile;
}

// Key of every point: its coordinate along the widest (axis 0) or the second widest
// (axis 1) axis of the box, quantised to kCells bins.
__global__ void __launch_bounds__(256) k_axis_keys(const double *__restrict__ pos, int n,
                                                   const double *__restrict__ bbox, int which,
                                                   uint16_t *__restrict__ keys) {
  int a0, a1;
  widest_axes(bbox, &a0, &a1);
  const int a = which ? a1 : a0;
  const double ext = bbox[3 + a] - bbox[a];
  const double sc = ext > 0.0 ? kCells / ext : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int c = (int)((pos[3 * (size_t)i + a] - bbox[a]) * sc);
    keys[i] = (uint16_t)min(max(c, 0), kCells - 1);
  }
}

// strip[order_x[r]] = r / (points per strip): the strip of each point by its rank
// along the widest axis.
__global__ void __launch_bounds__(256) k_strip_keys(const int32_t *__restrict__ order_x, int n,
                                                    const double *__restrict__ bbox,
                                                    uint16_t *__restrict__ strip) {
  const long long per = strip_points(bbox, n);
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    strip[order_x[r]] = (uint16_t)(r / per);
}

// out[r] = src[perm[r]]
__global__ void __launch_bounds__(256) k_permute_keys(const uint16_t *__restrict__ src,
                                                      const int32_t *__restrict__ perm, int n,
                                                      uint16_t *__restrict__ out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    out[r] = src[perm[r]];
}

// out[r] = a[b[r]]
__global__ void __launch_bounds__(256) k_compose(const int32_t *__restrict__ a,
                                                 const int32_t *__restrict__ b, int n,
                                                 int32_t *__restrict__ out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    out[r] = a[b[r]];
}

__device__ __forceinline__ uint32_t ordered_bits(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ordered_bits(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Segment holding position i of a super tile of nl points after `level` splits:
// a segment longer than kLeafTile splits off its largest power-of-two prefix, so
// every split point is a multiple of each smaller tile size (256, 512, 1024).
__device__ __forceinline__ void bisect_segment(int i, int nl, int level, int *start, int *len) {
  int s = 0, l = nl;
  for (int k = 0; k < level && l > kLeafTile; ++k) {
    const int unit = 1 << (31 - __clz(l - 1));  // largest power of two below l
    if (i < s + unit) {
      l = unit;
    } else {
      s += unit;
      l -= unit;
    }
  }
  *start = s;
  *len = l;
}

// Compare-exchange of the bitonic network on a pair whose lower index is `lo_i`:
// keep the smaller key at the lower index when (lo_i & k) == 0, else the larger.
__device__ __forceinline__ uint64_t bitonic_keep(uint64_t mine, uint64_t other, bool lower,
                                                 bool ascending) {
  const uint64_t mn = mine < other ? mine : other, mx = mine < other ? other : mine;
  return (lower == ascending) ? mn : mx;
}

// The in-register stages (partner distance J < 8) of the network below.
template <int J>
__device__ __forceinline__ void bitonic_reg_stage(uint64_t (&v)[8], int t, int k) {
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    if (e & J) continue;
    const uint64_t a = v[e], b = v[e | J];
    if ((a > b) == (((8 * t + e) & k) == 0)) {
      v[e] = b;
      v[e | J] = a;
    }
  }
}

// Bitonic sort of kSuperTile keys, 8 consecutive keys per thread (1024 threads):
// partner distance j < 8 within a thread's registers, 8 <= j < 256 by warp
// shuffles, j >= 256 through shared memory (element i at (i % 8) * 1024 + i / 8, so
// a warp's accesses are consecutive).  Sorts each aligned block of kmax keys (a
// power of two) ascending: the merge phases stop at kmax, whose phase runs
// ascending everywhere.
__device__ void bitonic_sort_8192(uint64_t (&v)[8], uint64_t *sh, int kmax) {
  const int t = threadIdx.x;
  for (int k = 2; k <= kmax; k <<= 1) {
    const int kd = k == kmax ? 2 * kSuperTile : k;  // (i & kd) == 0: ascending
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 256) {
#pragma unroll
        for (int e = 0; e < 8; ++e) sh[e * 1024 + t] = v[e];
        __syncthreads();
        const int pt = t ^ (j >> 3);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int i = 8 * t + e;
          v[e] = bitonic_keep(v[e], sh[e * 1024 + pt], (t & (j >> 3)) == 0, (i & kd) == 0);
        }
        __syncthreads();
      } else if (j >= 8) {
        const int m = j >> 3;  // partner lane offset (< 32)
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int i = 8 * t + e;
          const uint64_t o = __shfl_xor_sync(0xffffffffu, v[e], m);
          v[e] = bitonic_keep(v[e], o, (t & m) == 0, (i & kd) == 0);
        }
      } else if (j == 4) {
        bitonic_reg_stage<4>(v, t, kd);
      } else if (j == 2) {
        bitonic_reg_stage<2>(v, t, kd);
      } else {
        bitonic_reg_stage<1>(v, t, kd);
      }
    }
  }
}

// Recursive bisection of each super tile of kSuperTile consecutive points of
// `order` (in place): at each of five levels every segment longer than kLeafTile
// is sorted along the widest axis of its own box and split off at its largest
// power-of-two prefix, so tiles of 256, 512 and 1024 points are each one segment,
// of nearly square extent.  One bitonic sort of 64-bit keys (segment start,
// coordinate, position) per level keeps segments in place and ties in order.
__global__ void __launch_bounds__(1024) k_local_bisect(const double *__restrict__ pos, int n,
                                                       int32_t *__restrict__ order) {
  extern __shared__ __align__(16) unsigned char bsm[];
  uint64_t *sh = reinterpret_cast<uint64_t *>(bsm);                     // [kSuperTile]
  int32_t *idx = reinterpret_cast<int32_t *>(sh + kSuperTile);          // [2][kSuperTile]
  __shared__ uint32_t box[kSuperTile / kLeafTile][6];                   // ordered min, max
  __shared__ double ref[3];  // coordinates relative to the tile's first point, as floats
  __shared__ int kmax;       // sort blocks of this level: each segment lies in one
  const int t = threadIdx.x;
  const int base = blockIdx.x * kSuperTile;
  const int nl = min(kSuperTile, n - base);
  for (int i = t; i < nl; i += blockDim.x) idx[i] = order[base + i];
  if (t < 3) ref[t] = pos[3 * (size_t)order[base] + t];
  int cur = 0;
  for (int level = 0; level < 5; ++level) {
    for (int c = t; c < (kSuperTile / kLeafTile) * 6; c += blockDim.x)
      box[c / 6][c % 6] = (c % 6) < 3 ? 0xffffffffu : 0u;
    if (t == 0) kmax = 2;
    __syncthreads();
    // a warp's 256 consecutive positions lie in one segment (segments longer than
    // kLeafTile start at multiples of it): reduce in the warp, one atomic per warp
    int st[8], ln[8];
    uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0u, 0u, 0u};
    int blk = 2;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int i = 8 * t + e;
      st[e] = 0;
      ln[e] = 0;
      if (i >= nl) continue;
      bisect_segment(i, nl, level, &st[e], &ln[e]);
      // smallest aligned power-of-two block holding the whole segment
      const int last = st[e] + ln[e] - 1;
      const int b = ln[e] > 1 ? 2 << (31 - __clz(st[e] ^ last)) : 2;
      blk = max(blk, b);
      if (ln[e] > kLeafTile) {
        const double *p = pos + 3 * (size_t)idx[cur * kSuperTile + i];
        for (int d = 0; d < 3; ++d) {
          const uint32_t o = ordered_bits((float)(p[d] - ref[d]));
          mn[d] = min(mn[d], o);
          mx[d] = max(mx[d], o);
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      for (int d = 0; d < 3; ++d) {
        mn[d] = min(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
        mx[d] = max(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
      }
      blk = max(blk, __shfl_xor_sync(0xffffffffu, blk, o));
    }
    if ((t & 31) == 0) {
      const int i0 = 8 * t;  // the warp's first position
      if (i0 < nl && ln[0] > kLeafTile)
        for (int d = 0; d < 3; ++d) {
          atomicMin(&box[st[0] / kLeafTile][d], mn[d]);
          atomicMax(&box[st[0] / kLeafTile][3 + d], mx[d]);
        }
      atomicMax(&kmax, blk);
    }
    __syncthreads();
    uint64_t v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int i = 8 * t + e;
      uint64_t k = ~0ull;  // padding sorts last
      if (i < nl) {
        uint32_t c = 0;
        if (ln[e] > kLeafTile) {
          const uint32_t *b = box[st[e] / kLeafTile];
          int a = 0;
          float ext = -1.f;
          for (int d = 0; d < 3; ++d) {
            const float ed = from_ordered_bits(b[3 + d]) - from_ordered_bits(b[d]);
            if (ed > ext) {
              ext = ed;
              a = d;
            }
          }
          c = ordered_bits((float)(pos[3 * (size_t)idx[cur * kSuperTile + i] + a] - ref[a]));
        }
        k = ((uint64_t)st[e] << 45) | ((uint64_t)c << 13) | (uint64_t)i;
      }
      v[e] = k;
    }
    bitonic_sort_8192(v, sh, kmax);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int i = 8 * t + e;
      if (i < nl)
        idx[(cur ^ 1) * kSuperTile + i] = idx[cur * kSuperTile + (int)(v[e] & (kSuperTile - 1))];
    }
    cur ^= 1;
    __syncthreads();
  }
  for (int i = t; i < nl; i += blockDim.x) order[base + i] = idx[cur * kSuperTile + i];
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

// Stable counting sort of n keys (< kCells) into order (indices 0..n-1).
static int counting_sort(const uint16_t *keys, int n, int32_t *order, uint32_t *hist,
                         uint32_t *scan_tmp, cudaStream_t s) {
  const int nblk = (n + kSortBlock - 1) / kSortBlock;
  if (nblk > 4096) return fail(HOLO_ERR_INVALID, "point set too large for the tiler (%d)", n);
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

int tile_order(const double *pos, int n, int32_t *order, const TileScratch &t, cudaStream_t s,
               int tiling) {
  if (n <= 0) return HOLO_OK;
  if (tiling == kTileHilbert) {
    HOLO_TRY(launch_bbox(pos, n, t.bbox, t.bbox_scratch, 1024, s));
    k_cell_keys<<<grid_for(n, 256, 4096), 256, 0, s>>>(pos, n, t.bbox, t.keys); note_launches(1);
    return counting_sort(t.keys, n, order, t.hist, t.scan, s);
  }
  constexpr int kBisectSmem = kSuperTile * (8 + 2 * 4);
  HOLO_TRY(kernel_setup<k_local_bisect>(1024, kBisectSmem, nullptr));
  if (n <= kSuperTile) {
    HOLO_TRY(launch_iota(order, n, s));
  } else {
    HOLO_TRY(launch_bbox(pos, n, t.bbox, t.bbox_scratch, 1024, s));
    const int g = grid_for(n, 256, 8192);
    // order along the widest axis -> each point's strip
    k_axis_keys<<<g, 256, 0, s>>>(pos, n, t.bbox, 0, t.keys); note_launches(1);
    HOLO_TRY(counting_sort(t.keys, n, t.tmp_a, t.hist, t.scan, s));
    k_strip_keys<<<g, 256, 0, s>>>(t.tmp_a, n, t.bbox, t.keys2); note_launches(1);
    // along the second axis, then (stably) by strip
    k_axis_keys<<<g, 256, 0, s>>>(pos, n, t.bbox, 1, t.keys); note_launches(1);
    HOLO_TRY(counting_sort(t.keys, n, t.tmp_b, t.hist, t.scan, s));
    k_permute_keys<<<g, 256, 0, s>>>(t.keys2, t.tmp_b, n, t.keys); note_launches(1);
    HOLO_TRY(counting_sort(t.keys, n, t.tmp_a, t.hist, t.scan, s));
    k_compose<<<g, 256, 0, s>>>(t.tmp_b, t.tmp_a, n, order); note_launches(1);
  }
  k_local_bisect<<<(n + kSuperTile - 1) / kSuperTile, 1024, kBisectSmem, s>>>(pos, n, order);
  note_launches(1);
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

int tiler_preload_hilbert() {
  cudaFuncAttributes a;
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_bbox_partial));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_bbox_final));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_cell_keys));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_hist));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_scan_blocks));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_scan_sums));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_scan_add));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_scatter));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_gather_pos));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_tile_bbox));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_rel_hilo));
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_gather_apf));
  return HOLO_OK;
}

int launch_iota(int32_t *order, int n, cudaStream_t s) {
  if (n <= 0) return HOLO_OK;
  k_iota<<<grid_for(n, 256, 8192), 256, 0, s>>>(order, n); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

}  // namespace holo

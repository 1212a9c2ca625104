// gen.cu -- the CLI's generated-data mode on the device: projector / projection
// lattices (init::plane, cuda/init.h:89-158) and object shapes (init::sparse_plane,
// cuda/init.h:160-234), written into device memory and copied to the caller's host
// vector (the CLI writes them to .dat files too).
//
// Every lattice and line coordinate is the reference's host expression evaluated
// operation by operation with explicitly rounded FP64 intrinsics (no fused
// multiply-add), so it equals the reference's own output bit for bit; the circle
// and log-line shapes call CUDA's sin, cos, pow and log10, which differ from a C
// library's in the last place on some arguments.
//
// The lattice's -r jitter takes the reference's cuRAND XORWOW numbers with the same
// calls in the same order (per row: x + y uniforms, then a second, discarded call of
// (x + y) / 8), read directly from device memory.  The reference indexes them as
// random[2 j], random[2 j + 1] for every column j < y, past its x + y numbers when
// y > x (aspect ratio below 1: undefined behaviour there); here those indices wrap
// modulo x + y.
#include <cuda_runtime.h>
#include <curand.h>
#include <math.h>

#include "gen.h"

namespace holo_gen {
namespace {

constexpr double kTwoPi = 2 * M_PI;

// Rows [i0, i0 + rows) of the x * y lattice, column-fastest (v[3 (j + i y) + d]).
__global__ void k_lattice(double *__restrict__ v, size_t i0, size_t rows, size_t y, double dx,
                          double dy, double x_half, double y_half, double ox, double oy,
                          double oz, const float *__restrict__ rnd, size_t n_rnd, double x_range,
                          double y_range) {
  const size_t count = rows * y;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < count;
       q += (size_t)gridDim.x * blockDim.x) {
    const size_t i = i0 + q / y, j = q % y, k = 3 * (j + i * y);
    // i * dx - x_half + offset.x (cuda/init.h:128-129), left to right
    double px = __dadd_rn(__dsub_rn(__dmul_rn((double)i, dx), x_half), ox);
    double py = __dadd_rn(__dsub_rn(__dmul_rn((double)j, dy), y_half), oy);
    if (rnd) {  // += range * (random - 0.5) (cuda/init.h:133-134)
      px = __dadd_rn(px, __dmul_rn(x_range, __dsub_rn((double)rnd[(2 * j) % n_rnd], 0.5)));
      py = __dadd_rn(py, __dmul_rn(y_range, __dsub_rn((double)rnd[(2 * j + 1) % n_rnd], 0.5)));
    }
    v[k] = px;
    v[k + 1] = py;
    v[k + 2] = oz;
  }
}

// Points of the lattice beyond x * y repeat point 0.
__global__ void k_fill_rest(double *__restrict__ v, size_t from, size_t n) {
  for (size_t i = from + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) v[3 * i + d] = v[d];
}

__global__ void k_object(double *__restrict__ u, size_t n, int shape, double width, double ox,
                         double oy, double oz, double arbitrary_offset) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double *p = u + 3 * i;
    p[2] = oz;
    if (n == 1) {
      p[0] = ox;
      p[1] = oy;
      continue;
    }
    const double radius = width / 2.0;
    switch (shape) {
      case kShapeLine:  // i * du - half_width, du = width / (n - 1) (cuda/init.h:179-185)
        p[0] = __dsub_rn(__dmul_rn((double)i, __ddiv_rn(width, (double)(n - 1))), width / 2.0);
        break;
      case kShapeLogLine: {
        // geomspace(n, 1, 1 + width) (cuda/algebra.h:55-91): 10^(a + delta i) over the
        // logs; then x - 1 + width / 2 (cuda/init.h:188-190)
        const double a = log10(1.0), b = log10(__dadd_rn(1.0, width));
        const double delta = __ddiv_rn(__dsub_rn(b, a), __dsub_rn((double)n, 1.0));
        p[0] = __dadd_rn(__dsub_rn(pow(10.0, __dadd_rn(a, __dmul_rn(delta, (double)i))), 1.0),
                         width / 2.);
        break;
      }
      case kShapeCircle: {  // (cuda/init.h:192-205)
        const double ph = __dadd_rn(__dmul_rn((double)i, __ddiv_rn(kTwoPi, (double)n)),
                                    arbitrary_offset);
        p[0] = __dmul_rn(sin(ph), radius);
        p[1] = __dmul_rn(cos(ph), radius);
        break;
      }
      default: {  // dotted circle: point 0 keeps the previous plane's values (:206-220)
        if (i == 0) break;
        const double ph = __dadd_rn(__dmul_rn((double)i, __ddiv_rn(kTwoPi, (double)(n - 1))),
                                    arbitrary_offset);
        p[0] = __dmul_rn(sin(ph), radius);
        p[1] = __dmul_rn(cos(ph), radius);
      }
    }
    if (ox != 0 || oy != 0) {
      p[0] = __dadd_rn(p[0], ox);
      p[1] = __dadd_rn(p[1], oy);
    }
  }
}

int grid_of(size_t count) {
  const size_t b = (count + 255) / 256;
  return (int)(b < 4096 ? (b ? b : 1) : 4096);
}

}  // namespace

int lattice(double *v_host, size_t n, const holo_io::Plane &p, unsigned int seed) {
  if (n == 0) return 0;
  const size_t x = (size_t)sqrt(n * p.aspect_ratio), y = x ? n / x : 0;
  if (x == 0 || y == 0) return -1;
  const double height = p.width / p.aspect_ratio, dx = p.width / (double)x,
               dy = height / (double)y, x_half = (p.width - dx) / 2., y_half = (height - dy) / 2.;
  // x_margin = rel_margin dx, x_random_range = dx - 0.5 x_margin (cuda/init.h:109-114)
  const double rel_margin = p.randomize ? 0.05 : 0.0, x_margin = rel_margin * dx,
               y_margin = rel_margin * dy, x_range = dx - 0.5 * x_margin,
               y_range = dy - 0.5 * y_margin;
  const size_t n_random = x + y;
  double *d_v = nullptr;
  float *d_random = nullptr;
  curandGenerator_t gen = nullptr;
  int rc = 0;
  if (cudaMalloc((void **)&d_v, 3 * n * sizeof(double)) != cudaSuccess) return -1;
  if (!p.randomize) {
    k_lattice<<<grid_of(x * y), 256>>>(d_v, 0, x, y, dx, dy, x_half, y_half, p.offset[0],
                                       p.offset[1], p.offset[2], nullptr, 1, 0.0, 0.0);
  } else if (curandCreateGenerator(&gen, CURAND_RNG_PSEUDO_XORWOW) != CURAND_STATUS_SUCCESS ||
             curandSetPseudoRandomGeneratorSeed(gen, seed) != CURAND_STATUS_SUCCESS ||
             cudaMalloc((void **)&d_random, n_random * sizeof(float)) != cudaSuccess) {
    rc = -1;
  } else {
    // per row, the reference's two calls (the second one's numbers are unused), then
    // the row from the first call's numbers; all in order on the default stream
    for (size_t i = 0; i < x && rc == 0; ++i) {
      if (curandGenerateUniform(gen, d_random, n_random) != CURAND_STATUS_SUCCESS ||
          curandGenerateUniform(gen, d_random, n_random * sizeof(float) / 32) !=
              CURAND_STATUS_SUCCESS)
        rc = -1;
      else
        k_lattice<<<grid_of(y), 256>>>(d_v, i, 1, y, dx, dy, x_half, y_half, p.offset[0],
                                       p.offset[1], p.offset[2], d_random, n_random, x_range,
                                       y_range);
    }
  }
  if (rc == 0 && x * y < n) k_fill_rest<<<grid_of(n - x * y), 256>>>(d_v, x * y, n);
  if (rc == 0 && cudaGetLastError() != cudaSuccess) rc = -1;
  if (rc == 0 && cudaMemcpy(v_host, d_v, 3 * n * sizeof(double), cudaMemcpyDeviceToHost) !=
                     cudaSuccess)
    rc = -1;
  if (gen) curandDestroyGenerator(gen);
  cudaFree(d_random);
  cudaFree(d_v);
  return rc;
}

int object_points(double *u_host, size_t n, int shape, double width, const double *offset,
                  double modulate) {
  if (n == 0) return 0;
  double *d_u = nullptr;
  // the previous values come along: line shapes set x only, the dotted circle
  // leaves point 0 as it was
  if (cudaMalloc((void **)&d_u, 3 * n * sizeof(double)) != cudaSuccess) return -1;
  int rc = 0;
  if (cudaMemcpy(d_u, u_host, 3 * n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    rc = -1;
  if (rc == 0) {
    k_object<<<grid_of(n), 256>>>(d_u, n, shape, width, offset[0], offset[1], offset[2],
                                  0.1125 + modulate * kTwoPi);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(u_host, d_u, 3 * n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = -1;
  }
  cudaFree(d_u);
  return rc;
}

}  // namespace holo_gen

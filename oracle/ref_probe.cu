/*
 * ref_probe.cu -- host-side probe of the reference's own per-pair function.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled (never copied) from the reference's
 * sources where they lie, by oracle/Makefile, into oracle/_ref/.  It wraps
 * superposition::phasor_displacement<dir> (cuda/superposition.cu:35-51), which
 * is __host__ __device__, so it runs on the CPU with NORM_3D=norm3d_host
 * (the hook at cuda/macros.h:44-46).  LAMBDA is a compile-time macro in the
 * reference (cuda/macros.h:23-25), so the Makefile builds one probe per
 * wavelength.  Used only to pin the C oracle and to write golden fixtures.
 * It also wraps the reference's host-side data generators, init::plane (the
 * projector / projection lattice without -r, cuda/init.h:89-158) and
 * init::sparse_plane (the object shapes, cuda/init.h:160-234), whose outputs pin
 * the device generators of the holo CLI.
 */
#include <cuComplex.h>
#include <curand.h>
#include <curand_kernel.h>
#include <thrust/host_vector.h>
#include <cub/cub.cuh>
#include <string>
#include <vector>

/* per_block (never instantiated here) names cub::BlockReduce with six template
 * arguments, which CCCL 3 no longer accepts even in an uninstantiated template.
 * The probe only needs phasor_displacement, so the name is redirected to an
 * inert stand-in for the duration of the include. */
namespace cub {
template <typename T, int A, BlockReduceAlgorithm B, int C, int D, int E>
struct ProbeBlockReduce {
  struct TempStorage {};
  __host__ __device__ explicit ProbeBlockReduce(TempStorage &) {}
  __host__ __device__ T Sum(T x) { return x; }
};
}  // namespace cub
#define BlockReduce ProbeBlockReduce

#include "macros.h"
#include "main.h"
#include "kernel.cu"
#include "superposition.cu"
#include "init.h"

extern "C" {

double ref_lambda(void) { return LAMBDA; }

double ref_two_pi_over_lambda(void) { return TWO_PI_OVER_LAMBDA; }

/* sign > 0: Direction::Forwards, otherwise Direction::Backwards. */
void ref_phasor(double amp, double phase, const double *u, const double *v, int sign,
                double *out) {
  const Polar x = {amp, phase};
  const WAVE y = sign > 0 ? superposition::phasor_displacement<Direction::Forwards>(x, u, v)
                          : superposition::phasor_displacement<Direction::Backwards>(x, u, v);
  out[0] = y.x;
  out[1] = y.y;
}

/* Sum of the reference's own phasors for every target, source order 0..N-1,
 * added with cuCadd as per_block does (cuda/superposition.cu:107-111). */
void ref_transform(size_t N, const double *amp, const double *phase, const double *u,
                   size_t M, const double *v, int sign, double *y) {
  for (size_t m = 0; m < M; ++m) {
    WAVE acc = {0.0, 0.0};
    for (size_t n = 0; n < N; ++n) {
      const Polar x = {amp[n], phase[n]};
      const WAVE t = sign > 0
          ? superposition::phasor_displacement<Direction::Forwards>(x, &u[n * DIMS], &v[m * DIMS])
          : superposition::phasor_displacement<Direction::Backwards>(x, &u[n * DIMS], &v[m * DIMS]);
      acc = cuCadd(acc, t);
    }
    y[2 * m] = acc.x;
    y[2 * m + 1] = acc.y;
  }
}

/* init::plane without -r (no CUDA call is made then): n points, xyz-interleaved. */
void ref_plane(size_t n, double width, double ox, double oy, double oz, double aspect,
               double *out) {
  std::vector<SPACE> v(n * DIMS, 0.0);
  Plane p;
  p.width = width;
  p.offset = {ox, oy, oz};
  p.aspect_ratio = aspect;
  p.randomize = false;
  init::plane(v, p);
  for (size_t i = 0; i < n * DIMS; ++i) out[i] = v[i];
}

/* init::sparse_plane on `inout` (n points, xyz-interleaved; entries the shape leaves
 * alone keep their values).  shape: 0 Line, 1 LogLine, 2 Circle, 3 DottedCircle. */
void ref_sparse_plane(size_t n, int shape, double width, double ox, double oy, double oz,
                      double modulate, double *inout) {
  std::vector<SPACE> u(inout, inout + n * DIMS);
  const Cartesian<double> off = {ox, oy, oz};
  init::sparse_plane(u, static_cast<Shape>(shape), width, off, modulate);
  for (size_t i = 0; i < n * DIMS; ++i) inout[i] = u[i];
}

}  // extern "C"

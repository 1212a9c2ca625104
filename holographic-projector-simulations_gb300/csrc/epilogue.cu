// epilogue.cu -- deterministic cross-CTA reductions and the output semantics.
//
//   launch_reduce          sum of per-split partials in split order, scattered
//                          back to the caller's target order; replaces the
//                          reference's cublasZgemv row sum (cuda/kernel.cu:179-195)
//   launch_max_abs / launch_normalize_polar
//                          normalize_amp<false> + polar output
//                          (cuda/transform.cu:106-139, 376, 402-405)
//   launch_reference_wave  amplitude-only projector (cuda/transform.cu:379-395)
//   launch_complex_to_polar / launch_adjoint_epilogue   the adjoint's ends
#include <float.h>

#include "internal.cuh"

namespace holo {
namespace {

__global__ void __launch_bounds__(256) k_reduce(const double2 *__restrict__ partial, int splits,
                                                int M, const int32_t *__restrict__ order,
                                                double2 *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int s = 0; s < splits; ++s) {
      const double2 v = partial[(size_t)s * M + i];
      re += v.x;
      im += v.y;
    }
    y[order ? order[i] : i] = make_double2(re, im);
  }
}

__global__ void __launch_bounds__(256) k_reduce_batched(const SplitProblem *__restrict__ probs,
                                                        const int *__restrict__ offsets,
                                                        int n_probs, int total) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    // problem p with offsets[p] <= g < offsets[p + 1]
    int lo = 0, hi = n_probs;
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (offsets[mid] <= g) lo = mid; else hi = mid;
    }
    const SplitProblem &P = probs[lo];
    if (P.splits == 1) continue;
    const int i = g - offsets[lo];
    double re = 0.0, im = 0.0;
    for (int s = 0; s < P.splits; ++s) {
      const double2 v = P.partial[(size_t)s * P.M + i];
      re += v.x;
      im += v.y;
    }
    P.y[P.order_t[i]] = make_double2(re, im);
  }
}

__global__ void __launch_bounds__(256) k_max_abs_partial(const double2 *__restrict__ y, int M,
                                                         double *__restrict__ partial) {
  __shared__ double s[256];
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x)
    m = fmax(m, hypot(y[i].x, y[i].y));
  s[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void __launch_bounds__(256) k_max_final(const double *__restrict__ partial, int n,
                                                   double *__restrict__ out) {
  __shared__ double s[256];
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, partial[i]);
  s[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

__global__ void __launch_bounds__(256) k_normalize_polar(const double2 *__restrict__ y, int M,
                                                         const double *__restrict__ max_abs,
                                                         double *__restrict__ amp,
                                                         double *__restrict__ phase) {
  const double mx = *max_abs;
  const bool scale = !(mx < 1e-6);  // below 1e-6 the reference leaves y unnormalised
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
    double re = y[i].x, im = y[i].y;
    if (scale) {
      re = __ddiv_rn(re, mx);
      im = __ddiv_rn(im, mx);
    }
    amp[i] = hypot(re, im);
    phase[i] = atan2(im, re);
  }
}

__global__ void __launch_bounds__(256) k_complex_to_polar(const double2 *__restrict__ g, int M,
                                                          double *__restrict__ amp,
                                                          double *__restrict__ phase) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
    amp[i] = hypot(g[i].x, g[i].y);
    phase[i] = atan2(g[i].y, g[i].x);
  }
}

__global__ void __launch_bounds__(256) k_adjoint_epilogue(const double2 *__restrict__ h,
                                                          const double *__restrict__ amp,
                                                          const double *__restrict__ phase,
                                                          int N, double *__restrict__ grad_amp,
                                                          double *__restrict__ grad_phase) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    double sp, cp;
    sincos(phase[n], &sp, &cp);
    // w = e^{i phi} conj(H)
    const double wr = cp * h[n].x + sp * h[n].y;
    const double wi = sp * h[n].x - cp * h[n].y;
    grad_amp[n] = wr;
    grad_phase[n] = -amp[n] * wi;
  }
}

__global__ void __launch_bounds__(256) k_reference_wave(const double2 *__restrict__ y,
                                                        const double2 *__restrict__ y_ref, int M,
                                                        const double *__restrict__ max_y,
                                                        const double *__restrict__ max_ref,
                                                        double *__restrict__ amp,
                                                        double *__restrict__ phase) {
  const double my = *max_y, mr = *max_ref;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
    double yr = y[i].x, yi = y[i].y, rr = y_ref[i].x, ri = y_ref[i].y;
    if (!(my < 1e-6)) { yr = __ddiv_rn(yr, my); yi = __ddiv_rn(yi, my); }
    if (!(mr < 1e-6)) { rr = __ddiv_rn(rr, mr); ri = __ddiv_rn(ri, mr); }
    // interference, then the phase of the reference wave (the projector only
    // modulates amplitude): y = from_polar(|y + y_ref|, angle(y_ref))
    const double a = hypot(yr + rr, yi + ri);
    const double p = atan2(ri, rr);
    double sp, cp;
    sincos(p, &sp, &cp);
    const double tr = a * cp, ti = a * sp;
    amp[i] = hypot(tr, ti);
    phase[i] = atan2(ti, tr);
  }
}

int blocks_for(int n) {
  int g = (n + 255) / 256;
  return g < 1 ? 1 : (g > 8192 ? 8192 : g);
}

}  // namespace

int epilogue_preload() {
  cudaFuncAttributes a;
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_reduce));
  return HOLO_OK;
}

int launch_reduce(const double2 *partial, int splits, int M, const int32_t *order, double2 *y,
                  cudaStream_t s) {
  if (M <= 0) return HOLO_OK;
  k_reduce<<<blocks_for(M), 256, 0, s>>>(partial, splits, M, order, y); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_reduce_batched(const SplitProblem *probs_dev, const int *prob_offsets, int n_probs,
                          int total_targets, cudaStream_t s) {
  if (total_targets <= 0) return HOLO_OK;
  k_reduce_batched<<<blocks_for(total_targets), 256, 0, s>>>(probs_dev, prob_offsets, n_probs,
                                                             total_targets); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_max_abs(const double2 *y, int M, double *partials, int n_partials, double *max_out,
                   cudaStream_t s) {
  int nb = (M + 2047) / 2048;
  nb = nb < 1 ? 1 : (nb > n_partials ? n_partials : nb);
  k_max_abs_partial<<<nb, 256, 0, s>>>(y, M, partials); note_launches(1);
  k_max_final<<<1, 256, 0, s>>>(partials, nb, max_out); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_normalize_polar(const double2 *y, int M, const double *max_abs, double *amp,
                           double *phase, cudaStream_t s) {
  if (M <= 0) return HOLO_OK;
  k_normalize_polar<<<blocks_for(M), 256, 0, s>>>(y, M, max_abs, amp, phase); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_complex_to_polar(const double2 *g, int M, double *amp, double *phase,
                            cudaStream_t s) {
  if (M <= 0) return HOLO_OK;
  k_complex_to_polar<<<blocks_for(M), 256, 0, s>>>(g, M, amp, phase); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_adjoint_epilogue(const double2 *h, const double *amp, const double *phase, int N,
                            double *grad_amp, double *grad_phase, cudaStream_t s) {
  if (N <= 0) return HOLO_OK;
  k_adjoint_epilogue<<<blocks_for(N), 256, 0, s>>>(h, amp, phase, N, grad_amp, grad_phase); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

int launch_reference_wave(double2 *y, const double2 *y_ref, int M, const double *max_y,
                          const double *max_ref, double *amp_out, double *phase_out,
                          cudaStream_t s) {
  if (M <= 0) return HOLO_OK;
  k_reference_wave<<<blocks_for(M), 256, 0, s>>>(y, y_ref, M, max_y, max_ref, amp_out,
                                                 phase_out); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

}  // namespace holo

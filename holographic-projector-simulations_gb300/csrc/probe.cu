// probe.cu -- measurement support: the kernel-launch counter, CUDA-event timing
// of the dominant (pair-evaluation) kernel, and pipe-throughput probes that
// measure this GPU's MUFU (XU pipe) and FP32 FMA issue rates, the denominators
// of the split kernel's roofline.  The reference timed whole transforms with
// clock_gettime (cuda/transform.cu:355, 397-398) and counted FLOP_PER_POINT = 29
// per pair (cuda/macros.h:71-80).
#include <algorithm>
#include <atomic>

#include "internal.cuh"
#include "ptx.cuh"

namespace holo {

static std::atomic<long long> g_launches{0};

void note_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int profile_mark(holo_handle h, cudaStream_t s, bool begin) {
  if (!h->profiling) return HOLO_OK;
  if (begin) {
    cudaEvent_t e0, e1;
    HOLO_CUDA(cudaEventCreate(&e0));
    HOLO_CUDA(cudaEventCreate(&e1));
    h->prof.push_back({e0, e1});
    HOLO_CUDA(cudaEventRecord(e0, s));
  } else if (!h->prof.empty()) {
    HOLO_CUDA(cudaEventRecord(h->prof.back().second, s));
  }
  return HOLO_OK;
}

namespace {

// 8 independent chains per thread keep the pipe busy; the result is stored so
// the work cannot be removed.
__global__ void __launch_bounds__(256) k_probe_mufu(float *out, int iters, float seed) {
  float x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = seed + 0.001f * (threadIdx.x + j);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = ptx::sin_approx(x[j]);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  if (s == 12345.f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_probe_ffma(float *out, int iters, float seed) {
  float x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = seed + 0.001f * (threadIdx.x + j);
  const float a = 0.999f, b = 0.0001f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fmaf(x[j], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  if (s == 12345.f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// packed pairs: one fma.rn.f32x2 = two FP32 FMAs
__global__ void __launch_bounds__(256) k_probe_ffma2(float *out, int iters, float seed) {
  uint64_t x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j)
    x[j] = ptx::pack2(seed + 0.001f * (threadIdx.x + j), seed - 0.001f * (threadIdx.x + j));
  const uint64_t a = ptx::pack2(0.999f, 0.998f), b = ptx::pack2(0.0001f, 0.0002f);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = ptx::fma2(x[j], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float lo, hi;
    ptx::unpack2(x[j], lo, hi);
    s += lo + hi;
  }
  if (s == 12345.f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 FMA chains: the rate of the DFMA pipe, the denominator of the plain FP64
// kernel's roofline (every FP64 operation of a pair issues on that pipe).  16
// independent chains per thread: a warp's DFMA holds the pipe for many cycles,
// so the probe needs more operations in flight than the FP32 ones.
__global__ void __launch_bounds__(256) k_probe_dfma(float *out, int iters, float seed) {
  double x[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) x[j] = (double)seed + 0.001 * (threadIdx.x + j);
  const double a = 0.999, b = 0.0001;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = fma(x[j], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 16; ++j) s += x[j];
  if (s == 12345.0) out[blockIdx.x * blockDim.x + threadIdx.x] = (float)s;
}

// One thread waits, bounded, on a barrier phase that nothing completes: the
// timeout path of every pipelined kernel here (raise the error word, return).
__global__ void k_selftest_wait(long long max_cycles, int *err) {
  __shared__ __align__(8) uint64_t bar;
  ptx::mbar_init(&bar, 1);
  ptx::fence_barrier_init();
  if (!ptx::mbar_wait_bounded(&bar, 0u, max_cycles)) atomicExch(err, kDevErrTimeout);
}

}  // namespace
}  // namespace holo

using namespace holo;

extern "C" {

int holo_kernel_launches(long long *out) {
  if (!out) return fail(HOLO_ERR_INVALID, "null output");
  *out = g_launches.load();
  return HOLO_OK;
}

int holo_profile_begin(holo_handle h) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  std::lock_guard<std::mutex> lk(h->mu);
  for (auto &e : h->prof) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  h->prof.clear();
  h->profiling = true;
  return HOLO_OK;
}

int holo_profile_end(holo_handle h, double *total_ms, int *launches) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  std::lock_guard<std::mutex> lk(h->mu);
  h->profiling = false;
  double total = 0.0;
  for (auto &e : h->prof) {
    HOLO_CUDA(cudaEventSynchronize(e.second));
    float ms = 0.f;
    HOLO_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
    total += ms;
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  if (launches) *launches = (int)h->prof.size();
  h->prof.clear();
  if (total_ms) *total_ms = total;
  return HOLO_OK;
}

int holo_selftest_bounded_wait(holo_handle h, long long max_cycles, holo_stream_t stream) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  if (max_cycles <= 0 || max_cycles > kWaitCycles)
    return fail(HOLO_ERR_INVALID, "max_cycles must be in (0, %lld]", kWaitCycles);
  std::lock_guard<std::mutex> lk(h->mu);
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  k_selftest_wait<<<1, 1, 0, (cudaStream_t)stream>>>(max_cycles, h->dev_err);
  const cudaError_t e = cudaGetLastError();
  if (prev >= 0) cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_fail(e, "self-test kernel", __FILE__, __LINE__);
  return HOLO_OK;
}

// kind 0: MUFU sin.approx.f32 ops/s, kind 1: FP32 FMA ops/s (one op = one
// lane-instruction), kind 2: packed fma.rn.f32x2 lane-instructions/s (each is
// two FMAs), kind 3: FP64 FMA ops/s
int holo_probe_peak(holo_handle h, int kind, double *ops_per_s) {
  if (!h || !ops_per_s) return fail(HOLO_ERR_INVALID, "null argument");
  if (kind < 0 || kind > 3) return fail(HOLO_ERR_INVALID, "unknown probe %d", kind);
  std::lock_guard<std::mutex> lk(h->mu);
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  const int blocks = h->sm_count * 8, threads = 256;
  const int iters = kind == 0 ? 4096 : kind == 3 ? 512 : 32768;
  float *out = nullptr;
  HOLO_CUDA(cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    if (kind == 0) k_probe_mufu<<<blocks, threads>>>(out, iters, 0.1f + rep);
    else if (kind == 1) k_probe_ffma<<<blocks, threads>>>(out, iters, 0.1f + rep);
    else if (kind == 2) k_probe_ffma2<<<blocks, threads>>>(out, iters, 0.1f + rep);
    else k_probe_dfma<<<blocks, threads>>>(out, iters, 0.1f + rep);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double ops = (double)blocks * threads * iters * (kind == 3 ? 16.0 : 8.0);
    if (rep > 0 && ms > 0) best = std::max(best, ops / (ms * 1e-3));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  cudaError_t e = cudaGetLastError();
  if (prev >= 0) cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_fail(e, "probe kernel", __FILE__, __LINE__);
  *ops_per_s = best;
  return HOLO_OK;
}

}  // extern "C"

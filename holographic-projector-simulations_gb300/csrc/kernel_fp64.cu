// kernel_fp64.cu -- plain FP64 Huygens superposition (HOLO_FP64).
//
// Term for term the reference's FP64 path: phasor_displacement<dir>
// (cuda/superposition.cu:35-51) with norm3d_host (cuda/kernel.cu:95-99) and
// from_polar (cuda/kernel.cu:158-166).  Every product, sum, square root and
// quotient is rounded separately (explicit __d*_rn intrinsics, no FMA
// contraction), so each term equals the CPU oracle's bit for bit up to the
// last-ulp difference of sin/cos; only the order of the additions differs.
//
// Organisation (replacing per_block + cublasZgemv row sums,
// cuda/superposition.cu:59-154, cuda/kernel.cu:179-195): persistent CTAs over
// (target tile, source split) items; source tiles of CS points are staged in
// shared memory by TMA bulk copies (double-buffered, mbarrier-tracked); each
// thread owns R targets in registers; splits of the source range are reduced
// afterwards in a fixed order (deterministic, no atomics).
#include "internal.cuh"
#include "ptx.cuh"

namespace holo {
namespace {

template <int THREADS, int R, int CS>
struct Fp64Smem {
  static constexpr size_t raw_pos = 0;                                     // double [2][CS*3]
  static constexpr size_t raw_ap = raw_pos + 2 * CS * 3 * sizeof(double);  // double2 [2][CS]
  static constexpr size_t bar = raw_ap + 2 * CS * sizeof(double2);         // uint64 [2]
  static constexpr size_t bytes = bar + 2 * sizeof(uint64_t);
};

// MINB: CTAs per SM the register allocation must leave room for (the FP64 pipe
// needs enough resident warps to hide the latency of its MUFU-seeded sqrt,
// division and sin/cos sequences).
template <int THREADS, int R, int CS, int MINB, bool CONST>
__global__ void __launch_bounds__(THREADS, MINB)
    k_fp64(const Fp64Problem P, int n_items, int *err) {
  extern __shared__ __align__(128) unsigned char smem[];
  using L = Fp64Smem<THREADS, R, CS>;
  constexpr int TT = THREADS * R;
  double *raw_pos = reinterpret_cast<double *>(smem + L::raw_pos);
  double2 *raw_ap = reinterpret_cast<double2 *>(smem + L::raw_ap);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::bar);
  const int tid = threadIdx.x;
  if (tid == 0) {
    ptx::mbar_init(&bar[0], 1);
    ptx::mbar_init(&bar[1], 1);
    ptx::fence_barrier_init();
  }
  __syncthreads();
  uint32_t par[2] = {0u, 0u};

  auto issue = [&](int j, int buf) {
    ptx::mbar_arrive_expect_tx(&bar[buf], CS * (3 * sizeof(double) + sizeof(double2)));
    ptx::bulk_g2s(raw_pos + buf * CS * 3, P.pos_s + (size_t)j * CS * 3,
                  CS * 3 * sizeof(double), &bar[buf]);
    ptx::bulk_g2s(raw_ap + buf * CS, P.ap_s + (size_t)j * CS, CS * sizeof(double2),
                  &bar[buf]);
  };

  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int tt = item / P.splits;
    const int split = item % P.splits;
    const int sb = (int)(((long long)P.n_stiles * split) / P.splits);
    const int se = (int)(((long long)P.n_stiles * (split + 1)) / P.splits);

    double vx[R], vy[R], vz[R], re[R], im[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int ti = tt * TT + tid + r * THREADS;
      const bool ok = ti < P.M;
      vx[r] = ok ? P.pos_t[3 * (size_t)ti] : 0.0;
      vy[r] = ok ? P.pos_t[3 * (size_t)ti + 1] : 0.0;
      vz[r] = ok ? P.pos_t[3 * (size_t)ti + 2] : 1.0;
      re[r] = 0.0;
      im[r] = 0.0;
    }
    if (tid == 0 && sb < se) issue(sb, 0);

    for (int j = sb; j < se; ++j) {
      const int buf = (j - sb) & 1;
      if (tid == 0 && j + 1 < se) issue(j + 1, buf ^ 1);
      const bool ok = ptx::mbar_wait_bounded(&bar[buf], par[buf], kWaitCycles);
      par[buf] ^= 1u;
      if (!__syncthreads_and(ok)) {
        if (tid == 0) atomicExch(err, kDevErrTimeout);
        return;
      }
      const double *sp = raw_pos + buf * CS * 3;
      const double2 *sa = raw_ap + buf * CS;
      const int count = min(CS, P.N - j * CS);
      for (int s = 0; s < count; ++s) {
        const double ux = sp[3 * s], uy = sp[3 * s + 1], uz = sp[3 * s + 2];
        const double2 a2 = sa[s];  // (phase, amp)
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (CONST) {
            re[r] = __dadd_rn(re[r], 1.0);
          } else {
            const double a = __dsub_rn(vx[r], ux);
            const double b = __dsub_rn(vy[r], uy);
            const double c = __dsub_rn(vz[r], uz);
            const double ss = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
            const double dist = __dsqrt_rn(ss);
            const double kr = __dmul_rn(dist, P.k);
            const double ph = P.sign > 0 ? __dadd_rn(a2.x, kr) : __dsub_rn(a2.x, kr);
            const double rr = __ddiv_rn(a2.y, dist);
            double sn, cs;
            sincos(ph, &sn, &cs);
            re[r] = __dadd_rn(re[r], __dmul_rn(rr, cs));
            im[r] = __dadd_rn(im[r], __dmul_rn(rr, sn));
          }
        }
      }
      __syncthreads();  // buffer `buf` is refilled two tiles later
    }

#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int ti = tt * TT + tid + r * THREADS;
      if (ti < P.M) {
        const double2 v = make_double2(re[r], im[r]);
        if (P.splits == 1)
          P.y[ti] = v;
        else
          P.partial[(size_t)split * P.M + ti] = v;
      }
    }
  }
}

constexpr Variant kVariants[] = {
    {128, 4, 256},  // 0
    {256, 2, 256},  // 1
    {128, 2, 256},  // 2
    {64, 4, 256},   // 3
    {128, 2, 256},  // 4: registers for 8 CTAs per SM
    {128, 1, 256},  // 5: registers for 12 CTAs per SM
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

template <int THREADS, int R, int CS, int MINB>
int launch_variant(const Fp64Problem &p, int grid, bool cst, int *err, cudaStream_t s) {
  using L = Fp64Smem<THREADS, R, CS>;
  const int n_items = p.n_ttiles * p.splits;
  if (n_items <= 0) return HOLO_OK;
  if (cst) {
    auto kern = k_fp64<THREADS, R, CS, MINB, true>;
    HOLO_TRY((kernel_setup<k_fp64<THREADS, R, CS, MINB, true>>(THREADS, (int)L::bytes, nullptr)));
    kern<<<grid, THREADS, L::bytes, s>>>(p, n_items, err); note_launches(1);
  } else {
    auto kern = k_fp64<THREADS, R, CS, MINB, false>;
    HOLO_TRY((kernel_setup<k_fp64<THREADS, R, CS, MINB, false>>(THREADS, (int)L::bytes, nullptr)));
    kern<<<grid, THREADS, L::bytes, s>>>(p, n_items, err); note_launches(1);
  }
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

template <int THREADS, int R, int CS, int MINB>
int occupancy_variant(int *out) {
  using L = Fp64Smem<THREADS, R, CS>;
  return kernel_setup<k_fp64<THREADS, R, CS, MINB, false>>(THREADS, (int)L::bytes, out);
}

}  // namespace

int fp64_variant_count() { return kNumVariants; }
Variant fp64_variant(int i) { return kVariants[i]; }

#define HOLO_FP64_DISPATCH(V, CALL)                                        \
  switch (V) {                                                             \
    case 0: return CALL(128, 4, 256, 1);                                   \
    case 1: return CALL(256, 2, 256, 1);                                   \
    case 2: return CALL(128, 2, 256, 1);                                   \
    case 3: return CALL(64, 4, 256, 1);                                    \
    case 4: return CALL(128, 2, 256, 8);                                   \
    case 5: return CALL(128, 1, 256, 12);                                  \
    default: return fail(HOLO_ERR_INVALID, "unknown fp64 variant %d", V);  \
  }

int launch_fp64(const Fp64Problem &p, int variant, int grid, bool const_phase, int *err,
                cudaStream_t s) {
#define CALL(T, R, C, B) launch_variant<T, R, C, B>(p, grid, const_phase, err, s)
  HOLO_FP64_DISPATCH(variant, CALL)
#undef CALL
}

int fp64_occupancy(int variant, int *ctas_per_sm) {
#define CALL(T, R, C, B) occupancy_variant<T, R, C, B>(ctas_per_sm)
  HOLO_FP64_DISPATCH(variant, CALL)
#undef CALL
}

}  // namespace holo

// kernel_split.cu -- split-precision Huygens superposition (HOLO_SPLIT32).
//
// Reference hot path: superposition::per_block + phasor_displacement
// (cuda/superposition.cu:35-51, 59-154) in FP64.  Here each CTA owns a tile of
// TT = THREADS * R targets (R per thread, in registers) and walks source tiles
// of CS points that a TMA bulk copy stages in shared memory (mbarrier-tracked;
// the copy of the next tile overlaps the current pair loop).  For every
// (target tile, source tile) pair a frame is
// built in FP64 from the two tile centres T0, S0:
//   D = T0 - S0, r0 = |D|, e = D / r0, (e1, e2) an orthonormal basis of e-perp.
// With t' = t - T0, s' = s - S0 and d = t' - s':
//   r = |D + d| = q + rho,   q = r0 + e.d,   c = |d_perp|^2,
//   rho = c / (q + r) = (c / 2r) (1 + c / (4 r^2) + O(c^2 / r^4)),
//   s k r = [phi-independent] s k (r0 + e.t')  - s k e.s'  + s k rho.
// The two linear terms are separable and large (k |t'| ~ 1e3 rad): they are
// evaluated once per target (B) and once per source (A) per tile pair, in
// float-float arithmetic on the FP32 pipe from offsets the plan precomputes as
// hi/lo float pairs, and reduced mod 2 pi (three-part Cody-Waite); only the
// frame itself (one thread per tile pair) is FP64.  Per pair only the small
// curvature term s k rho (|rho| / r0 ~ 1e-6) and the amplitude 1/r are formed
// in FP32; their sensitivity to FP32 rounding of d is suppressed by |d| / r0.
// Per pair: 12 FP32 ops + 3 MUFU ops (rsqrt, sin, cos); 10 + 3 without the
// curvature correction, 8 + 2 with 1/r replaced by a first-order series of 1/q
// (pair models 0, 1, 2: the planner takes 1 or 2 only where the error bound of
// the tiling allows).  POLY of the R targets per thread take sin/cos from an
// FMA-pipe polynomial instead (+16 FP32 ops, -2 MUFU).  Sums run in FP32 over
// one source tile (CS terms), are rotated by e^{iB} and carried in FP64.
#include "internal.cuh"
#include "ptx.cuh"

namespace holo {
namespace {

#include "split_frame.cuh"

// Philox4x32-10 (Salmon et al., SC'11); same rounds as the oracle.
__device__ __forceinline__ uint32_t philox_first(uint32_t c0, uint32_t c1, uint32_t k0,
                                                 uint32_t k1) {
  uint32_t c2 = 0, c3 = 0;
#pragma unroll
  for (int round = 0; round < 10; ++round) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c0;
}

// One staging buffer of source records (float-float offsets + (phase, amp)):
// the bulk copy of tile j+1 is issued once the frame phase of tile j has
// consumed it, so it overlaps tile j's pair loop.
template <int THREADS, int R, int CS>
struct SplitSmem {
  static constexpr size_t raw_geo = 0;                                   // float [CS*6]
  static constexpr size_t raw_apf = raw_geo + CS * 6 * sizeof(float);    // float2 [CS]
  static constexpr size_t rec = raw_apf + CS * sizeof(float2);           // float4 [CS]
  static constexpr size_t amp = rec + CS * sizeof(float4);                // float2 [CS]
  static constexpr size_t acc = (amp + CS * sizeof(float2) + 15) / 16 * 16;  // double2 [R][THREADS]
  static constexpr size_t bphase = acc + R * THREADS * sizeof(double2);      // float [R][THREADS]
  static constexpr size_t frame = (bphase + R * THREADS * sizeof(float) + 15) / 16 * 16;
  static constexpr size_t bar = frame + sizeof(Frame);                    // uint64 [2]
  static constexpr size_t bytes = bar + 2 * sizeof(uint64_t);
};

// CTAs per SM the launch bounds ask for: as many as shared memory holds (228 KB
// per SM, 1 KB reserved per CTA), at most what 128 (R >= 8) or 80 (R < 8)
// registers per thread allow.
template <int THREADS, int R, int CS>
struct SplitMinBlocks {
  static constexpr int by_smem = (int)(233472 / (SplitSmem<THREADS, R, CS>::bytes + 1024));
  static constexpr int by_regs = 65536 / (THREADS * (R >= 8 ? 128 : 80));
  static constexpr int m = by_smem < by_regs ? by_smem : by_regs;
  static constexpr int value = m < 1 ? 1 : (m > 8 ? 8 : m);
};

// Process one work item: target tile `tt`, source tiles [sb, se), writing into
// partial slot `split` (or the final output when the problem has one split).
template <int THREADS, int R, int CS, int POLY, bool CONST, bool MC>
__device__ __forceinline__ bool process_item(const SplitProblem &P, int tt, int split, int sb,
                                             int se, unsigned char *smem, uint32_t &par0,
                                             uint32_t &par1, int *err) {
  using L = SplitSmem<THREADS, R, CS>;
  constexpr int TT = THREADS * R;
  float *raw_geo = reinterpret_cast<float *>(smem + L::raw_geo);
  float2 *raw_apf = reinterpret_cast<float2 *>(smem + L::raw_apf);
  float4 *rec = reinterpret_cast<float4 *>(smem + L::rec);
  float2 *ramp = reinterpret_cast<float2 *>(smem + L::amp);
  Frame *fr = reinterpret_cast<Frame *>(smem + L::frame);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::bar);
  // FP64 carries and the per-target phase B live in shared memory (index
  // [r][tid]) so that the pair loop keeps only 5 R registers per thread.
  double2 *acc = reinterpret_cast<double2 *>(smem + L::acc);
  float *bph = reinterpret_cast<float *>(smem + L::bphase);
  const int tid = threadIdx.x;
  const double sk = P.sk;
  const float kap2 = (float)(0.5 * sk);    // s k / 2
  const int n_strata = MC ? (P.N + P.sub - 1) / P.sub : 0;
  // POLY = (targets per thread on the FMA-pipe sin/cos) | 16 (pair model 1) or
  // | 32 (pair model 2); neither bit: model 0, with the curvature correction.
  // Model 1 stores the curvature quantities scaled: c_s = kap2^2 c, q_s =
  // |kap2| q, so r2_s = q_s^2 + c_s = kap2^2 r^2 and the phase is one FMA,
  // theta' = c_s rsqrt(r2_s) + sign A, where theta = sign theta' (the sign
  // flips the imaginary part at the end) and the amplitude a |kap2| absorbs
  // the 1 / |kap2| of rsqrt(r2_s).
  // Model 2 replaces 1/r by 1/q = 1 / (Qt - Ps) ~ (1 + Ps / Qt) / Qt: with
  // iq = |kap2| / Qt + Ps |kap2| / Qt^2 (one FMA of per-target constants),
  // theta' = c iq + sign A.  c / 2q is the curvature term rho = c / (q + r) to
  // the same order as c / 2r (error c^2 / 8q^3 against c^2 / 8r^3).  The
  // amplitude 1/r ~ 1/q ~ (1 + Ps / r0) / Qt (relative error c / 2q^2 +
  // |Ps| |Qt - r0| / (Qt r0) + (Ps / Qt)^2) is split into a per-source factor,
  // folded into the record, and 1 / Qt, applied to the tile sum per target.
  // | 64 (model 2 only): the pair loop runs on packed FP32 pairs (f32x2), one
  // instruction for the same target and two consecutive sources, the records
  // stored pairwise: (qx, qx', qy, qy'), (qz, qz', qw, qw'), (a, a', S2, S2').
  // Model 2 per pair: 7 FP32 ops (c: 3, iq, theta, two accumulations) + the
  // sin/cos.
  constexpr int NPOLY = POLY & 15;
  constexpr bool LIN = (POLY & 32) != 0;
  constexpr bool CORR = (POLY & 48) == 0;
  constexpr bool PK = (POLY & 64) != 0;
  // | 128 (packed only): warp-specialised sin/cos -- a quarter of the warps on the
  // polynomial for all their targets, the rest on the MUFU pipe
  constexpr bool WS = (POLY & 128) != 0;
  static_assert(!PK || LIN, "packed pair loop: pair model 2 only");
  static_assert(!WS || (PK && THREADS % 128 == 0 && THREADS >= 512),
                "warp specialisation: packed, one polynomial warp per sub-partition");
  const float ak = fabsf(kap2), ak2 = kap2 * kap2, iak = 1.f / fabsf(kap2);
  const float sgn = kap2 < 0.f ? -1.f : 1.f;

  auto issue = [&](int j) {
    // tile j of CS sources: CS*24 B of float-float offsets + CS*8 B of (phase, amp)
    ptx::mbar_arrive_expect_tx(&bar[0], CS * (6 * sizeof(float) + sizeof(float2)));
    ptx::bulk_g2s(raw_geo, P.geo_s + (size_t)j * CS * 6, CS * 6 * sizeof(float), &bar[0]);
    ptx::bulk_g2s(raw_apf, P.apf_s + (size_t)j * CS, CS * sizeof(float2), &bar[0]);
  };
  (void)par1;

  if (!MC && tid == 0 && sb < se) issue(sb);

#pragma unroll
  for (int r = 0; r < R; ++r) acc[r * THREADS + tid] = make_double2(0.0, 0.0);

  for (int j = sb; j < se; ++j) {
    // sources with records in this tile (the pair loop skips the padding)
    const int count = MC ? min(CS, n_strata - j * CS) : min(CS, P.N - j * CS);
    if (tid == 0) {
      const double *tc = P.tiles_t + 6 * (size_t)tt;
      double sc[3];
      if (!MC) {
        for (int d = 0; d < 3; ++d) sc[d] = P.tiles_s[6 * (size_t)j + d];
      } else {
        // union of the source tiles that hold this chunk's strata
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        const int t_first = j * P.sub;
        const int t_last = min(P.n_stiles, (j + 1) * P.sub);
        for (int t = t_first; t < t_last; ++t)
          for (int d = 0; d < 3; ++d) {
            const double c = P.tiles_s[6 * (size_t)t + d], h = P.tiles_s[6 * (size_t)t + 3 + d];
            lo[d] = fmin(lo[d], c - h);
            hi[d] = fmax(hi[d], c + h);
          }
        for (int d = 0; d < 3; ++d) sc[d] = 0.5 * (lo[d] + hi[d]);
      }
      build_frame(fr, tc, sc, sk);
    }
    if (!MC) {
      const bool ok = ptx::mbar_wait_bounded(&bar[0], par0, kWaitCycles);
      par0 ^= 1u;
      if (!__syncthreads_and(ok)) {
        if (tid == 0) atomicExch(err, kDevErrTimeout);
        return false;
      }
    } else {
      __syncthreads();
    }

    // ---- phase A: per-source records of this tile pair (FP32 pipe) ----
    // A = phi - s k e.s' needs ~1e-7 rad of ~1e3 rad: float-float products of
    // (s k e) and the offset s' (precomputed per plan), then a float reduction.
    const float f1x = fr->e1[0], f1y = fr->e1[1], f1z = fr->e1[2];
    const float f2x = fr->e2[0], f2y = fr->e2[1], f2z = fr->e2[2];
    const float fex = fr->ef[0], fey = fr->ef[1], fez = fr->ef[2];
    const float ir0 = fr->r0f > 0.f ? 1.f / fr->r0f : 0.f;
    float ah[3], al[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      ah[d] = fr->ah[d];
      al[d] = fr->al[d];
    }
    for (int i = tid; i < CS; i += THREADS) {
      bool valid;
      float sh[3], A, am;
      if (!MC) {
        valid = j * CS + i < P.N;
        const float *g = raw_geo + 6 * i;
        const float sl[3] = {g[3], g[4], g[5]};
        sh[0] = g[0]; sh[1] = g[1]; sh[2] = g[2];
        const float2 pa = raw_apf[i];
        float S, E;
        dot3_ff(ah, al, sh, sl, S, E);
        float S2, E2;
        two_sum(pa.x, -S, S2, E2);
        A = CONST ? 0.f : reduce_two_pi_ff(S2, __fsub_rn(E2, E));
        am = CONST ? 1.f : pa.y;
      } else {
        // Monte Carlo: sampled sources from anywhere in the chunk's strata, FP64
        const int st = j * CS + i;
        valid = st < n_strata;
        sh[0] = sh[1] = sh[2] = 0.f;
        A = 0.f;
        am = 0.f;
        if (valid) {
          const int start = st * P.sub;
          const int size = min(P.sub, P.N - start);
          const uint32_t rnd = philox_first((uint32_t)st, (uint32_t)tt, P.seed_lo, P.seed_hi);
          const int sidx = start + (int)(rnd % (uint32_t)size);
          const double *sp = P.pos_s + 3 * (size_t)sidx;
          const double2 a2 = P.ap_s[sidx];
          const double dx = sp[0] - fr->s0[0], dy = sp[1] - fr->s0[1], dz = sp[2] - fr->s0[2];
          const double ps = fma(fr->e[0], dx, fma(fr->e[1], dy, fr->e[2] * dz));
          A = CONST ? 0.f : (float)reduce_two_pi(fma(-sk, ps, a2.x));
          sh[0] = (float)dx; sh[1] = (float)dy; sh[2] = (float)dz;
          am = CONST ? (float)size : (float)(a2.y * (double)size);
        }
      }
      // record: (-2 Sx, -2 Sy, Ps, A) and (a, Sx^2 + Sy^2), so that per pair
      // c = |d_perp|^2 = (T2 + S2) - 2 (Tx Sx + Ty Sy) costs one add and two FMAs
      float4 q;
      float2 a;
      if (valid) {
        const float Sx = fmaf(f1x, sh[0], fmaf(f1y, sh[1], f1z * sh[2]));
        const float Sy = fmaf(f2x, sh[0], fmaf(f2y, sh[1], f2z * sh[2]));
        const float Ps = fmaf(fex, sh[0], fmaf(fey, sh[1], fez * sh[2]));
        if (CORR || CONST) {
          q = make_float4(-2.f * Sx, -2.f * Sy, Ps, A);
          a = make_float2(am, fmaf(Sx, Sx, Sy * Sy));
        } else if (LIN) {
          q = make_float4(-2.f * Sx, -2.f * Sy, Ps, sgn * A);
          a = make_float2(am * fmaf(Ps, ir0, 1.f), fmaf(Sx, Sx, Sy * Sy));
        } else {
          q = make_float4(-2.f * ak2 * Sx, -2.f * ak2 * Sy, ak * Ps, sgn * A);
          a = make_float2(am * ak, ak2 * fmaf(Sx, Sx, Sy * Sy));
        }
      } else {
        // padding: zero amplitude at the frame origin (finite terms times 0)
        q = make_float4(0.f, 0.f, 0.f, 0.f);
        a = make_float2(0.f, 0.f);
      }
      if (PK) {
        float *pa = reinterpret_cast<float *>(rec), *pb = pa + 2 * CS;
        float *pc = reinterpret_cast<float *>(ramp);
        const int o = 4 * (i >> 1) + (i & 1);
        pa[o] = q.x;
        pa[o + 2] = q.y;
        pb[o] = q.z;
        pb[o + 2] = q.w;
        pc[o] = a.x;
        pc[o + 2] = a.y;
      } else {
        rec[i] = q;
        ramp[i] = a;
      }
    }

    // ---- per-thread target frame (FP32 pipe, float-float for B) ----
    float Tx[R], Ty[R], Qt[R], T2[R], kq[R];
    const float r0f = fr->r0f, b0h = fr->b0h, b0l = fr->b0l;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int ti = tt * TT + tid + r * THREADS;
      float th[3] = {0.f, 0.f, 0.f}, tl[3] = {0.f, 0.f, 0.f};
      if (ti < P.M) {
        const float *g = P.geo_t + 6 * (size_t)ti;
        th[0] = g[0]; th[1] = g[1]; th[2] = g[2];
        tl[0] = g[3]; tl[1] = g[4]; tl[2] = g[5];
      }
      // B = s k (r0 + e.t') mod 2 pi
      float S, E, S2, E2;
      dot3_ff(ah, al, th, tl, S, E);
      two_sum(S, b0h, S2, E2);
      const float B = reduce_two_pi_ff(S2, __fadd_rn(__fadd_rn(E, E2), b0l));
      Tx[r] = fmaf(f1x, th[0], fmaf(f1y, th[1], f1z * th[2]));
      Ty[r] = fmaf(f2x, th[0], fmaf(f2y, th[1], f2z * th[2]));
      Qt[r] = r0f + fmaf(fex, th[0], fmaf(fey, th[1], fez * th[2]));
      T2[r] = fmaf(Tx[r], Tx[r], Ty[r] * Ty[r]);
      // curvature correction s k c^2 / (8 r^3) = h * c * (s k / 8) / r^2 with
      // 1/r^2 taken as 1/Qt^2 (relative error ~2 |Ps| / r0 of a ~1e-6 rad term)
      kq[r] = __fdividef(0.25f * kap2, Qt[r] * Qt[r]);
      if (LIN && !CONST) {
        // Qt[r] <- |kap2| / Qt and kq[r] <- |kap2| / Qt^2 (correctly rounded)
        const float iq = ak / Qt[r];
        kq[r] = iq / Qt[r];
        Qt[r] = iq;
      } else if (!CORR && !CONST) {
        Qt[r] *= ak;
        T2[r] *= ak2;
      }
      bph[r * THREADS + tid] = B;
    }
    __syncthreads();
    // the staging buffer is free: fetch the next tile while this one is summed
    if (!MC && tid == 0 && j + 1 < se) issue(j + 1);

    // ---- pair loop: count sources x R targets ----
    float re[R], im[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      re[r] = 0.f;
      im[r] = 0.f;
    }
    if (PK) {
      // two consecutive sources per instruction; an odd count reads one padding
      // record (zero amplitude), so (count + 1) / 2 pairs cover the tile
      const float4 *pa = reinterpret_cast<const float4 *>(rec), *pb = pa + CS / 2;
      const float4 *pc = reinterpret_cast<const float4 *>(ramp);
      const int npair = (count + 1) >> 1;
      if (WS) {
        // the last quarter of the warps (one per SM sub-partition) take every
        // sin/cos from the polynomial, the others from the MUFU pipe
        if ((tid >> 5) >= (THREADS >> 5) * 3 / 4)
          packed_pairs<R, R, CONST>(pa, pb, pc, npair, Tx, Ty, T2, Qt, kq, re, im);
        else
          packed_pairs<R, 0, CONST>(pa, pb, pc, npair, Tx, Ty, T2, Qt, kq, re, im);
      } else {
        packed_pairs<R, NPOLY, CONST>(pa, pb, pc, npair, Tx, Ty, T2, Qt, kq, re, im);
      }
    } else {
#pragma unroll 2
      for (int s = 0; s < count; ++s) {
        const float4 q = rec[s];
        const float2 as = ramp[s];
        if (CONST) {
#pragma unroll
          for (int r = 0; r < R; ++r) re[r] += as.x;
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float c = fmaf(Tx[r], q.x, fmaf(Ty[r], q.y, T2[r] + as.y));
            float th, w;
            if (LIN) {
              const float iq = fmaf(q.z, kq[r], Qt[r]);  // |kap2| / q to first order
              th = fmaf(c, iq, q.w);                     // sign * theta
              w = as.x;                                  // 1 / Qt after the sum
            } else {
              const float qq = Qt[r] - q.z;
              const float r2 = fmaf(qq, qq, c);
              const float ir = ptx::rsqrt_approx(r2);
              if (CORR) {
                const float h = c * ir;
                th = fmaf(h, fmaf(c, kq[r], kap2), q.w);
              } else {
                th = fmaf(c, ir, q.w);  // scaled: sign * theta
              }
              w = as.x * ir;
            }
            float sn, cs;
            if (r < NPOLY) {
              poly_sincos(th, &sn, &cs);  // FMA pipe
            } else {
              sn = ptx::sin_approx(th);   // XU (MUFU) pipe
              cs = ptx::cos_approx(th);
            }
            re[r] = fmaf(w, cs, re[r]);
            im[r] = fmaf(w, sn, im[r]);
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      double2 a = acc[r * THREADS + tid];
      if (CONST) {
        a.x += (double)re[r];
        a.y += (double)im[r];
      } else {
        float sb, cb;
        __sincosf(bph[r * THREADS + tid], &sb, &cb);
        const float sc = LIN ? Qt[r] * iak : 1.f;  // model 2: 1 / Qt
        const float rer = re[r] * sc, imr = (CORR ? im[r] : sgn * im[r]) * sc;
        a.x += (double)fmaf(rer, cb, -imr * sb);
        a.y += (double)fmaf(rer, sb, imr * cb);
      }
      acc[r * THREADS + tid] = a;
    }
    __syncthreads();  // rec, ramp and the frame are rewritten next tile
  }

#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int ti = tt * TT + tid + r * THREADS;
    if (ti < P.M) {
      const double2 v = acc[r * THREADS + tid];
      if (P.splits == 1)
        P.y[P.order_t[ti]] = v;
      else
        P.partial[(size_t)split * P.M + ti] = v;
    }
  }
  return true;
}

__device__ __forceinline__ void split_range(int n, int splits, int s, int *b, int *e) {
  *b = (int)(((long long)n * s) / splits);
  *e = (int)(((long long)n * (s + 1)) / splits);
}

template <int THREADS, int R, int CS, int POLY, bool CONST, bool MC>
__global__ void __launch_bounds__(THREADS, SplitMinBlocks<THREADS, R, CS>::value)
    k_split(const SplitProblem P, int n_items, int *err) {
  extern __shared__ __align__(128) unsigned char smem[];
  using L = SplitSmem<THREADS, R, CS>;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::bar);
  if (threadIdx.x == 0) {
    ptx::mbar_init(&bar[0], 1);
    ptx::mbar_init(&bar[1], 1);
    ptx::fence_barrier_init();
  }
  __syncthreads();
  uint32_t par0 = 0, par1 = 0;
  const int n_src = MC ? ((P.N + P.sub - 1) / P.sub + CS - 1) / CS : P.n_stiles;
  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int tt = item / P.splits;
    const int split = item % P.splits;
    int sb, se;
    split_range(n_src, P.splits, split, &sb, &se);
    if (!process_item<THREADS, R, CS, POLY, CONST, MC>(P, tt, split, sb, se, smem, par0, par1, err))
      return;
  }
}

template <int THREADS, int R, int CS, int POLY>
__global__ void __launch_bounds__(THREADS, SplitMinBlocks<THREADS, R, CS>::value)
    k_split_batched(const SplitProblem *__restrict__ probs, const WorkItem *__restrict__ items,
                    int n_items, int *queue, int *err) {
  extern __shared__ __align__(128) unsigned char smem[];
  using L = SplitSmem<THREADS, R, CS>;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::bar);
  __shared__ int s_item;
  if (threadIdx.x == 0) {
    ptx::mbar_init(&bar[0], 1);
    ptx::mbar_init(&bar[1], 1);
    ptx::fence_barrier_init();
  }
  uint32_t par0 = 0, par1 = 0;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) break;
    const WorkItem w = items[it];
    const SplitProblem P = probs[w.problem];
    if (!process_item<THREADS, R, CS, POLY, false, false>(P, w.ttile, w.split, w.s_begin, w.s_end,
                                                    smem, par0, par1, err))
      return;
  }
}

// ---- variant table ------------------------------------------------------------
constexpr Variant kVariants[] = {
    {256, 8, 1024, 0},  // 0: TT 2048
    {128, 8, 1024, 0},  // 1: TT 1024
    {256, 4, 1024, 0},  // 2: TT 1024
    {128, 4, 512, 0},   // 3: TT 512
    {128, 2, 256, 0},   // 4: TT 256 (Monte Carlo blocks of 256 targets)
    {256, 8, 512, 0},   // 5: TT 2048, short source tiles
    {256, 8, 1024, 1},  // 6: as 0, 1 of 8 targets per thread on the FMA-pipe sin/cos
    {256, 8, 1024, 2},  // 7: as 0, 2 of 8
    {256, 8, 1024, 3},  // 8: as 0, 3 of 8
    {256, 4, 1024, 1},  // 9: as 2, 1 of 4
    {256, 8, 1024, 4},  // 10: as 0, 4 of 8
    {256, 4, 512, 1},   // 11: 3 CTAs/SM
    {128, 4, 512, 1},   // 12: 5 CTAs/SM
    // pair model 1: no curvature correction (10 FP32 ops + 3 MUFU per pair)
    {256, 4, 1024, 1, 1},  // 13: as 9
    {256, 8, 1024, 2, 1},  // 14: as 7
    {256, 8, 1024, 3, 1},  // 15: as 8
    {256, 4, 512, 1, 1},   // 16: as 11
    // pair model 2: 1/q to first order, no rsqrt (8 FP32 ops + 2 MUFU per pair)
    {256, 4, 1024, 1, 2},  // 17: as 9
    {256, 4, 1024, 0, 2},  // 18: as 2
    {256, 8, 1024, 1, 2},  // 19: as 6
    {256, 8, 1024, 2, 2},  // 20: as 7
    {256, 4, 512, 1, 2},   // 21: as 11
    // pair model 2 on packed FP32 pairs (f32x2: two sources per instruction)
    {256, 4, 1024, 0, 2, 1},  // 22: as 18
    {256, 4, 1024, 1, 2, 1},  // 23: as 17
    {256, 4, 1024, 2, 2, 1},  // 24: 2 of 4 targets on the FMA-pipe sin/cos
    {256, 2, 1024, 1, 2, 1},  // 25: TT 512, 1 of 2
    {128, 4, 1024, 1, 2, 1},  // 26: TT 512, 1 of 4
    {256, 4, 512, 1, 2, 1},   // 27: as 23 with source tiles of 512 (3 CTAs/SM)
    {256, 4, 512, 0, 2, 1},   // 28: as 22 with source tiles of 512
    {128, 4, 512, 1, 2, 1},   // 29: TT 512, source tiles of 512 (5 CTAs/SM)
    {512, 4, 1024, 1, 2, 1},     // 30: as 23 with 512 threads (TT 2048)
    {512, 4, 1024, 0, 2, 1, 1},  // 31: as 30, warp-specialised sin/cos (4 of 16 warps polynomial)
    {512, 2, 1024, 0, 2, 1, 1},  // 32: TT 1024 (tiles of 23), warp-specialised sin/cos
    // pair model 3: the phase on the tensor cores (kernel_tc.cu), TT 512, source tiles
    // of 1024; `poly` of every 16 source pairs on the FMA-pipe sin/cos
    {512, 1, 1024, 4, 3, 1, 0, 1},     // 33
    {512, 1, 1024, 6, 3, 1, 0, 1},     // 34
    {512, 1, 1024, 8, 3, 1, 0, 1},     // 35
    {512, 1, 1024, 7, 3, 1, 0, 1},     // 36
    {512, 1, 1024, 5, 3, 1, 0, 1},     // 37
    {512, 1, 1024, 6, 3, 1, 0, 1, 1},  // 38: as 34, MUFU pairs accumulated unpacked
    {512, 1, 1024, 7, 3, 1, 0, 1, 1},  // 39: as 36, MUFU pairs accumulated unpacked
    {128, 4, 768, 1, 2, 1},            // 40: packed model 2, TT 512 x source tiles of 768
    // pair model 3 with 24 consumer warps (6 per TMEM lane group), source tiles of 768
    {512, 1, 768, 6, 3, 1, 0, 1},      // 41
    {512, 1, 768, 5, 3, 1, 0, 1},      // 42
    {512, 1, 768, 7, 3, 1, 0, 1},      // 43
    // pair model 3 on shorter source tiles (512, 256): four times and twice the tile
    // pairs of variant 34, for point sets whose error bound needs narrower tiles
    {512, 1, 512, 6, 3, 1, 0, 1},      // 44
    {512, 1, 256, 6, 3, 1, 0, 1},      // 45
    {128, 4, 256, 1, 2, 1},            // 46: packed model 2, TT 512 x source tiles of 256
    // pair model 3, build flags 4 (chunk loop half unrolled) and 8 (one reciprocal for
    // the target row's 1/Qt and 1/Qt^2)
    {512, 1, 1024, 6, 3, 1, 0, 1, 4},   // 47: as 34
    {512, 1, 1024, 6, 3, 1, 0, 1, 8},   // 48: as 34
    {512, 1, 1024, 6, 3, 1, 0, 1, 12},  // 49: as 34
    {512, 1, 1024, 7, 3, 1, 0, 1, 4},   // 50: as 36
    // build flag 16: the next block's first TMEM load during a block's last chunk
    {512, 1, 1024, 6, 3, 1, 0, 1, 16},  // 51: as 34
    {512, 1, 1024, 6, 3, 1, 0, 1, 24},  // 52: as 34, with flag 8
    {512, 1, 1024, 7, 3, 1, 0, 1, 16},  // 53: as 36
    // build flags 32 / 64: the MMA warp's / the consumers' waits sleep between polls
    {512, 1, 1024, 6, 3, 1, 0, 1, 32},  // 54: as 34
    {512, 1, 1024, 6, 3, 1, 0, 1, 96},  // 55: as 34
    {512, 1, 1024, 6, 3, 1, 0, 1, 48},  // 56: as 51
    // build flags 128 (polynomial columns in half turns from the tensor cores) and 256
    // (degree-7 sine): cheaper FMA-pipe sin/cos, so more polynomial pairs
    {512, 1, 1024, 6, 3, 1, 0, 1, 128},   // 57: as 34
    {512, 1, 1024, 6, 3, 1, 0, 1, 384},   // 58: as 34
    {512, 1, 1024, 7, 3, 1, 0, 1, 384},   // 59: 7 of 16
    {512, 1, 1024, 8, 3, 1, 0, 1, 384},   // 60: 8 of 16
    {512, 1, 1024, 9, 3, 1, 0, 1, 384},   // 61: 9 of 16
    {512, 1, 1024, 7, 3, 1, 0, 1, 432},   // 62: as 59, with flags 16 and 32
    {512, 1, 1024, 8, 3, 1, 0, 1, 432},   // 63: as 60, with flags 16 and 32
    {512, 1, 1024, 6, 3, 1, 0, 1, 400},   // 64: as 58, with flag 16
    {512, 1, 1024, 6, 3, 1, 0, 1, 432},   // 65: as 58, with flags 16 and 32
    {512, 1, 1024, 6, 3, 1, 0, 1, 392},   // 66: as 58, with flag 8
    {512, 1, 512, 6, 3, 1, 0, 1, 384},    // 67: as 44, flags 128 and 256
    {512, 1, 512, 6, 3, 1, 0, 1, 400},    // 68: as 67, with flag 16
    {512, 1, 256, 6, 3, 1, 0, 1, 384},    // 69: as 45, flags 128 and 256
    {512, 1, 256, 6, 3, 1, 0, 1, 400},    // 70: as 69, with flag 16
    {512, 1, 768, 6, 3, 1, 0, 1, 384},    // 71: as 41 (24 consumer warps), flags 128 and 256
    {512, 1, 768, 7, 3, 1, 0, 1, 384},    // 72: as 43, flags 128 and 256
    // the builder-warp kernel (flag 512; 1024: two builder warps, not four) with the
    // half-turn polynomial: as 58, 71, 67, 69
    {512, 1, 1024, 6, 3, 1, 0, 1, 896},   // 73
    {512, 1, 768, 6, 3, 1, 0, 1, 896},    // 74
    {512, 1, 512, 6, 3, 1, 0, 1, 896},    // 75
    {512, 1, 256, 6, 3, 1, 0, 1, 1920},   // 76
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

template <int THREADS, int R, int CS, int POLY, bool CONST, bool MC>
int launch_one(const SplitProblem &p, int grid, int *err, cudaStream_t s) {
  using L = SplitSmem<THREADS, R, CS>;
  auto kern = k_split<THREADS, R, CS, POLY, CONST, MC>;
  HOLO_TRY((kernel_setup<k_split<THREADS, R, CS, POLY, CONST, MC>>(THREADS, (int)L::bytes,
                                                                   nullptr)));
  const int n_items = p.n_ttiles * p.splits;
  if (n_items <= 0) return HOLO_OK;
  kern<<<grid, THREADS, L::bytes, s>>>(p, n_items, err); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

template <int THREADS, int R, int CS, int POLY>
int launch_variant(const SplitProblem &p, int grid, bool cst, bool mc, int *err,
                   cudaStream_t s) {
  if (cst && mc) return launch_one<THREADS, R, CS, POLY, true, true>(p, grid, err, s);
  if (cst) return launch_one<THREADS, R, CS, POLY, true, false>(p, grid, err, s);
  if (mc) return launch_one<THREADS, R, CS, POLY, false, true>(p, grid, err, s);
  return launch_one<THREADS, R, CS, POLY, false, false>(p, grid, err, s);
}

template <int THREADS, int R, int CS, int POLY>
int batched_variant(const SplitProblem *probs, const WorkItem *items, int n_items, int *queue,
                    int grid, int *err, cudaStream_t s) {
  using L = SplitSmem<THREADS, R, CS>;
  auto kern = k_split_batched<THREADS, R, CS, POLY>;
  HOLO_TRY((kernel_setup<k_split_batched<THREADS, R, CS, POLY>>(THREADS, (int)L::bytes, nullptr)));
  kern<<<grid, THREADS, L::bytes, s>>>(probs, items, n_items, queue, err); note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

template <int THREADS, int R, int CS, int POLY>
int occupancy_variant(bool mc, int *out) {
  using L = SplitSmem<THREADS, R, CS>;
  if (mc) return kernel_setup<k_split<THREADS, R, CS, POLY, false, true>>(THREADS, (int)L::bytes, out);
  return kernel_setup<k_split<THREADS, R, CS, POLY, false, false>>(THREADS, (int)L::bytes, out);
}

}  // namespace

int split_variant_count() { return kNumVariants; }
Variant split_variant(int i) { return kVariants[i]; }

// The tensor-core variants have no Monte Carlo or constant-phase build: those
// calls run a CUDA-core variant with the same tiles (512 targets and 1024, 768, 512
// or 256 sources: variant 26, 40, 29 or 46).
static bool is_tc(int v) { return v >= 0 && v < kNumVariants && kVariants[v].tc; }
static int tc_fallback(int v) {
  switch (kVariants[v].cs) {
    case 768: return 40;
    case 512: return 29;
    case 256: return 46;
    default: return 26;
  }
}

std::vector<int> split_preferences(size_t N, size_t M) {
  (void)N;
  // fewer targets than one 1024-target tile: the tensor-core builds' 512-target tiles
  // waste no more than variant 3's, then the CUDA-core model 0 on 512 and 256
  if (M < 1024) return {73, 75, 76, 3, 4};
  // fastest first: the tensor-core phase (pair model 3) in the builder-warp kernel on
  // source tiles of 1024, 512 and 256 (on the 512^2 -> 1024^2 y pass, one GB300: 90.8,
  // 94.6 and 99.0 ms, against 91.8, 98.5 and 110.7 ms for the same tiles with the operands
  // built between tile pairs, variants 58, 67 and 69; 768-source tiles, 71 at 97.0 ms,
  // are slower than 512 and their bound wider, so they never come first), then the
  // CUDA-core pair models 2, 1, 0 on ever smaller tiles
  return {73, 75, 76, 23, 13, 9, 27, 21, 16, 11, 3, 4};
}

#define HOLO_SPLIT_DISPATCH(V, CALL)                      \
  switch (V) {                                            \
    case 0: return CALL(256, 8, 1024, 0);                 \
    case 1: return CALL(128, 8, 1024, 0);                 \
    case 2: return CALL(256, 4, 1024, 0);                 \
    case 3: return CALL(128, 4, 512, 0);                  \
    case 4: return CALL(128, 2, 256, 0);                  \
    case 5: return CALL(256, 8, 512, 0);                  \
    case 6: return CALL(256, 8, 1024, 1);                 \
    case 7: return CALL(256, 8, 1024, 2);                 \
    case 8: return CALL(256, 8, 1024, 3);                 \
    case 9: return CALL(256, 4, 1024, 1);                 \
    case 10: return CALL(256, 8, 1024, 4);                \
    case 11: return CALL(256, 4, 512, 1);                 \
    case 12: return CALL(128, 4, 512, 1);                 \
    case 13: return CALL(256, 4, 1024, 1 | 16);           \
    case 14: return CALL(256, 8, 1024, 2 | 16);           \
    case 15: return CALL(256, 8, 1024, 3 | 16);           \
    case 16: return CALL(256, 4, 512, 1 | 16);            \
    case 17: return CALL(256, 4, 1024, 1 | 32);           \
    case 18: return CALL(256, 4, 1024, 0 | 32);           \
    case 19: return CALL(256, 8, 1024, 1 | 32);           \
    case 20: return CALL(256, 8, 1024, 2 | 32);           \
    case 21: return CALL(256, 4, 512, 1 | 32);            \
    case 22: return CALL(256, 4, 1024, 0 | 96);           \
    case 23: return CALL(256, 4, 1024, 1 | 96);           \
    case 24: return CALL(256, 4, 1024, 2 | 96);           \
    case 25: return CALL(256, 2, 1024, 1 | 96);           \
    case 26: return CALL(128, 4, 1024, 1 | 96);           \
    case 27: return CALL(256, 4, 512, 1 | 96);            \
    case 28: return CALL(256, 4, 512, 0 | 96);            \
    case 29: return CALL(128, 4, 512, 1 | 96);            \
    case 40: return CALL(128, 4, 768, 1 | 96);            \
    case 46: return CALL(128, 4, 256, 1 | 96);            \
    case 30: return CALL(512, 4, 1024, 1 | 96);           \
    case 31: return CALL(512, 4, 1024, 0 | 96 | 128);     \
    case 32: return CALL(512, 2, 1024, 0 | 96 | 128);     \
    default: return fail(HOLO_ERR_INVALID, "unknown split variant %d", V); \
  }

int launch_split(const SplitProblem &p, int variant, int grid, bool const_phase, bool mc,
                 int *err, cudaStream_t s) {
  if (is_tc(variant)) {
    if (!const_phase && !mc)
      return launch_split_tc(p, kVariants[variant].cs, kVariants[variant].poly,
                             kVariants[variant].sc, grid, err, s);
    variant = tc_fallback(variant);
  }
#define CALL(T, R, C, P) launch_variant<T, R, C, P>(p, grid, const_phase, mc, err, s)
  HOLO_SPLIT_DISPATCH(variant, CALL)
#undef CALL
}

int launch_split_batched(const SplitProblem *probs_dev, const WorkItem *items, int n_items,
                         int *queue, int variant, int grid, int *err, cudaStream_t s) {
  if (is_tc(variant))
    return launch_split_tc_batched(probs_dev, items, n_items, queue, kVariants[variant].cs,
                                   kVariants[variant].poly, kVariants[variant].sc, grid, err,
                                   s);
#define CALL(T, R, C, P) batched_variant<T, R, C, P>(probs_dev, items, n_items, queue, grid, err, s)
  HOLO_SPLIT_DISPATCH(variant, CALL)
#undef CALL
}

int split_occupancy(int variant, bool mc, int *ctas_per_sm) {
  if (is_tc(variant)) {
    if (!mc)
      return split_tc_occupancy(kVariants[variant].cs, kVariants[variant].poly,
                                kVariants[variant].sc, ctas_per_sm);
    variant = tc_fallback(variant);
  }
#define CALL(T, R, C, P) occupancy_variant<T, R, C, P>(mc, ctas_per_sm)
  HOLO_SPLIT_DISPATCH(variant, CALL)
#undef CALL
}

}  // namespace holo

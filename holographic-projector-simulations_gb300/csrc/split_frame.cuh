// split_frame.cuh -- per-tile-pair frame and float-float helpers shared by the
// split-precision kernels (kernel_split.cu: CUDA-core pair loop; kernel_tc.cu:
// tensor-core phase).  Included inside an anonymous namespace of holo.
#pragma once

struct __align__(16) Frame {
  double e[3];
  double r0;
  double b0;     // s k r0 reduced mod 2 pi
  double t0[3];  // target tile centre
  double s0[3];  // source tile centre
  float ef[3], e1[3], e2[3];
  float r0f;
  float ah[3], al[3];  // s k e as float-float (hi + lo)
  float b0h, b0l;      // b0 as float-float
};

// ---- float-float (double-single) helpers: error-free transformations --------
// (Knuth's TwoSum; the product error by FMA).  The _rn intrinsics keep the
// compiler from fusing or reassociating the steps that must round alone.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// S + E ~ (ah + al) . (th + tl) over 3 components, relative error ~2^-44.
__device__ __forceinline__ void dot3_ff(const float *ah, const float *al, const float *th,
                                        const float *tl, float &S, float &E) {
  float p[3], e[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    p[d] = __fmul_rn(ah[d], th[d]);
    e[d] = fmaf(ah[d], th[d], -p[d]);
    e[d] = fmaf(ah[d], tl[d], e[d]);
    e[d] = fmaf(al[d], th[d], e[d]);
  }
  float s1, t1, t2;
  two_sum(p[0], p[1], s1, t1);
  two_sum(s1, p[2], S, t2);
  E = __fadd_rn(__fadd_rn(t1, t2), __fadd_rn(__fadd_rn(e[0], e[1]), e[2]));
}

// (S + E) reduced mod 2 pi to about [-pi, pi] in float, |S| < 2^16: three-part
// Cody-Waite with C1 = 6.28125 (8 significant bits, so n C1 and S - n C1 are exact).
__device__ __forceinline__ float reduce_two_pi_ff(float S, float E) {
  const float n = __fsub_rn(__fadd_rn(__fmul_rn(S, 0.159154943f), 12582912.0f), 12582912.0f);
  float r = fmaf(-n, 6.28125f, S);
  r = fmaf(-n, 1.935307169e-3f, r);   // fl32(2 pi - C1)
  r = fmaf(-n, 1.025313168e-11f, r);  // fl32(2 pi - C1 - C2)
  return __fadd_rn(r, E);
}

__device__ __forceinline__ void build_frame(Frame *fr, const double *t0, const double *s0,
                                            double sk) {
  double D[3], r2 = 0.0;
  for (int d = 0; d < 3; ++d) {
    fr->t0[d] = t0[d];
    fr->s0[d] = s0[d];
    D[d] = t0[d] - s0[d];
    r2 = fma(D[d], D[d], r2);
  }
  const double r0 = sqrt(r2);
  const double inv = r0 > 0.0 ? 1.0 / r0 : 0.0;
  double e[3] = {D[0] * inv, D[1] * inv, D[2] * inv};
  if (r0 == 0.0) { e[0] = 0.0; e[1] = 0.0; e[2] = 1.0; }
  // e1: the coordinate axis least aligned with e, made orthogonal to e
  const double ax = fabs(e[0]), ay = fabs(e[1]), az = fabs(e[2]);
  double a[3] = {0.0, 0.0, 0.0};
  if (ax <= ay && ax <= az) a[0] = 1.0; else if (ay <= az) a[1] = 1.0; else a[2] = 1.0;
  const double ae = a[0] * e[0] + a[1] * e[1] + a[2] * e[2];
  double e1[3] = {a[0] - ae * e[0], a[1] - ae * e[1], a[2] - ae * e[2]};
  const double n1 = rsqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
  for (int d = 0; d < 3; ++d) e1[d] *= n1;
  const double e2[3] = {e[1] * e1[2] - e[2] * e1[1], e[2] * e1[0] - e[0] * e1[2],
                        e[0] * e1[1] - e[1] * e1[0]};
  for (int d = 0; d < 3; ++d) {
    fr->e[d] = e[d];
    fr->ef[d] = (float)e[d];
    fr->e1[d] = (float)e1[d];
    fr->e2[d] = (float)e2[d];
  }
  fr->r0 = r0;
  fr->r0f = (float)r0;
  fr->b0 = reduce_two_pi(sk * r0);
  for (int d = 0; d < 3; ++d) {
    const double a = sk * e[d];
    fr->ah[d] = (float)a;
    fr->al[d] = (float)(a - (double)fr->ah[d]);
  }
  fr->b0h = (float)fr->b0;
  fr->b0l = (float)(fr->b0 - (double)fr->b0h);
}

// sin and cos of theta on the FMA pipe: theta -> f = theta / 2 pi - rint(theta / 2 pi)
// in [-1/2, 1/2] turns, then sin(2 pi f) = f P(f^2) (degree 11) and
// cos(2 pi f) = Q(f^2) (degree 12), minimax fits made by gen_sincos_poly.py
// (Lawson's iteration on Chebyshev nodes); float32 Horner error <= 7.6e-7.
// Used for POLY of the R targets per thread so the XU pipe (MUFU sin/cos,
// 16 lanes/clk/SM) and the FMA pipe (128 lanes/clk/SM) share the work.
__device__ __forceinline__ void poly_sincos(float th, float *sn, float *cs) {
  const float t = th * 0.159154943f;
  const float n = (t + 12582912.0f) - 12582912.0f;  // round to nearest for |t| < 2^22
  const float f = t - n;
  const float f2 = f * f;
  float s = fmaf(-1.227126217e+01f, f2, 4.120539474e+01f);
  s = fmaf(s, f2, -7.658010101e+01f);
  s = fmaf(s, f2, 8.159618378e+01f);
  s = fmaf(s, f2, -4.134142303e+01f);
  s = fmaf(s, f2, 6.283182621e+00f);
  float c = fmaf(6.529610157e+00f, f2, -2.596831322e+01f);
  c = fmaf(c, f2, 6.016783142e+01f);
  c = fmaf(c, f2, -8.545016479e+01f);
  c = fmaf(c, f2, 6.493911743e+01f);
  c = fmaf(c, f2, -1.973920441e+01f);
  c = fmaf(c, f2, 1.0f);
  *sn = s * f;
  *cs = c;
}

// Both halves of a packed pair set to one compile-time constant.
__device__ __forceinline__ uint64_t splat2(float k) {
  const uint64_t b = __float_as_uint(k);
  return (b << 32) | b;
}

// sin and cos of a packed pair of angles reduced to half turns: th = pi (n + g),
// n = rint(th / pi), |g| <= 1/2.  sin(pi g) = g P(g^2) (degree 9) and cos(pi g) =
// Q(g^2) (degree 8), minimax fits on |g| <= 1/2 made by gen_sincos_poly.py (float32
// Horner error 2.0e-7 and 1.9e-7, against 7.5e-7 and 4.2e-7 for poly_sincos2); beyond
// |th| = pi the rounding of th / pi dominates, as for any FP32 reduction.  The (-1)^n
// that both share is returned as a sign mask (bit 31 of each half) for the caller to
// put on the amplitude: 14 packed FP32 instructions per two angles against 17 for
// poly_sincos2, plus two integer ones per half for the sign.  Measured on one GB300:
// the tensor-core kernel 1.6 % faster at 6 of 16 source pairs; in packed_pairs, where
// each of a thread's targets needs its own flip of the shared amplitudes, 1.1-1.3 %
// slower for 1024-source tiles (2.4 % faster for 256), so packed_pairs keeps poly_sincos2.
__device__ __forceinline__ void poly_sincos2_half(uint64_t th, uint64_t &sn, uint64_t &cs,
                                                  uint64_t &sign) {
  const uint64_t h = ptx::mul2(th, splat2(3.183098733e-01f));
  const uint64_t u = ptx::add2(h, splat2(12582912.0f));  // rint(h) in the low bits
  const uint64_t g = ptx::sub2(h, ptx::sub2(u, splat2(12582912.0f)));
  const uint64_t g2 = ptx::mul2(g, g);
  uint64_t s = ptx::fma2(splat2(7.722012699e-02f), g2, splat2(-5.980451703e-01f));
  s = ptx::fma2(s, g2, splat2(2.550031424e+00f));
  s = ptx::fma2(s, g2, splat2(-5.167706966e+00f));
  s = ptx::fma2(s, g2, splat2(3.141592503e+00f));
  uint64_t c = ptx::fma2(splat2(2.196968049e-01f), g2, splat2(-1.331880212e+00f));
  c = ptx::fma2(c, g2, splat2(4.058412075e+00f));
  c = ptx::fma2(c, g2, splat2(-4.934792995e+00f));
  c = ptx::fma2(c, g2, splat2(9.999999404e-01f));
  sn = ptx::mul2(s, g);
  cs = c;
  sign = (u << 31) & 0x8000000080000000ull;  // bit 0 of each half: n odd
}

// The same as poly_sincos2_half for angles given in half turns already, h = theta / pi
// (the tensor-core kernel scales the phase of its polynomial columns by 1 / pi in the
// operand build, so the first multiply goes), with a sine of degree 7 when SIN7 (float32
// Horner error 7.4e-7 on |g| <= 1/2, the size of MUFU sin.approx's own error; fitted by
// gen_sincos_poly.py) instead of 9.  SIN7 saves one more packed FMA: 12 packed FP32
// instructions per two angles against 14.
template <bool SIN7>
__device__ __forceinline__ void poly_sincos2_ht(uint64_t h, uint64_t &sn, uint64_t &cs,
                                                uint64_t &sign) {
  const uint64_t u = ptx::add2(h, splat2(12582912.0f));  // rint(h) in the low bits
  const uint64_t g = ptx::sub2(h, ptx::sub2(u, splat2(12582912.0f)));
  const uint64_t g2 = ptx::mul2(g, g);
  uint64_t s;
  if (SIN7) {
    s = ptx::fma2(splat2(-5.546361804e-01f), g2, splat2(2.541898966e+00f));
    s = ptx::fma2(s, g2, splat2(-5.167142868e+00f));
    s = ptx::fma2(s, g2, splat2(3.141582012e+00f));
  } else {
    s = ptx::fma2(splat2(7.722012699e-02f), g2, splat2(-5.980451703e-01f));
    s = ptx::fma2(s, g2, splat2(2.550031424e+00f));
    s = ptx::fma2(s, g2, splat2(-5.167706966e+00f));
    s = ptx::fma2(s, g2, splat2(3.141592503e+00f));
  }
  uint64_t c = ptx::fma2(splat2(2.196968049e-01f), g2, splat2(-1.331880212e+00f));
  c = ptx::fma2(c, g2, splat2(4.058412075e+00f));
  c = ptx::fma2(c, g2, splat2(-4.934792995e+00f));
  c = ptx::fma2(c, g2, splat2(9.999999404e-01f));
  sn = ptx::mul2(s, g);
  cs = c;
  sign = (u << 31) & 0x8000000080000000ull;  // bit 0 of each half: n odd
}

// poly_sincos on a packed pair of angles (fma.rn.f32x2 and friends): the same
// polynomial and operation order as poly_sincos, two angles per instruction.
__device__ __forceinline__ void poly_sincos2(uint64_t th, uint64_t &sn, uint64_t &cs) {
  const uint64_t t = ptx::mul2(th, splat2(0.159154943f));
  const uint64_t n = ptx::sub2(ptx::add2(t, splat2(12582912.0f)), splat2(12582912.0f));
  const uint64_t f = ptx::sub2(t, n);
  const uint64_t f2 = ptx::mul2(f, f);
  uint64_t s = ptx::fma2(splat2(-1.227126217e+01f), f2, splat2(4.120539474e+01f));
  s = ptx::fma2(s, f2, splat2(-7.658010101e+01f));
  s = ptx::fma2(s, f2, splat2(8.159618378e+01f));
  s = ptx::fma2(s, f2, splat2(-4.134142303e+01f));
  s = ptx::fma2(s, f2, splat2(6.283182621e+00f));
  uint64_t c = ptx::fma2(splat2(6.529610157e+00f), f2, splat2(-2.596831322e+01f));
  c = ptx::fma2(c, f2, splat2(6.016783142e+01f));
  c = ptx::fma2(c, f2, splat2(-8.545016479e+01f));
  c = ptx::fma2(c, f2, splat2(6.493911743e+01f));
  c = ptx::fma2(c, f2, splat2(-1.973920441e+01f));
  c = ptx::fma2(c, f2, splat2(1.0f));
  sn = ptx::mul2(s, f);
  cs = c;
}

// Pair loop of pair model 2 on packed FP32 pairs: two consecutive sources per
// instruction for each of the R targets of this thread; the first NP targets
// take sin/cos from the FMA-pipe polynomial.  Per-target inputs: frame
// coordinates Tx, Ty, T2 = Tx^2 + Ty^2, Iq = |kap2| / Qt, Kq = |kap2| / Qt^2;
// outputs the FP32 tile sums (re, im) per target (before the 1 / Qt factor).
template <int R, int NP, bool CONST>
__device__ __forceinline__ void packed_pairs(const float4 *pa, const float4 *pb, const float4 *pc,
                                             int npair, const float *Tx, const float *Ty,
                                             const float *T2, const float *Iq, const float *Kq,
                                             float *re, float *im) {
  uint64_t tx2[R], ty2[R], t22[R], iq2[R], kq2[R], re2[R], im2[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    tx2[r] = ptx::pack2(Tx[r], Tx[r]);
    ty2[r] = ptx::pack2(Ty[r], Ty[r]);
    t22[r] = ptx::pack2(T2[r], T2[r]);
    iq2[r] = ptx::pack2(Iq[r], Iq[r]);
    kq2[r] = ptx::pack2(Kq[r], Kq[r]);
    re2[r] = 0ull;
    im2[r] = 0ull;
  }
#pragma unroll 2
  for (int p = 0; p < npair; ++p) {
    const float4 c4 = pc[p];
    if (CONST) {
#pragma unroll
      for (int r = 0; r < R; ++r) re[r] += c4.x + c4.y;
    } else {
      const float4 a4 = pa[p], b4 = pb[p];
      const uint64_t qx = ptx::pack2(a4.x, a4.y), qy = ptx::pack2(a4.z, a4.w);
      const uint64_t qz = ptx::pack2(b4.x, b4.y), qw = ptx::pack2(b4.z, b4.w);
      const uint64_t am = ptx::pack2(c4.x, c4.y), s2 = ptx::pack2(c4.z, c4.w);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const uint64_t c = ptx::fma2(tx2[r], qx, ptx::fma2(ty2[r], qy, ptx::add2(t22[r], s2)));
        const uint64_t iq = ptx::fma2(qz, kq2[r], iq2[r]);  // |kap2| / q, first order
        const uint64_t th = ptx::fma2(c, iq, qw);           // sign * theta
        uint64_t sn, cs;
        if (r < NP) {
          poly_sincos2(th, sn, cs);  // FMA pipe
        } else {
          float t0, t1;
          ptx::unpack2(th, t0, t1);
          sn = ptx::pack2(ptx::sin_approx(t0), ptx::sin_approx(t1));  // XU pipe
          cs = ptx::pack2(ptx::cos_approx(t0), ptx::cos_approx(t1));
        }
        re2[r] = ptx::fma2(am, cs, re2[r]);
        im2[r] = ptx::fma2(am, sn, im2[r]);
      }
    }
  }
  if (!CONST) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      float a, b;
      ptx::unpack2(re2[r], a, b);
      re[r] = a + b;
      ptx::unpack2(im2[r], a, b);
      im[r] = a + b;
    }
  }
}


// kernel_tc.cu -- split-precision Huygens superposition with the per-pair phase
// on the 5th-generation tensor cores (HOLO_SPLIT32, pair model 3).
//
// Same frame decomposition as kernel_split.cu (cuda/superposition.cu:35-51,
// 59-154 restated per (target tile, source tile) pair) and the same first-order
// 1/q model as pair model 2, but the phase of every pair is one inner product
// of per-target and per-source features in the tile-pair frame:
//   theta'(t, s) = sign A_s + (S2 - 2 T.S) (Iq + Kq Ps) + Kq T2 Ps   (+ Iq T2 per target)
//                = sum_k f_k(t) g_k(s) + (1, 1, 1) . (a0, a1, a2)_s,
//   f = [Iq, -2 Iq Tx, -2 Iq Ty, Kq T2, Kq, -2 Kq Tx, -2 Kq Ty, 0],
//   g = [S2, Sx, Sy, Ps, Ps S2, Ps Sx, Ps Sy, 0]     (Iq = |kap2| / Qt, Kq = |kap2| / Qt^2,
//                                                    a0 + a1 + a2 = sign A in TF32 parts)
// with Iq T2 moved into the per-target rotation.  A tile of 128 targets x 256
// sources of theta' is one tcgen05.mma of kind::tf32 (M = 128, N = 256, K = 8)
// per product: the geometric features in three TF32 products (hi hi + hi lo +
// lo hi, the 3xTF32 split: ~2^-21 relative), and sign A split three ways into
// TF32 parts against constant ones (exact products) in a second K block.  The
// accumulator lives in tensor memory (two buffers of 256 columns); 16 consumer
// warps read it with tcgen05.ld (warp w: TMEM lanes 32 (w % 4).., columns
// 64 (w / 4)..), take sin/cos (MUFU, or the FMA-pipe polynomial for NPP0 /
// NPP1 of the 8 source pairs of even / odd 16-column chunks) and accumulate
// a' e^{i theta'} on packed f32x2 pairs (SC: the MUFU pairs in scalar FP32).
// One more warp allocates the tensor memory and issues the MMAs (one thread),
// tracked by mbarriers: full[b] (tcgen05.commit) and free[b] (16 consumer
// arrivals).  A last warp builds the next tile pair's FP64 frame while the
// pairs of this one are summed: FP64 is slow on this part (a frame is ~6000
// cycles of dependent FP64 work), so a frame built in the MMA warp held back
// the first MMA of every tile.  Per pair on the CUDA cores: 3 FP32-pipe ops +
// 2 MUFU ops.  Per tile pair the consumers build the operands (each thread its
// target row and source rows in one straight-line block), then carry the previous
// tile's sums (float-float, per target) while the first MMAs run.
//
// Tiles: 512 targets per CTA (4 blocks of 128), NBLK blocks of 256 sources per
// tile (1024, 512 or 256 sources; 768 in blocks of 192 with 24 consumer warps);
// one CTA per SM (up to 217 KB of shared memory).  Shorter source tiles narrow
// the tile pairs, which tightens the error bound of the first-order model for
// close or wide point sets, at more per-tile work per pair.  Every wait is bounded:
// after a timeout the kernel raises the device error word and skips the rest
// of its work, then waits (bounded) for the MMAs it issued and frees the
// tensor memory.
#include <type_traits>

#include "internal.cuh"
#include "ptx.cuh"

namespace holo {
namespace {

#include "split_frame.cuh"

constexpr int kTcTT = 512;                    // targets per CTA (4 blocks of 128)
constexpr int kTcM = 128, kTcK = 8;
constexpr int kTcCols = 512;                  // TMEM columns allocated: two accumulator buffers
constexpr uint32_t kTcLbo = 128, kTcSbo = 256;  // operand layout (bytes), see tc_off

// Shape of one build: CG column groups of consumer warps per TMEM lane group (4 lane
// groups of 32 targets), NB sources per MMA block (TMEM columns per buffer), CS = NBLK NB
// sources per tile.  CG = 4: 16 consumer warps, NB 256; CG = 6: 24 warps, NB 192.
template <int CG, int NBLK>
struct TcShape {
  static_assert(CG == 4 || CG == 6, "tensor-core split kernel: 4 or 6 column groups");
  static_assert(NBLK == 1 || NBLK == 2 || NBLK == 4, "tensor-core split kernel: 1, 2 or 4 blocks");
  static constexpr int NB = CG == 4 ? 256 : 192;
  static constexpr int CS = NBLK * NB;
  static constexpr int Consumers = 4 * CG;        // consumer warps
  static constexpr int Threads = 32 * (Consumers + 2);  // + the MMA warp + the frame warp
  static constexpr int Cols = NB / CG;            // columns per consumer warp per block
  static constexpr int Chunks = Cols / 16;        // 16-column loads per block
};

// Float offset of element (row r, feature k) of a K-major tf32 operand with K = 8:
// core matrices of 8 rows x 4 features (16 B rows, 128 B), the two along K 128 B
// apart (LBO), 8-row groups 256 B apart (SBO).  Rows of one 128- or 256-row block
// are contiguous, so block b starts at row 128 b / 256 b.
__host__ __device__ __forceinline__ int tc_off(int r, int k) {
  return (r >> 3) * 64 + (k >> 2) * 32 + (r & 7) * 4 + (k & 3);
}

template <int CG, int NBLK>
struct TcSmem {
  static constexpr int kTcCS = TcShape<CG, NBLK>::CS;
  static constexpr size_t raw_geo = 0;                                 // float [CS*6]
  static constexpr size_t raw_apf = raw_geo + kTcCS * 6 * 4;           // float2 [CS]
  static constexpr size_t opb_hi = raw_apf + kTcCS * 8;                // float [CS*8]
  static constexpr size_t opb_lo = opb_hi + kTcCS * kTcK * 4;          // float [CS*8]
  static constexpr size_t opb_a = opb_lo + kTcCS * kTcK * 4;           // float [CS*8]: A parts
  static constexpr size_t opa_hi = opb_a + kTcCS * kTcK * 4;           // float [TT*8]
  static constexpr size_t opa_lo = opa_hi + kTcTT * kTcK * 4;          // float [TT*8]
  static constexpr size_t opa_one = opa_lo + kTcTT * kTcK * 4;         // float [128*8]: (1,1,1,0..)
  static constexpr size_t amp = opa_one + kTcM * kTcK * 4;             // float [2][CS]
  // partial sums, [PB][CG][TT] float2: a tile's are carried during the next tile, and
  // with fewer than three source blocks per tile a consumer can write the next
  // tile's before a slower one has carried them, so those builds keep two buffers
  static constexpr int PB = NBLK >= 3 ? 1 : 2;
  static constexpr size_t part = amp + 2 * kTcCS * 4;
  static constexpr size_t acc = part + PB * CG * kTcTT * 8;            // float4 [TT]
  static constexpr size_t tph = acc + kTcTT * 16;                      // float [2][TT]
  static constexpr size_t tsc = tph + 2 * kTcTT * 4;                   // float [2][TT]
  static constexpr size_t tgeo = tsc + 2 * kTcTT * 4;                  // float [6][TT]
  static constexpr size_t frame = tgeo + 6 * kTcTT * 4;                // Frame [2]
  static constexpr size_t bars = (frame + 2 * sizeof(Frame) + 15) / 16 * 16;  // uint64 [6]
  static constexpr size_t misc = bars + 6 * 8;                         // uint32 taddr, abort
  static constexpr size_t bytes = misc + 16;
};
template <int CG, int NBLK>
constexpr bool tc_layout_ok() {
  using L = TcSmem<CG, NBLK>;
  return L::bytes <= 227 * 1024 && L::raw_apf % 16 == 0 && L::opb_hi % 128 == 0 &&
         L::opb_lo % 128 == 0 && L::opb_a % 128 == 0 && L::opa_hi % 128 == 0 &&
         L::opa_lo % 128 == 0 && L::opa_one % 128 == 0 && L::amp % 16 == 0 && L::acc % 16 == 0;
}
static_assert(tc_layout_ok<4, 4>() && tc_layout_ok<4, 2>() && tc_layout_ok<4, 1>() &&
                  tc_layout_ok<6, 4>(),
              "tensor-core split kernel: shared memory size and operand alignment");

__device__ __forceinline__ void split_range_tc(int n, int splits, int s, int *b, int *e) {
  *b = (int)(((long long)n * s) / splits);
  *e = (int)(((long long)n * (s + 1)) / splits);
}

// Row r of an operand pair (hi, lo): the 8 features split into TF32 high parts and
// TF32 remainders, written as four 16-byte stores (features 0-3 and 4-7 of a row
// are contiguous; eight consecutive rows fill 128 bytes, so a warp's stores are
// free of bank conflicts).
__device__ __forceinline__ void store_row_split(float *hi, float *lo, int r, const float *x) {
  float h[kTcK], l[kTcK];
#pragma unroll
  for (int k = 0; k < kTcK; ++k) {
    h[k] = ptx::to_tf32_int(x[k]);
    l[k] = ptx::to_tf32_int(__fsub_rn(x[k], h[k]));
  }
  *reinterpret_cast<float4 *>(hi + tc_off(r, 0)) = make_float4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<float4 *>(hi + tc_off(r, 4)) = make_float4(h[4], h[5], h[6], h[7]);
  *reinterpret_cast<float4 *>(lo + tc_off(r, 0)) = make_float4(l[0], l[1], l[2], l[3]);
  *reinterpret_cast<float4 *>(lo + tc_off(r, 4)) = make_float4(l[4], l[5], l[6], l[7]);
}

// Bounded wait that gives up at once when the CTA has aborted; sleep_ns > 0: poll with
// that much sleep in between.
__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                        int *err, unsigned sleep_ns = 0) {
  if (*abort_flag) return false;
  if (sleep_ns ? ptx::mbar_wait_bounded_sleep(bar, parity, kWaitCycles, sleep_ns)
               : ptx::mbar_wait_bounded(bar, parity, kWaitCycles))
    return true;
  *abort_flag = 1;
  atomicExch(err, kDevErrTimeout);
  return false;
}

// Build flags: kTcScalar -- the MUFU pairs accumulated in scalar FP32 (no packing);
// kTcHalfUnroll -- the 16-column chunks of a block in a loop of chunk pairs instead
// of fully unrolled (half the pair-loop code); kTcRcp -- the target row's 1/Qt and
// 1/Qt^2 from one correctly rounded reciprocal instead of two divisions; kTcPrefetch --
// during a block's last chunk, if the next block's accumulator is already complete
// (non-blocking barrier test), its first chunk's TMEM load is issued then instead of
// after the block (the latency of that load otherwise opens every block);
// kTcSleepMma / kTcSleepUse -- the MMA warp's waits for free buffers / the consumers'
// waits for complete blocks poll with a short sleep in between (a spinning warp takes
// issue slots from the four consumer warps of its SM sub-partition); kTcHalfTurns --
// the source rows of the polynomial columns are scaled by 1 / pi in the operand build,
// so the tensor cores deliver their phases in half turns and the polynomial needs no
// multiply; kTcSin7 -- with kTcHalfTurns, a sine of degree 7 instead of 9.  Together
// they take the FMA-pipe sin/cos from 16 to 14 lane operations per source, so more
// source pairs can leave the XU pipe; kTcBuilders -- the builder-warp kernel
// (k_split_tc_bw: operands, carries and results by warps of their own; it takes
// kTcSleepMma, kTcRcp and the sin/cos flags); kTcBuilders2 -- with kTcBuilders and 16
// consumer warps, two builder warps instead of four (96 registers a thread instead of 80).
constexpr int kTcScalar = 1, kTcHalfUnroll = 4, kTcRcp = 8, kTcPrefetch = 16, kTcSleepMma = 32,
              kTcSleepUse = 64, kTcHalfTurns = 128, kTcSin7 = 256, kTcBuilders = 512,
              kTcBuilders2 = 1024;

// The FP32 part of a tile pair's frame, as the operand builds read it.
struct TcBasis {
  float e1[3], e2[3], ef[3], ah[3], al[3];
  float r0f, ir0, b0h, b0l;
};
__device__ __forceinline__ TcBasis tc_basis(const Frame *fr) {
  TcBasis B;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    B.e1[d] = fr->e1[d];
    B.e2[d] = fr->e2[d];
    B.ef[d] = fr->ef[d];
    B.ah[d] = fr->ah[d];
    B.al[d] = fr->al[d];
  }
  B.r0f = fr->r0f;
  B.ir0 = fr->r0f > 0.f ? 1.f / fr->r0f : 0.f;
  B.b0h = fr->b0h;
  B.b0l = fr->b0l;
  return B;
}

// Target row of the phase operand: features f (see the file header), the target's
// rotation (its phase at the source tile centre plus the Iq T2 term) and 1 / Qt.
// th, tl: the target's offset from its tile centre as float-float.
template <int FL>
__device__ __forceinline__ void tc_target_row(const TcBasis &B, const float th[3],
                                              const float tl[3], float ak, float iak, float sgn,
                                              float f[kTcK], float &tph, float &tsc) {
  float S, E, S2, E2;
  dot3_ff(B.ah, B.al, th, tl, S, E);
  two_sum(S, B.b0h, S2, E2);
  const float Bt = reduce_two_pi_ff(S2, __fadd_rn(__fadd_rn(E, E2), B.b0l));
  const float Tx = fmaf(B.e1[0], th[0], fmaf(B.e1[1], th[1], B.e1[2] * th[2]));
  const float Ty = fmaf(B.e2[0], th[0], fmaf(B.e2[1], th[1], B.e2[2] * th[2]));
  const float Qt = B.r0f + fmaf(B.ef[0], th[0], fmaf(B.ef[1], th[1], B.ef[2] * th[2]));
  const float T2 = fmaf(Tx, Tx, Ty * Ty);
  float Iq, Kq;
  if (FL & kTcRcp) {
    const float rq = __frcp_rn(Qt);
    Iq = ak * rq;
    Kq = Iq * rq;
  } else {
    Iq = ak / Qt;
    Kq = Iq / Qt;
  }
  f[0] = Iq; f[1] = -2.f * Iq * Tx; f[2] = -2.f * Iq * Ty; f[3] = Kq * T2;
  f[4] = Kq; f[5] = -2.f * Kq * Tx; f[6] = -2.f * Kq * Ty; f[7] = 0.f;
  tph = Bt + sgn * Iq * T2;  // the target's rotation, incl. the Iq T2 term
  tsc = Iq * iak;            // 1 / Qt
}

// Source row i of its tile: features g, the sign A parts a3 (a0 + a1 + a2 = sign A, each
// a TF32 number) and the amplitude a' = a (1 + Ps / r0).  sh, sl: the source's offset
// from its tile centre as float-float; pa: (phase, amplitude).  With kTcHalfTurns the
// rows of the polynomial columns (source pair pp < NPP0 / NPP1 of an even / odd
// 16-column chunk of a consumer's COLS columns of a block of NB) are scaled by 1 / pi.
template <int FL, int NB, int COLS, int NPP0, int NPP1>
__device__ __forceinline__ void tc_source_row(const TcBasis &B, const float sh[3],
                                              const float sl[3], float2 pa, float sgn, int i,
                                              float g[kTcK], float a3[3], float &am) {
  float S, E, S2, E2;
  dot3_ff(B.ah, B.al, sh, sl, S, E);
  two_sum(pa.x, -S, S2, E2);
  const float sA = sgn * reduce_two_pi_ff(S2, __fsub_rn(E2, E));
  const float Sx = fmaf(B.e1[0], sh[0], fmaf(B.e1[1], sh[1], B.e1[2] * sh[2]));
  const float Sy = fmaf(B.e2[0], sh[0], fmaf(B.e2[1], sh[1], B.e2[2] * sh[2]));
  const float Ps = fmaf(B.ef[0], sh[0], fmaf(B.ef[1], sh[1], B.ef[2] * sh[2]));
  const float s2 = fmaf(Sx, Sx, Sy * Sy);
  g[0] = s2; g[1] = Sx; g[2] = Sy; g[3] = Ps;
  g[4] = Ps * s2; g[5] = Ps * Sx; g[6] = Ps * Sy; g[7] = 0.f;
  float sAh = sA;
  if (FL & kTcHalfTurns) {
    // column of row i in its block, and whether the pair loop takes its sin/cos
    // from the polynomial (source pair pp < npp of its 16-column chunk)
    const int c = (i % NB) % COLS, pp = (c % 16) / 2;
    if (pp < (((c / 16) & 1) ? NPP1 : NPP0)) {
      constexpr float kInvPi = 0.318309886f;
#pragma unroll
      for (int k = 0; k < kTcK; ++k) g[k] *= kInvPi;
      sAh = sA * kInvPi;
    }
  }
  // sign A = a0 + a1 + a2 exactly, each part a TF32 number
  a3[0] = ptx::to_tf32_int(sAh);
  const float r1 = __fsub_rn(sAh, a3[0]);
  a3[1] = ptx::to_tf32_int(r1);
  a3[2] = ptx::to_tf32_int(__fsub_rn(r1, a3[1]));
  am = pa.y * fmaf(Ps, B.ir0, 1.f);
}

// 16 columns of one accumulator row: the phases th of 8 source pairs, their amplitudes av;
// the first NPP pairs take sin/cos from the FMA-pipe polynomial (their amplitude's sign
// carries the reduction's (-1)^n), the others from MUFU.  re2 / im2: packed f32x2 sums;
// res / ims: with kTcScalar the MUFU pairs' sums, unpacked.
template <int FL, int NPP>
__device__ __forceinline__ void tc_pairs16(const uint32_t (&th)[16], const float (&av)[16],
                                           uint64_t &re2, uint64_t &im2, float (&res)[2],
                                           float (&ims)[2]) {
#pragma unroll
  for (int pp = 0; pp < 8; ++pp) {
    const float t0 = __uint_as_float(th[2 * pp]);
    const float t1 = __uint_as_float(th[2 * pp + 1]);
    if ((FL & kTcScalar) && pp >= NPP) {
      // XU pipe, scalar accumulation (no packing of the MUFU results)
      res[0] = fmaf(av[2 * pp], ptx::cos_approx(t0), res[0]);
      ims[0] = fmaf(av[2 * pp], ptx::sin_approx(t0), ims[0]);
      res[1] = fmaf(av[2 * pp + 1], ptx::cos_approx(t1), res[1]);
      ims[1] = fmaf(av[2 * pp + 1], ptx::sin_approx(t1), ims[1]);
      continue;
    }
    const uint64_t t2 = ptx::pack2(t0, t1);
    uint64_t am = ptx::pack2(av[2 * pp], av[2 * pp + 1]);
    uint64_t sn, cs;
    if (pp < NPP) {
      uint64_t sign;
      if (FL & kTcHalfTurns)
        poly_sincos2_ht<(FL & kTcSin7) != 0>(t2, sn, cs, sign);  // FMA pipe
      else
        poly_sincos2_half(t2, sn, cs, sign);  // FMA pipe
      am ^= sign;
    } else {
      sn = ptx::pack2(ptx::sin_approx(t0), ptx::sin_approx(t1));  // XU pipe
      cs = ptx::pack2(ptx::cos_approx(t0), ptx::cos_approx(t1));
    }
    re2 = ptx::fma2(am, cs, re2);
    im2 = ptx::fma2(am, sn, im2);
  }
}

// BATCHED: work items (problem, target tile, source range, split) come from a
// device queue (atomic counter) and each names its own problem descriptor;
// otherwise item i of problem P0 is target tile i / splits, split i % splits.
template <int CG, int NBLK, int NPP0, int NPP1, int FL, bool BATCHED>
__global__ void __launch_bounds__(TcShape<CG, NBLK>::Threads, 1)
    k_split_tc(const SplitProblem P0, const SplitProblem *__restrict__ probs,
               const WorkItem *__restrict__ items, int n_items, int *queue, int *err) {
  extern __shared__ __align__(128) unsigned char smem[];
  using L = TcSmem<CG, NBLK>;
  using S = TcShape<CG, NBLK>;
  constexpr int kTcCS = S::CS, kTcN = S::NB, kTcConsumers = S::Consumers;
  constexpr int kTcThreads = S::Threads;
  float *raw_geo = reinterpret_cast<float *>(smem + L::raw_geo);
  float2 *raw_apf = reinterpret_cast<float2 *>(smem + L::raw_apf);
  float *opb_hi = reinterpret_cast<float *>(smem + L::opb_hi);
  float *opb_lo = reinterpret_cast<float *>(smem + L::opb_lo);
  float *opb_a = reinterpret_cast<float *>(smem + L::opb_a);
  float *opa_hi = reinterpret_cast<float *>(smem + L::opa_hi);
  float *opa_lo = reinterpret_cast<float *>(smem + L::opa_lo);
  float *opa_one = reinterpret_cast<float *>(smem + L::opa_one);
  float *amp = reinterpret_cast<float *>(smem + L::amp);
  float2 *part = reinterpret_cast<float2 *>(smem + L::part);
  // per target, the running sum of the tile sums as float-float pairs
  // (re hi, re lo, im hi, im lo): FP64 runs at a small fraction of the FP32 rate here
  float4 *acc = reinterpret_cast<float4 *>(smem + L::acc);
  float *tph = reinterpret_cast<float *>(smem + L::tph);
  float *tsc = reinterpret_cast<float *>(smem + L::tsc);
  float *tgeo = reinterpret_cast<float *>(smem + L::tgeo);  // this item's target records
  Frame *frames = reinterpret_cast<Frame *>(smem + L::frame);  // tile j in frames[j & 1]
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::bars);
  uint64_t *bar_tma = bars, *full = bars + 1, *freeb = bars + 3, *frame_ready = bars + 5;
  uint32_t *taddr_slot = reinterpret_cast<uint32_t *>(smem + L::misc);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + L::misc + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool consumer = warp < kTcConsumers;
  const bool producer = warp == kTcConsumers;     // TMEM owner, MMA issue
  const bool framer = warp == kTcConsumers + 1;   // next tile pair's frame
  constexpr int NC = kTcConsumers * 32;  // consumer threads

  if (tid == 0) {
    ptx::mbar_init(bar_tma, 1);
    ptx::mbar_init(&full[0], 1);
    ptx::mbar_init(&full[1], 1);
    ptx::mbar_init(&freeb[0], kTcConsumers);
    ptx::mbar_init(&freeb[1], kTcConsumers);
    ptx::mbar_init(frame_ready, 1);
    *abort_flag = 0;
    ptx::fence_barrier_init();
  }
  // constant operand of the phase term: every row (1, 1, 1, 0, ..)
  for (int i = tid; i < kTcM * kTcK; i += kTcThreads)
    opa_one[tc_off(i / kTcK, i % kTcK)] = (i % kTcK) < 3 ? 1.f : 0.f;
  if (producer) ptx::tmem_alloc(taddr_slot, kTcCols);
  ptx::fence_proxy_async_smem();
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tbase = *taddr_slot;

  constexpr uint32_t idesc = ptx::tc_idesc_tf32(kTcM, kTcN);
  uint32_t par_tma = 0, n_frames = 0;
  // producer: MMA groups issued per TMEM buffer; consumers: completions consumed
  uint32_t uses[2] = {0u, 0u};
  __shared__ int s_item;

  for (int it = 0;; ++it) {
    int item;
    if (BATCHED) {
      if (tid == 0) s_item = atomicAdd(queue, 1);
      __syncthreads();
      item = s_item;
      __syncthreads();  // s_item is rewritten for the next item
    } else {
      item = blockIdx.x + it * gridDim.x;
    }
    if (item >= n_items) break;
    const SplitProblem &P = BATCHED ? probs[items[item].problem] : P0;
    int tt, split, sb, se;
    if (BATCHED) {
      const WorkItem w = items[item];
      tt = w.ttile;
      split = w.split;
      sb = w.s_begin;
      se = w.s_end;
    } else {
      tt = item / P.splits;
      split = item % P.splits;
      split_range_tc(P.n_stiles, P.splits, split, &sb, &se);
    }
    const double sk = P.sk;
    const float kap2 = (float)(0.5 * sk), ak = fabsf(kap2), iak = 1.f / fabsf(kap2);
    const float sgn = kap2 < 0.f ? -1.f : 1.f;
    auto issue = [&](int j) {
      ptx::mbar_arrive_expect_tx(bar_tma, kTcCS * (6 * sizeof(float) + sizeof(float2)));
      ptx::bulk_g2s(raw_geo, P.geo_s + (size_t)j * kTcCS * 6, kTcCS * 6 * sizeof(float), bar_tma);
      ptx::bulk_g2s(raw_apf, P.apf_s + (size_t)j * kTcCS, kTcCS * sizeof(float2), bar_tma);
    };
    // per target: sum the column groups of tile jj, scale, rotate, carry (float-float);
    // run by consumer thread t during the next tile, after its operand build, so
    // that it fills the wait for that tile's first MMA block
    auto carry = [&](int jj) {
      const int t = tid;
      float sx = 0.f, sy = 0.f;
#pragma unroll
      for (int c = 0; c < CG; ++c) {
        const float2 v = part[((jj & 1) % L::PB) * CG * kTcTT + c * kTcTT + t];
        sx += v.x;
        sy += v.y;
      }
      const float sc = tsc[(jj & 1) * kTcTT + t];
      const float re = sx * sc;
      const float im = sgn * sy * sc;
      float sr, cr;
      __sincosf(tph[(jj & 1) * kTcTT + t], &sr, &cr);
      float4 a = acc[t];
      float h, e;
      two_sum(a.x, fmaf(re, cr, -im * sr), h, e);  // h + e: the exact sum
      a.x = h;
      a.y = __fadd_rn(a.y, e);
      two_sum(a.z, fmaf(re, sr, im * cr), h, e);
      a.z = h;
      a.w = __fadd_rn(a.w, e);
      acc[t] = a;
    };
    for (int t = tid; t < kTcTT; t += kTcThreads) {
      acc[t] = make_float4(0.f, 0.f, 0.f, 0.f);
      const int ti = tt * kTcTT + t;
#pragma unroll
      for (int k = 0; k < 6; ++k) tgeo[k * kTcTT + t] = ti < P.M ? P.geo_t[6 * (size_t)ti + k] : 0.f;
    }
    if (tid == 0 && sb < se && !*abort_flag) issue(sb);

    for (int j = sb; j < se; ++j) {
      Frame *fr = frames + (j & 1);
      // the first tile's frame here; the next ones by the frame warp during the
      // previous tile's pair work
      if (framer && lane == 0 && j == sb) {
        build_frame(fr, P.tiles_t + 6 * (size_t)tt, P.tiles_s + 6 * (size_t)j, sk);
        ptx::mbar_arrive(frame_ready);
      }
      // With kOverlapTiles there is no block-wide barrier here after an item's first
      // tile: consumers done with the previous tile build this one's operands while
      // slower ones finish it.  What the barrier orders is then ordered per consumer:
      // the staged records by the bulk copy's barrier, the frame by frame_ready, the
      // amplitudes by their second buffer; the operand tiles are read only by MMAs of
      // the previous tile, all complete once this consumer saw its last block, and
      // each thread writes and carries only its own target's rotation.  Measured on
      // one GB300 (each build against itself, two runs, 0.02 % apart): the overlap
      // is 0.8 % faster for single problems with 1024- and 256-source tiles, 0.85 %
      // slower with 512-source tiles, and 1.25 % faster for a batch of 64 uneven
      // problems than a work queue that keeps the barrier for its 2-block builds.
      constexpr bool kOverlapTiles = BATCHED || NBLK != 2;
      if (j == sb || !kOverlapTiles) {
        tc_wait(bar_tma, par_tma, abort_flag, err);
        __syncthreads();  // frame and staged records visible (and, first tile, the rest)
      } else if (consumer) {
        tc_wait(bar_tma, par_tma, abort_flag, err);
      }
      par_tma ^= 1u;
      if (kOverlapTiles && consumer) tc_wait(frame_ready, n_frames & 1u, abort_flag, err);
      ++n_frames;

      // ---- operands of this tile pair (consumer threads) ----
      if (consumer && !*abort_flag) {
        const TcBasis B = tc_basis(fr);
        // the target row and the source rows of this thread: all computed, then all
        // stored, in one straight-line block so that their dependent chains interleave
        // (with 512 consumers and 512 targets, and source tiles a multiple of 512,
        // both guards below are compile-time true).  Source records past N are
        // staged as zeros (offsets, phase and amplitude), from which the row comes
        // out all zeros, as it must.
        constexpr bool kAllTargets = NC <= kTcTT;  // every consumer thread owns a target
        const bool has_t = kAllTargets || tid < kTcTT;
        float f[kTcK], tph_v = 0.f, tsc_v = 0.f;
        if (has_t) {
          const int t = tid;
          const float th[3] = {tgeo[t], tgeo[kTcTT + t], tgeo[2 * kTcTT + t]};
          const float tl[3] = {tgeo[3 * kTcTT + t], tgeo[4 * kTcTT + t], tgeo[5 * kTcTT + t]};
          tc_target_row<FL>(B, th, tl, ak, iak, sgn, f, tph_v, tsc_v);
        }
        constexpr int R = (kTcCS + NC - 1) / NC;
        static_assert(kTcCS % NC == 0 || NC % kTcCS == 0, "source rows per consumer thread");
        float g[R][kTcK], a3[R][3], am[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int i = tid + r * NC;
#pragma unroll
          for (int k = 0; k < kTcK; ++k) g[r][k] = 0.f;
          a3[r][0] = a3[r][1] = a3[r][2] = 0.f;
          am[r] = 0.f;
          if (kTcCS >= NC || i < kTcCS) {
            const float *q = raw_geo + 6 * i;
            const float sh[3] = {q[0], q[1], q[2]}, sl[3] = {q[3], q[4], q[5]};
            tc_source_row<FL, kTcN, S::Cols, NPP0, NPP1>(B, sh, sl, raw_apf[i], sgn, i, g[r],
                                                         a3[r], am[r]);
          }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int i = tid + r * NC;
          if (kTcCS < NC && i >= kTcCS) break;
          store_row_split(opb_hi, opb_lo, i, g[r]);
          const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
          *reinterpret_cast<float4 *>(opb_a + tc_off(i, 0)) =
              make_float4(a3[r][0], a3[r][1], a3[r][2], 0.f);
          *reinterpret_cast<float4 *>(opb_a + tc_off(i, 4)) = z;
          amp[(j & 1) * kTcCS + i] = am[r];
        }
        if (has_t) {
          store_row_split(opa_hi, opa_lo, tid, f);
          tph[(j & 1) * kTcTT + tid] = tph_v;
          tsc[(j & 1) * kTcTT + tid] = tsc_v;
        }
      }
      ptx::fence_proxy_async_smem();
      ptx::tc_fence_before();
      __syncthreads();  // operands complete; the staging buffer is free
      ptx::tc_fence_after();
      if (tid == 0 && j + 1 < se && !*abort_flag) issue(j + 1);

      if (framer) {
        // frames[(j + 1) & 1] was last read by the operand build of tile j - 1, and it
        // is read next after frame_ready's next phase: it runs at most one phase ahead
        if (lane == 0 && j + 1 < se) {
          build_frame(frames + ((j + 1) & 1), P.tiles_t + 6 * (size_t)tt,
                      P.tiles_s + 6 * (size_t)(j + 1), sk);
          ptx::mbar_arrive(frame_ready);
        }
        __syncwarp();
      } else if (producer) {
        // ---- MMA issue: 4 target blocks x NBLK source blocks, double-buffered ----
        if (lane == 0) {
          for (int blk = 0; blk < 4 * NBLK; ++blk) {
            const int m = blk / NBLK, n = blk % NBLK, b = blk & 1;
            if (uses[b] > 0)
              tc_wait(&freeb[b], (uses[b] - 1) & 1u, abort_flag, err,
                      (FL & kTcSleepMma) ? 64u : 0u);
            if (*abort_flag) break;
            ptx::tc_fence_after();
            const uint32_t d = tbase + (uint32_t)(b * kTcN);
            const uint64_t dah = ptx::tc_smem_desc(opa_hi + m * kTcM * kTcK, kTcLbo, kTcSbo);
            const uint64_t dal = ptx::tc_smem_desc(opa_lo + m * kTcM * kTcK, kTcLbo, kTcSbo);
            const uint64_t dbh = ptx::tc_smem_desc(opb_hi + n * kTcN * kTcK, kTcLbo, kTcSbo);
            const uint64_t dbl = ptx::tc_smem_desc(opb_lo + n * kTcN * kTcK, kTcLbo, kTcSbo);
            const uint64_t dba = ptx::tc_smem_desc(opb_a + n * kTcN * kTcK, kTcLbo, kTcSbo);
            const uint64_t d1 = ptx::tc_smem_desc(opa_one, kTcLbo, kTcSbo);
            ptx::tc_mma_tf32(d, dah, dbh, idesc, 0u);
            ptx::tc_mma_tf32(d, dah, dbl, idesc, 1u);
            ptx::tc_mma_tf32(d, dal, dbh, idesc, 1u);
            ptx::tc_mma_tf32(d, d1, dba, idesc, 1u);
            ptx::tc_commit(&full[b]);
            ++uses[b];
          }
        }
        __syncwarp();
      } else {
        // the previous tile's carry while this tile's first MMAs run: its partial
        // sums are complete (written before the operand sync).  With one buffer
        // (NBLK >= 3) they are rewritten only after block NBLK - 1 >= 2 of this
        // tile, whose MMA waits for every consumer to free block 0, i.e. to have
        // passed this point; with fewer blocks the next tile writes the other buffer
        if (j > sb && tid < kTcTT && !*abort_flag) carry(j - 1);
        // ---- consumers: sin/cos and accumulation of a' e^{i theta'} ----
        const int lg = warp & 3, cg = warp >> 2;
        uint32_t rv[2][16];
        bool pre = false;  // kTcPrefetch: chunk 0 of this block already requested into rv[0]
        for (int m = 0; m < 4; ++m) {
          uint64_t re2 = 0ull, im2 = 0ull;
          float res[2] = {0.f, 0.f}, ims[2] = {0.f, 0.f};  // SC: the MUFU pairs
          for (int n = 0; n < NBLK; ++n) {
            const int blk = m * NBLK + n, b = blk & 1;
            bool ok = true;
            if (!pre) {
              ok = __all_sync(0xffffffffu, tc_wait(&full[b], uses[b] & 1u, abort_flag, err,
                                                   (FL & kTcSleepUse) ? 32u : 0u));
              ++uses[b];
              ptx::tc_fence_after();
            }
            if (ok) {
              // the load of chunk ch + 1 is in flight while chunk ch is summed
              const uint32_t ta =
                  tbase + ((uint32_t)(32 * lg) << 16) + (uint32_t)(b * kTcN + cg * S::Cols);
              if (!pre) ptx::tmem_ld16_nowait(ta, rv[0]);
              ptx::tmem_wait16(rv[0]);
              pre = false;
              const int bn = (blk + 1) & 1;  // the next block's accumulator buffer
              const uint32_t ta_next =
                  tbase + ((uint32_t)(32 * lg) << 16) + (uint32_t)(bn * kTcN + cg * S::Cols);
              // chunk ch (parity P = ch & 1, a compile-time constant): its phases are in
              // rv[P]; the load of chunk ch + 1 into rv[P ^ 1] is in flight meanwhile
              auto chunk = [&](auto parity, auto npp_tag, const int ch) {
                constexpr int P = decltype(parity)::value;
                if (ch + 1 < S::Chunks) {
                  ptx::tmem_ld16_nowait(ta + (uint32_t)(16 * (ch + 1)), rv[P ^ 1]);
                } else if ((FL & kTcPrefetch) && blk + 1 < 4 * NBLK) {
                  // the last chunk (P = 1, rv[0] free): the next block's first load now,
                  // if its MMAs are complete already; else after this block as usual
                  const bool ready = __all_sync(
                      0xffffffffu, !*abort_flag && ptx::mbar_test_wait(&full[bn], uses[bn] & 1u));
                  if (ready) {
                    ++uses[bn];
                    ptx::tc_fence_after();
                    ptx::tmem_ld16_nowait(ta_next, rv[P ^ 1]);
                    pre = true;
                  }
                }
                const float4 *ap =
                    reinterpret_cast<const float4 *>(amp + (j & 1) * kTcCS + n * kTcN +
                                                     cg * S::Cols + 16 * ch);
                float av[16];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                  const float4 v = ap[q];
                  av[4 * q] = v.x;
                  av[4 * q + 1] = v.y;
                  av[4 * q + 2] = v.z;
                  av[4 * q + 3] = v.w;
                }
                constexpr int npp = decltype(npp_tag)::value;
                tc_pairs16<FL, npp>(rv[P], av, re2, im2, res, ims);
                if (ch + 1 < S::Chunks) ptx::tmem_wait16(rv[P ^ 1]);
              };
              static_assert(S::Chunks % 2 == 0, "chunks come in pairs");
              using Even = std::integral_constant<int, 0>;
              using Odd = std::integral_constant<int, 1>;
              using NppEven = std::integral_constant<int, NPP0>;
              using NppOdd = std::integral_constant<int, NPP1>;
              if (FL & kTcHalfUnroll) {
#pragma unroll 1
                for (int ch = 0; ch < S::Chunks; ch += 2) {
                  chunk(Even{}, NppEven{}, ch);
                  chunk(Odd{}, NppOdd{}, ch + 1);
                }
              } else {
#pragma unroll
                for (int ch = 0; ch < S::Chunks; ch += 2) {
                  chunk(Even{}, NppEven{}, ch);
                  chunk(Odd{}, NppOdd{}, ch + 1);
                }
              }
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&freeb[b]);
          }
          float x, y;
          ptx::unpack2(re2, x, y);
          const float re = (x + y) + (res[0] + res[1]);
          ptx::unpack2(im2, x, y);
          part[((j & 1) % L::PB) * CG * kTcTT + cg * kTcTT + m * kTcM + 32 * lg + lane] =
              make_float2(re, (x + y) + (ims[0] + ims[1]));
        }
      }
    }
    // the last tile's partial sums, once every consumer has written them
    __syncthreads();
    if (tid < kTcTT && se > sb && !*abort_flag) carry(se - 1);

    for (int t = tid; t < kTcTT; t += kTcThreads) {
      const int ti = tt * kTcTT + t;
      if (ti < P.M) {
        const float4 a = acc[t];
        const double2 v = make_double2((double)a.x + (double)a.y, (double)a.z + (double)a.w);
        if (P.splits == 1)
          P.y[P.order_t[ti]] = v;
        else
          P.partial[(size_t)split * P.M + ti] = v;
      }
    }
    __syncthreads();  // acc is reset by the next item
  }

  // ---- teardown: the MMAs this CTA issued have completed, then free the TMEM ----
  if (producer && lane == 0)
    for (int b = 0; b < 2; ++b)
      if (uses[b] > 0) ptx::mbar_wait_bounded(&full[b], (uses[b] - 1) & 1u, kWaitCycles);
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  if (producer) ptx::tmem_dealloc(tbase, kTcCols);
}

// ---- builder-warp kernel (kTcBuilders) -----------------------------------------------------
// The same tile pairs and pair loop as k_split_tc, with the operands built by warps of
// their own while the consumers sum: the consumers never stop for a build, a frame or a
// carry.
// Blocks run source block outer (n), target block inner (m), so that source block n is
// free for the next tile pair once the MMAs of (3, n) are complete, a quarter tile
// after it was built, and the next tile pair's target rows go to a second buffer (the
// source rows of a tile pair thus have 3/4 of a tile pair of time, the target rows all
// of it).  A consumer adds each block's sums into its partial sums of the tile pair in
// shared memory.  The builders read the source records from global memory (they stay
// in L2), carry each tile pair's partial sums into the running sums two tile pairs
// later, and write the item's results.  Hand-offs, one phase per tile pair q:
//   opa_ready[q & 1]   target rows of q built (one arrival per builder thread) -> MMA warp
//   opb_ready[n]       source block n of q built (the same)                -> MMA warp,
//                      and for the consumers, that block's amplitudes
//   opb_free[n]        the MMAs of (3, n) of q are complete (tcgen05.commit) -> builders
//   tile_done[q & 1]   every MMA of q is complete (tcgen05.commit)         -> builders
//   parts_ready[q & 1] every consumer thread has added its sums of q       -> builders
//   frame_ready[q & 1] / frame_free[q & 1]: frame q (frame warp / builders).
// The barriers a wait may trail by two phases come in pairs by q & 1, so that no wait
// can miss its phase: the phase after the awaited one needs work that follows the
// waiting thread's own.
// builder warps: four (one per SM sub-partition) beside 16 consumer warps (two with
// kTcBuilders2), two beside 24
template <int CG, int FL>
__host__ __device__ constexpr int tc_builder_warps() {
  return CG == 4 && (FL & kTcBuilders2) == 0 ? 4 : 2;
}

template <int CG, int NBLK>
struct TcBwSmem {
  static constexpr int kTcCS = TcShape<CG, NBLK>::CS;
  static constexpr size_t opb_hi = 0;                                  // float [CS*8]
  static constexpr size_t opb_lo = opb_hi + kTcCS * kTcK * 4;          // float [CS*8]
  static constexpr size_t opb_a = opb_lo + kTcCS * kTcK * 4;           // float [CS*8]: A parts
  static constexpr size_t opa = opb_a + kTcCS * kTcK * 4;              // float [2][hi, lo][TT*8]
  static constexpr size_t opa_one = opa + 4 * kTcTT * kTcK * 4;        // float [128*8]
  static constexpr size_t amp = opa_one + kTcM * kTcK * 4;             // float [2][CS]
  static constexpr size_t part = amp + 2 * kTcCS * 4;                  // float2 [2][CG][TT]
  static constexpr size_t acc = part + 2 * CG * kTcTT * 8;             // float4 [TT]
  static constexpr size_t tph = acc + kTcTT * 16;                      // float [2][TT]
  static constexpr size_t tsc = tph + 2 * kTcTT * 4;                   // float [2][TT]
  static constexpr size_t frame = tsc + 2 * kTcTT * 4;                 // Frame [2]
  static constexpr int kBars = 22;
  static constexpr size_t bars = (frame + 2 * sizeof(Frame) + 15) / 16 * 16;  // uint64 [22]
  static constexpr size_t misc = bars + kBars * 8;                     // uint32 taddr, abort
  static constexpr size_t bytes = misc + 16;
};
template <int CG, int NBLK>
constexpr bool tc_bw_layout_ok() {
  using L = TcBwSmem<CG, NBLK>;
  return L::bytes <= 227 * 1024 && L::opb_lo % 128 == 0 && L::opb_a % 128 == 0 &&
         L::opa % 128 == 0 && L::opa_one % 128 == 0 && L::amp % 16 == 0 && L::part % 16 == 0 &&
         L::acc % 16 == 0 && L::frame % 16 == 0;
}
static_assert(tc_bw_layout_ok<4, 4>() && tc_bw_layout_ok<4, 2>() && tc_bw_layout_ok<4, 1>() &&
                  tc_bw_layout_ok<6, 4>(),
              "builder-warp kernel: shared memory size and operand alignment");

template <int CG, int NBLK, int NPP0, int NPP1, int FL, bool BATCHED>
__global__ void __launch_bounds__(TcShape<CG, NBLK>::Threads + 32 * tc_builder_warps<CG, FL>(), 1)
    k_split_tc_bw(const SplitProblem P0, const SplitProblem *__restrict__ probs,
                  const WorkItem *__restrict__ items, int n_items, int *queue, int *err) {
  extern __shared__ __align__(128) unsigned char smem[];
  using L = TcBwSmem<CG, NBLK>;
  using S = TcShape<CG, NBLK>;
  constexpr int kTcCS = S::CS, kTcN = S::NB, kTcConsumers = S::Consumers;
  constexpr int kTcThreads = S::Threads + 32 * tc_builder_warps<CG, FL>();
  constexpr int NBT = 32 * tc_builder_warps<CG, FL>();  // builder threads
  constexpr int kRowsB = (kTcN + NBT - 1) / NBT;  // source rows per builder thread and block
  constexpr int kRowsT = kTcTT / NBT;             // target rows per builder thread
  static_assert(kTcTT % NBT == 0 && kRowsT % 4 == 0, "builder rows");
  static_assert((FL & (kTcScalar | kTcPrefetch | kTcHalfUnroll)) == 0,
                "builder-warp kernel: packed MUFU pairs, full unroll, no prefetch");
  float *opb_hi = reinterpret_cast<float *>(smem + L::opb_hi);
  float *opb_lo = reinterpret_cast<float *>(smem + L::opb_lo);
  float *opb_a = reinterpret_cast<float *>(smem + L::opb_a);
  float *opa = reinterpret_cast<float *>(smem + L::opa);  // tile pair q: hi at 2 (q & 1), lo after
  float *opa_one = reinterpret_cast<float *>(smem + L::opa_one);
  float *amp = reinterpret_cast<float *>(smem + L::amp);
  float2 *part = reinterpret_cast<float2 *>(smem + L::part);
  // per target, the running sum of the tile sums as float-float pairs
  // (re hi, re lo, im hi, im lo): FP64 runs at a small fraction of the FP32 rate here
  float4 *acc = reinterpret_cast<float4 *>(smem + L::acc);
  float *tph = reinterpret_cast<float *>(smem + L::tph);
  float *tsc = reinterpret_cast<float *>(smem + L::tsc);
  Frame *frames = reinterpret_cast<Frame *>(smem + L::frame);  // tile pair q in frames[q & 1]
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::bars);
  uint64_t *full = bars, *freeb = bars + 2, *frame_ready = bars + 4, *frame_free = bars + 6,
           *opa_ready = bars + 8, *tile_done = bars + 10, *parts_ready = bars + 12,
           *opb_ready = bars + 14, *opb_free = bars + 18;
  uint32_t *taddr_slot = reinterpret_cast<uint32_t *>(smem + L::misc);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + L::misc + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool consumer = warp < kTcConsumers;
  const bool producer = warp == kTcConsumers;     // TMEM owner, MMA issue
  const bool framer = warp == kTcConsumers + 1;   // frames
  const int bt = tid - 32 * (kTcConsumers + 2);   // builder thread (>= 0: a builder)
  constexpr int NC = kTcConsumers * 32;           // consumer threads

  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&full[b], 1);
      ptx::mbar_init(&freeb[b], kTcConsumers);
      ptx::mbar_init(&frame_ready[b], 1);
      ptx::mbar_init(&frame_free[b], NBT);
      ptx::mbar_init(&opa_ready[b], NBT);
      ptx::mbar_init(&tile_done[b], 1);
      ptx::mbar_init(&parts_ready[b], NC);
    }
    for (int n = 0; n < NBLK; ++n) {
      ptx::mbar_init(&opb_ready[n], NBT);
      ptx::mbar_init(&opb_free[n], 1);
    }
    *abort_flag = 0;
    ptx::fence_barrier_init();
  }
  // constant operand of the phase term: every row (1, 1, 1, 0, ..)
  for (int i = tid; i < kTcM * kTcK; i += kTcThreads)
    opa_one[tc_off(i / kTcK, i % kTcK)] = (i % kTcK) < 3 ? 1.f : 0.f;
  if (producer) ptx::tmem_alloc(taddr_slot, kTcCols);
  ptx::fence_proxy_async_smem();
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tbase = *taddr_slot;

  constexpr uint32_t idesc = ptx::tc_idesc_tf32(kTcM, kTcN);
  // producer: MMA groups issued per TMEM buffer; consumers: completions consumed
  uint32_t uses[2] = {0u, 0u};
  // producer: commits issued to tile_done[b] and opb_free[n]
  uint32_t n_done[2] = {0u, 0u}, n_free[NBLK] = {};
  uint32_t q0 = 0;  // sequence number of the item's first tile pair
  __shared__ int s_item;

  for (int it = 0;; ++it) {
    int item;
    if (BATCHED) {
      if (tid == 0) s_item = atomicAdd(queue, 1);
      __syncthreads();
      item = s_item;
      __syncthreads();  // s_item is rewritten for the next item
    } else {
      item = blockIdx.x + it * gridDim.x;
    }
    if (item >= n_items) break;
    const SplitProblem &P = BATCHED ? probs[items[item].problem] : P0;
    int tt, split, sb, se;
    if (BATCHED) {
      const WorkItem w = items[item];
      tt = w.ttile;
      split = w.split;
      sb = w.s_begin;
      se = w.s_end;
    } else {
      tt = item / P.splits;
      split = item % P.splits;
      split_range_tc(P.n_stiles, P.splits, split, &sb, &se);
    }
    const int nt = se > sb ? se - sb : 0;
    const double sk = P.sk;

    if (framer) {
      if (lane == 0)
        for (int j = sb; j < se; ++j) {
          const uint32_t q = q0 + (uint32_t)(j - sb);
          // the slot was last read by the builds of tile pair q - 2
          if (q >= 2 && !tc_wait(&frame_free[q & 1], ((q - 2) >> 1) & 1u, abort_flag, err)) break;
          build_frame(frames + (q & 1), P.tiles_t + 6 * (size_t)tt, P.tiles_s + 6 * (size_t)j, sk);
          ptx::mbar_arrive(&frame_ready[q & 1]);
        }
      __syncwarp();
    } else if (producer) {
      // ---- MMA issue: NBLK source blocks x 4 target blocks per tile pair ----
      if (lane == 0) {
        for (int j = sb; j < se && !*abort_flag; ++j) {
          const uint32_t q = q0 + (uint32_t)(j - sb);
          const float *oah = opa + (q & 1) * 2 * kTcTT * kTcK, *oal = oah + kTcTT * kTcK;
          for (int blk = 0; blk < 4 * NBLK; ++blk) {
            const int n = blk / 4, m = blk % 4, b = blk & 1;
            if (blk == 0) tc_wait(&opa_ready[q & 1], (q >> 1) & 1u, abort_flag, err);
            if (m == 0) tc_wait(&opb_ready[n], q & 1u, abort_flag, err);
            if (uses[b] > 0)
              tc_wait(&freeb[b], (uses[b] - 1) & 1u, abort_flag, err,
                      (FL & kTcSleepMma) ? 64u : 0u);
            if (*abort_flag) break;
            ptx::tc_fence_after();
            const uint32_t d = tbase + (uint32_t)(b * kTcN);
            const uint64_t dah = ptx::tc_smem_desc(oah + m * kTcM * kTcK, kTcLbo, kTcSbo);
            const uint64_t dal = ptx::tc_smem_desc(oal + m * kTcM * kTcK, kTcLbo, kTcSbo);
            const uint64_t dbh = ptx::tc_smem_desc(opb_hi + n * kTcN * kTcK, kTcLbo, kTcSbo);
            const uint64_t dbl = ptx::tc_smem_desc(opb_lo + n * kTcN * kTcK, kTcLbo, kTcSbo);
            const uint64_t dba = ptx::tc_smem_desc(opb_a + n * kTcN * kTcK, kTcLbo, kTcSbo);
            const uint64_t d1 = ptx::tc_smem_desc(opa_one, kTcLbo, kTcSbo);
            ptx::tc_mma_tf32(d, dah, dbh, idesc, 0u);
            ptx::tc_mma_tf32(d, dah, dbl, idesc, 1u);
            ptx::tc_mma_tf32(d, dal, dbh, idesc, 1u);
            ptx::tc_mma_tf32(d, d1, dba, idesc, 1u);
            ptx::tc_commit(&full[b]);
            ++uses[b];
            if (m == 3) {
              ptx::tc_commit(&opb_free[n]);  // source block n is read no more
              ++n_free[n];
            }
          }
          if (!*abort_flag) {
            ptx::tc_commit(&tile_done[q & 1]);
            ++n_done[q & 1];
          }
        }
      }
      __syncwarp();
    } else if (consumer) {
      // ---- consumers: sin/cos and accumulation of a' e^{i theta'} ----
      const int lg = warp & 3, cg = warp >> 2;
      for (int j = sb; j < se; ++j) {
        const uint32_t q = q0 + (uint32_t)(j - sb);
        float2 *pq = part + (q & 1) * CG * kTcTT + cg * kTcTT + 32 * lg + lane;
        uint32_t rv[2][16];
        for (int blk = 0; blk < 4 * NBLK; ++blk) {
          const int n = blk / 4, m = blk % 4, b = blk & 1;
          const bool ok = __all_sync(0xffffffffu, tc_wait(&full[b], uses[b] & 1u, abort_flag, err));
          ++uses[b];
          ptx::tc_fence_after();
          uint64_t re2 = 0ull, im2 = 0ull;
          if (ok) {
            const uint32_t ta =
                tbase + ((uint32_t)(32 * lg) << 16) + (uint32_t)(b * kTcN + cg * S::Cols);
            ptx::tmem_ld16_nowait(ta, rv[0]);
            // the block's amplitudes were written by the builders: acquire them
            if (m == 0) tc_wait(&opb_ready[n], q & 1u, abort_flag, err);
            ptx::tmem_wait16(rv[0]);
            float res[2] = {0.f, 0.f}, ims[2] = {0.f, 0.f};  // unused: packed MUFU pairs
            // chunk ch (parity P = ch & 1, a compile-time constant): its phases are in
            // rv[P]; the load of chunk ch + 1 into rv[P ^ 1] is in flight meanwhile
            auto chunk = [&](auto parity, auto npp_tag, const int ch) {
              constexpr int P = decltype(parity)::value;
              if (ch + 1 < S::Chunks)
                ptx::tmem_ld16_nowait(ta + (uint32_t)(16 * (ch + 1)), rv[P ^ 1]);
              const float4 *ap = reinterpret_cast<const float4 *>(
                  amp + (q & 1) * kTcCS + n * kTcN + cg * S::Cols + 16 * ch);
              float av[16];
#pragma unroll
              for (int v4 = 0; v4 < 4; ++v4) {
                const float4 v = ap[v4];
                av[4 * v4] = v.x;
                av[4 * v4 + 1] = v.y;
                av[4 * v4 + 2] = v.z;
                av[4 * v4 + 3] = v.w;
              }
              constexpr int npp = decltype(npp_tag)::value;
              tc_pairs16<FL, npp>(rv[P], av, re2, im2, res, ims);
              if (ch + 1 < S::Chunks) ptx::tmem_wait16(rv[P ^ 1]);
            };
            static_assert(S::Chunks % 2 == 0, "chunks come in pairs");
            using Even = std::integral_constant<int, 0>;
            using Odd = std::integral_constant<int, 1>;
            using NppEven = std::integral_constant<int, NPP0>;
            using NppOdd = std::integral_constant<int, NPP1>;
#pragma unroll
            for (int ch = 0; ch < S::Chunks; ch += 2) {
              chunk(Even{}, NppEven{}, ch);
              chunk(Odd{}, NppOdd{}, ch + 1);
            }
          }
          ptx::tc_fence_before();
          __syncwarp();
          if (lane == 0) ptx::mbar_arrive(&freeb[b]);
          // this block's sums into the tile pair's partial sums of target 128 m + 32 lg + lane
          float x, y, u, w;
          ptx::unpack2(re2, x, y);
          ptx::unpack2(im2, u, w);
          float2 s = make_float2(x + y, u + w);
          if (n > 0) {
            const float2 o = pq[m * kTcM];
            s = make_float2(o.x + s.x, o.y + s.y);
          }
          pq[m * kTcM] = s;
        }
        ptx::mbar_arrive(&parts_ready[q & 1]);
      }
    } else {
      // ---- builders: operands, carries and results ----
      const float kap2 = (float)(0.5 * sk), ak = fabsf(kap2), iak = 1.f / fabsf(kap2);
      const float sgn = kap2 < 0.f ? -1.f : 1.f;
      for (int r = 0; r < kRowsT; ++r) acc[bt + NBT * r] = make_float4(0.f, 0.f, 0.f, 0.f);
      // tile pair q's partial sums of this thread's targets, scaled, rotated and carried
      auto carry = [&](uint32_t q) {
        if (!tc_wait(&parts_ready[q & 1], (q >> 1) & 1u, abort_flag, err)) return;
        for (int r = 0; r < kRowsT; ++r) {
          const int t = bt + NBT * r;
          float sx = 0.f, sy = 0.f;
#pragma unroll
          for (int c = 0; c < CG; ++c) {
            const float2 v = part[(q & 1) * CG * kTcTT + c * kTcTT + t];
            sx += v.x;
            sy += v.y;
          }
          const float sc = tsc[(q & 1) * kTcTT + t];
          const float re = sx * sc;
          const float im = sgn * sy * sc;
          float sr, cr;
          __sincosf(tph[(q & 1) * kTcTT + t], &sr, &cr);
          float4 a = acc[t];
          float h, e;
          two_sum(a.x, fmaf(re, cr, -im * sr), h, e);  // h + e: the exact sum
          a.x = h;
          a.y = __fadd_rn(a.y, e);
          two_sum(a.z, fmaf(re, sr, im * cr), h, e);
          a.z = h;
          a.w = __fadd_rn(a.w, e);
          acc[t] = a;
        }
      };
      for (int j = sb; j < se; ++j) {
        const uint32_t q = q0 + (uint32_t)(j - sb);
        // tile pair q - 2 used the rotations and partial sums that q's build rewrites
        if (j - 2 >= sb) carry(q - 2);
        if (!tc_wait(&frame_ready[q & 1], (q >> 1) & 1u, abort_flag, err)) break;
        const TcBasis B = tc_basis(frames + (q & 1));
        // ---- target rows into the second buffer: the MMAs of q - 2 read it last ----
        if (q >= 2 && !tc_wait(&tile_done[q & 1], ((q - 2) >> 1) & 1u, abort_flag, err)) break;
        float *oah = opa + (q & 1) * 2 * kTcTT * kTcK, *oal = oah + kTcTT * kTcK;
        for (int r0 = 0; r0 < kRowsT; r0 += 4) {
          float f[4][kTcK], pv[4], sv[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int t = bt + NBT * (r0 + r), ti = tt * kTcTT + t;
            float th[3] = {0.f, 0.f, 0.f}, tl[3] = {0.f, 0.f, 0.f};
            if (ti < P.M) {
#pragma unroll
              for (int k = 0; k < 3; ++k) {
                th[k] = P.geo_t[6 * (size_t)ti + k];
                tl[k] = P.geo_t[6 * (size_t)ti + 3 + k];
              }
            }
            tc_target_row<FL>(B, th, tl, ak, iak, sgn, f[r], pv[r], sv[r]);
          }
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int t = bt + NBT * (r0 + r);
            store_row_split(oah, oal, t, f[r]);
            tph[(q & 1) * kTcTT + t] = pv[r];
            tsc[(q & 1) * kTcTT + t] = sv[r];
          }
        }
        ptx::fence_proxy_async_smem();  // the MMAs read the rows through the async proxy
        ptx::mbar_arrive(&opa_ready[q & 1]);
        // ---- source blocks, each once the MMAs of (3, n) of q - 1 are complete.  Records
        // past N are zeros (offsets, phase and amplitude): the row comes out all zeros ----
        const float *gs = P.geo_s + (size_t)j * kTcCS * 6;
        const float2 *as = P.apf_s + (size_t)j * kTcCS;
        for (int n = 0; n < NBLK; ++n) {
          if (q >= 1 && !tc_wait(&opb_free[n], (q - 1) & 1u, abort_flag, err)) break;
          float g[kRowsB][kTcK], a3[kRowsB][3], am[kRowsB];
#pragma unroll
          for (int r = 0; r < kRowsB; ++r) {
            if (kTcN % NBT != 0 && bt + NBT * r >= kTcN) break;
            const int i = n * kTcN + bt + NBT * r;
            const float *rec = gs + 6 * (size_t)i;
            const float sh[3] = {rec[0], rec[1], rec[2]}, sl[3] = {rec[3], rec[4], rec[5]};
            tc_source_row<FL, kTcN, S::Cols, NPP0, NPP1>(B, sh, sl, as[i], sgn, i, g[r], a3[r],
                                                         am[r]);
          }
#pragma unroll
          for (int r = 0; r < kRowsB; ++r) {
            if (kTcN % NBT != 0 && bt + NBT * r >= kTcN) break;
            const int i = n * kTcN + bt + NBT * r;
            store_row_split(opb_hi, opb_lo, i, g[r]);
            *reinterpret_cast<float4 *>(opb_a + tc_off(i, 0)) =
                make_float4(a3[r][0], a3[r][1], a3[r][2], 0.f);
            *reinterpret_cast<float4 *>(opb_a + tc_off(i, 4)) = make_float4(0.f, 0.f, 0.f, 0.f);
            amp[(q & 1) * kTcCS + i] = am[r];
          }
          ptx::fence_proxy_async_smem();
          ptx::mbar_arrive(&opb_ready[n]);
        }
        ptx::mbar_arrive(&frame_free[q & 1]);  // frame q is read no more
      }
      if (nt >= 2 && !*abort_flag) carry(q0 + (uint32_t)(nt - 2));
      if (nt >= 1 && !*abort_flag) carry(q0 + (uint32_t)(nt - 1));
      for (int r = 0; r < kRowsT; ++r) {
        const int t = bt + NBT * r, ti = tt * kTcTT + t;
        if (ti < P.M) {
          const float4 a = acc[t];
          const double2 v = make_double2((double)a.x + (double)a.y, (double)a.z + (double)a.w);
          if (P.splits == 1)
            P.y[P.order_t[ti]] = v;
          else
            P.partial[(size_t)split * P.M + ti] = v;
        }
      }
    }
    q0 += (uint32_t)nt;
  }

  // ---- teardown: every commit of this CTA has arrived (the MMAs are complete), then
  // free the TMEM ----
  if (producer && lane == 0) {
    for (int b = 0; b < 2; ++b) {
      if (uses[b] > 0) ptx::mbar_wait_bounded(&full[b], (uses[b] - 1) & 1u, kWaitCycles);
      if (n_done[b] > 0) ptx::mbar_wait_bounded(&tile_done[b], (n_done[b] - 1) & 1u, kWaitCycles);
    }
    for (int n = 0; n < NBLK; ++n)
      if (n_free[n] > 0) ptx::mbar_wait_bounded(&opb_free[n], (n_free[n] - 1) & 1u, kWaitCycles);
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  if (producer) ptx::tmem_dealloc(tbase, kTcCols);
}

// The kernel of a build: kTcBuilders selects the builder-warp kernel.
template <int CG, int NBLK, int NPP0, int NPP1, int FL, bool BATCHED>
constexpr auto tc_kernel() {
  if constexpr ((FL & kTcBuilders) != 0)
    return k_split_tc_bw<CG, NBLK, NPP0, NPP1, FL, BATCHED>;
  else
    return k_split_tc<CG, NBLK, NPP0, NPP1, FL, BATCHED>;
}
template <int CG, int NBLK, int FL>
constexpr int tc_smem_bytes() {
  return (FL & kTcBuilders) != 0 ? (int)TcBwSmem<CG, NBLK>::bytes : (int)TcSmem<CG, NBLK>::bytes;
}
template <int CG, int NBLK, int FL>
constexpr int tc_threads() {
  return TcShape<CG, NBLK>::Threads + ((FL & kTcBuilders) != 0 ? 32 * tc_builder_warps<CG, FL>() : 0);
}

template <int CG, int NBLK, int NPP0, int NPP1, int FL>
int launch_tc(const SplitProblem &p, int grid, int *err, cudaStream_t s) {
  constexpr auto kern = tc_kernel<CG, NBLK, NPP0, NPP1, FL, false>();
  constexpr int bytes = tc_smem_bytes<CG, NBLK, FL>();
  constexpr int threads = tc_threads<CG, NBLK, FL>();
  HOLO_TRY((kernel_setup<kern>(threads, bytes, nullptr)));
  const int n_items = p.n_ttiles * p.splits;
  if (n_items <= 0) return HOLO_OK;
  kern<<<grid, threads, bytes, s>>>(p, nullptr, nullptr, n_items, nullptr, err);
  note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

template <int CG, int NBLK, int NPP0, int NPP1, int FL>
int launch_tc_batched(const SplitProblem *probs, const WorkItem *items, int n_items, int *queue,
                      int grid, int *err, cudaStream_t s) {
  constexpr auto kern = tc_kernel<CG, NBLK, NPP0, NPP1, FL, true>();
  constexpr int bytes = tc_smem_bytes<CG, NBLK, FL>();
  constexpr int threads = tc_threads<CG, NBLK, FL>();
  HOLO_TRY((kernel_setup<kern>(threads, bytes, nullptr)));
  kern<<<grid, threads, bytes, s>>>(SplitProblem{}, probs, items, n_items, queue, err);
  note_launches(1);
  HOLO_CUDA(cudaGetLastError());
  return HOLO_OK;
}

template <int CG, int NBLK, int NPP0, int NPP1, int FL>
int occupancy_tc(int *out) {
  return kernel_setup<tc_kernel<CG, NBLK, NPP0, NPP1, FL, false>()>(
      tc_threads<CG, NBLK, FL>(), tc_smem_bytes<CG, NBLK, FL>(), out);
}

// builds: source tile CS, polynomial pairs A of even and B of odd chunks (A + B of every
// 16 source pairs), build flags (kTcScalar, kTcHalfUnroll, kTcRcp).  The key and the template
// arguments come from the same four numbers: 768-source tiles are 4 blocks of 192 with
// 6 column groups, the others CS / 256 blocks of 256 with 4.  A use site defines
// CALL(CG, NBLK, A, B, FL) and expands HOLO_TC_SWITCH.
#define HOLO_TC_KEY(CS, NP16, FLAGS) ((CS) * 100000 + (NP16) * 1000 + (FLAGS))
#define HOLO_TC_CASE(CS, A, B, FL)     \
  case HOLO_TC_KEY(CS, (A) + (B), FL): \
    return CALL(((CS) == 768 ? 6 : 4), ((CS) == 768 ? 4 : (CS) / 256), A, B, FL);
#define HOLO_TC_BUILDS                        \
  HOLO_TC_CASE(1024, 2, 2, 0)                 \
  HOLO_TC_CASE(1024, 2, 3, 0)                 \
  HOLO_TC_CASE(1024, 3, 3, 0)                 \
  HOLO_TC_CASE(1024, 3, 3, kTcScalar)         \
  HOLO_TC_CASE(1024, 3, 3, kTcHalfUnroll)     \
  HOLO_TC_CASE(1024, 3, 3, kTcRcp)            \
  HOLO_TC_CASE(1024, 3, 3, kTcHalfUnroll | kTcRcp) \
  HOLO_TC_CASE(1024, 3, 3, kTcPrefetch)       \
  HOLO_TC_CASE(1024, 3, 3, kTcPrefetch | kTcRcp) \
  HOLO_TC_CASE(1024, 3, 4, kTcPrefetch)       \
  HOLO_TC_CASE(1024, 3, 3, kTcSleepMma)       \
  HOLO_TC_CASE(1024, 3, 3, kTcSleepMma | kTcSleepUse) \
  HOLO_TC_CASE(1024, 3, 3, kTcSleepMma | kTcPrefetch) \
  HOLO_TC_CASE(1024, 3, 3, kTcHalfTurns)      \
  HOLO_TC_CASE(1024, 3, 3, kTcHalfTurns | kTcSin7) \
  HOLO_TC_CASE(1024, 3, 4, kTcHalfTurns | kTcSin7) \
  HOLO_TC_CASE(1024, 4, 4, kTcHalfTurns | kTcSin7) \
  HOLO_TC_CASE(1024, 4, 5, kTcHalfTurns | kTcSin7) \
  HOLO_TC_CASE(1024, 3, 4, kTcHalfTurns | kTcSin7 | kTcPrefetch | kTcSleepMma) \
  HOLO_TC_CASE(1024, 4, 4, kTcHalfTurns | kTcSin7 | kTcPrefetch | kTcSleepMma) \
  HOLO_TC_CASE(1024, 3, 3, kTcHalfTurns | kTcSin7 | kTcPrefetch) \
  HOLO_TC_CASE(1024, 3, 3, kTcHalfTurns | kTcSin7 | kTcPrefetch | kTcSleepMma) \
  HOLO_TC_CASE(1024, 3, 3, kTcHalfTurns | kTcSin7 | kTcRcp) \
  HOLO_TC_CASE(512, 3, 3, kTcHalfTurns | kTcSin7) \
  HOLO_TC_CASE(512, 3, 3, kTcHalfTurns | kTcSin7 | kTcPrefetch) \
  HOLO_TC_CASE(256, 3, 3, kTcHalfTurns | kTcSin7) \
  HOLO_TC_CASE(256, 3, 3, kTcHalfTurns | kTcSin7 | kTcPrefetch) \
  HOLO_TC_CASE(768, 3, 3, kTcHalfTurns | kTcSin7) \
  HOLO_TC_CASE(768, 3, 4, kTcHalfTurns | kTcSin7) \
  HOLO_TC_CASE(1024, 3, 3, kTcHalfTurns | kTcSin7 | kTcBuilders) \
  HOLO_TC_CASE(768, 3, 3, kTcHalfTurns | kTcSin7 | kTcBuilders) \
  HOLO_TC_CASE(512, 3, 3, kTcHalfTurns | kTcSin7 | kTcBuilders) \
  HOLO_TC_CASE(256, 3, 3, kTcHalfTurns | kTcSin7 | kTcBuilders | kTcBuilders2) \
  HOLO_TC_CASE(1024, 3, 4, 0)                 \
  HOLO_TC_CASE(1024, 3, 4, kTcScalar)         \
  HOLO_TC_CASE(1024, 3, 4, kTcHalfUnroll)     \
  HOLO_TC_CASE(1024, 4, 4, 0)                 \
  HOLO_TC_CASE(512, 3, 3, 0)                  \
  HOLO_TC_CASE(256, 3, 3, 0)                  \
  HOLO_TC_CASE(768, 2, 3, 0)                  \
  HOLO_TC_CASE(768, 3, 3, 0)                  \
  HOLO_TC_CASE(768, 3, 4, 0)
#define HOLO_TC_SWITCH(CS, NP16, FLAGS)                                                   \
  switch (HOLO_TC_KEY(CS, NP16, FLAGS)) {                                                 \
    HOLO_TC_BUILDS                                                                        \
    default:                                                                              \
      return fail(HOLO_ERR_INVALID,                                                       \
                  "tensor-core split kernel: no build for source tiles of %d, %d of 16, "  \
                  "flags %d", CS, NP16, FLAGS);                                           \
  }

}  // namespace

int launch_split_tc(const SplitProblem &p, int cs, int poly16, int flags, int grid, int *err,
                    cudaStream_t s) {
#define CALL(G, NB, A, B, C) launch_tc<G, NB, A, B, C>(p, grid, err, s)
  HOLO_TC_SWITCH(cs, poly16, flags)
#undef CALL
}

int launch_split_tc_batched(const SplitProblem *probs, const WorkItem *items, int n_items,
                            int *queue, int cs, int poly16, int flags, int grid, int *err,
                            cudaStream_t s) {
#define CALL(G, NB, A, B, C) \
  launch_tc_batched<G, NB, A, B, C>(probs, items, n_items, queue, grid, err, s)
  HOLO_TC_SWITCH(cs, poly16, flags)
#undef CALL
}

int split_tc_occupancy(int cs, int poly16, int flags, int *ctas_per_sm) {
#define CALL(G, NB, A, B, C) occupancy_tc<G, NB, A, B, C>(ctas_per_sm)
  HOLO_TC_SWITCH(cs, poly16, flags)
#undef CALL
}

bool split_tc_has_build(int cs, int poly16, int flags) {
#define CALL(G, NB, A, B, C) true
  switch (HOLO_TC_KEY(cs, poly16, flags)) {
    HOLO_TC_BUILDS
    default: return false;
  }
#undef CALL
}

}  // namespace holo

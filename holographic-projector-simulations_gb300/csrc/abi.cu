// abi.cu -- the C ABI: handles, plans, one-shot transforms, the x->y->z chain,
// the adjoint, the Monte Carlo estimator, batched problems and the autotuner.
//
// Replaces the reference's host side: transform_full (cuda/transform.cu:147-340:
// staging, streams, batching, kernel dispatch, cuBLAS row sum), time_transform
// (cuda/transform.cu:346-406) and the geometry derivation (cuda/init.h:42-84).
// No call exits the process: every failure is a status code plus a message.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <memory>

#include "internal.cuh"

namespace holo {

// ---- errors -------------------------------------------------------------------------
static thread_local std::string g_error;

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
}

int fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  const int code = (e == cudaErrorMemoryAllocation) ? HOLO_ERR_ALLOC
                   : (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice) ? HOLO_ERR_NO_DEVICE
                                                                             : HOLO_ERR_CUDA;
  return fail(code, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

namespace {

struct DeviceGuard {
  int prev = -1;
  bool ok = false;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess) ok = true;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

enum class Mem { Host, Device, Null };

Mem classify(const void *p) {
  if (!p) return Mem::Null;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear: an unregistered host pointer on old runtimes
    return Mem::Host;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? Mem::Device
                                                                            : Mem::Host;
}

// All non-null pointers must agree; returns HOLO_OK and sets *dev.
int classify_all(std::initializer_list<const void *> ptrs, bool *dev) {
  int n_host = 0, n_dev = 0;
  for (const void *p : ptrs) {
    const Mem m = classify(p);
    if (m == Mem::Host) ++n_host;
    if (m == Mem::Device) ++n_dev;
  }
  if (n_host && n_dev)
    return fail(HOLO_ERR_INVALID, "mixed host and device pointers in one call");
  *dev = n_dev > 0;
  return HOLO_OK;
}

bool finite_positive(double x) { return isfinite(x) && x > 0.0; }

int check_sign(int sign) {
  if (sign != 1 && sign != -1) return fail(HOLO_ERR_INVALID, "sign must be +1 or -1 (got %d)", sign);
  return HOLO_OK;
}

int check_sizes(size_t N, size_t M) {
  const size_t lim = (size_t)kSortBlock * 4096;  // tiler limit, also < 2^31
  if (N > lim || M > lim)
    return fail(HOLO_ERR_INVALID, "point count above the supported %zu (N=%zu, M=%zu)", lim, N, M);
  return HOLO_OK;
}

// Scoped device buffers from the handle's pool, freed stream-ordered.
struct Scratch {
  holo_handle h;
  cudaStream_t s;
  std::vector<void *> ptrs;
  Scratch(holo_handle h_, cudaStream_t s_) : h(h_), s(s_) {}
  ~Scratch() {
    for (void *p : ptrs) pool_free(p, s);
  }
  template <typename T>
  T *get(size_t count) {
    void *p = pool_alloc(h, count * sizeof(T) + 16, s);
    if (p) ptrs.push_back(p);
    return static_cast<T *>(p);
  }
};

int default_fp64_variant(size_t N, size_t M) {
  (void)N;
  (void)M;
  return 0;
}

// Choose the number of source splits S for T target tiles over n_src source
// tiles and G resident CTAs: minimise ceil(T S / G) * (n_src / S + overhead).
int choose_splits(int T, int n_src, int G, size_t M, int max_scratch_splits) {
  if (T <= 0 || n_src <= 0) return 1;
  double best = 1e300;
  int best_s = 1;
  const int cap = std::max(1, std::min(n_src, max_scratch_splits));
  for (int S = 1; S <= cap; ++S) {
    const long long items = (long long)T * S;
    const long long waves = (items + G - 1) / G;
    const double per_item = ceil((double)n_src / S) + 0.35;
    const double cost = waves * per_item;
    if (cost < best * 0.999) {
      best = cost;
      best_s = S;
    }
  }
  (void)M;
  return best_s;
}

}  // namespace

void *pool_alloc(holo_handle h, size_t bytes, cudaStream_t s) {
  void *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (cudaMallocFromPoolAsync(&p, bytes, h->pool, s) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void pool_free(void *p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

int size_bucket(size_t N, size_t M) {
  const double pairs = (double)N * (double)M;
  int b = 0;
  if (pairs >= 1e7) b = 1;
  if (pairs >= 1e8) b = 2;
  if (pairs >= 1e9) b = 3;
  if (pairs >= 1e10) b = 4;
  if (pairs >= 1e11) b = 5;
  if (M < 4096) b = 6 + (M >= 1024 ? 1 : 0);  // few targets: split-heavy buckets
  return b;
}

// ---- plans ------------------------------------------------------------------------
static int alloc_plan(holo_plan_s *p, void **dst, size_t bytes, cudaStream_t s) {
  void *q = pool_alloc(p->h, bytes, s);
  if (!q) return fail(HOLO_ERR_ALLOC, "device allocation of %zu bytes failed", bytes);
  p->owned.push_back(q);
  *dst = q;
  return HOLO_OK;
}

void plan_release(holo_plan_s *p, cudaStream_t s) {
  if (!p) return;
  if (p->transposed) plan_release(p->transposed, s);
  for (void *q : p->owned) pool_free(q, s);
  delete p;
}

// Tile order of a point set into the plan's buffers (the order does not depend on
// the tile size), or `known`, the order another plan computed for the same array.
static int order_set(holo_plan_s *p, const double *pos, int n, int n_pad, double *pos_sorted,
                     int32_t *order, cudaStream_t s, const int32_t *known, int tiling) {
  if (n == 0) return launch_gather_pos(pos, nullptr, 0, n_pad, pos_sorted, s);
  if (known) {
    HOLO_CUDA(cudaMemcpyAsync(order, known, (size_t)n * sizeof(int32_t),
                              cudaMemcpyDeviceToDevice, s));
    return launch_gather_pos(pos, order, n, n_pad, pos_sorted, s);
  }
  Scratch tmp(p->h, s);
  const size_t hist_n = sort_hist_entries(n);
  TileScratch t{};
  t.bbox = tmp.get<double>(6);
  t.bbox_scratch = tmp.get<double>(6 * 1024);
  t.keys = tmp.get<uint16_t>(n);
  t.keys2 = tmp.get<uint16_t>(n);
  t.hist = tmp.get<uint32_t>(hist_n);
  t.scan = tmp.get<uint32_t>(hist_n + 4096 + 16);
  t.tmp_a = tmp.get<int32_t>(n);
  t.tmp_b = tmp.get<int32_t>(n);
  if (!t.bbox || !t.bbox_scratch || !t.keys || !t.keys2 || !t.hist || !t.scan || !t.tmp_a ||
      !t.tmp_b)
    return fail(HOLO_ERR_ALLOC, "tiler scratch");
  HOLO_TRY(tile_order(pos, n, order, t, s, tiling));
  HOLO_TRY(launch_gather_pos(pos, order, n, n_pad, pos_sorted, s));
  return HOLO_OK;
}

// Error model of the split path (declared in internal.cuh), in metres of path
// length.  gap = distance between the two point sets' boxes (r >= gap),
// c = |d_perp|^2 <= (h_s + h_t)^2 over the worst tile pair, rho = c / 2r:
//   base = FP32 rounding of rho (~4 ulp) and of the in-tile offsets
//          (c / r * 2^-24), and the truncated series term rho (c / r^2)^2 / 8;
//   curv = c^2 / 8r^3 = rho (c / r^2) / 4;
//   lin  = for 1/q ~ (1 + x) / Qt, x = Ps / Qt: the phase error rho x^2 / (1 - x)
//          plus the relative amplitude error of 1/r ~ (1 + Ps / r0) / Qt,
//          x^2 + c / 2q^2 + |Ps| h_t / (Qt r0), as the path length of the same
//          phase at 400 nm.  |Ps| = |e.s'| <= sum_d |e_d| hd_s[d] with
//   gemm = rho 2^-22: the curvature term of pair model 3 comes from 3xTF32
//          tensor-core products (each ~2^-22 relative) summed in the FP32
//          accumulator, taken as 4 more ulps than the FP32 evaluation in base.
//          |e_d| <= min(1, span_d / gap) (span_d: the largest target-source
//          coordinate difference along d), and Qt >= gap - h_t.
void split_error_model(const TileStats &st, double *base, double *curv, double *lin,
                       double *gemm) {
  double gap2 = 0.0, ps = 0.0;
  for (int d = 0; d < 3; ++d) {
    const double g = std::max(0.0, std::max(st.lo_s[d] - st.hi_t[d], st.lo_t[d] - st.hi_s[d]));
    gap2 += g * g;
  }
  const double gap = sqrt(gap2);
  if (!(gap > 0.0)) {
    *base = *curv = *lin = *gemm = INFINITY;
    return;
  }
  for (int d = 0; d < 3; ++d) {
    const double span = std::max(fabs(st.hi_t[d] - st.lo_s[d]), fabs(st.hi_s[d] - st.lo_t[d]));
    ps += std::min(1.0, span / gap) * st.hd_s[d];
  }
  const double c = (st.h_s + st.h_t) * (st.h_s + st.h_t), rho = c / (2.0 * gap), y = c / gap2;
  *base = rho * ldexp(1.0, -21) + c / gap * ldexp(1.0, -24) + rho * y * y / 8.0;
  *curv = rho * y / 4.0;
  *gemm = rho * ldexp(1.0, -22);
  const double qt = gap - st.h_t, x = qt > 0.0 ? ps / qt : INFINITY;
  if (!(x < 0.5)) {
    *lin = INFINITY;
    return;
  }
  const double x2 = x * x / (1.0 - x);
  *lin = rho * x2 + (x2 + y / 2.0 + ps * st.h_t / (qt * gap)) * (400e-9 / (2.0 * M_PI));
}

// Tile boxes for source tiles of `cs` and target tiles of `tt` points, and the
// split-path error model of that tiling.
static int tile_error_bound(holo_plan_s *p, int cs, int tt, double *bound, double *curv,
                            double *lin, double *gemm, cudaStream_t s) {
  const int ns = (p->N + cs - 1) / cs, nt = (p->M + tt - 1) / tt;
  HOLO_TRY(launch_tile_bbox(p->pos_s, p->N, cs, p->tiles_s, s));
  HOLO_TRY(launch_tile_bbox(p->pos_t, p->M, tt, p->tiles_t, s));
  if (ns == 0 || nt == 0) {
    *bound = *curv = *lin = *gemm = 0.0;
    return HOLO_OK;
  }
  std::vector<double> ts((size_t)6 * ns), tg((size_t)6 * nt);
  HOLO_CUDA(cudaMemcpyAsync(ts.data(), p->tiles_s, ts.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  HOLO_CUDA(cudaMemcpyAsync(tg.data(), p->tiles_t, tg.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  HOLO_CUDA(cudaStreamSynchronize(s));
  auto boxes = [](const std::vector<double> &t, int n, double *lo, double *hi, double *hmax,
                  double *hd) {
    for (int d = 0; d < 3; ++d) { lo[d] = 1e300; hi[d] = -1e300; hd[d] = 0.0; }
    *hmax = 0.0;
    for (int i = 0; i < n; ++i) {
      const double *c = &t[6 * (size_t)i];
      double h2 = 0.0;
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], c[d] - c[3 + d]);
        hi[d] = std::max(hi[d], c[d] + c[3 + d]);
        hd[d] = std::max(hd[d], c[3 + d]);
        h2 += c[3 + d] * c[3 + d];
      }
      *hmax = std::max(*hmax, sqrt(h2));
    }
  };
  TileStats st;
  boxes(ts, ns, st.lo_s, st.hi_s, &st.h_s, st.hd_s);
  boxes(tg, nt, st.lo_t, st.hi_t, &st.h_t, st.hd_t);
  split_error_model(st, bound, curv, lin, gemm);
  return HOLO_OK;
}


int plan_create_impl(holo_handle h, const double *u, size_t N, const double *v, size_t M,
                     int precision, int forced_variant, cudaStream_t s, holo_plan_s **out,
                     const int32_t *known_order_s, const int32_t *known_order_t,
                     int known_tiling_s, int known_tiling_t) {
  if (precision != HOLO_FP64 && precision != HOLO_SPLIT32)
    return fail(HOLO_ERR_INVALID, "unknown precision %d", precision);
  HOLO_TRY(check_sizes(N, M));
  std::unique_ptr<holo_plan_s> p(new holo_plan_s());
  p->h = h;
  p->precision = precision;
  p->N = (int)N;
  p->M = (int)M;
  p->last_stream = s;
  const int bucket = size_bucket(N, M);
  const int nv = precision == HOLO_SPLIT32 ? split_variant_count() : fp64_variant_count();
  if (forced_variant >= nv) return fail(HOLO_ERR_INVALID, "variant %d out of range", forced_variant);
  // FP64: the forced, tuned or default variant; split: chosen below by error bound
  int variant = forced_variant;
  if (variant < 0 && precision == HOLO_FP64) {
    variant = h->variant_table[precision][bucket];
    if (variant < 0) variant = default_fp64_variant(N, M);
  }

  if (precision == HOLO_SPLIT32) {
    // tile order (independent of the tile size, so one order serves every
    // candidate); pad sources to a multiple of every source tile size (3072 =
    // lcm of 1024 and 768; the others divide 1024)
    p->n_pad = std::max<int>(1, (int)((N + 3071) / 3072)) * 3072;
    holo_plan_s *pp = p.get();
    HOLO_TRY(alloc_plan(pp, (void **)&p->pos_s, (size_t)3 * p->n_pad * sizeof(double), s));
    HOLO_TRY(alloc_plan(pp, (void **)&p->order_s, std::max<size_t>(N, 1) * sizeof(int32_t), s));
    HOLO_TRY(alloc_plan(pp, (void **)&p->pos_t, (size_t)3 * std::max<size_t>(M, 1) * sizeof(double), s));
    HOLO_TRY(alloc_plan(pp, (void **)&p->order_t, std::max<size_t>(M, 1) * sizeof(int32_t), s));
    HOLO_TRY(alloc_plan(pp, (void **)&p->tiles_s, (size_t)6 * (N / 256 + 1) * sizeof(double), s));
    HOLO_TRY(alloc_plan(pp, (void **)&p->tiles_t, (size_t)6 * (M / 256 + 1) * sizeof(double), s));
    auto order_both = [&](int tiling, const int32_t *ks, const int32_t *kt) -> int {
      HOLO_TRY(order_set(pp, u, (int)N, p->n_pad, p->pos_s, p->order_s, s, ks, tiling));
      HOLO_TRY(order_set(pp, v, (int)M, (int)M, p->pos_t, p->order_t, s, kt, tiling));
      p->tiling_s = ks ? known_tiling_s : tiling;
      p->tiling_t = kt ? known_tiling_t : tiling;
      return HOLO_OK;
    };
    // candidates: a forced variant alone; else the variant tuned for this size
    // bucket, then the preference list (fastest first, ever smaller tiles); the
    // first whose path-length error bound holds is taken (sparse, wide or close
    // point sets need small tiles and the curvature correction)
    std::vector<int> cands;
    if (forced_variant >= 0) {
      cands.push_back(forced_variant);
    } else {
      if (h->variant_table[precision][bucket] >= 0) cands.push_back(h->variant_table[precision][bucket]);
      for (int c : split_preferences(N, M)) cands.push_back(c);
    }
    // the first candidate whose bound holds on the current tiles (else the last);
    // leaves that candidate's tile boxes in tiles_s / tiles_t
    auto choose = [&](size_t *chosen) -> int {
      int shape_tt = -1, shape_cs = -1;
      double mb[4] = {0.0, 0.0, 0.0, 0.0};
      for (size_t i = 0; i < cands.size(); ++i) {
        const Variant C = split_variant(cands[i]);
        if (C.tt() != shape_tt || C.cs != shape_cs) {
          double bound = 0.0, curv = 0.0, lin = 0.0, gemm = 0.0;
          HOLO_TRY(tile_error_bound(pp, C.cs, C.tt(), &bound, &curv, &lin, &gemm, s));
          mb[0] = bound;
          mb[1] = bound + curv;
          mb[2] = mb[1] + lin;
          mb[3] = mb[2] + gemm;
          shape_tt = C.tt();
          shape_cs = C.cs;
        }
        variant = cands[i];
        *chosen = i;
        for (int m = 0; m < 4; ++m) p->model_bounds[m] = mb[m];
        p->err_bound = mb[C.model];
        if (p->err_bound <= kSplitBoundMetres) break;
      }
      return HOLO_OK;
    };
    // Hilbert tiles first (cheap); where their bound rules out the first candidate,
    // the packed tiles (narrower for most point counts) get a second try, and the
    // tiling that admits the earlier candidate is kept
    size_t ci = 0;
    HOLO_TRY(order_both(kTileHilbert, known_order_s, known_order_t));
    HOLO_TRY(choose(&ci));
    if (ci > 0 && forced_variant < 0) {
      size_t cp = 0;
      HOLO_TRY(order_both(kTilePacked, nullptr, nullptr));
      HOLO_TRY(choose(&cp));
      if (cp >= ci) {  // no gain: back to the Hilbert tiles
        HOLO_TRY(order_both(kTileHilbert, nullptr, nullptr));
        HOLO_TRY(choose(&ci));
      }
    }
  }
  const Variant V = precision == HOLO_SPLIT32 ? split_variant(variant) : fp64_variant(variant);
  p->variant = variant;
  p->n_stiles = (int)((N + V.cs - 1) / V.cs);
  if (precision != HOLO_SPLIT32) p->n_pad = std::max(p->n_stiles, 1) * V.cs;
  p->n_ttiles = (int)((M + V.tt() - 1) / V.tt());

  int occ = 0;
  if (precision == HOLO_SPLIT32) {
    HOLO_TRY(split_occupancy(variant, false, &occ));
  } else {
    HOLO_TRY(fp64_occupancy(variant, &occ));
  }
  const int G = std::max(1, occ) * h->sm_count;
  const size_t scratch_cap = (size_t)1 << 30;  // partial sums at most 1 GiB
  const int max_splits = (int)std::max<size_t>(1, scratch_cap / (std::max<size_t>(M, 1) * 16));
  p->splits = choose_splits(p->n_ttiles, p->n_stiles, G, M, max_splits);
  p->grid = std::max(1, std::min(G, p->n_ttiles * p->splits));

  if (precision == HOLO_SPLIT32) {
    // float-float offsets of every point from its tile's centre (tiles of the
    // chosen variant, whose boxes the last bound evaluation left in tiles_s/t)
    HOLO_TRY(alloc_plan(p.get(), (void **)&p->geo_s, (size_t)6 * p->n_pad * sizeof(float), s));
    HOLO_TRY(alloc_plan(p.get(), (void **)&p->geo_t, (size_t)6 * std::max<size_t>(M, 1) * sizeof(float), s));
    HOLO_TRY(launch_rel_hilo(p->pos_s, (int)N, p->n_pad, p->tiles_s, V.cs, p->geo_s, s));
    HOLO_TRY(launch_rel_hilo(p->pos_t, (int)M, (int)M, p->tiles_t, V.tt(), p->geo_t, s));
  } else {
    HOLO_TRY(alloc_plan(p.get(), (void **)&p->pos_s, (size_t)3 * p->n_pad * sizeof(double), s));
    HOLO_TRY(alloc_plan(p.get(), (void **)&p->pos_t, (size_t)3 * std::max<size_t>(M, 1) * sizeof(double), s));
    HOLO_TRY(launch_pack_pos(u, (int)N, p->n_pad, p->pos_s, s));
    p->tiling_s = p->tiling_t = -1;  // the caller's order
    if (M) HOLO_CUDA(cudaMemcpyAsync(p->pos_t, v, 3 * M * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  // keep original-order positions for the adjoint's transposed plan
  double *u_keep = nullptr, *v_keep = nullptr;
  HOLO_TRY(alloc_plan(p.get(), (void **)&u_keep, 3 * std::max<size_t>(N, 1) * sizeof(double), s));
  HOLO_TRY(alloc_plan(p.get(), (void **)&v_keep, 3 * std::max<size_t>(M, 1) * sizeof(double), s));
  if (N) HOLO_CUDA(cudaMemcpyAsync(u_keep, u, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (M) HOLO_CUDA(cudaMemcpyAsync(v_keep, v, 3 * M * sizeof(double), cudaMemcpyDeviceToDevice, s));
  p->u_orig = u_keep;
  p->v_orig = v_keep;
  *out = p.release();
  return HOLO_OK;
}

int plan_execute_impl(holo_plan_s *p, int sign, double lambda, const double *amp,
                      const double *phase, double2 *y, int flags, cudaStream_t s) {
  HOLO_TRY(check_sign(sign));
  if (!finite_positive(lambda)) return fail(HOLO_ERR_INVALID, "lambda must be finite and > 0");
  p->last_stream = s;
  if (p->M == 0) return HOLO_OK;
  if (p->N == 0) {
    HOLO_CUDA(cudaMemsetAsync(y, 0, (size_t)p->M * sizeof(double2), s));
    return HOLO_OK;
  }
  Scratch tmp(p->h, s);
  double2 *ap = tmp.get<double2>(p->n_pad);
  double2 *partial = p->splits > 1 ? tmp.get<double2>((size_t)p->splits * p->M) : nullptr;
  if (!ap || (p->splits > 1 && !partial)) return fail(HOLO_ERR_ALLOC, "execute scratch");
  const double k = (2.0 * M_PI) / lambda;
  const bool cst = (flags & HOLO_FLAG_CONST_PHASE) != 0;
  if (p->precision == HOLO_SPLIT32) {
    float2 *apf = reinterpret_cast<float2 *>(ap);  // n_pad float pairs fit in the buffer
    HOLO_TRY(launch_gather_apf(amp, phase, p->order_s, p->N, p->n_pad, apf, s));
    SplitProblem P{};
    P.geo_s = p->geo_s;
    P.apf_s = apf;
    P.geo_t = p->geo_t;
    P.pos_s = p->pos_s;
    P.ap_s = nullptr;
    P.tiles_s = p->tiles_s;
    P.pos_t = p->pos_t;
    P.tiles_t = p->tiles_t;
    P.order_t = p->order_t;
    P.partial = partial;
    P.y = y;
    P.N = p->N;
    P.M = p->M;
    P.n_stiles = p->n_stiles;
    P.n_ttiles = p->n_ttiles;
    P.splits = p->splits;
    P.sign = sign;
    P.sk = sign * k;
    P.sub = 1;
    HOLO_TRY(profile_mark(p->h, s, true));
    HOLO_TRY(launch_split(P, p->variant, p->grid, cst, false, p->h->dev_err, s));
    HOLO_TRY(profile_mark(p->h, s, false));
    if (p->splits > 1) HOLO_TRY(launch_reduce(partial, p->splits, p->M, p->order_t, y, s));
  } else {
    HOLO_TRY(launch_pack_ap(amp, phase, p->N, p->n_pad, ap, s));
    Fp64Problem P{};
    P.pos_s = p->pos_s;
    P.ap_s = ap;
    P.pos_t = p->pos_t;
    P.partial = partial;
    P.y = y;
    P.N = p->N;
    P.M = p->M;
    P.n_stiles = p->n_stiles;
    P.n_ttiles = p->n_ttiles;
    P.splits = p->splits;
    P.sign = sign;
    P.k = k;
    HOLO_TRY(profile_mark(p->h, s, true));
    HOLO_TRY(launch_fp64(P, p->variant, p->grid, cst, p->h->dev_err, s));
    HOLO_TRY(profile_mark(p->h, s, false));
    if (p->splits > 1) HOLO_TRY(launch_reduce(partial, p->splits, p->M, nullptr, y, s));
  }
  return HOLO_OK;
}

// Monte Carlo needs a plan whose target tile equals the block size and whose
// source tiles match the variant's CS: build one for the requested block.
static int mc_variant_for_block(int block) {
  for (int v = 0; v < split_variant_count(); ++v)
    if (split_variant(v).tt() == block) return v;
  return -1;
}

static int plan_execute_mc_impl(holo_plan_s *p, int sign, double lambda, const double *amp,
                                const double *phase, double2 *y, uint64_t seed, int sub,
                                int block, cudaStream_t s) {
  HOLO_TRY(check_sign(sign));
  if (!finite_positive(lambda)) return fail(HOLO_ERR_INVALID, "lambda must be finite and > 0");
  if (p->precision != HOLO_SPLIT32)
    return fail(HOLO_ERR_INVALID, "the Monte Carlo estimator runs in HOLO_SPLIT32 only");
  if (sub < 1) return fail(HOLO_ERR_INVALID, "subsample must be >= 1");
  const int v = mc_variant_for_block(block);
  if (v < 0) return fail(HOLO_ERR_INVALID, "targets_per_block %d: use 256, 512, 1024 or 2048", block);
  p->last_stream = s;
  if (p->M == 0) return HOLO_OK;
  if (p->N == 0) {
    HOLO_CUDA(cudaMemsetAsync(y, 0, (size_t)p->M * sizeof(double2), s));
    return HOLO_OK;
  }
  const Variant V = split_variant(v);
  const int n_stiles = (p->N + V.cs - 1) / V.cs, n_ttiles = (p->M + V.tt() - 1) / V.tt();
  const int n_strata = (p->N + sub - 1) / sub;
  const int n_chunks = (n_strata + V.cs - 1) / V.cs;
  int occ = 0;
  HOLO_TRY(split_occupancy(v, true, &occ));
  const int G = std::max(1, occ) * p->h->sm_count;
  const int max_splits = (int)std::max<size_t>(1, ((size_t)1 << 30) / ((size_t)p->M * 16));
  const int splits = choose_splits(n_ttiles, n_chunks, G, p->M, max_splits);
  Scratch tmp(p->h, s);
  double2 *ap = tmp.get<double2>(p->n_pad);
  double2 *partial = splits > 1 ? tmp.get<double2>((size_t)splits * p->M) : nullptr;
  if (!ap || (splits > 1 && !partial)) return fail(HOLO_ERR_ALLOC, "execute scratch");
  // tile boxes for the Monte Carlo block size when the plan was tiled differently
  const double *tiles_s = p->tiles_s, *tiles_t = p->tiles_t;
  const float *geo_t = p->geo_t;
  if (v != p->variant) {
    double *ts = tmp.get<double>((size_t)6 * n_stiles);
    double *tt = tmp.get<double>((size_t)6 * n_ttiles);
    float *gt = tmp.get<float>((size_t)6 * p->M);
    if (!ts || !tt || !gt) return fail(HOLO_ERR_ALLOC, "execute scratch");
    HOLO_TRY(launch_tile_bbox(p->pos_s, p->N, V.cs, ts, s));
    HOLO_TRY(launch_tile_bbox(p->pos_t, p->M, V.tt(), tt, s));
    HOLO_TRY(launch_rel_hilo(p->pos_t, p->M, p->M, tt, V.tt(), gt, s));
    tiles_s = ts;
    tiles_t = tt;
    geo_t = gt;
  }
  HOLO_TRY(launch_gather_ap(amp, phase, p->order_s, p->N, p->n_pad, ap, s));
  SplitProblem P{};
  P.geo_t = geo_t;
  P.pos_s = p->pos_s;
  P.ap_s = ap;
  P.tiles_s = tiles_s;
  P.pos_t = p->pos_t;
  P.tiles_t = tiles_t;
  P.order_t = p->order_t;
  P.partial = partial;
  P.y = y;
  P.N = p->N;
  P.M = p->M;
  P.n_stiles = n_stiles;
  P.n_ttiles = n_ttiles;
  P.splits = splits;
  P.sign = sign;
  P.sk = sign * ((2.0 * M_PI) / lambda);
  P.seed_lo = (uint32_t)seed;
  P.seed_hi = (uint32_t)(seed >> 32);
  P.sub = sub;
  const int grid = std::max(1, std::min(G, n_ttiles * splits));
  HOLO_TRY(profile_mark(p->h, s, true));
  HOLO_TRY(launch_split(P, v, grid, false, true, p->h->dev_err, s));
  HOLO_TRY(profile_mark(p->h, s, false));
  if (splits > 1) HOLO_TRY(launch_reduce(partial, splits, p->M, p->order_t, y, s));
  return HOLO_OK;
}

static int read_device_error(holo_handle h, cudaStream_t s) {
  int e = 0;
  HOLO_CUDA(cudaMemcpyAsync(&e, h->dev_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  HOLO_CUDA(cudaStreamSynchronize(s));
  if (e) {
    cudaMemsetAsync(h->dev_err, 0, sizeof(int), s);
    return fail(HOLO_ERR_TIMEOUT, "a device-side wait ran out of time (code %d)", e);
  }
  return HOLO_OK;
}

// Host-pointer calls: stage inputs on the device, run, copy results back.
struct Staged {
  Scratch sc;
  explicit Staged(holo_handle h, cudaStream_t s) : sc(h, s) {}
  int up(const double *src, size_t count, const double **dst) {
    if (!src || count == 0) {
      *dst = nullptr;
      return HOLO_OK;
    }
    double *d = sc.get<double>(count);
    if (!d) return fail(HOLO_ERR_ALLOC, "staging allocation");
    HOLO_CUDA(cudaMemcpyAsync(d, src, count * sizeof(double), cudaMemcpyHostToDevice, sc.s));
    *dst = d;
    return HOLO_OK;
  }
  int out(size_t count, double **dst) {
    double *d = sc.get<double>(std::max<size_t>(count, 1));
    if (!d) return fail(HOLO_ERR_ALLOC, "staging allocation");
    *dst = d;
    return HOLO_OK;
  }
};

}  // namespace holo

using namespace holo;

// =================================================================================
extern "C" {

int holo_abi_version(void) { return HOLO_ABI_VERSION; }

const char *holo_last_error_string(void) { return g_error.c_str(); }

int holo_create(int device, holo_handle *out) {
  if (!out) return fail(HOLO_ERR_INVALID, "null output handle");
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(HOLO_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= count) return fail(HOLO_ERR_INVALID, "device %d out of range", device);
  DeviceGuard g(device);
  if (!g.ok) return fail(HOLO_ERR_NO_DEVICE, "cannot select device %d", device);
  std::unique_ptr<holo_handle_s> h(new holo_handle_s());
  h->device = device;
  HOLO_CUDA(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device));
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  HOLO_CUDA(cudaMemPoolCreate(&h->pool, &props));
  uint64_t thr = UINT64_MAX;
  HOLO_CUDA(cudaMemPoolSetAttribute(h->pool, cudaMemPoolAttrReleaseThreshold, &thr));
  HOLO_CUDA(cudaMalloc(&h->dev_err, sizeof(int)));
  HOLO_CUDA(cudaMemset(h->dev_err, 0, sizeof(int)));
  *out = h.release();
  return HOLO_OK;
}

int holo_destroy(holo_handle h) {
  if (!h) return HOLO_OK;
  {
    DeviceGuard g(h->device);
    cudaDeviceSynchronize();
    if (h->dev_err) cudaFree(h->dev_err);
    if (h->pool) cudaMemPoolDestroy(h->pool);
  }
  delete h;
  return HOLO_OK;
}

int holo_device_status(holo_handle h, holo_stream_t stream) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  return read_device_error(h, (cudaStream_t)stream);
}

int holo_plan_create(holo_handle h, const double *u_xyz, size_t N, const double *v_xyz,
                     size_t M, int precision, holo_stream_t stream, holo_plan *out) {
  if (!h || !out) return fail(HOLO_ERR_INVALID, "null handle or output");
  if ((N && !u_xyz) || (M && !v_xyz)) return fail(HOLO_ERR_INVALID, "null position array");
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  cudaStream_t s = (cudaStream_t)stream;
  bool dev = false;
  HOLO_TRY(classify_all({u_xyz, v_xyz}, &dev));
  if (dev) return plan_create_impl(h, u_xyz, N, v_xyz, M, precision, -1, s, out);
  Staged st(h, s);
  const double *du, *dv;
  HOLO_TRY(st.up(u_xyz, 3 * N, &du));
  HOLO_TRY(st.up(v_xyz, 3 * M, &dv));
  HOLO_TRY(plan_create_impl(h, du, N, dv, M, precision, -1, s, out));
  HOLO_CUDA(cudaStreamSynchronize(s));
  return HOLO_OK;
}

int holo_plan_destroy(holo_plan p) {
  if (!p) return HOLO_OK;
  holo_handle h = p->h;
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  plan_release(p, p->last_stream);
  return HOLO_OK;
}

int holo_plan_info(holo_plan p, int *variant, int *splits, int *target_tile, int *source_tile) {
  if (!p) return fail(HOLO_ERR_INVALID, "null plan");
  const Variant V = p->precision == HOLO_SPLIT32 ? split_variant(p->variant) : fp64_variant(p->variant);
  if (variant) *variant = p->variant;
  if (splits) *splits = p->splits;
  if (target_tile) *target_tile = V.tt();
  if (source_tile) *source_tile = V.cs;
  return HOLO_OK;
}

int holo_plan_error_bound(holo_plan p, double *metres) {
  if (!p || !metres) return fail(HOLO_ERR_INVALID, "null argument");
  *metres = p->precision == HOLO_SPLIT32 ? p->err_bound : 0.0;
  return HOLO_OK;
}

int holo_plan_tiling(holo_plan p, int *tiling_sources, int *tiling_targets) {
  if (!p) return fail(HOLO_ERR_INVALID, "null plan");
  if (tiling_sources) *tiling_sources = p->tiling_s;
  if (tiling_targets) *tiling_targets = p->tiling_t;
  return HOLO_OK;
}

int holo_tile_order(holo_handle h, const double *xyz, size_t n, int tiling, int32_t *order,
                    holo_stream_t stream) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  if (tiling != HOLO_TILE_HILBERT && tiling != HOLO_TILE_PACKED)
    return fail(HOLO_ERR_INVALID, "unknown tiling %d", tiling);
  if (n && (!xyz || !order)) return fail(HOLO_ERR_INVALID, "null point or order array");
  HOLO_TRY(check_sizes(n, 0));
  if (n == 0) return HOLO_OK;
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  cudaStream_t s = (cudaStream_t)stream;
  bool dev = false;
  HOLO_TRY(classify_all({xyz}, &dev));
  Staged st(h, s);
  const double *dxyz = xyz;
  if (!dev) HOLO_TRY(st.up(xyz, 3 * n, &dxyz));
  Scratch tmp(h, s);
  const size_t hist_n = sort_hist_entries((int)n);
  TileScratch t{};
  t.bbox = tmp.get<double>(6);
  t.bbox_scratch = tmp.get<double>(6 * 1024);
  t.keys = tmp.get<uint16_t>(n);
  t.keys2 = tmp.get<uint16_t>(n);
  t.hist = tmp.get<uint32_t>(hist_n);
  t.scan = tmp.get<uint32_t>(hist_n + 4096 + 16);
  t.tmp_a = tmp.get<int32_t>(n);
  t.tmp_b = tmp.get<int32_t>(n);
  int32_t *dorder = tmp.get<int32_t>(n);
  if (!t.bbox || !t.bbox_scratch || !t.keys || !t.keys2 || !t.hist || !t.scan || !t.tmp_a ||
      !t.tmp_b || !dorder)
    return fail(HOLO_ERR_ALLOC, "tiler scratch");
  HOLO_TRY(tile_order(dxyz, (int)n, dorder, t, s, tiling));
  HOLO_CUDA(cudaMemcpyAsync(order, dorder, n * sizeof(int32_t), cudaMemcpyDefault, s));
  HOLO_CUDA(cudaStreamSynchronize(s));
  return HOLO_OK;
}

int holo_plan_get_order(holo_plan p, int which, int32_t *out) {
  if (!p || !out) return fail(HOLO_ERR_INVALID, "null plan or output");
  const int n = which == 0 ? p->N : p->M;
  if (n == 0) return HOLO_OK;
  std::lock_guard<std::mutex> lk(p->h->mu);
  DeviceGuard g(p->h->device);
  const int32_t *src = which == 0 ? p->order_s : p->order_t;
  if (p->precision != HOLO_SPLIT32 || !src) {
    for (int i = 0; i < n; ++i) out[i] = i;
    return HOLO_OK;
  }
  HOLO_CUDA(cudaStreamSynchronize(p->last_stream));
  HOLO_CUDA(cudaMemcpy(out, src, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return HOLO_OK;
}

static int execute_any(holo_plan p, int sign, double lambda, const double *amp,
                       const double *phase, double *y, int flags, cudaStream_t s, bool mc,
                       uint64_t seed, int sub, int block) {
  if (!p) return fail(HOLO_ERR_INVALID, "null plan");
  if (p->M && !y) return fail(HOLO_ERR_INVALID, "null output");
  if (p->N && (!amp || !phase)) return fail(HOLO_ERR_INVALID, "null amplitude or phase");
  holo_handle h = p->h;
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  bool dev = false;
  HOLO_TRY(classify_all({amp, phase, y}, &dev));
  auto run = [&](const double *a, const double *ph, double *yo) {
    return mc ? plan_execute_mc_impl(p, sign, lambda, a, ph, (double2 *)yo, seed, sub, block, s)
              : plan_execute_impl(p, sign, lambda, a, ph, (double2 *)yo, flags, s);
  };
  if (dev) return run(amp, phase, y);
  Staged st(h, s);
  const double *da, *dp;
  double *dy;
  HOLO_TRY(st.up(amp, p->N, &da));
  HOLO_TRY(st.up(phase, p->N, &dp));
  HOLO_TRY(st.out(2 * (size_t)p->M, &dy));
  HOLO_TRY(run(da, dp, dy));
  if (p->M) HOLO_CUDA(cudaMemcpyAsync(y, dy, 2 * (size_t)p->M * sizeof(double), cudaMemcpyDeviceToHost, s));
  return read_device_error(h, s);
}

int holo_plan_execute(holo_plan p, int sign, double lambda, const double *amp,
                      const double *phase, double *y_re_im, holo_stream_t stream) {
  return execute_any(p, sign, lambda, amp, phase, y_re_im, 0, (cudaStream_t)stream, false, 0, 1, 0);
}

int holo_plan_execute_flags(holo_plan p, int sign, double lambda, const double *amp,
                            const double *phase, double *y_re_im, int flags,
                            holo_stream_t stream) {
  return execute_any(p, sign, lambda, amp, phase, y_re_im, flags, (cudaStream_t)stream, false, 0,
                     1, 0);
}

int holo_plan_execute_mc(holo_plan p, int sign, double lambda, const double *amp,
                         const double *phase, double *y_re_im, uint64_t seed, int subsample,
                         int targets_per_block, holo_stream_t stream) {
  return execute_any(p, sign, lambda, amp, phase, y_re_im, 0, (cudaStream_t)stream, true, seed,
                     subsample, targets_per_block);
}

// One-shot calls: plan, execute, release (stream-ordered frees).
static int one_shot(holo_handle h, int sign, double lambda, const double *amp,
                    const double *phase, const double *u, size_t N, const double *v, size_t M,
                    double *y, int precision, int forced_variant, cudaStream_t s, bool mc,
                    uint64_t seed, int sub, int block) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  if ((N && (!amp || !phase || !u)) || (M && (!v || !y)))
    return fail(HOLO_ERR_INVALID, "null input or output array");
  HOLO_TRY(check_sign(sign));
  if (!finite_positive(lambda)) return fail(HOLO_ERR_INVALID, "lambda must be finite and > 0");
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  bool dev = false;
  HOLO_TRY(classify_all({amp, phase, u, v, y}, &dev));
  Staged st(h, s);
  const double *da = amp, *dp = phase, *du = u, *dv = v;
  double *dy = y;
  if (!dev) {
    HOLO_TRY(st.up(amp, N, &da));
    HOLO_TRY(st.up(phase, N, &dp));
    HOLO_TRY(st.up(u, 3 * N, &du));
    HOLO_TRY(st.up(v, 3 * M, &dv));
    HOLO_TRY(st.out(2 * M, &dy));
  }
  if (mc) {
    forced_variant = mc_variant_for_block(block);
    if (forced_variant < 0)
      return fail(HOLO_ERR_INVALID, "targets_per_block %d: use 256, 512, 1024 or 2048", block);
  }
  holo_plan_s *p = nullptr;
  HOLO_TRY(plan_create_impl(h, du, N, dv, M, precision, forced_variant, s, &p));
  const int rc = mc ? plan_execute_mc_impl(p, sign, lambda, da, dp, (double2 *)dy, seed, sub, block, s)
                    : plan_execute_impl(p, sign, lambda, da, dp, (double2 *)dy, 0, s);
  plan_release(p, s);
  HOLO_TRY(rc);
  if (!dev) {
    if (M) HOLO_CUDA(cudaMemcpyAsync(y, dy, 2 * M * sizeof(double), cudaMemcpyDeviceToHost, s));
    return read_device_error(h, s);
  }
  return HOLO_OK;
}

int holo_transform(holo_handle h, int sign, double lambda, const double *amp,
                   const double *phase, const double *u_xyz, size_t N, const double *v_xyz,
                   size_t M, double *y_re_im, int precision, holo_stream_t stream) {
  return one_shot(h, sign, lambda, amp, phase, u_xyz, N, v_xyz, M, y_re_im, precision, -1,
                  (cudaStream_t)stream, false, 0, 1, 0);
}

int holo_transform_variant(holo_handle h, int sign, double lambda, const double *amp,
                           const double *phase, const double *u_xyz, size_t N,
                           const double *v_xyz, size_t M, double *y_re_im, int precision,
                           int variant, holo_stream_t stream) {
  return one_shot(h, sign, lambda, amp, phase, u_xyz, N, v_xyz, M, y_re_im, precision, variant,
                  (cudaStream_t)stream, false, 0, 1, 0);
}

int holo_transform_mc(holo_handle h, int sign, double lambda, const double *amp,
                      const double *phase, const double *u_xyz, size_t N, const double *v_xyz,
                      size_t M, double *y_re_im, uint64_t seed, int subsample,
                      int targets_per_block, holo_stream_t stream) {
  if (subsample < 1) return fail(HOLO_ERR_INVALID, "subsample must be >= 1");
  return one_shot(h, sign, lambda, amp, phase, u_xyz, N, v_xyz, M, y_re_im, HOLO_SPLIT32, -1,
                  (cudaStream_t)stream, true, seed, subsample, targets_per_block);
}

// ---- adjoint -------------------------------------------------------------------
static int adjoint_impl(holo_plan_s *p, int sign, double lambda, const double *amp,
                        const double *phase, const double *grad_y, double *grad_amp,
                        double *grad_phase, cudaStream_t s) {
  HOLO_TRY(check_sign(sign));
  if (!finite_positive(lambda)) return fail(HOLO_ERR_INVALID, "lambda must be finite and > 0");
  p->last_stream = s;
  if (p->N == 0) return HOLO_OK;
  if (!p->transposed)
    HOLO_TRY(plan_create_impl(p->h, p->v_orig, p->M, p->u_orig, p->N, p->precision, -1, s,
                              &p->transposed, p->order_t, p->order_s, p->tiling_t,
                              p->tiling_s));
  Scratch tmp(p->h, s);
  double *g_amp = tmp.get<double>(std::max(p->M, 1));
  double *g_phase = tmp.get<double>(std::max(p->M, 1));
  double2 *H = tmp.get<double2>(p->N);
  if (!g_amp || !g_phase || !H) return fail(HOLO_ERR_ALLOC, "adjoint scratch");
  HOLO_TRY(launch_complex_to_polar((const double2 *)grad_y, p->M, g_amp, g_phase, s));
  // H_n = sum_m G_m e^{-i s k r_nm} / r_nm: the transform with roles swapped, sign -s
  HOLO_TRY(plan_execute_impl(p->transposed, -sign, lambda, g_amp, g_phase, H, 0, s));
  HOLO_TRY(launch_adjoint_epilogue(H, amp, phase, p->N, grad_amp, grad_phase, s));
  return HOLO_OK;
}

int holo_plan_adjoint(holo_plan p, int sign, double lambda, const double *amp,
                      const double *phase, const double *grad_y, double *grad_amp,
                      double *grad_phase, holo_stream_t stream) {
  if (!p) return fail(HOLO_ERR_INVALID, "null plan");
  if (p->N && (!amp || !phase || !grad_amp || !grad_phase))
    return fail(HOLO_ERR_INVALID, "null source array");
  if (p->M && !grad_y) return fail(HOLO_ERR_INVALID, "null grad_y");
  holo_handle h = p->h;
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  cudaStream_t s = (cudaStream_t)stream;
  bool dev = false;
  HOLO_TRY(classify_all({amp, phase, grad_y, grad_amp, grad_phase}, &dev));
  if (dev) return adjoint_impl(p, sign, lambda, amp, phase, grad_y, grad_amp, grad_phase, s);
  Staged st(h, s);
  const double *da, *dp, *dg;
  double *dga, *dgp;
  HOLO_TRY(st.up(amp, p->N, &da));
  HOLO_TRY(st.up(phase, p->N, &dp));
  HOLO_TRY(st.up(grad_y, 2 * (size_t)p->M, &dg));
  HOLO_TRY(st.out(p->N, &dga));
  HOLO_TRY(st.out(p->N, &dgp));
  HOLO_TRY(adjoint_impl(p, sign, lambda, da, dp, dg, dga, dgp, s));
  if (p->N) {
    HOLO_CUDA(cudaMemcpyAsync(grad_amp, dga, p->N * sizeof(double), cudaMemcpyDeviceToHost, s));
    HOLO_CUDA(cudaMemcpyAsync(grad_phase, dgp, p->N * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  return read_device_error(h, s);
}

int holo_adjoint(holo_handle h, int sign, double lambda, const double *amp, const double *phase,
                 const double *u_xyz, size_t N, const double *v_xyz, size_t M,
                 const double *grad_y, double *grad_amp, double *grad_phase, int precision,
                 holo_stream_t stream) {
  holo_plan p = nullptr;
  HOLO_TRY(holo_plan_create(h, u_xyz, N, v_xyz, M, precision, stream, &p));
  const int rc = holo_plan_adjoint(p, sign, lambda, amp, phase, grad_y, grad_amp, grad_phase, stream);
  holo_plan_destroy(p);
  return rc;
}

// ---- normalisation and polar output ------------------------------------------------
static int normalize_polar_dev(holo_handle h, const double2 *y, size_t M, double *amp,
                               double *phase, double *max_dev, cudaStream_t s) {
  Scratch tmp(h, s);
  double *partials = tmp.get<double>(1024);
  if (!partials) return fail(HOLO_ERR_ALLOC, "normalize scratch");
  HOLO_TRY(launch_max_abs(y, (int)M, partials, 1024, max_dev, s));
  HOLO_TRY(launch_normalize_polar(y, (int)M, max_dev, amp, phase, s));
  return HOLO_OK;
}

int holo_normalize_polar(holo_handle h, const double *y_re_im, size_t M, double *amp_out,
                         double *phase_out, double *max_amp_out, holo_stream_t stream) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  if (M && (!y_re_im || !amp_out || !phase_out)) return fail(HOLO_ERR_INVALID, "null array");
  HOLO_TRY(check_sizes(0, M));
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  cudaStream_t s = (cudaStream_t)stream;
  bool dev = false;
  HOLO_TRY(classify_all({y_re_im, amp_out, phase_out}, &dev));
  Staged st(h, s);
  const double *dy = y_re_im;
  double *da = amp_out, *dp = phase_out, *dmax = nullptr;
  HOLO_TRY(st.out(1, &dmax));
  if (!dev) {
    HOLO_TRY(st.up(y_re_im, 2 * M, &dy));
    HOLO_TRY(st.out(M, &da));
    HOLO_TRY(st.out(M, &dp));
  }
  if (M == 0) {
    if (max_amp_out) *max_amp_out = 0.0;
    return HOLO_OK;
  }
  HOLO_TRY(normalize_polar_dev(h, (const double2 *)dy, M, da, dp, dmax, s));
  if (!dev) {
    HOLO_CUDA(cudaMemcpyAsync(amp_out, da, M * sizeof(double), cudaMemcpyDeviceToHost, s));
    HOLO_CUDA(cudaMemcpyAsync(phase_out, dp, M * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  if (max_amp_out) {
    HOLO_CUDA(cudaMemcpyAsync(max_amp_out, dmax, sizeof(double), cudaMemcpyDeviceToHost, s));
    HOLO_CUDA(cudaStreamSynchronize(s));
  } else if (!dev) {
    HOLO_CUDA(cudaStreamSynchronize(s));
  }
  return HOLO_OK;
}

// ---- x -> y -> z chain ----------------------------------------------------------------
static int project_dev(holo_handle h, double lambda, const double *xa, const double *xp,
                       const double *u, size_t N, const double *v, size_t M, const double *w,
                       size_t P, double *ya, double *yp, double *za, double *zp, int precision,
                       int reference_wave, double reference_distance, cudaStream_t s) {
  Scratch tmp(h, s);
  double2 *y = tmp.get<double2>(std::max<size_t>(M, 1));
  double *mx = tmp.get<double>(2);
  double *partials = tmp.get<double>(1024);
  if (!y || !mx || !partials) return fail(HOLO_ERR_ALLOC, "project scratch");
  holo_plan_s *p1 = nullptr;
  HOLO_TRY(plan_create_impl(h, u, N, v, M, precision, -1, s, &p1));
  // p1 lives until the reference-wave and z plans have taken its tile order of v
  std::unique_ptr<holo_plan_s, void (*)(holo_plan_s *)> keep(p1, [](holo_plan_s *q) {
    plan_release(q, q->last_stream);
  });
  const int32_t *order_v = precision == HOLO_SPLIT32 ? p1->order_t : nullptr;
  const int tiling_v = p1->tiling_t;
  HOLO_TRY(plan_execute_impl(p1, HOLO_BACKWARDS, lambda, xa, xp, y, 0, s));
  int rc = HOLO_OK;
  if (!reference_wave) {
    HOLO_TRY(normalize_polar_dev(h, y, M, ya, yp, mx, s));
  } else {
    // amplitude-only projector: one unit source at (0, 0, v_z - distance),
    // Forwards (cuda/transform.cu:379-395; v[:, 2] is taken from the first target)
    double2 *yref = tmp.get<double2>(std::max<size_t>(M, 1));
    double *src = tmp.get<double>(8);
    if (!yref || !src) return fail(HOLO_ERR_ALLOC, "reference wave scratch");
    double vz = 0.0;
    if (M) {
      HOLO_CUDA(cudaMemcpyAsync(&vz, v + 2, sizeof(double), cudaMemcpyDeviceToHost, s));
      HOLO_CUDA(cudaStreamSynchronize(s));
    }
    const double host_src[5] = {0.0, 0.0, vz - reference_distance, 1.0, 0.0};  // xyz, amp, phase
    HOLO_CUDA(cudaMemcpyAsync(src, host_src, sizeof(host_src), cudaMemcpyHostToDevice, s));
    holo_plan_s *pr = nullptr;
    HOLO_TRY(plan_create_impl(h, src, 1, v, M, precision, -1, s, &pr, nullptr, order_v,
                              holo::kTileHilbert, tiling_v));
    rc = plan_execute_impl(pr, HOLO_FORWARDS, lambda, src + 3, src + 4, yref, 0, s);
    plan_release(pr, s);
    HOLO_TRY(rc);
    HOLO_TRY(launch_max_abs(y, (int)M, partials, 1024, mx, s));
    HOLO_TRY(launch_max_abs(yref, (int)M, partials, 1024, mx + 1, s));
    HOLO_TRY(launch_reference_wave(y, yref, (int)M, mx, mx + 1, ya, yp, s));
    HOLO_CUDA(cudaStreamSynchronize(s));  // host_src must outlive the copy
  }
  if (P == 0) return HOLO_OK;
  double2 *z = tmp.get<double2>(P);
  if (!z) return fail(HOLO_ERR_ALLOC, "project scratch");
  holo_plan_s *p2 = nullptr;
  HOLO_TRY(plan_create_impl(h, v, M, w, P, precision, -1, s, &p2, order_v, nullptr, tiling_v));
  rc = plan_execute_impl(p2, HOLO_FORWARDS, lambda, ya, yp, z, 0, s);
  plan_release(p2, s);
  HOLO_TRY(rc);
  return normalize_polar_dev(h, z, P, za, zp, mx, s);
}

int holo_project(holo_handle h, double lambda, const double *x_amp, const double *x_phase,
                 const double *u_xyz, size_t N, const double *v_xyz, size_t M,
                 const double *w_xyz, size_t P, double *y_amp, double *y_phase, double *z_amp,
                 double *z_phase, int precision, int reference_wave, double reference_distance,
                 holo_stream_t stream) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  if (!finite_positive(lambda)) return fail(HOLO_ERR_INVALID, "lambda must be finite and > 0");
  if ((N && (!x_amp || !x_phase || !u_xyz)) || (M && (!v_xyz || !y_amp || !y_phase)) ||
      (P && (!w_xyz || !z_amp || !z_phase)))
    return fail(HOLO_ERR_INVALID, "null input or output array");
  HOLO_TRY(check_sizes(N, M));
  HOLO_TRY(check_sizes(M, P));
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  cudaStream_t s = (cudaStream_t)stream;
  bool dev = false;
  HOLO_TRY(classify_all({x_amp, x_phase, u_xyz, v_xyz, w_xyz, y_amp, y_phase, z_amp, z_phase}, &dev));
  if (dev)
    return project_dev(h, lambda, x_amp, x_phase, u_xyz, N, v_xyz, M, w_xyz, P, y_amp, y_phase,
                       z_amp, z_phase, precision, reference_wave, reference_distance, s);
  Staged st(h, s);
  const double *da, *dp, *du, *dv, *dw;
  double *dya, *dyp, *dza = nullptr, *dzp = nullptr;
  HOLO_TRY(st.up(x_amp, N, &da));
  HOLO_TRY(st.up(x_phase, N, &dp));
  HOLO_TRY(st.up(u_xyz, 3 * N, &du));
  HOLO_TRY(st.up(v_xyz, 3 * M, &dv));
  HOLO_TRY(st.up(w_xyz, 3 * P, &dw));
  HOLO_TRY(st.out(M, &dya));
  HOLO_TRY(st.out(M, &dyp));
  if (P) {
    HOLO_TRY(st.out(P, &dza));
    HOLO_TRY(st.out(P, &dzp));
  }
  HOLO_TRY(project_dev(h, lambda, da, dp, du, N, dv, M, dw, P, dya, dyp, dza, dzp, precision,
                       reference_wave, reference_distance, s));
  if (M) {
    HOLO_CUDA(cudaMemcpyAsync(y_amp, dya, M * sizeof(double), cudaMemcpyDeviceToHost, s));
    HOLO_CUDA(cudaMemcpyAsync(y_phase, dyp, M * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  if (P) {
    HOLO_CUDA(cudaMemcpyAsync(z_amp, dza, P * sizeof(double), cudaMemcpyDeviceToHost, s));
    HOLO_CUDA(cudaMemcpyAsync(z_phase, dzp, P * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  return read_device_error(h, s);
}

// ---- variants and the autotuner --------------------------------------------------------
int holo_variant_count(int precision) {
  if (precision == HOLO_SPLIT32) return split_variant_count();
  if (precision == HOLO_FP64) return fp64_variant_count();
  return fail(HOLO_ERR_INVALID, "unknown precision %d", precision);
}

int holo_variant_describe(int precision, int variant, int *threads, int *targets_per_thread,
                          int *source_tile, int *fma_sincos_targets, int *pair_model,
                          int *pair_loop) {
  const int n = holo_variant_count(precision);
  if (n < 0) return n;
  if (variant < 0 || variant >= n) return fail(HOLO_ERR_INVALID, "variant %d out of range", variant);
  const Variant V = precision == HOLO_SPLIT32 ? split_variant(variant) : fp64_variant(variant);
  if (V.tc && !split_tc_has_build(V.cs, V.poly, V.sc))
    return fail(HOLO_ERR_INVALID, "split variant %d names no tensor-core kernel build", variant);
  if (threads) *threads = V.threads;
  if (targets_per_thread) *targets_per_thread = V.r;
  if (source_tile) *source_tile = V.cs;
  if (fma_sincos_targets) *fma_sincos_targets = V.poly;
  if (pair_model) *pair_model = V.model;
  if (pair_loop) *pair_loop = V.tc ? 3 : (V.ws ? 2 : V.packed);
  return HOLO_OK;
}

int holo_size_bucket(size_t N, size_t M) { return size_bucket(N, M); }

int holo_set_variant(holo_handle h, int precision, int bucket, int variant) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  if (precision != HOLO_FP64 && precision != HOLO_SPLIT32)
    return fail(HOLO_ERR_INVALID, "unknown precision %d", precision);
  if (bucket < 0 || bucket >= 8) return fail(HOLO_ERR_INVALID, "bucket %d out of range", bucket);
  if (variant >= holo_variant_count(precision)) return fail(HOLO_ERR_INVALID, "variant out of range");
  std::lock_guard<std::mutex> lk(h->mu);
  h->variant_table[precision][bucket] = variant < 0 ? -1 : variant;
  return HOLO_OK;
}

int holo_get_variant(holo_handle h, int precision, int bucket, int *variant) {
  if (!h || !variant) return fail(HOLO_ERR_INVALID, "null argument");
  if (precision != HOLO_FP64 && precision != HOLO_SPLIT32)
    return fail(HOLO_ERR_INVALID, "unknown precision %d", precision);
  if (bucket < 0 || bucket >= 8) return fail(HOLO_ERR_INVALID, "bucket %d out of range", bucket);
  *variant = h->variant_table[precision][bucket];
  return HOLO_OK;
}

int holo_autotune(holo_handle h, int precision, size_t N, size_t M, int repeats,
                  holo_stream_t stream, int *best_variant, double *best_pairs_per_s) {
  if (!h) return fail(HOLO_ERR_INVALID, "null handle");
  if (N == 0 || M == 0) return fail(HOLO_ERR_INVALID, "autotune needs N, M > 0");
  const int nv = holo_variant_count(precision);
  if (nv < 0) return nv;
  HOLO_TRY(check_sizes(N, M));
  if (repeats < 1) repeats = 1;
  std::lock_guard<std::mutex> lk(h->mu);
  DeviceGuard g(h->device);
  cudaStream_t s = (cudaStream_t)stream;
  // synthetic problem: two parallel square lattices 0.35 m apart (10 um / 7.56 um pitch)
  std::vector<double> u(3 * N), v(3 * M), amp(N), ph(N);
  const int nu = (int)ceil(sqrt((double)N)), nvv = (int)ceil(sqrt((double)M));
  for (size_t i = 0; i < N; ++i) {
    u[3 * i] = ((double)(i % nu) - nu / 2.0) * 10e-6;
    u[3 * i + 1] = ((double)(i / nu) - nu / 2.0) * 10e-6;
    u[3 * i + 2] = 0.35;
    amp[i] = 0.5 + 0.5 * sin(0.37 * i);
    ph[i] = fmod(1.7 * i, 6.283185307179586);
  }
  for (size_t i = 0; i < M; ++i) {
    v[3 * i] = ((double)(i % nvv) - nvv / 2.0) * 7.56e-6;
    v[3 * i + 1] = ((double)(i / nvv) - nvv / 2.0) * 7.56e-6;
    v[3 * i + 2] = 0.0;
  }
  Staged st(h, s);
  const double *du, *dv, *da, *dp;
  double *dy;
  HOLO_TRY(st.up(u.data(), 3 * N, &du));
  HOLO_TRY(st.up(v.data(), 3 * M, &dv));
  HOLO_TRY(st.up(amp.data(), N, &da));
  HOLO_TRY(st.up(ph.data(), N, &dp));
  HOLO_TRY(st.out(2 * M, &dy));
  cudaEvent_t e0, e1;
  HOLO_CUDA(cudaEventCreate(&e0));
  HOLO_CUDA(cudaEventCreate(&e1));
  double best = -1.0;
  int best_v = -1;
  for (int var = 0; var < nv; ++var) {
    holo_plan_s *p = nullptr;
    if (plan_create_impl(h, du, N, dv, M, precision, var, s, &p) != HOLO_OK) continue;
    int rc = plan_execute_impl(p, HOLO_BACKWARDS, 632.8e-9, da, dp, (double2 *)dy, 0, s);  // warm-up
    float ms_total = 0.f;
    for (int r = 0; r < repeats && rc == HOLO_OK; ++r) {
      cudaEventRecord(e0, s);
      rc = plan_execute_impl(p, HOLO_BACKWARDS, 632.8e-9, da, dp, (double2 *)dy, 0, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms_total += ms;
    }
    plan_release(p, s);
    if (rc != HOLO_OK) continue;
    const double rate = (double)N * (double)M * repeats / (ms_total * 1e-3);
    if (rate > best) {
      best = rate;
      best_v = var;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  HOLO_TRY(read_device_error(h, s));
  if (best_v < 0) return fail(HOLO_ERR_CUDA, "no variant ran");
  h->variant_table[precision][size_bucket(N, M)] = best_v;
  if (best_variant) *best_variant = best_v;
  if (best_pairs_per_s) *best_pairs_per_s = best;
  return HOLO_OK;
}

}  // extern "C"

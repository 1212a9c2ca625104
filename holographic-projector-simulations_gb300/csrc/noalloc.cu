// noalloc.cu -- holo_transform_noalloc: the split-precision transform for
// callers that cannot allocate GPU memory.
//
// Who needs it: code that runs where a cudaMalloc (or a memory-pool call)
// is not allowed or not safe -- a host application that hands the library a
// fixed memory budget and owns every byte on the device, a plugin loaded into
// a process whose allocator must not be bypassed, a real-time loop that must
// not hit the implicit device synchronisation of cudaMalloc/cudaFree, or a
// context that must not grow its footprint after start-up.  Such a caller
// passes its own device buffers for the inputs and the output; every other
// byte this transform needs (tile-ordered positions, gathered amplitudes,
// tile boxes, sort scratch, cross-CTA partial sums, the error word) comes from
// one fixed array below, reserved when the library's device code is loaded
// on a GPU and held until the process exits.
//
// Limits and rules:
//   - the array is kNoAllocBytes (64 MiB); a call whose problem does not fit
//     is rejected with HOLO_ERR_INVALID and a message giving the bytes needed;
//   - all calls on a device share the array and each call overwrites it: two
//     calls that overlap on the GPU would race.  Calls in this process are
//     serialised by a lock and each call returns only after its work on
//     `stream` has finished -- on failure too, once anything was queued;
//   - input and output pointers must be memory of `device` (or managed
//     memory): the path enables no peer access;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and keeps it for the life of the
//     process; a cudaDeviceReset may move the array, after which this path must not be
//     used again in the process;
//   - a call waits for its stream partway (the tile statistics are read back), so a
//     stream being captured into a graph is refused with HOLO_ERR_INVALID.
//   - no cudaMalloc, cudaFree, memory-pool or allocating library routine is
//     called on this path.
#include <math.h>

#include <algorithm>
#include <mutex>

#include "internal.cuh"

namespace holo {
namespace {

constexpr size_t kNoAllocBytes = (size_t)64 << 20;
constexpr int kMaxDevices = 64;

// The scratch of every holo_transform_noalloc call on this device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[kMaxDevices] = {};

int noalloc_preload();

// Device address of the array on `device` (looked up once per device, which also
// loads every kernel of the path).
int noalloc_scratch(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return fail(HOLO_ERR_INVALID, "device %d out of range", device);
  if (!g_noalloc_addr[device]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)", __FILE__, __LINE__);
    HOLO_TRY(noalloc_preload());
    g_noalloc_addr[device] = ptr;
  }
  *out = static_cast<unsigned char *>(g_noalloc_addr[device]);
  return HOLO_OK;
}

// Reduce the tile boxes of both point sets to 20 numbers, 10 per set: box
// lo/hi, largest tile half-diagonal, largest half-extent along each axis.
__global__ void __launch_bounds__(256) k_tile_stats(const double *__restrict__ ts, int ns,
                                                    const double *__restrict__ tt, int nt,
                                                    double *__restrict__ out) {
  __shared__ double red[256];
  const double *tiles[2] = {ts, tt};
  const int counts[2] = {ns, nt};
  for (int set = 0; set < 2; ++set) {
    for (int q = 0; q < 10; ++q) {  // 3 lo (min), 3 hi, half-diagonal, 3 half-extents (max)
      const bool is_min = q < 3;
      double v = is_min ? 1e300 : (q < 6 ? -1e300 : 0.0);
      for (int i = threadIdx.x; i < counts[set]; i += blockDim.x) {
        const double *c = tiles[set] + 6 * (size_t)i;
        if (q < 3) v = fmin(v, c[q] - c[3 + q]);
        else if (q < 6) v = fmax(v, c[q - 3] + c[q]);
        else if (q == 6) v = fmax(v, sqrt(c[3] * c[3] + c[4] * c[4] + c[5] * c[5]));
        else v = fmax(v, c[q - 4]);
      }
      red[threadIdx.x] = v;
      __syncthreads();
      for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
          red[threadIdx.x] = is_min ? fmin(red[threadIdx.x], red[threadIdx.x + w])
                                    : fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
      }
      if (threadIdx.x == 0) out[10 * set + q] = red[0];
      __syncthreads();
    }
  }
}

// Every kernel this path can launch, loaded now: CUDA maps a kernel's code into
// device memory on its first use, which a later call must not do.
int noalloc_preload() {
  HOLO_TRY(tiler_preload_hilbert());
  HOLO_TRY(epilogue_preload());
  cudaFuncAttributes a;
  HOLO_CUDA(cudaFuncGetAttributes(&a, k_tile_stats));
  for (const size_t m : {(size_t)1, (size_t)1 << 20})  // both preference lists
    for (const int v : split_preferences(1, m)) {
      int occ = 0;
      HOLO_TRY(split_occupancy(v, false, &occ));  // sets the kernel up (and loads it)
    }
  return HOLO_OK;
}


size_t align256(size_t x) { return (x + 255) / 256 * 256; }

struct Carve {
  unsigned char *base;
  size_t off = 0;
  template <typename T>
  T *take(size_t count) {
    T *p = reinterpret_cast<T *>(base + off);
    off = align256(off + count * sizeof(T));
    return p;
  }
};

// The error model of the allocating planner, from the 20 tile statistics.
void model_from_stats(const double *st, double *base, double *curv, double *lin,
                      double *gemm) {
  TileStats t;
  for (int d = 0; d < 3; ++d) {
    t.lo_s[d] = st[d];
    t.hi_s[d] = st[3 + d];
    t.hd_s[d] = st[7 + d];
    t.lo_t[d] = st[10 + d];
    t.hi_t[d] = st[13 + d];
    t.hd_t[d] = st[17 + d];
  }
  t.h_s = st[6];
  t.h_t = st[16];
  split_error_model(t, base, curv, lin, gemm);
}

// Memory the kernels on `device` may read and write: device memory of that GPU
// (memory of another GPU would need peer access, which this path never enables)
// or managed memory.
bool is_device_pointer(const void *p, int device) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == device;
}

// Once work is queued on the stream, every return -- the failure paths included
// -- waits for it: the scratch array is shared, and the next call (let in by the
// lock as soon as this one returns) overwrites it.
struct DrainOnReturn {
  cudaStream_t s;
  bool armed = false;
  ~DrainOnReturn() {
    if (armed) cudaStreamSynchronize(s);  // its status: already reported by the failing call
  }
};

int transform_noalloc(int device, int sign, double lambda, const double *amp,
                      const double *phase, const double *u, size_t N, const double *v,
                      size_t M, double *y, cudaStream_t s) {
  // the call reads the tile statistics back and waits for its stream partway, which a
  // stream being captured into a graph does not allow: refuse before queuing anything
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  HOLO_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(HOLO_ERR_INVALID,
                "holo_transform_noalloc waits for its stream partway and cannot be captured "
                "into a graph");
  if (sign != 1 && sign != -1) return fail(HOLO_ERR_INVALID, "sign must be +1 or -1 (got %d)", sign);
  if (!(lambda > 0.0) || !isfinite(lambda)) return fail(HOLO_ERR_INVALID, "lambda must be finite and > 0");
  if ((N && (!amp || !phase || !u)) || (M && (!v || !y)))
    return fail(HOLO_ERR_INVALID, "null input or output array");
  for (const void *p : {(const void *)amp, (const void *)phase, (const void *)u, (const void *)v,
                        (const void *)y})
    if (p && !is_device_pointer(p, device))
      return fail(HOLO_ERR_INVALID,
                  "holo_transform_noalloc takes device pointers of device %d (or managed "
                  "memory) only",
                  device);
  const size_t lim = (size_t)kSortBlock * 4096;
  if (N > lim || M > lim) return fail(HOLO_ERR_INVALID, "point count above the supported %zu", lim);
  if (M == 0) return HOLO_OK;

  unsigned char *base = nullptr;
  HOLO_TRY(noalloc_scratch(device, &base));
  DrainOnReturn drain{s};  // armed at the first work queued on `s`
  if (N == 0) {
    drain.armed = true;
    HOLO_CUDA(cudaMemsetAsync(y, 0, M * sizeof(double2), s));
    HOLO_CUDA(cudaStreamSynchronize(s));
    return HOLO_OK;
  }

  // ---- carve the array ----
  const int n_pad = (int)((N + 3071) / 3072) * 3072;  // a multiple of every source tile
  Carve cv{base};
  int *err = cv.take<int>(16);
  double *stats = cv.take<double>(20);
  double *pos_s = cv.take<double>(3 * (size_t)n_pad);
  int32_t *order_s = cv.take<int32_t>(N);
  double *pos_t = cv.take<double>(3 * M);
  int32_t *order_t = cv.take<int32_t>(M);
  double *tiles_s = cv.take<double>(6 * (N / 256 + 1));
  double *tiles_t = cv.take<double>(6 * (M / 256 + 1));
  double2 *ap = cv.take<double2>(n_pad);
  float *geo_s = cv.take<float>(6 * (size_t)n_pad);
  float *geo_t = cv.take<float>(6 * M);
  const size_t shared_off = cv.off;  // sort scratch first, partial sums later
  const size_t nmax = std::max(N, M);
  const size_t hist_n = sort_hist_entries((int)nmax);
  TileScratch ts{};  // the Hilbert tiling: the cheaper sort, and its smaller scratch
  ts.bbox = cv.take<double>(6);
  ts.bbox_scratch = cv.take<double>(6 * 1024);
  ts.keys = cv.take<uint16_t>(nmax);
  ts.hist = cv.take<uint32_t>(hist_n);
  ts.scan = cv.take<uint32_t>(hist_n + 4096 + 16);
  const size_t sort_end = cv.off;
  const size_t partial_min = align256(M * sizeof(double2));  // one split: written to y directly
  const size_t need = std::max(sort_end, shared_off);
  if (need > kNoAllocBytes || shared_off + partial_min > kNoAllocBytes)
    return fail(HOLO_ERR_INVALID,
                "problem needs %zu bytes of the %zu-byte no-alloc scratch (N=%zu, M=%zu)",
                std::max(need, shared_off + partial_min), kNoAllocBytes, N, M);

  drain.armed = true;
  HOLO_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));  // the error word starts at zero
  // ---- tile order of both point sets ----
  HOLO_TRY(tile_order(u, (int)N, order_s, ts, s, kTileHilbert));
  HOLO_TRY(launch_gather_pos(u, order_s, (int)N, n_pad, pos_s, s));
  HOLO_TRY(tile_order(v, (int)M, order_t, ts, s, kTileHilbert));
  HOLO_TRY(launch_gather_pos(v, order_t, (int)M, (int)M, pos_t, s));

  // ---- kernel: the planner's preference list, first whose error bound holds ----
  const std::vector<int> cands = split_preferences(N, M);
  const double budget = kSplitBoundMetres;
  int variant = cands[0];
  int shape_tt = -1, shape_cs = -1;
  double mb[4] = {0.0, 0.0, 0.0, 0.0};
  for (size_t i = 0; i < cands.size(); ++i) {
    const Variant C = split_variant(cands[i]);
    if (C.tt() != shape_tt || C.cs != shape_cs) {
      const int ns = (int)((N + C.cs - 1) / C.cs), nt = (int)((M + C.tt() - 1) / C.tt());
      HOLO_TRY(launch_tile_bbox(pos_s, (int)N, C.cs, tiles_s, s));
      HOLO_TRY(launch_tile_bbox(pos_t, (int)M, C.tt(), tiles_t, s));
      k_tile_stats<<<1, 256, 0, s>>>(tiles_s, ns, tiles_t, nt, stats);
      HOLO_CUDA(cudaGetLastError());
      double st[20];
      HOLO_CUDA(cudaMemcpyAsync(st, stats, sizeof(st), cudaMemcpyDeviceToHost, s));
      HOLO_CUDA(cudaStreamSynchronize(s));
      double base = 0.0, curv = 0.0, lin = 0.0, gemm = 0.0;
      model_from_stats(st, &base, &curv, &lin, &gemm);
      mb[0] = base;
      mb[1] = base + curv;
      mb[2] = mb[1] + lin;
      mb[3] = mb[2] + gemm;
      shape_tt = C.tt();
      shape_cs = C.cs;
    }
    variant = cands[i];
    if (mb[C.model] <= budget) break;
  }
  const Variant V = split_variant(variant);
  // the last bound evaluation left this variant's tile boxes in tiles_s / tiles_t
  HOLO_TRY(launch_rel_hilo(pos_s, (int)N, n_pad, tiles_s, V.cs, geo_s, s));
  HOLO_TRY(launch_rel_hilo(pos_t, (int)M, (int)M, tiles_t, V.tt(), geo_t, s));

  // ---- splits: as many as the occupancy wants and the array holds ----
  int sm = 0, occ = 0;
  HOLO_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device));
  HOLO_TRY(split_occupancy(variant, false, &occ));
  const int G = std::max(1, occ) * sm;
  const int n_stiles = (int)((N + V.cs - 1) / V.cs), n_ttiles = (int)((M + V.tt() - 1) / V.tt());
  const int fit = (int)std::max<size_t>(1, (kNoAllocBytes - shared_off) / (M * sizeof(double2)));
  int splits = 1;
  {
    double best = 1e300;
    for (int S = 1; S <= std::min(n_stiles, fit); ++S) {
      const long long waves = ((long long)n_ttiles * S + G - 1) / G;
      const double cost = waves * (ceil((double)n_stiles / S) + 0.35);
      if (cost < best * 0.999) {
        best = cost;
        splits = S;
      }
    }
  }
  Carve pc{base, shared_off};
  double2 *partial = splits > 1 ? pc.take<double2>((size_t)splits * M) : nullptr;

  // ---- gather, pair kernel, split reduction ----
  float2 *apf = reinterpret_cast<float2 *>(ap);
  HOLO_TRY(launch_gather_apf(amp, phase, order_s, (int)N, n_pad, apf, s));
  SplitProblem P{};
  P.geo_s = geo_s;
  P.apf_s = apf;
  P.geo_t = geo_t;
  P.pos_s = pos_s;
  P.tiles_s = tiles_s;
  P.pos_t = pos_t;
  P.tiles_t = tiles_t;
  P.order_t = order_t;
  P.partial = partial;
  P.y = reinterpret_cast<double2 *>(y);
  P.N = (int)N;
  P.M = (int)M;
  P.n_stiles = n_stiles;
  P.n_ttiles = n_ttiles;
  P.splits = splits;
  P.sign = sign;
  P.sk = sign * ((2.0 * M_PI) / lambda);
  P.sub = 1;
  const int grid = std::max(1, std::min(G, n_ttiles * splits));
  HOLO_TRY(launch_split(P, variant, grid, false, false, err, s));
  if (splits > 1) HOLO_TRY(launch_reduce(partial, splits, (int)M, order_t, P.y, s));
  int e = 0;
  HOLO_CUDA(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  HOLO_CUDA(cudaStreamSynchronize(s));
  if (e) return fail(HOLO_ERR_TIMEOUT, "a device-side wait ran out of time (code %d)", e);
  return HOLO_OK;
}

}  // namespace
}  // namespace holo

extern "C" int holo_transform_noalloc(int device, int sign, double lambda, const double *amp,
                                      const double *phase, const double *u_xyz, size_t N,
                                      const double *v_xyz, size_t M, double *y_re_im,
                                      holo_stream_t stream) {
  std::lock_guard<std::mutex> lk(holo::g_noalloc_mu);
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    cudaGetLastError();
    return holo::fail(HOLO_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return holo::fail(HOLO_ERR_INVALID, "cannot select device %d", device);
  }
  const int rc = holo::transform_noalloc(device, sign, lambda, amp, phase, u_xyz, N, v_xyz, M,
                                         y_re_im, (cudaStream_t)stream);
  cudaSetDevice(prev);
  return rc;
}

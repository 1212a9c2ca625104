// batch.cu -- many independent problems of uneven size in one persistent launch.
//
// The reference only loops over planes sequentially (cuda/main.cu:125-199),
// one transform_full per plane.  Here every problem is planned once, its
// (target tile, source range) work items go into one device work queue sorted
// longest-first, and a persistent split-precision kernel drains the queue with
// an atomic counter (no CTA waits on another).  Gathers, the queue reset, the
// persistent kernel and the cross-split reductions are captured once into a
// CUDA graph; holo_batch_execute replays it.
#include <algorithm>
#include <memory>

#include "internal.cuh"

using namespace holo;

namespace {

struct BatchState {
  std::vector<SplitProblem> probs;     // host copies of the descriptors
  std::vector<double2 *> ap;           // per-problem gathered (phase, amp)
  std::vector<const double *> amp, phase;
  SplitProblem *probs_dev = nullptr;
  WorkItem *items_dev = nullptr;
  int *queue = nullptr;
  int *offsets_dev = nullptr;
  int n_items = 0;
  int total_targets = 0;
  int variant = 0;
  int grid = 0;
};

int batch_build(holo_batch_s *b, const holo_problem *pr, int n, int precision, cudaStream_t s) {
  holo_handle h = b->h;
  BatchState st;
  // FP64 batches are captured as a sequence of per-problem launches.
  const bool split = precision == HOLO_SPLIT32;
  st.variant = 9;  // the default variant for target sets of 1024 and more
  const Variant V = split ? split_variant(st.variant) : fp64_variant(0);
  int occ = 1;
  if (split) HOLO_TRY(split_occupancy(st.variant, false, &occ));
  const int G = std::max(1, occ) * h->sm_count;

  long long work = 0;  // tile pairs
  for (int i = 0; i < n; ++i) {
    holo_plan_s *p = nullptr;
    HOLO_TRY(plan_create_impl(h, pr[i].u_xyz, pr[i].N, pr[i].v_xyz, pr[i].M, precision,
                              split ? st.variant : -1, s, &p));
    b->plans.push_back(p);
    work += (long long)p->n_ttiles * p->n_stiles;
    b->total_pairs += (long long)pr[i].N * (long long)pr[i].M;
  }
  if (!split) return HOLO_OK;

  // split every problem's source range so that items are ~1/8 of a CTA's share
  const double target_item = std::max(1.0, (double)work / ((double)G * 8.0));
  std::vector<WorkItem> items;
  std::vector<int> offsets(n + 1, 0);
  st.probs.resize(n);
  for (int i = 0; i < n; ++i) {
    holo_plan_s *p = b->plans[i];
    int splits = (int)std::min<double>(p->n_stiles, std::max(1.0, ceil(p->n_stiles / target_item)));
    splits = std::max(1, std::min(splits, (int)std::max<size_t>(1, ((size_t)1 << 28) / std::max(p->M, 1))));
    p->splits = splits;
    SplitProblem &P = st.probs[i];
    P = SplitProblem{};
    P.pos_s = p->pos_s;
    P.geo_s = p->geo_s;
    P.geo_t = p->geo_t;
    P.tiles_s = p->tiles_s;
    P.pos_t = p->pos_t;
    P.tiles_t = p->tiles_t;
    P.order_t = p->order_t;
    P.y = (double2 *)pr[i].y_re_im;
    P.N = p->N;
    P.M = p->M;
    P.n_stiles = p->n_stiles;
    P.n_ttiles = p->n_ttiles;
    P.splits = splits;
    P.sign = pr[i].sign;
    P.sk = pr[i].sign * ((2.0 * M_PI) / pr[i].lambda);
    P.sub = 1;
    double2 *ap = (double2 *)pool_alloc(h, (size_t)p->n_pad * sizeof(double2), s);
    if (!ap) return fail(HOLO_ERR_ALLOC, "batch gather buffer");
    b->owned.push_back(ap);
    P.apf_s = reinterpret_cast<float2 *>(ap);
    if (splits > 1) {
      double2 *part = (double2 *)pool_alloc(h, (size_t)splits * p->M * sizeof(double2), s);
      if (!part) return fail(HOLO_ERR_ALLOC, "batch partial buffer");
      b->owned.push_back(part);
      P.partial = part;
    }
    for (int t = 0; t < p->n_ttiles; ++t)
      for (int sp = 0; sp < splits; ++sp) {
        WorkItem w{};
        w.problem = i;
        w.ttile = t;
        w.split = sp;
        w.s_begin = (int)(((long long)p->n_stiles * sp) / splits);
        w.s_end = (int)(((long long)p->n_stiles * (sp + 1)) / splits);
        if (p->N > 0 && w.s_end > w.s_begin) items.push_back(w);
      }
    offsets[i + 1] = offsets[i] + p->M;
  }
  // longest items first: the atomic queue then approximates LPT scheduling
  std::stable_sort(items.begin(), items.end(), [&](const WorkItem &a, const WorkItem &c) {
    const long long ca = (long long)(a.s_end - a.s_begin);
    const long long cc = (long long)(c.s_end - c.s_begin);
    return ca > cc;
  });
  st.n_items = (int)items.size();
  st.total_targets = offsets[n];
  st.grid = std::max(1, std::min(G, st.n_items));
  st.probs_dev = (SplitProblem *)pool_alloc(h, sizeof(SplitProblem) * std::max(n, 1), s);
  st.items_dev = (WorkItem *)pool_alloc(h, sizeof(WorkItem) * std::max<size_t>(items.size(), 1), s);
  st.queue = (int *)pool_alloc(h, sizeof(int), s);
  st.offsets_dev = (int *)pool_alloc(h, sizeof(int) * (n + 1), s);
  if (!st.probs_dev || !st.items_dev || !st.queue || !st.offsets_dev)
    return fail(HOLO_ERR_ALLOC, "batch descriptors");
  b->owned.push_back(st.probs_dev);
  b->owned.push_back(st.items_dev);
  b->owned.push_back(st.queue);
  b->owned.push_back(st.offsets_dev);
  HOLO_CUDA(cudaMemcpyAsync(st.probs_dev, st.probs.data(), sizeof(SplitProblem) * n,
                            cudaMemcpyHostToDevice, s));
  if (!items.empty())
    HOLO_CUDA(cudaMemcpyAsync(st.items_dev, items.data(), sizeof(WorkItem) * items.size(),
                              cudaMemcpyHostToDevice, s));
  HOLO_CUDA(cudaMemcpyAsync(st.offsets_dev, offsets.data(), sizeof(int) * (n + 1),
                            cudaMemcpyHostToDevice, s));
  HOLO_CUDA(cudaStreamSynchronize(s));  // host vectors above are about to go away

  // ---- capture the graph ----
  cudaStream_t cap;
  HOLO_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  int rc = HOLO_OK;
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaStreamDestroy(cap);
    return cuda_fail(e, "cudaStreamBeginCapture", __FILE__, __LINE__);
  }
  for (int i = 0; i < n && rc == HOLO_OK; ++i)
    rc = launch_gather_apf(pr[i].amp, pr[i].phase, b->plans[i]->order_s, b->plans[i]->N,
                          b->plans[i]->n_pad, const_cast<float2 *>(st.probs[i].apf_s), cap);
  if (rc == HOLO_OK && cudaMemsetAsync(st.queue, 0, sizeof(int), cap) != cudaSuccess)
    rc = fail(HOLO_ERR_CUDA, "queue reset during capture");
  if (rc == HOLO_OK && st.n_items > 0)
    rc = launch_split_batched(st.probs_dev, st.items_dev, st.n_items, st.queue, st.variant,
                              st.grid, h->dev_err, cap);
  if (rc == HOLO_OK)
    rc = launch_reduce_batched(st.probs_dev, st.offsets_dev, n, st.total_targets, cap);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(cap, &graph);
  cudaStreamDestroy(cap);
  if (rc != HOLO_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  b->graph = graph;
  HOLO_CUDA(cudaGraphInstantiate(&b->exec, graph, 0));
  (void)V;
  return HOLO_OK;
}

void batch_release(holo_batch_s *b, cudaStream_t s) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (holo_plan_s *p : b->plans) plan_release(p, s);
  for (void *q : b->owned) pool_free(q, s);
  delete b;
}

}  // namespace

extern "C" {

int holo_batch_create(holo_handle h, const holo_problem *problems, int n_problems,
                      int precision, holo_stream_t stream, holo_batch *out) {
  if (!h || !out || (n_problems > 0 && !problems) || n_problems < 0)
    return fail(HOLO_ERR_INVALID, "bad batch arguments");
  if (precision != HOLO_SPLIT32 && precision != HOLO_FP64)
    return fail(HOLO_ERR_INVALID, "unknown precision %d", precision);
  *out = nullptr;
  for (int i = 0; i < n_problems; ++i) {
    const holo_problem &q = problems[i];
    if ((q.N && (!q.amp || !q.phase || !q.u_xyz)) || (q.M && (!q.v_xyz || !q.y_re_im)))
      return fail(HOLO_ERR_INVALID, "problem %d: null array", i);
    if (q.sign != 1 && q.sign != -1) return fail(HOLO_ERR_INVALID, "problem %d: bad sign", i);
    if (!(q.lambda > 0.0) || !isfinite(q.lambda)) return fail(HOLO_ERR_INVALID, "problem %d: bad lambda", i);
    for (const void *ptr : {(const void *)q.amp, (const void *)q.phase, (const void *)q.u_xyz,
                            (const void *)q.v_xyz, (const void *)q.y_re_im}) {
      if (!ptr) continue;
      cudaPointerAttributes a;
      if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess ||
          (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)) {
        cudaGetLastError();
        return fail(HOLO_ERR_INVALID, "problem %d: batched problems need device pointers", i);
      }
    }
  }
  std::lock_guard<std::mutex> lk(h->mu);
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  cudaStream_t s = (cudaStream_t)stream;
  holo_batch_s *b = new holo_batch_s();
  b->h = h;
  int rc = batch_build(b, problems, n_problems, precision, s);
  if (rc == HOLO_OK && precision == HOLO_FP64) {
    // FP64: capture the per-problem launches
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) {
      rc = fail(HOLO_ERR_CUDA, "capture stream");
    } else {
      cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
      for (int i = 0; i < n_problems && rc == HOLO_OK; ++i)
        rc = plan_execute_impl(b->plans[i], problems[i].sign, problems[i].lambda,
                               problems[i].amp, problems[i].phase,
                               (double2 *)problems[i].y_re_im, 0, cap);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(cap, &g);
      cudaStreamDestroy(cap);
      if (rc == HOLO_OK && e != cudaSuccess) rc = cuda_fail(e, "capture", __FILE__, __LINE__);
      if (rc == HOLO_OK) {
        b->graph = g;
        if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess)
          rc = fail(HOLO_ERR_CUDA, "graph instantiate");
      } else if (g) {
        cudaGraphDestroy(g);
      }
    }
  }
  if (rc != HOLO_OK) {
    batch_release(b, s);
    if (prev >= 0) cudaSetDevice(prev);
    return rc;
  }
  if (prev >= 0) cudaSetDevice(prev);
  *out = b;
  return HOLO_OK;
}

int holo_batch_execute(holo_batch b, holo_stream_t stream) {
  if (!b) return fail(HOLO_ERR_INVALID, "null batch");
  std::lock_guard<std::mutex> lk(b->h->mu);
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(b->h->device);
  cudaError_t e = b->exec ? cudaGraphLaunch(b->exec, (cudaStream_t)stream) : cudaSuccess;
  if (prev >= 0) cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch", __FILE__, __LINE__);
  return HOLO_OK;
}

int holo_batch_destroy(holo_batch b) {
  if (!b) return HOLO_OK;
  holo_handle h = b->h;
  std::lock_guard<std::mutex> lk(h->mu);
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  cudaDeviceSynchronize();
  batch_release(b, nullptr);
  if (prev >= 0) cudaSetDevice(prev);
  return HOLO_OK;
}

int holo_batch_pairs(holo_batch b, long long *pairs) {
  if (!b || !pairs) return fail(HOLO_ERR_INVALID, "null argument");
  *pairs = b->total_pairs;
  return HOLO_OK;
}

int holo_transform_batched(holo_handle h, const holo_problem *problems, int n_problems,
                           int precision, holo_stream_t stream) {
  holo_batch b = nullptr;
  HOLO_TRY(holo_batch_create(h, problems, n_problems, precision, stream, &b));
  int rc = holo_batch_execute(b, stream);
  if (rc == HOLO_OK) rc = holo_device_status(h, stream);
  holo_batch_destroy(b);
  return rc;
}

}  // extern "C"

// batch.cu -- many independent problems of uneven size in persistent launches.
//
// The reference only loops over planes sequentially (cuda/main.cu:125-199),
// one transform_full per plane.  Here every problem is planned once (tile
// shape and pair model as for a single transform); problems whose plans chose
// the same kernel variant form a group, whose (target tile, source range) work
// items go into one device work queue sorted longest-first, drained by one
// persistent split-precision kernel with an atomic counter (no CTA waits on
// another).  Gathers, the queue reset, one queue kernel per group and the
// cross-split reductions are captured once into a CUDA graph;
// holo_batch_execute replays it.
#include <algorithm>
#include <memory>

#include "internal.cuh"

using namespace holo;

namespace {

// Problems whose plans chose the same kernel variant share one persistent
// queue kernel; each group has its own work items and queue counter.
struct Group {
  int variant = 0;
  std::vector<WorkItem> items;
  WorkItem *items_dev = nullptr;
  int grid = 0;
};

// The split-precision descriptor of problem i with its source range cut into
// `splits` parts; its work items go to `items`.
int describe_problem(holo_batch_s *b, const holo_problem &q, holo_plan_s *p, int i, int splits,
                     SplitProblem *P, std::vector<WorkItem> *items, cudaStream_t s) {
  holo_handle h = b->h;
  p->splits = splits;
  *P = SplitProblem{};
  P->pos_s = p->pos_s;
  P->geo_s = p->geo_s;
  P->geo_t = p->geo_t;
  P->tiles_s = p->tiles_s;
  P->pos_t = p->pos_t;
  P->tiles_t = p->tiles_t;
  P->order_t = p->order_t;
  P->y = (double2 *)q.y_re_im;
  P->N = p->N;
  P->M = p->M;
  P->n_stiles = p->n_stiles;
  P->n_ttiles = p->n_ttiles;
  P->splits = splits;
  P->sign = q.sign;
  P->sk = q.sign * ((2.0 * M_PI) / q.lambda);
  P->sub = 1;
  float2 *apf = (float2 *)pool_alloc(h, (size_t)p->n_pad * sizeof(float2), s);
  if (!apf) return fail(HOLO_ERR_ALLOC, "batch gather buffer");
  b->owned.push_back(apf);
  P->apf_s = apf;
  if (splits > 1) {
    double2 *part = (double2 *)pool_alloc(h, (size_t)splits * p->M * sizeof(double2), s);
    if (!part) return fail(HOLO_ERR_ALLOC, "batch partial buffer");
    b->owned.push_back(part);
    P->partial = part;
  }
  for (int t = 0; t < p->n_ttiles; ++t)
    for (int sp = 0; sp < splits; ++sp) {
      WorkItem w{};
      w.problem = i;
      w.ttile = t;
      w.split = sp;
      w.s_begin = (int)(((long long)p->n_stiles * sp) / splits);
      w.s_end = (int)(((long long)p->n_stiles * (sp + 1)) / splits);
      if (p->N > 0 && w.s_end > w.s_begin) items->push_back(w);
    }
  return HOLO_OK;
}

int batch_build(holo_batch_s *b, const holo_problem *pr, int n, int precision, cudaStream_t s) {
  holo_handle h = b->h;
  // every problem planned on its own: tile shape and pair model as for a
  // single transform of it (FP64 batches are captured by the caller as a
  // sequence of per-problem launches)
  for (int i = 0; i < n; ++i) {
    holo_plan_s *p = nullptr;
    HOLO_TRY(plan_create_impl(h, pr[i].u_xyz, pr[i].N, pr[i].v_xyz, pr[i].M, precision, -1, s,
                              &p));
    b->plans.push_back(p);
    b->total_pairs += (long long)pr[i].N * (long long)pr[i].M;
  }
  if (precision != HOLO_SPLIT32) return HOLO_OK;

  std::vector<Group> groups;
  std::vector<int> group_of(n);
  for (int i = 0; i < n; ++i) {
    size_t g = 0;
    const int v = b->plans[i]->variant;
    while (g < groups.size() && groups[g].variant != v) ++g;
    if (g == groups.size()) {
      groups.emplace_back();
      groups.back().variant = v;
    }
    group_of[i] = (int)g;
  }
  std::vector<SplitProblem> probs(n);
  std::vector<int> offsets(n + 1, 0);
  for (int i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + b->plans[i]->M;
  for (size_t g = 0; g < groups.size(); ++g) {
    Group &G = groups[g];
    int occ = 1;
    HOLO_TRY(split_occupancy(G.variant, false, &occ));
    const int slots = std::max(1, occ) * h->sm_count;
    long long work = 0;  // tile pairs of the group
    for (int i = 0; i < n; ++i)
      if (group_of[i] == (int)g) work += (long long)b->plans[i]->n_ttiles * b->plans[i]->n_stiles;
    // split every problem's source range so that items are ~1/8 of a CTA's share
    const double target_item = std::max(1.0, (double)work / ((double)slots * 8.0));
    for (int i = 0; i < n; ++i) {
      if (group_of[i] != (int)g) continue;
      holo_plan_s *p = b->plans[i];
      int splits = (int)std::min<double>(p->n_stiles, std::max(1.0, ceil(p->n_stiles / target_item)));
      splits = std::max(1, std::min(splits, (int)std::max<size_t>(1, ((size_t)1 << 28) / std::max(p->M, 1))));
      HOLO_TRY(describe_problem(b, pr[i], p, i, splits, &probs[i], &G.items, s));
    }
    // longest items first: the atomic queue then approximates LPT scheduling
    std::stable_sort(G.items.begin(), G.items.end(), [](const WorkItem &x, const WorkItem &y) {
      return x.s_end - x.s_begin > y.s_end - y.s_begin;
    });
    G.grid = std::max(1, std::min(slots, (int)G.items.size()));
  }
  const int ng = (int)groups.size();
  SplitProblem *probs_dev = (SplitProblem *)pool_alloc(h, sizeof(SplitProblem) * std::max(n, 1), s);
  int *queues = (int *)pool_alloc(h, sizeof(int) * std::max(ng, 1), s);
  int *offsets_dev = (int *)pool_alloc(h, sizeof(int) * (n + 1), s);
  if (!probs_dev || !queues || !offsets_dev) return fail(HOLO_ERR_ALLOC, "batch descriptors");
  b->owned.push_back(probs_dev);
  b->owned.push_back(queues);
  b->owned.push_back(offsets_dev);
  for (Group &G : groups) {
    G.items_dev = (WorkItem *)pool_alloc(h, sizeof(WorkItem) * std::max<size_t>(G.items.size(), 1), s);
    if (!G.items_dev) return fail(HOLO_ERR_ALLOC, "batch work items");
    b->owned.push_back(G.items_dev);
    if (!G.items.empty())
      HOLO_CUDA(cudaMemcpyAsync(G.items_dev, G.items.data(), sizeof(WorkItem) * G.items.size(),
                                cudaMemcpyHostToDevice, s));
  }
  if (n > 0)
    HOLO_CUDA(cudaMemcpyAsync(probs_dev, probs.data(), sizeof(SplitProblem) * n,
                              cudaMemcpyHostToDevice, s));
  HOLO_CUDA(cudaMemcpyAsync(offsets_dev, offsets.data(), sizeof(int) * (n + 1),
                            cudaMemcpyHostToDevice, s));
  HOLO_CUDA(cudaStreamSynchronize(s));  // host vectors above are about to go away

  // ---- capture the graph: gathers, queue reset, one queue kernel per group, reductions ----
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
                           b->plans[i]->n_pad, const_cast<float2 *>(probs[i].apf_s), cap);
  if (rc == HOLO_OK && ng > 0 && cudaMemsetAsync(queues, 0, sizeof(int) * ng, cap) != cudaSuccess)
    rc = fail(HOLO_ERR_CUDA, "queue reset during capture");
  for (int g = 0; g < ng && rc == HOLO_OK; ++g)
    if (!groups[g].items.empty())
      rc = launch_split_batched(probs_dev, groups[g].items_dev, (int)groups[g].items.size(),
                                queues + g, groups[g].variant, groups[g].grid, h->dev_err, cap);
  if (rc == HOLO_OK) rc = launch_reduce_batched(probs_dev, offsets_dev, n, offsets[n], cap);
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

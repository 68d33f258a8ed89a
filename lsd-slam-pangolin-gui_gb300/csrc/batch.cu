// batch.cu -- batched alignment of many independent frame pairs of mixed size (a11).
//
// A batch owns one arena with 2n frames: frames 0..n-1 are the keyframes (with depth), n..2n-1 the
// frames to track.  The level-0 inputs of all pairs sit back to back per kind, so a batch upload is
// four host->device copies.  lsdg_batch_run is one CUDA graph: image pyramids of all 2n frames,
// depth pyramids + point compaction of the keyframes, then ONE persistent cluster launch that runs
// every pair's full coarse-to-fine LM loop on the device (pairs taken largest first from an atomic
// queue).  The graph is captured after the autotuner has picked the (threads, cluster) shape for
// the batch's size mix, and it is recaptured when the parameters change.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "lsdg_host.h"

using namespace lsdg;

namespace lsdg {
int launch_frame_pyramid(const FrameDev* frames, int n, int levels, long max_pix, int max_h, bool with_grads,
                         cudaStream_t s);
int launch_frame_points(const FrameDev* frames, int n, int levels, int max_h, cudaStream_t s);
}  // namespace lsdg

#define CK(ctx, expr)                                         \
  do {                                                        \
    lsdg_status _s = ctx_cuda((ctx), (expr), #expr);          \
    if (_s != LSDG_OK) return _s;                             \
  } while (0)

struct lsdg_batch {
  int n = 0;
  bool sim3 = false;  // Sim3 constraint tracking: both keyframes of a pair carry depth
  int pose_len = 12;  // doubles per pose: 12 (SE3) or 13 (Sim3: R, t, s)
  FrameSet fs;
  PairDev* d_pairs = nullptr;
  int* d_order = nullptr;
  double* d_init = nullptr;
  double* d_out = nullptr;
  lsdg_track_stats* d_stats = nullptr;
  int* d_work = nullptr;
  double* h_out = nullptr;
  lsdg_track_stats* h_stats = nullptr;
  int* h_counts = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_epoch = -1;
  int launches_per_run = 0;
  TuneChoice tc;
  std::string key;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // run start, build done, track done
  bool ran = false;
};

static void batch_free(lsdg_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  frameset_free(b->fs);
  if (b->d_pairs) cudaFree(b->d_pairs);
  if (b->d_order) cudaFree(b->d_order);
  if (b->d_init) cudaFree(b->d_init);
  if (b->d_out) cudaFree(b->d_out);
  if (b->d_stats) cudaFree(b->d_stats);
  if (b->d_work) cudaFree(b->d_work);
  if (b->h_out) cudaFreeHost(b->h_out);
  if (b->h_stats) cudaFreeHost(b->h_stats);
  if (b->h_counts) cudaFreeHost(b->h_counts);
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  delete b;
}

static lsdg_status batch_track_args(lsdg_ctx* ctx, lsdg_batch* b, TrackArgs* a) {
  *a = make_track_args(ctx->params);
  a->pairs = b->d_pairs;
  a->order = b->d_order;
  a->n_pairs = b->n;
  a->work_counter = b->d_work;
  a->init = b->d_init;
  a->init_is_ref_to_frame = 0;
  a->out_pose = b->d_out;
  a->out_stats = b->d_stats;
  a->out_sums = nullptr;
  return LSDG_OK;
}

static lsdg_status enqueue_build(lsdg_ctx* ctx, lsdg_batch* b, int* launches) {
  // band pass over all 2n frames (also the depth pyramids of the second keyframes in Sim3 mode);
  // reference points only for the first n
  const int L = ctx->params.levels;
  int k = launch_frame_pyramid(b->fs.d_frames, 2 * b->n, L, b->fs.max_pix, b->fs.max_h, false, ctx->stream);
  k += launch_frame_points(b->fs.d_frames, b->n, L, b->fs.max_h, ctx->stream);
  CK(ctx, cudaGetLastError());
  *launches = k;
  return LSDG_OK;
}

static lsdg_status batch_create(lsdg_ctx* ctx, int n, const int* widths, const int* heights, const lsdg_intrinsics* intr,
                                bool sim3, lsdg_batch** out) {
  if (!ctx || !widths || !heights || !intr || !out || n <= 0) return ctx_fail(ctx, LSDG_INVALID_ARG, "bad batch arguments");
  *out = nullptr;
  CK(ctx, cudaSetDevice(ctx->device));
  lsdg_batch* b = new (std::nothrow) lsdg_batch();
  if (!b) return LSDG_OUT_OF_MEMORY;
  b->n = n;
  b->sim3 = sim3;
  b->pose_len = sim3 ? 13 : 12;
  std::vector<int> w(2 * n), h(2 * n);
  std::vector<lsdg_intrinsics> k(2 * n);
  bool* dep = new bool[2 * n];
  for (int i = 0; i < n; ++i) {
    w[i] = w[n + i] = widths[i];
    h[i] = h[n + i] = heights[i];
    k[i] = k[n + i] = intr[i];
    dep[i] = true;
    dep[n + i] = sim3;
  }
  // the tracker samples intensity planes only: no gradient pyramid for batch frames
  lsdg_status st = frameset_alloc(ctx, b->fs, 2 * n, w.data(), h.data(), k.data(), dep, ctx->params.levels, false);
  delete[] dep;
  if (st != LSDG_OK) {
    batch_free(b);
    return st;
  }
  std::vector<PairDev> pairs(n);
  for (int i = 0; i < n; ++i) pairs[i] = PairDev{b->fs.d_frames + i, b->fs.d_frames + n + i};
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return (long)widths[a] * heights[a] > (long)widths[c] * heights[c]; });
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&b->d_pairs, sizeof(PairDev) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_order, sizeof(int) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_init, sizeof(double) * b->pose_len * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_out, sizeof(double) * b->pose_len * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_stats, sizeof(lsdg_track_stats) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_work, sizeof(int) * 4);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_out, sizeof(double) * b->pose_len * n);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_stats, sizeof(lsdg_track_stats) * n);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_counts, sizeof(int) * kMaxLevels * n);
  for (auto& ev : b->ev)
    if (e == cudaSuccess) e = cudaEventCreate(&ev);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_pairs, pairs.data(), sizeof(PairDev) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    st = ctx_cuda(ctx, e, "batch allocation");
    batch_free(b);
    return st;
  }
  // autotuner key: the multiset of sizes
  std::vector<std::pair<int, int>> sz(n);
  for (int i = 0; i < n; ++i) sz[i] = {widths[i], heights[i]};
  std::sort(sz.begin(), sz.end());
  std::string key = sim3 ? "batch-sim3:" : "batch:";
  for (int i = 0; i < n;) {
    int j = i;
    while (j < n && sz[j] == sz[i]) ++j;
    key += std::to_string(j - i) + "x" + std::to_string(sz[i].first) + "x" + std::to_string(sz[i].second) + ";";
    i = j;
  }
  b->key = key;
  *out = b;
  return LSDG_OK;
}

extern "C" {

lsdg_status lsdg_batch_create(lsdg_ctx* ctx, int n, const int* widths, const int* heights, const lsdg_intrinsics* intr,
                              lsdg_batch** out) {
  return batch_create(ctx, n, widths, heights, intr, false, out);
}

lsdg_status lsdg_batch_create_sim3(lsdg_ctx* ctx, int n, const int* widths, const int* heights,
                                   const lsdg_intrinsics* intr, lsdg_batch** out) {
  return batch_create(ctx, n, widths, heights, intr, true, out);
}

lsdg_status lsdg_batch_destroy(lsdg_ctx* ctx, lsdg_batch* b) {
  if (!ctx || !b) return LSDG_INVALID_ARG;
  cudaStreamSynchronize(ctx->stream);
  batch_free(b);
  return LSDG_OK;
}

lsdg_status lsdg_batch_load(lsdg_ctx* ctx, lsdg_batch* b, const float* ref_images, const float* ref_idepth,
                            const float* ref_var, const float* new_images, const double* init) {
  if (!ctx || !b || !ref_images || !ref_idepth || !ref_var || !new_images || !init)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (b->sim3) return ctx_fail(ctx, LSDG_INVALID_ARG, "Sim3 batch: use lsdg_batch_load_sim3");
  const size_t half = b->fs.pix_depth * 4;  // the keyframes come first, all with depth
  char* base = (char*)b->fs.arena;
  CK(ctx, cudaMemcpyAsync(b->fs.plane0, ref_images, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync((char*)b->fs.plane0 + half, new_images, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(base + b->fs.off_id0, ref_idepth, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(base + b->fs.off_var0, ref_var, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(b->d_init, init, sizeof(double) * 12 * b->n, cudaMemcpyHostToDevice, ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_batch_load_sim3(lsdg_ctx* ctx, lsdg_batch* b, const float* ref_images, const float* ref_idepth,
                                 const float* ref_var, const float* new_images, const float* new_idepth,
                                 const float* new_var, const double* init) {
  if (!ctx || !b || !ref_images || !ref_idepth || !ref_var || !new_images || !new_idepth || !new_var || !init)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!b->sim3) return ctx_fail(ctx, LSDG_INVALID_ARG, "not a Sim3 batch (lsdg_batch_create_sim3)");
  for (int i = 0; i < b->n; ++i)
    if (!(init[13 * i + 12] > 0)) return ctx_fail(ctx, LSDG_INVALID_ARG, "pair %d: Sim3 scale must be > 0", i);
  const size_t half = b->fs.pix_depth / 2 * 4;  // both halves carry depth: the keyframes i, then j
  char* base = (char*)b->fs.arena;
  CK(ctx, cudaMemcpyAsync(b->fs.plane0, ref_images, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync((char*)b->fs.plane0 + half, new_images, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(base + b->fs.off_id0, ref_idepth, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(base + b->fs.off_id0 + half, new_idepth, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(base + b->fs.off_var0, ref_var, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(base + b->fs.off_var0 + half, new_var, half, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(b->d_init, init, sizeof(double) * 13 * b->n, cudaMemcpyHostToDevice, ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_batch_run(lsdg_ctx* ctx, lsdg_batch* b) {
  if (!ctx || !b) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!b->exec || b->graph_epoch != ctx->params_epoch) {
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    // eager build so that the autotuner times the tracker on this batch's real points
    int k = 0;
    lsdg_status st = enqueue_build(ctx, b, &k);
    if (st != LSDG_OK) return st;
    ctx->launches += k;
    TrackArgs a;
    batch_track_args(ctx, b, &a);
    st = autotune(ctx, b->key, a, &b->tc, b->sim3);
    if (st != LSDG_OK) return st;
    // capture: events, build, tracker
    CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int nl = 0;
    // external records become event-record nodes of the graph (timed on every replay)
    cudaEventRecordWithFlags(b->ev[0], ctx->stream, cudaEventRecordExternal);
    st = enqueue_build(ctx, b, &nl);
    cudaEventRecordWithFlags(b->ev[1], ctx->stream, cudaEventRecordExternal);
    int64_t before = ctx->launches;
    if (st == LSDG_OK) st = run_tracker(ctx, a, b->tc, b->sim3);
    nl += (int)(ctx->launches - before);
    ctx->launches = before;
    cudaEventRecordWithFlags(b->ev[2], ctx->stream, cudaEventRecordExternal);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (st != LSDG_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    CK(ctx, e);
    e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    CK(ctx, e);
    b->launches_per_run = nl;
    b->graph_epoch = ctx->params_epoch;
  }
  CK(ctx, cudaGraphLaunch(b->exec, ctx->stream));
  ctx->launches += b->launches_per_run;
  b->ran = true;
  return LSDG_OK;
}

lsdg_status lsdg_batch_read(lsdg_ctx* ctx, lsdg_batch* b, double* out, lsdg_track_stats* stats) {
  if (!ctx || !b) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  CK(ctx, cudaMemcpyAsync(b->h_out, b->d_out, sizeof(double) * b->pose_len * b->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(b->h_stats, b->d_stats, sizeof(lsdg_track_stats) * b->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (out) std::memcpy(out, b->h_out, sizeof(double) * b->pose_len * b->n);
  if (stats) std::memcpy(stats, b->h_stats, sizeof(lsdg_track_stats) * b->n);
  return LSDG_OK;
}

lsdg_status lsdg_batch_track_sim3(lsdg_ctx* ctx, lsdg_batch* b, const float* ref_images, const float* ref_idepth,
                                  const float* ref_var, const float* new_images, const float* new_idepth,
                                  const float* new_var, const double* init, double* out, lsdg_track_stats* stats) {
  lsdg_status st = lsdg_batch_load_sim3(ctx, b, ref_images, ref_idepth, ref_var, new_images, new_idepth, new_var, init);
  if (st != LSDG_OK) return st;
  st = lsdg_batch_run(ctx, b);
  if (st != LSDG_OK) return st;
  return lsdg_batch_read(ctx, b, out, stats);
}

lsdg_status lsdg_batch_track_se3(lsdg_ctx* ctx, lsdg_batch* b, const float* ref_images, const float* ref_idepth,
                                 const float* ref_var, const float* new_images, const double* init, double* out,
                                 lsdg_track_stats* stats) {
  lsdg_status st = lsdg_batch_load(ctx, b, ref_images, ref_idepth, ref_var, new_images, init);
  if (st != LSDG_OK) return st;
  st = lsdg_batch_run(ctx, b);
  if (st != LSDG_OK) return st;
  return lsdg_batch_read(ctx, b, out, stats);
}

// Device time of the last run's two phases (pyramids + points, tracker), from the events the
// graph records on the context stream.  Synchronises.
lsdg_status lsdg_batch_timing(lsdg_ctx* ctx, lsdg_batch* b, float* build_ms, float* track_ms) {
  if (!ctx || !b || !b->ran) return ctx_fail(ctx, LSDG_INVALID_ARG, "no run to time");
  CK(ctx, cudaEventSynchronize(b->ev[2]));
  float a = 0, c = 0;
  CK(ctx, cudaEventElapsedTime(&a, b->ev[0], b->ev[1]));
  CK(ctx, cudaEventElapsedTime(&c, b->ev[1], b->ev[2]));
  if (build_ms) *build_ms = a;
  if (track_ms) *track_ms = c;
  return LSDG_OK;
}

lsdg_status lsdg_batch_work(lsdg_ctx* ctx, lsdg_batch* b, int64_t* passes, double* pass_bytes, double* unique_bytes) {
  if (!ctx || !b || !b->ran) return ctx_fail(ctx, LSDG_INVALID_ARG, "no run to account");
  const int L = ctx->params.levels;
  for (int i = 0; i < b->n; ++i)
    CK(ctx, cudaMemcpyAsync(b->h_counts + kMaxLevels * i, b->fs.h_frames[i].pcount, sizeof(int) * kMaxLevels,
                            cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(b->h_stats, b->d_stats, sizeof(lsdg_track_stats) * b->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  int64_t np = 0;
  double pb = 0, ub = 0;
  for (int i = 0; i < b->n; ++i) {
    for (int l = 0; l < L; ++l) {
      const double pts = b->h_counts[kMaxLevels * i + l];
      const double pix = (double)(b->fs.w[i] >> l) * (b->fs.h[i] >> l);
      const int ps = b->h_stats[i].passes[l];
      np += ps;
      // per pass: each point's float4 + its frozen variance (psig; the first pass reads pvar and
      // writes psig instead), the frame level's intensity plane, the sums.  Sim3 adds the point's
      // depth variance (psigd) and the other keyframe's inverse depth and variance planes.
      const double per_pt = b->sim3 ? 24.0 : 20.0, per_px = b->sim3 ? 12.0 : 4.0;
      const double sums = b->sim3 ? 36 * 4.0 : 28 * 4.0;
      pb += ps * (pts * per_pt + pix * per_px + sums);
      if (ps > 0) ub += pts * per_pt + pix * per_px;
    }
  }
  if (passes) *passes = np;
  if (pass_bytes) *pass_bytes = pb;
  if (unique_bytes) *unique_bytes = ub;
  return LSDG_OK;
}

// The tile shape the autotuner chose for this batch.
lsdg_status lsdg_batch_shape(lsdg_ctx* ctx, lsdg_batch* b, int* threads, int* minblocks, int* cluster, int* clusters,
                             int* launches_per_run) {
  if (!ctx || !b) return LSDG_INVALID_ARG;
  if (threads) *threads = b->tc.threads;
  if (minblocks) *minblocks = b->tc.minblocks;
  if (cluster) *cluster = b->tc.cluster;
  if (clusters) *clusters = std::min(b->n, b->tc.max_clusters);
  if (launches_per_run) *launches_per_run = b->launches_per_run;
  return LSDG_OK;
}

}  // extern "C"

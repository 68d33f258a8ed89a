// batch.cu -- batched alignment of many independent frame pairs of mixed size (a11).
//
// A batch slot owns one arena with 2n frames: frames 0..n-1 are the keyframes (with depth), n..2n-1
// the frames to track.  The level-0 inputs of all pairs sit back to back per kind, so a batch upload
// is four host->device copies (two byte copies for 8-bit images).  A run is one CUDA graph: one
// launch builds the image pyramids of all 2n frames, the depth pyramids and the compacted points of
// the keyframes (frame.cu), a one-CTA kernel ranks the pairs by their keyframes' points, then the
// persistent cluster tracker runs every pair's full coarse-to-fine LM loop on the device (pairs
// taken largest first from an atomic queue; coarse and fine levels in two launches when the tuner
// splits them).  The graph is captured after the autotuner has picked the launch plan for the
// batch's size mix, and it is recaptured when the parameters change.
//
// Two slots make the pipelined form (lsdg_batch_submit_* / lsdg_batch_collect): step k+1's inputs
// are uploaded into the other slot on a copy stream while step k's graph runs, and each step's
// poses come back on a read-back stream behind its graph (off the graphs' stream), so the
// host<->device copies overlap the tracking.  The synchronous calls (load / run / read / track) use slot 0.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lsdg_host.h"

using namespace lsdg;

namespace lsdg {
int launch_frame_pyramid(const FrameDev* frames, int n, int levels, long max_pix, int max_h, bool with_grads,
                         cudaStream_t s);
int launch_frame_points(const FrameDev* frames, int n, int levels, int max_h, cudaStream_t s);
size_t frame_build_ws_bytes(int n, int levels, int max_h);
int launch_frame_build(const FrameDev* frames, int n, int n_point_frames, int levels, int max_h,
                       unsigned long long* ws, cudaStream_t s, int withhold_frame, const uint8_t* u8,
                       const float* plane0, const int* mode);
}  // namespace lsdg

#define CK(ctx, expr)                                         \
  do {                                                        \
    lsdg_status _s = ctx_cuda((ctx), (expr), #expr);          \
    if (_s != LSDG_OK) return _s;                             \
  } while (0)

namespace {

struct BatchSlot {
  bool ready = false;  // allocated
  FrameSet fs;
  PairDev* d_pairs = nullptr;
  double* d_init = nullptr;
  double* d_out = nullptr;
  lsdg_track_stats* d_stats = nullptr;
  int* d_work = nullptr;
  double* d_mid = nullptr;            // coarse-phase poses of a split run
  int* d_order = nullptr;             // processing order of the pairs (by reference points, set on the device)
  uint8_t* d_u8 = nullptr;            // 8-bit staging of the level-0 images (SE3 batches)
  int* d_mode = nullptr;              // 1: this step's level-0 images are the bytes in d_u8
  int* h_mode = nullptr;              // pinned {0, 1}: the sources of the mode word
  unsigned long long* d_scan = nullptr;  // one-launch build workspace (ticket, error word, band counts)
  unsigned* h_err = nullptr;          // pinned copy of the build's error word
  double* h_out = nullptr;            // pinned staging of the results
  lsdg_track_stats* h_stats = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_epoch = -1;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // run start, build done, track done (timing)
  cudaEvent_t copied = nullptr;       // inputs are in the arena (copy stream)
  cudaEvent_t done = nullptr;         // graph + result read-back finished (read-back stream)
  cudaEvent_t graph_done = nullptr;   // the step's graph finished (context stream)
  bool ran = false;
};

}  // namespace

struct lsdg_batch {
  int n = 0;
  bool sim3 = false;  // Sim3 constraint tracking: both keyframes of a pair carry depth
  int pose_len = 12;  // doubles per pose: 12 (SE3) or 13 (Sim3: R, t, s)
  std::vector<int> w, h;
  std::vector<lsdg_intrinsics> intr;
  BatchSlot slot[2];
  int last = 0;                 // slot of the last run (timing / work)
  int test_withhold = -1;  // lsdg_batch_test_withhold: keyframe whose band 0 publishes no counts
  int* h_counts = nullptr;
  cudaStream_t copy = nullptr;      // upload stream of the pipelined form
  cudaStream_t readback = nullptr;  // result stream of the pipelined form (off the graphs' stream)
  int inflight[2] = {-1, -1};   // slots of the submitted, not yet collected steps (oldest first)
  int n_inflight = 0;
  int next = 0;                 // slot of the next submit
  int launches_per_run = 0;
  int tune_epoch = -1;          // params epoch the shape was tuned for
  TuneChoice tc;
  std::string key;
};

static void slot_free(BatchSlot& s) {
  if (s.exec) cudaGraphExecDestroy(s.exec);
  frameset_free(s.fs);
  if (s.d_pairs) cudaFree(s.d_pairs);
  if (s.d_init) cudaFree(s.d_init);
  if (s.d_out) cudaFree(s.d_out);
  if (s.d_stats) cudaFree(s.d_stats);
  if (s.d_work) cudaFree(s.d_work);
  if (s.d_mid) cudaFree(s.d_mid);
  if (s.d_order) cudaFree(s.d_order);
  if (s.d_u8) cudaFree(s.d_u8);
  if (s.d_mode) cudaFree(s.d_mode);
  if (s.h_mode) cudaFreeHost(s.h_mode);
  if (s.d_scan) cudaFree(s.d_scan);
  if (s.h_err) cudaFreeHost(s.h_err);
  if (s.h_out) cudaFreeHost(s.h_out);
  if (s.h_stats) cudaFreeHost(s.h_stats);
  for (auto& e : s.ev)
    if (e) cudaEventDestroy(e);
  if (s.copied) cudaEventDestroy(s.copied);
  if (s.done) cudaEventDestroy(s.done);
  if (s.graph_done) cudaEventDestroy(s.graph_done);
  s = BatchSlot{};
}

static void batch_free(lsdg_batch* b) {
  for (auto& s : b->slot) slot_free(s);
  if (b->h_counts) cudaFreeHost(b->h_counts);
  if (b->copy) cudaStreamDestroy(b->copy);
  if (b->readback) cudaStreamDestroy(b->readback);
  delete b;
}

static lsdg_status slot_alloc(lsdg_ctx* ctx, lsdg_batch* b, BatchSlot& s) {
  const int n = b->n;
  std::vector<int> w(2 * n), h(2 * n);
  std::vector<lsdg_intrinsics> k(2 * n);
  bool* dep = new (std::nothrow) bool[2 * n];
  if (!dep) return LSDG_OUT_OF_MEMORY;
  for (int i = 0; i < n; ++i) {
    w[i] = w[n + i] = b->w[i];
    h[i] = h[n + i] = b->h[i];
    k[i] = k[n + i] = b->intr[i];
    dep[i] = true;
    dep[n + i] = b->sim3;
  }
  // the tracker samples intensity planes only: no gradient pyramid for batch frames
  lsdg_status st = frameset_alloc(ctx, s.fs, 2 * n, w.data(), h.data(), k.data(), dep, ctx->params.levels, false);
  delete[] dep;
  if (st != LSDG_OK) return st;
  std::vector<PairDev> pairs(n);
  for (int i = 0; i < n; ++i) pairs[i] = PairDev{s.fs.d_frames + i, s.fs.d_frames + n + i};
  cudaError_t e = cudaMalloc(&s.d_pairs, sizeof(PairDev) * n);
  if (e == cudaSuccess) e = cudaMalloc(&s.d_init, sizeof(double) * b->pose_len * n);
  if (e == cudaSuccess) e = cudaMalloc(&s.d_out, sizeof(double) * b->pose_len * n);
  if (e == cudaSuccess) e = cudaMalloc(&s.d_stats, sizeof(lsdg_track_stats) * n);
  if (e == cudaSuccess) e = cudaMalloc(&s.d_work, sizeof(int) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&s.d_order, sizeof(int) * n);
  if (e == cudaSuccess) e = cudaMalloc(&s.d_scan, frame_build_ws_bytes(2 * b->n, s.fs.levels, s.fs.max_h));
  if (e == cudaSuccess) e = cudaMallocHost(&s.h_err, sizeof(unsigned));
  if (e == cudaSuccess) *s.h_err = 0;
  if (e == cudaSuccess && !b->sim3) e = cudaMalloc(&s.d_u8, s.fs.pix_total);
  if (e == cudaSuccess) e = cudaMalloc(&s.d_mode, sizeof(int));
  if (e == cudaSuccess) e = cudaMallocHost(&s.h_mode, 2 * sizeof(int));
  if (e == cudaSuccess) {
    s.h_mode[0] = 0;
    s.h_mode[1] = 1;
    e = cudaMemsetAsync(s.d_mode, 0, sizeof(int), ctx->stream);
  }
  if (e == cudaSuccess) e = cudaMalloc(&s.d_mid, sizeof(double) * b->pose_len * n);
  if (e == cudaSuccess) e = cudaMallocHost(&s.h_out, sizeof(double) * b->pose_len * n);
  if (e == cudaSuccess) e = cudaMallocHost(&s.h_stats, sizeof(lsdg_track_stats) * n);
  for (auto& ev : s.ev)
    if (e == cudaSuccess) e = cudaEventCreate(&ev);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.graph_done, cudaEventDisableTiming);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s.d_pairs, pairs.data(), sizeof(PairDev) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return ctx_cuda(ctx, e, "batch slot allocation");
  s.ready = true;
  return LSDG_OK;
}

static TrackArgs slot_track_args(lsdg_ctx* ctx, lsdg_batch* b, BatchSlot& s) {
  TrackArgs a = make_track_args(ctx->params);
  a.pairs = s.d_pairs;
  a.order = s.d_order;
  a.n_pairs = b->n;
  a.work_counter = s.d_work;
  a.init = s.d_init;
  a.init_is_ref_to_frame = 0;
  a.out_pose = s.d_out;
  a.out_stats = s.d_stats;
  a.out_sums = nullptr;
  return a;
}

// Processing order of a batch's pairs: by the reference keyframe's level-0 points, largest first
// (ties by pair index), so that the persistent tracker's queue hands out the longest pairs first
// (longest-processing-time-first: with more pairs than resident clusters the last round is short).
// One CTA; rank of pair i = the pairs ordered before it.
__global__ void order_by_points_kernel(const PairDev* __restrict__ pairs, int n, int* __restrict__ order) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int ki = pairs[i].ref->pcount[0];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const int kj = pairs[j].ref->pcount[0];
      rank += (kj > ki || (kj == ki && j < i)) ? 1 : 0;
    }
    order[rank] = i;
  }
}

static lsdg_status enqueue_build(lsdg_ctx* ctx, lsdg_batch* b, BatchSlot& s, int* launches) {
  // one launch over all 2n frames: pyramids (also the depth pyramids of the second keyframes in
  // Sim3 mode), reference points only for the first n
  int k = launch_frame_build(s.fs.d_frames, 2 * b->n, b->n, s.fs.levels, s.fs.max_h, s.d_scan, ctx->stream,
                             b->test_withhold, s.d_u8, s.fs.plane0, s.d_mode);
  order_by_points_kernel<<<1, 256, 0, ctx->stream>>>(s.d_pairs, b->n, s.d_order);
  ++k;
  CK(ctx, cudaGetLastError());
  *launches = k;
  return LSDG_OK;
}

// Launch slot si's graph on the context stream, tuning the shape (once per parameter set) and
// capturing the slot's graph first when needed.
static lsdg_status slot_run(lsdg_ctx* ctx, lsdg_batch* b, int si) {
  BatchSlot& s = b->slot[si];
  if (!s.exec || s.graph_epoch != ctx->params_epoch) {
    if (s.exec) {
      cudaGraphExecDestroy(s.exec);
      s.exec = nullptr;
    }
    TrackArgs a = slot_track_args(ctx, b, s);
    if (b->tune_epoch != ctx->params_epoch) {
      // eager build so that the autotuner times the tracker on this batch's real points
      int k = 0;
      lsdg_status st = enqueue_build(ctx, b, s, &k);
      if (st != LSDG_OK) return st;
      ctx->launches += k;
      st = autotune(ctx, b->key, a, &b->tc, b->sim3, s.d_mid);
      if (st != LSDG_OK) return st;
      b->tune_epoch = ctx->params_epoch;
    }
    // capture: events, build, tracker
    CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int nl = 0;
    // external records become event-record nodes of the graph (timed on every replay)
    cudaEventRecordWithFlags(s.ev[0], ctx->stream, cudaEventRecordExternal);
    lsdg_status st = enqueue_build(ctx, b, s, &nl);
    cudaEventRecordWithFlags(s.ev[1], ctx->stream, cudaEventRecordExternal);
    int64_t before = ctx->launches;
    if (st == LSDG_OK) st = run_tracker(ctx, a, b->tc, b->sim3, s.d_mid);
    nl += (int)(ctx->launches - before);
    ctx->launches = before;
    cudaEventRecordWithFlags(s.ev[2], ctx->stream, cudaEventRecordExternal);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (st != LSDG_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    CK(ctx, e);
    e = cudaGraphInstantiate(&s.exec, g, 0);
    cudaGraphDestroy(g);
    CK(ctx, e);
    b->launches_per_run = nl;
    s.graph_epoch = ctx->params_epoch;
  }
  CK(ctx, cudaGraphLaunch(s.exec, ctx->stream));
  ctx->launches += b->launches_per_run;
  s.ran = true;
  b->last = si;
  return LSDG_OK;
}

// Host -> device copies of one step's inputs into slot s on stream `st` (new_idepth / new_var:
// Sim3 batches only).
// Images as floats (ref_images / new_images) or as bytes (ref_u8 / new_u8: copied into the slot's
// staging, then widened into the level-0 planes by a kernel on the same stream).
static lsdg_status slot_upload(lsdg_ctx* ctx, lsdg_batch* b, BatchSlot& s, cudaStream_t st, const float* ref_images,
                               const float* ref_idepth, const float* ref_var, const float* new_images,
                               const float* new_idepth, const float* new_var, const double* init,
                               const uint8_t* ref_u8 = nullptr, const uint8_t* new_u8 = nullptr) {
  // keyframes first; all keyframes carry depth (and, for Sim3, the second half too)
  const size_t npix = b->sim3 ? s.fs.pix_depth / 2 : s.fs.pix_depth;
  const size_t half = npix * 4;
  char* base = (char*)s.fs.arena;
  if (ref_u8) {
    // the bytes go to the staging (laid out like the level-0 planes); the build widens them
    if (!s.d_u8) return ctx_fail(ctx, LSDG_INVALID_ARG, "8-bit images need an SE3 batch");
    CK(ctx, cudaMemcpyAsync(s.d_u8, ref_u8, npix, cudaMemcpyHostToDevice, st));
    CK(ctx, cudaMemcpyAsync(s.d_u8 + npix, new_u8, npix, cudaMemcpyHostToDevice, st));
    CK(ctx, cudaMemcpyAsync(s.d_mode, s.h_mode + 1, sizeof(int), cudaMemcpyHostToDevice, st));
  } else {
    CK(ctx, cudaMemcpyAsync(s.fs.plane0, ref_images, half, cudaMemcpyHostToDevice, st));
    CK(ctx, cudaMemcpyAsync((char*)s.fs.plane0 + half, new_images, half, cudaMemcpyHostToDevice, st));
    CK(ctx, cudaMemcpyAsync(s.d_mode, s.h_mode, sizeof(int), cudaMemcpyHostToDevice, st));
  }
  CK(ctx, cudaMemcpyAsync(base + s.fs.off_id0, ref_idepth, half, cudaMemcpyHostToDevice, st));
  CK(ctx, cudaMemcpyAsync(base + s.fs.off_var0, ref_var, half, cudaMemcpyHostToDevice, st));
  if (b->sim3) {
    CK(ctx, cudaMemcpyAsync(base + s.fs.off_id0 + half, new_idepth, half, cudaMemcpyHostToDevice, st));
    CK(ctx, cudaMemcpyAsync(base + s.fs.off_var0 + half, new_var, half, cudaMemcpyHostToDevice, st));
  }
  CK(ctx, cudaMemcpyAsync(s.d_init, init, sizeof(double) * b->pose_len * b->n, cudaMemcpyHostToDevice, st));
  return LSDG_OK;
}

// The step's one-launch build reports a band wait that ran out (its error word, copied back with
// the results): the poses of that step are not to be trusted.
static lsdg_status build_error(lsdg_ctx* ctx, const BatchSlot& s) {
  if (s.h_err && *s.h_err)
    return ctx_fail(ctx, LSDG_TIMEOUT, "keyframe build: a band's wait for the point counts of the bands before it ran out");
  return LSDG_OK;
}

static lsdg_status check_sim3_init(lsdg_ctx* ctx, const lsdg_batch* b, const double* init) {
  for (int i = 0; i < b->n; ++i)
    if (!(init[13 * i + 12] > 0)) return ctx_fail(ctx, LSDG_INVALID_ARG, "pair %d: Sim3 scale must be > 0", i);
  return LSDG_OK;
}

static lsdg_status no_pipeline(lsdg_ctx* ctx, const lsdg_batch* b) {
  if (b->n_inflight) return ctx_fail(ctx, LSDG_INVALID_ARG, "collect the submitted steps first");
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
  b->w.assign(widths, widths + n);
  b->h.assign(heights, heights + n);
  b->intr.assign(intr, intr + n);
  lsdg_status st = slot_alloc(ctx, b, b->slot[0]);
  if (st != LSDG_OK) {
    batch_free(b);
    return st;
  }
  cudaError_t e = cudaMallocHost(&b->h_counts, sizeof(int) * kMaxLevels * n);
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

// One pipelined step: upload into the free slot on the copy stream, run its graph behind the
// upload, read the results back behind the graph.
static lsdg_status batch_submit(lsdg_ctx* ctx, lsdg_batch* b, const float* ri, const float* rd, const float* rv,
                                const float* ni, const float* nd, const float* nv, const double* init,
                                const uint8_t* ri8 = nullptr, const uint8_t* ni8 = nullptr) {
  if (b->n_inflight >= 2) return ctx_fail(ctx, LSDG_INVALID_ARG, "two steps in flight: collect one first");
  const int si = b->next;
  BatchSlot& s = b->slot[si];
  if (!s.ready) {
    lsdg_status st = slot_alloc(ctx, b, s);
    if (st != LSDG_OK) return st;
  }
  if (!b->copy) CK(ctx, cudaStreamCreateWithFlags(&b->copy, cudaStreamNonBlocking));
  if (!b->readback) CK(ctx, cudaStreamCreateWithFlags(&b->readback, cudaStreamNonBlocking));
  if (!s.exec || s.graph_epoch != ctx->params_epoch) {
    // first use of this slot (or new parameters): upload on the context stream, then tune/capture
    lsdg_status st = slot_upload(ctx, b, s, ctx->stream, ri, rd, rv, ni, nd, nv, init, ri8, ni8);
    if (st == LSDG_OK) st = slot_run(ctx, b, si);
    if (st != LSDG_OK) return st;
  } else {
    // the slot's arena is free once its previous step has finished (event `done`)
    CK(ctx, cudaStreamWaitEvent(b->copy, s.done, 0));
    lsdg_status st = slot_upload(ctx, b, s, b->copy, ri, rd, rv, ni, nd, nv, init, ri8, ni8);
    if (st != LSDG_OK) return st;
    CK(ctx, cudaEventRecord(s.copied, b->copy));
    CK(ctx, cudaStreamWaitEvent(ctx->stream, s.copied, 0));
    st = slot_run(ctx, b, si);
    if (st != LSDG_OK) return st;
  }
  // the results come back on the read-back stream, so the next step's graph does not queue behind
  // these copies; the slot's next upload waits for them (event done)
  CK(ctx, cudaEventRecord(s.graph_done, ctx->stream));
  CK(ctx, cudaStreamWaitEvent(b->readback, s.graph_done, 0));
  CK(ctx, cudaMemcpyAsync(s.h_out, s.d_out, sizeof(double) * b->pose_len * b->n, cudaMemcpyDeviceToHost, b->readback));
  CK(ctx, cudaMemcpyAsync(s.h_stats, s.d_stats, sizeof(lsdg_track_stats) * b->n, cudaMemcpyDeviceToHost, b->readback));
  CK(ctx, cudaMemcpyAsync(s.h_err, reinterpret_cast<unsigned*>(s.d_scan) + 1, sizeof(unsigned), cudaMemcpyDeviceToHost,
                          b->readback));
  CK(ctx, cudaEventRecord(s.done, b->readback));
  b->inflight[b->n_inflight++] = si;
  b->next = si ^ 1;
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
  if (b->copy) cudaStreamSynchronize(b->copy);
  if (b->readback) cudaStreamSynchronize(b->readback);
  batch_free(b);
  return LSDG_OK;
}

lsdg_status lsdg_batch_load(lsdg_ctx* ctx, lsdg_batch* b, const float* ref_images, const float* ref_idepth,
                            const float* ref_var, const float* new_images, const double* init) {
  if (!ctx || !b || !ref_images || !ref_idepth || !ref_var || !new_images || !init)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (b->sim3) return ctx_fail(ctx, LSDG_INVALID_ARG, "Sim3 batch: use lsdg_batch_load_sim3");
  lsdg_status st = no_pipeline(ctx, b);
  if (st != LSDG_OK) return st;
  return slot_upload(ctx, b, b->slot[0], ctx->stream, ref_images, ref_idepth, ref_var, new_images, nullptr, nullptr,
                     init);
}

lsdg_status lsdg_batch_load_sim3(lsdg_ctx* ctx, lsdg_batch* b, const float* ref_images, const float* ref_idepth,
                                 const float* ref_var, const float* new_images, const float* new_idepth,
                                 const float* new_var, const double* init) {
  if (!ctx || !b || !ref_images || !ref_idepth || !ref_var || !new_images || !new_idepth || !new_var || !init)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!b->sim3) return ctx_fail(ctx, LSDG_INVALID_ARG, "not a Sim3 batch (lsdg_batch_create_sim3)");
  lsdg_status st = check_sim3_init(ctx, b, init);
  if (st == LSDG_OK) st = no_pipeline(ctx, b);
  if (st != LSDG_OK) return st;
  return slot_upload(ctx, b, b->slot[0], ctx->stream, ref_images, ref_idepth, ref_var, new_images, new_idepth,
                     new_var, init);
}

lsdg_status lsdg_batch_load_frames(lsdg_ctx* ctx, lsdg_batch* b, const lsdg_frame* const* refs,
                                   const lsdg_frame* const* frames, const double* init) {
  if (!ctx || !b || !refs || !frames || !init) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  lsdg_status st = no_pipeline(ctx, b);
  if (st == LSDG_OK && b->sim3) st = check_sim3_init(ctx, b, init);
  if (st != LSDG_OK) return st;
  BatchSlot& s = b->slot[0];
  for (int i = 0; i < b->n; ++i) {
    if (!refs[i] || !frames[i]) return ctx_fail(ctx, LSDG_INVALID_ARG, "pair %d: null frame", i);
    const FrameDev& R = refs[i]->fs.h_frames[0];
    const FrameDev& F = frames[i]->fs.h_frames[0];
    if (R.w != b->w[i] || R.h != b->h[i] || F.w != b->w[i] || F.h != b->h[i])
      return ctx_fail(ctx, LSDG_INVALID_ARG, "pair %d: frame size differs from the batch's", i);
    if (!refs[i]->has_image || !frames[i]->has_image || !R.has_depth || (b->sim3 && !F.has_depth))
      return ctx_fail(ctx, LSDG_INVALID_ARG, "pair %d: image or depth missing", i);
  }
  for (int i = 0; i < b->n; ++i) {
    const FrameDev& R = refs[i]->fs.h_frames[0];
    const FrameDev& F = frames[i]->fs.h_frames[0];
    const FrameDev& Ki = s.fs.h_frames[i];
    const FrameDev& Kj = s.fs.h_frames[b->n + i];
    const size_t bytes = (size_t)b->w[i] * b->h[i] * 4;
    const cudaMemcpyKind d2d = cudaMemcpyDeviceToDevice;
    if (i == 0) CK(ctx, cudaMemcpyAsync(s.d_mode, s.h_mode, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaMemcpyAsync(Ki.plane[0], R.plane[0], bytes, d2d, ctx->stream));
    CK(ctx, cudaMemcpyAsync(Ki.idepth[0], R.idepth[0], bytes, d2d, ctx->stream));
    CK(ctx, cudaMemcpyAsync(Ki.ivar[0], R.ivar[0], bytes, d2d, ctx->stream));
    CK(ctx, cudaMemcpyAsync(Kj.plane[0], F.plane[0], bytes, d2d, ctx->stream));
    if (b->sim3) {
      CK(ctx, cudaMemcpyAsync(Kj.idepth[0], F.idepth[0], bytes, d2d, ctx->stream));
      CK(ctx, cudaMemcpyAsync(Kj.ivar[0], F.ivar[0], bytes, d2d, ctx->stream));
    }
  }
  CK(ctx, cudaMemcpyAsync(s.d_init, init, sizeof(double) * b->pose_len * b->n, cudaMemcpyHostToDevice, ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_batch_run(lsdg_ctx* ctx, lsdg_batch* b) {
  if (!ctx || !b) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  lsdg_status st = no_pipeline(ctx, b);
  if (st != LSDG_OK) return st;
  return slot_run(ctx, b, 0);
}

lsdg_status lsdg_batch_read(lsdg_ctx* ctx, lsdg_batch* b, double* out, lsdg_track_stats* stats) {
  if (!ctx || !b) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  lsdg_status st = no_pipeline(ctx, b);
  if (st != LSDG_OK) return st;
  BatchSlot& s = b->slot[0];
  CK(ctx, cudaMemcpyAsync(s.h_out, s.d_out, sizeof(double) * b->pose_len * b->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(s.h_stats, s.d_stats, sizeof(lsdg_track_stats) * b->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(s.h_err, reinterpret_cast<unsigned*>(s.d_scan) + 1, sizeof(unsigned), cudaMemcpyDeviceToHost,
                          ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (out) std::memcpy(out, s.h_out, sizeof(double) * b->pose_len * b->n);
  if (stats) std::memcpy(stats, s.h_stats, sizeof(lsdg_track_stats) * b->n);
  return build_error(ctx, s);
}

lsdg_status lsdg_batch_submit_se3(lsdg_ctx* ctx, lsdg_batch* b, const float* ref_images, const float* ref_idepth,
                                  const float* ref_var, const float* new_images, const double* init) {
  if (!ctx || !b || !ref_images || !ref_idepth || !ref_var || !new_images || !init)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (b->sim3) return ctx_fail(ctx, LSDG_INVALID_ARG, "Sim3 batch: use lsdg_batch_submit_sim3");
  return batch_submit(ctx, b, ref_images, ref_idepth, ref_var, new_images, nullptr, nullptr, init);
}

lsdg_status lsdg_batch_submit_se3_u8(lsdg_ctx* ctx, lsdg_batch* b, const uint8_t* ref_images, const float* ref_idepth,
                                     const float* ref_var, const uint8_t* new_images, const double* init) {
  if (!ctx || !b || !ref_images || !ref_idepth || !ref_var || !new_images || !init)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (b->sim3) return ctx_fail(ctx, LSDG_INVALID_ARG, "Sim3 batch: use lsdg_batch_submit_sim3");
  return batch_submit(ctx, b, nullptr, ref_idepth, ref_var, nullptr, nullptr, nullptr, init, ref_images, new_images);
}

lsdg_status lsdg_batch_submit_sim3(lsdg_ctx* ctx, lsdg_batch* b, const float* ref_images, const float* ref_idepth,
                                   const float* ref_var, const float* new_images, const float* new_idepth,
                                   const float* new_var, const double* init) {
  if (!ctx || !b || !ref_images || !ref_idepth || !ref_var || !new_images || !new_idepth || !new_var || !init)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!b->sim3) return ctx_fail(ctx, LSDG_INVALID_ARG, "not a Sim3 batch (lsdg_batch_create_sim3)");
  lsdg_status st = check_sim3_init(ctx, b, init);
  if (st != LSDG_OK) return st;
  return batch_submit(ctx, b, ref_images, ref_idepth, ref_var, new_images, new_idepth, new_var, init);
}

lsdg_status lsdg_batch_collect(lsdg_ctx* ctx, lsdg_batch* b, double* out, lsdg_track_stats* stats) {
  if (!ctx || !b) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!b->n_inflight) return ctx_fail(ctx, LSDG_INVALID_ARG, "no submitted step to collect");
  const int si = b->inflight[0];
  BatchSlot& s = b->slot[si];
  CK(ctx, cudaEventSynchronize(s.done));
  if (out) std::memcpy(out, s.h_out, sizeof(double) * b->pose_len * b->n);
  if (stats) std::memcpy(stats, s.h_stats, sizeof(lsdg_track_stats) * b->n);
  b->inflight[0] = b->inflight[1];
  b->inflight[1] = -1;
  --b->n_inflight;
  return build_error(ctx, s);
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
  if (!ctx || !b || !b->slot[b->last].ran) return ctx_fail(ctx, LSDG_INVALID_ARG, "no run to time");
  BatchSlot& s = b->slot[b->last];
  CK(ctx, cudaEventSynchronize(s.ev[2]));
  float a = 0, c = 0;
  CK(ctx, cudaEventElapsedTime(&a, s.ev[0], s.ev[1]));
  CK(ctx, cudaEventElapsedTime(&c, s.ev[1], s.ev[2]));
  if (build_ms) *build_ms = a;
  if (track_ms) *track_ms = c;
  return LSDG_OK;
}

lsdg_status lsdg_batch_work(lsdg_ctx* ctx, lsdg_batch* b, int64_t* passes, double* pass_bytes, double* unique_bytes) {
  if (!ctx || !b || !b->slot[b->last].ran) return ctx_fail(ctx, LSDG_INVALID_ARG, "no run to account");
  BatchSlot& s = b->slot[b->last];
  const int L = ctx->params.levels;
  std::vector<lsdg_track_stats> stats(b->n);
  for (int i = 0; i < b->n; ++i)
    CK(ctx, cudaMemcpyAsync(b->h_counts + kMaxLevels * i, s.fs.h_frames[i].pcount, sizeof(int) * kMaxLevels,
                            cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaMemcpyAsync(stats.data(), s.d_stats, sizeof(lsdg_track_stats) * b->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  int64_t np = 0;
  double pb = 0, ub = 0;
  for (int i = 0; i < b->n; ++i) {
    for (int l = 0; l < L; ++l) {
      const double pts = b->h_counts[kMaxLevels * i + l];
      const double pix = (double)(b->w[i] >> l) * (b->h[i] >> l);
      const int ps = stats[i].passes[l];
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

// The coarse phase of the autotuner's plan for this batch (split = -1: one launch).
lsdg_status lsdg_batch_split(lsdg_ctx* ctx, lsdg_batch* b, int* split, int* threads, int* minblocks, int* cluster) {
  if (!ctx || !b) return LSDG_INVALID_ARG;
  if (split) *split = b->tc.split;
  if (threads) *threads = b->tc.c_threads;
  if (minblocks) *minblocks = b->tc.c_minblocks;
  if (cluster) *cluster = b->tc.c_cluster;
  return LSDG_OK;
}

lsdg_status lsdg_batch_test_withhold(lsdg_ctx* ctx, lsdg_batch* b, int frame) {
  if (!ctx || !b) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (frame < -1 || frame >= b->n) return ctx_fail(ctx, LSDG_INVALID_ARG, "frame out of range");
  lsdg_status st = no_pipeline(ctx, b);
  if (st != LSDG_OK) return st;
  b->test_withhold = frame;
  for (auto& s : b->slot) s.graph_epoch = -1;  // capture again with the new launch argument
  b->tune_epoch = -1;  // a shape tuned on withheld (incomplete) points is not kept: tune again
  return LSDG_OK;
}

lsdg_status lsdg_batch_get_points(lsdg_ctx* ctx, lsdg_batch* b, int pair, int level, float* xyzi, float* var,
                                  int capacity, int* count) {
  if (!ctx || !b || !count) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (pair < 0 || pair >= b->n) return ctx_fail(ctx, LSDG_INVALID_ARG, "pair out of range");
  const BatchSlot& s = b->slot[b->last];
  if (!s.ready) return ctx_fail(ctx, LSDG_INVALID_ARG, "the batch has not run");
  const FrameDev& F = s.fs.h_frames[pair];
  if (level < 0 || level >= F.levels) return ctx_fail(ctx, LSDG_INVALID_ARG, "level out of range");
  if (b->n_inflight) CK(ctx, cudaEventSynchronize(s.done));
  int c = 0;
  CK(ctx, cudaMemcpyAsync(ctx->h_small, F.pcount + level, 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  std::memcpy(&c, ctx->h_small, 4);
  *count = c;
  if (c > capacity) return ctx_fail(ctx, LSDG_INVALID_ARG, "capacity %d < %d points", capacity, c);
  if (xyzi && c) CK(ctx, cudaMemcpyAsync(xyzi, F.pxyzi[level], (size_t)c * 16, cudaMemcpyDeviceToHost, ctx->stream));
  if (var && c) CK(ctx, cudaMemcpyAsync(var, F.pvar[level], (size_t)c * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
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

// api.cu -- host side of the C-ABI declared in include/lsdg.h: contexts, frames, batches, the
// CUDA-graph capture of a batch step and the tile-shape autotuner.  No compute happens here; every
// result comes from the kernels in frame.cu / track.cu / depth.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "lsdg_internal.cuh"
#include "lsdg_host.h"

using namespace lsdg;

namespace lsdg {
int launch_frame_pyramid(const FrameDev* frames, int n, int levels, long max_pix, int max_h, bool with_grads,
                         cudaStream_t s);
int launch_frame_points(const FrameDev* frames, int n, int levels, int max_h, cudaStream_t s);
void launch_u8_to_plane(const uint8_t* src, float* dst, int n, cudaStream_t s);
cudaError_t launch_track(const TrackArgs& a, int threads, int minblocks, int cluster, int n_clusters, cudaStream_t s,
                         bool sim3);
int track_max_clusters(int threads, int minblocks, int cluster, bool sim3);
cudaError_t track_prepare();
int track_shape_count();
void track_shape(int i, int* threads, int* minblocks);
}  // namespace lsdg

// ============================================================================================
// Context
// ============================================================================================

lsdg_status ctx_fail(lsdg_ctx* ctx, lsdg_status st, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return st;
}

lsdg_status ctx_cuda(lsdg_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return LSDG_OK;
  return ctx_fail(ctx, e == cudaErrorMemoryAllocation ? LSDG_OUT_OF_MEMORY : LSDG_CUDA_ERROR, "%s: %s (%s)", what,
                  cudaGetErrorString(e), cudaGetErrorName(e));
}

#define CK(ctx, expr)                                         \
  do {                                                        \
    lsdg_status _s = ctx_cuda((ctx), (expr), #expr);          \
    if (_s != LSDG_OK) return _s;                             \
  } while (0)

extern "C" {

int32_t lsdg_abi_version(void) { return 1; }

void lsdg_default_params(lsdg_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->levels = 5;
  const int iters[LSDG_MAX_LEVELS] = {6, 8, 10, 12, 16, 16};
  for (int i = 0; i < LSDG_MAX_LEVELS; ++i) p->max_iterations[i] = iters[i];
  p->photometric_variance = 16.0f;
  p->huber_delta = 2.0f;
  p->min_z = 0.01f;
  p->border_margin = 2.5f;
  p->lm_lambda_initial = 0.01f;
  p->lm_lambda_up = 4.0f;
  p->lm_lambda_down = 0.5f;
  p->step_eps = 1e-5f;
  p->stall_eps = 5e-4f;
  p->min_good_ratio = 0.5f;
  p->min_usage = 0.2f;
  p->sim3_depth_variance = 1e-4f;
  p->sim3_depth_weight = 1.0f;
  p->min_grad = 5.0f;
  p->min_idepth = 0.05f;
  p->max_idepth = 2.0f;
  p->epipolar_var = 0.25f;
  p->image_var = 4.0f;
  p->min_grad_along_epl2 = 0.1f;
  p->max_ssd = 100.0f;
  p->unique_ratio = 1.2f;
  p->search_sigmas = 2.0f;
  p->max_search_len = 120.0f;
  p->min_search_len = 3.0f;
  p->fuse_chi2 = 6.25f;
  p->min_epl_length = 1.0f;
  p->validity_init = 2;
  p->validity_max = 20;
  p->validity_penalty = 2;
  p->blacklist_limit = 5;
  p->prediction_var = 1e-4f;
  p->propagate_max_photo_diff = 30.0f;
  p->reg_radius = 2;
  p->reg_chi2 = 4.0f;
  p->reg_min_support = 2;
  p->fill_min_support = 8;
  p->fill_var_factor = 2.0f;
  p->refine_prior_weight = 1.0f;
}

static lsdg_status check_params(lsdg_ctx* ctx, const lsdg_params* p) {
  if (p->levels < 1 || p->levels > LSDG_MAX_LEVELS) return ctx_fail(ctx, LSDG_INVALID_ARG, "levels must be in 1..%d", LSDG_MAX_LEVELS);
  for (int i = 0; i < LSDG_MAX_LEVELS; ++i)
    if (p->max_iterations[i] < 0 || p->max_iterations[i] > 1000) return ctx_fail(ctx, LSDG_INVALID_ARG, "max_iterations out of range");
  if (!(p->photometric_variance > 0) || !(p->huber_delta > 0)) return ctx_fail(ctx, LSDG_INVALID_ARG, "variance and huber_delta must be > 0");
  if (p->reg_radius < 0 || p->reg_radius > 4) return ctx_fail(ctx, LSDG_INVALID_ARG, "reg_radius must be in 0..4");
  if (!(p->max_search_len > 0) || p->max_search_len > 1024) return ctx_fail(ctx, LSDG_INVALID_ARG, "max_search_len must be in (0, 1024]");
  if (!(p->refine_prior_weight >= 0)) return ctx_fail(ctx, LSDG_INVALID_ARG, "refine_prior_weight must be >= 0");
  return LSDG_OK;
}

lsdg_status lsdg_create(lsdg_ctx** out, const lsdg_params* params, int device) {
  if (!out) return LSDG_INVALID_ARG;
  *out = nullptr;
  lsdg_ctx* ctx = new (std::nothrow) lsdg_ctx();
  if (!ctx) return LSDG_OUT_OF_MEMORY;
  if (params) ctx->params = *params;
  else lsdg_default_params(&ctx->params);
  lsdg_status st = check_params(ctx, &ctx->params);
  if (st != LSDG_OK) { delete ctx; return st; }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev <= device || device < 0) {
    cudaGetLastError();
    delete ctx;
    return LSDG_CUDA_ERROR;
  }
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return LSDG_CUDA_ERROR;
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  int cc_major = 0, cc_minor = 0;
  cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&cc_minor, cudaDevAttrComputeCapabilityMinor, device);
  if (cc_major != 10 || cc_minor != 3) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return LSDG_NOT_SUPPORTED;  // built for sm_103a only
  }
  if (track_prepare() != cudaSuccess) cudaGetLastError();  // clusters then stay <= 8 (the tuner sees 0 for 16)
  if (cudaMalloc(&ctx->d_small, kSmallBytes) != cudaSuccess || cudaMallocHost(&ctx->h_small, kSmallBytes) != cudaSuccess) {
    cudaGetLastError();
    if (ctx->d_small) cudaFree(ctx->d_small);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return LSDG_OUT_OF_MEMORY;
  }
  *out = ctx;
  return LSDG_OK;
}

lsdg_status lsdg_destroy(lsdg_ctx* ctx) {
  if (!ctx) return LSDG_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->d_small) cudaFree(ctx->d_small);
  if (ctx->h_small) cudaFreeHost(ctx->h_small);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return LSDG_OK;
}

lsdg_status lsdg_set_params(lsdg_ctx* ctx, const lsdg_params* p) {
  if (!ctx || !p) return LSDG_INVALID_ARG;
  lsdg_status st = check_params(ctx, p);
  if (st != LSDG_OK) return st;
  ctx->params = *p;
  ctx->params_epoch++;
  return LSDG_OK;
}

const char* lsdg_last_error(const lsdg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }
void* lsdg_stream(lsdg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
int64_t lsdg_launch_count(const lsdg_ctx* ctx) { return ctx ? ctx->launches : 0; }

lsdg_status lsdg_sync(lsdg_ctx* ctx) {
  if (!ctx) return LSDG_INVALID_ARG;
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

}  // extern "C"

// ============================================================================================
// Frame sets: device storage for n frames of possibly different sizes
// ============================================================================================

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

lsdg_status frameset_alloc(lsdg_ctx* ctx, FrameSet& fs, int n, const int* w, const int* h,
                           const lsdg_intrinsics* intr, const bool* depth, int levels, bool grads) {
  fs.n = n;
  fs.levels = levels;
  fs.w.assign(w, w + n);
  fs.h.assign(h, h + n);
  fs.intr.assign(intr, intr + n);
  fs.depth.assign(depth, depth + n);
  fs.max_pix = 0;
  fs.max_h = 0;
  const int mult = 1 << (levels - 1);
  for (int i = 0; i < n; ++i) {
    if (w[i] <= 0 || h[i] <= 0 || w[i] % mult || h[i] % mult || (w[i] >> (levels - 1)) < 4 || (h[i] >> (levels - 1)) < 4)
      return ctx_fail(ctx, LSDG_INVALID_ARG, "frame %d: %dx%d must be positive multiples of %d with >= 4 pixels at the top level", i, w[i], h[i], mult);
    if (!(intr[i].fx > 0) || !(intr[i].fy > 0)) return ctx_fail(ctx, LSDG_INVALID_ARG, "frame %d: focal lengths must be > 0", i);
    fs.max_pix = std::max(fs.max_pix, (long)w[i] * h[i]);
    fs.max_h = std::max(fs.max_h, h[i]);
  }
  // sections: level-0 intensity of every frame back to back, then level-0 idepth and variance of
  // the depth frames back to back (so a batch upload is one copy per kind), then per-frame rest.
  size_t off = 0;
  std::vector<size_t> o_plane0(n), o_id0(n), o_var0(n);
  for (int i = 0; i < n; ++i) { o_plane0[i] = off; off += (size_t)w[i] * h[i] * 4; }
  off = al256(off);
  fs.off_id0 = off;
  for (int i = 0; i < n; ++i) if (depth[i]) { o_id0[i] = off; off += (size_t)w[i] * h[i] * 4; }
  off = al256(off);
  fs.off_var0 = off;
  for (int i = 0; i < n; ++i) if (depth[i]) { o_var0[i] = off; off += (size_t)w[i] * h[i] * 4; }
  off = al256(off);
  struct Rest { size_t plane[kMaxLevels], pyr[kMaxLevels], id[kMaxLevels], var[kMaxLevels], pxyzi[kMaxLevels], pvar[kMaxLevels], psig[kMaxLevels], psigd[kMaxLevels], ppix[kMaxLevels], blk[kMaxLevels], cnt; };
  std::vector<Rest> rest(n);
  for (int i = 0; i < n; ++i) {
    Rest& r = rest[i];
    for (int l = 0; l < levels; ++l) {
      size_t pix = (size_t)(w[i] >> l) * (h[i] >> l);
      if (l > 0) { r.plane[l] = off; off = al256(off + pix * 4); }
      if (grads) { r.pyr[l] = off; off = al256(off + pix * 16); }
      if (depth[i]) {
        if (l > 0) {
          r.id[l] = off; off = al256(off + pix * 4);
          r.var[l] = off; off = al256(off + pix * 4);
        }
        r.pxyzi[l] = off; off = al256(off + pix * 16);
        r.pvar[l] = off; off = al256(off + pix * 4);
        r.psig[l] = off; off = al256(off + pix * 4);
        r.psigd[l] = off; off = al256(off + pix * 4);
        if (grads) { r.ppix[l] = off; off = al256(off + pix * 4); }
        r.blk[l] = off; off = al256(off + (size_t)(h[i] >> (levels - 1)) * 4);  // one count per band
      }
    }
    r.cnt = off;
    off = al256(off + kMaxLevels * 4);
  }
  fs.arena_bytes = off;
  CK(ctx, cudaMalloc(&fs.arena, off));
  CK(ctx, cudaMemsetAsync(fs.arena, 0, off, ctx->stream));
  char* base = (char*)fs.arena;
  fs.h_frames.assign(n, FrameDev{});
  for (int i = 0; i < n; ++i) {
    FrameDev& F = fs.h_frames[i];
    const Rest& r = rest[i];
    F.w = w[i];
    F.h = h[i];
    F.has_depth = depth[i] ? 1 : 0;
    F.levels = levels;
    double fx = intr[i].fx, fy = intr[i].fy, cx = intr[i].cx, cy = intr[i].cy;
    for (int l = 0; l < levels; ++l) {
      F.plane[l] = (float*)(base + (l == 0 ? o_plane0[i] : r.plane[l]));
      F.pyr[l] = grads ? (float4*)(base + r.pyr[l]) : nullptr;
      if (depth[i]) {
        F.idepth[l] = (float*)(base + (l == 0 ? o_id0[i] : r.id[l]));
        F.ivar[l] = (float*)(base + (l == 0 ? o_var0[i] : r.var[l]));
        F.pxyzi[l] = (float4*)(base + r.pxyzi[l]);
        F.pvar[l] = (float*)(base + r.pvar[l]);
        F.psig[l] = (float*)(base + r.psig[l]);
        F.psigd[l] = (float*)(base + r.psigd[l]);
        F.ppix[l] = grads ? (int*)(base + r.ppix[l]) : nullptr;
        F.blk_count[l] = (int*)(base + r.blk[l]);
      }
      F.rowdiv[l] = 0xffffffffffffffffull / (unsigned long long)(w[i] >> l) + 1ull;
      F.fx[l] = (float)fx; F.fy[l] = (float)fy; F.cx[l] = (float)cx; F.cy[l] = (float)cy;
      F.fxi[l] = (float)(1.0 / fx); F.fyi[l] = (float)(1.0 / fy);
      fx *= 0.5; fy *= 0.5;
      cx = (cx + 0.5) * 0.5 - 0.5;
      cy = (cy + 0.5) * 0.5 - 0.5;
    }
    F.pcount = (int*)(base + r.cnt);
  }
  fs.plane0 = (float*)base;
  fs.pix_total = 0;
  fs.pix_depth = 0;
  for (int i = 0; i < n; ++i) {
    fs.pix_total += (size_t)w[i] * h[i];
    if (depth[i]) fs.pix_depth += (size_t)w[i] * h[i];
  }
  CK(ctx, cudaMalloc(&fs.d_frames, sizeof(FrameDev) * n));
  CK(ctx, cudaMemcpyAsync(fs.d_frames, fs.h_frames.data(), sizeof(FrameDev) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

void frameset_free(FrameSet& fs) {
  if (fs.arena) cudaFree(fs.arena);
  if (fs.d_frames) cudaFree(fs.d_frames);
  fs.arena = nullptr;
  fs.d_frames = nullptr;
}

// ============================================================================================
// Tracker launch configuration and autotuner
// ============================================================================================

TrackArgs make_track_args(const lsdg_params& p) {
  TrackArgs a;
  std::memset(&a, 0, sizeof(a));
  a.top_level = p.levels - 1;
  a.bottom_level = 0;
  for (int i = 0; i < kMaxLevels; ++i) a.max_iter[i] = p.max_iterations[i];
  a.photometric_variance = p.photometric_variance;
  a.huber_delta = p.huber_delta;
  a.min_z = p.min_z;
  a.lambda0 = p.lm_lambda_initial;
  a.lambda_up = p.lm_lambda_up;
  a.lambda_down = p.lm_lambda_down;
  a.border_margin = p.border_margin;
  a.step_eps = p.step_eps;
  a.stall_eps = p.stall_eps;
  a.min_good_ratio = p.min_good_ratio;
  a.min_usage = p.min_usage;
  a.sim3_depth_variance = p.sim3_depth_variance;
  a.sim3_depth_weight = p.sim3_depth_weight;
  return a;
}

// Candidate tile shapes: (threads per CTA, register budget for that many CTAs per SM) x CTAs per
// cluster (the cluster owns one pair).
static const int kCandCluster[] = {2, 4, 8, 16};

static lsdg_status launch_phase(lsdg_ctx* ctx, const TrackArgs& a, int threads, int minblocks, int cluster,
                                int max_clusters, bool sim3) {
  const int n_clusters = std::min(a.n_pairs, std::max(1, max_clusters));
  CK(ctx, cudaMemsetAsync(a.work_counter, 0, sizeof(int), ctx->stream));
  CK(ctx, launch_track(a, threads, minblocks, cluster, n_clusters, ctx->stream, sim3));
  ctx->launches += 1;
  return LSDG_OK;
}

static bool use_split(const TrackArgs& a, const TuneChoice& tc, const double* mid) {
  return tc.split >= 1 && mid && a.top_level >= tc.split && a.bottom_level < tc.split;
}

// The two phases of a split run: coarse levels [top, split] (out_pose -> mid), then the finer
// levels from those poses, continuing each pair's pass counts.
static void split_args(const TrackArgs& a, int split, double* mid, TrackArgs* a1, TrackArgs* a2) {
  *a1 = a;
  a1->bottom_level = split;
  a1->out_pose = mid;
  a1->out_sums = nullptr;
  a1->accumulate_stats = 0;
  *a2 = a;
  a2->top_level = split - 1;
  a2->init = mid;
  a2->init_is_ref_to_frame = 0;
  a2->accumulate_stats = 1;
}

lsdg_status run_tracker(lsdg_ctx* ctx, const TrackArgs& a, const TuneChoice& tc, bool sim3, double* mid) {
  if (use_split(a, tc, mid)) {
    TrackArgs a1, a2;
    split_args(a, tc.split, mid, &a1, &a2);
    lsdg_status st = launch_phase(ctx, a1, tc.c_threads, tc.c_minblocks, tc.c_cluster, tc.c_max_clusters, sim3);
    if (st != LSDG_OK) return st;
    return launch_phase(ctx, a2, tc.threads, tc.minblocks, tc.cluster, tc.max_clusters, sim3);
  }
  return launch_phase(ctx, a, tc.threads, tc.minblocks, tc.cluster, tc.max_clusters, sim3);
}

// Times one launch shape on `a` (best of three runs).
static lsdg_status time_phase(lsdg_ctx* ctx, const TrackArgs& a, int nt, int mb, int c, int mc, bool sim3,
                              cudaEvent_t e0, cudaEvent_t e1, float* ms_out) {
  float t_best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    CK(ctx, cudaEventRecord(e0, ctx->stream));
    lsdg_status st = launch_phase(ctx, a, nt, mb, c, mc, sim3);
    if (st != LSDG_OK) return st;
    CK(ctx, cudaEventRecord(e1, ctx->stream));
    CK(ctx, cudaEventSynchronize(e1));
    float ms = 0;
    CK(ctx, cudaEventElapsedTime(&ms, e0, e1));
    t_best = std::min(t_best, ms);
  }
  *ms_out = t_best;
  return LSDG_OK;
}

// Best shape over the candidates for one phase; clusters: the cluster sizes to try.
static lsdg_status best_phase(lsdg_ctx* ctx, const TrackArgs& a, const int* clusters, int n_clusters, bool sim3,
                              cudaEvent_t e0, cudaEvent_t e1, int* nt_o, int* mb_o, int* c_o, int* mc_o,
                              float* ms_o) {
  *ms_o = 1e30f;
  *nt_o = 0;
  for (int si = 0; si < track_shape_count(); ++si)
    for (int k = 0; k < n_clusters; ++k) {
      int nt = 0, mb = 0;
      track_shape(si, &nt, &mb);
      const int c = clusters[k];
      const int mc = track_max_clusters(nt, mb, c, sim3);
      if (mc <= 0) continue;
      float ms = 0;
      lsdg_status st = time_phase(ctx, a, nt, mb, c, mc, sim3, e0, e1, &ms);
      if (st != LSDG_OK) return st;
      if (ms < *ms_o) {
        *ms_o = ms;
        *nt_o = nt;
        *mb_o = mb;
        *c_o = c;
        *mc_o = mc;
      }
    }
  return LSDG_OK;
}

// Picks (threads, cluster) for a workload signature by timing every feasible candidate on the
// caller's own data (two runs each, best kept).  The choice is cached per context.
// The environment variable LSDG_TRACK_SHAPE="threads,cluster" pins the shape instead (used to
// profile one known configuration); it is ignored when that shape does not fit the device.
// Picks the tracker's launch plan for a workload signature by timing candidates on the caller's
// own data (three runs each, best kept): the best single launch over all levels, and, when the caller
// provides pose scratch, split runs (coarse levels first with each pair on a cluster of 1, 2 or 4 CTAs,
// then the finer levels with their own best shape).  The fastest plan is cached per context.
// LSDG_TRACK_SHAPE="threads,cluster[,minblocks]" pins a single-launch shape;
// LSDG_TRACK_SPLIT="split,threads,cluster[,minblocks]" adds a pinned coarse phase to it.
lsdg_status autotune(lsdg_ctx* ctx, const std::string& key, const TrackArgs& a, TuneChoice* out, bool sim3,
                     double* mid) {
  auto it = ctx->tune_cache.find(key);
  if (it != ctx->tune_cache.end()) {
    *out = it->second;
    return LSDG_OK;
  }
  if (const char* env = std::getenv("LSDG_TRACK_SHAPE")) {
    int nt = 0, c = 0, mb = 1;
    if (std::sscanf(env, "%d,%d,%d", &nt, &c, &mb) >= 2) {
      int mc = track_max_clusters(nt, mb, c, sim3);
      if (mc > 0) {
        TuneChoice tc;
        tc.threads = nt;
        tc.minblocks = mb;
        tc.cluster = c;
        tc.max_clusters = mc;
        const char* sp = std::getenv("LSDG_TRACK_SPLIT");
        int s = -1, cnt = 0, cc = 0, cmb = 1;
        if (sp && mid && std::sscanf(sp, "%d,%d,%d,%d", &s, &cnt, &cc, &cmb) >= 3) {
          const int cmc = track_max_clusters(cnt, cmb, cc, sim3);
          if (cmc > 0 && s >= 1) {
            tc.split = s;
            tc.c_threads = cnt;
            tc.c_minblocks = cmb;
            tc.c_cluster = cc;
            tc.c_max_clusters = cmc;
          }
        }
        ctx->tune_cache[key] = tc;
        *out = tc;
        return LSDG_OK;
      }
    }
  }
  cudaEvent_t e0, e1;
  CK(ctx, cudaEventCreate(&e0));
  CK(ctx, cudaEventCreate(&e1));
  TuneChoice best;
  int nt = 0, mb = 0, c = 0, mc = 0;
  float best_ms = 0;
  lsdg_status st = best_phase(ctx, a, kCandCluster, 4, sim3, e0, e1, &nt, &mb, &c, &mc, &best_ms);
  if (st == LSDG_OK && nt == 0) st = ctx_fail(ctx, LSDG_NOT_SUPPORTED, "no cluster launch shape fits this device");
  if (st == LSDG_OK) {
    best.threads = nt;
    best.minblocks = mb;
    best.cluster = c;
    best.max_clusters = mc;
    best.split = -1;
  }
  static const int kCoarseCluster[] = {1, 2, 4};
  for (int split = 2; st == LSDG_OK && mid && split >= 1; --split) {
    if (!(a.top_level >= split && a.bottom_level < split)) continue;
    TrackArgs a1, a2;
    split_args(a, split, mid, &a1, &a2);
    int cnt = 0, cmb = 0, cc = 0, cmc = 0, fnt = 0, fmb = 0, fc = 0, fmc = 0;
    float cms = 0, fms = 0;
    st = best_phase(ctx, a1, kCoarseCluster, 3, sim3, e0, e1, &cnt, &cmb, &cc, &cmc, &cms);
    if (st != LSDG_OK || cnt == 0) break;
    st = launch_phase(ctx, a1, cnt, cmb, cc, cmc, sim3);  // the coarse poses the fine phase starts from
    if (st == LSDG_OK) st = best_phase(ctx, a2, kCandCluster, 4, sim3, e0, e1, &fnt, &fmb, &fc, &fmc, &fms);
    if (st != LSDG_OK || fnt == 0) break;
    if (cms + fms < best_ms) {
      best_ms = cms + fms;
      best.threads = fnt;
      best.minblocks = fmb;
      best.cluster = fc;
      best.max_clusters = fmc;
      best.split = split;
      best.c_threads = cnt;
      best.c_minblocks = cmb;
      best.c_cluster = cc;
      best.c_max_clusters = cmc;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != LSDG_OK) return st;
  best.tuned_ms = best_ms;
  ctx->tune_cache[key] = best;
  *out = best;
  return LSDG_OK;
}

extern "C" lsdg_status lsdg_tune_info(lsdg_ctx* ctx, int index, char* key, int key_len, int* threads, int* minblocks,
                                      int* cluster, int* max_clusters, float* ms) {
  if (!ctx) return LSDG_INVALID_ARG;
  int i = 0;
  for (auto& kv : ctx->tune_cache) {
    if (i++ != index) continue;
    if (key && key_len > 0) {
      std::strncpy(key, kv.first.c_str(), key_len - 1);
      key[key_len - 1] = 0;
    }
    if (threads) *threads = kv.second.threads;
    if (minblocks) *minblocks = kv.second.minblocks;
    if (cluster) *cluster = kv.second.cluster;
    if (max_clusters) *max_clusters = kv.second.max_clusters;
    if (ms) *ms = kv.second.tuned_ms;
    return LSDG_OK;
  }
  return LSDG_INVALID_ARG;
}

// ============================================================================================
// Single frames
// ============================================================================================
extern "C" {

lsdg_status lsdg_frame_create(lsdg_ctx* ctx, int width, int height, const lsdg_intrinsics* intr, lsdg_frame** out) {
  if (!ctx || !intr || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  *out = nullptr;
  CK(ctx, cudaSetDevice(ctx->device));
  lsdg_frame* f = new (std::nothrow) lsdg_frame();
  if (!f) return LSDG_OUT_OF_MEMORY;
  bool depth = true;
  lsdg_status st = frameset_alloc(ctx, f->fs, 1, &width, &height, intr, &depth, ctx->params.levels, true);
  if (st != LSDG_OK) {
    frameset_free(f->fs);
    delete f;
    return st;
  }
  f->fs.h_frames[0].has_depth = 0;  // until lsdg_frame_set_depth
  CK(ctx, cudaMemcpyAsync(f->fs.d_frames, f->fs.h_frames.data(), sizeof(FrameDev), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  *out = f;
  return LSDG_OK;
}

lsdg_status lsdg_frame_destroy(lsdg_ctx* ctx, lsdg_frame* f) {
  if (!ctx || !f) return LSDG_INVALID_ARG;
  cudaStreamSynchronize(ctx->stream);
  frameset_free(f->fs);
  delete f;
  return LSDG_OK;
}

lsdg_status lsdg_frame_upload(lsdg_ctx* ctx, lsdg_frame* f, const float* image) {
  if (!ctx || !f || !image) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const FrameDev& F = f->fs.h_frames[0];
  CK(ctx, cudaMemcpyAsync(F.plane[0], image, (size_t)F.w * F.h * 4, cudaMemcpyHostToDevice, ctx->stream));
  ctx->launches += launch_frame_pyramid(f->fs.d_frames, 1, F.levels, f->fs.max_pix, f->fs.max_h, true, ctx->stream);
  CK(ctx, cudaGetLastError());
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  f->has_image = true;
  return LSDG_OK;
}

lsdg_status lsdg_frame_upload_u8(lsdg_ctx* ctx, lsdg_frame* f, const uint8_t* image) {
  if (!ctx || !f || !image) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const FrameDev& F = f->fs.h_frames[0];
  size_t n = (size_t)F.w * F.h;
  // stage the bytes in the (not yet built) level-0 gradient plane, which is 16x larger
  uint8_t* tmp = (uint8_t*)F.pyr[0];
  CK(ctx, cudaMemcpyAsync(tmp, image, n, cudaMemcpyHostToDevice, ctx->stream));
  launch_u8_to_plane(tmp, F.plane[0], (int)n, ctx->stream);
  ctx->launches += 1 + launch_frame_pyramid(f->fs.d_frames, 1, F.levels, f->fs.max_pix, f->fs.max_h, true, ctx->stream);
  CK(ctx, cudaGetLastError());
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  f->has_image = true;
  return LSDG_OK;
}

lsdg_status lsdg_frame_set_depth(lsdg_ctx* ctx, lsdg_frame* f, const float* idepth, const float* var) {
  if (!ctx || !f || !idepth || !var) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!f->has_image) return ctx_fail(ctx, LSDG_INVALID_ARG, "upload the keyframe image before its depth");
  FrameDev& F = f->fs.h_frames[0];
  F.has_depth = 1;
  CK(ctx, cudaMemcpyAsync(f->fs.d_frames, &F, sizeof(FrameDev), cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(F.idepth[0], idepth, (size_t)F.w * F.h * 4, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(F.ivar[0], var, (size_t)F.w * F.h * 4, cudaMemcpyHostToDevice, ctx->stream));
  // band pass again (intensity levels are rebuilt identically) for the depth pyramid and counts
  ctx->launches += launch_frame_pyramid(f->fs.d_frames, 1, F.levels, f->fs.max_pix, f->fs.max_h, false, ctx->stream);
  ctx->launches += launch_frame_points(f->fs.d_frames, 1, F.levels, f->fs.max_h, ctx->stream);
  CK(ctx, cudaGetLastError());
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_frame_get_level(lsdg_ctx* ctx, const lsdg_frame* f, int level, float* out) {
  if (!ctx || !f || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const FrameDev& F = f->fs.h_frames[0];
  if (level < 0 || level >= F.levels) return ctx_fail(ctx, LSDG_INVALID_ARG, "level out of range");
  size_t n = (size_t)(F.w >> level) * (F.h >> level);
  CK(ctx, cudaMemcpyAsync(out, F.pyr[level], n * 16, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_frame_get_depth(lsdg_ctx* ctx, const lsdg_frame* f, int level, float* idepth, float* var) {
  if (!ctx || !f) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const FrameDev& F = f->fs.h_frames[0];
  if (!F.has_depth) return ctx_fail(ctx, LSDG_INVALID_ARG, "frame has no depth");
  if (level < 0 || level >= F.levels) return ctx_fail(ctx, LSDG_INVALID_ARG, "level out of range");
  size_t n = (size_t)(F.w >> level) * (F.h >> level);
  if (idepth) CK(ctx, cudaMemcpyAsync(idepth, F.idepth[level], n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (var) CK(ctx, cudaMemcpyAsync(var, F.ivar[level], n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_frame_get_points(lsdg_ctx* ctx, const lsdg_frame* f, int level, float* xyzi, float* var, int capacity,
                                  int* count) {
  if (!ctx || !f || !count) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const FrameDev& F = f->fs.h_frames[0];
  if (!F.has_depth) return ctx_fail(ctx, LSDG_INVALID_ARG, "frame has no depth");
  if (level < 0 || level >= F.levels) return ctx_fail(ctx, LSDG_INVALID_ARG, "level out of range");
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

}  // extern "C"

// ============================================================================================
// One-pair tracking and fixed-pose normal equations
// ============================================================================================

// Small-transfer layout inside ctx->d_small / h_small.
struct SmallLayout {
  PairDev pair;
  int work;
  int pad;
  double init[13];
  double out_pose[13];
  double out_sums[40];
  lsdg_track_stats stats;
};
static_assert(sizeof(SmallLayout) <= kSmallBytes, "small staging buffer too small");

static lsdg_status track_one(lsdg_ctx* ctx, const lsdg_frame* ref, const lsdg_frame* cur, const double* init,
                             bool init_is_ref_to_frame, int top, int bottom, bool eval_only, double* pose_out,
                             lsdg_track_stats* stats, double* sums, bool sim3) {
  if (!ref->fs.h_frames[0].has_depth) return ctx_fail(ctx, LSDG_INVALID_ARG, "reference frame has no depth");
  if (sim3 && !cur->fs.h_frames[0].has_depth) return ctx_fail(ctx, LSDG_INVALID_ARG, "Sim3: the other keyframe has no depth");
  if (!cur->has_image || !ref->has_image) return ctx_fail(ctx, LSDG_INVALID_ARG, "frame image not uploaded");
  const FrameDev& R = ref->fs.h_frames[0];
  const FrameDev& Cf = cur->fs.h_frames[0];
  if (R.w != Cf.w || R.h != Cf.h) return ctx_fail(ctx, LSDG_INVALID_ARG, "reference and frame sizes differ");
  SmallLayout* hs = (SmallLayout*)ctx->h_small;
  SmallLayout* ds = (SmallLayout*)ctx->d_small;
  hs->pair.ref = ref->fs.d_frames;
  hs->pair.cur = cur->fs.d_frames;
  std::memcpy(hs->init, init, sizeof(double) * (sim3 ? 13 : 12));
  CK(ctx, cudaMemcpyAsync(ds, hs, offsetof(SmallLayout, out_pose), cudaMemcpyHostToDevice, ctx->stream));
  TrackArgs a = make_track_args(ctx->params);
  a.pairs = &ds->pair;
  a.order = nullptr;
  a.n_pairs = 1;
  a.work_counter = &ds->work;
  a.init = ds->init;
  a.init_is_ref_to_frame = init_is_ref_to_frame ? 1 : 0;
  a.out_pose = ds->out_pose;
  a.out_stats = &ds->stats;
  a.out_sums = ds->out_sums;
  a.top_level = top;
  a.bottom_level = bottom;
  if (eval_only)
    for (int i = 0; i < kMaxLevels; ++i) a.max_iter[i] = 0;
  char key[64];
  std::snprintf(key, sizeof(key), "%s:%dx%d", sim3 ? "one-sim3" : "one", R.w, R.h);
  TuneChoice tc;
  if (eval_only) {
    tc = TuneChoice{256, 2, 8, 1, 0.f};  // a single pass: any shape, deterministic for the parity tests
  } else {
    lsdg_status st = autotune(ctx, key, a, &tc, sim3);
    if (st != LSDG_OK) return st;
  }
  lsdg_status st = run_tracker(ctx, a, tc, sim3);
  if (st != LSDG_OK) return st;
  CK(ctx, cudaMemcpyAsync(&hs->out_pose, &ds->out_pose, sizeof(SmallLayout) - offsetof(SmallLayout, out_pose),
                          cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (pose_out) std::memcpy(pose_out, hs->out_pose, sizeof(double) * (sim3 ? 13 : 12));
  if (stats) *stats = hs->stats;
  if (sums) std::memcpy(sums, hs->out_sums, sizeof(double) * (sim3 ? 40 : 32));
  return (lsdg_status)hs->stats.status;
}

extern "C" {

lsdg_status lsdg_se3_normal_equations(lsdg_ctx* ctx, const lsdg_frame* reference, const lsdg_frame* frame, int level,
                                      const double ref_to_frame[12], double out[LSDG_NE_SIZE]) {
  if (!ctx || !reference || !frame || !ref_to_frame || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (level < 0 || level >= ctx->params.levels) return ctx_fail(ctx, LSDG_INVALID_ARG, "level out of range");
  double sums[40];
  lsdg_status st = track_one(ctx, reference, frame, ref_to_frame, true, level, level, true, nullptr, nullptr, sums, false);
  if (st != LSDG_OK && st != LSDG_TRACKING_LOST) return st;
  std::memcpy(out, sums, sizeof(double) * LSDG_NE_SIZE);
  return LSDG_OK;
}

lsdg_status lsdg_sim3_normal_equations(lsdg_ctx* ctx, const lsdg_frame* reference, const lsdg_frame* frame, int level,
                                       const double ref_to_frame[13], double out[LSDG_NE_SIZE_SIM3]) {
  if (!ctx || !reference || !frame || !ref_to_frame || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (level < 0 || level >= ctx->params.levels) return ctx_fail(ctx, LSDG_INVALID_ARG, "level out of range");
  if (!(ref_to_frame[12] > 0)) return ctx_fail(ctx, LSDG_INVALID_ARG, "Sim3 scale must be > 0");
  double sums[40];
  lsdg_status st = track_one(ctx, reference, frame, ref_to_frame, true, level, level, true, nullptr, nullptr, sums, true);
  if (st != LSDG_OK && st != LSDG_TRACKING_LOST) return st;
  std::memcpy(out, sums, sizeof(double) * LSDG_NE_SIZE_SIM3);
  return LSDG_OK;
}

lsdg_status lsdg_track_sim3(lsdg_ctx* ctx, const lsdg_frame* reference, const lsdg_frame* frame,
                            const double frame_to_ref_init[13], double frame_to_ref_out[13], lsdg_track_stats* stats) {
  if (!ctx || !reference || !frame || !frame_to_ref_init || !frame_to_ref_out)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!(frame_to_ref_init[12] > 0)) return ctx_fail(ctx, LSDG_INVALID_ARG, "Sim3 scale must be > 0");
  return track_one(ctx, reference, frame, frame_to_ref_init, false, ctx->params.levels - 1, 0, false, frame_to_ref_out,
                   stats, nullptr, true);
}

lsdg_status lsdg_track_se3(lsdg_ctx* ctx, const lsdg_frame* reference, const lsdg_frame* frame,
                           const double frame_to_ref_init[12], double frame_to_ref_out[12], lsdg_track_stats* stats) {
  if (!ctx || !reference || !frame || !frame_to_ref_init || !frame_to_ref_out)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  return track_one(ctx, reference, frame, frame_to_ref_init, false, ctx->params.levels - 1, 0, false, frame_to_ref_out,
                   stats, nullptr, false);
}

}  // extern "C"

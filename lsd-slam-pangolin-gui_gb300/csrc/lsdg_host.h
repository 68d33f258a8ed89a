// lsdg_host.h -- host-side objects behind the opaque C-ABI handles.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "lsdg_internal.cuh"

constexpr size_t kSmallBytes = 4096;

struct TuneChoice {
  int threads = 256;
  int minblocks = 2;
  int cluster = 8;
  int max_clusters = 1;
  float tuned_ms = 0.f;
  // split run: levels [top, split] first, each pair on a small cluster (c_*), then the finer levels
  // with the shape above starting from the coarse poses; split = -1: one launch over all levels
  int split = -1;
  int c_threads = 256, c_minblocks = 2, c_cluster = 1, c_max_clusters = 1;
};

struct lsdg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  lsdg_params params{};
  int params_epoch = 0;
  std::string err;
  int64_t launches = 0;
  int sm_count = 0;
  void* d_small = nullptr;  // small device staging (pair descriptor, pose, stats)
  void* h_small = nullptr;  // pinned mirror
  std::map<std::string, TuneChoice> tune_cache;
};

struct FrameSet {
  int n = 0, levels = 0;
  std::vector<int> w, h;
  std::vector<lsdg_intrinsics> intr;
  std::vector<bool> depth;
  long max_pix = 0;
  int max_h = 0;
  size_t pix_total = 0, pix_depth = 0;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  size_t off_id0 = 0, off_var0 = 0;  // byte offsets of the level-0 idepth / variance sections
  float* plane0 = nullptr;           // level-0 intensity of all frames, back to back
  lsdg::FrameDev* d_frames = nullptr;
  std::vector<lsdg::FrameDev> h_frames;
};

struct lsdg_frame {
  FrameSet fs;
  bool has_image = false;
};

lsdg_status ctx_fail(lsdg_ctx* ctx, lsdg_status st, const char* fmt, ...);

// The depth map's current keyframe as the viewer reads it (depth.cu): smoothed inverse depth and
// variance, keyframe intensity (device planes, row-major w x h).  False when no keyframe is set.
bool depth_key_planes(const lsdg_depthmap* dm, const float** idepth, const float** var, const float** image,
                      int* w, int* h, lsdg_intrinsics* K);
lsdg_status ctx_cuda(lsdg_ctx* ctx, cudaError_t e, const char* what);
lsdg_status frameset_alloc(lsdg_ctx* ctx, FrameSet& fs, int n, const int* w, const int* h, const lsdg_intrinsics* intr,
                           const bool* depth, int levels, bool grads);
void frameset_free(FrameSet& fs);
lsdg::TrackArgs make_track_args(const lsdg_params& p);
// mid: device scratch of one pose per pair (12 or 13 doubles) for a split run; nullptr = one launch
lsdg_status run_tracker(lsdg_ctx* ctx, const lsdg::TrackArgs& a, const TuneChoice& tc, bool sim3,
                        double* mid = nullptr);
lsdg_status autotune(lsdg_ctx* ctx, const std::string& key, const lsdg::TrackArgs& a, TuneChoice* out, bool sim3,
                     double* mid = nullptr);

// lsdg_internal.cuh -- device-side data layout shared by the kernels and the C-ABI host code.
//
// HBM layout (one "frame" = one camera image with its pyramid; a keyframe also carries depth):
//   plane[l]   float  [h_l * w_l]   intensity of level l (level 0 is the upload target)
//   pyr[l]     float4 [h_l * w_l]   {I, gx, gy, 0} (frames that keep gradients: single frames and
//                                   depth-filter keyframes; batch frames only keep the planes)
//   idepth[l], ivar[l]  float [h_l * w_l]  keyframe depth pyramid (idepth <= 0: none)
//   pxyzi[l]   float4 [n_l]         tracking reference points, SoA: {X, Y, Z, I_keyframe}
//   pvar[l]    float  [n_l]         inverse-depth variance of each point
//   psig[l]    float  [n_l]         tracker scratch: residual variance of each point, fixed by the
//                                   first pass of a level (0 = the point sits out the level)
//   pcount[l]  int                  n_l, written on the device by the compaction
// All per-pixel planes are row-major and 256-byte aligned.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lsdg.h"  // include/ is on the include path (build_lib.py)

namespace lsdg {

constexpr int kMaxLevels = LSDG_MAX_LEVELS;

struct FrameDev {
  int w, h;  // level 0
  int has_depth;
  int levels;
  float* plane[kMaxLevels];
  float4* pyr[kMaxLevels];
  float* idepth[kMaxLevels];
  float* ivar[kMaxLevels];
  float4* pxyzi[kMaxLevels];
  float* pvar[kMaxLevels];
  float* psig[kMaxLevels];
  float* psigd[kMaxLevels];      // Sim3 tracker scratch: variance of the inverse-depth residual
  int* pcount;                   // [kMaxLevels]
  int* blk_count[kMaxLevels];    // compaction scratch: valid pixels per band, then offsets
  float fx[kMaxLevels], fy[kMaxLevels], cx[kMaxLevels], cy[kMaxLevels];
  float fxi[kMaxLevels], fyi[kMaxLevels];
};

struct PairDev {
  const FrameDev* ref;   // keyframe (carries depth and points)
  const FrameDev* cur;   // frame being tracked
};

// Tracker launch arguments (kernel parameter, passed by value).
struct TrackArgs {
  const PairDev* pairs;
  const int* order;          // processing order (largest first); nullptr = identity
  int n_pairs;
  int* work_counter;         // zeroed before the launch
  const double* init;        // 12 or 13 per pair: frame_to_ref, or ref_to_frame if init_is_ref_to_frame
  int init_is_ref_to_frame;
  double* out_pose;          // 12 (SE3) or 13 (Sim3: R, t, s) per pair: frame_to_ref
  lsdg_track_stats* out_stats;
  double* out_sums;          // optional: 32 (SE3) or 40 (Sim3) per pair, the last accepted pass
  int top_level;             // first (coarsest) level to run
  int bottom_level;          // last level to run
  int max_iter[kMaxLevels];
  float photometric_variance, huber_delta, min_z, border_margin, sim3_depth_variance, sim3_depth_weight;
  double lambda0, lambda_up, lambda_down, step_eps, stall_eps;
  float min_good_ratio, min_usage;
};

}  // namespace lsdg

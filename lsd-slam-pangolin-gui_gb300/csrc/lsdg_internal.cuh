// lsdg_internal.cuh -- device-side data layout shared by the kernels and the C-ABI host code.
//
// HBM layout (one "frame" = one camera image with its pyramid; a keyframe also carries depth):
//   plane[l]   float  [h_l * w_l]   intensity of level l (level 0 is the upload target)
//   pyr[l]     float4 [h_l * w_l]   {I, gx, gy, 0} (frames that keep gradients: single frames and
//                                   depth-filter keyframes; batch frames only keep the planes)
//   idepth[l], ivar[l]  float [h_l * w_l]  keyframe depth pyramid (idepth <= 0: none)
//   pxyzi[l]   float4 [n_l]         tracking reference points, SoA: {X, Y, Z, I_keyframe}
//   pvar[l]    float  [n_l]         inverse-depth variance of each point
//   psig[l]    float  [n_l]         tracker scratch: 1 / residual variance of each point, fixed by
//                                   the first pass of a level (0 = the point sits out the level)
//   psigd[l]   float  [n_l]         Sim3 tracker scratch: 1 / variance of the inverse-depth residual
//   ppix[l]    int    [n_l]         row-major pixel index of each point (single frames only; the
//                                   photometric energy maps its points back to pixels with it)
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
  float* psigd[kMaxLevels];      // Sim3 tracker scratch: 1 / variance of the inverse-depth residual
  int* ppix[kMaxLevels];         // pixel index of each point, or nullptr (batch frames)
  int* pcount;                   // [kMaxLevels]
  int* blk_count[kMaxLevels];    // compaction scratch: valid pixels per band, then offsets
  float fx[kMaxLevels], fy[kMaxLevels], cx[kMaxLevels], cy[kMaxLevels];
  float fxi[kMaxLevels], fyi[kMaxLevels];
  // floor((2^64 - 1) / (w >> l)) + 1: the row of a flat pixel index at level l is the high word of
  // index * rowdiv[l] (computed on the host; a 64-bit division per thread is costly on the GPU)
  unsigned long long rowdiv[kMaxLevels];
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
  float lambda0, lambda_up, lambda_down, step_eps, stall_eps;  // the LM schedule runs in float
  float min_good_ratio, min_usage;
  int accumulate_stats;      // continue the pass counts already in out_stats (second phase of a split run)
};

// Kahan-compensated float sum (value = s - c) and the merge of two of them (an exact TwoSum of the
// heads; the CPU oracle's KSum performs the same operations).
__device__ __forceinline__ void kadd(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}
__device__ __forceinline__ void kmerge(float& s, float& c, float os, float oc) {
  const float t = s + os;
  const float bp = t - s;
  const float err = (s - (t - bp)) + (os - bp);
  s = t;
  c = (c + oc) - err;
}

// Catmull-Rom cubic (C1, interpolating): weights of taps -1, 0, 1, 2 at fraction t and their
// derivatives; at t = 0 the derivative weights are the central difference (-1/2, 0, 1/2, 0).
// The tracker and the photometric energy sample the frame with it (the CPU oracle spells out the
// same operations).
__device__ __forceinline__ void catmull_rom(float t, float w[4], float d[4]) {
  const float t2 = t * t, t3 = t2 * t;
  w[0] = 0.5f * ((2.f * t2 - t3) - t);
  w[1] = 0.5f * ((3.f * t3 - 5.f * t2) + 2.f);
  w[2] = 0.5f * ((4.f * t2 - 3.f * t3) + t);
  w[3] = 0.5f * (t3 - t2);
  d[0] = 0.5f * ((4.f * t - 3.f * t2) - 1.f);
  d[1] = 0.5f * (9.f * t2 - 10.f * t);
  d[2] = 0.5f * ((8.f * t - 9.f * t2) + 1.f);
  d[3] = 0.5f * (3.f * t2 - 2.f * t);
}

}  // namespace lsdg

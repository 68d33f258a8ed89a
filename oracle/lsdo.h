// lsdo.h -- internal declarations of the CPU ORACLE (test infrastructure only; see lsdo_track.cpp).
#ifndef LSDO_H_
#define LSDO_H_

#include <atomic>
#include <vector>

#include "../include/lsdg.h"

namespace lsdo {

struct LevelCam {
  double fx, fy, cx, cy, fxi, fyi;
  int w, h;
};

template <class T>
struct FrameLevel {
  std::vector<T> I, gx, gy;
};

template <class T>
struct FrameData {
  int levels = 0;
  LevelCam cam[LSDG_MAX_LEVELS];
  std::vector<FrameLevel<T>> lv;
};

template <class T>
struct Points {
  std::vector<T> xyzi;  // 4 per point
  std::vector<T> var;
};

template <class T>
struct KeyframeData {
  LevelCam cam[LSDG_MAX_LEVELS];
  std::vector<std::vector<T>> D, V;  // depth pyramid
  std::vector<Points<T>> pts;
};

void default_params(lsdg_params* p);
void level_intrinsics(const lsdg_intrinsics& k0, int levels, LevelCam* out, int w0, int h0);
void se3_exp(const double xi[6], double T[12]);
void se3_mul(const double A[12], const double B[12], double C[12]);
void se3_inv(const double A[12], double B[12]);
bool ldlt_solve(int n, const double* hu, const double* g, double lambda, double* x);

template <class T>
void make_frame(const float* img, int w, int h, const lsdg_intrinsics& k, int levels, FrameData<T>& F);
template <class T>
void make_keyframe(const FrameData<T>& F, const float* idepth, const float* var, KeyframeData<T>& K);

}  // namespace lsdo

#endif

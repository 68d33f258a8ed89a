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
  std::vector<int> pix;  // row-major pixel index of each point in its level
};

template <class T>
struct KeyframeData {
  LevelCam cam[LSDG_MAX_LEVELS];
  std::vector<std::vector<T>> D, V;  // depth pyramid
  std::vector<Points<T>> pts;
};

// ------------------------------------------------------------------------------------------
// Kahan-compensated sum (value = s - c)
// ------------------------------------------------------------------------------------------
template <class T>
struct KSum {
  T s = 0, c = 0;
  inline void add(T x) {
    T y = x - c;
    T t = s + y;
    c = (t - s) - y;
    s = t;
  }
  inline void merge(const KSum& o) {  // (s,c) + (o.s,o.c) with an exact TwoSum of the heads
    T t = s + o.s;
    T bp = t - s;
    T err = (s - (t - bp)) + (o.s - bp);
    s = t;
    c = (c + o.c) - err;
  }
  inline double value() const { return (double)s - (double)c; }
};

// ------------------------------------------------------------------------------------------
// Catmull-Rom cubic (C1, interpolating): weights of taps -1, 0, 1, 2 at fraction t and their
// derivatives.  At t = 0 the derivative weights are (-1/2, 0, 1/2, 0): the central difference.
// ------------------------------------------------------------------------------------------
template <class T>
inline void catmull_rom(T t, T w[4], T d[4]) {
  const T t2 = t * t, t3 = t2 * t;
  const T h = (T)0.5;
  w[0] = h * (((T)2 * t2 - t3) - t);
  w[1] = h * (((T)3 * t3 - (T)5 * t2) + (T)2);
  w[2] = h * (((T)4 * t2 - (T)3 * t3) + t);
  w[3] = h * (t3 - t2);
  d[0] = h * (((T)4 * t - (T)3 * t2) - (T)1);
  d[1] = h * ((T)9 * t2 - (T)10 * t);
  d[2] = h * (((T)8 * t - (T)9 * t2) + (T)1);
  d[3] = h * ((T)3 * t2 - (T)2 * t);
}

void default_params(lsdg_params* p);

void level_intrinsics(const lsdg_intrinsics& k0, int levels, LevelCam* out, int w0, int h0);
void se3_exp(const double xi[6], double T[12]);
void se3_mul(const double A[12], const double B[12], double C[12]);
void se3_inv(const double A[12], double B[12]);
bool ldlt_solve(int n, const double* hu, const double* g, double lambda, double* x);
void se3_coeffs(double th2, double* A, double* B, double* C);

template <class T>
void make_frame(const float* img, int w, int h, const lsdg_intrinsics& k, int levels, FrameData<T>& F);
template <class T>
void make_keyframe(const FrameData<T>& F, const float* idepth, const float* var, KeyframeData<T>& K);

}  // namespace lsdo

#endif

// formats.cu -- host-side pose wire formats of the viewer and the text output (no device code):
// Sophus' 7-parameter Sim3 layout used by GraphFramePose (lib/Pangolin_IOWrapper/Keyframe.h:23-27,
// PangolinOutputIOWrapper.cpp:161) and the pose-file rows of TextOutputIOWrapper
// (lib/Pangolin_IOWrapper/TextOutputIOWrapper.cpp:104-117).
#include <cmath>
#include <cstdio>

#include "lsdg.h"

namespace {

// Unit quaternion (x, y, z, w) of a rotation matrix (row-major), largest-diagonal branch for
// accuracy, w >= 0.
void rot_to_quat(const double* R, double q[4]) {
  const double tr = R[0] + R[4] + R[8];
  if (tr > 0) {
    const double s = 2.0 * std::sqrt(tr + 1.0);
    q[3] = 0.25 * s;
    q[0] = (R[7] - R[5]) / s;
    q[1] = (R[2] - R[6]) / s;
    q[2] = (R[3] - R[1]) / s;
  } else if (R[0] > R[4] && R[0] > R[8]) {
    const double s = 2.0 * std::sqrt(1.0 + R[0] - R[4] - R[8]);
    q[3] = (R[7] - R[5]) / s;
    q[0] = 0.25 * s;
    q[1] = (R[1] + R[3]) / s;
    q[2] = (R[2] + R[6]) / s;
  } else if (R[4] > R[8]) {
    const double s = 2.0 * std::sqrt(1.0 + R[4] - R[0] - R[8]);
    q[3] = (R[2] - R[6]) / s;
    q[0] = (R[1] + R[3]) / s;
    q[1] = 0.25 * s;
    q[2] = (R[5] + R[7]) / s;
  } else {
    const double s = 2.0 * std::sqrt(1.0 + R[8] - R[0] - R[4]);
    q[3] = (R[3] - R[1]) / s;
    q[0] = (R[2] + R[6]) / s;
    q[1] = (R[5] + R[7]) / s;
    q[2] = 0.25 * s;
  }
  if (q[3] < 0)
    for (int i = 0; i < 4; ++i) q[i] = -q[i];
  const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int i = 0; i < 4; ++i) q[i] /= n;
}

}  // namespace

extern "C" {

void lsdg_sim3_to_sophus7(const double p[13], float out[7]) {
  double q[4];
  rot_to_quat(p, q);
  const double r = std::sqrt(p[12]);  // |q|^2 = scale
  for (int i = 0; i < 4; ++i) out[i] = (float)(q[i] * r);
  for (int i = 0; i < 3; ++i) out[4 + i] = (float)p[9 + i];
}

void lsdg_sophus7_to_sim3(const float in[7], double p[13]) {
  const double x = in[0], y = in[1], z = in[2], w = in[3];
  const double s = x * x + y * y + z * z + w * w;
  const double n = std::sqrt(s);
  const double a = x / n, b = y / n, c = z / n, d = w / n;
  p[0] = 1 - 2 * (b * b + c * c);
  p[1] = 2 * (a * b - c * d);
  p[2] = 2 * (a * c + b * d);
  p[3] = 2 * (a * b + c * d);
  p[4] = 1 - 2 * (a * a + c * c);
  p[5] = 2 * (b * c - a * d);
  p[6] = 2 * (a * c - b * d);
  p[7] = 2 * (b * c + a * d);
  p[8] = 1 - 2 * (a * a + b * b);
  for (int i = 0; i < 3; ++i) p[9 + i] = in[4 + i];
  p[12] = s;
}

int lsdg_format_pose_row(int id, const double c[13], const double t[13], char* buf, int len) {
  if (!c || !t || !buf || len <= 0) return -1;
  const int n = std::snprintf(buf, (size_t)len, "%d,%g,%g,%g,%g,%g,%g\n", id, c[9], c[10], c[11], t[9], t[10], t[11]);
  return (n < 0 || n >= len) ? -1 : n;
}

}  // extern "C"

// lsdo_input.cpp -- CPU ORACLE (test infrastructure only) of the input step: the undistortion remap
// table of a calibration and the 8-bit bilinear remap of a raw frame.  The reference's undistorter is
// libvideoio's (absent, unpinned: fips.yml:8-9; used at tools/LSD.cpp:88 and
// lib/App/InputThread.cpp:62); the "frame" model of its sample calibration (d2_camera.xml) is the
// published radial-tangential model with focal length f, principal-point offset (cx, cy) from the
// image centre, affinity/skew (b1, b2), radial k1..k4 and tangential p1, p2 (see include/lsdg.h).
// Same operations and order as the kernels (double for the table, float for the remap).
#include <cstdint>

#include "lsdo.h"

extern "C" {

// map: out_w * out_h pairs (u, v) in pixel-centre coordinates of the raw image.
void lsdo_undistort_map(const lsdg_calibration* c0, int out_w, int out_h, const lsdg_intrinsics* K, float* map) {
  lsdg_calibration c = *c0;
  if (c.model == LSDG_CALIB_PINHOLE) c.b1 = c.b2 = c.k1 = c.k2 = c.k3 = c.k4 = c.p1 = c.p2 = 0.0;
  const double fx = K->fx, fy = K->fy, cx = K->cx, cy = K->cy;
  for (int py = 0; py < out_h; ++py)
    for (int px = 0; px < out_w; ++px) {
      const double x = ((double)px - cx) / fx;
      const double y = ((double)py - cy) / fy;
      const double r2 = x * x + y * y;
      const double rad = 1.0 + r2 * (c.k1 + r2 * (c.k2 + r2 * (c.k3 + r2 * c.k4)));
      const double xd = x * rad + (c.p1 * (r2 + 2.0 * x * x) + 2.0 * c.p2 * x * y);
      const double yd = y * rad + (c.p2 * (r2 + 2.0 * y * y) + 2.0 * c.p1 * x * y);
      const double u = ((0.5 * c.width + c.cx) + xd * c.f) + (xd * c.b1 + yd * c.b2);
      const double v = (0.5 * c.height + c.cy) + yd * c.f;
      map[2 * ((size_t)py * out_w + px) + 0] = (float)(u - 0.5);
      map[2 * ((size_t)py * out_w + px) + 1] = (float)(v - 0.5);
    }
}

// Bilinear remap of a raw 8-bit image through `map` (n output pixels), rounded to 8 bits; 0 outside.
void lsdo_undistort(const uint8_t* raw, int in_w, int in_h, const float* map, int n, uint8_t* out) {
  for (int i = 0; i < n; ++i) {
    const float u = map[2 * i], v = map[2 * i + 1];
    float val = 0.f;
    if (u >= 0.f && v >= 0.f && u <= (float)(in_w - 1) && v <= (float)(in_h - 1)) {
      const int x0 = (int)u, y0 = (int)v;
      const int x1 = x0 + 1 < in_w ? x0 + 1 : x0, y1 = y0 + 1 < in_h ? y0 + 1 : y0;
      const float ax = u - (float)x0, ay = v - (float)y0;
      const float bx = 1.f - ax, by = 1.f - ay;
      const float i00 = raw[(size_t)y0 * in_w + x0], i10 = raw[(size_t)y0 * in_w + x1];
      const float i01 = raw[(size_t)y1 * in_w + x0], i11 = raw[(size_t)y1 * in_w + x1];
      val = (((bx * by) * i00 + (ax * by) * i10) + (bx * ay) * i01) + (ax * ay) * i11;
    }
    int q = (int)(val + 0.5f);
    q = q < 0 ? 0 : (q > 255 ? 255 : q);
    out[i] = (uint8_t)q;
  }
}

}  // extern "C"

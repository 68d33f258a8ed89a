// lsdo_cloud.cpp -- CPU ORACLE (test infrastructure only) of the keyframe point cloud the viewer
// builds: Keyframe::computeVbo's variance / neighbour-support filter and back-projection
// (lib/Pangolin_IOWrapper/Keyframe.h:66-143; constants at :78-82, support test :113-132,
// back-projection :134-141), restated without OpenGL.  It follows the loop's steps operation for
// operation (float arithmetic, the order of the products, the colour swizzle), is compiled without FP
// contraction like the kernels, and is checked byte for byte against the reference's own loop
// (oracle/ref_build.py compiles it from Keyframe.h into oracle/_ref; tests/golden/cloud_ref.npz holds
// its outputs).
#include <cstdint>

#include "lsdo.h"

extern "C" {

// points: w * h InputPointDense records; out: capacity w * h vertices.  Returns the vertex count.
int lsdo_cloud_build(int w, int h, float fx, float fy, float cx, float cy, float scale, const lsdg_cloud_params* p,
                     const lsdg_input_point_dense* points, lsdg_cloud_vertex* out) {
  const float scaled_th = p->scaled_th, abs_th = p->abs_th;
  const int min_support = p->min_near_support;
  const float fxi = 1.0f / fx, fyi = 1.0f / fy;
  const float cxi = -cx / fx, cyi = -cy / fy;
  int n = 0;
  for (int y = 1; y < h - 1; ++y) {
    for (int x = 1; x < w - 1; ++x) {
      const lsdg_input_point_dense& c = points[x + y * w];
      if (c.idepth <= 0.f) continue;
      const float depth = 1.0f / c.idepth;
      float depth4 = depth * depth;
      depth4 = depth4 * depth4;
      if (c.idepth_var * depth4 > scaled_th) continue;
      if (((c.idepth_var * depth4) * scale) * scale > abs_th) continue;
      if (min_support > 1) {
        int support = 0;
        for (int dx = -1; dx < 2; ++dx)
          for (int dy = -1; dy < 2; ++dy) {
            const float nb = points[x + dx + (y + dy) * w].idepth;
            if (nb > 0.f) {
              const float diff = nb - 1.0f / depth;
              if (diff * diff < 2.0f * c.idepth_var) ++support;
            }
          }
        if (support < min_support) continue;
      }
      lsdg_cloud_vertex& v = out[n++];
      v.point[0] = ((float)x * fxi + cxi) * depth;
      v.point[1] = ((float)y * fyi + cyi) * depth;
      v.point[2] = depth;
      v.color[3] = 100;
      v.color[2] = c.color[0];
      v.color[1] = c.color[1];
      v.color[0] = c.color[2];
    }
  }
  return n;
}

}  // extern "C"

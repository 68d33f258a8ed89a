// input.cu -- the input step ahead of the path (InputThread, lib/App/InputThread.cpp:59-71): a raw
// 8-bit frame is undistorted into the SLAM camera and handed to the tracker as a frame pyramid.
// The reference does this with libvideoio's Undistorter (absent, no pinned version: fips.yml:8-9),
// configured from a calibration file (tools/LSD.cpp:88; sample d2_camera.xml, "frame" model).
//
// GB300 design: the remap table (source position of every output pixel) is computed once per
// calibration on the device, in FP64 (the distortion polynomial is evaluated per pixel), and stored
// as float pairs (8 B/px).  Each frame is then one gather kernel over the output pixels: 4 taps of
// the raw image (L1/L2), bilinear, rounded to 8 bits (the undistorted CV_8UC1 image), written both
// as the 8-bit live image and as the frame's level-0 intensity plane; the band kernels build the
// pyramid from there.  Built with -fmad=false: the table and the image are bit-identical to the CPU
// oracle (oracle/lsdo_input.cpp).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "lsdg_host.h"

using namespace lsdg;

namespace lsdg {
int launch_frame_pyramid(const FrameDev* frames, int n, int levels, long max_pix, int max_h, bool with_grads,
                         cudaStream_t s);
}

#define CK(ctx, expr)                                \
  do {                                               \
    lsdg_status _s = ctx_cuda((ctx), (expr), #expr); \
    if (_s != LSDG_OK) return _s;                    \
  } while (0)

struct lsdg_undistorter {
  lsdg_calibration cal{};
  int out_w = 0, out_h = 0;
  lsdg_intrinsics K{};
  float2* map = nullptr;   // out_w * out_h source positions (pixel-centre coordinates of the raw image)
  uint8_t* raw = nullptr;  // raw frame staging
  uint8_t* und = nullptr;  // last undistorted 8-bit image
};

namespace {

struct MapArgs {
  lsdg_calibration c;
  int out_w, out_h;
  double fx, fy, cx, cy;  // output camera (pixel-centre coordinates)
  float2* map;
};

// Source position of output pixel (px, py) under the calibration's model.
__global__ void undistort_map_kernel(const MapArgs a) {
  const int px = blockIdx.x * blockDim.x + threadIdx.x;
  const int py = blockIdx.y;
  if (px >= a.out_w) return;
  const lsdg_calibration& c = a.c;
  const double x = ((double)px - a.cx) / a.fx;
  const double y = ((double)py - a.cy) / a.fy;
  const double r2 = x * x + y * y;
  const double rad = 1.0 + r2 * (c.k1 + r2 * (c.k2 + r2 * (c.k3 + r2 * c.k4)));
  const double xd = x * rad + (c.p1 * (r2 + 2.0 * x * x) + 2.0 * c.p2 * x * y);
  const double yd = y * rad + (c.p2 * (r2 + 2.0 * y * y) + 2.0 * c.p1 * x * y);
  const double u = ((0.5 * c.width + c.cx) + xd * c.f) + (xd * c.b1 + yd * c.b2);
  const double v = (0.5 * c.height + c.cy) + yd * c.f;
  a.map[(size_t)py * a.out_w + px] = make_float2((float)(u - 0.5), (float)(v - 0.5));
}

// One output pixel: bilinear gather of the raw 8-bit image at its source position, rounded to 8
// bits; 0 outside the raw image.
__global__ void undistort_kernel(const uint8_t* __restrict__ raw, int in_w, int in_h, const float2* __restrict__ map,
                                 int n, uint8_t* __restrict__ und, float* __restrict__ plane) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 m = map[i];
  const float u = m.x, v = m.y;
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
  und[i] = (uint8_t)q;
  plane[i] = (float)q;
}

bool find_tag(const std::string& s, const char* tag, std::string* out) {
  const std::string open = std::string("<") + tag + ">", close = std::string("</") + tag + ">";
  const size_t a = s.find(open);
  if (a == std::string::npos) return false;
  const size_t b = s.find(close, a + open.size());
  if (b == std::string::npos) return false;
  *out = s.substr(a + open.size(), b - a - open.size());
  return true;
}

bool tag_number(const std::string& s, const char* tag, double* v) {
  std::string t;
  if (!find_tag(s, tag, &t)) return false;
  char* end = nullptr;
  const double x = std::strtod(t.c_str(), &end);
  if (end == t.c_str()) return false;
  *v = x;
  return true;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\n' || s[a] == '\r' || s[a] == '\t')) ++a;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\n' || s[b - 1] == '\r' || s[b - 1] == '\t')) --b;
  return s.substr(a, b - a);
}

}  // namespace

extern "C" {

lsdg_status lsdg_calibration_load_xml(const char* path, lsdg_calibration* out) {
  if (!path || !out) return LSDG_INVALID_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return LSDG_INVALID_ARG;
  std::string s;
  char buf[4096];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, k);
  std::fclose(f);
  if (s.find("<calibration>") == std::string::npos) return LSDG_INVALID_ARG;
  lsdg_calibration c;
  std::memset(&c, 0, sizeof(c));
  std::string proj;
  if (find_tag(s, "projection", &proj)) {
    proj = trim(proj);
    if (proj == "frame") c.model = LSDG_CALIB_FRAME;
    else if (proj == "pinhole") c.model = LSDG_CALIB_PINHOLE;
    else return LSDG_NOT_SUPPORTED;
  } else {
    c.model = LSDG_CALIB_PINHOLE;
  }
  double w = 0, h = 0;
  if (!tag_number(s, "width", &w) || !tag_number(s, "height", &h) || !tag_number(s, "f", &c.f)) return LSDG_INVALID_ARG;
  c.width = (int32_t)w;
  c.height = (int32_t)h;
  tag_number(s, "cx", &c.cx);
  tag_number(s, "cy", &c.cy);
  if (c.model == LSDG_CALIB_FRAME) {
    tag_number(s, "b1", &c.b1);
    tag_number(s, "b2", &c.b2);
    tag_number(s, "k1", &c.k1);
    tag_number(s, "k2", &c.k2);
    tag_number(s, "k3", &c.k3);
    tag_number(s, "k4", &c.k4);
    tag_number(s, "p1", &c.p1);
    tag_number(s, "p2", &c.p2);
  }
  if (c.width <= 0 || c.height <= 0 || !(c.f > 0)) return LSDG_INVALID_ARG;
  *out = c;
  return LSDG_OK;
}

lsdg_status lsdg_undistorter_create(lsdg_ctx* ctx, const lsdg_calibration* calib, int out_w, int out_h,
                                    const lsdg_intrinsics* out_K, lsdg_undistorter** out) {
  if (!ctx || !calib || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  *out = nullptr;
  if (calib->model != LSDG_CALIB_PINHOLE && calib->model != LSDG_CALIB_FRAME)
    return ctx_fail(ctx, LSDG_NOT_SUPPORTED, "calibration model %d", calib->model);
  if (calib->width <= 0 || calib->height <= 0 || !(calib->f > 0) || (long)calib->width * calib->height > (1l << 28))
    return ctx_fail(ctx, LSDG_INVALID_ARG, "bad calibration size or focal length");
  if (out_w <= 0 || out_h <= 0 || (long)out_w * out_h > (1l << 28))
    return ctx_fail(ctx, LSDG_INVALID_ARG, "bad output size %dx%d", out_w, out_h);
  if (out_K && (!(out_K->fx > 0) || !(out_K->fy > 0))) return ctx_fail(ctx, LSDG_INVALID_ARG, "bad output intrinsics");
  CK(ctx, cudaSetDevice(ctx->device));
  lsdg_undistorter* u = new (std::nothrow) lsdg_undistorter();
  if (!u) return LSDG_OUT_OF_MEMORY;
  u->cal = *calib;
  if (calib->model == LSDG_CALIB_PINHOLE) {
    u->cal.b1 = u->cal.b2 = u->cal.k1 = u->cal.k2 = u->cal.k3 = u->cal.k4 = u->cal.p1 = u->cal.p2 = 0.0;
  }
  u->out_w = out_w;
  u->out_h = out_h;
  if (out_K) {
    u->K = *out_K;
  } else {
    u->K.fx = u->K.fy = (float)calib->f;
    u->K.cx = (float)(0.5 * calib->width + calib->cx - 0.5);
    u->K.cy = (float)(0.5 * calib->height + calib->cy - 0.5);
  }
  const size_t n_out = (size_t)out_w * out_h, n_in = (size_t)calib->width * calib->height;
  cudaError_t e = cudaMalloc(&u->map, n_out * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&u->raw, n_in);
  if (e == cudaSuccess) e = cudaMalloc(&u->und, n_out);
  if (e == cudaSuccess) {
    MapArgs a;
    a.c = u->cal;
    a.out_w = out_w;
    a.out_h = out_h;
    a.fx = u->K.fx;
    a.fy = u->K.fy;
    a.cx = u->K.cx;
    a.cy = u->K.cy;
    a.map = u->map;
    undistort_map_kernel<<<dim3((out_w + 127) / 128, out_h), 128, 0, ctx->stream>>>(a);
    ctx->launches += 1;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(u->und, 0, n_out, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(u->map);
    cudaFree(u->raw);
    cudaFree(u->und);
    delete u;
    return ctx_cuda(ctx, e, "lsdg_undistorter_create");
  }
  *out = u;
  return LSDG_OK;
}

lsdg_status lsdg_undistorter_destroy(lsdg_ctx* ctx, lsdg_undistorter* u) {
  if (!ctx || !u) return LSDG_INVALID_ARG;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(u->map);
  cudaFree(u->raw);
  cudaFree(u->und);
  delete u;
  return LSDG_OK;
}

lsdg_status lsdg_undistorter_camera(lsdg_ctx* ctx, const lsdg_undistorter* u, int* out_w, int* out_h,
                                    lsdg_intrinsics* out_K) {
  if (!ctx || !u) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (out_w) *out_w = u->out_w;
  if (out_h) *out_h = u->out_h;
  if (out_K) *out_K = u->K;
  return LSDG_OK;
}

lsdg_status lsdg_frame_upload_distorted_u8(lsdg_ctx* ctx, lsdg_undistorter* u, lsdg_frame* f, const uint8_t* raw) {
  if (!ctx || !u || !f || !raw) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const FrameDev& F = f->fs.h_frames[0];
  if (F.w != u->out_w || F.h != u->out_h)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "frame is %dx%d, the undistorter's output %dx%d", F.w, F.h, u->out_w,
                    u->out_h);
  const size_t n_in = (size_t)u->cal.width * u->cal.height;
  const int n_out = u->out_w * u->out_h;
  CK(ctx, cudaMemcpyAsync(u->raw, raw, n_in, cudaMemcpyHostToDevice, ctx->stream));
  undistort_kernel<<<(n_out + 255) / 256, 256, 0, ctx->stream>>>(u->raw, u->cal.width, u->cal.height, u->map, n_out,
                                                                 u->und, F.plane[0]);
  ctx->launches += 1 + launch_frame_pyramid(f->fs.d_frames, 1, F.levels, f->fs.max_pix, f->fs.max_h, true, ctx->stream);
  CK(ctx, cudaGetLastError());
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  f->has_image = true;
  return LSDG_OK;
}

lsdg_status lsdg_undistorter_last_image(lsdg_ctx* ctx, const lsdg_undistorter* u, uint8_t* out) {
  if (!ctx || !u || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  CK(ctx, cudaMemcpyAsync(out, u->und, (size_t)u->out_w * u->out_h, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

}  // extern "C"

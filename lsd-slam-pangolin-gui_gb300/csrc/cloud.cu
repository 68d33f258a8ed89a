// cloud.cu -- the keyframe point cloud of the viewer's data path, headless: publishKeyframe's
// per-pixel export (lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:79-89) and
// Keyframe::computeVbo's filter + back-projection (lib/Pangolin_IOWrapper/Keyframe.h:66-143), with
// the GL vertex buffer replaced by a device (or host) array of the same 16-byte vertices.
//
// computeVbo walks the interior pixels row by row and appends every kept point, so the vertex order
// is row-major.  The GPU keeps that order with two launches of one CTA per row: the first counts the
// row's kept points, the second sums the counts of the rows above (its output offset), then writes
// the row's points in x order with a ballot prefix per warp and a warp-offset scan per chunk.  The
// 3x3 support test reads the neighbours' inverse depth from L1.  Built with -fmad=false: every
// float operation rounds as in the CPU oracle (and as in the reference's loop compiled without
// contraction), so the vertices are bit-identical.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "lsdg_host.h"

using namespace lsdg;

#define CK(ctx, expr)                                \
  do {                                               \
    lsdg_status _s = ctx_cuda((ctx), (expr), #expr); \
    if (_s != LSDG_OK) return _s;                    \
  } while (0)

namespace {

constexpr int kCloudThreads = 256;

struct CloudArgs {
  int w, h;
  float fxi, fyi, cxi, cyi;  // 1/fx, 1/fy, -cx/fx, -cy/fy (Keyframe.h:86-89)
  float scale;               // camToWorld.scale()
  float scaled_th, abs_th;
  int min_support;
  const lsdg_input_point_dense* dense;     // source: InputPointDense records, or
  const float* idepth;                     // the depth map's smoothed planes + keyframe intensity
  const float* var;
  const float* image;
  int* rowcnt;                             // h
  int* total;
  lsdg_cloud_vertex* out;
};

// publishKeyframe stores the float intensity into each colour byte (a float -> unsigned char
// conversion: truncation for values in [0, 256)); out-of-range values are undefined there and
// saturate here.
__device__ __forceinline__ unsigned char to_u8(float f) {
  return f >= 255.f ? (unsigned char)255 : (f > 0.f ? (unsigned char)(int)f : (unsigned char)0);
}

template <bool DENSE>
__device__ __forceinline__ float idepth_at(const CloudArgs& a, int i) {
  return DENSE ? a.dense[i].idepth : a.idepth[i];
}

// The filter of Keyframe::computeVbo for interior pixel (x, y); returns depth = 1 / idepth.
template <bool DENSE>
__device__ __forceinline__ bool keep(const CloudArgs& a, int x, int y, float& depth) {
  if (x < 1 || x >= a.w - 1 || y < 1 || y >= a.h - 1) return false;
  const int i = x + y * a.w;
  const float id = idepth_at<DENSE>(a, i);
  if (id <= 0.f) return false;
  const float var = DENSE ? a.dense[i].idepth_var : a.var[i];
  depth = 1.0f / id;
  float depth4 = depth * depth;
  depth4 = depth4 * depth4;
  if (var * depth4 > a.scaled_th) return false;
  if (((var * depth4) * a.scale) * a.scale > a.abs_th) return false;
  if (a.min_support > 1) {
    int support = 0;
    const float back = 1.0f / depth;
    const float lim = 2.f * var;
#pragma unroll
    for (int dx = -1; dx < 2; ++dx)
#pragma unroll
      for (int dy = -1; dy < 2; ++dy) {
        const float n = idepth_at<DENSE>(a, x + dx + (y + dy) * a.w);
        if (n > 0.f) {
          const float diff = n - back;
          if (diff * diff < lim) ++support;
        }
      }
    if (support < a.min_support) return false;
  }
  return true;
}

template <bool DENSE>
__global__ void __launch_bounds__(kCloudThreads) cloud_count_kernel(const CloudArgs a) {
  __shared__ int wsum[kCloudThreads / 32];
  const int y = blockIdx.x;
  int c = 0;
  for (int x = threadIdx.x; x < a.w; x += blockDim.x) {
    float depth;
    c += keep<DENSE>(a, x, y, depth) ? 1 : 0;
  }
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < kCloudThreads / 32; ++k) s += wsum[k];
    a.rowcnt[y] = s;
  }
}

template <bool DENSE>
__global__ void __launch_bounds__(kCloudThreads) cloud_write_kernel(const CloudArgs a) {
  __shared__ int wsum[kCloudThreads / 32];
  __shared__ int base;
  const int y = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // output offset of this row: the kept points of all rows above
  int part = 0;
  for (int r = threadIdx.x; r < y; r += blockDim.x) part += a.rowcnt[r];
  part = __reduce_add_sync(0xffffffffu, part);
  if (lane == 0) wsum[wid] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < kCloudThreads / 32; ++k) s += wsum[k];
    base = s;
    if (y == a.h - 1) *a.total = s + a.rowcnt[y];
  }
  __syncthreads();
  for (int x0 = 0; x0 < a.w; x0 += blockDim.x) {
    const int x = x0 + threadIdx.x;
    float depth = 0.f;
    const bool k = x < a.w && keep<DENSE>(a, x, y, depth);
    const unsigned m = __ballot_sync(0xffffffffu, k);
    __syncthreads();  // the previous chunk's readers of wsum / base are done
    if (lane == 0) wsum[wid] = __popc(m);
    __syncthreads();
    int off = base;
    for (int q = 0; q < wid; ++q) off += wsum[q];
    if (k) {
      const int i = x + y * a.w;
      unsigned char c0, c1, c2;
      if (DENSE) {
        c0 = a.dense[i].color[0];
        c1 = a.dense[i].color[1];
        c2 = a.dense[i].color[2];
      } else {
        c0 = c1 = c2 = to_u8(a.image[i]);
      }
      const float px = ((float)x * a.fxi + a.cxi) * depth;
      const float py = ((float)y * a.fyi + a.cyi) * depth;
      // MyVertex colour: [0] = input B (colour[2]), [1] = G, [2] = input colour[0], [3] = 100
      const unsigned rgba = (unsigned)c2 | ((unsigned)c1 << 8) | ((unsigned)c0 << 16) | (100u << 24);
      float4 v = make_float4(px, py, depth, __uint_as_float(rgba));
      reinterpret_cast<float4*>(a.out)[off + __popc(m & ((1u << lane) - 1u))] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int s = 0;
      for (int q = 0; q < kCloudThreads / 32; ++q) s += wsum[q];
      base += s;
    }
  }
}

__global__ void export_points_kernel(const float* __restrict__ idepth, const float* __restrict__ var,
                                     const float* __restrict__ image, int n, lsdg_input_point_dense* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned char c = to_u8(image[i]);
  lsdg_input_point_dense p;
  p.idepth = idepth[i];
  p.idepth_var = var[i];
  p.color[0] = p.color[1] = p.color[2] = p.color[3] = c;
  out[i] = p;
}

CloudArgs make_args(int w, int h, float fx, float fy, float cx, float cy, float scale, const lsdg_cloud_params& p) {
  CloudArgs a{};
  a.w = w;
  a.h = h;
  a.fxi = 1.0f / fx;
  a.fyi = 1.0f / fy;
  a.cxi = -cx / fx;
  a.cyi = -cy / fy;
  a.scale = scale;
  a.scaled_th = p.scaled_th;
  a.abs_th = p.abs_th;
  a.min_support = p.min_near_support;
  return a;
}

template <bool DENSE>
lsdg_status launch_cloud(lsdg_ctx* ctx, CloudArgs& a, int* count) {
  CK(ctx, cudaMallocAsync(&a.rowcnt, sizeof(int) * ((size_t)a.h + 1), ctx->stream));
  a.total = a.rowcnt + a.h;
  cloud_count_kernel<DENSE><<<a.h, kCloudThreads, 0, ctx->stream>>>(a);
  cloud_write_kernel<DENSE><<<a.h, kCloudThreads, 0, ctx->stream>>>(a);
  ctx->launches += 2;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_small, a.total, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaFreeAsync(a.rowcnt, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return ctx_cuda(ctx, e, "cloud kernels");
  std::memcpy(count, ctx->h_small, sizeof(int));
  return LSDG_OK;
}

lsdg_status check_cloud_args(lsdg_ctx* ctx, int w, int h, float fx, float fy, const lsdg_cloud_params& p) {
  if (w < 3 || h < 3 || (long)w * h > (1l << 28)) return ctx_fail(ctx, LSDG_INVALID_ARG, "bad cloud size %dx%d", w, h);
  if (!(fx != 0.f) || !(fy != 0.f)) return ctx_fail(ctx, LSDG_INVALID_ARG, "focal lengths must be non-zero");
  if (p.min_near_support > 9) return ctx_fail(ctx, LSDG_INVALID_ARG, "min_near_support must be <= 9");
  return LSDG_OK;
}

}  // namespace

extern "C" {

void lsdg_cloud_default_params(lsdg_cloud_params* p) {
  if (!p) return;
  p->scaled_th = 1e-3f;
  p->abs_th = 1e-1f;
  p->min_near_support = 9;
  p->reserved = 0;
}

lsdg_status lsdg_depth_export_points(lsdg_ctx* ctx, lsdg_depthmap* dm, lsdg_input_point_dense* out) {
  if (!ctx || !dm || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const float *id, *var, *img;
  int w, h;
  lsdg_intrinsics K;
  if (!depth_key_planes(dm, &id, &var, &img, &w, &h, &K)) return ctx_fail(ctx, LSDG_INVALID_ARG, "no keyframe set");
  const int n = w * h;
  lsdg_input_point_dense* d = nullptr;
  CK(ctx, cudaMallocAsync(&d, sizeof(lsdg_input_point_dense) * (size_t)n, ctx->stream));
  export_points_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(id, var, img, n, d);
  ctx->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d, sizeof(lsdg_input_point_dense) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaFreeAsync(d, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return ctx_cuda(ctx, e, "lsdg_depth_export_points");
  return LSDG_OK;
}

lsdg_status lsdg_cloud_build(lsdg_ctx* ctx, int w, int h, float fx, float fy, float cx, float cy, float scale,
                             const lsdg_cloud_params* params, const lsdg_input_point_dense* points,
                             lsdg_cloud_vertex* out, int* count) {
  if (!ctx || !points || !out || !count) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (w > 0 && h > 0 && (w < 3 || h < 3)) {  // no interior pixel: computeVbo's loop keeps nothing
    *count = 0;
    return LSDG_OK;
  }
  lsdg_cloud_params p;
  if (params) p = *params;
  else lsdg_cloud_default_params(&p);
  lsdg_status st = check_cloud_args(ctx, w, h, fx, fy, p);
  if (st != LSDG_OK) return st;
  const size_t n = (size_t)w * h;
  CloudArgs a = make_args(w, h, fx, fy, cx, cy, scale, p);
  lsdg_input_point_dense* din = nullptr;
  lsdg_cloud_vertex* dout = nullptr;
  CK(ctx, cudaMallocAsync(&din, sizeof(lsdg_input_point_dense) * n, ctx->stream));
  cudaError_t e = cudaMallocAsync(&dout, sizeof(lsdg_cloud_vertex) * n, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(din, points, sizeof(lsdg_input_point_dense) * n, cudaMemcpyHostToDevice,
                                            ctx->stream);
  if (e != cudaSuccess) {
    cudaFreeAsync(din, ctx->stream);
    if (dout) cudaFreeAsync(dout, ctx->stream);
    return ctx_cuda(ctx, e, "lsdg_cloud_build");
  }
  a.dense = din;
  a.out = dout;
  st = launch_cloud<true>(ctx, a, count);
  if (st == LSDG_OK && *count > 0)
    e = cudaMemcpyAsync(out, dout, sizeof(lsdg_cloud_vertex) * (size_t)*count, cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(din, ctx->stream);
  cudaFreeAsync(dout, ctx->stream);
  if (st != LSDG_OK) return st;
  CK(ctx, e);
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_cloud_from_depthmap(lsdg_ctx* ctx, lsdg_depthmap* dm, float scale, const lsdg_cloud_params* params,
                                     lsdg_cloud_vertex* out_device, int* count) {
  if (!ctx || !dm || !out_device || !count) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (reinterpret_cast<uintptr_t>(out_device) & 15u)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "out_device must be 16-byte aligned");
  const float *id, *var, *img;
  int w, h;
  lsdg_intrinsics K;
  if (!depth_key_planes(dm, &id, &var, &img, &w, &h, &K)) return ctx_fail(ctx, LSDG_INVALID_ARG, "no keyframe set");
  lsdg_cloud_params p;
  if (params) p = *params;
  else lsdg_cloud_default_params(&p);
  lsdg_status st = check_cloud_args(ctx, w, h, K.fx, K.fy, p);
  if (st != LSDG_OK) return st;
  CloudArgs a = make_args(w, h, K.fx, K.fy, K.cx, K.cy, scale, p);
  a.idepth = id;
  a.var = var;
  a.image = img;
  a.out = out_device;
  return launch_cloud<false>(ctx, a, count);
}

}  // extern "C"

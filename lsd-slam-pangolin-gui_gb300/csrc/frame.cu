// frame.cu -- a1/a2 of the hot path: the {I, gx, gy} image pyramid of every frame and, for a
// keyframe, its inverse-depth pyramid and the compacted SoA tracking reference points.
//
// Upstream this is lsd-slam's Frame construction (absent from the reference; its consumers read
// Frame::image(lvl) / idepth(lvl) / idepthVar(lvl), lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:77-79).
// All kernels are batched over a set of frames of possibly different sizes: grid.y indexes the
// frame, grid.x covers the largest frame's pixel count at that level and surplus blocks return.
// Memory-bound streaming: one pass over each level, 256 threads per block, coalesced rows.
//
// Operation order matches the CPU oracle exactly (this translation unit is built with
// -fmad=false), so pyramids and points are bit-identical to it.
#include "lsdg_internal.cuh"

namespace lsdg {

__device__ __forceinline__ float mean4(const float* P, int pw, int x, int y) {
  const float* r0 = P + (size_t)(2 * y) * pw + 2 * x;
  const float* r1 = r0 + pw;
  return ((r0[0] + r0[1]) + (r1[0] + r1[1])) * 0.25f;
}

// 8-bit input image -> level-0 intensity plane.
__global__ void u8_to_plane_kernel(const uint8_t* __restrict__ src, float* __restrict__ dst, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

// Level `level` of every frame: intensity (2x2 mean of level-1, or the input at level 0) and, for
// frames that keep a gradient pyramid, the float4 {I, gx, gy, 0} with central-difference gradients
// (zero on the one-pixel border).  The tracker samples the intensity planes only.
__global__ void __launch_bounds__(256) pyramid_level_kernel(const FrameDev* __restrict__ frames, int level) {
  const FrameDev& F = frames[blockIdx.y];
  if (level >= F.levels) return;
  const int w = F.w >> level, h = F.h >> level;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= w * h) return;
  const int x = idx % w, y = idx / w;
  const bool ix = (x >= 1 && x <= w - 2), iy = (y >= 1 && y <= h - 2);
  float4* __restrict__ out = F.pyr[level];  // null for frames that only need intensity
  float I, Il = 0.f, Ir = 0.f, Iu = 0.f, Id = 0.f;
  if (level == 0) {
    if (!out) return;
    const float* P = F.plane[0];
    I = P[idx];
    if (ix) { Il = P[idx - 1]; Ir = P[idx + 1]; }
    if (iy) { Iu = P[idx - w]; Id = P[idx + w]; }
  } else {
    const float* P = F.plane[level - 1];
    const int pw = 2 * w;
    I = mean4(P, pw, x, y);
    F.plane[level][idx] = I;
    if (!out) return;
    if (ix) { Il = mean4(P, pw, x - 1, y); Ir = mean4(P, pw, x + 1, y); }
    if (iy) { Iu = mean4(P, pw, x, y - 1); Id = mean4(P, pw, x, y + 1); }
  }
  const float gx = ix ? (Ir - Il) * 0.5f : 0.f;
  const float gy = iy ? (Id - Iu) * 0.5f : 0.f;
  out[idx] = make_float4(I, gx, gy, 0.f);
}

// Depth pyramid level `level` (level 0: sanitise the upload in place; level l: inverse-variance
// weighted mean of the valid 2x2 children, variance = n / sum(1/var)) and the number of valid
// pixels per block of kCountBlock pixels (first pass of the point compaction).
__global__ void __launch_bounds__(kCountBlock) depth_level_kernel(const FrameDev* __restrict__ frames, int level) {
  const FrameDev& F = frames[blockIdx.y];
  if (!F.has_depth || level >= F.levels) return;
  const int w = F.w >> level, h = F.h >> level;
  if ((int)(blockIdx.x * kCountBlock) >= w * h) return;  // whole block outside this frame
  const int idx = blockIdx.x * kCountBlock + threadIdx.x;
  bool valid = false;
  if (idx < w * h) {
    if (level == 0) {
      const float d = F.idepth[0][idx], v = F.ivar[0][idx];
      valid = d > 0.f && v > 0.f;
      if (!valid) { F.idepth[0][idx] = -1.f; F.ivar[0][idx] = -1.f; }
    } else {
      const int x = idx % w, y = idx / w, pw = 2 * w;
      const float* D = F.idepth[level - 1];
      const float* V = F.ivar[level - 1];
      const size_t c0 = (size_t)(2 * y) * pw + 2 * x;
      const size_t c[4] = {c0, c0 + 1, c0 + pw, c0 + pw + 1};
      float sw = 0.f, swd = 0.f;
      int n = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float d = D[c[k]], v = V[c[k]];
        if (d > 0.f && v > 0.f) {
          const float wt = 1.0f / v;
          sw = sw + wt;
          swd = swd + wt * d;
          ++n;
        }
      }
      valid = n > 0;
      F.idepth[level][idx] = valid ? swd / sw : -1.f;
      F.ivar[level][idx] = valid ? (float)n / sw : -1.f;
    }
  }
  const int cnt = __syncthreads_count(valid);
  if (threadIdx.x == 0) F.blk_count[level][blockIdx.x] = cnt;
}

// Second pass: per (frame, level) exclusive scan of the per-block counts (in place, counts ->
// offsets) and the level's point count.  One 1024-thread block per (frame, level).
__global__ void __launch_bounds__(1024) point_scan_kernel(const FrameDev* __restrict__ frames) {
  const FrameDev& F = frames[blockIdx.x];
  const int level = blockIdx.y;
  if (!F.has_depth || level >= F.levels) return;
  const int w = F.w >> level, h = F.h >> level;
  const int nblk = (w * h + kCountBlock - 1) / kCountBlock;
  int* blk = F.blk_count[level];
  __shared__ int warp_tot[32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nblk; base += 1024) {
    const int i = base + threadIdx.x;
    const int c = i < nblk ? blk[i] : 0;
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      int v = warp_tot[lane];
      int s = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += t;
      }
      warp_tot[lane] = s - v;  // exclusive warp offsets
    }
    __syncthreads();
    const int run = carry;
    if (i < nblk) blk[i] = run + warp_tot[wid] + (incl - c);
    __syncthreads();
    if (threadIdx.x == 1023) carry = run + warp_tot[wid] + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) F.pcount[level] = carry;
}

// Third pass: write the valid pixels of level `level` as SoA points in row-major order.
__global__ void __launch_bounds__(kCountBlock) point_scatter_kernel(const FrameDev* __restrict__ frames, int level) {
  const FrameDev& F = frames[blockIdx.y];
  if (!F.has_depth || level >= F.levels) return;
  const int w = F.w >> level, h = F.h >> level;
  if ((int)(blockIdx.x * kCountBlock) >= w * h) return;
  const int idx = blockIdx.x * kCountBlock + threadIdx.x;
  float d = -1.f, v = -1.f;
  if (idx < w * h) {
    d = F.idepth[level][idx];
    v = F.ivar[level][idx];
  }
  const bool valid = d > 0.f && v > 0.f;
  const unsigned m = __ballot_sync(0xffffffffu, valid);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __shared__ int woff[kCountBlock / 32];
  if (lane == 0) woff[wid] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < kCountBlock / 32; ++k) {
      int t = woff[k];
      woff[k] = s;
      s += t;
    }
  }
  __syncthreads();
  if (!valid) return;
  const int pos = F.blk_count[level][blockIdx.x] + woff[wid] + __popc(m & ((1u << lane) - 1u));
  const int x = idx % w, y = idx / w;
  const float z = 1.0f / d;
  const float X = (((float)x - F.cx[level]) * F.fxi[level]) * z;
  const float Y = (((float)y - F.cy[level]) * F.fyi[level]) * z;
  F.pxyzi[level][pos] = make_float4(X, Y, z, F.plane[level][idx]);
  F.pvar[level][pos] = v;
}

// ------------------------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------------------------
static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

void launch_u8_to_plane(const uint8_t* src, float* dst, int n, cudaStream_t s) {
  u8_to_plane_kernel<<<cdiv(n, 256), 256, 0, s>>>(src, dst, n);
}

// Image pyramids of frames[0..n) (largest level-0 pixel count max_pix).  Returns launches issued.
int launch_frame_pyramid(const FrameDev* frames, int n, int levels, long max_pix, cudaStream_t s) {
  for (int l = 0; l < levels; ++l) {
    long pix = max_pix >> (2 * l);
    pyramid_level_kernel<<<dim3(cdiv(pix, 256), n), 256, 0, s>>>(frames, l);
  }
  return levels;
}

// Depth pyramids and reference points of the frames among frames[0..n) that carry depth (their
// image pyramids must be built).  Returns launches issued.
int launch_frame_points(const FrameDev* frames, int n, int levels, long max_pix, cudaStream_t s) {
  for (int l = 0; l < levels; ++l) {
    long pix = max_pix >> (2 * l);
    depth_level_kernel<<<dim3(cdiv(pix, kCountBlock), n), kCountBlock, 0, s>>>(frames, l);
  }
  point_scan_kernel<<<dim3(n, levels), 1024, 0, s>>>(frames);
  for (int l = 0; l < levels; ++l) {
    long pix = max_pix >> (2 * l);
    point_scatter_kernel<<<dim3(cdiv(pix, kCountBlock), n), kCountBlock, 0, s>>>(frames, l);
  }
  return 2 * levels + 1;
}

}  // namespace lsdg

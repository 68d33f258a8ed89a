// frame.cu -- a1/a2 of the hot path: the intensity pyramid of every frame (plus, for frames that
// keep it, the float4 {I, gx, gy} gradient pyramid) and, for a keyframe, its inverse-depth pyramid
// and the compacted SoA tracking reference points.
//
// Upstream this is lsd-slam's Frame construction (absent from the reference; its consumers read
// Frame::image(lvl) / idepth(lvl) / idepthVar(lvl), lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:77-79).
//
// GB300 layout of the work: a CTA owns one BAND of 2^(levels-1) level-0 rows of one frame.  Every
// coarser level of that band is built from rows of the same band (2x2 means nest), so one launch
// builds all levels of all frames, with __syncthreads between levels instead of a launch per level.
// The point compaction is band-ordered too: pass 1 counts the valid pixels of every (band, level),
// a scan turns the counts into offsets, pass 2 writes the points -- bands in order, pixels in
// row-major order inside a band, so the point arrays are in global row-major order.  Three launches
// build a keyframe, whatever the number of levels or frames; all are memory-bound streaming.
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

// Pass 1, one CTA per (band, frame): intensity levels 1..L-1 of the band; for keyframes also the
// depth pyramid (level 0 sanitised in place: idepth <= 0 or var <= 0 -> -1; level l: inverse-
// variance weighted mean of the valid 2x2 children, variance = n / sum(1/var)) and the number of
// valid pixels of the band at every level.
__global__ void __launch_bounds__(256) band_build_kernel(const FrameDev* __restrict__ frames) {
  const FrameDev& F = frames[blockIdx.y];
  const int L = F.levels;
  const int band_rows = 1 << (L - 1);
  const int band = blockIdx.x;
  if (band * band_rows >= F.h) return;
  for (int l = 1; l < L; ++l) {
    const int w = F.w >> l, rows = band_rows >> l, y0 = (band * band_rows) >> l;
    const float* P = F.plane[l - 1];
    float* Q = F.plane[l];
    for (int i = threadIdx.x; i < rows * w; i += blockDim.x) {
      const int x = i % w, y = y0 + i / w;
      Q[(size_t)y * w + x] = mean4(P, 2 * w, x, y);
    }
    __syncthreads();  // level l is read by level l + 1 (other threads of this CTA)
  }
  if (!F.has_depth) return;
  for (int l = 0; l < L; ++l) {
    const int w = F.w >> l, rows = band_rows >> l, y0 = (band * band_rows) >> l;
    int count = 0;
    for (int base = 0; base < rows * w; base += blockDim.x) {
      const int i = base + threadIdx.x;
      bool valid = false;
      if (i < rows * w) {
        const int x = i % w, y = y0 + i / w;
        const size_t idx = (size_t)y * w + x;
        if (l == 0) {
          const float d = F.idepth[0][idx], v = F.ivar[0][idx];
          valid = d > 0.f && v > 0.f;
          if (!valid) {
            F.idepth[0][idx] = -1.f;
            F.ivar[0][idx] = -1.f;
          }
        } else {
          const int pw = 2 * w;
          const float* D = F.idepth[l - 1];
          const float* V = F.ivar[l - 1];
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
          F.idepth[l][idx] = valid ? swd / sw : -1.f;
          F.ivar[l][idx] = valid ? (float)n / sw : -1.f;
        }
      }
      // block-wide count; the barrier also orders this level's writes before the next level's reads
      count += __syncthreads_count(valid);
    }
    if (threadIdx.x == 0) F.blk_count[l][band] = count;
  }
}

// Gradients of every level for frames that keep the float4 {I, gx, gy, 0} pyramid (central
// differences, zero on the one-pixel border).  grid: (pixels of level 0 / 256, frames, levels).
__global__ void __launch_bounds__(256) gradient_kernel(const FrameDev* __restrict__ frames) {
  const FrameDev& F = frames[blockIdx.y];
  const int l = blockIdx.z;
  if (l >= F.levels || !F.pyr[l]) return;
  const int w = F.w >> l, h = F.h >> l;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= w * h) return;
  const int x = idx % w, y = idx / w;
  const float* P = F.plane[l];
  const float I = P[idx];
  const float gx = (x >= 1 && x <= w - 2) ? (P[idx + 1] - P[idx - 1]) * 0.5f : 0.f;
  const float gy = (y >= 1 && y <= h - 2) ? (P[idx + w] - P[idx - w]) * 0.5f : 0.f;
  F.pyr[l][idx] = make_float4(I, gx, gy, 0.f);
}

// Per (frame, level) exclusive scan of the per-band counts (in place, counts -> offsets) and the
// level's point count.  One warp per (frame, level); bands per frame are few (h / 2^(L-1)).
__global__ void __launch_bounds__(32) point_scan_kernel(const FrameDev* __restrict__ frames) {
  const FrameDev& F = frames[blockIdx.x];
  const int level = blockIdx.y;
  if (!F.has_depth || level >= F.levels) return;
  const int nband = F.h >> (F.levels - 1);
  int* blk = F.blk_count[level];
  const int lane = threadIdx.x;
  int carry = 0;
  for (int base = 0; base < nband; base += 32) {
    const int i = base + lane;
    const int c = i < nband ? blk[i] : 0;
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (i < nband) blk[i] = carry + incl - c;
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) F.pcount[level] = carry;
}

// Pass 2, one CTA per (band, keyframe): the valid pixels of every level of the band as SoA points
// {X, Y, Z, I} + var, in row-major order, starting at the band's offset.
__global__ void __launch_bounds__(256) band_scatter_kernel(const FrameDev* __restrict__ frames) {
  const FrameDev& F = frames[blockIdx.y];
  if (!F.has_depth) return;
  const int L = F.levels;
  const int band_rows = 1 << (L - 1);
  const int band = blockIdx.x;
  if (band * band_rows >= F.h) return;
  __shared__ int woff[8];
  __shared__ int chunk_total;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int l = 0; l < L; ++l) {
    const int w = F.w >> l, rows = band_rows >> l, y0 = (band * band_rows) >> l;
    int pos0 = F.blk_count[l][band];
    const float cx = F.cx[l], cy = F.cy[l], fxi = F.fxi[l], fyi = F.fyi[l];
    for (int base = 0; base < rows * w; base += blockDim.x) {
      const int i = base + threadIdx.x;
      float d = -1.f, v = -1.f;
      int x = 0, y = 0;
      size_t idx = 0;
      if (i < rows * w) {
        x = i % w;
        y = y0 + i / w;
        idx = (size_t)y * w + x;
        d = F.idepth[l][idx];
        v = F.ivar[l][idx];
      }
      const bool valid = d > 0.f && v > 0.f;
      const unsigned m = __ballot_sync(0xffffffffu, valid);
      if (lane == 0) woff[wid] = __popc(m);
      __syncthreads();
      if (threadIdx.x == 0) {
        int s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
          const int t = woff[k];
          woff[k] = s;
          s += t;
        }
        chunk_total = s;
      }
      __syncthreads();
      if (valid) {
        const int pos = pos0 + woff[wid] + __popc(m & ((1u << lane) - 1u));
        const float z = 1.0f / d;
        const float X = (((float)x - cx) * fxi) * z;
        const float Y = (((float)y - cy) * fyi) * z;
        F.pxyzi[l][pos] = make_float4(X, Y, z, F.plane[l][idx]);
        F.pvar[l][pos] = v;
        if (F.ppix[l]) F.ppix[l][pos] = (int)idx;
      }
      pos0 += chunk_total;
      __syncthreads();  // woff / chunk_total are rewritten by the next chunk
    }
  }
}

// ------------------------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------------------------
static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

void launch_u8_to_plane(const uint8_t* src, float* dst, int n, cudaStream_t s) {
  u8_to_plane_kernel<<<cdiv(n, 256), 256, 0, s>>>(src, dst, n);
}

// Intensity pyramids of frames[0..n) (largest frame max_pix pixels, tallest max_h rows) and, for
// the frames that carry depth, the depth pyramids and per-band point counts.  with_grads: also the
// gradient pyramid of the frames that keep one.  Returns the number of launches issued.
int launch_frame_pyramid(const FrameDev* frames, int n, int levels, long max_pix, int max_h, bool with_grads,
                         cudaStream_t s) {
  const int bands = max_h >> (levels - 1);
  band_build_kernel<<<dim3(bands, n), 256, 0, s>>>(frames);
  if (!with_grads) return 1;
  gradient_kernel<<<dim3(cdiv(max_pix, 256), n, levels), 256, 0, s>>>(frames);
  return 2;
}

// Reference points of the frames among frames[0..n) that carry depth (band_build_kernel must have
// run on them with their depth uploaded).  Returns the number of launches issued.
int launch_frame_points(const FrameDev* frames, int n, int levels, int max_h, cudaStream_t s) {
  const int bands = max_h >> (levels - 1);
  point_scan_kernel<<<dim3(n, levels), 32, 0, s>>>(frames);
  band_scatter_kernel<<<dim3(bands, n), 256, 0, s>>>(frames);
  return 2;
}

}  // namespace lsdg

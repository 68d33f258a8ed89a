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
// The point compaction is band-ordered too: the valid pixels of every (band, level) are counted,
// the counts of the bands before give the band's offsets, and the band writes its points -- bands
// in order, pixels in row-major order inside a band, so the point arrays are in global row-major
// order.  Single frames do it in three launches (counts, scan, scatter); a batch step in one
// (frame_build_kernel: the offsets come from a bounded look-back over the bands before, inside the
// launch), whatever the number of levels or frames.
//
// Operation order matches the CPU oracle exactly (this translation unit is built with
// -fmad=false), so pyramids and points are bit-identical to it.
#include "lsdg_internal.cuh"

namespace lsdg {

// Row of flat pixel index i at level l, without a division: with M = floor((2^64 - 1) / w) + 1
// (FrameDev::rowdiv, from the host), M w = 2^64 + e (0 <= e < w), so the high word of i M is
// floor(i / w + i e / (w 2^64)), which is floor(i / w) whenever i e < 2^64 (any 32-bit i).
struct RowDiv {
  unsigned long long m;
  __device__ RowDiv(const FrameDev& F, int l) : m(F.rowdiv[l]) {}
  __device__ int row(int i) const { return (int)__umul64hi((unsigned long long)i, m); }
};

// 8-bit input image -> level-0 intensity plane.
__global__ void u8_to_plane_kernel(const uint8_t* __restrict__ src, float* __restrict__ dst, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

// ------------------------------------------------------------------------------------------
// The per-band steps (one CTA of 256 threads owns one band of 2^(L-1) level-0 rows)
// ------------------------------------------------------------------------------------------

// Intensity levels 1..L-1 of the band (2x2 means of the level above, rows of the same band).
// src8 (or nullptr): the frame's 8-bit level-0 image; level 1 then reads the bytes and also writes
// the level-0 float plane (each level-0 pixel belongs to exactly one 2x2 block), so an 8-bit upload
// needs no separate widening pass.  (float)byte is exact: the planes equal a float upload's.
__device__ __forceinline__ void band_intensity(const FrameDev& F, int band, const uint8_t* src8 = nullptr) {
  const int L = F.levels;
  const int band_rows = 1 << (L - 1);
  for (int l = 1; l < L; ++l) {
    const int w = F.w >> l, rows = band_rows >> l, y0 = (band * band_rows) >> l;
    const float* P = F.plane[l - 1];
    float* Q = F.plane[l] + (size_t)y0 * w;
    const int n = rows * w, pw = 2 * w;
    const RowDiv rd(F, l);
    // B outputs per thread per round: their 2 B float2 loads are in flight together
    constexpr int B = 2;
    for (int i0 = threadIdx.x; i0 < n; i0 += 256 * B) {
      float2 r0[B], r1[B];
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int i = i0 + u * 256;
        if (i < n) {
          const int r = rd.row(i), x = i - r * w, y = y0 + r;
          const size_t o = (size_t)(2 * y) * pw + 2 * x;
          if (l == 1 && src8) {
            const uchar2 b0 = *reinterpret_cast<const uchar2*>(src8 + o);
            const uchar2 b1 = *reinterpret_cast<const uchar2*>(src8 + o + pw);
            r0[u] = make_float2((float)b0.x, (float)b0.y);
            r1[u] = make_float2((float)b1.x, (float)b1.y);
            *reinterpret_cast<float2*>(F.plane[0] + o) = r0[u];
            *reinterpret_cast<float2*>(F.plane[0] + o + pw) = r1[u];
          } else {
            r0[u] = *reinterpret_cast<const float2*>(P + o);
            r1[u] = *reinterpret_cast<const float2*>(P + o + pw);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int i = i0 + u * 256;
        if (i < n) Q[i] = ((r0[u].x + r0[u].y) + (r1[u].x + r1[u].y)) * 0.25f;
      }
    }
    __syncthreads();  // level l is read by level l + 1 (other threads of this CTA)
  }
}

// Level-0 staging of the one-launch build: the band's valid level-0 pixels, in row-major order, as
// {idepth, var, intensity, band-local pixel index}, kept in shared memory from the depth pass to the
// point writes so that the writes need not read the level-0 planes a second time.  A band with more
// valid pixels than this keeps the second read (band_points' general path).
constexpr int kStageCap = 2560;

// Depth pyramid of the band (level 0 sanitised in place: idepth <= 0 or var <= 0 -> -1, written
// only where the value is not -1 already; level l: inverse-variance weighted mean of the valid 2x2
// children, variance = n / sum(1/var)) and its valid pixels per level into cnt[l] (shared memory,
// visible to the whole CTA on return).  Each thread counts its own pixels; one block sum per level.
// stage (or nullptr): shared memory of kStageCap entries that receives the level-0 valid pixels in
// row-major order (the first kStageCap of them); off: 64 ints of shared memory, total: two (both
// double-buffered by chunk parity, so a chunk's scan results stay readable while the next chunk
// publishes its counts: two barriers per chunk).
__device__ __forceinline__ void band_depth(const FrameDev& F, int band, int* cnt, int* wsum, float4* stage = nullptr,
                                           int* off = nullptr, int* total = nullptr) {
  const int L = F.levels;
  const int band_rows = 1 << (L - 1);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int l = 0; l < L; ++l) {
    const int w = F.w >> l, rows = band_rows >> l, y0 = (band * band_rows) >> l;
    int count = 0;
    if (l == 0) {
      float* D = F.idepth[0] + (size_t)y0 * w;
      float* V = F.ivar[0] + (size_t)y0 * w;
      const float* P = F.plane[0] + (size_t)y0 * w;
      const int n = rows * w;
      constexpr int B = 4, NWARP = 8;  // blockDim.x == 256
      const unsigned lt = (1u << lane) - 1u;
      int run = 0;  // staged entries so far (uniform across the CTA)
      int parity = 0;
      for (int base = 0; base < n; base += 256 * B, parity ^= 1) {
        float d[B], v[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
          const int i = base + u * 256 + (int)threadIdx.x;
          d[u] = -1.f;
          v[u] = -1.f;
          if (i < n) {
            d[u] = D[i];
            v[u] = V[i];
          }
        }
        unsigned m[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
          const int i = base + u * 256 + (int)threadIdx.x;
          const bool valid = d[u] > 0.f && v[u] > 0.f;
          count += valid ? 1 : 0;
          m[u] = stage ? __ballot_sync(0xffffffffu, valid) : 0u;
          if (i < n && !valid && !(d[u] == -1.f && v[u] == -1.f)) {
            D[i] = -1.f;
            V[i] = -1.f;
          }
        }
        if (stage) {  // same (j, warp) scan as band_points: staged in row-major order
          int* offp = off + 32 * parity;
          int* totp = total + parity;
          float I[B];
#pragma unroll
          for (int u = 0; u < B; ++u)
            I[u] = ((m[u] >> lane) & 1u) ? P[base + u * 256 + (int)threadIdx.x] : 0.f;
          if (lane < B) {
            unsigned mm = m[0];
#pragma unroll
            for (int u = 1; u < B; ++u)
              if (lane == u) mm = m[u];
            offp[lane * NWARP + wid] = __popc(mm);
          }
          __syncthreads();
          if (wid == 0) {
            const int c = offp[lane];
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const int t = __shfl_up_sync(0xffffffffu, incl, o);
              if (lane >= o) incl += t;
            }
            offp[lane] = incl - c;
            if (lane == 31) *totp = incl;
          }
          __syncthreads();
#pragma unroll
          for (int u = 0; u < B; ++u) {
            if ((m[u] >> lane) & 1u) {
              const int k = run + offp[u * NWARP + wid] + __popc(m[u] & lt);
              if (k < kStageCap)
                stage[k] = make_float4(d[u], v[u], I[u], __int_as_float(base + u * 256 + (int)threadIdx.x));
            }
          }
          run += *totp;
        }
      }
    } else {
      const int pw = 2 * w, n = rows * w;
      const RowDiv rd(F, l);
      const float* Dp = F.idepth[l - 1];
      const float* Vp = F.ivar[l - 1];
      float* Dq = F.idepth[l] + (size_t)y0 * w;
      float* Vq = F.ivar[l] + (size_t)y0 * w;
      constexpr int B = 2;
      for (int base = 0; base < n; base += 256 * B) {
        float2 d0[B], d1[B], v0[B], v1[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
          const int i = base + u * 256 + (int)threadIdx.x;
          if (i < n) {
            const int r = rd.row(i), x = i - r * w, y = y0 + r;
            const size_t c0 = (size_t)(2 * y) * pw + 2 * x;
            d0[u] = *reinterpret_cast<const float2*>(Dp + c0);
            d1[u] = *reinterpret_cast<const float2*>(Dp + c0 + pw);
            v0[u] = *reinterpret_cast<const float2*>(Vp + c0);
            v1[u] = *reinterpret_cast<const float2*>(Vp + c0 + pw);
          }
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
          const int i = base + u * 256 + (int)threadIdx.x;
          bool valid = false;
          if (i < n) {
            const float dd[4] = {d0[u].x, d0[u].y, d1[u].x, d1[u].y};
            const float vv[4] = {v0[u].x, v0[u].y, v1[u].x, v1[u].y};
            float sw = 0.f, swd = 0.f;
            int nv = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              if (dd[k] > 0.f && vv[k] > 0.f) {
                const float wt = 1.0f / vv[k];
                sw = sw + wt;
                swd = swd + wt * dd[k];
                ++nv;
              }
            }
            valid = nv > 0;
            count += valid ? 1 : 0;
            Dq[i] = valid ? swd / sw : -1.f;
            Vq[i] = valid ? (float)nv / sw : -1.f;
          }
        }
      }
    }
    // block sum of the counts; the barrier also orders this level's writes before the next level's reads
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
    if (lane == 0) wsum[wid] = count;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += wsum[k];
      cnt[l] = t;
    }
    __syncthreads();  // wsum is rewritten by the next level; cnt[l] is visible
  }
}

// The band's valid pixels of every level as SoA points {X, Y, Z, I} + var, in row-major order,
// level l starting at pos[l] (shared memory).  A chunk is 4 x 256 pixels (pixel base + 256 j +
// thread, j = 0..3): one ballot per j and warp, one warp-wide scan of the 32 (j, warp) counts, so
// three barriers per 1024 pixels.  off: 32 ints of shared memory, total: one.  stage / n_stage0:
// level 0's valid pixels as band_depth staged them (n_stage0 of them, all of the level's when
// n_stage0 <= kStageCap): they are written from shared memory without reading the level-0 planes.
__device__ __forceinline__ void band_points(const FrameDev& F, int band, const int* pos, int* off, int* total,
                                            const float4* stage = nullptr, int n_stage0 = 0) {
  const int L = F.levels;
  const int band_rows = 1 << (L - 1);
  constexpr int J = 4, NWARP = 8;  // blockDim.x == 256
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (int l = 0; l < L; ++l) {
    const int w = F.w >> l, rows = band_rows >> l, y0 = (band * band_rows) >> l;
    const int npix = rows * w;
    const RowDiv rd(F, l);
    const float* D = F.idepth[l] + (size_t)y0 * w;
    const float* V = F.ivar[l] + (size_t)y0 * w;
    const float* P = F.plane[l] + (size_t)y0 * w;
    int pos0 = pos[l];
    const float cx = F.cx[l], cy = F.cy[l], fxi = F.fxi[l], fyi = F.fyi[l];
    if (l == 0 && stage && n_stage0 <= kStageCap) {
      for (int k = (int)threadIdx.x; k < n_stage0; k += 256) {
        const float4 e = stage[k];
        const int i = __float_as_int(e.w);
        const int r = rd.row(i), x = i - r * w, y = y0 + r;
        const int p = pos0 + k;
        const float z = 1.0f / e.x;
        const float X = (((float)x - cx) * fxi) * z;
        const float Y = (((float)y - cy) * fyi) * z;
        F.pxyzi[0][p] = make_float4(X, Y, z, e.z);
        F.pvar[0][p] = e.y;
        if (F.ppix[0]) F.ppix[0][p] = y * w + x;
      }
      continue;
    }
    for (int base = 0; base < npix; base += J * 256) {
      float d[J], v[J];
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const int i = base + j * 256 + (int)threadIdx.x;
        d[j] = -1.f;
        v[j] = -1.f;
        if (i < npix) {
          d[j] = D[i];
          v[j] = V[i];
        }
      }
      unsigned m[J];
      float I[J];
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const bool ok = d[j] > 0.f && v[j] > 0.f;
        m[j] = __ballot_sync(0xffffffffu, ok);
        I[j] = ok ? P[base + j * 256 + (int)threadIdx.x] : 0.f;  // in flight across the scan
      }
      if (lane < J) {
        unsigned mm = m[0];
#pragma unroll
        for (int j = 1; j < J; ++j)
          if (lane == j) mm = m[j];
        off[lane * NWARP + wid] = __popc(mm);
      }
      __syncthreads();
      if (wid == 0) {  // exclusive scan of the (j, warp) counts, j-major = pixel order
        const int c = off[lane];
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        off[lane] = incl - c;
        if (lane == 31) *total = incl;
      }
      __syncthreads();
#pragma unroll
      for (int j = 0; j < J; ++j) {
        if ((m[j] >> lane) & 1u) {
          const int i = base + j * 256 + (int)threadIdx.x;
          const int r = rd.row(i), x = i - r * w, y = y0 + r;
          const size_t idx = (size_t)y * w + x;
          const int p = pos0 + off[j * NWARP + wid] + __popc(m[j] & lt);
          const float z = 1.0f / d[j];
          const float X = (((float)x - cx) * fxi) * z;
          const float Y = (((float)y - cy) * fyi) * z;
          F.pxyzi[l][p] = make_float4(X, Y, z, I[j]);
          F.pvar[l][p] = v[j];
          if (F.ppix[l]) F.ppix[l][p] = (int)idx;
        }
      }
      pos0 += *total;
      __syncthreads();  // off / total are rewritten by the next chunk
    }
  }
}

// ------------------------------------------------------------------------------------------
// Three-launch build (single frames): pyramids and band counts, scan, scatter
// ------------------------------------------------------------------------------------------

// One CTA per (band, frame, part): part 0 the intensity pyramid, part 1 (frames with depth) the
// depth pyramid and the band's valid pixels per level (blk_count).
__global__ void __launch_bounds__(256, 5) band_build_kernel(const FrameDev* __restrict__ frames) {
  const FrameDev& F = frames[blockIdx.y];
  const int band = blockIdx.x;
  if (band * (1 << (F.levels - 1)) >= F.h) return;
  __shared__ int wsum[8];
  __shared__ int cnt[kMaxLevels];
  if (blockIdx.z == 0) {
    band_intensity(F, band);
    return;
  }
  if (!F.has_depth) return;
  band_depth(F, band, cnt, wsum);
  if ((int)threadIdx.x < F.levels) F.blk_count[threadIdx.x][band] = cnt[threadIdx.x];
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

// One CTA per (band, keyframe): the band's points from the offsets point_scan_kernel left.
__global__ void __launch_bounds__(256) band_scatter_kernel(const FrameDev* __restrict__ frames) {
  const FrameDev& F = frames[blockIdx.y];
  if (!F.has_depth) return;
  const int band = blockIdx.x;
  if (band * (1 << (F.levels - 1)) >= F.h) return;
  __shared__ int pos[kMaxLevels];
  __shared__ int off[32];
  __shared__ int total;
  if ((int)threadIdx.x < F.levels) pos[threadIdx.x] = F.blk_count[threadIdx.x][band];
  __syncthreads();
  band_points(F, band, pos, off, &total);
}

// ------------------------------------------------------------------------------------------
// One-launch build (batches): every band's pyramids, then its points at offsets found in the
// same launch by a decoupled look-back over the bands before it
// ------------------------------------------------------------------------------------------
// Workspace (zeroed before the launch): word 0 = {ticket, error}, then one status word per
// (frame, band, level): 0 = nothing yet, 1 << 32 | n = the band's own count, 2 << 32 | n = the
// count of bands 0..band inclusive.  A CTA takes the next ticket as its (frame, band) in
// frame-major, band-minor order, so every band it waits for has started (tickets are issued in CTA
// start order) and waits only for bands that started before it: no wait can be circular.  Each
// wait is bounded; when one runs out the CTA records the error word, counts what it has, and its
// point writes stay inside the level's arrays (offsets never exceed the true ones).
constexpr int kBuildSpinLimit = 1 << 20;

// withhold_frame (>= 0 only in tests of the bounded wait): band 0 of that frame publishes nothing,
// so the frame's other bands wait until their limit and the error word is set.
// u8 / plane0 / mode: when *mode is 1 the level-0 images are the bytes at u8 (laid out like the
// float planes from plane0 on) and the build widens them (band_intensity).
// The level-0 points are staged in shared memory by the depth pass (40 KB a CTA, kStageCap) and
// written from there after the look-back; four CTAs per SM leave 64 registers a thread (five, at 48,
// spilled and ran slower).
__global__ void __launch_bounds__(256, 4) frame_build_kernel(const FrameDev* __restrict__ frames, int n_frames,
                                                             int n_point_frames, int bands,
                                                             unsigned long long* __restrict__ ws, int withhold_frame,
                                                             const uint8_t* __restrict__ u8,
                                                             const float* __restrict__ plane0, const int* __restrict__ mode) {
  __shared__ int s_ticket;
  __shared__ int wsum[8];
  __shared__ int cnt[kMaxLevels];
  __shared__ int pos[kMaxLevels];
  __shared__ int off[64];
  __shared__ int total[2];
  __shared__ float4 stage[kStageCap];
  if (threadIdx.x == 0) s_ticket = (int)atomicAdd(reinterpret_cast<unsigned int*>(ws), 1u);
  __syncthreads();
  const int t = s_ticket;
  const int fi = t / bands, band = t % bands;
  if (fi >= n_frames) return;
  const FrameDev& F = frames[fi];
  const int L = F.levels;
  const int nb = F.h >> (L - 1);
  if (band >= nb) return;
  const uint8_t* src8 = (mode && *mode == 1) ? u8 + (F.plane[0] - plane0) : nullptr;
  band_intensity(F, band, src8);
  if (!F.has_depth) return;
  const bool points = fi < n_point_frames;
  band_depth(F, band, cnt, wsum, points ? stage : nullptr, off, total);
  if (!points) return;
  if ((int)threadIdx.x < L) {
    const int l = threadIdx.x;
    volatile unsigned long long* st = ws + 1 + (size_t)fi * bands * kMaxLevels;
    const unsigned c = (unsigned)cnt[l];
    unsigned prefix = 0;
    if (band > 0) {
      st[band * kMaxLevels + l] = (1ull << 32) | c;
      for (int j = band - 1; j >= 0; --j) {
        unsigned long long wv = st[j * kMaxLevels + l];
        for (int it = 0; (wv >> 32) == 0ull; ++it) {
          if (it == kBuildSpinLimit) {
            atomicExch(reinterpret_cast<unsigned int*>(ws) + 1, 1u);
            wv = 2ull << 32;  // give up on the bands before: offsets stay below the true ones
            break;
          }
          __nanosleep(128);
          wv = st[j * kMaxLevels + l];
        }
        prefix += (unsigned)wv;
        if ((wv >> 32) == 2ull) break;
      }
    }
    if (!(band == 0 && fi == withhold_frame)) st[band * kMaxLevels + l] = (2ull << 32) | (prefix + c);
    pos[l] = (int)prefix;
    if (band == nb - 1) F.pcount[l] = (int)(prefix + c);
  }
  __syncthreads();
  band_points(F, band, pos, off, total, stage, cnt[0]);
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
  band_build_kernel<<<dim3(bands, n, 2), 256, 0, s>>>(frames);
  if (!with_grads) return 1;
  gradient_kernel<<<dim3(cdiv(max_pix, 256), n, levels), 256, 0, s>>>(frames);
  return 2;
}

// Bytes of the one-launch build's workspace for n frames of at most max_h rows.
size_t frame_build_ws_bytes(int n, int levels, int max_h) {
  return sizeof(unsigned long long) * (1 + (size_t)n * (max_h >> (levels - 1)) * kMaxLevels);
}

// One launch: intensity pyramids of frames[0..n), depth pyramids of those that carry depth,
// reference points of the first n_point_frames (which must all carry depth).  ws: the zeroed
// workspace (frame_build_ws_bytes; zeroed here on the stream).  Returns the launches issued.
int launch_frame_build(const FrameDev* frames, int n, int n_point_frames, int levels, int max_h,
                       unsigned long long* ws, cudaStream_t s, int withhold_frame, const uint8_t* u8,
                       const float* plane0, const int* mode) {
  const int bands = max_h >> (levels - 1);
  cudaMemsetAsync(ws, 0, frame_build_ws_bytes(n, levels, max_h), s);
  frame_build_kernel<<<bands * n, 256, 0, s>>>(frames, n, n_point_frames, bands, ws, withhold_frame, u8, plane0,
                                               mode);
  return 1;
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

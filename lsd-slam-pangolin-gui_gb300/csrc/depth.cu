// depth.cu -- a7/a8/a9 of the hot path: the semi-dense inverse-depth filter.
//
// Upstream: DepthMap::updateKeyframe -> observeDepth, DepthMap::createKeyFrame -> propagateDepth,
// regularizeDepthMap (lsd-slam fips import, absent from the reference; its output is what
// PangolinOutputIOWrapper::publishKeyframe copies out, lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:77-89).
// Method: ICCV 2013 semi-dense VO (epipolar 5-sample SSD search, geometric + photometric disparity
// error, Gaussian fusion, propagation with (d'/d)^4 variance growth, neighbourhood regularisation).
//
// GB300 design:
//   observe    one thread per keyframe pixel, a warp per 32-pixel strip of a row; the pixel's
//              state stays in registers while it is observed against every reference in turn
//              (one launch per updateKeyframe, state read and written once).  The sliding 5-sample
//              window keeps the last five reference samples in registers, so every reference
//              sample is interpolated once per pixel.  Reference images are L2-resident planes.
//   regularize one thread per pixel over a (2r+1)^2 window (L1-cached neighbour reads), writing
//              the smoothed planes; a second pass commits removals to the raw state.
//   propagate  forward warp with a 64-bit atomicMin z-buffer {float bits of z, old index} per
//              target pixel (deterministic: nearest wins, ties to the lower old index), then a
//              gather pass that writes the new keyframe's state.
// Built with -fmad=false: every float operation rounds as in the CPU oracle, so the state is
// bit-identical to it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>

#include "lsdg_host.h"

using namespace lsdg;

namespace lsdg {
int launch_frame_pyramid(const FrameDev* frames, int n, int levels, long max_pix, int max_h, bool with_grads,
                         cudaStream_t s);
void launch_u8_to_plane(const uint8_t* src, float* dst, int n, cudaStream_t s);
}

#define CK(ctx, expr)                                \
  do {                                               \
    lsdg_status _s = ctx_cuda((ctx), (expr), #expr); \
    if (_s != LSDG_OK) return _s;                    \
  } while (0)

namespace {

struct RefGeomF {
  float M[9], b[3], c[3];
};

struct DepthPlanes {
  float* d;
  float* v;
  float* sm;
  float* vsm;
  int* val;
  int* bl;
};

struct ObserveArgs {
  int w, h;
  float fx, fy, cx, cy;
  const float4* key;  // keyframe {I, gx, gy, 0}
  const float* refs;  // reference planes back to back
  int n_refs;
  RefGeomF geom[LSDG_MAX_REFS];
  DepthPlanes st;
  float min_grad, min_grad_along_epl2, min_epl_length, min_idepth, max_idepth, search_sigmas;
  float min_search_len, max_search_len, max_ssd, unique_ratio, epipolar_var, image_var, fuse_chi2;
  int validity_init, validity_max, validity_penalty, blacklist_limit;
};

__device__ __forceinline__ float bilinear_plane(const float* I, int w, float x, float y) {
  const int ix = (int)x, iy = (int)y;
  const float ax = x - (float)ix, ay = y - (float)iy;
  const float bx = 1.f - ax, by = 1.f - ay;
  const float* p = I + (size_t)iy * w + ix;
  return (((bx * by) * __ldg(p) + (ax * by) * __ldg(p + 1)) + (bx * ay) * __ldg(p + w)) + (ax * ay) * __ldg(p + w + 1);
}

__device__ __forceinline__ float bilinear_key(const float4* K, int w, float x, float y) {
  const int ix = (int)x, iy = (int)y;
  const float ax = x - (float)ix, ay = y - (float)iy;
  const float bx = 1.f - ax, by = 1.f - ay;
  const float4* p = K + (size_t)iy * w + ix;
  return (((bx * by) * __ldg(p).x + (ax * by) * __ldg(p + 1).x) + (bx * ay) * __ldg(p + w).x) + (ax * ay) * __ldg(p + w + 1).x;
}

// The 5-sample SSD search along the reference epipolar segment: windows s = 0..n centred at
// pf + s lr, the best (s1, e1), its neighbours' SSDs (ebefore, eafter) and the second best e2 of the
// online rule (a window counts for e2 when it is at least 2 windows from the best standing when it
// is met, or when it was the best and a better one appears at least 2 windows later).
struct SearchResult {
  float e1, e2, ebefore, eafter;
  int s1;
};

__device__ __forceinline__ SearchResult search_seq(const float* __restrict__ Ir, int w, float umax, float vmax,
                                                   float pfx, float pfy, float lrx, float lry, int n,
                                                   const float (&tk)[5]) {
  const float INF = __int_as_float(0x7f800000);
  float r0 = 0.f, r1 = 0.f, r2 = 0.f, r3 = 0.f, r4 = 0.f;
  bool o0 = false, o1 = false, o2 = false, o3 = false, o4 = false;
  float e1 = INF, e2 = INF, eprev = INF, ebefore = INF, eafter = INF;
  int s1 = -1;
  for (int j = -2; j <= n + 2; ++j) {
    r0 = r1; r1 = r2; r2 = r3; r3 = r4;
    o0 = o1; o1 = o2; o2 = o3; o3 = o4;
    const float sx = pfx + (float)j * lrx, sy = pfy + (float)j * lry;
    o4 = sx >= 0.f && sy >= 0.f && sx < umax && sy < vmax;
    r4 = o4 ? bilinear_plane(Ir, w, sx, sy) : 0.f;
    if (j < 2) continue;
    const int s = j - 2;
    float e = INF;
    if (o0 && o1 && o2 && o3 && o4) {
      const float d0 = r0 - tk[0], d1 = r1 - tk[1], d2 = r2 - tk[2], d3 = r3 - tk[3], d4 = r4 - tk[4];
      e = (((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3) + d4 * d4;
    }
    if (e < e1) {
      if (s1 >= 0 && s - s1 >= 2 && e1 < e2) e2 = e1;
      ebefore = eprev;
      e1 = e;
      s1 = s;
      eafter = INF;
    } else {
      if (s == s1 + 1) eafter = e;
      if (s - s1 >= 2 && e < e2) e2 = e;
    }
    eprev = e;
  }
  return SearchResult{e1, e2, ebefore, eafter, s1};
}

// The same search shared by the G lanes of a group (lane u of G, `mask` the group's lanes, `buf`
// 2 * kSplitCap floats of the group's shared memory), with the same results bit for bit: the samples
// (INF outside the image) and the window SSDs are computed in parallel with the same operations;
// then each lane takes a contiguous chunk of windows.  The best standing before a window is a prefix
// minimum (earliest index on ties, as the strict comparison of the online rule keeps it), so every
// lane learns the best before its chunk from the lanes before it, walks its chunk with the online
// rule's two eligibility tests, and e2 is the minimum over the lanes -- a minimum, like the online
// rule's assignments, so its value does not depend on the order of the candidates.
constexpr int kSplitCap = 128;  // samples per segment the split search holds (n + 5)

template <int G>
__device__ __forceinline__ SearchResult search_split(const float* __restrict__ Ir, int w, float umax, float vmax,
                                                     float pfx, float pfy, float lrx, float lry, int n,
                                                     const float (&tk)[5], int u, int lane0, unsigned mask,
                                                     float* __restrict__ buf) {
  const float INF = __int_as_float(0x7f800000);
  float* samp = buf;
  float* es = buf + kSplitCap;
  for (int j = -2 + u; j <= n + 2; j += G) {
    const float sx = pfx + (float)j * lrx, sy = pfy + (float)j * lry;
    const bool ok = sx >= 0.f && sy >= 0.f && sx < umax && sy < vmax;
    samp[j + 2] = ok ? bilinear_plane(Ir, w, sx, sy) : INF;
  }
  __syncwarp(mask);
  for (int s = u; s <= n; s += G) {
    const float r0 = samp[s], r1 = samp[s + 1], r2 = samp[s + 2], r3 = samp[s + 3], r4 = samp[s + 4];
    float e = INF;
    if (r0 < INF && r1 < INF && r2 < INF && r3 < INF && r4 < INF) {  // all five inside the image
      const float d0 = r0 - tk[0], d1 = r1 - tk[1], d2 = r2 - tk[2], d3 = r3 - tk[3], d4 = r4 - tk[4];
      e = (((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3) + d4 * d4;
    }
    es[s] = e;
  }
  __syncwarp(mask);
  const int nw = n + 1;
  const int chunk = (nw + G - 1) / G;
  const int c0 = min(nw, u * chunk), c1 = min(nw, c0 + chunk);
  float cm = INF;  // this chunk's best, first occurrence
  int ci = -1;
  for (int s = c0; s < c1; ++s) {
    const float e = es[s];
    if (e < cm) {
      cm = e;
      ci = s;
    }
  }
  float pm = INF, e1 = INF;  // best before this chunk; best overall
  int pi = -1, s1 = -1;
#pragma unroll
  for (int v = 0; v < G; ++v) {
    const float vm = __shfl_sync(mask, cm, lane0 + v);
    const int vi = __shfl_sync(mask, ci, lane0 + v);
    if (v < u && vm < pm) {
      pm = vm;
      pi = vi;
    }
    if (vm < e1) {
      e1 = vm;
      s1 = vi;
    }
  }
  float e2l = INF;
  float cur = pm;
  int curi = pi;
  for (int s = c0; s < c1; ++s) {
    const float e = es[s];
    if (e < cur) {
      if (curi >= 0 && s - curi >= 2 && cur < e2l) e2l = cur;
      cur = e;
      curi = s;
    } else if (s - curi >= 2 && e < e2l) {
      e2l = e;
    }
  }
  float e2 = INF;
#pragma unroll
  for (int v = 0; v < G; ++v) {
    const float x = __shfl_sync(mask, e2l, lane0 + v);
    if (x < e2) e2 = x;
  }
  SearchResult r;
  r.e1 = e1;
  r.e2 = e2;
  r.s1 = s1;
  r.ebefore = s1 >= 1 ? es[s1 - 1] : INF;
  r.eafter = (s1 >= 0 && s1 < n) ? es[s1 + 1] : INF;
  __syncwarp(mask);  // the buffer is rewritten by the next search
  return r;
}

// observeDepth of one pixel against one reference: the same operations, in the same order, as the
// CPU oracle's observe_pixel.  G > 1: the G lanes of a group run it together, each with the whole
// state, sharing the epipolar search (search_split); G = 1: one lane per pixel.
template <int NG>
__device__ void observe_one(const ObserveArgs& A, const RefGeomF& G, const float* __restrict__ Ir, int x, int y,
                            float gx, float gy, float& d, float& var, int& val, int& bl, int u = 0, int lane0 = 0,
                            unsigned mask = 0xffffffffu, float* buf = nullptr) {
  const int w = A.w, h = A.h;
  const float g2 = gx * gx + gy * gy;
  const float mg = A.min_grad;
  if (!(g2 >= mg * mg)) return;
  const float xf = (float)x, yf = (float)y;
  float lkx = G.c[2] * (xf - A.cx) - A.fx * G.c[0];
  float lky = G.c[2] * (yf - A.cy) - A.fy * G.c[1];
  const float el2 = lkx * lkx + lky * lky;
  if (!(el2 > 1e-12f)) return;
  const float einv = 1.0f / sqrtf(el2);
  lkx = lkx * einv;
  lky = lky * einv;
  const float gp = gx * lkx + gy * lky;
  const float cos2 = (gp * gp) / g2;
  if (!(cos2 >= A.min_grad_along_epl2)) return;
  const float ax = (G.M[0] * xf + G.M[1] * yf) + G.M[2];
  const float ay = (G.M[3] * xf + G.M[4] * yf) + G.M[5];
  const float az = (G.M[6] * xf + G.M[7] * yf) + G.M[8];
  const float bx = G.b[0], by = G.b[1], bz = G.b[2];
  if (!(az > 0.f)) return;
  const float rx = bx * az - ax * bz, ry = by * az - ay * bz;
  const float rn = sqrtf(rx * rx + ry * ry);
  if (!(rn / (az * az) >= A.min_epl_length)) return;
  const float lrx = rx / rn, lry = ry / rn;
  float dlo, dhi;
  if (val > 0) {
    const float sd = sqrtf(var);
    dlo = d - A.search_sigmas * sd;
    dhi = d + A.search_sigmas * sd;
    if (dlo < A.min_idepth) dlo = A.min_idepth;
    if (dhi > A.max_idepth) dhi = A.max_idepth;
  } else {
    dlo = A.min_idepth;
    dhi = A.max_idepth;
  }
  if (!(dlo < dhi)) return;
  const float zlo = az + bz * dlo, zhi = az + bz * dhi;
  if (!(zlo > 0.f && zhi > 0.f)) return;
  float pfx = (ax + bx * dlo) / zlo, pfy = (ay + by * dlo) / zlo;
  const float pnx = (ax + bx * dhi) / zhi, pny = (ay + by * dhi) / zhi;
  float L = (pnx - pfx) * lrx + (pny - pfy) * lry;
  if (L < A.min_search_len) {
    const float pad = (A.min_search_len - L) * 0.5f;
    pfx = pfx - lrx * pad;
    pfy = pfy - lry * pad;
    L = A.min_search_len;
  }
  if (L > A.max_search_len) L = A.max_search_len;
  {
    const float dm = (dlo + dhi) * 0.5f;
    const float z0 = az + bz * dm;
    const float a1x = ax + (G.M[0] * lkx + G.M[1] * lky), a1y = ay + (G.M[3] * lkx + G.M[4] * lky);
    const float a1z = az + (G.M[6] * lkx + G.M[7] * lky);
    const float z1 = a1z + bz * dm;
    const float qx = (a1x + bx * dm) / z1 - (ax + bx * dm) / z0;
    const float qy = (a1y + by * dm) / z1 - (ay + by * dm) / z0;
    if (qx * lrx + qy * lry < 0.f) {
      lkx = -lkx;
      lky = -lky;
    }
  }
  float tk[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) tk[k] = bilinear_key(A.key, w, xf + (float)(k - 2) * lkx, yf + (float)(k - 2) * lky);
  const int n = (int)L;
  const float INF = __int_as_float(0x7f800000);
  const float umax = (float)(w - 1), vmax = (float)(h - 1);
  SearchResult sr;
  if (NG > 1 && n + 5 <= kSplitCap) sr = search_split<NG>(Ir, w, umax, vmax, pfx, pfy, lrx, lry, n, tk, u, lane0, mask, buf);
  else sr = search_seq(Ir, w, umax, vmax, pfx, pfy, lrx, lry, n, tk);
  const float e1 = sr.e1, e2 = sr.e2, ebefore = sr.ebefore, eafter = sr.eafter;
  const int s1 = sr.s1;
  if (s1 < 0) return;
  if (e1 > A.max_ssd * 5.f) {
    ++bl;
    return;
  }
  if (!(e2 > A.unique_ratio * e1)) return;
  float off = 0.f;
  if (ebefore < INF && eafter < INF) {
    const float den = (ebefore - 2.f * e1) + eafter;
    if (den > 0.f) {
      off = (0.5f * (ebefore - eafter)) / den;
      if (off > 0.5f) off = 0.5f;
      if (off < -0.5f) off = -0.5f;
    }
  }
  const float sm = (float)s1 + off;
  const float mx = pfx + sm * lrx, my = pfy + sm * lry;
  float dobs, alpha;
  if (fabsf(lrx) >= fabsf(lry)) {
    const float den = mx * bz - bx;
    dobs = (ax - mx * az) / den;
    alpha = fabsf(lrx * (bx * az - ax * bz)) / (den * den);
  } else {
    const float den = my * bz - by;
    dobs = (ay - my * az) / den;
    alpha = fabsf(lry * (by * az - ay * bz)) / (den * den);
  }
  if (!(dobs > 0.f)) return;
  const float geo = A.epipolar_var / cos2;
  const float photo = (2.f * A.image_var) / (gp * gp);
  const float vobs = (alpha * alpha) * (geo + photo);
  if (val <= 0) {
    d = dobs;
    var = vobs;
    val = A.validity_init;
    return;
  }
  const float dd = dobs - d;
  const float chi2 = (dd * dd) / (var + vobs);
  if (chi2 > A.fuse_chi2) {
    ++bl;
    val -= A.validity_penalty;
    if (val <= 0) {
      val = 0;
      d = -1.f;
      var = -1.f;
    }
    return;
  }
  const float sv = var + vobs;
  d = (d * vobs + dobs * var) / sv;
  var = (var * vobs) / sv;
  val = val + 1 < A.validity_max ? val + 1 : A.validity_max;
}

// Work list of the observe step: the keyframe pixels a reference can change (inside the 3-pixel
// border, gradient magnitude at least min_grad; the same test, in the same float operations, that
// observe_pixel_all repeats).  A warp appends its pixels with one atomic, so the list's order
// varies from run to run; that is immaterial, every pixel's state depends on that pixel alone.
// counters[0] receives the list length (zeroed before the launch).
__global__ void __launch_bounds__(256) depth_worklist_kernel(const float4* __restrict__ key, int w, int h,
                                                             float min_grad, int* __restrict__ list,
                                                             int* __restrict__ counters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  bool ok = false;
  if (i < w * h) {
    const int y = i / w, x = i - y * w;
    if (!(x < 3 || y < 3 || x > w - 4 || y > h - 4)) {
      const float4 kp = __ldg(&key[i]);
      const float g2 = kp.y * kp.y + kp.z * kp.z;
      ok = g2 >= min_grad * min_grad;
    }
  }
  const unsigned m = __ballot_sync(0xffffffffu, ok);
  int base = 0;
  if (lane == 0 && m) base = atomicAdd(&counters[0], __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (ok) list[base + __popc(m & ((1u << lane) - 1u))] = i;
}

// observeDepth of keyframe pixel i against every reference in order (its state in registers; with
// NG > 1 every lane of the pixel's group holds it and the writes come from lane u = 0).
template <int NG>
__device__ __forceinline__ void observe_pixel_all(const ObserveArgs& A, int i, int u = 0, int lane0 = 0,
                                                  unsigned mask = 0xffffffffu, float* buf = nullptr) {
  const int w = A.w;
  const int y = i / w, x = i - y * w;
  const float4 kp = __ldg(&A.key[i]);
  const float g2 = kp.y * kp.y + kp.z * kp.z;
  if (!(g2 >= A.min_grad * A.min_grad)) return;  // no reference can change this pixel
  float d = A.st.d[i], var = A.st.v[i];
  int val = A.st.val[i], bl = A.st.bl[i];
  const size_t plane = (size_t)w * A.h;
  for (int r = 0; r < A.n_refs; ++r) {
    if (bl >= A.blacklist_limit) break;
    observe_one<NG>(A, A.geom[r], A.refs + plane * r, x, y, kp.y, kp.z, d, var, val, bl, u, lane0, mask, buf);
  }
  if (u == 0) {
    A.st.d[i] = d;
    A.st.v[i] = var;
    A.st.val[i] = val;
    A.st.bl[i] = bl;
  }
}

// A persistent grid over the work list: each warp takes the next 32 listed pixels (one atomic),
// so every lane holds a pixel that searches and warps that draw short epipolar segments come back
// for more.  counters[0] = list length, counters[1] = next list entry (zeroed before the list
// kernel).
__global__ void __launch_bounds__(128) depth_observe_kernel(const ObserveArgs A, const int* __restrict__ list,
                                                            int* __restrict__ counters) {
  const int lane = threadIdx.x & 31;
  const int n = *reinterpret_cast<volatile const int*>(&counters[0]);
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&counters[1], 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const int t = base + lane;
    if (t < n) observe_pixel_all<1>(A, __ldg(&list[t]));
  }
}

// The same over groups of NG lanes per listed pixel: a warp takes 32 / NG pixels at a time and each
// group shares its pixel's epipolar searches (search_split), so a pixel's chain of dependent samples
// is NG times shorter.
template <int NG>
__global__ void __launch_bounds__(128) depth_observe_split_kernel(const ObserveArgs A, const int* __restrict__ list,
                                                                  int* __restrict__ counters) {
  constexpr int PPW = 32 / NG;
  __shared__ float buf[4][PPW][2 * kSplitCap];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int gi = lane / NG, u = lane % NG, lane0 = gi * NG;
  const unsigned mask = (NG == 32) ? 0xffffffffu : (((1u << NG) - 1u) << lane0);
  const int n = *reinterpret_cast<volatile const int*>(&counters[0]);
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&counters[1], PPW);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const int t = base + gi;
    if (t < n) observe_pixel_all<NG>(A, __ldg(&list[t]), u, lane0, mask, buf[wid][gi]);
  }
}

struct RegArgs {
  int w, h, radius, min_support, fill_min_support;
  float chi2, fill_var_factor;
  DepthPlanes st;
};

__global__ void __launch_bounds__(256) depth_regularize_kernel(const RegArgs A) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int w = A.w, h = A.h, R = A.radius;
  if (x >= w || y >= h) return;
  const size_t i = (size_t)y * w + x;
  float sw = 0.f, swd = 0.f;
  int cnt = 0;
  const int* __restrict__ val = A.st.val;
  const float* __restrict__ D = A.st.d;
  const float* __restrict__ V = A.st.v;
  if (val[i] > 0) {
    const float d = D[i], v = V[i];
    for (int dy = -R; dy <= R; ++dy)
      for (int dx = -R; dx <= R; ++dx) {
        const int nx = x + dx, ny = y + dy;
        if (nx < 0 || ny < 0 || nx >= w || ny >= h) continue;
        const size_t j = (size_t)ny * w + nx;
        if (__ldg(&val[j]) <= 0) continue;
        const float dj = __ldg(&D[j]), vj = __ldg(&V[j]);
        const float dd = dj - d;
        if (dd * dd <= A.chi2 * (vj + v)) {
          const float wt = 1.0f / vj;
          sw = sw + wt;
          swd = swd + wt * dj;
          if (dx != 0 || dy != 0) ++cnt;
        }
      }
    if (cnt < A.min_support) {
      A.st.sm[i] = -1.f;
      A.st.vsm[i] = -2.f;  // removal, committed by depth_commit_kernel
    } else {
      A.st.sm[i] = swd / sw;
      A.st.vsm[i] = v;
    }
  } else {
    for (int dy = -R; dy <= R; ++dy)
      for (int dx = -R; dx <= R; ++dx) {
        const int nx = x + dx, ny = y + dy;
        if (nx < 0 || ny < 0 || nx >= w || ny >= h) continue;
        const size_t j = (size_t)ny * w + nx;
        if (__ldg(&val[j]) <= 0) continue;
        const float wt = 1.0f / __ldg(&V[j]);
        sw = sw + wt;
        swd = swd + wt * __ldg(&D[j]);
        ++cnt;
      }
    if (cnt >= A.fill_min_support) {
      A.st.sm[i] = swd / sw;
      A.st.vsm[i] = A.fill_var_factor * ((float)cnt / sw);
    } else {
      A.st.sm[i] = -1.f;
      A.st.vsm[i] = -1.f;
    }
  }
}

__global__ void __launch_bounds__(256) depth_commit_kernel(DepthPlanes st, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (st.vsm[i] == -2.f) {
    st.val[i] = 0;
    st.d[i] = -1.f;
    st.v[i] = -1.f;
  }
}

struct PropArgs {
  int w, h;
  float fx, fy, cx, cy, fxi, fyi, min_z, max_photo_diff, prediction_var;
  float R[9], t[3];
  const float* Iold;
  const float* Inew;
  DepthPlanes src, dst;
  unsigned long long* key;
};

struct PropWarp {
  float izn;
  int ti;
  float zn;
  bool ok;
};

__device__ __forceinline__ PropWarp prop_warp(const PropArgs& A, int x, int y) {
  PropWarp r{0.f, 0, 0.f, false};
  const int w = A.w, h = A.h;
  const size_t i = (size_t)y * w + x;
  const float z = 1.0f / A.src.d[i];
  const float X = (((float)x - A.cx) * A.fxi) * z, Y = (((float)y - A.cy) * A.fyi) * z;
  const float Xn = ((A.R[0] * X + A.R[1] * Y) + A.R[2] * z) + A.t[0];
  const float Yn = ((A.R[3] * X + A.R[4] * Y) + A.R[5] * z) + A.t[1];
  const float Zn = ((A.R[6] * X + A.R[7] * Y) + A.R[8] * z) + A.t[2];
  if (!(Zn > A.min_z)) return r;
  const float izn = 1.0f / Zn;
  const float un = A.fx * (Xn * izn) + A.cx, vn = A.fy * (Yn * izn) + A.cy;
  const float fxr = floorf(un + 0.5f), fyr = floorf(vn + 0.5f);
  if (!(fxr >= 0.f && fyr >= 0.f && fxr <= (float)(w - 1) && fyr <= (float)(h - 1))) return r;
  const int xi = (int)fxr, yi = (int)fyr;
  const float diff = A.Inew[(size_t)yi * w + xi] - A.Iold[i];
  if (fabsf(diff) > A.max_photo_diff) return r;
  r.izn = izn;
  r.zn = Zn;
  r.ti = yi * w + xi;
  r.ok = true;
  return r;
}

__global__ void __launch_bounds__(256) depth_prop_key_kernel(const PropArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.w * A.h) return;
  if (A.src.val[i] <= 0) return;
  const PropWarp r = prop_warp(A, i % A.w, i / A.w);
  if (!r.ok) return;
  const unsigned long long k = ((unsigned long long)__float_as_uint(r.zn) << 32) | (unsigned long long)(unsigned)i;
  atomicMin(&A.key[r.ti], k);
}

__global__ void __launch_bounds__(256) depth_prop_write_kernel(const PropArgs A) {
  const int ti = blockIdx.x * blockDim.x + threadIdx.x;
  if (ti >= A.w * A.h) return;
  const unsigned long long k = A.key[ti];
  if (k == ~0ull) {
    A.dst.d[ti] = -1.f;
    A.dst.v[ti] = -1.f;
    A.dst.sm[ti] = -1.f;
    A.dst.vsm[ti] = -1.f;
    A.dst.val[ti] = 0;
    A.dst.bl[ti] = 0;
    return;
  }
  const unsigned o = (unsigned)(k & 0xffffffffu);
  const PropWarp r = prop_warp(A, (int)(o % (unsigned)A.w), (int)(o / (unsigned)A.w));
  const float d = A.src.d[o], v = A.src.v[o];
  const float ratio = r.izn / d;
  const float r2 = ratio * ratio;
  const float nv = v * (r2 * r2) + A.prediction_var;
  A.dst.d[ti] = r.izn;
  A.dst.v[ti] = nv;
  A.dst.sm[ti] = r.izn;
  A.dst.vsm[ti] = nv;
  A.dst.val[ti] = A.src.val[o];
  A.dst.bl[ti] = 0;
}

__global__ void __launch_bounds__(256) depth_init_kernel(DepthPlanes st, int n, int validity_init) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float d = st.d[i], v = st.v[i];
  const bool ok = d > 0.f && v > 0.f;
  st.d[i] = ok ? d : -1.f;
  st.v[i] = ok ? v : -1.f;
  st.sm[i] = ok ? d : -1.f;
  st.vsm[i] = ok ? v : -1.f;
  st.val[i] = ok ? validity_init : 0;
  st.bl[i] = 0;
}

// Per-reference geometry in double, rounded to float -- the same expressions and order as the CPU
// oracle's ref_geom.
RefGeomF ref_geom(const double* P, double fx, double fy, double cx, double cy) {
  const double K[9] = {fx, 0, cx, 0, fy, cy, 0, 0, 1};
  const double Ki[9] = {1.0 / fx, 0, -cx / fx, 0, 1.0 / fy, -cy / fy, 0, 0, 1};
  double R[9], t[3], RKi[9], M[9];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) R[3 * i + j] = P[4 * i + j];
    t[i] = P[4 * i + 3];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) RKi[3 * i + j] = (R[3 * i + 0] * Ki[j] + R[3 * i + 1] * Ki[3 + j]) + R[3 * i + 2] * Ki[6 + j];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[3 * i + j] = (K[3 * i + 0] * RKi[j] + K[3 * i + 1] * RKi[3 + j]) + K[3 * i + 2] * RKi[6 + j];
  RefGeomF g;
  for (int i = 0; i < 9; ++i) g.M[i] = (float)M[i];
  for (int i = 0; i < 3; ++i) {
    g.b[i] = (float)((K[3 * i + 0] * t[0] + K[3 * i + 1] * t[1]) + K[3 * i + 2] * t[2]);
    g.c[i] = (float)(-((R[0 + i] * t[0] + R[3 + i] * t[1]) + R[6 + i] * t[2]));
  }
  return g;
}

}  // namespace

struct lsdg_depthmap {
  int w = 0, h = 0;
  lsdg_intrinsics intr{};
  FrameSet key, next;      // level-0 frames with gradients: current keyframe, next keyframe
  void* arena = nullptr;   // state A, state B, references, propagation keys
  DepthPlanes cur{}, alt{};
  float* refs = nullptr;
  uint8_t* refs_u8 = nullptr;  // staging of 8-bit reference frames (lsdg_depth_update_u8)
  unsigned long long* keys = nullptr;
  int* work = nullptr;      // observe work list: the keyframe pixels that search (one per pixel at most)
  int* counters = nullptr;  // [0] work list length, [1] next entry
  bool has_key = false;
};

bool depth_key_planes(const lsdg_depthmap* dm, const float** idepth, const float** var, const float** image,
                      int* w, int* h, lsdg_intrinsics* K) {
  if (!dm || !dm->has_key) return false;
  *K = dm->intr;
  *idepth = dm->cur.sm;
  *var = dm->cur.vsm;
  *image = dm->key.h_frames[0].plane[0];
  *w = dm->w;
  *h = dm->h;
  return true;
}

static DepthPlanes carve_planes(char*& p, size_t n) {
  DepthPlanes s;
  s.d = (float*)p; p += n * 4;
  s.v = (float*)p; p += n * 4;
  s.sm = (float*)p; p += n * 4;
  s.vsm = (float*)p; p += n * 4;
  s.val = (int*)p; p += n * 4;
  s.bl = (int*)p; p += n * 4;
  return s;
}

static void depth_free(lsdg_depthmap* dm) {
  frameset_free(dm->key);
  frameset_free(dm->next);
  if (dm->arena) cudaFree(dm->arena);
  delete dm;
}

static dim3 pixel_grid(int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); }

static lsdg_status enqueue_regularize(lsdg_ctx* ctx, lsdg_depthmap* dm) {
  const lsdg_params& p = ctx->params;
  RegArgs A;
  A.w = dm->w;
  A.h = dm->h;
  A.radius = p.reg_radius;
  A.min_support = p.reg_min_support;
  A.fill_min_support = p.fill_min_support;
  A.chi2 = p.reg_chi2;
  A.fill_var_factor = p.fill_var_factor;
  A.st = dm->cur;
  depth_regularize_kernel<<<pixel_grid(dm->w, dm->h), 256, 0, ctx->stream>>>(A);
  const int n = dm->w * dm->h;
  depth_commit_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(dm->cur, n);
  ctx->launches += 2;
  CK(ctx, cudaGetLastError());
  return LSDG_OK;
}

extern "C" {

lsdg_status lsdg_depth_create(lsdg_ctx* ctx, int width, int height, const lsdg_intrinsics* intr, lsdg_depthmap** out) {
  if (!ctx || !intr || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  *out = nullptr;
  if (width < 8 || height < 8 || !(intr->fx > 0) || !(intr->fy > 0))
    return ctx_fail(ctx, LSDG_INVALID_ARG, "depth map needs at least 8x8 pixels and positive focal lengths");
  CK(ctx, cudaSetDevice(ctx->device));
  lsdg_depthmap* dm = new (std::nothrow) lsdg_depthmap();
  if (!dm) return LSDG_OUT_OF_MEMORY;
  dm->w = width;
  dm->h = height;
  dm->intr = *intr;
  const bool nodepth = false;
  lsdg_status st = frameset_alloc(ctx, dm->key, 1, &width, &height, intr, &nodepth, 1, true);
  if (st == LSDG_OK) st = frameset_alloc(ctx, dm->next, 1, &width, &height, intr, &nodepth, 1, true);
  if (st != LSDG_OK) {
    depth_free(dm);
    return st;
  }
  const size_t n = (size_t)width * height;
  const size_t bytes = 2 * 6 * n * 4 + (size_t)LSDG_MAX_REFS * n * 5 + n * 8 + n * 4 + 4096;
  cudaError_t e = cudaMalloc(&dm->arena, bytes);
  if (e != cudaSuccess) {
    depth_free(dm);
    return ctx_cuda(ctx, e, "cudaMalloc(depth map)");
  }
  char* p = (char*)dm->arena;
  dm->cur = carve_planes(p, n);
  dm->alt = carve_planes(p, n);
  dm->refs = (float*)p;
  p += (size_t)LSDG_MAX_REFS * n * 4;
  p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
  dm->refs_u8 = (uint8_t*)p;
  p += (size_t)LSDG_MAX_REFS * n;
  p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
  dm->keys = (unsigned long long*)p;
  p += n * 8;
  dm->work = (int*)p;
  p += n * 4;
  p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
  dm->counters = (int*)p;
  *out = dm;
  return LSDG_OK;
}

lsdg_status lsdg_depth_destroy(lsdg_ctx* ctx, lsdg_depthmap* dm) {
  if (!ctx || !dm) return LSDG_INVALID_ARG;
  cudaStreamSynchronize(ctx->stream);
  depth_free(dm);
  return LSDG_OK;
}

lsdg_status lsdg_depth_set_keyframe(lsdg_ctx* ctx, lsdg_depthmap* dm, const float* image, const float* idepth,
                                    const float* var) {
  if (!ctx || !dm || !image || !idepth || !var) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const size_t n = (size_t)dm->w * dm->h;
  CK(ctx, cudaMemcpyAsync(dm->key.h_frames[0].plane[0], image, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  ctx->launches += launch_frame_pyramid(dm->key.d_frames, 1, 1, dm->key.max_pix, dm->key.max_h, true, ctx->stream);
  CK(ctx, cudaMemcpyAsync(dm->cur.d, idepth, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  CK(ctx, cudaMemcpyAsync(dm->cur.v, var, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  depth_init_kernel<<<(int)((n + 255) / 256), 256, 0, ctx->stream>>>(dm->cur, (int)n, ctx->params.validity_init);
  ctx->launches += 1;
  CK(ctx, cudaGetLastError());
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  dm->has_key = true;
  return LSDG_OK;
}

lsdg_status lsdg_depth_load_refs(lsdg_ctx* ctx, lsdg_depthmap* dm, int n_refs, const float* ref_images) {
  if (!ctx || !dm || !ref_images) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (n_refs < 1 || n_refs > LSDG_MAX_REFS) return ctx_fail(ctx, LSDG_INVALID_ARG, "n_refs must be in 1..%d", LSDG_MAX_REFS);
  const size_t n = (size_t)dm->w * dm->h;
  CK(ctx, cudaMemcpyAsync(dm->refs, ref_images, n * 4 * n_refs, cudaMemcpyHostToDevice, ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_depth_update_loaded(lsdg_ctx* ctx, lsdg_depthmap* dm, int n_refs, const double* key_to_ref,
                                     int regularize) {
  if (!ctx || !dm || !key_to_ref) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!dm->has_key) return ctx_fail(ctx, LSDG_INVALID_ARG, "set the keyframe first");
  if (n_refs < 1 || n_refs > LSDG_MAX_REFS) return ctx_fail(ctx, LSDG_INVALID_ARG, "n_refs must be in 1..%d", LSDG_MAX_REFS);
  const lsdg_params& p = ctx->params;
  ObserveArgs A;
  std::memset(&A, 0, sizeof(A));
  A.w = dm->w;
  A.h = dm->h;
  A.fx = dm->intr.fx;
  A.fy = dm->intr.fy;
  A.cx = dm->intr.cx;
  A.cy = dm->intr.cy;
  A.key = dm->key.h_frames[0].pyr[0];
  A.refs = dm->refs;
  A.n_refs = n_refs;
  for (int r = 0; r < n_refs; ++r)
    A.geom[r] = ref_geom(key_to_ref + 12 * r, dm->intr.fx, dm->intr.fy, dm->intr.cx, dm->intr.cy);
  A.st = dm->cur;
  A.min_grad = p.min_grad;
  A.min_grad_along_epl2 = p.min_grad_along_epl2;
  A.min_epl_length = p.min_epl_length;
  A.min_idepth = p.min_idepth;
  A.max_idepth = p.max_idepth;
  A.search_sigmas = p.search_sigmas;
  A.min_search_len = p.min_search_len;
  A.max_search_len = p.max_search_len;
  A.max_ssd = p.max_ssd;
  A.unique_ratio = p.unique_ratio;
  A.epipolar_var = p.epipolar_var;
  A.image_var = p.image_var;
  A.fuse_chi2 = p.fuse_chi2;
  A.validity_init = p.validity_init;
  A.validity_max = p.validity_max;
  A.validity_penalty = p.validity_penalty;
  A.blacklist_limit = p.blacklist_limit;
  // the pixels that search, then a persistent grid that deals them out 32 at a time
  const int npix = dm->w * dm->h;
  CK(ctx, cudaMemsetAsync(dm->counters, 0, 2 * sizeof(int), ctx->stream));
  depth_worklist_kernel<<<(npix + 255) / 256, 256, 0, ctx->stream>>>(A.key, dm->w, dm->h, p.min_grad, dm->work,
                                                                       dm->counters);
  // Lanes per listed pixel: 4 (a group shares each epipolar search; measured fastest of 1, 2, 4, 8 at
  // 640x480); LSDG_OBSERVE_GROUP=1|2|4|8 pins another form (used to profile them side by side; results
  // are the same bit for bit).
  static const int group = [] {
    const char* e = std::getenv("LSDG_OBSERVE_GROUP");
    const int g = e ? std::atoi(e) : 4;
    return (g == 1 || g == 2 || g == 4 || g == 8) ? g : 4;
  }();
  // resident CTAs of the observe kernel per SM (a property of the kernel on this architecture)
  auto occupancy = [](const void* k) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, 128, 0) != cudaSuccess) {
      cudaGetLastError();
      b = 4;
    }
    return b > 0 ? b : 1;
  };
  static const int per_sm1 = occupancy((const void*)depth_observe_kernel);
  static const int per_sm4 = occupancy((const void*)depth_observe_split_kernel<4>);
  static const int per_sm8 = occupancy((const void*)depth_observe_split_kernel<8>);
  static const int per_sm2 = occupancy((const void*)depth_observe_split_kernel<2>);
  const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
  if (group == 1) depth_observe_kernel<<<per_sm1 * sms, 128, 0, ctx->stream>>>(A, dm->work, dm->counters);
  else if (group == 2) depth_observe_split_kernel<2><<<per_sm2 * sms, 128, 0, ctx->stream>>>(A, dm->work, dm->counters);
  else if (group == 4) depth_observe_split_kernel<4><<<per_sm4 * sms, 128, 0, ctx->stream>>>(A, dm->work, dm->counters);
  else depth_observe_split_kernel<8><<<per_sm8 * sms, 128, 0, ctx->stream>>>(A, dm->work, dm->counters);
  ctx->launches += 2;
  CK(ctx, cudaGetLastError());
  if (regularize) return enqueue_regularize(ctx, dm);
  return LSDG_OK;
}

lsdg_status lsdg_depth_update(lsdg_ctx* ctx, lsdg_depthmap* dm, int n_refs, const float* ref_images,
                              const double* key_to_ref, int regularize) {
  lsdg_status st = lsdg_depth_load_refs(ctx, dm, n_refs, ref_images);
  if (st != LSDG_OK) return st;
  st = lsdg_depth_update_loaded(ctx, dm, n_refs, key_to_ref, regularize);
  if (st != LSDG_OK) return st;
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_depth_update_u8(lsdg_ctx* ctx, lsdg_depthmap* dm, int n_refs, const uint8_t* ref_images,
                                 const double* key_to_ref, int regularize) {
  if (!ctx || !dm || !ref_images) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (n_refs < 1 || n_refs > LSDG_MAX_REFS) return ctx_fail(ctx, LSDG_INVALID_ARG, "n_refs must be in 1..%d", LSDG_MAX_REFS);
  const size_t n = (size_t)dm->w * dm->h * n_refs;
  CK(ctx, cudaMemcpyAsync(dm->refs_u8, ref_images, n, cudaMemcpyHostToDevice, ctx->stream));
  launch_u8_to_plane(dm->refs_u8, dm->refs, (int)n, ctx->stream);
  ctx->launches += 1;
  CK(ctx, cudaGetLastError());
  lsdg_status st = lsdg_depth_update_loaded(ctx, dm, n_refs, key_to_ref, regularize);
  if (st != LSDG_OK) return st;
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_depth_regularize(lsdg_ctx* ctx, lsdg_depthmap* dm) {
  if (!ctx || !dm) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  lsdg_status st = enqueue_regularize(ctx, dm);
  if (st != LSDG_OK) return st;
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_depth_create_keyframe(lsdg_ctx* ctx, lsdg_depthmap* dm, const float* new_image,
                                       const double key_to_new[12], int regularize) {
  if (!ctx || !dm || !new_image || !key_to_new) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!dm->has_key) return ctx_fail(ctx, LSDG_INVALID_ARG, "set the keyframe first");
  const size_t n = (size_t)dm->w * dm->h;
  CK(ctx, cudaMemcpyAsync(dm->next.h_frames[0].plane[0], new_image, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  ctx->launches += launch_frame_pyramid(dm->next.d_frames, 1, 1, dm->next.max_pix, dm->next.max_h, true, ctx->stream);
  const lsdg_params& p = ctx->params;
  PropArgs A;
  A.w = dm->w;
  A.h = dm->h;
  A.fx = dm->intr.fx;
  A.fy = dm->intr.fy;
  A.cx = dm->intr.cx;
  A.cy = dm->intr.cy;
  A.fxi = (float)(1.0 / dm->intr.fx);
  A.fyi = (float)(1.0 / dm->intr.fy);
  A.min_z = p.min_z;
  A.max_photo_diff = p.propagate_max_photo_diff;
  A.prediction_var = p.prediction_var;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) A.R[3 * i + j] = (float)key_to_new[4 * i + j];
    A.t[i] = (float)key_to_new[4 * i + 3];
  }
  A.Iold = dm->key.h_frames[0].plane[0];
  A.Inew = dm->next.h_frames[0].plane[0];
  A.src = dm->cur;
  A.dst = dm->alt;
  A.key = dm->keys;
  CK(ctx, cudaMemsetAsync(dm->keys, 0xff, n * 8, ctx->stream));
  const int blocks = (int)((n + 255) / 256);
  depth_prop_key_kernel<<<blocks, 256, 0, ctx->stream>>>(A);
  depth_prop_write_kernel<<<blocks, 256, 0, ctx->stream>>>(A);
  ctx->launches += 2;
  CK(ctx, cudaGetLastError());
  std::swap(dm->cur, dm->alt);
  std::swap(dm->key, dm->next);
  if (regularize) {
    lsdg_status st = enqueue_regularize(ctx, dm);
    if (st != LSDG_OK) return st;
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_depth_get(lsdg_ctx* ctx, lsdg_depthmap* dm, float* idepth, float* var, float* sm, float* vsm,
                           int32_t* validity, int32_t* blacklist) {
  if (!ctx || !dm) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  const size_t n = (size_t)dm->w * dm->h * 4;
  if (idepth) CK(ctx, cudaMemcpyAsync(idepth, dm->cur.d, n, cudaMemcpyDeviceToHost, ctx->stream));
  if (var) CK(ctx, cudaMemcpyAsync(var, dm->cur.v, n, cudaMemcpyDeviceToHost, ctx->stream));
  if (sm) CK(ctx, cudaMemcpyAsync(sm, dm->cur.sm, n, cudaMemcpyDeviceToHost, ctx->stream));
  if (vsm) CK(ctx, cudaMemcpyAsync(vsm, dm->cur.vsm, n, cudaMemcpyDeviceToHost, ctx->stream));
  if (validity) CK(ctx, cudaMemcpyAsync(validity, dm->cur.val, n, cudaMemcpyDeviceToHost, ctx->stream));
  if (blacklist) CK(ctx, cudaMemcpyAsync(blacklist, dm->cur.bl, n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

}  // extern "C"

// ============================================================================================
// propagateDepth without allocation (lsdg_depth_propagate_noalloc)
// ============================================================================================
// Some callers cannot call cudaMalloc at the moment they need a keyframe change: an application
// that reserves all device memory up front and forbids allocation in its real-time mapping thread,
// one that runs the mapping step inside its own stream capture (allocation is not capturable), or
// one that cannot afford the device-wide synchronisation cudaMalloc may imply.  For them the z-buffer
// of the propagation -- its only scratch -- lives in this file-scope device array instead of a
// context.  Every GPU that loads the library holds it until the process exits.

constexpr long kNoAllocMaxPixels = 1280L * 960L;  // largest keyframe: 1,228,800 pixels (9.8 MB of keys)

static __device__ __align__(256) unsigned long long g_noalloc_zbuffer[kNoAllocMaxPixels];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the z-buffer on the current device, looked up once per device (the name is a
// host-side stand-in, not a device address).
lsdg_status noalloc_zbuffer(unsigned long long** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return LSDG_CUDA_ERROR;
  }
  if (dev < 0 || dev >= kNoAllocMaxDevices) return LSDG_NOT_SUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_zbuffer);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return LSDG_CUDA_ERROR;
    }
    g_noalloc_ptr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return LSDG_OK;
}
}  // namespace

extern "C" lsdg_status lsdg_depth_propagate_noalloc(void* stream, int width, int height, const lsdg_intrinsics* intr,
                                                   const lsdg_params* params, const double old_to_new[12],
                                                   const float* old_image, const float* new_image,
                                                   const float* old_idepth, const float* old_var,
                                                   const int32_t* old_validity, float* new_idepth, float* new_var,
                                                   float* new_idepth_smoothed, float* new_var_smoothed,
                                                   int32_t* new_validity, int32_t* new_blacklist) {
  if (!intr || !params || !old_to_new || !old_image || !new_image || !old_idepth || !old_var || !old_validity ||
      !new_idepth || !new_var || !new_idepth_smoothed || !new_var_smoothed || !new_validity || !new_blacklist)
    return LSDG_INVALID_ARG;
  if (width < 1 || height < 1 || (long)width * height > kNoAllocMaxPixels) return LSDG_INVALID_ARG;
  if (!(intr->fx > 0) || !(intr->fy > 0)) return LSDG_INVALID_ARG;
  // an error someone else left pending stays theirs: the final cudaGetLastError then reports this
  // call's launches only
  if (cudaPeekAtLastError() != cudaSuccess) return LSDG_CUDA_ERROR;
  unsigned long long* keys = nullptr;
  const lsdg_status st = noalloc_zbuffer(&keys);
  if (st != LSDG_OK) return st;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  PropArgs A;
  A.w = width;
  A.h = height;
  A.fx = intr->fx;
  A.fy = intr->fy;
  A.cx = intr->cx;
  A.cy = intr->cy;
  A.fxi = (float)(1.0 / intr->fx);
  A.fyi = (float)(1.0 / intr->fy);
  A.min_z = params->min_z;
  A.max_photo_diff = params->propagate_max_photo_diff;
  A.prediction_var = params->prediction_var;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) A.R[3 * i + j] = (float)old_to_new[4 * i + j];
    A.t[i] = (float)old_to_new[4 * i + 3];
  }
  A.Iold = old_image;
  A.Inew = new_image;
  A.src = DepthPlanes{const_cast<float*>(old_idepth), const_cast<float*>(old_var), nullptr, nullptr,
                      const_cast<int*>(old_validity), nullptr};  // propagation reads idepth, var, validity
  A.dst = DepthPlanes{new_idepth, new_var, new_idepth_smoothed, new_var_smoothed, new_validity, new_blacklist};
  A.key = keys;
  const size_t n = (size_t)width * height;
  // the array keeps the previous call's keys: every call starts from an empty z-buffer
  if (cudaMemsetAsync(keys, 0xff, n * sizeof(unsigned long long), s) != cudaSuccess) {
    cudaGetLastError();
    return LSDG_CUDA_ERROR;
  }
  const int blocks = (int)((n + 255) / 256);
  depth_prop_key_kernel<<<blocks, 256, 0, s>>>(A);
  depth_prop_write_kernel<<<blocks, 256, 0, s>>>(A);
  return cudaGetLastError() == cudaSuccess ? LSDG_OK : LSDG_CUDA_ERROR;
}

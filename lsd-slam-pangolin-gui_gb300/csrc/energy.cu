// energy.cu -- a10 of the hot path: the differentiable photometric energy of a keyframe against a
// frame, its adjoint with respect to the pose twist and every keyframe inverse depth, and the
// per-point photometric inverse-depth refinement that the adjoint drives.  There is no upstream
// counterpart; the residual model is the tracker's (same points, Catmull-Rom sampling of the frame
// level, Huber norm of the variance-normalised residual), so the pose gradient is twice the
// J^T W r of calculateWarpUpdate at the same pose.
//
// GB300 design:
//   forward / backward  one thread per point, grid-stride; nothing is stored per residual: the
//              backward recomputes each residual from (pose, inverse depth) and writes only the
//              per-point gradient (4 B/point, coalesced).  The scalar sums (E and the 6/7 pose
//              gradients) are per-thread Kahan pairs, merged by warp shuffles, then across warps in
//              a fixed order, then across CTAs by the last CTA to finish (a ticket counter; the
//              merge order is the CTA index, so the result does not depend on scheduling).
//   refine     8 lanes per point, lane g owning frames g and g + 8: every damped Newton step
//              re-evaluates the point in all its frames at once and sums the per-frame terms with
//              a 3-level xor shuffle tree, so all 8 lanes hold identical sums and take the same
//              accept/reject decision.  The frames (8 x 1.2 MB at 640x480) stay L2-resident across
//              the 50 steps; each point's state lives in registers for the whole refinement, one
//              launch in total.
// Built with -fmad=false: per-point values are bit-identical to the float CPU oracle, which spells
// out the same operations (oracle/lsdo_energy.cpp).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>

#include "lsdg_host.h"

using namespace lsdg;

#define CK(ctx, expr)                                \
  do {                                               \
    lsdg_status _s = ctx_cuda((ctx), (expr), #expr); \
    if (_s != LSDG_OK) return _s;                    \
  } while (0)

namespace {

constexpr int kEThreads = 256;
constexpr int kMaxCtas = 1216;     // 8 CTAs per SM on 152 SMs; the grid only depends on n
constexpr int kPartStride = 20;    // per-CTA partial: 8 sums, 8 compensations, count, pad
constexpr int kOut = 16;           // doubles of the device result record

// One observation of point (qx, qy, rho) in frame level `img`; same operations as the oracle's
// observe() (oracle/lsdo_energy.cpp).  margin_box: the first-pass participation test, else only
// the sampling box [1, w - 2) x [1, h - 2).
struct Obs {
  float r, rho_h, wgt, a0, a1, a2, Xp, Yp, Zp, Rpx, Rpy, Rpz, z;
};

struct Cam {
  const float* img;
  int w, h;
  float fx, fy, cx, cy;
};

struct Huber {
  float minz, margin, delta;
};

__device__ __forceinline__ bool observe(float qx, float qy, float rho, float Ik, float s2, const Cam& c,
                                        const float* M, const Huber& hp, bool margin_box, Obs& o) {
  if (!(rho > 0.f)) return false;
  const float z = 1.0f / rho;
  const float X = qx * z, Y = qy * z, Z = z;
  const float Rpx = (M[0] * X + M[1] * Y) + M[2] * Z;
  const float Rpy = (M[4] * X + M[5] * Y) + M[6] * Z;
  const float Rpz = (M[8] * X + M[9] * Y) + M[10] * Z;
  const float Xp = Rpx + M[3], Yp = Rpy + M[7], Zp = Rpz + M[11];
  if (!(Zp > hp.minz)) return false;
  const float iz = 1.0f / Zp;
  const float u = c.fx * (Xp * iz) + c.cx;
  const float v = c.fy * (Yp * iz) + c.cy;
  if (margin_box) {
    const float m = hp.margin;
    if (!(u >= m && v >= m && u < (float)(c.w - 1) - m && v < (float)(c.h - 1) - m)) return false;
  } else if (!(u >= 1.f && v >= 1.f && u < (float)(c.w - 2) && v < (float)(c.h - 2))) {
    return false;
  }
  const int ix = (int)u, iy = (int)v;
  const float ax = u - (float)ix, ay = v - (float)iy;
  float wx[4], dxw[4], wy[4], dyw[4];
  catmull_rom(ax, wx, dxw);
  catmull_rom(ay, wy, dyw);
  float rI[4], rD[4];
  const float* q = c.img + (size_t)(iy - 1) * c.w + (ix - 1);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float i0 = __ldg(q), i1 = __ldg(q + 1), i2 = __ldg(q + 2), i3 = __ldg(q + 3);
    rI[j] = ((wx[0] * i0 + wx[1] * i1) + wx[2] * i2) + wx[3] * i3;
    rD[j] = ((dxw[0] * i0 + dxw[1] * i1) + dxw[2] * i2) + dxw[3] * i3;
    q += c.w;
  }
  const float In = ((wy[0] * rI[0] + wy[1] * rI[1]) + wy[2] * rI[2]) + wy[3] * rI[3];
  const float Gx = ((wy[0] * rD[0] + wy[1] * rD[1]) + wy[2] * rD[2]) + wy[3] * rD[3];
  const float Gy = ((dyw[0] * rI[0] + dyw[1] * rI[1]) + dyw[2] * rI[2]) + dyw[3] * rI[3];
  o.r = In - Ik;
  o.a0 = (Gx * c.fx) * iz;
  o.a1 = (Gy * c.fy) * iz;
  o.a2 = -((o.a0 * Xp + o.a1 * Yp) * iz);
  const float e2 = (o.r * o.r) / s2;
  const float ae = sqrtf(e2);
  float wh;
  if (ae <= hp.delta) { wh = 1.f; o.rho_h = e2; }
  else { wh = hp.delta / ae; o.rho_h = hp.delta * (2.f * ae - hp.delta); }
  o.wgt = wh / s2;
  o.Xp = Xp; o.Yp = Yp; o.Zp = Zp;
  o.Rpx = Rpx; o.Rpy = Rpy; o.Rpz = Rpz;
  o.z = z;
  return true;
}

__device__ __forceinline__ float drho_of(const Obs& o) {
  return -(((o.a0 * o.Rpx + o.a1 * o.Rpy) + o.a2 * o.Rpz) * o.z);
}

// ------------------------------------------------------------------------------------------
// Deterministic reduction of K compensated sums (+ one integer count) over the whole grid.
// ------------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void grid_reduce(float (&s)[K], float (&c)[K], int cnt, float* part, unsigned* ticket,
                                            double* out) {
  __shared__ float ws[kEThreads / 32][K], wc[kEThreads / 32][K];
  __shared__ int wn[kEThreads / 32];
  __shared__ int is_last;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  constexpr int NW = kEThreads / 32;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
    for (int i = 0; i < K; ++i)
      kmerge(s[i], c[i], __shfl_xor_sync(0xffffffffu, s[i], o), __shfl_xor_sync(0xffffffffu, c[i], o));
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < K; ++i) { ws[wid][i] = s[i]; wc[wid][i] = c[i]; }
    wn[wid] = cnt;
  }
  __syncthreads();
  if (wid == 0) {
    if (lane < K) {
      float a = 0.f, b = 0.f;
      for (int w = 0; w < NW; ++w) kmerge(a, b, ws[w][lane], wc[w][lane]);
      part[(size_t)blockIdx.x * kPartStride + lane] = a;
      part[(size_t)blockIdx.x * kPartStride + 8 + lane] = b;
    } else if (lane == 16) {
      int v = 0;
      for (int w = 0; w < NW; ++w) v += wn[w];
      reinterpret_cast<int*>(part)[(size_t)blockIdx.x * kPartStride + 16] = v;
    }
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) is_last = atomicAdd(ticket, 1u) == gridDim.x - 1 ? 1 : 0;
  __syncthreads();
  if (is_last && wid == 0) {
    __threadfence();
    if (lane < K) {
      float a = 0.f, b = 0.f;
      for (unsigned k = 0; k < gridDim.x; ++k)
        kmerge(a, b, __ldcg(&part[(size_t)k * kPartStride + lane]), __ldcg(&part[(size_t)k * kPartStride + 8 + lane]));
      out[lane] = (double)a - (double)b;
    }
    long long v = 0;
    for (unsigned k = lane; k < gridDim.x; k += 32)
      v += __ldcg(&reinterpret_cast<const int*>(part)[(size_t)k * kPartStride + 16]);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) {
      out[8] = (double)v;
      *ticket = 0u;  // ready for the next launch (stream order)
    }
  }
}

// ------------------------------------------------------------------------------------------
// Forward / backward
// ------------------------------------------------------------------------------------------
struct EnergyArgs {
  const float4* ray;   // {qx, qy, I_keyframe, var} per point
  const float* rho;
  const float* sig2;   // per-point residual variance, or nullptr
  int n;
  Cam cam;
  float M[12];
  Huber hp;
  float pvar;
  float gscale;        // dL/dE (backward; scales the per-point gradients)
  float* grho;         // backward: dL/drho per point
  float* part;
  unsigned* ticket;
  double* out;         // [0] E, [1..7] dE/dxi, [8] points taking part
};

template <bool BWD, int DOF>
__global__ void __launch_bounds__(kEThreads) energy_kernel(const EnergyArgs a) {
  constexpr int K = BWD ? 1 + DOF : 1;
  float s[K], c[K];
#pragma unroll
  for (int i = 0; i < K; ++i) { s[i] = 0.f; c[i] = 0.f; }
  int cnt = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.n; k += gridDim.x * blockDim.x) {
    const float4 ry = __ldg(&a.ray[k]);
    const float rk = __ldg(&a.rho[k]);
    const float s2 = a.sig2 ? __ldg(&a.sig2[k]) : a.pvar;
    Obs o;
    if (!observe(ry.x, ry.y, rk, ry.z, s2, a.cam, a.M, a.hp, true, o)) {
      if (BWD) a.grho[k] = 0.f;
      continue;
    }
    ++cnt;
    kadd(s[0], c[0], o.rho_h);
    if (BWD) {
      const float cc = (2.f * o.wgt) * o.r;  // dh/dr
      float J[7];
      J[0] = o.a0; J[1] = o.a1; J[2] = o.a2;
      J[3] = o.Yp * o.a2 - o.Zp * o.a1;
      J[4] = o.Zp * o.a0 - o.Xp * o.a2;
      J[5] = o.Xp * o.a1 - o.Yp * o.a0;
      J[6] = (o.a0 * o.Xp + o.a1 * o.Yp) + o.a2 * o.Zp;
#pragma unroll
      for (int i = 0; i < DOF; ++i)
        if (i + 1 < K) kadd(s[i + 1], c[i + 1], cc * J[i]);
      a.grho[k] = a.gscale * (cc * drho_of(o));
    }
  }
  grid_reduce<K>(s, c, cnt, a.part, a.ticket, a.out);
}

// ------------------------------------------------------------------------------------------
// Refinement: 8 lanes per point
// ------------------------------------------------------------------------------------------
struct RefineFrame {
  const float* img;
  float M[12];
};

struct RefineArgs {
  const float4* ray;
  float* rho;
  const float* sig2;
  int n, nf, steps;
  int w, h;
  float fx, fy, cx, cy;
  Huber hp;
  float pvar, rho_lo, rho_hi, lam0, lam_up, lam_down, prior_w;
  float* part;
  unsigned* ticket;
  double* out;   // [0] E before, [1] E after, [8] points refined
  const RefineFrame* fr;  // nf entries (device)
};

// Slot sums of this lane's frames (g, g + 8) at rho; `first`: the margin test decides which frames
// see the point (bits of *mask); else only the frames in mask, each of which must stay inside the
// sampling box (ok).
__device__ __forceinline__ void refine_terms(const RefineArgs& a, int g, float qx, float qy, float Ik, float s2,
                                             float rho, bool first, unsigned& mask, float& e, float& gg, float& hh,
                                             bool& ok) {
  e = 0.f; gg = 0.f; hh = 0.f;
  ok = true;
  Cam cam{nullptr, a.w, a.h, a.fx, a.fy, a.cx, a.cy};
#pragma unroll 1
  for (int j = g; j < a.nf; j += 8) {
    if (!first && !((mask >> j) & 1u)) continue;
    cam.img = a.fr[j].img;
    Obs o;
    if (!observe(qx, qy, rho, Ik, s2, cam, a.fr[j].M, a.hp, first, o)) {
      if (!first) ok = false;
      continue;
    }
    if (first) mask |= 1u << j;
    const float jr = drho_of(o);
    const float c = 2.f * o.wgt;
    e = e + o.rho_h;
    gg = gg + (c * o.r) * jr;
    hh = hh + (c * jr) * jr;
  }
}

__device__ __forceinline__ float group_sum8(float v) {
  v = v + __shfl_xor_sync(0xffffffffu, v, 4);
  v = v + __shfl_xor_sync(0xffffffffu, v, 2);
  v = v + __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

__global__ void __launch_bounds__(kEThreads) energy_refine_kernel(const RefineArgs a) {
  constexpr int G = kEThreads / 8;  // points per CTA per sweep
  const int g = threadIdx.x & 7;
  float s[2] = {0.f, 0.f}, c[2] = {0.f, 0.f};
  int refined = 0;
  for (int base = blockIdx.x * G; base < a.n; base += gridDim.x * G) {
    const int k = base + (threadIdx.x >> 3);
    const bool inb = k < a.n;
    const float4 ry = inb ? __ldg(&a.ray[k]) : make_float4(0.f, 0.f, 0.f, 1.f);
    float rho = inb ? a.rho[k] : 0.f;
    const float rho0 = rho;
    const float s2 = (inb && a.sig2) ? __ldg(&a.sig2[k]) : a.pvar;
    const float pk = a.prior_w / ry.w;
    unsigned mask = 0u;
    float e, gg, hh;
    bool ok;
    refine_terms(a, g, ry.x, ry.y, ry.z, s2, rho, true, mask, e, gg, hh, ok);
    unsigned gm = mask;
    gm |= __shfl_xor_sync(0xffffffffu, gm, 4);
    gm |= __shfl_xor_sync(0xffffffffu, gm, 2);
    gm |= __shfl_xor_sync(0xffffffffu, gm, 1);
    const float pe0 = 0.f * pk;  // (pk * 0) * 0: the prior at its centre
    float E = group_sum8(e) + (pe0 * 0.f);
    float Gs = group_sum8(gg) + (2.f * pk) * 0.f;
    float H = group_sum8(hh) + 2.f * pk;
    const bool live = inb && gm != 0u && H > 0.f;
    if (g == 0 && inb) kadd(s[0], c[0], E);
    float lam = a.lam0;
#pragma unroll 1
    for (int st = 0; st < a.steps; ++st) {
      float rt = rho;
      if (live) {
        const float d = -(Gs / (H * (1.f + lam)));
        rt = rho + d;
        rt = rt < a.rho_lo ? a.rho_lo : (rt > a.rho_hi ? a.rho_hi : rt);
      }
      float et, gt, ht;
      bool okt;
      unsigned m2 = mask;
      refine_terms(a, g, ry.x, ry.y, ry.z, s2, rt, false, m2, et, gt, ht, okt);
      const unsigned gbit = 1u << ((threadIdx.x & 31) >> 3);  // this point's bit among the warp's 4
      const bool okg = (__reduce_or_sync(0xffffffffu, okt ? 0u : gbit) & gbit) == 0u;
      const float dq = rt - rho0;
      const float Et = group_sum8(et) + (pk * dq) * dq;
      const float Gt = group_sum8(gt) + (2.f * pk) * dq;
      const float Ht = group_sum8(ht) + 2.f * pk;
      const bool better = Et < E;
      if (live && okg && better && Ht > 0.f) {
        rho = rt;
        E = Et;
        Gs = Gt;
        H = Ht;
        lam = lam * a.lam_down;
      } else {
        lam = lam * a.lam_up;
      }
    }
    if (g == 0 && inb) {
      kadd(s[1], c[1], E);
      a.rho[k] = rho;
      if (live) ++refined;
    }
  }
  grid_reduce<2>(s, c, refined, a.part, a.ticket, a.out);
}

__global__ void energy_setup_kernel(const float4* __restrict__ pxyzi, const float* __restrict__ pvar,
                                    const int* __restrict__ ppix, const float* __restrict__ idepth, int n, int w,
                                    float cx, float cy, float fxi, float fyi, float4* ray, float* rho, float* rho_init) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int idx = ppix[k];
  const int x = idx % w, y = idx / w;
  ray[k] = make_float4(((float)x - cx) * fxi, ((float)y - cy) * fyi, pxyzi[k].w, pvar[k]);
  const float r = idepth[idx];
  rho[k] = r;
  rho_init[k] = r;
}

int grid_for(int n, int per_cta) {
  const int need = (n + per_cta - 1) / per_cta;
  return need < 1 ? 1 : (need > kMaxCtas ? kMaxCtas : need);
}

}  // namespace

struct lsdg_energy {
  int level = 0, n = 0, w = 0, h = 0;
  float fx = 0, fy = 0, cx = 0, cy = 0;
  float4* ray = nullptr;
  float* rho = nullptr;
  float* rho_init = nullptr;
  float* sig2 = nullptr;
  float* grho = nullptr;
  int* pix = nullptr;
  float* part = nullptr;
  unsigned* ticket = nullptr;
  double* out = nullptr;
  double* h_out = nullptr;
  RefineFrame* d_fr = nullptr;  // refine: frame table (LSDG_MAX_REFS entries)
  RefineFrame* h_fr = nullptr;  // pinned staging
  cudaEvent_t ev[6] = {};
  // saved by the forward (the autograd context)
  bool saved = false;
  const lsdg_frame* frame = nullptr;
  double pose[12] = {};
  int dof = 6;
  unsigned long long version = 0, saved_version = 0;
};

static void energy_free(lsdg_energy* e) {
  if (!e) return;
  cudaFree(e->ray);
  cudaFree(e->rho);
  cudaFree(e->rho_init);
  cudaFree(e->sig2);
  cudaFree(e->grho);
  cudaFree(e->pix);
  cudaFree(e->part);
  cudaFree(e->ticket);
  cudaFree(e->out);
  cudaFreeHost(e->h_out);
  cudaFree(e->d_fr);
  cudaFreeHost(e->h_fr);
  for (auto& ev : e->ev)
    if (ev) cudaEventDestroy(ev);
  delete e;
}

static Huber huber_of(const lsdg_params& p) { return Huber{p.min_z, p.border_margin, p.huber_delta}; }

static lsdg_status read_out(lsdg_ctx* ctx, lsdg_energy* e) {
  CK(ctx, cudaMemcpyAsync(e->h_out, e->out, sizeof(double) * kOut, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

extern "C" {

lsdg_status lsdg_energy_create(lsdg_ctx* ctx, const lsdg_frame* keyframe, int level, lsdg_energy** out) {
  if (!ctx || !keyframe || !out) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  *out = nullptr;
  const FrameDev& F = keyframe->fs.h_frames[0];
  if (!F.has_depth) return ctx_fail(ctx, LSDG_INVALID_ARG, "keyframe has no depth");
  if (level < 0 || level >= F.levels) return ctx_fail(ctx, LSDG_INVALID_ARG, "level out of range");
  if (!F.ppix[level]) return ctx_fail(ctx, LSDG_NOT_SUPPORTED, "keyframe keeps no pixel index (batch frame)");
  CK(ctx, cudaSetDevice(ctx->device));
  int n = 0;
  CK(ctx, cudaMemcpyAsync(ctx->h_small, F.pcount + level, 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  std::memcpy(&n, ctx->h_small, 4);
  lsdg_energy* e = new (std::nothrow) lsdg_energy();
  if (!e) return LSDG_OUT_OF_MEMORY;
  e->level = level;
  e->n = n;
  e->w = F.w >> level;
  e->h = F.h >> level;
  e->fx = F.fx[level];
  e->fy = F.fy[level];
  e->cx = F.cx[level];
  e->cy = F.cy[level];
  const size_t m = (size_t)(n > 0 ? n : 1);
  cudaError_t err = cudaMalloc(&e->ray, m * sizeof(float4));
  if (err == cudaSuccess) err = cudaMalloc(&e->rho, m * 4);
  if (err == cudaSuccess) err = cudaMalloc(&e->rho_init, m * 4);
  if (err == cudaSuccess) err = cudaMalloc(&e->grho, m * 4);
  if (err == cudaSuccess) err = cudaMalloc(&e->pix, m * 4);
  if (err == cudaSuccess) err = cudaMalloc(&e->part, (size_t)kMaxCtas * kPartStride * 4);
  if (err == cudaSuccess) err = cudaMalloc(&e->ticket, sizeof(unsigned));
  if (err == cudaSuccess) err = cudaMalloc(&e->out, sizeof(double) * kOut);
  if (err == cudaSuccess) err = cudaMallocHost(&e->h_out, sizeof(double) * kOut);
  if (err == cudaSuccess) err = cudaMalloc(&e->d_fr, sizeof(RefineFrame) * LSDG_MAX_REFS);
  if (err == cudaSuccess) err = cudaMallocHost(&e->h_fr, sizeof(RefineFrame) * LSDG_MAX_REFS);
  for (auto& ev : e->ev)
    if (err == cudaSuccess) err = cudaEventCreate(&ev);
  if (err == cudaSuccess) err = cudaMemsetAsync(e->ticket, 0, sizeof(unsigned), ctx->stream);
  if (err == cudaSuccess) err = cudaMemsetAsync(e->out, 0, sizeof(double) * kOut, ctx->stream);
  if (err == cudaSuccess && n > 0) {
    energy_setup_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(F.pxyzi[level], F.pvar[level], F.ppix[level],
                                                                  F.idepth[level], n, e->w, F.cx[level], F.cy[level],
                                                                  F.fxi[level], F.fyi[level], e->ray, e->rho,
                                                                  e->rho_init);
    err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaMemcpyAsync(e->pix, F.ppix[level], (size_t)n * 4, cudaMemcpyDeviceToDevice,
                                                  ctx->stream);
    ctx->launches += 1;
  }
  if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
  if (err != cudaSuccess) {
    energy_free(e);
    return ctx_cuda(ctx, err, "lsdg_energy_create");
  }
  *out = e;
  return LSDG_OK;
}

lsdg_status lsdg_energy_destroy(lsdg_ctx* ctx, lsdg_energy* e) {
  if (!ctx || !e) return LSDG_INVALID_ARG;
  cudaStreamSynchronize(ctx->stream);
  energy_free(e);
  return LSDG_OK;
}

lsdg_status lsdg_energy_size(lsdg_ctx* ctx, const lsdg_energy* e, int* n_points) {
  if (!ctx || !e || !n_points) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  *n_points = e->n;
  return LSDG_OK;
}

lsdg_status lsdg_energy_pixels(lsdg_ctx* ctx, const lsdg_energy* e, int32_t* pixels) {
  if (!ctx || !e || !pixels) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (e->n) CK(ctx, cudaMemcpyAsync(pixels, e->pix, (size_t)e->n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_energy_set_idepth(lsdg_ctx* ctx, lsdg_energy* e, const float* idepth) {
  if (!ctx || !e) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (e->n) {
    if (idepth)
      CK(ctx, cudaMemcpyAsync(e->rho, idepth, (size_t)e->n * 4, cudaMemcpyHostToDevice, ctx->stream));
    else
      CK(ctx, cudaMemcpyAsync(e->rho, e->rho_init, (size_t)e->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  ++e->version;
  return LSDG_OK;
}

lsdg_status lsdg_energy_get_idepth(lsdg_ctx* ctx, const lsdg_energy* e, float* idepth) {
  if (!ctx || !e || !idepth) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (e->n) CK(ctx, cudaMemcpyAsync(idepth, e->rho, (size_t)e->n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(ctx, cudaStreamSynchronize(ctx->stream));
  return LSDG_OK;
}

lsdg_status lsdg_energy_set_sigma2(lsdg_ctx* ctx, lsdg_energy* e, const float* sigma2) {
  if (!ctx || !e) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!sigma2) {
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(e->sig2);
    e->sig2 = nullptr;
  } else {
    for (int i = 0; i < e->n; ++i)
      if (!(sigma2[i] > 0)) return ctx_fail(ctx, LSDG_INVALID_ARG, "sigma2[%d] must be > 0", i);
    if (!e->sig2) CK(ctx, cudaMalloc(&e->sig2, (size_t)(e->n > 0 ? e->n : 1) * 4));
    if (e->n) CK(ctx, cudaMemcpyAsync(e->sig2, sigma2, (size_t)e->n * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
  }
  ++e->version;
  return LSDG_OK;
}

static lsdg_status check_frame(lsdg_ctx* ctx, const lsdg_energy* e, const lsdg_frame* f) {
  if (!f) return ctx_fail(ctx, LSDG_INVALID_ARG, "null frame");
  if (!f->has_image) return ctx_fail(ctx, LSDG_INVALID_ARG, "frame image not uploaded");
  const FrameDev& F = f->fs.h_frames[0];
  if ((F.w >> e->level) != e->w || (F.h >> e->level) != e->h || F.levels <= e->level)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "frame size differs from the keyframe's");
  return LSDG_OK;
}

static lsdg_status launch_energy(lsdg_ctx* ctx, lsdg_energy* e, bool bwd, double grad) {
  EnergyArgs a{};
  a.ray = e->ray;
  a.rho = e->rho;
  a.sig2 = e->sig2;
  a.n = e->n;
  const FrameDev& F = e->frame->fs.h_frames[0];
  a.cam = Cam{F.plane[e->level], e->w, e->h, e->fx, e->fy, e->cx, e->cy};
  for (int i = 0; i < 12; ++i) a.M[i] = (float)e->pose[i];
  a.hp = huber_of(ctx->params);
  a.pvar = ctx->params.photometric_variance;
  a.gscale = (float)grad;
  a.grho = e->grho;
  a.part = e->part;
  a.ticket = e->ticket;
  a.out = e->out;
  const int grid = grid_for(e->n, kEThreads);
  CK(ctx, cudaEventRecord(e->ev[bwd ? 2 : 0], ctx->stream));
  if (!bwd) energy_kernel<false, 6><<<grid, kEThreads, 0, ctx->stream>>>(a);
  else if (e->dof == 7) energy_kernel<true, 7><<<grid, kEThreads, 0, ctx->stream>>>(a);
  else energy_kernel<true, 6><<<grid, kEThreads, 0, ctx->stream>>>(a);
  CK(ctx, cudaGetLastError());
  CK(ctx, cudaEventRecord(e->ev[bwd ? 3 : 1], ctx->stream));
  ctx->launches += 1;
  return read_out(ctx, e);
}

lsdg_status lsdg_energy_forward(lsdg_ctx* ctx, lsdg_energy* e, const lsdg_frame* frame, const double ref_to_frame[12],
                                int dof, double* energy, int* n_active) {
  if (!ctx || !e || !ref_to_frame) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (dof != 6 && dof != 7) return ctx_fail(ctx, LSDG_INVALID_ARG, "dof must be 6 or 7");
  lsdg_status st = check_frame(ctx, e, frame);
  if (st != LSDG_OK) return st;
  e->frame = frame;
  std::memcpy(e->pose, ref_to_frame, sizeof(e->pose));
  e->dof = dof;
  e->saved = false;
  st = launch_energy(ctx, e, false, 1.0);
  if (st != LSDG_OK) return st;
  e->saved = true;
  e->saved_version = e->version;
  if (energy) *energy = e->h_out[0];
  if (n_active) *n_active = (int)e->h_out[8];
  return LSDG_OK;
}

lsdg_status lsdg_energy_backward(lsdg_ctx* ctx, lsdg_energy* e, double grad_energy, double* grad_xi,
                                 float* grad_idepth) {
  if (!ctx || !e) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (!e->saved) return ctx_fail(ctx, LSDG_INVALID_ARG, "backward without a forward");
  if (e->version != e->saved_version)
    return ctx_fail(ctx, LSDG_INVALID_ARG, "inverse depths or variances changed since the forward");
  lsdg_status st = launch_energy(ctx, e, true, grad_energy);
  if (st != LSDG_OK) return st;
  if (grad_xi)  // the kernel sums dE/dxi; the chain rule's dL/dE is applied here in FP64
    for (int i = 0; i < e->dof; ++i) grad_xi[i] = grad_energy * e->h_out[1 + i];
  if (grad_idepth && e->n) {
    CK(ctx, cudaMemcpyAsync(grad_idepth, e->grho, (size_t)e->n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return LSDG_OK;
}

lsdg_status lsdg_energy_refine(lsdg_ctx* ctx, lsdg_energy* e, int n_frames, const lsdg_frame* const* frames,
                               const double* ref_to_frames, int steps, double* energy_before, double* energy_after,
                               int* n_refined) {
  if (!ctx || !e || !frames || !ref_to_frames) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  if (n_frames < 1 || n_frames > LSDG_MAX_REFS) return ctx_fail(ctx, LSDG_INVALID_ARG, "n_frames must be in 1..%d", LSDG_MAX_REFS);
  if (steps < 0 || steps > 100000) return ctx_fail(ctx, LSDG_INVALID_ARG, "steps out of range");
  RefineArgs a{};
  CK(ctx, cudaStreamSynchronize(ctx->stream));  // h_fr may still feed an earlier copy
  for (int j = 0; j < n_frames; ++j) {
    lsdg_status st = check_frame(ctx, e, frames[j]);
    if (st != LSDG_OK) return st;
    e->h_fr[j].img = frames[j]->fs.h_frames[0].plane[e->level];
    for (int i = 0; i < 12; ++i) e->h_fr[j].M[i] = (float)ref_to_frames[12 * j + i];
  }
  CK(ctx, cudaMemcpyAsync(e->d_fr, e->h_fr, sizeof(RefineFrame) * n_frames, cudaMemcpyHostToDevice, ctx->stream));
  a.fr = e->d_fr;
  const lsdg_params& p = ctx->params;
  a.ray = e->ray;
  a.rho = e->rho;
  a.sig2 = e->sig2;
  a.n = e->n;
  a.nf = n_frames;
  a.steps = steps;
  a.w = e->w;
  a.h = e->h;
  a.fx = e->fx;
  a.fy = e->fy;
  a.cx = e->cx;
  a.cy = e->cy;
  a.hp = huber_of(p);
  a.pvar = p.photometric_variance;
  a.rho_lo = p.min_idepth;
  a.rho_hi = p.max_idepth;
  a.lam0 = (float)p.lm_lambda_initial;
  a.lam_up = (float)p.lm_lambda_up;
  a.lam_down = (float)p.lm_lambda_down;
  a.prior_w = p.refine_prior_weight;
  a.part = e->part;
  a.ticket = e->ticket;
  a.out = e->out;
  const int grid = grid_for(e->n, kEThreads / 8);
  CK(ctx, cudaEventRecord(e->ev[4], ctx->stream));
  energy_refine_kernel<<<grid, kEThreads, 0, ctx->stream>>>(a);
  CK(ctx, cudaGetLastError());
  CK(ctx, cudaEventRecord(e->ev[5], ctx->stream));
  ctx->launches += 1;
  ++e->version;
  lsdg_status st = read_out(ctx, e);
  if (st != LSDG_OK) return st;
  if (energy_before) *energy_before = e->h_out[0];
  if (energy_after) *energy_after = e->h_out[1];
  if (n_refined) *n_refined = (int)e->h_out[8];
  return LSDG_OK;
}

lsdg_status lsdg_energy_timing(lsdg_ctx* ctx, const lsdg_energy* e, float* forward_ms, float* backward_ms,
                               float* refine_ms) {
  if (!ctx || !e) return ctx_fail(ctx, LSDG_INVALID_ARG, "null argument");
  float* dst[3] = {forward_ms, backward_ms, refine_ms};
  for (int i = 0; i < 3; ++i) {
    if (!dst[i]) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e->ev[2 * i], e->ev[2 * i + 1]) != cudaSuccess) {
      cudaGetLastError();
      ms = -1.f;  // that kernel has not run yet
    }
    *dst[i] = ms;
  }
  return LSDG_OK;
}

}  // extern "C"

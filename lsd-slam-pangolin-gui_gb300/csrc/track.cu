// track.cu -- a3/a4/a5/a11 of the hot path: SE3 direct image alignment.
//
// Upstream: SE3Tracker::trackFrame and its calculateWarpUpdate (lsd-slam fips import, absent from
// the reference; the call chain starts at lib/App/InputThread.cpp:71).  Method: ECCV 2014 sec. 3.2
// -- variance-normalised photometric residual, Huber weights, LM on se(3), coarse to fine.
//
// GB300 design.  One persistent kernel tracks any number of pairs.  Each pair is owned by one
// thread-block cluster (C CTAs of NT threads, C up to 16); clusters pull pairs from an atomic work
// queue (largest first).  A residual pass over a level's points is:
//   1. every thread walks the SoA points with stride C*NT (coalesced float4 loads), warps the point
//      with the current pose, samples the new frame's intensity with the C1 Catmull-Rom
//      interpolant and its exact derivative (4x4 taps, L1/L2 resident), and accumulates the
//      21 + 6 + 1 Kahan-compensated float sums of J^T W J, J^T W r and the Huber energy.  The
//      first pass of a level fixes each point's residual variance in the psig scratch array (and
//      leaves out points that do not land border_margin pixels inside the image), so each level
//      minimises one fixed, continuous energy whose gradient is exactly 2 J^T W r;
//   2. warp shuffles merge the compensated pairs, then a fixed-order block merge in shared memory;
//   3. cluster.sync(); rank 0 merges the C block partials through distributed shared memory (fixed
//      rank order, so the result is deterministic for a given C and NT);
//   4. thread 0 of rank 0 runs the LM step in FP64 (6x6 LDLT, se(3) exp, composition, accept /
//      reject, convergence and level changes) and publishes the next pose in its shared memory;
//   5. cluster.sync(); every CTA reads the pose through DSMEM and starts the next pass.
// The whole LM loop over all levels therefore runs on the device without a host round trip and
// without global-memory scratch for the reduction.  The one-pair form (lsdg_track_se3) is the same
// kernel with a single cluster.
//
// Arithmetic: FP32 residuals/weights/Jacobians (this translation unit is built with FMA contraction,
// so per-point values differ from the CPU oracle in the last bits; parity is by tolerance),
// Kahan-compensated sums, FP64 only in the LM step.
#include <cooperative_groups.h>

#include "lsdg_internal.cuh"

namespace cg = cooperative_groups;

namespace lsdg {

constexpr int kSums = 28;  // 21 (H) + 6 (g) + 1 (energy)

__device__ __forceinline__ void kadd(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}
__device__ __forceinline__ void kmerge(float& s, float& c, float os, float oc) {
  const float t = s + os;
  const float bp = t - s;
  const float err = (s - (t - bp)) + (os - bp);
  s = t;
  c = (c + oc) - err;
}

// Catmull-Rom cubic (C1, interpolating): weights of taps -1, 0, 1, 2 at fraction t and their
// derivatives; at t = 0 the derivative weights are the central difference (-1/2, 0, 1/2, 0).
__device__ __forceinline__ void catmull_rom(float t, float w[4], float d[4]) {
  const float t2 = t * t, t3 = t2 * t;
  w[0] = 0.5f * ((2.f * t2 - t3) - t);
  w[1] = 0.5f * ((3.f * t3 - 5.f * t2) + 2.f);
  w[2] = 0.5f * ((4.f * t2 - 3.f * t3) + t);
  w[3] = 0.5f * (t3 - t2);
  d[0] = 0.5f * ((4.f * t - 3.f * t2) - 1.f);
  d[1] = 0.5f * (9.f * t2 - 10.f * t);
  d[2] = 0.5f * ((8.f * t - 9.f * t2) + 1.f);
  d[3] = 0.5f * (3.f * t2 - 2.f * t);
}

struct Ctl {
  float R[9];
  float t[3];
  int pair;  // -1: no more work
  int level;
  int first;  // first pass of the level: fixes each point's residual variance and participation
  int pad;
};

struct CtaPart {
  float s[kSums];
  float c[kSums];
  int cnt[3];  // good, bad, out-of-image
};

enum { PH_INIT = 0, PH_TRY = 1 };

struct LMState {
  double T[12];     // ref_to_frame, accepted
  double Ttry[12];  // ref_to_frame being evaluated
  double S[32];     // sums of the last accepted pass
  double E, lambda, gnmax;
  int it, phase, level, pair, have_final, fresh;
  lsdg_track_stats st;
};

// ------------------------------------------------------------------------------------------
// FP64 SE(3) helpers (thread 0 of rank 0 only)
// ------------------------------------------------------------------------------------------
__device__ __noinline__ void se3_inv_d(const double* A, double* B) {
  double o[12];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) o[4 * i + j] = A[4 * j + i];
  for (int i = 0; i < 3; ++i) o[4 * i + 3] = -((o[4 * i + 0] * A[3] + o[4 * i + 1] * A[7]) + o[4 * i + 2] * A[11]);
  for (int i = 0; i < 12; ++i) B[i] = o[i];
}

__device__ __noinline__ void se3_exp_mul_d(const double* xi, const double* Tin, double* Tout) {
  const double v0 = xi[0], v1 = xi[1], v2 = xi[2], w0 = xi[3], w1 = xi[4], w2 = xi[5];
  const double th2 = w0 * w0 + w1 * w1 + w2 * w2;
  const double th = sqrt(th2);
  double A, B, Cc;
  if (th < 1e-4) {
    A = 1.0 - th2 / 6.0;
    B = 0.5 - th2 / 24.0;
    Cc = 1.0 / 6.0 - th2 / 120.0;
  } else {
    double s, c;
    sincos(th, &s, &c);
    A = s / th;
    B = (1.0 - c) / th2;
    Cc = (th - s) / (th2 * th);
  }
  const double K[9] = {0, -w2, w1, w2, 0, -w0, -w1, w0, 0};
  double K2[9], E[12];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s = s + K[3 * i + k] * K[3 * k + j];
      K2[3 * i + j] = s;
    }
  double R[9], V[9];
  for (int i = 0; i < 9; ++i) {
    const double I = (i % 4 == 0) ? 1.0 : 0.0;
    R[i] = (I + A * K[i]) + B * K2[i];
    V[i] = (I + B * K[i]) + Cc * K2[i];
  }
  for (int i = 0; i < 3; ++i) {
    E[4 * i + 0] = R[3 * i + 0];
    E[4 * i + 1] = R[3 * i + 1];
    E[4 * i + 2] = R[3 * i + 2];
    E[4 * i + 3] = (V[3 * i + 0] * v0 + V[3 * i + 1] * v1) + V[3 * i + 2] * v2;
  }
  double o[12];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      o[4 * i + j] = (E[4 * i + 0] * Tin[j] + E[4 * i + 1] * Tin[4 + j]) + E[4 * i + 2] * Tin[8 + j];
    o[4 * i + 3] = ((E[4 * i + 0] * Tin[3] + E[4 * i + 1] * Tin[7]) + E[4 * i + 2] * Tin[11]) + E[4 * i + 3];
  }
  for (int i = 0; i < 12; ++i) Tout[i] = o[i];
}

// (H + lambda diag H) x = -g, H given as its upper triangle.  False if a pivot is not positive.
__device__ __noinline__ bool ldlt_solve_d(int n, const double* hu, const double* g, double lambda, double* x) {
  double A[7][7], L[7][7], d[7], y[7];
  int q = 0;
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) {
      A[i][j] = hu[q];
      A[j][i] = hu[q];
      ++q;
    }
  for (int i = 0; i < n; ++i) A[i][i] = A[i][i] * (1.0 + lambda);
  for (int j = 0; j < n; ++j) {
    double s = A[j][j];
    for (int k = 0; k < j; ++k) s = s - (L[j][k] * L[j][k]) * d[k];
    if (!(s > 1e-30)) return false;
    d[j] = s;
    L[j][j] = 1.0;
    for (int i = j + 1; i < n; ++i) {
      double t = A[i][j];
      for (int k = 0; k < j; ++k) t = t - (L[i][k] * L[j][k]) * d[k];
      L[i][j] = t / s;
    }
  }
  for (int i = 0; i < n; ++i) {
    double s = -g[i];
    for (int k = 0; k < i; ++k) s = s - L[i][k] * y[k];
    y[i] = s;
  }
  for (int i = 0; i < n; ++i) y[i] = y[i] / d[i];
  for (int i = n - 1; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < n; ++k) s = s - L[k][i] * x[k];
    x[i] = s;
  }
  return true;
}

// ------------------------------------------------------------------------------------------
// LM control (thread 0 of cluster rank 0)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void publish_pose(Ctl& c, const double* T) {
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) c.R[3 * i + j] = (float)T[4 * i + j];
    c.t[i] = (float)T[4 * i + 3];
  }
}

__device__ __forceinline__ int level_points(const TrackArgs& a, int pair, int level) {
  return a.pairs[pair].ref->pcount[level];
}

__device__ bool start_level(const TrackArgs& a, LMState& lm, Ctl& ctl, int level) {
  for (int l = level; l >= a.bottom_level; --l) {
    if (level_points(a, lm.pair, l) > 0) {
      lm.level = l;
      lm.phase = PH_INIT;
      ctl.level = l;
      ctl.pair = lm.pair;
      ctl.first = 1;
      publish_pose(ctl, lm.T);
      return true;
    }
  }
  return false;
}

__device__ __noinline__ void finish_pair(const TrackArgs& a, LMState& lm) {
  const int p = lm.pair;
  lsdg_track_stats& st = lm.st;
  double out[12];
  se3_inv_d(lm.T, out);
  for (int i = 0; i < 12; ++i) a.out_pose[12 * p + i] = out[i];
  int tot = 0;
  for (int l = 0; l < kMaxLevels; ++l) tot += st.passes[l];
  st.total_passes = tot;
  st.n_points = level_points(a, p, 0);
  const double* S = lm.S;
  if (lm.have_final) {
    st.n_valid = (int)S[28];
    st.n_good = (int)S[29];
    st.mean_energy = S[28] > 0 ? (float)(S[27] / S[28]) : 0.f;
    st.good_ratio = S[28] > 0 ? (float)(S[29] / S[28]) : 0.f;
    st.usage = st.n_points > 0 ? (float)(S[28] / st.n_points) : 0.f;
    for (int i = 0; i < 21; ++i) st.hessian[i] = S[i];
  }
  const bool lost = !lm.have_final || st.good_ratio < a.min_good_ratio || st.usage < a.min_usage;
  st.status = lost ? LSDG_TRACKING_LOST : LSDG_OK;
  a.out_stats[p] = st;
  if (a.out_sums)
    for (int i = 0; i < 32; ++i) a.out_sums[32 * p + i] = S[i];
}

// Takes pairs off the queue until one has a level to run; publishes it (or pair = -1).
__device__ __noinline__ void fetch_pair(const TrackArgs& a, LMState& lm, Ctl& ctl) {
  for (;;) {
    const int k = atomicAdd(a.work_counter, 1);
    if (k >= a.n_pairs) {
      ctl.pair = -1;
      return;
    }
    const int p = a.order ? a.order[k] : k;
    lm.pair = p;
    lm.have_final = 0;
    lm.it = 0;
    lm.E = 0;
    lm.lambda = a.lambda0;
    for (int i = 0; i < 32; ++i) lm.S[i] = 0;
    char* sp = reinterpret_cast<char*>(&lm.st);
    for (int i = 0; i < (int)sizeof(lsdg_track_stats); ++i) sp[i] = 0;
    if (a.init_is_ref_to_frame) {
      for (int i = 0; i < 12; ++i) lm.T[i] = a.init[12 * p + i];
    } else {
      se3_inv_d(a.init + 12 * p, lm.T);
    }
    if (start_level(a, lm, ctl, a.top_level)) return;
    finish_pair(a, lm);
  }
}

__device__ void next_level(const TrackArgs& a, LMState& lm, Ctl& ctl) {
  if (lm.level > a.bottom_level && start_level(a, lm, ctl, lm.level - 1)) return;
  finish_pair(a, lm);
  fetch_pair(a, lm, ctl);
}

// One LM iteration decision on the current linearisation lm.S (same rules as the CPU oracle):
// converged when the undamped Gauss-Newton step is below step_eps * 2^level; otherwise solve the
// damped system and publish the trial pose, unless the level's iteration budget is spent.
__device__ void try_step(const TrackArgs& a, LMState& lm, Ctl& ctl) {
  const double thr = a.step_eps * (double)(1 << lm.level);
  for (;;) {
    if (lm.fresh) {
      double gn[6];
      lm.gnmax = 1e300;
      if (ldlt_solve_d(6, lm.S, lm.S + 21, 0.0, gn)) {
        double m = 0;
        for (int i = 0; i < 6; ++i) m = fmax(m, fabs(gn[i]));
        lm.gnmax = m;
        if (m < thr) break;
      }
      lm.fresh = 0;
    }
    if (lm.it >= a.max_iter[lm.level]) break;
    lm.it++;
    double dx[6];
    if (!ldlt_solve_d(6, lm.S, lm.S + 21, lm.lambda, dx)) {
      lm.lambda *= a.lambda_up;
      continue;
    }
    se3_exp_mul_d(dx, lm.T, lm.Ttry);
    lm.phase = PH_TRY;
    ctl.pair = lm.pair;
    ctl.level = lm.level;
    ctl.first = 0;
    publish_pose(ctl, lm.Ttry);
    return;
  }
  next_level(a, lm, ctl);
}

__device__ __noinline__ void lm_advance(const TrackArgs& a, LMState& lm, Ctl& ctl, const double* tot) {
  lm.st.passes[lm.level]++;
  const double N = tot[28];
  if (lm.phase == PH_INIT) {
    if (N > 0) {
      for (int i = 0; i < 32; ++i) lm.S[i] = tot[i];
      lm.E = tot[27] / N;
      lm.lambda = a.lambda0;
      lm.it = 0;
      lm.fresh = 1;
      if (lm.level == a.bottom_level) lm.have_final = 1;
      try_step(a, lm, ctl);
    } else {
      next_level(a, lm, ctl);
    }
    return;
  }
  if (N > 0 && tot[27] / N < lm.E) {
    for (int i = 0; i < 12; ++i) lm.T[i] = lm.Ttry[i];
    for (int i = 0; i < 32; ++i) lm.S[i] = tot[i];
    lm.E = tot[27] / N;
    lm.lambda *= a.lambda_down;
    lm.fresh = 1;
  } else {
    if (lm.gnmax < a.stall_eps * (double)(1 << lm.level)) {  // noise floor of this level
      next_level(a, lm, ctl);
      return;
    }
    lm.lambda *= a.lambda_up;
  }
  try_step(a, lm, ctl);
}

// ------------------------------------------------------------------------------------------
// The persistent cluster kernel
// ------------------------------------------------------------------------------------------
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) track_se3_kernel(const TrackArgs a) {
  constexpr int NW = NT / 32;
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const unsigned C = cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  __shared__ float ws[NW][kSums];
  __shared__ float wc[NW][kSums];
  __shared__ int wn[NW][3];
  __shared__ CtaPart part;
  __shared__ Ctl ctl;
  __shared__ double tot[32];
  __shared__ LMState lm;

  if (rank == 0 && tid == 0) fetch_pair(a, lm, ctl);
  cluster.sync();

  for (;;) {
    if (rank != 0 && tid < (int)(sizeof(Ctl) / 4)) {
      const int* src = reinterpret_cast<const int*>(cluster.map_shared_rank(&ctl, 0));
      reinterpret_cast<int*>(&ctl)[tid] = src[tid];
    }
    __syncthreads();
    const int pair = ctl.pair;
    if (pair < 0) break;
    const int level = ctl.level;

    const PairDev pd = a.pairs[pair];
    const FrameDev* __restrict__ R = pd.ref;
    const FrameDev* __restrict__ Fc = pd.cur;
    const int n = R->pcount[level];
    const float4* __restrict__ pts = R->pxyzi[level];
    const float* __restrict__ pvar = R->pvar[level];
    float* __restrict__ psig = R->psig[level];
    const float* __restrict__ img = Fc->plane[level];
    const int w = Fc->w >> level, h = Fc->h >> level;
    const float fx = Fc->fx[level], fy = Fc->fy[level], cx = Fc->cx[level], cy = Fc->cy[level];
    const float umax = (float)(w - 2), vmax = (float)(h - 2);
    const float margin = a.border_margin;
    const float ulo = margin, vlo = margin, uhi = (float)(w - 1) - margin, vhi = (float)(h - 1) - margin;
    const bool first = ctl.first != 0;
    const float R00 = ctl.R[0], R01 = ctl.R[1], R02 = ctl.R[2];
    const float R10 = ctl.R[3], R11 = ctl.R[4], R12 = ctl.R[5];
    const float R20 = ctl.R[6], R21 = ctl.R[7], R22 = ctl.R[8];
    const float t0 = ctl.t[0], t1 = ctl.t[1], t2 = ctl.t[2];
    const float pvr = a.photometric_variance, delta = a.huber_delta, minz = a.min_z;

    float hs[21], hc[21], gs[6], gc[6], es = 0.f, ec = 0.f;
#pragma unroll
    for (int i = 0; i < 21; ++i) { hs[i] = 0.f; hc[i] = 0.f; }
#pragma unroll
    for (int i = 0; i < 6; ++i) { gs[i] = 0.f; gc[i] = 0.f; }
    int good = 0, bad = 0, oob = 0;

    for (int k = (int)rank * NT + tid; k < n; k += (int)C * NT) {
      float s2 = 0.f;
      if (!first) {
        s2 = psig[k];
        if (!(s2 > 0.f)) continue;  // sits out this level
      }
      const float4 p = __ldg(&pts[k]);
      const float X = p.x, Y = p.y, Z = p.z, Ik = p.w;
      const float Rpx = (R00 * X + R01 * Y) + R02 * Z;
      const float Rpy = (R10 * X + R11 * Y) + R12 * Z;
      const float Rpz = (R20 * X + R21 * Y) + R22 * Z;
      const float Xp = Rpx + t0, Yp = Rpy + t1, Zp = Rpz + t2;
      if (!(Zp > minz)) {
        if (first) psig[k] = 0.f;
        ++oob;
        continue;
      }
      const float iz = 1.0f / Zp;
      const float u = fx * (Xp * iz) + cx;
      const float v = fy * (Yp * iz) + cy;
      if (first) {
        if (!(u >= ulo && v >= vlo && u < uhi && v < vhi)) {
          psig[k] = 0.f;
          ++oob;
          continue;
        }
      } else if (!(u >= 1.f && v >= 1.f && u < umax && v < vmax)) {
        ++oob;
        continue;
      }
      const int ix = (int)u, iy = (int)v;
      const float ax = u - (float)ix, ay = v - (float)iy;
      float wx[4], dxw[4], wy[4], dyw[4];
      catmull_rom(ax, wx, dxw);
      catmull_rom(ay, wy, dyw);
      float rI[4], rD[4];
      const float* q = img + (size_t)(iy - 1) * w + (ix - 1);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float i0 = __ldg(q), i1 = __ldg(q + 1), i2 = __ldg(q + 2), i3 = __ldg(q + 3);
        rI[j] = ((wx[0] * i0 + wx[1] * i1) + wx[2] * i2) + wx[3] * i3;
        rD[j] = ((dxw[0] * i0 + dxw[1] * i1) + dxw[2] * i2) + dxw[3] * i3;
        q += w;
      }
      const float In = ((wy[0] * rI[0] + wy[1] * rI[1]) + wy[2] * rI[2]) + wy[3] * rI[3];
      const float Gx = ((wy[0] * rD[0] + wy[1] * rD[1]) + wy[2] * rD[2]) + wy[3] * rD[3];
      const float Gy = ((dyw[0] * rI[0] + dyw[1] * rI[1]) + dyw[2] * rI[2]) + dyw[3] * rI[3];
      const float r = In - Ik;
      const float gxs = Gx * fx, gys = Gy * fy;
      const float a0 = gxs * iz, a1 = gys * iz;
      const float a2 = -((a0 * Xp + a1 * Yp) * iz);
      float J[6];
      J[0] = a0;
      J[1] = a1;
      J[2] = a2;
      J[3] = Yp * a2 - Zp * a1;
      J[4] = Zp * a0 - Xp * a2;
      J[5] = Xp * a1 - Yp * a0;
      if (first) {
        const float drd = -(((a0 * Rpx + a1 * Rpy) + a2 * Rpz) * Z);
        s2 = pvr + (drd * drd) * __ldg(&pvar[k]);
        psig[k] = s2;
      }
      const float e2 = (r * r) / s2;
      const float ae = sqrtf(e2);
      float wh, rho;
      if (ae <= delta) { wh = 1.f; rho = e2; ++good; }
      else { wh = delta / ae; rho = delta * (2.f * ae - delta); ++bad; }
      const float wgt = wh / s2;
      float wJ[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) wJ[i] = wgt * J[i];
      int q2 = 0;
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j) { kadd(hs[q2], hc[q2], wJ[i] * J[j]); ++q2; }
#pragma unroll
      for (int i = 0; i < 6; ++i) kadd(gs[i], gc[i], wJ[i] * r);
      kadd(es, ec, rho);
    }

    // warp merge
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int i = 0; i < 21; ++i) kmerge(hs[i], hc[i], __shfl_xor_sync(0xffffffffu, hs[i], o), __shfl_xor_sync(0xffffffffu, hc[i], o));
#pragma unroll
      for (int i = 0; i < 6; ++i) kmerge(gs[i], gc[i], __shfl_xor_sync(0xffffffffu, gs[i], o), __shfl_xor_sync(0xffffffffu, gc[i], o));
      kmerge(es, ec, __shfl_xor_sync(0xffffffffu, es, o), __shfl_xor_sync(0xffffffffu, ec, o));
    }
    good = __reduce_add_sync(0xffffffffu, good);
    bad = __reduce_add_sync(0xffffffffu, bad);
    oob = __reduce_add_sync(0xffffffffu, oob);
    if (lane == 0) {
#pragma unroll
      for (int i = 0; i < 21; ++i) { ws[wid][i] = hs[i]; wc[wid][i] = hc[i]; }
#pragma unroll
      for (int i = 0; i < 6; ++i) { ws[wid][21 + i] = gs[i]; wc[wid][21 + i] = gc[i]; }
      ws[wid][27] = es;
      wc[wid][27] = ec;
      wn[wid][0] = good;
      wn[wid][1] = bad;
      wn[wid][2] = oob;
    }
    __syncthreads();
    if (tid < kSums) {
      float s = 0.f, c = 0.f;
      for (int k = 0; k < NW; ++k) kmerge(s, c, ws[k][tid], wc[k][tid]);
      part.s[tid] = s;
      part.c[tid] = c;
    } else if (tid < kSums + 3) {
      int v = 0;
      for (int k = 0; k < NW; ++k) v += wn[k][tid - kSums];
      part.cnt[tid - kSums] = v;
    }
    cluster.sync();

    if (rank == 0) {
      if (tid < kSums) {
        float s = 0.f, c = 0.f;
        for (unsigned r = 0; r < C; ++r) {
          const CtaPart* pr = cluster.map_shared_rank(&part, r);
          kmerge(s, c, pr->s[tid], pr->c[tid]);
        }
        tot[tid] = (double)s - (double)c;
      } else if (tid < kSums + 3) {
        int v = 0;
        for (unsigned r = 0; r < C; ++r) v += cluster.map_shared_rank(&part, r)->cnt[tid - kSums];
        tot[tid + 1] = (double)v;  // 29 good, 30 bad, 31 out of image
      }
      __syncthreads();
      if (tid == 0) {
        tot[28] = tot[29] + tot[30];
        lm_advance(a, lm, ctl, tot);
      }
    }
    cluster.sync();
  }
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// ------------------------------------------------------------------------------------------
// Host side: launch with a cluster shape.  Shapes are (threads per CTA, CTAs the register budget
// must leave room for on one SM); the autotuner picks one together with the cluster size.
// ------------------------------------------------------------------------------------------
template <int NT, int MINB>
static cudaError_t launch_nt(const TrackArgs& a, int cluster, int n_clusters, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster * n_clusters);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, track_se3_kernel<NT, MINB>, a);
}

template <int NT, int MINB>
static int max_clusters_nt(int cluster) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster);
  cfg.blockDim = dim3(NT);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, track_se3_kernel<NT, MINB>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

#define LSDG_TRACK_SHAPES(X) X(128, 4) X(128, 8) X(256, 2) X(256, 4) X(512, 1) X(512, 2)

// Allows clusters of up to 16 CTAs (non-portable size) for every instantiation.  Called once
// per context, outside any stream capture.
cudaError_t track_prepare() {
  cudaError_t e = cudaSuccess;
#define X(nt, mb) \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(track_se3_kernel<nt, mb>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  LSDG_TRACK_SHAPES(X)
#undef X
  return e;
}

int track_shape_count() {
  int n = 0;
#define X(nt, mb) ++n;
  LSDG_TRACK_SHAPES(X)
#undef X
  return n;
}

void track_shape(int i, int* threads, int* minblocks) {
  int k = 0;
#define X(nt, mb)       \
  if (k++ == i) {       \
    *threads = nt;      \
    *minblocks = mb;    \
  }
  LSDG_TRACK_SHAPES(X)
#undef X
}

cudaError_t launch_track(const TrackArgs& a, int threads, int minblocks, int cluster, int n_clusters, cudaStream_t s) {
#define X(nt, mb) \
  if (threads == nt && minblocks == mb) return launch_nt<nt, mb>(a, cluster, n_clusters, s);
  LSDG_TRACK_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

int track_max_clusters(int threads, int minblocks, int cluster) {
#define X(nt, mb) \
  if (threads == nt && minblocks == mb) return max_clusters_nt<nt, mb>(cluster);
  LSDG_TRACK_SHAPES(X)
#undef X
  return 0;
}

}  // namespace lsdg

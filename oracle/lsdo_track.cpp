// lsdo_track.cpp -- CPU ORACLE (test infrastructure only) for the direct-alignment half of the
// LSD-SLAM hot path: frame pyramid, keyframe depth pyramid and tracking reference points, the
// per-point SE3 residual / Jacobian / Huber weight, calculateWarpUpdate's normal equations and
// SE3Tracker::trackFrame's Levenberg-Marquardt loop.
//
// Only tests/, the smoke check and bench.py's cpu_baseline leg call this.  The product library
// (lsd-slam-pangolin-gui_gb300/csrc) never links or loads it.
//
// What it restates.  The reference repository (apl-ocean-engineering/lsd-slam-pangolin-gui) does
// not contain these functions: SE3Tracker, Frame and DepthMap live in the lsd-slam fips import
// (fips.yml:2-4, branch "unstable", no pinned commit), which is not vendored and cannot be built
// here.  This file follows the published method instead -- Engel, Sturm, Cremers, "Semi-Dense
// Visual Odometry for a Monocular Camera" (ICCV 2013) and Engel, Schoeps, Cremers, "LSD-SLAM:
// Large-Scale Direct Monocular SLAM" (ECCV 2014, sec. 3.2: variance-normalised photometric
// residual r / sigma_r with sigma_r^2 = 2 sigma_I^2 + (dr/dD)^2 V, Huber norm, iteratively
// re-weighted Gauss-Newton / LM on se(3)) -- with the conventions the reference's own code pins:
//   - back-projection X = (x - cx)/fx * z, z = 1/idepth   (lib/Pangolin_IOWrapper/Keyframe.h:86-89,134-136)
//   - per-level row-major float planes idepth/idepthVar/image (PangolinOutputIOWrapper.cpp:77-89)
//   - idepth <= 0 means "no depth"                        (Keyframe.h:95)
// Parity with upstream is UNPINNED: the reference has no tests beyond ASSERT_TRUE(true)
// (test/unit/test_test.cpp:4-7) and no golden vectors.  The tuning table is lsdg_params.
//
// Every function is a template on the arithmetic type T: T = float is the parity oracle (same
// operation order as the CUDA kernels; built with -ffp-contract=off so that a*b+c is never
// fused), T = double is the FP64 accuracy oracle.  The LM solve, exp map and pose composition
// are double in both, as on the GPU.
#include "lsdo.h"

#include <cmath>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>

namespace lsdo {

// ------------------------------------------------------------------------------------------
// Intrinsics per level (computed in double, used as T)
// ------------------------------------------------------------------------------------------
void level_intrinsics(const lsdg_intrinsics& k0, int levels, LevelCam* out, int w0, int h0) {
  double fx = k0.fx, fy = k0.fy, cx = k0.cx, cy = k0.cy;
  int w = w0, h = h0;
  for (int l = 0; l < levels; ++l) {
    out[l].fx = fx; out[l].fy = fy; out[l].cx = cx; out[l].cy = cy;
    out[l].fxi = 1.0 / fx; out[l].fyi = 1.0 / fy;
    out[l].w = w; out[l].h = h;
    fx *= 0.5; fy *= 0.5;
    cx = (cx + 0.5) * 0.5 - 0.5;
    cy = (cy + 0.5) * 0.5 - 0.5;
    w /= 2; h /= 2;
  }
}

// ------------------------------------------------------------------------------------------
// a1: intensity + gradient pyramid
// ------------------------------------------------------------------------------------------
template <class T>
void build_pyramid(const float* img, int w0, int h0, int levels, std::vector<std::vector<T>>& I,
                   std::vector<std::vector<T>>& gx, std::vector<std::vector<T>>& gy) {
  I.assign(levels, {});
  gx.assign(levels, {});
  gy.assign(levels, {});
  int w = w0, h = h0;
  for (int l = 0; l < levels; ++l) {
    I[l].resize((size_t)w * h);
    if (l == 0) {
      for (size_t i = 0; i < (size_t)w * h; ++i) I[0][i] = (T)img[i];
    } else {
      const std::vector<T>& P = I[l - 1];
      int pw = w * 2;
      for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
          const T* r0 = &P[(size_t)(2 * y) * pw + 2 * x];
          const T* r1 = r0 + pw;
          I[l][(size_t)y * w + x] = ((r0[0] + r0[1]) + (r1[0] + r1[1])) * (T)0.25;
        }
    }
    gx[l].assign((size_t)w * h, (T)0);
    gy[l].assign((size_t)w * h, (T)0);
    const std::vector<T>& L = I[l];
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        size_t i = (size_t)y * w + x;
        if (x >= 1 && x <= w - 2) gx[l][i] = (L[i + 1] - L[i - 1]) * (T)0.5;
        if (y >= 1 && y <= h - 2) gy[l][i] = (L[i + w] - L[i - w]) * (T)0.5;
      }
    w /= 2;
    h /= 2;
  }
}

// ------------------------------------------------------------------------------------------
// a2: keyframe depth pyramid (inverse-variance weighted 2x2 mean) and reference points
// ------------------------------------------------------------------------------------------
template <class T>
void build_depth_pyramid(const float* idepth, const float* var, int w0, int h0, int levels,
                         std::vector<std::vector<T>>& D, std::vector<std::vector<T>>& V) {
  D.assign(levels, {});
  V.assign(levels, {});
  int w = w0, h = h0;
  for (int l = 0; l < levels; ++l) {
    D[l].resize((size_t)w * h);
    V[l].resize((size_t)w * h);
    if (l == 0) {
      for (size_t i = 0; i < (size_t)w * h; ++i) {
        T d = (T)idepth[i], v = (T)var[i];
        bool ok = d > (T)0 && v > (T)0;
        D[0][i] = ok ? d : (T)-1;
        V[0][i] = ok ? v : (T)-1;
      }
    } else {
      int pw = w * 2;
      for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
          size_t c[4] = {(size_t)(2 * y) * pw + 2 * x, (size_t)(2 * y) * pw + 2 * x + 1,
                         (size_t)(2 * y + 1) * pw + 2 * x, (size_t)(2 * y + 1) * pw + 2 * x + 1};
          T sw = 0, swd = 0;
          int n = 0;
          for (int k = 0; k < 4; ++k) {
            T d = D[l - 1][c[k]], v = V[l - 1][c[k]];
            if (d > (T)0 && v > (T)0) {
              T wt = (T)1 / v;
              sw = sw + wt;
              swd = swd + wt * d;
              ++n;
            }
          }
          size_t i = (size_t)y * w + x;
          if (n > 0) {
            D[l][i] = swd / sw;
            V[l][i] = (T)n / sw;
          } else {
            D[l][i] = (T)-1;
            V[l][i] = (T)-1;
          }
        }
    }
    w /= 2;
    h /= 2;
  }
}

template <class T>
void build_points(const std::vector<std::vector<T>>& I, const std::vector<std::vector<T>>& D,
                  const std::vector<std::vector<T>>& V, const LevelCam* cam, int levels,
                  std::vector<Points<T>>& pts) {
  pts.assign(levels, {});
  for (int l = 0; l < levels; ++l) {
    const int w = cam[l].w, h = cam[l].h;
    const T cx = (T)cam[l].cx, cy = (T)cam[l].cy, fxi = (T)cam[l].fxi, fyi = (T)cam[l].fyi;
    Points<T>& P = pts[l];
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        size_t i = (size_t)y * w + x;
        T d = D[l][i], v = V[l][i];
        if (!(d > (T)0 && v > (T)0)) continue;
        T z = (T)1 / d;
        P.xyzi.push_back((((T)x - cx) * fxi) * z);
        P.xyzi.push_back((((T)y - cy) * fyi) * z);
        P.xyzi.push_back(z);
        P.xyzi.push_back(I[l][i]);
        P.var.push_back(v);
        P.pix.push_back((int)i);
      }
  }
}

// ------------------------------------------------------------------------------------------
// a3 + a4: one residual pass (calculateWarpUpdate) over [begin, end) of a level's points
// ------------------------------------------------------------------------------------------
template <class T>
struct PassSums {
  KSum<T> h[21], g[6], e;
  long n = 0, good = 0, bad = 0, oob = 0;
  void merge(const PassSums& o) {
    for (int i = 0; i < 21; ++i) h[i].merge(o.h[i]);
    for (int i = 0; i < 6; ++i) g[i].merge(o.g[i]);
    e.merge(o.e);
    n += o.n; good += o.good; bad += o.bad; oob += o.oob;
  }
};

// Residual model (own restatement of ECCV 2014 sec. 3.2):
//   r = I_new(pi(R p + t)) - I_key(p), I_new sampled with the C1 Catmull-Rom interpolant,
//   J = dr/dxi with the exact derivative of that interpolant (so that 2 J^T W r is the gradient
//       of the energy the LM step is accepted on, and J is continuous in the pose -- at pixel
//       centres it equals the central-difference gradient),
//   sigma^2 = sigma_I^2 + (dr/dd)^2 V(p), d = inverse depth, Huber weight on r / sigma,
//   energy = sum of Huber(r / sigma) (rho = e^2 inside delta, delta (2|e| - delta) outside).
// The first pass of a level ("first") fixes, per point, sigma^2 and whether the point takes part
// in the level (its warp must land border_margin pixels inside the image); sig2[k] stores sigma^2,
// or 0 for a point left out.  The later passes of the level reuse them, so every level minimises
// one fixed, continuous energy.
template <class T>
static void se3_pass_range(const Points<T>& P, size_t begin, size_t end, const FrameLevel<T>& F,
                           const LevelCam& cam, const double Tp[12], const lsdg_params& prm,
                           bool first, T* sig2, PassSums<T>& S) {
  const T R00 = (T)Tp[0], R01 = (T)Tp[1], R02 = (T)Tp[2], t0 = (T)Tp[3];
  const T R10 = (T)Tp[4], R11 = (T)Tp[5], R12 = (T)Tp[6], t1 = (T)Tp[7];
  const T R20 = (T)Tp[8], R21 = (T)Tp[9], R22 = (T)Tp[10], t2 = (T)Tp[11];
  const T fx = (T)cam.fx, fy = (T)cam.fy, cx = (T)cam.cx, cy = (T)cam.cy;
  // the 4x4 Catmull-Rom footprint of u needs columns floor(u)-1 .. floor(u)+2
  const T umax = (T)(cam.w - 2), vmax = (T)(cam.h - 2);
  const T margin = (T)prm.border_margin;
  const T ulo = margin, vlo = margin, uhi = (T)(cam.w - 1) - margin, vhi = (T)(cam.h - 1) - margin;
  const T pvar = (T)prm.photometric_variance, delta = (T)prm.huber_delta, minz = (T)prm.min_z;
  const int w = cam.w;
  for (size_t k = begin; k < end; ++k) {
    if (!first && !(sig2[k] > (T)0)) continue;
    const T X = P.xyzi[4 * k + 0], Y = P.xyzi[4 * k + 1], Z = P.xyzi[4 * k + 2], Ik = P.xyzi[4 * k + 3];
    const T Rpx = (R00 * X + R01 * Y) + R02 * Z;
    const T Rpy = (R10 * X + R11 * Y) + R12 * Z;
    const T Rpz = (R20 * X + R21 * Y) + R22 * Z;
    const T Xp = Rpx + t0, Yp = Rpy + t1, Zp = Rpz + t2;
    if (!(Zp > minz)) {
      if (first) sig2[k] = (T)0;
      ++S.oob;
      continue;
    }
    const T iz = (T)1 / Zp;
    const T u = fx * (Xp * iz) + cx;
    const T v = fy * (Yp * iz) + cy;
    if (first) {
      if (!(u >= ulo && v >= vlo && u < uhi && v < vhi)) {
        sig2[k] = (T)0;
        ++S.oob;
        continue;
      }
    } else if (!(u >= (T)1 && v >= (T)1 && u < umax && v < vmax)) {
      ++S.oob;
      continue;
    }
    const int ix = (int)u, iy = (int)v;
    const T ax = u - (T)ix, ay = v - (T)iy;
    T wx[4], dx[4], wy[4], dy[4];
    catmull_rom(ax, wx, dx);
    catmull_rom(ay, wy, dy);
    T rI[4], rD[4];
    for (int j = 0; j < 4; ++j) {
      const T* row = &F.I[(size_t)(iy - 1 + j) * w + (ix - 1)];
      rI[j] = ((wx[0] * row[0] + wx[1] * row[1]) + wx[2] * row[2]) + wx[3] * row[3];
      rD[j] = ((dx[0] * row[0] + dx[1] * row[1]) + dx[2] * row[2]) + dx[3] * row[3];
    }
    const T In = ((wy[0] * rI[0] + wy[1] * rI[1]) + wy[2] * rI[2]) + wy[3] * rI[3];
    const T Gx = ((wy[0] * rD[0] + wy[1] * rD[1]) + wy[2] * rD[2]) + wy[3] * rD[3];
    const T Gy = ((dy[0] * rI[0] + dy[1] * rI[1]) + dy[2] * rI[2]) + dy[3] * rI[3];
    const T r = In - Ik;
    const T gxs = Gx * fx, gys = Gy * fy;
    const T a0 = gxs * iz, a1 = gys * iz;
    const T a2 = -((a0 * Xp + a1 * Yp) * iz);
    T J[6];
    J[0] = a0; J[1] = a1; J[2] = a2;
    J[3] = Yp * a2 - Zp * a1;
    J[4] = Zp * a0 - Xp * a2;
    J[5] = Xp * a1 - Yp * a0;
    T s2;
    if (first) {
      const T drd = -(((a0 * Rpx + a1 * Rpy) + a2 * Rpz) * Z);
      s2 = pvar + (drd * drd) * P.var[k];
      sig2[k] = s2;
    } else {
      s2 = sig2[k];
    }
    const T e2 = (r * r) / s2;
    const T ae = std::sqrt(e2);
    T wh, rho;
    if (ae <= delta) { wh = (T)1; rho = e2; ++S.good; }
    else { wh = delta / ae; rho = delta * ((T)2 * ae - delta); ++S.bad; }
    const T wgt = wh / s2;
    T wJ[6];
    for (int i = 0; i < 6; ++i) wJ[i] = wgt * J[i];
    int q = 0;
    for (int i = 0; i < 6; ++i)
      for (int j = i; j < 6; ++j) S.h[q++].add(wJ[i] * J[j]);
    for (int i = 0; i < 6; ++i) S.g[i].add(wJ[i] * r);
    S.e.add(rho);
    ++S.n;
  }
}

template <class T>
static void se3_pass(const Points<T>& P, const FrameLevel<T>& F, const LevelCam& cam,
                     const double Tp[12], const lsdg_params& prm, int threads, bool first,
                     std::vector<T>& sig2, double out[32]) {
  size_t n = P.var.size();
  if (sig2.size() != n) sig2.assign(n, (T)0);
  PassSums<T> total;
  if (threads <= 1 || n < 4096) {
    se3_pass_range(P, 0, n, F, cam, Tp, prm, first, sig2.data(), total);
  } else {
    std::vector<PassSums<T>> part(threads);
    std::vector<std::thread> th;
    for (int k = 0; k < threads; ++k) {
      size_t b = n * k / threads, e = n * (k + 1) / threads;
      th.emplace_back([&, k, b, e] { se3_pass_range(P, b, e, F, cam, Tp, prm, first, sig2.data(), part[k]); });
    }
    for (auto& t : th) t.join();
    for (int k = 0; k < threads; ++k) total.merge(part[k]);
  }
  for (int i = 0; i < 21; ++i) out[i] = total.h[i].value();
  for (int i = 0; i < 6; ++i) out[21 + i] = total.g[i].value();
  out[27] = total.e.value();
  out[28] = (double)total.n;
  out[29] = (double)total.good;
  out[30] = (double)total.bad;
  out[31] = (double)total.oob;
}

// ------------------------------------------------------------------------------------------
// SE3 in double: exp map, composition, inverse; 6x6 LDLT
// ------------------------------------------------------------------------------------------
// exp of a twist xi = (v, w): R = I + A K + B K^2, t = (I + B K + C K^2) v with K = [w]x,
// K^2 = w w^T - |w|^2 I, A = sin(t)/t, B = (1 - cos t)/t^2, C = (t - sin t)/t^3 (t = |w|).  For
// t < 0.05 the coefficients are their Taylor series in t^2 through t^10 (truncation < 1e-25).
void se3_coeffs(double th2, double* A, double* B, double* C) {
  if (th2 < 0.0025) {
    *A = 1.0 + th2 * (-1.0 / 6.0 + th2 * (1.0 / 120.0 + th2 * (-1.0 / 5040.0 + th2 * (1.0 / 362880.0 + th2 * (-1.0 / 39916800.0)))));
    *B = 0.5 + th2 * (-1.0 / 24.0 + th2 * (1.0 / 720.0 + th2 * (-1.0 / 40320.0 + th2 * (1.0 / 3628800.0 + th2 * (-1.0 / 479001600.0)))));
    *C = 1.0 / 6.0 + th2 * (-1.0 / 120.0 + th2 * (1.0 / 5040.0 + th2 * (-1.0 / 362880.0 + th2 * (1.0 / 39916800.0 + th2 * (-1.0 / 6227020800.0)))));
  } else {
    const double th = std::sqrt(th2), sn = std::sin(th), cs = std::cos(th);
    *A = sn / th;
    *B = (1.0 - cs) / th2;
    *C = (th - sn) / (th2 * th);
  }
}

void se3_exp(const double xi[6], double T[12]) {
  const double v[3] = {xi[0], xi[1], xi[2]}, w[3] = {xi[3], xi[4], xi[5]};
  const double th2 = (w[0] * w[0] + w[1] * w[1]) + w[2] * w[2];
  double A, B, C;
  se3_coeffs(th2, &A, &B, &C);
  const double K[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double R[9], V[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const int e = 3 * i + j;
      const double I = (i == j) ? 1.0 : 0.0;
      const double K2 = w[i] * w[j] - ((i == j) ? th2 : 0.0);
      R[e] = (I + A * K[e]) + B * K2;
      V[e] = (I + B * K[e]) + C * K2;
    }
  for (int i = 0; i < 3; ++i) {
    T[4 * i + 0] = R[3 * i + 0];
    T[4 * i + 1] = R[3 * i + 1];
    T[4 * i + 2] = R[3 * i + 2];
    T[4 * i + 3] = (V[3 * i + 0] * v[0] + V[3 * i + 1] * v[1]) + V[3 * i + 2] * v[2];
  }
}

void se3_mul(const double A[12], const double B[12], double C[12]) {
  double out[12];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      out[4 * i + j] = (A[4 * i + 0] * B[j] + A[4 * i + 1] * B[4 + j]) + A[4 * i + 2] * B[8 + j];
    out[4 * i + 3] = ((A[4 * i + 0] * B[3] + A[4 * i + 1] * B[7]) + A[4 * i + 2] * B[11]) + A[4 * i + 3];
  }
  std::memcpy(C, out, sizeof(out));
}

void se3_inv(const double A[12], double B[12]) {
  double out[12];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out[4 * i + j] = A[4 * j + i];
  for (int i = 0; i < 3; ++i)
    out[4 * i + 3] = -((out[4 * i + 0] * A[3] + out[4 * i + 1] * A[7]) + out[4 * i + 2] * A[11]);
  std::memcpy(B, out, sizeof(out));
}

// Solve (H + lambda diag(H)) x = -g for an n x n symmetric H given as its upper triangle
// (row-major).  Returns false when a pivot is not positive.
bool ldlt_solve(int n, const double* hu, const double* g, double lambda, double* x) {
  double A[8][8], L[8][8], d[8], y[8];
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

// Optional per-pass trace for debugging and tests: 8 doubles per pass
// {level, iteration, lambda, accepted, mean energy, points, max|undamped step|, 0}.
thread_local std::vector<double>* g_trace = nullptr;
static inline void trace(int lvl, int it, double lambda, int acc, double E, double N, double gn) {
  if (!g_trace) return;
  const double rec[8] = {(double)lvl, (double)it, lambda, (double)acc, E, N, gn, 0.0};
  g_trace->insert(g_trace->end(), rec, rec + 8);
}

// ------------------------------------------------------------------------------------------
// a5: SE3Tracker::trackFrame -- LM over the pyramid, coarse to fine
// ------------------------------------------------------------------------------------------
template <class T>
int track_se3(const KeyframeData<T>& kf, const FrameData<T>& fr, const lsdg_params& prm,
              const double frame_to_ref_init[12], double frame_to_ref_out[12],
              lsdg_track_stats* st, int threads) {
  std::memset(st, 0, sizeof(*st));
  double Tc[12];
  se3_inv(frame_to_ref_init, Tc);  // ref_to_frame
  double S[32] = {0};
  bool have_final = false;
  const int levels = prm.levels;
  for (int lvl = levels - 1; lvl >= 0; --lvl) {
    const Points<T>& P = kf.pts[lvl];
    if (P.var.empty()) continue;
    const LevelCam& cam = fr.cam[lvl];  // projection into the tracked frame
    std::vector<T> sig2;
    se3_pass(P, fr.lv[lvl], cam, Tc, prm, threads, true, sig2, S);
    st->passes[lvl]++;
    if (!(S[28] > 0)) continue;
    double E = S[27] / S[28];
    double lambda = prm.lm_lambda_initial;
    const double thr = (double)prm.step_eps * (double)(1 << lvl);
    const double stall = (double)prm.stall_eps * (double)(1 << lvl);
    bool fresh = true;  // S is the linearisation at Tc (first pass or an accepted step)
    double gnmax = 1e300;  // max |undamped Gauss-Newton step| of the current linearisation
    for (int it = 0;;) {
      if (fresh) {
        // converged when the undamped Gauss-Newton step of this linearisation is negligible
        double gn[6];
        gnmax = 1e300;
        if (ldlt_solve(6, S, S + 21, 0.0, gn)) {
          gnmax = 0;
          for (int i = 0; i < 6; ++i) gnmax = std::max(gnmax, std::fabs(gn[i]));
          trace(lvl, it, lambda, 2, E, S[28], gnmax);
          if (gnmax < thr) break;
        }
        fresh = false;
      }
      if (it >= prm.max_iterations[lvl]) break;
      double dx[6];
      ++it;
      if (!ldlt_solve(6, S, S + 21, lambda, dx)) {
        lambda *= prm.lm_lambda_up;
        continue;
      }
      double Ex[12], Tt[12];
      se3_exp(dx, Ex);
      se3_mul(Ex, Tc, Tt);
      double S2[32];
      se3_pass(P, fr.lv[lvl], cam, Tt, prm, threads, false, sig2, S2);
      st->passes[lvl]++;
      trace(lvl, it, lambda, S2[28] > 0 && S2[27] / S2[28] < E, S2[28] > 0 ? S2[27] / S2[28] : 0.0, S2[28], 0.0);
      if (S2[28] > 0 && S2[27] / S2[28] < E) {
        std::memcpy(Tc, Tt, sizeof(Tc));
        std::memcpy(S, S2, sizeof(S));
        E = S2[27] / S2[28];
        lambda *= prm.lm_lambda_down;
        fresh = true;
      } else {
        if (gnmax < stall) break;  // a step this small cannot lower the energy: noise floor
        lambda *= prm.lm_lambda_up;
      }
    }
    if (lvl == 0) have_final = true;
  }
  se3_inv(Tc, frame_to_ref_out);
  for (int l = 0; l < LSDG_MAX_LEVELS; ++l) st->total_passes += st->passes[l];
  st->n_points = (int)kf.pts[0].var.size();
  if (have_final) {
    st->n_valid = (int)S[28];
    st->n_good = (int)S[29];
    st->mean_energy = S[28] > 0 ? (float)(S[27] / S[28]) : 0.f;
    st->good_ratio = S[28] > 0 ? (float)(S[29] / S[28]) : 0.f;
    st->usage = st->n_points > 0 ? (float)(S[28] / st->n_points) : 0.f;
    for (int i = 0; i < 21; ++i) st->hessian[i] = S[i];
  }
  int status = LSDG_OK;
  if (!have_final || st->good_ratio < prm.min_good_ratio || st->usage < prm.min_usage)
    status = LSDG_TRACKING_LOST;
  st->status = status;
  return status;
}

template <class T>
void make_frame(const float* img, int w, int h, const lsdg_intrinsics& k, int levels, FrameData<T>& F) {
  F.levels = levels;
  level_intrinsics(k, levels, F.cam, w, h);
  std::vector<std::vector<T>> I, gx, gy;
  build_pyramid<T>(img, w, h, levels, I, gx, gy);
  F.lv.resize(levels);
  for (int l = 0; l < levels; ++l) {
    F.lv[l].I = std::move(I[l]);
    F.lv[l].gx = std::move(gx[l]);
    F.lv[l].gy = std::move(gy[l]);
  }
}

template <class T>
void make_keyframe(const FrameData<T>& F, const float* idepth, const float* var, KeyframeData<T>& K) {
  const int levels = F.levels;
  std::memcpy(K.cam, F.cam, sizeof(K.cam));
  std::vector<std::vector<T>> D, V, I(levels);
  build_depth_pyramid<T>(idepth, var, F.cam[0].w, F.cam[0].h, levels, D, V);
  for (int l = 0; l < levels; ++l) I[l] = F.lv[l].I;
  build_points<T>(I, D, V, F.cam, levels, K.pts);
  K.D = std::move(D);
  K.V = std::move(V);
}

template void make_frame<float>(const float*, int, int, const lsdg_intrinsics&, int, FrameData<float>&);
template void make_frame<double>(const float*, int, int, const lsdg_intrinsics&, int, FrameData<double>&);
template void make_keyframe<float>(const FrameData<float>&, const float*, const float*, KeyframeData<float>&);
template void make_keyframe<double>(const FrameData<double>&, const float*, const float*, KeyframeData<double>&);
template int track_se3<float>(const KeyframeData<float>&, const FrameData<float>&, const lsdg_params&, const double*, double*, lsdg_track_stats*, int);
template int track_se3<double>(const KeyframeData<double>&, const FrameData<double>&, const lsdg_params&, const double*, double*, lsdg_track_stats*, int);

}  // namespace lsdo

// ============================================================================================
// extern "C" surface for ctypes (tests / bench cpu leg)
// ============================================================================================
using namespace lsdo;

template <class T, class O>
static void copy_pyramid(const FrameData<T>& F, O* out) {
  size_t off = 0;
  for (int l = 0; l < F.levels; ++l) {
    size_t n = (size_t)F.cam[l].w * F.cam[l].h;
    for (size_t i = 0; i < n; ++i) {
      out[off + 4 * i + 0] = (O)F.lv[l].I[i];
      out[off + 4 * i + 1] = (O)F.lv[l].gx[i];
      out[off + 4 * i + 2] = (O)F.lv[l].gy[i];
      out[off + 4 * i + 3] = (O)0;
    }
    off += 4 * n;
  }
}

extern "C" {

void lsdo_default_params(lsdg_params* p) { lsdo::default_params(p); }

// Pyramid of all levels, float4 {I, gx, gy, 0} per pixel, levels back to back.
void lsdo_pyramid_f(const float* img, int w, int h, int levels, float* out) {
  FrameData<float> F;
  lsdg_intrinsics k{1, 1, 0, 0};
  make_frame<float>(img, w, h, k, levels, F);
  copy_pyramid(F, out);
}
void lsdo_pyramid_d(const float* img, int w, int h, int levels, double* out) {
  FrameData<double> F;
  lsdg_intrinsics k{1, 1, 0, 0};
  make_frame<double>(img, w, h, k, levels, F);
  copy_pyramid(F, out);
}

// Depth pyramid (idepth, var planes per level back to back) and points of every level:
// xyzi (4 per point) and var (1 per point), levels back to back; counts[levels].
int lsdo_keyframe_f(const float* img, const float* idepth, const float* var, int w, int h,
                    const lsdg_intrinsics* k, int levels, float* depth_out, float* var_out,
                    float* xyzi, float* pvar, int capacity, int* counts) {
  FrameData<float> F;
  make_frame<float>(img, w, h, *k, levels, F);
  KeyframeData<float> K;
  make_keyframe<float>(F, idepth, var, K);
  size_t off = 0, poff = 0;
  for (int l = 0; l < levels; ++l) {
    size_t n = (size_t)F.cam[l].w * F.cam[l].h;
    if (depth_out) std::memcpy(depth_out + off, K.D[l].data(), n * sizeof(float));
    if (var_out) std::memcpy(var_out + off, K.V[l].data(), n * sizeof(float));
    off += n;
    size_t np = K.pts[l].var.size();
    counts[l] = (int)np;
    if ((int)(poff + np) > capacity) return -1;
    if (xyzi) std::memcpy(xyzi + 4 * poff, K.pts[l].xyzi.data(), 4 * np * sizeof(float));
    if (pvar) std::memcpy(pvar + poff, K.pts[l].var.data(), np * sizeof(float));
    poff += np;
  }
  return 0;
}

}  // extern "C"

template <class T>
static int ne_impl(const float* kimg, const float* idepth, const float* var, const float* fimg, int w,
                   int h, const lsdg_intrinsics* k, const lsdg_params* p, int level,
                   const double ref_to_frame[12], double out[32]) {
  FrameData<T> KF, F;
  make_frame<T>(kimg, w, h, *k, p->levels, KF);
  make_frame<T>(fimg, w, h, *k, p->levels, F);
  KeyframeData<T> K;
  make_keyframe<T>(KF, idepth, var, K);
  if (level < 0 || level >= p->levels) return -1;
  std::vector<T> sig2;
  se3_pass(K.pts[level], F.lv[level], F.cam[level], ref_to_frame, *p, 1, true, sig2, out);
  return 0;
}

// Energy and normal equations at T_eval with the residual variances and the participating points
// fixed by a first pass at T_fix (the quantity one LM level minimises).
template <class T>
static int fixed_impl(const float* kimg, const float* idepth, const float* var, const float* fimg, int w, int h,
                      const lsdg_intrinsics* k, const lsdg_params* p, int level, const double T_fix[12],
                      const double T_eval[12], double out[32]) {
  FrameData<T> KF, F;
  make_frame<T>(kimg, w, h, *k, p->levels, KF);
  make_frame<T>(fimg, w, h, *k, p->levels, F);
  KeyframeData<T> K;
  make_keyframe<T>(KF, idepth, var, K);
  if (level < 0 || level >= p->levels) return -1;
  std::vector<T> sig2;
  double tmp[32];
  se3_pass(K.pts[level], F.lv[level], F.cam[level], T_fix, *p, 1, true, sig2, tmp);
  se3_pass(K.pts[level], F.lv[level], F.cam[level], T_eval, *p, 1, false, sig2, out);
  return 0;
}

extern "C" {

int lsdo_se3_fixed_energy_d(const float* kimg, const float* idepth, const float* var, const float* fimg, int w,
                            int h, const lsdg_intrinsics* k, const lsdg_params* p, int level, const double T_fix[12],
                            const double T_eval[12], double out[32]) {
  return fixed_impl<double>(kimg, idepth, var, fimg, w, h, k, p, level, T_fix, T_eval, out);
}

int lsdo_se3_normal_equations_f(const float* kimg, const float* idepth, const float* var,
                                const float* fimg, int w, int h, const lsdg_intrinsics* k,
                                const lsdg_params* p, int level, const double ref_to_frame[12],
                                double out[32]) {
  return ne_impl<float>(kimg, idepth, var, fimg, w, h, k, p, level, ref_to_frame, out);
}
int lsdo_se3_normal_equations_d(const float* kimg, const float* idepth, const float* var,
                                const float* fimg, int w, int h, const lsdg_intrinsics* k,
                                const lsdg_params* p, int level, const double ref_to_frame[12],
                                double out[32]) {
  return ne_impl<double>(kimg, idepth, var, fimg, w, h, k, p, level, ref_to_frame, out);
}

}  // extern "C"

template <class T>
static int track_impl(const float* kimg, const float* idepth, const float* var, const float* fimg,
                      int w, int h, const lsdg_intrinsics* k, const lsdg_params* p,
                      const double init[12], double out[12], lsdg_track_stats* st, int threads) {
  FrameData<T> KF, F;
  make_frame<T>(kimg, w, h, *k, p->levels, KF);
  make_frame<T>(fimg, w, h, *k, p->levels, F);
  KeyframeData<T> K;
  make_keyframe<T>(KF, idepth, var, K);
  return track_se3<T>(K, F, *p, init, out, st, threads);
}

extern "C" {

int lsdo_track_se3_f(const float* kimg, const float* idepth, const float* var, const float* fimg,
                     int w, int h, const lsdg_intrinsics* k, const lsdg_params* p,
                     const double init[12], double out[12], lsdg_track_stats* st, int threads) {
  return track_impl<float>(kimg, idepth, var, fimg, w, h, k, p, init, out, st, threads);
}
int lsdo_track_trace(int use_double, const float* kimg, const float* idepth, const float* var, const float* fimg,
                     int w, int h, const lsdg_intrinsics* k, const lsdg_params* p, const double init[12],
                     double out[12], lsdg_track_stats* st, double* trace_out, int trace_cap, int* trace_len) {
  std::vector<double> tr;
  g_trace = &tr;
  int rc = use_double ? track_impl<double>(kimg, idepth, var, fimg, w, h, k, p, init, out, st, 1)
                      : track_impl<float>(kimg, idepth, var, fimg, w, h, k, p, init, out, st, 1);
  g_trace = nullptr;
  int n = (int)std::min<size_t>(tr.size(), (size_t)trace_cap);
  std::memcpy(trace_out, tr.data(), n * sizeof(double));
  *trace_len = n / 8;
  return rc;
}

int lsdo_track_se3_d(const float* kimg, const float* idepth, const float* var, const float* fimg,
                     int w, int h, const lsdg_intrinsics* k, const lsdg_params* p,
                     const double init[12], double out[12], lsdg_track_stats* st, int threads) {
  return track_impl<double>(kimg, idepth, var, fimg, w, h, k, p, init, out, st, threads);
}

// The batched workload on the CPU: n independent pairs (arrays back to back, like
// lsdg_batch_load), pairs spread over `threads` std::threads, each pair tracked single-threaded.
// Includes both pyramids and the reference points, as the GPU batch step does.  The float form is
// the CPU baseline, the double form the FP64 oracle of a whole batch.
}  // extern "C"

template <class T>
static int track_batch_impl(int n, const int* widths, const int* heights, const lsdg_intrinsics* intr,
                            const float* ref_images, const float* ref_idepth, const float* ref_var,
                            const float* new_images, const double* init, double* out,
                            lsdg_track_stats* stats, const lsdg_params* p, int threads) {
  std::vector<size_t> off(n + 1, 0);
  for (int i = 0; i < n; ++i) off[i + 1] = off[i] + (size_t)widths[i] * heights[i];
  std::vector<std::thread> th;
  std::atomic<int> next{0};
  auto work = [&] {
    for (;;) {
      int i = next.fetch_add(1);
      if (i >= n) break;
      track_impl<T>(ref_images + off[i], ref_idepth + off[i], ref_var + off[i], new_images + off[i],
                    widths[i], heights[i], &intr[i], p, init + 12 * i, out + 12 * i, &stats[i], 1);
    }
  };
  int nt = std::max(1, threads);
  for (int k = 0; k < nt; ++k) th.emplace_back(work);
  for (auto& t : th) t.join();
  return 0;
}

extern "C" {

int lsdo_track_batch_f(int n, const int* widths, const int* heights, const lsdg_intrinsics* intr,
                       const float* ref_images, const float* ref_idepth, const float* ref_var,
                       const float* new_images, const double* init, double* out,
                       lsdg_track_stats* stats, const lsdg_params* p, int threads) {
  return track_batch_impl<float>(n, widths, heights, intr, ref_images, ref_idepth, ref_var, new_images, init, out,
                                 stats, p, threads);
}

int lsdo_track_batch_d(int n, const int* widths, const int* heights, const lsdg_intrinsics* intr,
                       const float* ref_images, const float* ref_idepth, const float* ref_var,
                       const float* new_images, const double* init, double* out,
                       lsdg_track_stats* stats, const lsdg_params* p, int threads) {
  return track_batch_impl<double>(n, widths, heights, intr, ref_images, ref_idepth, ref_var, new_images, init, out,
                                  stats, p, threads);
}

int lsdo_hardware_threads(void) { return (int)std::thread::hardware_concurrency(); }

}  // extern "C"

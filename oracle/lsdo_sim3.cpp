// lsdo_sim3.cpp -- CPU ORACLE (test infrastructure only) for Sim3Tracker::trackFrameSim3: 7-dof
// (rotation, translation, log-scale) direct alignment of one keyframe to another, with a
// photometric and an inverse-depth residual per point, as in Engel, Schoeps, Cremers, "LSD-SLAM",
// ECCV 2014 sec. 3.3 (the residual r_d = [p']_3 - D_j(p'), variance-normalised, Huber-weighted).
// The lsd-slam code is not available (unvendored fips import, fips.yml:2-4); parity with upstream is
// UNPINNED.  Template on T: float = parity oracle, double = FP64 oracle.
//
// Pose: M = sR (3x3, scale folded in) and t; a point p of keyframe i maps to p' = M p + t in frame j.
// Update: left increment exp(xi) * S, xi = (v, w, sigma):
//   exp(xi) = [e^sigma R(w) | V v],  V = a0 I + a1 K + a2 K^2,  K = [w]x,
//   a0 = int_0^1 e^{s tau} dtau, a1 = int_0^1 e^{s tau} sin(theta tau)/theta dtau,
//   a2 = int_0^1 e^{s tau} (1 - cos(theta tau))/theta^2 dtau  (theta = |w|, s = sigma).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "lsdo.h"

namespace lsdo {

// a0, a1, a2 of V: for theta < 0.05 and |sigma| < 1 the double series
//   a1 = sum_m (-theta^2)^m / (2m+1)! * sum_k sigma^k / (k! (2m+k+2)),
//   a2 = sum_m (-theta^2)^m / (2m+2)! * sum_k sigma^k / (k! (2m+k+3)),  a0 = sum_k sigma^k / (k+1)!
// (m <= 4, k <= 20); otherwise the closed forms of the integrals.
void sim3_coeffs(double th2, double sg, double* a0, double* a1, double* a2) {
  if (th2 < 0.0025 && std::fabs(sg) < 1.0) {
    auto poly = [&](int shift) {  // sum_k sigma^k / (k! (shift + k)), Horner from k = 20
      double f[21];
      f[0] = 1.0;
      for (int k = 1; k <= 20; ++k) f[k] = f[k - 1] * k;
      double acc = 0;
      for (int k = 20; k >= 0; --k) acc = acc * sg + 1.0 / (f[k] * (double)(shift + k));
      return acc;
    };
    double fact[12];
    fact[0] = 1.0;
    for (int k = 1; k < 12; ++k) fact[k] = fact[k - 1] * k;
    *a0 = poly(1);
    double s1 = 0, s2 = 0;
    for (int m = 4; m >= 0; --m) {
      s1 = s1 * (-th2) + poly(2 * m + 2) / fact[2 * m + 1];
      s2 = s2 * (-th2) + poly(2 * m + 3) / fact[2 * m + 2];
    }
    *a1 = s1;
    *a2 = s2;
    return;
  }
  if (th2 < 0.0025) {
    // theta < 0.05, |sigma| >= 1: the same theta series with I_n(sigma) = int_0^1 t^(n-1) e^(sigma t) dt
    // from the upward recurrence I_n = (e^sigma - (n-1) I_(n-1)) / sigma, I_1 = (e^sigma - 1) / sigma.
    // The recurrence amplifies the error of I_1 by (n-1)! / |sigma|^(n-1), which the 1/(n-1)! that
    // multiplies I_n in the series cancels.  (The closed forms below divide by theta.)
    const double es = std::exp(sg), is = 1.0 / sg;
    double I[12];
    I[1] = (es - 1.0) * is;
    for (int n = 2; n <= 11; ++n) I[n] = (es - (double)(n - 1) * I[n - 1]) * is;
    double fact[12];
    fact[0] = 1.0;
    for (int k = 1; k < 12; ++k) fact[k] = fact[k - 1] * k;
    *a0 = I[1];
    double s1 = 0, s2 = 0;
    for (int m = 4; m >= 0; --m) {
      s1 = s1 * (-th2) + I[2 * m + 2] / fact[2 * m + 1];
      s2 = s2 * (-th2) + I[2 * m + 3] / fact[2 * m + 2];
    }
    *a1 = s1;
    *a2 = s2;
    return;
  }
  const double th = std::sqrt(th2), es = std::exp(sg);
  const double sn = std::sin(th), cs = std::cos(th);
  const double D = sg * sg + th2;
  *a0 = std::fabs(sg) < 1e-8 ? 1.0 + 0.5 * sg : (es - 1.0) / sg;
  const double S1 = (es * (sg * sn - th * cs) + th) / D;
  const double C1 = (es * (sg * cs + th * sn) - sg) / D;
  *a1 = S1 / th;
  *a2 = (*a0 - C1) / th2;
}

void sim3_exp(const double xi[7], double T[12]) {
  const double v[3] = {xi[0], xi[1], xi[2]}, w[3] = {xi[3], xi[4], xi[5]}, sg = xi[6];
  const double th2 = (w[0] * w[0] + w[1] * w[1]) + w[2] * w[2];
  double A, B, C, a0, a1, a2;
  se3_coeffs(th2, &A, &B, &C);
  sim3_coeffs(th2, sg, &a0, &a1, &a2);
  const double s = std::exp(sg);
  const double K[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double M[9], V[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const int e = 3 * i + j;
      const double I = (i == j) ? 1.0 : 0.0;
      const double K2 = w[i] * w[j] - ((i == j) ? th2 : 0.0);
      M[e] = s * ((I + A * K[e]) + B * K2);
      V[e] = (a0 * I + a1 * K[e]) + a2 * K2;
    }
  for (int i = 0; i < 3; ++i) {
    T[4 * i + 0] = M[3 * i + 0];
    T[4 * i + 1] = M[3 * i + 1];
    T[4 * i + 2] = M[3 * i + 2];
    T[4 * i + 3] = (V[3 * i + 0] * v[0] + V[3 * i + 1] * v[1]) + V[3 * i + 2] * v[2];
  }
}

// [M | t]^-1 with M = sR: M^-1 = M^T / s^2.
void sim3_inv(const double A[12], double B[12]) {
  const double s2 = (A[0] * A[0] + A[1] * A[1]) + A[2] * A[2];
  double o[12];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) o[4 * i + j] = A[4 * j + i] / s2;
  for (int i = 0; i < 3; ++i) o[4 * i + 3] = -((o[4 * i + 0] * A[3] + o[4 * i + 1] * A[7]) + o[4 * i + 2] * A[11]);
  std::memcpy(B, o, sizeof(o));
}

// 13-double API pose {R (9, unscaled), t (3), s} <-> 3x4 [sR | t]
static void from13(const double* p, double T[12]) {
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) T[4 * i + j] = p[12] * p[3 * i + j];
    T[4 * i + 3] = p[9 + i];
  }
}
static void to13(const double T[12], double* p) {
  const double s = std::sqrt((T[0] * T[0] + T[1] * T[1]) + T[2] * T[2]);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) p[3 * i + j] = T[4 * i + j] / s;
    p[9 + i] = T[4 * i + 3];
  }
  p[12] = s;
}

template <class T>
struct Sim3Sums {
  KSum<T> h[28], g[7], e;
  long n = 0, good = 0, bad = 0, oob = 0;
  void merge(const Sim3Sums& o) {
    for (int i = 0; i < 28; ++i) h[i].merge(o.h[i]);
    for (int i = 0; i < 7; ++i) g[i].merge(o.g[i]);
    e.merge(o.e);
    n += o.n; good += o.good; bad += o.bad; oob += o.oob;
  }
};

// One Sim3 residual pass over [begin, end) of keyframe i's level points against frame j (image Ij
// with the Catmull-Rom interpolant, inverse depth Dj / variance Vj bilinear).  As in the SE3 pass,
// the first pass of a level fixes per point the photometric variance (sig2, 0 = sits out the level)
// and the inverse-depth residual variance (sig2d, 0 = no depth residual in this level).
template <class T>
static void sim3_pass_range(const Points<T>& P, size_t begin, size_t end, const FrameLevel<T>& F,
                            const std::vector<T>& Dj, const std::vector<T>& Vj, const LevelCam& cam,
                            const double Tp[12], const lsdg_params& prm, bool first, T* sig2, T* sig2d,
                            Sim3Sums<T>& S) {
  const T M00 = (T)Tp[0], M01 = (T)Tp[1], M02 = (T)Tp[2], t0 = (T)Tp[3];
  const T M10 = (T)Tp[4], M11 = (T)Tp[5], M12 = (T)Tp[6], t1 = (T)Tp[7];
  const T M20 = (T)Tp[8], M21 = (T)Tp[9], M22 = (T)Tp[10], t2 = (T)Tp[11];
  const T fx = (T)cam.fx, fy = (T)cam.fy, cx = (T)cam.cx, cy = (T)cam.cy;
  const T umax = (T)(cam.w - 2), vmax = (T)(cam.h - 2);
  const T margin = (T)prm.border_margin;
  const T ulo = margin, vlo = margin, uhi = (T)(cam.w - 1) - margin, vhi = (T)(cam.h - 1) - margin;
  const T pvar = (T)prm.photometric_variance, delta = (T)prm.huber_delta, minz = (T)prm.min_z;
  const T dfloor = (T)prm.sim3_depth_variance, wd = (T)prm.sim3_depth_weight;
  const int w = cam.w;
  for (size_t k = begin; k < end; ++k) {
    if (!first && !(sig2[k] > (T)0)) continue;
    const T X = P.xyzi[4 * k + 0], Y = P.xyzi[4 * k + 1], Z = P.xyzi[4 * k + 2], Ik = P.xyzi[4 * k + 3];
    const T Rpx = (M00 * X + M01 * Y) + M02 * Z;
    const T Rpy = (M10 * X + M11 * Y) + M12 * Z;
    const T Rpz = (M20 * X + M21 * Y) + M22 * Z;
    const T Xp = Rpx + t0, Yp = Rpy + t1, Zp = Rpz + t2;
    if (!(Zp > minz)) {
      if (first) { sig2[k] = (T)0; sig2d[k] = (T)0; }
      ++S.oob;
      continue;
    }
    const T iz = (T)1 / Zp;
    const T u = fx * (Xp * iz) + cx;
    const T v = fy * (Yp * iz) + cy;
    if (first) {
      if (!(u >= ulo && v >= vlo && u < uhi && v < vhi)) {
        sig2[k] = (T)0;
        sig2d[k] = (T)0;
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
    const T a0 = (Gx * fx) * iz, a1 = (Gy * fy) * iz;
    const T a2 = -((a0 * Xp + a1 * Yp) * iz);
    T J[7];
    J[0] = a0; J[1] = a1; J[2] = a2;
    J[3] = Yp * a2 - Zp * a1;
    J[4] = Zp * a0 - Xp * a2;
    J[5] = Xp * a1 - Yp * a0;
    J[6] = (a0 * Xp + a1 * Yp) + a2 * Zp;
    // inverse-depth residual against frame j's depth map (4 valid bilinear corners needed)
    const size_t i00 = (size_t)iy * w + ix;
    const T D00 = Dj[i00], D10 = Dj[i00 + 1], D01 = Dj[i00 + w], D11 = Dj[i00 + w + 1];
    bool dok = D00 > (T)0 && D10 > (T)0 && D01 > (T)0 && D11 > (T)0;
    if (!first && !(sig2d[k] > (T)0)) dok = false;
    T rd = 0, Jd[7] = {0, 0, 0, 0, 0, 0, 0}, s2d = 0;
    if (dok) {
      const T bx = (T)1 - ax, by = (T)1 - ay;
      const T w00 = bx * by, w10 = ax * by, w01 = bx * ay, w11 = ax * ay;
      const T Dv = ((w00 * D00 + w10 * D10) + w01 * D01) + w11 * D11;
      const T Ddx = by * (D10 - D00) + ay * (D11 - D01);
      const T Ddy = bx * (D01 - D00) + ax * (D11 - D10);
      rd = iz - Dv;
      const T c0 = (Ddx * fx) * iz, c1 = (Ddy * fy) * iz;
      const T c2 = -((c0 * Xp + c1 * Yp) * iz);
      const T b0 = -c0, b1 = -c1, b2 = -(iz * iz) - c2;
      Jd[0] = b0; Jd[1] = b1; Jd[2] = b2;
      Jd[3] = Yp * b2 - Zp * b1;
      Jd[4] = Zp * b0 - Xp * b2;
      Jd[5] = Xp * b1 - Yp * b0;
      Jd[6] = (b0 * Xp + b1 * Yp) + b2 * Zp;
      if (first) {
        const T Vv = ((w00 * Vj[i00] + w10 * Vj[i00 + 1]) + w01 * Vj[i00 + w]) + w11 * Vj[i00 + w + 1];
        const T bdd = -(((b0 * Rpx + b1 * Rpy) + b2 * Rpz) * Z);
        T sd = Vv + (bdd * bdd) * P.var[k];
        if (sd < dfloor) sd = dfloor;
        sig2d[k] = sd;
      }
      s2d = sig2d[k];
    } else if (first) {
      sig2d[k] = (T)0;
    }
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
    T wgd = 0, rhod = 0;
    if (dok) {
      const T e2d = (rd * rd) / s2d;
      const T aed = std::sqrt(e2d);
      if (aed <= delta) { wgd = wd / s2d; rhod = e2d; }
      else { wgd = (wd * (delta / aed)) / s2d; rhod = delta * ((T)2 * aed - delta); }
    }
    int q = 0;
    for (int i = 0; i < 7; ++i)
      for (int j = i; j < 7; ++j) S.h[q++].add((wgt * J[i]) * J[j] + (wgd * Jd[i]) * Jd[j]);
    for (int i = 0; i < 7; ++i) S.g[i].add((wgt * J[i]) * r + (wgd * Jd[i]) * rd);
    S.e.add(rho + wd * rhod);
    ++S.n;
  }
}

template <class T>
static void sim3_pass(const Points<T>& P, const FrameLevel<T>& F, const std::vector<T>& Dj, const std::vector<T>& Vj,
                      const LevelCam& cam, const double Tp[12], const lsdg_params& prm, bool first,
                      std::vector<T>& sig2, std::vector<T>& sig2d, double out[40]) {
  const size_t n = P.var.size();
  if (sig2.size() != n) sig2.assign(n, (T)0);
  if (sig2d.size() != n) sig2d.assign(n, (T)0);
  Sim3Sums<T> S;
  sim3_pass_range(P, 0, n, F, Dj, Vj, cam, Tp, prm, first, sig2.data(), sig2d.data(), S);
  for (int i = 0; i < 28; ++i) out[i] = S.h[i].value();
  for (int i = 0; i < 7; ++i) out[28 + i] = S.g[i].value();
  out[35] = S.e.value();
  out[36] = (double)S.n;
  out[37] = (double)S.good;
  out[38] = (double)S.bad;
  out[39] = (double)S.oob;
}

// Sim3Tracker::trackFrameSim3: the same LM rules as trackFrame with 7 parameters.
template <class T>
static int track_sim3(const KeyframeData<T>& Ki, const FrameData<T>& Fj, const KeyframeData<T>& Kj,
                      const lsdg_params& prm, const double init13[13], double out13[13], lsdg_track_stats* st) {
  std::memset(st, 0, sizeof(*st));
  double Tinit[12], Tc[12];
  from13(init13, Tinit);
  sim3_inv(Tinit, Tc);  // frame_to_ref given -> ref_to_frame
  double S[40] = {0};
  bool have_final = false;
  for (int lvl = prm.levels - 1; lvl >= 0; --lvl) {
    const Points<T>& P = Ki.pts[lvl];
    if (P.var.empty()) continue;
    const LevelCam& cam = Fj.cam[lvl];
    std::vector<T> sig2, sig2d;
    sim3_pass(P, Fj.lv[lvl], Kj.D[lvl], Kj.V[lvl], cam, Tc, prm, true, sig2, sig2d, S);
    st->passes[lvl]++;
    if (!(S[36] > 0)) continue;
    double E = S[35] / S[36];
    double lambda = prm.lm_lambda_initial;
    const double thr = (double)prm.step_eps * (double)(1 << lvl);
    const double stall = (double)prm.stall_eps * (double)(1 << lvl);
    bool fresh = true;
    double gnmax = 1e300;
    for (int it = 0;;) {
      if (fresh) {
        double gn[7];
        gnmax = 1e300;
        if (ldlt_solve(7, S, S + 28, 0.0, gn)) {
          gnmax = 0;
          for (int i = 0; i < 7; ++i) gnmax = std::max(gnmax, std::fabs(gn[i]));
          if (gnmax < thr) break;
        }
        fresh = false;
      }
      if (it >= prm.max_iterations[lvl]) break;
      ++it;
      double dx[7];
      if (!ldlt_solve(7, S, S + 28, lambda, dx)) {
        lambda *= prm.lm_lambda_up;
        continue;
      }
      double Ex[12], Tt[12];
      sim3_exp(dx, Ex);
      se3_mul(Ex, Tc, Tt);
      double S2[40];
      sim3_pass(P, Fj.lv[lvl], Kj.D[lvl], Kj.V[lvl], cam, Tt, prm, false, sig2, sig2d, S2);
      st->passes[lvl]++;
      if (S2[36] > 0 && S2[35] / S2[36] < E) {
        std::memcpy(Tc, Tt, sizeof(Tc));
        std::memcpy(S, S2, sizeof(S));
        E = S2[35] / S2[36];
        lambda *= prm.lm_lambda_down;
        fresh = true;
      } else {
        if (gnmax < stall) break;
        lambda *= prm.lm_lambda_up;
      }
    }
    if (lvl == 0) have_final = true;
  }
  double Tout[12];
  sim3_inv(Tc, Tout);
  to13(Tout, out13);
  for (int l = 0; l < LSDG_MAX_LEVELS; ++l) st->total_passes += st->passes[l];
  st->n_points = (int)Ki.pts[0].var.size();
  if (have_final) {
    st->n_valid = (int)S[36];
    st->n_good = (int)S[37];
    st->mean_energy = S[36] > 0 ? (float)(S[35] / S[36]) : 0.f;
    st->good_ratio = S[36] > 0 ? (float)(S[37] / S[36]) : 0.f;
    st->usage = st->n_points > 0 ? (float)(S[36] / st->n_points) : 0.f;
    for (int i = 0; i < 28; ++i) st->hessian[i] = S[i];
  }
  const int status = (!have_final || st->good_ratio < prm.min_good_ratio || st->usage < prm.min_usage)
                         ? LSDG_TRACKING_LOST : LSDG_OK;
  st->status = status;
  return status;
}

template <class T>
static void build_both(const float* img_i, const float* id_i, const float* var_i, const float* img_j,
                       const float* id_j, const float* var_j, int w, int h, const lsdg_intrinsics& k, int levels,
                       KeyframeData<T>& Ki, FrameData<T>& Fj, KeyframeData<T>& Kj) {
  FrameData<T> Fi;
  make_frame<T>(img_i, w, h, k, levels, Fi);
  make_keyframe<T>(Fi, id_i, var_i, Ki);
  make_frame<T>(img_j, w, h, k, levels, Fj);
  make_keyframe<T>(Fj, id_j, var_j, Kj);
}

}  // namespace lsdo

using namespace lsdo;

template <class T>
static int sim3_ne_impl(const float* img_i, const float* id_i, const float* var_i, const float* img_j,
                        const float* id_j, const float* var_j, int w, int h, const lsdg_intrinsics* k,
                        const lsdg_params* p, int level, const double ref_to_frame13[13], double out[40]) {
  KeyframeData<T> Ki, Kj;
  FrameData<T> Fj;
  build_both<T>(img_i, id_i, var_i, img_j, id_j, var_j, w, h, *k, p->levels, Ki, Fj, Kj);
  if (level < 0 || level >= p->levels) return -1;
  double Tp[12];
  from13(ref_to_frame13, Tp);
  std::vector<T> sig2, sig2d;
  sim3_pass(Ki.pts[level], Fj.lv[level], Kj.D[level], Kj.V[level], Fj.cam[level], Tp, *p, true, sig2, sig2d, out);
  return 0;
}

template <class T>
static int sim3_track_impl(const float* img_i, const float* id_i, const float* var_i, const float* img_j,
                           const float* id_j, const float* var_j, int w, int h, const lsdg_intrinsics* k,
                           const lsdg_params* p, const double init13[13], double out13[13], lsdg_track_stats* st) {
  KeyframeData<T> Ki, Kj;
  FrameData<T> Fj;
  build_both<T>(img_i, id_i, var_i, img_j, id_j, var_j, w, h, *k, p->levels, Ki, Fj, Kj);
  return track_sim3<T>(Ki, Fj, Kj, *p, init13, out13, st);
}

extern "C" {

int lsdo_sim3_normal_equations(int use_double, const float* img_i, const float* id_i, const float* var_i,
                               const float* img_j, const float* id_j, const float* var_j, int w, int h,
                               const lsdg_intrinsics* k, const lsdg_params* p, int level,
                               const double ref_to_frame13[13], double out[40]) {
  return use_double ? sim3_ne_impl<double>(img_i, id_i, var_i, img_j, id_j, var_j, w, h, k, p, level, ref_to_frame13, out)
                    : sim3_ne_impl<float>(img_i, id_i, var_i, img_j, id_j, var_j, w, h, k, p, level, ref_to_frame13, out);
}

int lsdo_track_sim3(int use_double, const float* img_i, const float* id_i, const float* var_i, const float* img_j,
                    const float* id_j, const float* var_j, int w, int h, const lsdg_intrinsics* k,
                    const lsdg_params* p, const double init13[13], double out13[13], lsdg_track_stats* st) {
  return use_double ? sim3_track_impl<double>(img_i, id_i, var_i, img_j, id_j, var_j, w, h, k, p, init13, out13, st)
                    : sim3_track_impl<float>(img_i, id_i, var_i, img_j, id_j, var_j, w, h, k, p, init13, out13, st);
}

// exp of a sim(3) twist, for tests: out = [sR | t] (12 doubles).
void lsdo_sim3_exp(const double xi[7], double out[12]) { sim3_exp(xi, out); }

}  // extern "C"

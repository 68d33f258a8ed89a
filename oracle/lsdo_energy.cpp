// lsdo_energy.cpp -- CPU ORACLE (test infrastructure only) of the differentiable photometric
// energy of a keyframe against a frame, its adjoint, and the per-point inverse-depth refinement
// that the adjoint drives.  There is no upstream counterpart (the energy and its backward are new);
// the residual model is the tracker's: the same points, the same Catmull-Rom sampling of the frame
// and the same Huber norm (see lsdo_track.cpp, se3_pass_range).  Template on T: float mirrors the
// kernels' operation order (parity oracle), double is the FP64 oracle of the finite-difference
// checks.
//
// Energy of keyframe level l against frame F at pose M (ref_to_frame, [M | t], M = R or sR):
//   point i: pixel (x_i, y_i), ray q_i = ((x - cx) / fx, (y - cy) / fy, 1), inverse depth rho_i,
//   p_i = q_i / rho_i,  p'_i = M p_i + t,  r_i = I_F(pi(p'_i)) - I_key(x_i, y_i),
//   E = sum_i h(r_i^2 / s_i),  h(e2) = e2 for sqrt(e2) <= delta, else delta (2 sqrt(e2) - delta)
// with s_i = sigma2[i] when given, else the photometric variance.  The point takes part when
// z' > min_z and its projection lies inside the border margin (the tracker's first-pass test).
// Gradients (IRLS weight w_i = (1, or delta / |r_i / sqrt(s_i)|) / s_i):
//   dE/dxi    = sum_i 2 w_i r_i J_i           (J_i: the calculateWarpUpdate Jacobian, left increment)
//   dE/drho_i = 2 w_i r_i (dr_i/dp') . (-(M p_i) / rho_i)
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "lsdo.h"

namespace lsdo {

// One observation of point (qx, qy, rho) in a frame level: residual, its IRLS weight and the
// derivatives.  `sample_box`: 0 = the margin box (first-pass participation test), 1 = the sampling
// box [1, w - 2) x [1, h - 2) only.  Returns false when the observation is not available.
template <class T>
struct Obs {
  T r, e2, rho_h, wgt;  // residual, squared normalised residual, Huber energy, IRLS weight / s
  T a0, a1, a2;         // dr/dp' (projected image gradient over z')
  T Xp, Yp, Zp, Rpx, Rpy, Rpz, z;
};

template <class T>
static inline bool observe(T qx, T qy, T rho, T Ik, T s2, const FrameLevel<T>& F, const LevelCam& cam,
                           const T M[12], const lsdg_params& prm, int sample_box, Obs<T>& o) {
  if (!(rho > (T)0)) return false;
  const T z = (T)1 / rho;
  const T X = qx * z, Y = qy * z, Z = z;
  const T Rpx = (M[0] * X + M[1] * Y) + M[2] * Z;
  const T Rpy = (M[4] * X + M[5] * Y) + M[6] * Z;
  const T Rpz = (M[8] * X + M[9] * Y) + M[10] * Z;
  const T Xp = Rpx + M[3], Yp = Rpy + M[7], Zp = Rpz + M[11];
  if (!(Zp > (T)prm.min_z)) return false;
  const T iz = (T)1 / Zp;
  const T fx = (T)cam.fx, fy = (T)cam.fy, cx = (T)cam.cx, cy = (T)cam.cy;
  const T u = fx * (Xp * iz) + cx;
  const T v = fy * (Yp * iz) + cy;
  if (sample_box == 0) {
    const T m = (T)prm.border_margin;
    if (!(u >= m && v >= m && u < (T)(cam.w - 1) - m && v < (T)(cam.h - 1) - m)) return false;
  } else if (!(u >= (T)1 && v >= (T)1 && u < (T)(cam.w - 2) && v < (T)(cam.h - 2))) {
    return false;
  }
  const int w = cam.w;
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
  o.r = In - Ik;
  o.a0 = (Gx * fx) * iz;
  o.a1 = (Gy * fy) * iz;
  o.a2 = -((o.a0 * Xp + o.a1 * Yp) * iz);
  const T delta = (T)prm.huber_delta;
  o.e2 = (o.r * o.r) / s2;
  const T ae = std::sqrt(o.e2);
  T wh;
  if (ae <= delta) { wh = (T)1; o.rho_h = o.e2; }
  else { wh = delta / ae; o.rho_h = delta * ((T)2 * ae - delta); }
  o.wgt = wh / s2;
  o.Xp = Xp; o.Yp = Yp; o.Zp = Zp;
  o.Rpx = Rpx; o.Rpy = Rpy; o.Rpz = Rpz;
  o.z = z;
  return true;
}

// dr/drho of an observation: dp'/drho = -(M p) / rho = -(M p) z.
template <class T>
static inline T drho_of(const Obs<T>& o) {
  return -(((o.a0 * o.Rpx + o.a1 * o.Rpy) + o.a2 * o.Rpz) * o.z);
}

// The energy points of keyframe level l: rays from the pixel index, keyframe intensity, initial
// inverse depth (the level's depth plane at the pixel).  Same set and order as the tracking points.
template <class T>
struct EPoints {
  std::vector<T> qx, qy, Ik, var;  // var: the keyframe's inverse-depth variance of the point
  std::vector<float> rho0;
  std::vector<int> pix;
};

template <class T>
static void energy_points(const KeyframeData<T>& K, int level, EPoints<T>& E) {
  const Points<T>& P = K.pts[level];
  const LevelCam& cam = K.cam[level];
  const T cx = (T)cam.cx, cy = (T)cam.cy, fxi = (T)cam.fxi, fyi = (T)cam.fyi;
  const size_t n = P.pix.size();
  E.qx.resize(n); E.qy.resize(n); E.Ik.resize(n); E.rho0.resize(n); E.pix = P.pix; E.var = P.var;
  for (size_t k = 0; k < n; ++k) {
    const int x = P.pix[k] % cam.w, y = P.pix[k] / cam.w;
    E.qx[k] = ((T)x - cx) * fxi;
    E.qy[k] = ((T)y - cy) * fyi;
    E.Ik[k] = P.xyzi[4 * k + 3];
    E.rho0[k] = (float)K.D[level][P.pix[k]];
  }
}

// Forward (and backward when gxi / grho are given) over all points, sequential Kahan sums.
// fixed_active (optional): the participation of every point is taken from it (the sampling box
// must still hold, else the call reports the point in `broken`), for finite differences at a
// frozen point set.
template <class T>
static void energy_eval(const EPoints<T>& P, const float* rho, const float* sig2, const FrameLevel<T>& F,
                        const LevelCam& cam, const double Tp[12], int dof, const lsdg_params& prm,
                        const unsigned char* fixed_active, double* E_out, double* gxi, double* grho,
                        double* e_point, unsigned char* active_out, int* n_active, int* broken) {
  T M[12];
  for (int i = 0; i < 12; ++i) M[i] = (T)Tp[i];
  KSum<T> E, G[7];
  int na = 0, nb = 0;
  const size_t n = P.qx.size();
  for (size_t k = 0; k < n; ++k) {
    const T s2 = sig2 ? (T)sig2[k] : (T)prm.photometric_variance;
    const T rk = rho ? (T)rho[k] : (T)P.rho0[k];
    Obs<T> o;
    bool ok;
    if (fixed_active) {
      ok = fixed_active[k] && observe<T>(P.qx[k], P.qy[k], rk, P.Ik[k], s2, F, cam, M, prm, 1, o);
      if (fixed_active[k] && !ok) ++nb;
    } else {
      ok = observe<T>(P.qx[k], P.qy[k], rk, P.Ik[k], s2, F, cam, M, prm, 0, o);
    }
    if (active_out) active_out[k] = ok ? 1 : 0;
    if (e_point) e_point[k] = ok ? (double)o.rho_h : 0.0;
    if (!ok) {
      if (grho) grho[k] = 0.0;
      continue;
    }
    ++na;
    E.add(o.rho_h);
    const T c = ((T)2 * o.wgt) * o.r;  // dh/dr
    if (gxi) {
      T J[7];
      J[0] = o.a0; J[1] = o.a1; J[2] = o.a2;
      J[3] = o.Yp * o.a2 - o.Zp * o.a1;
      J[4] = o.Zp * o.a0 - o.Xp * o.a2;
      J[5] = o.Xp * o.a1 - o.Yp * o.a0;
      J[6] = (o.a0 * o.Xp + o.a1 * o.Yp) + o.a2 * o.Zp;
      for (int i = 0; i < dof; ++i) G[i].add(c * J[i]);
    }
    if (grho) grho[k] = (double)(c * drho_of(o));
  }
  *E_out = E.value();
  if (gxi)
    for (int i = 0; i < dof; ++i) gxi[i] = G[i].value();
  if (n_active) *n_active = na;
  if (broken) *broken = nb;
}

// ------------------------------------------------------------------------------------------
// Inverse-depth refinement: every point independently (poses fixed), damped Newton steps on its
// own energy E_i(rho) = sum over observing frames of h(r^2 / s) + k_i (rho - rho_i0)^2, a Gaussian
// prior at the starting value with k_i = refine_prior_weight / var_i (the keyframe's variance of the
// point), so that points whose image gradient gives no depth information stay put (MAP estimate of
// the depth filter's hypothesis and the photometric evidence).  The frames observing a point are
// fixed at the start (margin test at rho0); a trial whose projection leaves the sampling box in
// one of them is rejected.  Per step: d = -g / (H (1 + lambda)), g = dE_i/drho, H = sum 2 w (dr/drho)^2
// (Gauss-Newton curvature of E_i); rho_t clamped to [min_idepth, max_idepth]; accepted when
// E_i(rho_t) < E_i(rho) (lambda *= lambda_down), else lambda *= lambda_up.  The per-point sums over
// frames use the kernels' grouping: frame j goes to slot j mod 8 (ascending j within a slot), then
// the slots are added pairwise ((0+4) + (2+6)) + ((1+5) + (3+7)).
// ------------------------------------------------------------------------------------------
constexpr int kSlots = 8;

template <class T>
struct PointSums {
  T E, g, H;
  bool ok;
};

template <class T>
static PointSums<T> point_sums(const EPoints<T>& P, size_t k, T rho, T rho0, T pk, T s2, int nf,
                               const FrameLevel<T>* const* F, const LevelCam& cam, const T (*M)[12],
                               const lsdg_params& prm, unsigned mask, bool first, unsigned* mask_out) {
  T e[kSlots], g[kSlots], h[kSlots];
  for (int s = 0; s < kSlots; ++s) e[s] = g[s] = h[s] = (T)0;
  bool ok = true;
  unsigned m = 0;
  for (int j = 0; j < nf; ++j) {
    if (!first && !((mask >> j) & 1u)) continue;
    Obs<T> o;
    const bool got = observe<T>(P.qx[k], P.qy[k], rho, P.Ik[k], s2, *F[j], cam, M[j], prm, first ? 0 : 1, o);
    if (!got) {
      if (!first) ok = false;
      continue;
    }
    m |= 1u << j;
    const T jr = drho_of(o);
    const T c = (T)2 * o.wgt;
    const int s = j % kSlots;
    e[s] = e[s] + o.rho_h;
    g[s] = g[s] + (c * o.r) * jr;
    h[s] = h[s] + (c * jr) * jr;
  }
  auto tree = [](const T* a) {
    const T s0 = a[0] + a[4], s1 = a[1] + a[5], s2_ = a[2] + a[6], s3 = a[3] + a[7];
    return (s0 + s2_) + (s1 + s3);
  };
  if (mask_out) *mask_out = m;
  const T dq = rho - rho0;
  const T pe = (pk * dq) * dq, pg = ((T)2 * pk) * dq, ph = (T)2 * pk;
  return PointSums<T>{tree(e) + pe, tree(g) + pg, tree(h) + ph, ok};
}

template <class T>
static void refine_range(const EPoints<T>& P, size_t begin, size_t end, float* rho_io, const float* sig2, int nf,
                         const FrameLevel<T>* const* F, const LevelCam& cam, const T (*M)[12],
                         const lsdg_params& prm, int steps, KSum<T>* E0, KSum<T>* E1, long* refined) {
  const T lo = (T)prm.min_idepth, hi = (T)prm.max_idepth;
  const T up = (T)prm.lm_lambda_up, down = (T)prm.lm_lambda_down;
  for (size_t k = begin; k < end; ++k) {
    const T s2 = sig2 ? (T)sig2[k] : (T)prm.photometric_variance;
    T rho = (T)rho_io[k];
    const T rho0 = rho;
    const T pk = (T)prm.refine_prior_weight / P.var[k];
    unsigned mask = 0;
    PointSums<T> cur = point_sums<T>(P, k, rho, rho0, pk, s2, nf, F, cam, M, prm, 0u, true, &mask);
    E0->add(cur.E);
    if (mask != 0u && cur.H > (T)0) {
      T lam = (T)prm.lm_lambda_initial;
      for (int s = 0; s < steps; ++s) {
        const T d = -(cur.g / (cur.H * ((T)1 + lam)));
        T rt = rho + d;
        rt = rt < lo ? lo : (rt > hi ? hi : rt);
        const PointSums<T> t = point_sums<T>(P, k, rt, rho0, pk, s2, nf, F, cam, M, prm, mask, false, nullptr);
        const bool better = (t.E) < (cur.E);
        if (t.ok && better && (t.H) > (T)0) {
          rho = rt;
          cur = t;
          lam = lam * down;
        } else {
          lam = lam * up;
        }
      }
      ++*refined;
    }
    E1->add(cur.E);
    rho_io[k] = (float)rho;
  }
}

template <class T>
static int energy_impl(const float* kimg, const float* kid, const float* kvar, const float* fimg, int w, int h,
                       const lsdg_intrinsics* k, const lsdg_params* p, int level, const double Tp[12], int dof,
                       const float* rho, const float* sig2, const unsigned char* fixed_active, double* E,
                       double* gxi, double* grho, double* e_point, unsigned char* active_out, int* n_active,
                       int* broken) {
  if (level < 0 || level >= p->levels || (dof != 6 && dof != 7)) return -1;
  FrameData<T> Fk, Ff;
  make_frame<T>(kimg, w, h, *k, p->levels, Fk);
  KeyframeData<T> K;
  make_keyframe<T>(Fk, kid, kvar, K);
  make_frame<T>(fimg, w, h, *k, p->levels, Ff);
  EPoints<T> P;
  energy_points<T>(K, level, P);
  energy_eval<T>(P, rho, sig2, Ff.lv[level], Ff.cam[level], Tp, dof, *p, fixed_active, E, gxi, grho, e_point,
                 active_out, n_active, broken);
  return 0;
}

template <class T>
static int refine_impl(const float* kimg, const float* kid, const float* kvar, int nf, const float* fimgs, int w,
                       int h, const lsdg_intrinsics* k, const lsdg_params* p, int level, const double* Tps,
                       int steps, const float* sig2, float* rho_io, double* E0, double* E1, long* refined,
                       int threads) {
  if (level < 0 || level >= p->levels || nf < 1 || nf > LSDG_MAX_REFS) return -1;
  FrameData<T> Fk;
  make_frame<T>(kimg, w, h, *k, p->levels, Fk);
  KeyframeData<T> K;
  make_keyframe<T>(Fk, kid, kvar, K);
  EPoints<T> P;
  energy_points<T>(K, level, P);
  std::vector<FrameData<T>> Fs(nf);
  std::vector<const FrameLevel<T>*> Fl(nf);
  std::vector<std::array<T, 12>> Ms(nf);
  for (int j = 0; j < nf; ++j) {
    make_frame<T>(fimgs + (size_t)j * w * h, w, h, *k, p->levels, Fs[j]);
    Fl[j] = &Fs[j].lv[level];
    for (int i = 0; i < 12; ++i) Ms[j][i] = (T)Tps[12 * j + i];
  }
  const T(*M)[12] = reinterpret_cast<const T(*)[12]>(Ms.data());
  const size_t n = P.qx.size();
  if (threads < 1) threads = 1;
  std::vector<KSum<T>> e0(threads), e1(threads);
  std::vector<long> cnt(threads, 0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    const size_t b = n * t / threads, e = n * (t + 1) / threads;
    pool.emplace_back([&, b, e, t] {
      refine_range<T>(P, b, e, rho_io, sig2, nf, Fl.data(), Fk.cam[level], M, *p, steps, &e0[t], &e1[t], &cnt[t]);
    });
  }
  for (auto& th : pool) th.join();
  KSum<T> a, b;
  long c = 0;
  for (int t = 0; t < threads; ++t) { a.merge(e0[t]); b.merge(e1[t]); c += cnt[t]; }
  *E0 = a.value();
  *E1 = b.value();
  if (refined) *refined = c;
  return 0;
}

}  // namespace lsdo

using namespace lsdo;

extern "C" {

// The energy points of a keyframe level: count, and optionally the pixel index and the initial
// inverse depth of each (arrays of the level's pixel count at most).
int lsdo_energy_points(const float* kimg, const float* kid, const float* kvar, int w, int h, const lsdg_intrinsics* k,
                       const lsdg_params* p, int level, int* pix_out, float* rho0_out) {
  FrameData<float> Fk;
  make_frame<float>(kimg, w, h, *k, p->levels, Fk);
  KeyframeData<float> K;
  make_keyframe<float>(Fk, kid, kvar, K);
  EPoints<float> P;
  energy_points<float>(K, level, P);
  const int n = (int)P.pix.size();
  for (int i = 0; i < n; ++i) {
    if (pix_out) pix_out[i] = P.pix[i];
    if (rho0_out) rho0_out[i] = P.rho0[i];
  }
  return n;
}

// Energy (and its gradients when gxi / grho are given) of keyframe level `level` against frame
// `fimg` at ref_to_frame Tp (12 doubles, [M | t]).  rho / sig2 (optional): per-point inverse depth
// and residual variance.  e_point (optional): each point's energy term.  fixed_active / active_out
// (optional): participation input (frozen set) / output.  broken: frozen points whose projection
// left the sampling box.
int lsdo_energy(int use_double, const float* kimg, const float* kid, const float* kvar, const float* fimg, int w,
                int h, const lsdg_intrinsics* k, const lsdg_params* p, int level, const double Tp[12], int dof,
                const float* rho, const float* sig2, const unsigned char* fixed_active, double* E, double* gxi,
                double* grho, double* e_point, unsigned char* active_out, int* n_active, int* broken) {
  return use_double ? energy_impl<double>(kimg, kid, kvar, fimg, w, h, k, p, level, Tp, dof, rho, sig2, fixed_active,
                                          E, gxi, grho, e_point, active_out, n_active, broken)
                    : energy_impl<float>(kimg, kid, kvar, fimg, w, h, k, p, level, Tp, dof, rho, sig2, fixed_active,
                                         E, gxi, grho, e_point, active_out, n_active, broken);
}

// Per-point inverse-depth refinement over nf frames (images back to back, ref_to_frame poses 12
// doubles each); rho_io holds the initial inverse depths (the level's points in order) and
// receives the refined ones.  E0 / E1: total energy before / after.
int lsdo_energy_refine(int use_double, const float* kimg, const float* kid, const float* kvar, int nf,
                       const float* fimgs, int w, int h, const lsdg_intrinsics* k, const lsdg_params* p, int level,
                       const double* Tps, int steps, const float* sig2, float* rho_io, double* E0, double* E1,
                       long* refined, int threads) {
  return use_double ? refine_impl<double>(kimg, kid, kvar, nf, fimgs, w, h, k, p, level, Tps, steps, sig2, rho_io, E0,
                                          E1, refined, threads)
                    : refine_impl<float>(kimg, kid, kvar, nf, fimgs, w, h, k, p, level, Tps, steps, sig2, rho_io, E0,
                                         E1, refined, threads);
}

}  // extern "C"

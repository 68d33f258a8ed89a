// lsdo_depth.cpp -- CPU ORACLE (test infrastructure only) for the semi-dense inverse-depth filter of
// the LSD-SLAM hot path: DepthMap::updateKeyframe -> observeDepth (epipolar line search + fusion),
// regularizeDepthMap (+ hole filling) and DepthMap::createKeyFrame -> propagateDepth.
//
// The reference repository does not contain DepthMap (it lives in the unvendored lsd-slam fips
// import, fips.yml:2-4); this file restates the published method -- Engel, Sturm, Cremers,
// "Semi-Dense Visual Odometry for a Monocular Camera", ICCV 2013: sec. 2.1 stereo on the epipolar
// line (5 equidistant samples, SSD), sec. 2.1.1-2.1.3 geometric disparity error
// sigma_l^2 / <g, l>^2 and photometric disparity error 2 sigma_i^2 / g_p^2, scaled to inverse depth
// by alpha = d(idepth)/d(lambda); sec. 2.2 Gaussian fusion of the observation with the prior;
// sec. 2.3 propagation with sigma'^2 = (d'/d)^4 sigma^2 + sigma_p^2; sec. 2.4 regularisation over a
// neighbourhood with outlier removal -- with this project's own parameter table (lsdg_params).
// Parity with upstream is UNPINNED (no upstream tests or golden vectors exist).
//
// Template on T: float is the parity oracle (every operation in the order the CUDA kernels use;
// built with -ffp-contract=off), double the FP64 oracle.  Poses enter in double and the per-reference
// geometry is formed in double and rounded to T, as the product's host code does.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "lsdo.h"

namespace lsdo {

template <class T>
struct DepthState {
  std::vector<T> d, v, sm, vsm;
  std::vector<int> val, bl;
  void init(size_t n) {
    d.assign(n, (T)-1); v.assign(n, (T)-1); sm.assign(n, (T)-1); vsm.assign(n, (T)-1);
    val.assign(n, 0); bl.assign(n, 0);
  }
};

// ---------------------------------------------------------------------------------------------
// Decision trace (tests only): every threshold decision of the filter can be recorded for the
// pixels of a mask, with the quantity it compares and its threshold, so that a test can find, for
// a pixel whose flags differ between the float and the FP64 runs, the first decision the two runs
// took differently and check that it straddles its threshold by a rounding-sized margin.  Tracing
// runs single-threaded; with no trace installed `note` is one predictable branch and changes no
// arithmetic (it receives values already computed).
// ---------------------------------------------------------------------------------------------
enum DecisionId {
  D_GRAD = 1, D_EPL, D_COS, D_AZ, D_EPLLEN, D_RANGE, D_Z, D_PAD, D_MAXLEN, D_ORIENT, D_NWIN, D_SAMPLE, D_WIN,
  D_ARGMIN, D_MAXSSD, D_UNIQUE, D_DEN, D_CLAMP_HI, D_CLAMP_LO, D_AXIS, D_DOBS, D_INIT, D_CHI2, D_VALDROP,
  D_BLLIMIT, D_RUNBEST, D_RUN2,
  D_R_HASDEPTH = 40, D_R_NVAL, D_R_COMPAT, D_R_SUPPORT, D_R_FILL,
  D_P_Z = 60, D_P_RX, D_P_RY, D_P_BOUND, D_P_PHOTO
};

struct DecisionRec {
  int32_t pixel, stage, ref, id, outcome, aux;
  double q, thr;
};

struct TraceSink {
  std::vector<DecisionRec>* out = nullptr;
  const uint8_t* mask = nullptr;  // [stage][pixel]: which pixels of which stage are traced
  size_t npix = 0;
  int pixel = 0, stage = 0, ref = 0;
};
static thread_local TraceSink t_sink;

static inline bool tracing() { return t_sink.out && t_sink.mask[(size_t)t_sink.stage * t_sink.npix + t_sink.pixel]; }

template <class T>
static inline bool note(int id, T q, T thr, bool outcome, int aux = 0) {
  if (tracing())
    t_sink.out->push_back({t_sink.pixel, t_sink.stage, t_sink.ref, id, outcome ? 1 : 0, aux, (double)q, (double)thr});
  return outcome;
}

template <class T>
static inline void note_value(int id, int value, T q, T thr, int aux = 0) {
  if (tracing()) t_sink.out->push_back({t_sink.pixel, t_sink.stage, t_sink.ref, id, value, aux, (double)q, (double)thr});
}

// Per-reference geometry: a(u) = K R K^-1 (x, y, 1), b = K t: the reference pixel of inverse depth
// d is (a.xy + b.xy d) / (a.z + b.z d).  c = -R^T t is the reference camera centre in the keyframe.
template <class T>
struct RefGeom {
  T M[9], b[3], c[3];
};

template <class T>
static RefGeom<T> ref_geom(const double P[12], double fx, double fy, double cx, double cy) {
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
  RefGeom<T> g;
  for (int i = 0; i < 9; ++i) g.M[i] = (T)M[i];
  for (int i = 0; i < 3; ++i) {
    g.b[i] = (T)((K[3 * i + 0] * t[0] + K[3 * i + 1] * t[1]) + K[3 * i + 2] * t[2]);
    g.c[i] = (T)(-((R[0 + i] * t[0] + R[3 + i] * t[1]) + R[6 + i] * t[2]));
  }
  return g;
}

template <class T>
static inline T bilinear(const T* I, int w, T x, T y) {
  const int ix = (int)x, iy = (int)y;
  const T ax = x - (T)ix, ay = y - (T)iy;
  const T bx = (T)1 - ax, by = (T)1 - ay;
  const T* p = I + (size_t)iy * w + ix;
  return (((bx * by) * p[0] + (ax * by) * p[1]) + (bx * ay) * p[w]) + (ax * ay) * p[w + 1];
}

// observeDepth for one pixel against one reference frame.  State (d, var, validity, blacklist) is
// updated in place.  Returns nothing; every early exit leaves the state unchanged unless noted.
template <class T>
static void observe_pixel(int x, int y, int w, int h, const T* Ik, const T* gxk, const T* gyk, const T* Ir,
                          const RefGeom<T>& G, T fx, T fy, T cx, T cy, const lsdg_params& p, T& d, T& var, int& val,
                          int& bl) {
  const size_t i = (size_t)y * w + x;
  const T gx = gxk[i], gy = gyk[i];
  const T g2 = gx * gx + gy * gy;
  const T mg = (T)p.min_grad;
  if (!note(D_GRAD, g2, mg * mg, g2 >= mg * mg)) return;
  const T xf = (T)x, yf = (T)y;
  // keyframe epipolar direction (away from the epipole of the reference camera)
  T lkx = G.c[2] * (xf - cx) - fx * G.c[0];
  T lky = G.c[2] * (yf - cy) - fy * G.c[1];
  const T el2 = lkx * lkx + lky * lky;
  if (!note(D_EPL, el2, (T)1e-12, el2 > (T)1e-12)) return;
  const T einv = (T)1 / std::sqrt(el2);
  lkx = lkx * einv;
  lky = lky * einv;
  const T gp = gx * lkx + gy * lky;
  const T cos2 = (gp * gp) / g2;
  if (!note(D_COS, cos2, (T)p.min_grad_along_epl2, cos2 >= (T)p.min_grad_along_epl2)) return;
  const T ax = (G.M[0] * xf + G.M[1] * yf) + G.M[2];
  const T ay = (G.M[3] * xf + G.M[4] * yf) + G.M[5];
  const T az = (G.M[6] * xf + G.M[7] * yf) + G.M[8];
  const T bx = G.b[0], by = G.b[1], bz = G.b[2];
  if (!note(D_AZ, az, (T)0, az > (T)0)) return;
  // reference epipolar direction (increasing inverse depth) and disparity per unit inverse depth
  const T rx = bx * az - ax * bz, ry = by * az - ay * bz;
  const T rn = std::sqrt(rx * rx + ry * ry);
  if (!note(D_EPLLEN, rn / (az * az), (T)p.min_epl_length, rn / (az * az) >= (T)p.min_epl_length)) return;
  const T lrx = rx / rn, lry = ry / rn;
  // search range in inverse depth
  T dlo, dhi;
  if (val > 0) {
    const T sd = std::sqrt(var);
    dlo = d - (T)p.search_sigmas * sd;
    dhi = d + (T)p.search_sigmas * sd;
    if (dlo < (T)p.min_idepth) dlo = (T)p.min_idepth;
    if (dhi > (T)p.max_idepth) dhi = (T)p.max_idepth;
  } else {
    dlo = (T)p.min_idepth;
    dhi = (T)p.max_idepth;
  }
  if (!note(D_RANGE, dlo, dhi, dlo < dhi)) return;
  const T zlo = az + bz * dlo, zhi = az + bz * dhi;
  if (!note(D_Z, zlo < zhi ? zlo : zhi, (T)0, zlo > (T)0 && zhi > (T)0)) return;
  T pfx = (ax + bx * dlo) / zlo, pfy = (ay + by * dlo) / zlo;
  const T pnx = (ax + bx * dhi) / zhi, pny = (ay + by * dhi) / zhi;
  T L = (pnx - pfx) * lrx + (pny - pfy) * lry;
  if (note(D_PAD, L, (T)p.min_search_len, L < (T)p.min_search_len)) {
    const T pad = ((T)p.min_search_len - L) * (T)0.5;
    pfx = pfx - lrx * pad;
    pfy = pfy - lry * pad;
    L = (T)p.min_search_len;
  }
  if (note(D_MAXLEN, L, (T)p.max_search_len, L > (T)p.max_search_len)) L = (T)p.max_search_len;
  // orient the keyframe template so that its image runs along +lr (checked at the mid depth)
  {
    const T dm = (dlo + dhi) * (T)0.5;
    const T z0 = az + bz * dm;
    const T a1x = ax + (G.M[0] * lkx + G.M[1] * lky), a1y = ay + (G.M[3] * lkx + G.M[4] * lky);
    const T a1z = az + (G.M[6] * lkx + G.M[7] * lky);
    const T z1 = a1z + bz * dm;
    const T qx = (a1x + bx * dm) / z1 - (ax + bx * dm) / z0;
    const T qy = (a1y + by * dm) / z1 - (ay + by * dm) / z0;
    if (note(D_ORIENT, qx * lrx + qy * lry, (T)0, qx * lrx + qy * lry < (T)0)) {
      lkx = -lkx;
      lky = -lky;
    }
  }
  T tk[5];
  for (int k = 0; k < 5; ++k) tk[k] = bilinear(Ik, w, xf + (T)(k - 2) * lkx, yf + (T)(k - 2) * lky);
  // slide the 5-sample window along the reference line: window s (0 <= s <= n) is centred at
  // pf + s lr and uses samples s-2 .. s+2
  const int n = (int)L;
  note_value(D_NWIN, n, L, (T)n);
  const T INF = (T)INFINITY;
  const T umax = (T)(w - 1), vmax = (T)(h - 1);
  T r[5] = {0, 0, 0, 0, 0};
  bool ok[5] = {false, false, false, false, false};
  T e1 = INF, e2 = INF, eprev = INF, ebefore = INF, eafter = INF;
  int s1 = -1;
  for (int j = -2; j <= n + 2; ++j) {
    for (int k = 0; k < 4; ++k) {
      r[k] = r[k + 1];
      ok[k] = ok[k + 1];
    }
    const T sx = pfx + (T)j * lrx, sy = pfy + (T)j * lry;
    ok[4] = sx >= (T)0 && sy >= (T)0 && sx < umax && sy < vmax;
    if (tracing()) {  // distance of the sample to the image border (negative: outside)
      T m = sx;
      if (sy < m) m = sy;
      if (umax - sx < m) m = umax - sx;
      if (vmax - sy < m) m = vmax - sy;
      note(D_SAMPLE, m, (T)0, ok[4], j);
    }
    r[4] = ok[4] ? bilinear(Ir, w, sx, sy) : (T)0;
    if (j < 2) continue;
    const int s = j - 2;
    T e = INF;
    if (ok[0] && ok[1] && ok[2] && ok[3] && ok[4]) {
      const T d0 = r[0] - tk[0], d1 = r[1] - tk[1], d2 = r[2] - tk[2], d3 = r[3] - tk[3], d4 = r[4] - tk[4];
      e = (((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3) + d4 * d4;
    }
    note_value(D_WIN, s, e, (T)0);
    if (note(D_RUNBEST, e, e1, e < e1, s)) {
      if (s1 >= 0 && s - s1 >= 2 && note(D_RUN2, e1, e2, e1 < e2, s)) e2 = e1;
      ebefore = eprev;
      e1 = e;
      s1 = s;
      eafter = INF;
    } else {
      if (s == s1 + 1) eafter = e;
      if (s - s1 >= 2 && note(D_RUN2, e, e2, e < e2, s)) e2 = e;
    }
    eprev = e;
  }
  note_value(D_ARGMIN, s1, e1, e2);
  if (s1 < 0) return;                          // no window inside the reference image
  if (note(D_MAXSSD, e1, (T)p.max_ssd * (T)5, e1 > (T)p.max_ssd * (T)5)) {  // no acceptable match: count a failure
    ++bl;
    return;
  }
  if (!note(D_UNIQUE, e2, (T)p.unique_ratio * e1, e2 > (T)p.unique_ratio * e1)) return;  // ambiguous
  T off = (T)0;
  if (ebefore < INF && eafter < INF) {
    const T den = (ebefore - (T)2 * e1) + eafter;
    if (note(D_DEN, den, (T)0, den > (T)0)) {
      off = ((T)0.5 * (ebefore - eafter)) / den;
      if (note(D_CLAMP_HI, off, (T)0.5, off > (T)0.5)) off = (T)0.5;
      if (note(D_CLAMP_LO, off, (T)-0.5, off < (T)-0.5)) off = (T)-0.5;
    }
  }
  const T sm = (T)s1 + off;
  const T mx = pfx + sm * lrx, my = pfy + sm * lry;
  T dobs, alpha;
  if (note(D_AXIS, std::fabs(lrx), std::fabs(lry), std::fabs(lrx) >= std::fabs(lry))) {
    const T den = mx * bz - bx;
    dobs = (ax - mx * az) / den;
    alpha = std::fabs(lrx * (bx * az - ax * bz)) / (den * den);
  } else {
    const T den = my * bz - by;
    dobs = (ay - my * az) / den;
    alpha = std::fabs(lry * (by * az - ay * bz)) / (den * den);
  }
  if (!note(D_DOBS, dobs, (T)0, dobs > (T)0)) return;
  const T geo = (T)p.epipolar_var / cos2;
  const T photo = ((T)2 * (T)p.image_var) / (gp * gp);
  const T vobs = (alpha * alpha) * (geo + photo);
  if (note(D_INIT, (T)val, (T)0, val <= 0)) {
    d = dobs;
    var = vobs;
    val = p.validity_init;
    return;
  }
  const T dd = dobs - d;
  const T chi2 = (dd * dd) / (var + vobs);
  if (note(D_CHI2, chi2, (T)p.fuse_chi2, chi2 > (T)p.fuse_chi2)) {
    ++bl;
    val -= p.validity_penalty;
    if (note(D_VALDROP, (T)val, (T)0, val <= 0)) {
      val = 0;
      d = (T)-1;
      var = (T)-1;
    }
    return;
  }
  const T sv = var + vobs;
  d = (d * vobs + dobs * var) / sv;
  var = (var * vobs) / sv;
  val = val + 1 < p.validity_max ? val + 1 : p.validity_max;
}

template <class T>
struct DepthFrame {
  int w, h;
  double fx, fy, cx, cy;
  std::vector<T> I, gx, gy;
};

template <class T>
static void make_depth_frame(const float* img, int w, int h, const lsdg_intrinsics& k, DepthFrame<T>& F) {
  F.w = w; F.h = h; F.fx = k.fx; F.fy = k.fy; F.cx = k.cx; F.cy = k.cy;
  F.I.resize((size_t)w * h);
  for (size_t i = 0; i < F.I.size(); ++i) F.I[i] = (T)img[i];
  F.gx.assign(F.I.size(), (T)0);
  F.gy.assign(F.I.size(), (T)0);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      if (x >= 1 && x <= w - 2) F.gx[i] = (F.I[i + 1] - F.I[i - 1]) * (T)0.5;
      if (y >= 1 && y <= h - 2) F.gy[i] = (F.I[i + w] - F.I[i - w]) * (T)0.5;
    }
}

template <class T>
static void observe_all(const DepthFrame<T>& K, int n_refs, const float* ref_images, const double* key_to_ref,
                        const lsdg_params& p, DepthState<T>& S, int threads) {
  const int w = K.w, h = K.h;
  std::vector<RefGeom<T>> G(n_refs);
  std::vector<std::vector<T>> R(n_refs);
  for (int r = 0; r < n_refs; ++r) {
    G[r] = ref_geom<T>(key_to_ref + 12 * r, K.fx, K.fy, K.cx, K.cy);
    R[r].resize((size_t)w * h);
    for (size_t i = 0; i < R[r].size(); ++i) R[r][i] = (T)ref_images[(size_t)r * w * h + i];
  }
  const T fx = (T)K.fx, fy = (T)K.fy, cx = (T)K.cx, cy = (T)K.cy;
  auto rows = [&](int y0, int y1) {
    for (int y = y0; y < y1; ++y)
      for (int x = 0; x < w; ++x) {
        if (x < 3 || y < 3 || x > w - 4 || y > h - 4) continue;
        const size_t i = (size_t)y * w + x;
        T d = S.d[i], v = S.v[i];
        int val = S.val[i], bl = S.bl[i];
        t_sink.pixel = (int)i;
        for (int r = 0; r < n_refs; ++r) {
          t_sink.ref = r;
          if (note(D_BLLIMIT, (T)bl, (T)p.blacklist_limit, bl >= p.blacklist_limit)) break;
          observe_pixel<T>(x, y, w, h, K.I.data(), K.gx.data(), K.gy.data(), R[r].data(), G[r], fx, fy, cx, cy, p,
                           d, v, val, bl);
        }
        S.d[i] = d; S.v[i] = v; S.val[i] = val; S.bl[i] = bl;
      }
  };
  if (threads <= 1) {
    rows(0, h);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t) th.emplace_back(rows, h * t / threads, h * (t + 1) / threads);
    for (auto& t : th) t.join();
  }
}

// regularizeDepthMap + hole filling: smoothed planes from the raw hypotheses, then the commit that
// drops removed hypotheses from the raw state (var_smoothed == -2 marks a removal).
template <class T>
static void regularize(int w, int h, const lsdg_params& p, DepthState<T>& S, int threads, int stage) {
  const int R = p.reg_radius;
  t_sink.stage = stage;
  t_sink.ref = 0;
  auto rows = [&](int y0, int y1) {
    for (int y = y0; y < y1; ++y)
      for (int x = 0; x < w; ++x) {
        const size_t i = (size_t)y * w + x;
        t_sink.pixel = (int)i;
        T sw = 0, swd = 0;
        int cnt = 0;
        if (note(D_R_HASDEPTH, (T)S.val[i], (T)0, S.val[i] > 0)) {
          const T d = S.d[i], v = S.v[i];
          for (int dy = -R; dy <= R; ++dy)
            for (int dx = -R; dx <= R; ++dx) {
              const int nx = x + dx, ny = y + dy;
              if (nx < 0 || ny < 0 || nx >= w || ny >= h) continue;
              const size_t j = (size_t)ny * w + nx;
              if (!note(D_R_NVAL, (T)S.val[j], (T)0, S.val[j] > 0, (int)j)) continue;
              const T dd = S.d[j] - d;
              if (note(D_R_COMPAT, dd * dd, (T)p.reg_chi2 * (S.v[j] + v), dd * dd <= (T)p.reg_chi2 * (S.v[j] + v), (int)j)) {
                const T wt = (T)1 / S.v[j];
                sw = sw + wt;
                swd = swd + wt * S.d[j];
                if (dx != 0 || dy != 0) ++cnt;
              }
            }
          if (note(D_R_SUPPORT, (T)cnt, (T)p.reg_min_support, cnt < p.reg_min_support)) {
            S.sm[i] = (T)-1;
            S.vsm[i] = (T)-2;
          } else {
            S.sm[i] = swd / sw;
            S.vsm[i] = v;
          }
        } else {
          for (int dy = -R; dy <= R; ++dy)
            for (int dx = -R; dx <= R; ++dx) {
              const int nx = x + dx, ny = y + dy;
              if (nx < 0 || ny < 0 || nx >= w || ny >= h) continue;
              const size_t j = (size_t)ny * w + nx;
              if (!note(D_R_NVAL, (T)S.val[j], (T)0, S.val[j] > 0, (int)j)) continue;
              const T wt = (T)1 / S.v[j];
              sw = sw + wt;
              swd = swd + wt * S.d[j];
              ++cnt;
            }
          if (note(D_R_FILL, (T)cnt, (T)p.fill_min_support, cnt >= p.fill_min_support)) {
            S.sm[i] = swd / sw;
            S.vsm[i] = (T)p.fill_var_factor * ((T)cnt / sw);
          } else {
            S.sm[i] = (T)-1;
            S.vsm[i] = (T)-1;
          }
        }
      }
  };
  if (threads <= 1) {
    rows(0, h);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t) th.emplace_back(rows, h * t / threads, h * (t + 1) / threads);
    for (auto& t : th) t.join();
  }
  for (size_t i = 0; i < S.d.size(); ++i)
    if (S.vsm[i] == (T)-2) {
      S.val[i] = 0;
      S.d[i] = (T)-1;
      S.v[i] = (T)-1;
    }
}

// propagateDepth: forward-warp every hypothesis of the old keyframe into the new one; the nearest
// (smallest z, then lowest old pixel index) wins a target pixel.
template <class T>
static void propagate(const DepthFrame<T>& Kold, const DepthFrame<T>& Knew, const double old_to_new[12],
                      const lsdg_params& p, const DepthState<T>& S, DepthState<T>& N) {
  const int w = Kold.w, h = Kold.h;
  const T fx = (T)Kold.fx, fy = (T)Kold.fy, cx = (T)Kold.cx, cy = (T)Kold.cy;
  const T fxi = (T)(1.0 / Kold.fx), fyi = (T)(1.0 / Kold.fy);
  T Rm[9], t[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) Rm[3 * i + j] = (T)old_to_new[4 * i + j];
    t[i] = (T)old_to_new[4 * i + 3];
  }
  std::vector<uint64_t> key((size_t)w * h, ~0ull);
  struct Warp { T zn, izn; int xi, yi; bool ok; };
  t_sink.stage = 2;
  t_sink.ref = 0;
  auto warp = [&](int x, int y, bool rec) {
    Warp r{0, 0, 0, 0, false};
    const size_t i = (size_t)y * w + x;
    TraceSink keep = t_sink;
    if (!rec) t_sink.out = nullptr;  // the gather pass repeats the warp of a winner: not traced again
    t_sink.pixel = (int)i;
    struct Restore { TraceSink& s; TraceSink k; ~Restore() { s = k; } } restore{t_sink, keep};
    const T z = (T)1 / S.d[i];
    const T X = (((T)x - cx) * fxi) * z, Y = (((T)y - cy) * fyi) * z;
    const T Xn = ((Rm[0] * X + Rm[1] * Y) + Rm[2] * z) + t[0];
    const T Yn = ((Rm[3] * X + Rm[4] * Y) + Rm[5] * z) + t[1];
    const T Zn = ((Rm[6] * X + Rm[7] * Y) + Rm[8] * z) + t[2];
    if (!note(D_P_Z, Zn, (T)p.min_z, Zn > (T)p.min_z)) return r;
    const T izn = (T)1 / Zn;
    const T un = fx * (Xn * izn) + cx, vn = fy * (Yn * izn) + cy;
    const T fxr = std::floor(un + (T)0.5), fyr = std::floor(vn + (T)0.5);
    note_value(D_P_RX, (int)fxr, un + (T)0.5, fxr);
    note_value(D_P_RY, (int)fyr, vn + (T)0.5, fyr);
    if (!note(D_P_BOUND, fxr, fyr, fxr >= (T)0 && fyr >= (T)0 && fxr <= (T)(w - 1) && fyr <= (T)(h - 1))) return r;
    r.xi = (int)fxr;
    r.yi = (int)fyr;
    const T diff = Knew.I[(size_t)r.yi * w + r.xi] - Kold.I[i];
    if (note(D_P_PHOTO, std::fabs(diff), (T)p.propagate_max_photo_diff, std::fabs(diff) > (T)p.propagate_max_photo_diff)) return r;
    r.zn = Zn;
    r.izn = izn;
    r.ok = true;
    return r;
  };
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      if (S.val[i] <= 0) continue;
      const Warp r = warp(x, y, true);
      if (!r.ok) continue;
      float zf = (float)r.zn;  // the key orders by the float depth (positive floats order as integers)
      uint32_t zb;
      std::memcpy(&zb, &zf, 4);
      const uint64_t k = ((uint64_t)zb << 32) | (uint64_t)(uint32_t)i;
      const size_t ti = (size_t)r.yi * w + r.xi;
      if (k < key[ti]) key[ti] = k;
    }
  N.init((size_t)w * h);
  for (size_t ti = 0; ti < key.size(); ++ti) {
    if (key[ti] == ~0ull) continue;
    const uint32_t o = (uint32_t)(key[ti] & 0xffffffffu);
    const int x = (int)(o % (uint32_t)w), y = (int)(o / (uint32_t)w);
    const Warp r = warp(x, y, false);
    const T d = S.d[o], v = S.v[o];
    const T ratio = r.izn / d;
    const T r2 = ratio * ratio;
    N.d[ti] = r.izn;
    N.v[ti] = v * (r2 * r2) + (T)p.prediction_var;
    N.val[ti] = S.val[o];
    N.bl[ti] = 0;
    N.sm[ti] = N.d[ti];
    N.vsm[ti] = N.v[ti];
  }
}

template <class T>
static void init_state(const float* idepth, const float* var, size_t n, const lsdg_params& p, DepthState<T>& S) {
  S.init(n);
  for (size_t i = 0; i < n; ++i) {
    const T d = (T)idepth[i], v = (T)var[i];
    if (d > (T)0 && v > (T)0) {
      S.d[i] = d;
      S.v[i] = v;
      S.val[i] = p.validity_init;
      S.sm[i] = d;
      S.vsm[i] = v;
    }
  }
}

template <class T>
static void dump(const DepthState<T>& S, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    out[0 * n + i] = (float)S.d[i];
    out[1 * n + i] = (float)S.v[i];
    out[2 * n + i] = (float)S.sm[i];
    out[3 * n + i] = (float)S.vsm[i];
    out[4 * n + i] = (float)S.val[i];
    out[5 * n + i] = (float)S.bl[i];
  }
}

// The whole depth-filter workload: initial hypotheses -> observe n_refs references in order
// (-> regularize if flags & 1) -> snapshot; then, if new_image is given, propagate into the new
// keyframe (-> regularize if flags & 2) -> snapshot.  Snapshots are 6 planes of w*h floats:
// idepth, var, idepth_smoothed, var_smoothed, validity, blacklist.
template <class T>
static int pipeline(int w, int h, const lsdg_intrinsics* k, const lsdg_params* p, const float* key_image,
                    const float* init_idepth, const float* init_var, int n_refs, const float* ref_images,
                    const double* key_to_ref, const float* new_image, const double* key_to_new, int flags,
                    float* upd_out, float* prop_out, int threads) {
  DepthFrame<T> K;
  make_depth_frame<T>(key_image, w, h, *k, K);
  DepthState<T> S;
  const size_t n = (size_t)w * h;
  init_state<T>(init_idepth, init_var, n, *p, S);
  t_sink.stage = 0;
  observe_all<T>(K, n_refs, ref_images, key_to_ref, *p, S, threads);
  if (flags & 1) regularize<T>(w, h, *p, S, threads, 1);
  if (upd_out) dump(S, upd_out, n);
  if (new_image && key_to_new) {
    DepthFrame<T> Kn;
    make_depth_frame<T>(new_image, w, h, *k, Kn);
    DepthState<T> N;
    propagate<T>(K, Kn, key_to_new, *p, S, N);
    if (flags & 2) regularize<T>(w, h, *p, N, threads, 3);
    if (prop_out) dump(N, prop_out, n);
  }
  return 0;
}

}  // namespace lsdo

extern "C" {

int lsdo_depth_pipeline_f(int w, int h, const lsdg_intrinsics* k, const lsdg_params* p, const float* key_image,
                          const float* init_idepth, const float* init_var, int n_refs, const float* ref_images,
                          const double* key_to_ref, const float* new_image, const double* key_to_new, int flags,
                          float* upd_out, float* prop_out, int threads) {
  return lsdo::pipeline<float>(w, h, k, p, key_image, init_idepth, init_var, n_refs, ref_images, key_to_ref,
                               new_image, key_to_new, flags, upd_out, prop_out, threads);
}

int lsdo_depth_pipeline_d(int w, int h, const lsdg_intrinsics* k, const lsdg_params* p, const float* key_image,
                          const float* init_idepth, const float* init_var, int n_refs, const float* ref_images,
                          const double* key_to_ref, const float* new_image, const double* key_to_new, int flags,
                          float* upd_out, float* prop_out, int threads) {
  return lsdo::pipeline<double>(w, h, k, p, key_image, init_idepth, init_var, n_refs, ref_images, key_to_ref,
                                new_image, key_to_new, flags, upd_out, prop_out, threads);
}

// The same pipeline with the decision trace on for the pixels where mask[stage * w * h + i] != 0
// (single-threaded):
// records in execution order, stage 0 observe (pixel = keyframe pixel, ref = reference index),
// 1 the update's regularisation, 2 propagation (pixel = old keyframe pixel), 3 the new keyframe's
// regularisation.  Returns the number of records (more than `cap` means some were dropped).
long lsdo_depth_trace(int use_double, int w, int h, const lsdg_intrinsics* k, const lsdg_params* p,
                      const float* key_image, const float* init_idepth, const float* init_var, int n_refs,
                      const float* ref_images, const double* key_to_ref, const float* new_image,
                      const double* key_to_new, int flags, const uint8_t* mask, lsdo::DecisionRec* out, long cap) {
  std::vector<lsdo::DecisionRec> rec;
  lsdo::t_sink.out = &rec;
  lsdo::t_sink.mask = mask;
  lsdo::t_sink.npix = (size_t)w * h;
  if (use_double)
    lsdo::pipeline<double>(w, h, k, p, key_image, init_idepth, init_var, n_refs, ref_images, key_to_ref, new_image,
                           key_to_new, flags, nullptr, nullptr, 1);
  else
    lsdo::pipeline<float>(w, h, k, p, key_image, init_idepth, init_var, n_refs, ref_images, key_to_ref, new_image,
                          key_to_new, flags, nullptr, nullptr, 1);
  lsdo::t_sink = lsdo::TraceSink{};
  const long n = (long)rec.size();
  std::memcpy(out, rec.data(), sizeof(lsdo::DecisionRec) * (size_t)(n < cap ? n : cap));
  return n;
}

}  // extern "C"

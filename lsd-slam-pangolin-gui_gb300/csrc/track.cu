// track.cu -- a3/a4/a5/a6/a11 of the hot path: SE3 and Sim3 direct image alignment.
//
// Upstream: SE3Tracker::trackFrame and its calculateWarpUpdate, Sim3Tracker::trackFrameSim3
// (lsd-slam fips import, absent from the reference; the call chain starts at
// lib/App/InputThread.cpp:71).  Method: ECCV 2014 sec. 3.2 -- variance-normalised photometric
// residual, Huber weights, LM on se(3), coarse to fine; sec. 3.3 -- Sim3 alignment of two keyframes
// with an added inverse-depth residual against the other keyframe's depth map, LM on sim(3).
// The kernel is one template: SIM3 = false tracks 6 parameters with 28 sums per pass, SIM3 = true
// 7 parameters (log-scale added) with 36 sums.
//
// GB300 design.  One persistent kernel tracks any number of pairs.  Each pair is owned by one
// thread-block cluster (C CTAs of NT threads, C up to 16); clusters pull pairs from an atomic work
// queue (largest first).  A residual pass over a level's points is:
//   1. every thread walks the SoA points with stride C*NT (coalesced float4 loads; SE3: two points
//      per iteration without branches, the next two prefetched), warps the point with the current
//      pose, samples the new frame's intensity with the C1 Catmull-Rom interpolant and its exact
//      derivative (4x4 taps, L1/L2 resident), and accumulates the 21 + 6 + 1 float sums of J^T W J,
//      J^T W r and the Huber energy (gradient and energy Kahan-compensated; SE3 Hessian sums plain
//      per thread).  The first pass of a level fixes each point's residual variance in the psig
//      scratch array (and leaves out points that do not land border_margin pixels inside the
//      image), so each level minimises one fixed, continuous energy whose gradient is exactly
//      2 J^T W r;
//   2. warp shuffles merge the compensated pairs (reduce-scatter), then a fixed-order block merge;
//   2'. every CTA stores its partial straight into rank 0's shared memory (distributed shared
//      memory stores, no global-memory scratch); cluster.sync(); rank 0 merges the C partials in
//      fixed rank order, so the result is deterministic for a given C and NT;
//   4. warp 0 of rank 0 runs the LM step: four lanes solve the systems the decision may need
//      (undamped; damped if accepted; damped after one or two rejections) with register-resident
//      LDL^T of the Jacobi-scaled system in float, lane 0 decides (accept / reject by an FP64
//      energy comparison, convergence, level changes), the warp copies the record and the pose,
//      12 lanes compose exp(step) with the FP64 pose, and the next pose goes into every rank's
//      shared memory;
//   5. cluster.sync(); every CTA reads the pose from its own shared memory and starts the next pass.
// The whole LM loop over all levels therefore runs on the device without a host round trip and
// without global-memory scratch for the reduction.  The one-pair form (lsdg_track_se3) is the same
// kernel with a single cluster.
//
// Arithmetic: FP32 residuals/weights/Jacobians (this translation unit is built with FMA contraction,
// so per-point values differ from the CPU oracle in the last bits; parity is by tolerance),
// compensated merges, float LM solves and schedule, FP64 for the pose and the energy comparison.
#include <cooperative_groups.h>

#include "lsdg_internal.cuh"

namespace cg = cooperative_groups;

namespace lsdg {

// Per-mode sizes: DOF parameters, NH entries of the upper triangle of H, NS compensated sums per
// pass (H, g, energy), REC doubles in the pass record (NS + points used, inliers, outliers,
// left the image).
template <bool SIM3>
struct Mode {
  static constexpr int DOF = SIM3 ? 7 : 6;
  static constexpr int NH = DOF * (DOF + 1) / 2;
  static constexpr int NS = NH + DOF + 1;
  static constexpr int REC = NS + 4;
  static constexpr int POSE = SIM3 ? 13 : 12;  // doubles per pose in the API
};
constexpr int kMaxSums = 36;
constexpr int kMaxRec = 40;

// Taylor coefficients 1 / (k! (shift + k)) of the sim(3) exp series, shift = 1..11, k = 0..20
// (filled by track_prepare).
__constant__ double c_sim3_tab[11][21];


struct Ctl {
  float R[9];
  float t[3];
  int pair;  // -1: no more work
  int level;
  int first;  // first pass of the level: fixes each point's residual variance and participation
  int pad;
};

struct CtaPart {
  float s[kMaxSums];
  float c[kMaxSums];
  int cnt[3];  // good, bad, out-of-image
};

enum { PH_INIT = 0, PH_TRY = 1 };

// The pose and the energy comparison are FP64; the linear algebra and the schedule are float.
// On GB300 an FP64 warp instruction costs ~64 issue cycles, and the solves work on float sums:
// their systems are Jacobi-scaled to a unit diagonal so float pivots keep the accuracy the sums have.
struct LMState {
  double T[12];     // ref_to_frame [M | t] (M = R, or sR for Sim3), accepted
  double Ttry[12];  // ref_to_frame being evaluated
  double S[kMaxRec];  // record of the last accepted pass
  float Sf[kMaxSums];  // its sums rounded to float (the kept linearisation the solves read)
  double E_num, E_den;  // mean energy of the last accepted pass, E_num / E_den (compared by cross-multiplying)
  float lambda, gnmax;
  int it, phase, level, pair, have_final, fresh;
  int s_src;  // 0: lm.S holds the sums of the pass just merged, 1: of an earlier pass
  int need_exp;  // try_step chose dx: the warp applies exp(dx) * T and publishes the trial pose
  float dx[7];
  lsdg_track_stats st;
};

// ------------------------------------------------------------------------------------------
// Pose helpers (warp 0 of rank 0 only)
// ------------------------------------------------------------------------------------------
// [M | t]^-1 for M = R (SE3) or M = sR (Sim3: M^-1 = M^T / s^2; s^2 = 1 for a rotation).
__device__ __noinline__ void se3_inv_d(const double* A, double* B, bool sim3) {
  const double s2 = sim3 ? (A[0] * A[0] + A[1] * A[1]) + A[2] * A[2] : 1.0;
  double o[12];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) o[4 * i + j] = sim3 ? A[4 * j + i] / s2 : A[4 * j + i];
  for (int i = 0; i < 3; ++i) o[4 * i + 3] = -((o[4 * i + 0] * A[3] + o[4 * i + 1] * A[7]) + o[4 * i + 2] * A[11]);
  for (int i = 0; i < 12; ++i) B[i] = o[i];
}

// On GB300 one FP64 warp instruction holds a sub-partition's FP64 pipe for ~64 cycles however few
// lanes are active, so the FP64 parts below are written lane-parallel: each lane owns one matrix
// element or row, and the instruction count on the critical path is what is minimised.

// Coefficients of the se(3) exp (A = sin t / t, B = (1 - cos t) / t^2, C = (t - sin t) / t^3 with
// t^2 = th2): Taylor series in t^2 through t^10 for t < 0.05 (no sqrt, sincos or division),
// closed form otherwise.  Same rule as the CPU oracle.
__device__ __forceinline__ void se3_coeffs(double th2, double& A, double& B, double& C) {
  if (th2 < 0.0025) {
    A = 1.0 + th2 * (-1.0 / 6.0 + th2 * (1.0 / 120.0 + th2 * (-1.0 / 5040.0 + th2 * (1.0 / 362880.0 + th2 * (-1.0 / 39916800.0)))));
    B = 0.5 + th2 * (-1.0 / 24.0 + th2 * (1.0 / 720.0 + th2 * (-1.0 / 40320.0 + th2 * (1.0 / 3628800.0 + th2 * (-1.0 / 479001600.0)))));
    C = 1.0 / 6.0 + th2 * (-1.0 / 120.0 + th2 * (1.0 / 5040.0 + th2 * (-1.0 / 362880.0 + th2 * (1.0 / 39916800.0 + th2 * (-1.0 / 6227020800.0)))));
  } else {
    const double th = sqrt(th2);
    double sn, cs;
    sincos(th, &sn, &cs);
    A = sn / th;
    B = (1.0 - cs) / th2;
    C = (th - sn) / (th2 * th);
  }
}

// The tracker's Catmull-Rom weights and derivative weights (the polynomials of catmull_rom in
// Horner form: 18 fused operations instead of ~30; the tracker is built with FMA contraction and
// its parity is by tolerance, the energy kernels keep the oracle's operation order).
__device__ __forceinline__ void catmull_rom_fma(float t, float w[4], float d[4]) {
  const float t2 = t * t;
  const float e = fmaf(-1.5f, t, 2.0f);
  w[0] = t * fmaf(t, fmaf(-0.5f, t, 1.0f), -0.5f);
  w[1] = fmaf(t2, fmaf(1.5f, t, -2.5f), 1.0f);
  w[2] = t * fmaf(t, e, 0.5f);
  w[3] = t2 * fmaf(0.5f, t, -0.5f);
  d[0] = fmaf(t, e, -0.5f);
  d[1] = t * fmaf(4.5f, t, -5.0f);
  d[2] = fmaf(t, fmaf(-4.5f, t, 4.0f), 0.5f);
  d[3] = t * fmaf(1.5f, t, -1.0f);
}

// Float twin of se3_coeffs for the SE3 tracker's increments (same rule: Taylor series below t = 0.05).
__device__ __forceinline__ void se3_coeffs_f(float th2, float& A, float& B, float& C) {
  if (th2 < 0.0025f) {
    A = 1.0f + th2 * (-1.0f / 6.0f + th2 * (1.0f / 120.0f + th2 * (-1.0f / 5040.0f + th2 * (1.0f / 362880.0f))));
    B = 0.5f + th2 * (-1.0f / 24.0f + th2 * (1.0f / 720.0f + th2 * (-1.0f / 40320.0f + th2 * (1.0f / 3628800.0f))));
    C = 1.0f / 6.0f + th2 * (-1.0f / 120.0f + th2 * (1.0f / 5040.0f + th2 * (-1.0f / 362880.0f + th2 * (1.0f / 39916800.0f))));
  } else {
    const float th = sqrtf(th2);
    float sn, cs;
    sincosf(th, &sn, &cs);
    A = sn / th;
    B = (1.0f - cs) / th2;
    C = (th - sn) / (th2 * th);
  }
}

// Tout = exp(xi) * Tin for an se(3) increment xi (float): the increment's rotation and V are built
// in float (lane e < 9 one element each, lanes 0..2 the translation), the product with the FP64
// pose in FP64 (lane o < 12 one element).  Every lane must call.
__device__ __forceinline__ void warp_exp_mul_se3f(const float* xi, const double* Tin, double* Tout, int lane) {
  const float v0 = xi[0], v1 = xi[1], v2 = xi[2], w0 = xi[3], w1 = xi[4], w2 = xi[5];
  const float th2 = (w0 * w0 + w1 * w1) + w2 * w2;
  float A, B, Cc;
  se3_coeffs_f(th2, A, B, Cc);
  const int e = lane < 9 ? lane : 0;
  const int i = e / 3, j = e % 3;
  const float wi = i == 0 ? w0 : i == 1 ? w1 : w2;
  const float wj = j == 0 ? w0 : j == 1 ? w1 : w2;
  const float K = e == 1 ? -w2 : e == 2 ? w1 : e == 3 ? w2 : e == 5 ? -w0 : e == 6 ? -w1 : e == 7 ? w0 : 0.0f;
  const float I = (i == j) ? 1.0f : 0.0f;
  const float K2 = wi * wj - ((i == j) ? th2 : 0.0f);
  const float R = (I + A * K) + B * K2;
  const float V = (I + B * K) + Cc * K2;
  const int tr = lane < 3 ? lane : 0;
  const float V0 = __shfl_sync(0xffffffffu, V, 3 * tr + 0);
  const float V1 = __shfl_sync(0xffffffffu, V, 3 * tr + 1);
  const float V2 = __shfl_sync(0xffffffffu, V, 3 * tr + 2);
  const float t = (V0 * v0 + V1 * v1) + V2 * v2;
  const int o = lane < 12 ? lane : 0;
  const int r = o / 4, c = o % 4;
  const float E0 = __shfl_sync(0xffffffffu, R, 3 * r + 0);
  const float E1 = __shfl_sync(0xffffffffu, R, 3 * r + 1);
  const float E2 = __shfl_sync(0xffffffffu, R, 3 * r + 2);
  const float Et = __shfl_sync(0xffffffffu, t, r);
  double out = ((double)E0 * Tin[c] + (double)E1 * Tin[4 + c]) + (double)E2 * Tin[8 + c];
  if (c == 3) out = out + (double)Et;
  if (lane < 12) Tout[o] = out;
}

// Coefficients a0, a1, a2 of V = a0 I + a1 K + a2 K^2 in the sim(3) exp (integrals of e^{sigma tau}
// against 1, sin(theta tau)/theta, (1 - cos(theta tau))/theta^2 over [0, 1]); same rule as the CPU
// oracle: for theta < 0.05 and |sigma| < 1 the double Taylor series, evaluated with lanes 0..4
// (a1 terms), 8..12 (a2 terms) and 16 (a0) running one 21-term Horner chain each; otherwise the
// closed forms.  Every lane must call; all lanes return the same values.
__device__ __forceinline__ void sim3_coeffs_warp(double th2, double sg, int lane, double& a0, double& a1, double& a2) {
  if (th2 < 0.0025 && fabs(sg) < 1.0) {
    const int m = lane & 7;
    const int shift = lane < 8 ? 2 * m + 2 : lane < 16 ? 2 * m + 3 : 1;
    const int row = (lane < 16 && m > 4) ? 0 : shift - 1;  // idle lanes read a valid row
    double acc = 0.0;
#pragma unroll
    for (int k = 20; k >= 0; --k) acc = acc * sg + c_sim3_tab[row][k];
    a0 = __shfl_sync(0xffffffffu, acc, 16);
    // 1/(2m+1)! and 1/(2m+2)! for m = 0..4
    const double if1[5] = {1.0, 1.0 / 6.0, 1.0 / 120.0, 1.0 / 5040.0, 1.0 / 362880.0};
    const double if2[5] = {0.5, 1.0 / 24.0, 1.0 / 720.0, 1.0 / 40320.0, 1.0 / 3628800.0};
    double s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int mm = 4; mm >= 0; --mm) {
      s1 = s1 * (-th2) + __shfl_sync(0xffffffffu, acc, mm) * if1[mm];
      s2 = s2 * (-th2) + __shfl_sync(0xffffffffu, acc, 8 + mm) * if2[mm];
    }
    a1 = s1;
    a2 = s2;
    return;
  }
  if (th2 < 0.0025) {
    // theta < 0.05, |sigma| >= 1 (rare: a scale step of e or more): the theta series with
    // I_n(sigma) = int_0^1 t^(n-1) e^(sigma t) dt from the upward recurrence
    // I_n = (e^sigma - (n-1) I_(n-1)) / sigma, whose error growth (n-1)!/|sigma|^(n-1) the series'
    // 1/(n-1)! cancels.  Every lane computes it.
    const double es = exp(sg), is = 1.0 / sg;
    double I[12];
    I[1] = (es - 1.0) * is;
#pragma unroll
    for (int n = 2; n <= 11; ++n) I[n] = (es - (double)(n - 1) * I[n - 1]) * is;
    const double f1[5] = {1.0, 6.0, 120.0, 5040.0, 362880.0};        // (2m+1)!
    const double f2[5] = {2.0, 24.0, 720.0, 40320.0, 3628800.0};     // (2m+2)!
    double s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int mm = 4; mm >= 0; --mm) {
      s1 = s1 * (-th2) + I[2 * mm + 2] / f1[mm];
      s2 = s2 * (-th2) + I[2 * mm + 3] / f2[mm];
    }
    a0 = I[1];
    a1 = s1;
    a2 = s2;
    return;
  }
  const double th = sqrt(th2), es = exp(sg);
  double sn, cs;
  sincos(th, &sn, &cs);
  const double D = sg * sg + th2;
  a0 = fabs(sg) < 1e-8 ? 1.0 + 0.5 * sg : (es - 1.0) / sg;
  const double S1 = (es * (sg * sn - th * cs) + th) / D;
  const double C1 = (es * (sg * cs + th * sn) - sg) / D;
  a1 = S1 / th;
  a2 = (a0 - C1) / th2;
}

// Tout = exp(xi) * Tin (3x4 row-major), computed by a whole warp: lane e < 9 builds element e of
// the rotation (times e^sigma for Sim3) and of V, lanes 0..2 the translation, lane o < 12 one element
// of the product.  xi (6 or 7 doubles), Tin, Tout are in shared memory; every lane must call.
template <bool SIM3, typename X>
__device__ __forceinline__ void warp_exp_mul(const X* xi, const double* Tin, double* Tout, int lane) {
  const double v0 = xi[0], v1 = xi[1], v2 = xi[2], w0 = xi[3], w1 = xi[4], w2 = xi[5];
  const double th2 = (w0 * w0 + w1 * w1) + w2 * w2;
  double A, B, Cc;
  se3_coeffs(th2, A, B, Cc);
  double sc = 1.0, a0 = 1.0, a1 = B, a2 = Cc;  // SE3: V = I + B K + C K^2
  if (SIM3) {
    sim3_coeffs_warp(th2, (double)xi[6], lane, a0, a1, a2);
    sc = exp((double)xi[6]);
  }
  const int e = lane < 9 ? lane : 0;
  const int i = e / 3, j = e % 3;
  const double wi = i == 0 ? w0 : i == 1 ? w1 : w2;
  const double wj = j == 0 ? w0 : j == 1 ? w1 : w2;
  // K = [w]x: K01 = -w2, K02 = w1, K10 = w2, K12 = -w0, K20 = -w1, K21 = w0
  const double K = e == 1 ? -w2 : e == 2 ? w1 : e == 3 ? w2 : e == 5 ? -w0 : e == 6 ? -w1 : e == 7 ? w0 : 0.0;
  const double I = (i == j) ? 1.0 : 0.0;
  const double K2 = wi * wj - ((i == j) ? th2 : 0.0);
  double R = (I + A * K) + B * K2;
  if (SIM3) R = sc * R;
  const double V = (a0 * I + a1 * K) + a2 * K2;
  // translation t_i = V_i0 v0 + V_i1 v1 + V_i2 v2 (lanes 0..2 gather their row of V)
  const int tr = lane < 3 ? lane : 0;
  const double V0 = __shfl_sync(0xffffffffu, V, 3 * tr + 0);
  const double V1 = __shfl_sync(0xffffffffu, V, 3 * tr + 1);
  const double V2 = __shfl_sync(0xffffffffu, V, 3 * tr + 2);
  const double t = (V0 * v0 + V1 * v1) + V2 * v2;
  // product: out[r][c] = sum_k E[r][k] Tin[k][c] (+ E[r][3] for c == 3)
  const int o = lane < 12 ? lane : 0;
  const int r = o / 4, c = o % 4;
  const double E0 = __shfl_sync(0xffffffffu, R, 3 * r + 0);
  const double E1 = __shfl_sync(0xffffffffu, R, 3 * r + 1);
  const double E2 = __shfl_sync(0xffffffffu, R, 3 * r + 2);
  const double Et = __shfl_sync(0xffffffffu, t, r);
  double out = (E0 * Tin[c] + E1 * Tin[4 + c]) + E2 * Tin[8 + c];
  if (c == 3) out = out + Et;
  if (lane < 12) Tout[o] = out;
}

// (H + lambda diag H) x = -g for N x N symmetric H given as its upper triangle (row-major), by an
// LDL^T factorisation of the Jacobi-scaled system (row and column j times 1/sqrt(H_jj), so the
// factorised matrix has the diagonal 1 + lambda) held in float registers.  Returns false when a
// pivot is not positive.  The LM step's four speculative solves and its rare further solves use it.
template <int N>
__device__ __forceinline__ bool ldlt_solve_reg(const float* __restrict__ hu, const float* __restrict__ g,
                                               float lambda, float* x) {
  float L[N * (N + 1) / 2];
  float d[N], id[N], y[N], sc[N];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const float h = hu[j * N - (j * (j - 1)) / 2];
    sc[j] = h > 0.f ? rsqrtf(h) : 1.f;
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) L[i * (i + 1) / 2 + j] = (hu[j * N - (j * (j - 1)) / 2 + (i - j)] * sc[i]) * sc[j];
#pragma unroll
  for (int i = 0; i < N; ++i) L[i * (i + 1) / 2 + i] *= (1.0f + lambda);
  bool ok = true;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    float sj = L[j * (j + 1) / 2 + j];
#pragma unroll
    for (int k = 0; k < j; ++k) sj -= (L[j * (j + 1) / 2 + k] * L[j * (j + 1) / 2 + k]) * d[k];
    ok = ok && (sj > 1e-20f);
    d[j] = sj;
    id[j] = 1.0f / sj;
#pragma unroll
    for (int i = j + 1; i < N; ++i) {
      float t = L[i * (i + 1) / 2 + j];
#pragma unroll
      for (int k = 0; k < j; ++k) t -= (L[i * (i + 1) / 2 + k] * L[j * (j + 1) / 2 + k]) * d[k];
      L[i * (i + 1) / 2 + j] = t * id[j];
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    float si = -(g[i] * sc[i]);
#pragma unroll
    for (int k = 0; k < i; ++k) si -= L[i * (i + 1) / 2 + k] * y[k];
    y[i] = si;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) y[i] *= id[i];
#pragma unroll
  for (int i = N - 1; i >= 0; --i) {
    float si = y[i];
#pragma unroll
    for (int k = i + 1; k < N; ++k) si -= L[k * (k + 1) / 2 + i] * x[k];
    x[i] = si;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) x[i] *= sc[i];
  return ok;
}

// Solves computed ahead of the LM decision by warp 0, four systems at once (lane g solves system
// g): [0] undamped step of the pass just merged, [1] damped step if that pass is
// accepted (or is a level's first pass), [2] and [3] damped steps on the kept linearisation after
// one or two rejections.  The decision logic takes an entry only when source and lambda match.
struct SolveCache {
  float x[4][8];
  float lambda[4];
  float gn[4];  // max |x_i| of the solution
  int src[4];  // 0: the sums of the pass just merged, 1: the sums kept from an earlier pass
  int ok[4];
  int valid[4];
};

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

template <bool SIM3>
__device__ __noinline__ void finish_pair(const TrackArgs& a, LMState& lm) {
  using Md = Mode<SIM3>;
  const int p = lm.pair;
  lsdg_track_stats& st = lm.st;
  double out[12];
  se3_inv_d(lm.T, out, SIM3);
  double* dst = a.out_pose + (size_t)Md::POSE * p;
  if (SIM3) {  // {R, t, s}
    const double sc = sqrt((out[0] * out[0] + out[1] * out[1]) + out[2] * out[2]);
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) dst[3 * i + j] = out[4 * i + j] / sc;
      dst[9 + i] = out[4 * i + 3];
    }
    dst[12] = sc;
  } else {
    for (int i = 0; i < 12; ++i) dst[i] = out[i];
  }
  int tot = 0;
  for (int l = 0; l < kMaxLevels; ++l) tot += st.passes[l];
  st.total_passes = tot;
  st.n_points = level_points(a, p, 0);
  const double* S = lm.S;
  const int iN = Md::NS;
  if (lm.have_final) {
    st.n_valid = (int)S[iN];
    st.n_good = (int)S[iN + 1];
    st.mean_energy = S[iN] > 0 ? (float)(S[iN - 1] / S[iN]) : 0.f;
    st.good_ratio = S[iN] > 0 ? (float)(S[iN + 1] / S[iN]) : 0.f;
    st.usage = st.n_points > 0 ? (float)(S[iN] / st.n_points) : 0.f;
    for (int i = 0; i < Md::NH; ++i) st.hessian[i] = S[i];
  }
  const bool lost = !lm.have_final || st.good_ratio < a.min_good_ratio || st.usage < a.min_usage;
  st.status = lost ? LSDG_TRACKING_LOST : LSDG_OK;
  a.out_stats[p] = st;
  if (a.out_sums)
    for (int i = 0; i < Md::REC; ++i) a.out_sums[(size_t)Md::REC * p + i] = S[i];
}

// Takes pairs off the queue until one has a level to run; publishes it (or pair = -1).
template <bool SIM3>
__device__ __noinline__ void fetch_pair(const TrackArgs& a, LMState& lm, Ctl& ctl) {
  using Md = Mode<SIM3>;
  for (;;) {
    const int k = atomicAdd(a.work_counter, 1);
    if (k >= a.n_pairs) {
      ctl.pair = -1;
      return;
    }
    const int p = a.order ? a.order[k] : k;
    lm.pair = p;
    lm.have_final = 0;
    lm.need_exp = 0;
    lm.s_src = 1;
    lm.it = 0;
    lm.E_num = 0;
    lm.E_den = 1;
    lm.lambda = a.lambda0;
    for (int i = 0; i < kMaxRec; ++i) lm.S[i] = 0;
    for (int i = 0; i < kMaxSums; ++i) lm.Sf[i] = 0.f;
    if (a.accumulate_stats) {
      lm.st = a.out_stats[p];  // the coarse levels' pass counts, from the first phase
    } else {
      char* sp = reinterpret_cast<char*>(&lm.st);
      for (int i = 0; i < (int)sizeof(lsdg_track_stats); ++i) sp[i] = 0;
    }
    const double* in = a.init + (size_t)Md::POSE * p;
    double Tin[12];
    if (SIM3) {  // {R, t, s} -> [sR | t]
      for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) Tin[4 * i + j] = in[12] * in[3 * i + j];
        Tin[4 * i + 3] = in[9 + i];
      }
    } else {
      for (int i = 0; i < 12; ++i) Tin[i] = in[i];
    }
    if (a.init_is_ref_to_frame) {
      for (int i = 0; i < 12; ++i) lm.T[i] = Tin[i];
    } else {
      se3_inv_d(Tin, lm.T, SIM3);
    }
    if (start_level(a, lm, ctl, a.top_level)) return;
    finish_pair<SIM3>(a, lm);
  }
}

template <bool SIM3>
__device__ void next_level(const TrackArgs& a, LMState& lm, Ctl& ctl) {
  if (lm.level > a.bottom_level && start_level(a, lm, ctl, lm.level - 1)) return;
  finish_pair<SIM3>(a, lm);
  fetch_pair<SIM3>(a, lm, ctl);
}

template <bool SIM3>
__device__ __forceinline__ bool cached_solve(LMState& lm, SolveCache& sc, float lambda, float* x, float* gn) {
  constexpr int D = Mode<SIM3>::DOF;
#pragma unroll 1
  for (int k = 0; k < 4; ++k) {
    if (sc.valid[k] && sc.src[k] == lm.s_src && sc.lambda[k] == lambda) {
      for (int i = 0; i < D; ++i) x[i] = sc.x[k][i];
      *gn = sc.gn[k];
      sc.valid[k] = 0;
      return sc.ok[k] != 0;
    }
  }
  const bool ok = ldlt_solve_reg<D>(lm.Sf, lm.Sf + Mode<SIM3>::NH, lambda, x);
  float m = 0.f;
  for (int i = 0; i < D; ++i) m = fmaxf(m, fabsf(x[i]));
  *gn = m;
  return ok;
}

// One LM iteration decision on the current linearisation lm.S (same rules as the CPU oracle):
// converged when the undamped Gauss-Newton step is below step_eps * 2^level; otherwise solve the
// damped system and ask the warp for the trial pose, unless the level's iteration budget is spent.
template <bool SIM3>
__device__ void try_step(const TrackArgs& a, LMState& lm, Ctl& ctl, SolveCache& sc) {
  constexpr int D = Mode<SIM3>::DOF;
  const float thr = a.step_eps * (float)(1 << lm.level);
  for (;;) {
    if (lm.fresh) {
      float gn[D], m = 0.f;
      lm.gnmax = 3e38f;
      if (cached_solve<SIM3>(lm, sc, 0.0f, gn, &m)) {
        lm.gnmax = m;
        if (m < thr) break;
      }
      lm.fresh = 0;
    }
    if (lm.it >= a.max_iter[lm.level]) break;
    lm.it++;
    float dx[D], m = 0.f;
    if (!cached_solve<SIM3>(lm, sc, lm.lambda, dx, &m)) {
      lm.lambda *= a.lambda_up;
      continue;
    }
    for (int i = 0; i < D; ++i) lm.dx[i] = dx[i];
    lm.need_exp = 1;  // the warp computes lm.Ttry = exp(dx) * lm.T and publishes it
    lm.phase = PH_TRY;
    ctl.pair = lm.pair;
    ctl.level = lm.level;
    ctl.first = 0;
    return;
  }
  next_level<SIM3>(a, lm, ctl);
}

// What the warp does after the LM decision (lm_decide): copy the pass just merged into the record
// (and the trial pose into the accepted pose), then take the next step or move to the next level.
enum { ACT_STEP = 1, ACT_NEXT_LEVEL = 2, ACT_COPY_S = 4, ACT_COPY_T = 8 };

// The accept / reject decision on the pass just merged (lane 0; same rules as the CPU oracle).
// The copies it asks for are made by the whole warp (lm_copy) before lm_continue runs.
template <bool SIM3>
__device__ __noinline__ int lm_decide(const TrackArgs& a, LMState& lm, const double* tot) {
  using Md = Mode<SIM3>;
  lm.st.passes[lm.level]++;
  const double N = tot[Md::NS];
  const double En = tot[Md::NS - 1];
  if (lm.phase == PH_INIT) {
    if (!(N > 0)) return ACT_NEXT_LEVEL;
    lm.s_src = 0;
    lm.E_num = En;
    lm.E_den = N;
    lm.lambda = a.lambda0;
    lm.it = 0;
    lm.fresh = 1;
    if (lm.level == a.bottom_level) lm.have_final = 1;
    return ACT_STEP | ACT_COPY_S;
  }
  if (N > 0 && En * lm.E_den < lm.E_num * N) {  // En / N below the accepted mean energy
    lm.s_src = 0;
    lm.E_num = En;
    lm.E_den = N;
    lm.lambda *= a.lambda_down;
    lm.fresh = 1;
    return ACT_STEP | ACT_COPY_S | ACT_COPY_T;
  }
  lm.s_src = 1;
  if (lm.gnmax < a.stall_eps * (float)(1 << lm.level)) return ACT_NEXT_LEVEL;  // noise floor of this level
  lm.lambda *= a.lambda_up;
  return ACT_STEP;
}

// Whole warp: the record / pose copies a decision asked for.
template <bool SIM3>
__device__ __forceinline__ void lm_copy(LMState& lm, const double* tot, const float* totf, int act, int lane) {
  using Md = Mode<SIM3>;
  if (act & ACT_COPY_S) {
    for (int i = lane; i < Md::REC; i += 32) lm.S[i] = tot[i];
    if (lane < Md::NS) lm.Sf[lane] = totf[lane];
  }
  if ((act & ACT_COPY_T) && lane < 12) lm.T[lane] = lm.Ttry[lane];
}

// Lane 0, after the copies: the next LM step of this level, or the next level / pair.
template <bool SIM3>
__device__ __noinline__ void lm_continue(const TrackArgs& a, LMState& lm, Ctl& ctl, SolveCache& sc, int act) {
  if (act & ACT_STEP) try_step<SIM3>(a, lm, ctl, sc);
  else next_level<SIM3>(a, lm, ctl);
}

// Warp 0 of cluster rank 0 solves the four systems the decision may need (see SolveCache): lane g
// solves system g in registers (a dependency chain of ~N pivots, no shuffles).
template <bool SIM3>
__device__ __forceinline__ void speculate(const TrackArgs& a, const LMState& lm, const double* tot, const float* totf,
                                          SolveCache& sc, int lane) {
  using Md = Mode<SIM3>;
  if (lane >= 4) return;
  const int grp = lane;
  const bool init = lm.phase == PH_INIT;
  const float* S = grp >= 2 ? lm.Sf : totf;
  const float lam = grp == 0 ? 0.0f
                  : grp == 1 ? (init ? a.lambda0 : lm.lambda * a.lambda_down)
                  : grp == 2 ? lm.lambda * a.lambda_up
                             : (lm.lambda * a.lambda_up) * a.lambda_up;
  float x[Md::DOF];
  const bool ok = ldlt_solve_reg<Md::DOF>(S, S + Md::NH, lam, x);
  float m = 0.f;
#pragma unroll
  for (int i = 0; i < Md::DOF; ++i) {
    sc.x[grp][i] = x[i];
    m = fmaxf(m, fabsf(x[i]));
  }
  sc.ok[grp] = ok ? 1 : 0;
  sc.gn[grp] = m;
  sc.lambda[grp] = lam;
  sc.src[grp] = grp >= 2 ? 1 : 0;
  sc.valid[grp] = (tot[Md::NS] > 0 && (grp < 2 || !init)) ? 1 : 0;
}

// ------------------------------------------------------------------------------------------
// The persistent cluster kernel
// ------------------------------------------------------------------------------------------
constexpr int kMaxCluster = 16;

// Merge of the 28 compensated sums of a warp by reduce-scatter: after five halving rounds (31
// shuffle pairs instead of the 140 of a butterfly) lane l holds the warp total of sum l.
__device__ __forceinline__ void warp_reduce_scatter(float (&s)[32], float (&c)[32], int lane) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < o; ++i) {
      const float ks = up ? s[i + o] : s[i], kc = up ? c[i + o] : c[i];
      const float ss = up ? s[i] : s[i + o], sc = up ? c[i] : c[i + o];
      const float rs = __shfl_xor_sync(0xffffffffu, ss, o), rc = __shfl_xor_sync(0xffffffffu, sc, o);
      float ns = ks, nc = kc;
      kmerge(ns, nc, rs, rc);
      s[i] = ns;
      c[i] = nc;
    }
  }
}

// Butterfly merge of a few compensated sums across the warp (every lane ends with the totals).
template <int K>
__device__ __forceinline__ void warp_butterfly(float (&s)[K], float (&c)[K]) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
    for (int i = 0; i < K; ++i) kmerge(s[i], c[i], __shfl_xor_sync(0xffffffffu, s[i], o), __shfl_xor_sync(0xffffffffu, c[i], o));
}

template <int NT, int MINB, bool SIM3>
__global__ void __launch_bounds__(NT, MINB) track_kernel(const TrackArgs a) {
  using Md = Mode<SIM3>;
  constexpr int NW = NT / 32;
  constexpr int D = Md::DOF, NH = Md::NH, NS = Md::NS;
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const unsigned C = cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  __shared__ float ws[NW][NS];
  __shared__ float wc[NW][NS];
  __shared__ int wn[NW][3];
  __shared__ CtaPart allpart[kMaxCluster];  // rank 0's copy receives every rank's partial
  __shared__ Ctl ctl;                       // every rank's copy is written by rank 0
  __shared__ double tot[kMaxRec];
  __shared__ float totf[kMaxSums];
  __shared__ LMState lm;
  __shared__ SolveCache sc;

  // rank 0 publishes the control word to the other ranks' shared memory
  auto push_ctl = [&]() {
    if (lane >= 1 && lane < (int)C) {
      int* dst = reinterpret_cast<int*>(cluster.map_shared_rank(&ctl, (unsigned)lane));
      const int* src = reinterpret_cast<const int*>(&ctl);
#pragma unroll
      for (int i = 0; i < (int)(sizeof(Ctl) / 4); ++i) dst[i] = src[i];
    }
  };

  if (rank == 0 && wid == 0) {
    if (lane == 0) fetch_pair<SIM3>(a, lm, ctl);
    __syncwarp();
    push_ctl();
  }
  cluster.sync();

  for (;;) {
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
    float* __restrict__ psigd = R->psigd[level];
    const float* __restrict__ img = Fc->plane[level];
    const float* __restrict__ Dj = SIM3 ? Fc->idepth[level] : nullptr;
    const float* __restrict__ Vj = SIM3 ? Fc->ivar[level] : nullptr;
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
    const float dfloor = a.sim3_depth_variance, wdep = a.sim3_depth_weight;

    float hs[NH], hc[NH], gs[D], gc[D], es = 0.f, ec = 0.f;
#pragma unroll
    for (int i = 0; i < NH; ++i) { hs[i] = 0.f; hc[i] = 0.f; }
#pragma unroll
    for (int i = 0; i < D; ++i) { gs[i] = 0.f; gc[i] = 0.f; }
    int good = 0, bad = 0, oob = 0;

    if (!SIM3) {
      // SE3: two points per iteration, each evaluated without branches (a point that sits out gathers
      // a clamped in-frame cell and gets zero weight), so both points' 32 gathers are in flight
      // together and one add per sum takes both products.  The level's first pass freezes 1/sigma^2
      // in psig, so later passes divide nothing; inliers take no square root.  A thread sums a few
      // dozen points per pass: the 21 Hessian sums (all terms of one sign on the diagonal, and only
      // the curvature of the step) are plain float sums there, the gradient and the energy (whose
      // terms cancel, and whose differences decide LM steps) stay compensated; every merge across
      // threads, warps and CTAs is compensated.
      const int stride = (int)C * NT;
      const float d2 = delta * delta;
      // a point's inputs: its float4 and frozen 1/sigma^2 (index 0 stands in past the end; the level's
      // arrays are allocated for every pixel, so it is in bounds)
      auto load = [&](int k, float4& p, float& sig) {
        const int kk = k < n ? k : 0;
        sig = first ? 1.f : psig[kk];
        p = __ldg(&pts[kk]);
      };
      auto eval = [&](int k, const float4 p, const float sig, float (&J)[D], float& wgt, float& res, float& rho) {
        const bool in = k < n;
        const int kk = in ? k : 0;
        const bool act = in && sig > 0.f;
        const float X = p.x, Y = p.y, Z = p.z, Ik = p.w;
        const float Rpx = (R00 * X + R01 * Y) + R02 * Z;
        const float Rpy = (R10 * X + R11 * Y) + R12 * Z;
        const float Rpz = (R20 * X + R21 * Y) + R22 * Z;
        const float Xp = Rpx + t0, Yp = Rpy + t1, Zp = Rpz + t2;
        const bool zok = Zp > minz;
        const float iz = __fdividef(1.0f, zok ? Zp : 1.f);  // ~1 ulp reciprocal
        const float u = fx * (Xp * iz) + cx;
        const float v = fy * (Yp * iz) + cy;
        const bool bok = first ? (u >= ulo && v >= vlo && u < uhi && v < vhi)
                               : (u >= 1.f && v >= 1.f && u < umax && v < vmax);
        const bool ok = act && zok && bok;
        if (act && !ok) {
          ++oob;
          if (first) psig[k] = 0.f;
        }
        const float uc = ok ? u : 1.f, vc = ok ? v : 1.f;
        const int ix = (int)uc, iy = (int)vc;
        const float ax = uc - (float)ix, ay = vc - (float)iy;
        float wx[4], dxw[4], wy[4], dyw[4];
        catmull_rom_fma(ax, wx, dxw);
        catmull_rom_fma(ay, wy, dyw);
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
        const float a0 = (Gx * fx) * iz, a1 = (Gy * fy) * iz;
        const float a2 = -((a0 * Xp + a1 * Yp) * iz);
        float isig = sig;
        if (first) {
          const float drd = -(((a0 * Rpx + a1 * Rpy) + a2 * Rpz) * Z);
          isig = 1.0f / (pvr + (drd * drd) * __ldg(&pvar[kk]));
          if (ok) psig[k] = isig;
        }
        const float e2 = (r * r) * isig;
        const bool inl = e2 <= d2;
        const float ir = rsqrtf(e2);
        good += (ok && inl) ? 1 : 0;
        bad += (ok && !inl) ? 1 : 0;
        wgt = ok ? (inl ? isig : (delta * ir) * isig) : 0.f;
        rho = ok ? (inl ? e2 : delta * (2.f * (e2 * ir) - delta)) : 0.f;
        res = ok ? r : 0.f;
        J[0] = ok ? a0 : 0.f;
        J[1] = ok ? a1 : 0.f;
        J[2] = ok ? a2 : 0.f;
        J[3] = ok ? Yp * a2 - Zp * a1 : 0.f;
        J[4] = ok ? Zp * a0 - Xp * a2 : 0.f;
        J[5] = ok ? Xp * a1 - Yp * a0 : 0.f;
      };
      // the next iteration's two points are loaded while this one's are evaluated
      int k = (int)rank * NT + tid;
      float4 pa, pb;
      float sa, sb;
      load(k, pa, sa);
      load(k + stride, pb, sb);
      for (; k < n; k += 2 * stride) {
        const float4 ca = pa, cb = pb;
        const float csa = sa, csb = sb;
        load(k + 2 * stride, pa, sa);
        load(k + 3 * stride, pb, sb);
        float Ja[D], Jb[D], wa, wb, ra, rb, ea, eb;
        eval(k, ca, csa, Ja, wa, ra, ea);
        eval(k + stride, cb, csb, Jb, wb, rb, eb);
        float wJa[D], wJb[D];
#pragma unroll
        for (int i = 0; i < D; ++i) { wJa[i] = wa * Ja[i]; wJb[i] = wb * Jb[i]; }
        int q2 = 0;
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = i; j < D; ++j) { hs[q2] = fmaf(wJb[i], Jb[j], fmaf(wJa[i], Ja[j], hs[q2])); ++q2; }
#pragma unroll
        for (int i = 0; i < D; ++i) kadd(gs[i], gc[i], wJa[i] * ra + wJb[i] * rb);
        kadd(es, ec, ea + eb);
      }
    }
    if (SIM3)
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
        if (first) {
          psig[k] = 0.f;
          if (SIM3) psigd[k] = 0.f;
        }
        ++oob;
        continue;
      }
      const float iz = 1.0f / Zp;
      const float u = fx * (Xp * iz) + cx;
      const float v = fy * (Yp * iz) + cy;
      if (first) {
        if (!(u >= ulo && v >= vlo && u < uhi && v < vhi)) {
          psig[k] = 0.f;
          if (SIM3) psigd[k] = 0.f;
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
      catmull_rom_fma(ax, wx, dxw);
      catmull_rom_fma(ay, wy, dyw);
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
      float J[D];
      J[0] = a0;
      J[1] = a1;
      J[2] = a2;
      J[3] = Yp * a2 - Zp * a1;
      J[4] = Zp * a0 - Xp * a2;
      J[5] = Xp * a1 - Yp * a0;
      if (SIM3) J[D - 1] = (a0 * Xp + a1 * Yp) + a2 * Zp;
      // as in the SE3 loop: psig (and psigd) hold 1/sigma^2 frozen at the level's first pass
      float isig = s2;
      if (first) {
        const float drd = -(((a0 * Rpx + a1 * Rpy) + a2 * Rpz) * Z);
        isig = 1.0f / (pvr + (drd * drd) * __ldg(&pvar[k]));
        psig[k] = isig;
      }
      const float e2 = (r * r) * isig;
      float wgt, rho;
      if (e2 <= delta * delta) { wgt = isig; rho = e2; ++good; }
      else {
        const float ir = rsqrtf(e2);
        wgt = (delta * ir) * isig;
        rho = delta * (2.f * (e2 * ir) - delta);
        ++bad;
      }
      float wJ[D];
#pragma unroll
      for (int i = 0; i < D; ++i) wJ[i] = wgt * J[i];
      {
        // inverse-depth residual against the other keyframe's depth map (4 valid bilinear corners)
        float Jd[D], rd = 0.f, wgd = 0.f, rhod = 0.f;
#pragma unroll
        for (int i = 0; i < D; ++i) Jd[i] = 0.f;
        const size_t i00 = (size_t)iy * w + ix;
        const float D00 = __ldg(&Dj[i00]), D10 = __ldg(&Dj[i00 + 1]), D01 = __ldg(&Dj[i00 + w]), D11 = __ldg(&Dj[i00 + w + 1]);
        bool dok = D00 > 0.f && D10 > 0.f && D01 > 0.f && D11 > 0.f;
        float s2d = 0.f;
        if (!first) {
          s2d = psigd[k];
          if (!(s2d > 0.f)) dok = false;
        }
        if (dok) {
          const float bx = 1.f - ax, by = 1.f - ay;
          const float w00 = bx * by, w10 = ax * by, w01 = bx * ay, w11 = ax * ay;
          const float Dv = ((w00 * D00 + w10 * D10) + w01 * D01) + w11 * D11;
          const float Ddx = by * (D10 - D00) + ay * (D11 - D01);
          const float Ddy = bx * (D01 - D00) + ax * (D11 - D10);
          rd = iz - Dv;
          const float c0 = (Ddx * fx) * iz, c1 = (Ddy * fy) * iz;
          const float c2 = -((c0 * Xp + c1 * Yp) * iz);
          const float b0 = -c0, b1 = -c1, b2 = -(iz * iz) - c2;
          Jd[0] = b0;
          Jd[1] = b1;
          Jd[2] = b2;
          Jd[3] = Yp * b2 - Zp * b1;
          Jd[4] = Zp * b0 - Xp * b2;
          Jd[5] = Xp * b1 - Yp * b0;
          Jd[D - 1] = (b0 * Xp + b1 * Yp) + b2 * Zp;
          if (first) {
            const float Vv = ((w00 * __ldg(&Vj[i00]) + w10 * __ldg(&Vj[i00 + 1])) + w01 * __ldg(&Vj[i00 + w])) +
                             w11 * __ldg(&Vj[i00 + w + 1]);
            const float bdd = -(((b0 * Rpx + b1 * Rpy) + b2 * Rpz) * Z);
            float sd = Vv + (bdd * bdd) * __ldg(&pvar[k]);
            if (sd < dfloor) sd = dfloor;
            s2d = 1.0f / sd;
            psigd[k] = s2d;
          }
          const float e2d = (rd * rd) * s2d;
          if (e2d <= delta * delta) { wgd = wdep * s2d; rhod = e2d; }
          else {
            const float ir = rsqrtf(e2d);
            wgd = (wdep * (delta * ir)) * s2d;
            rhod = delta * (2.f * (e2d * ir) - delta);
          }
        } else if (first) {
          psigd[k] = 0.f;
        }
        int q2 = 0;
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = i; j < D; ++j) { hs[q2] = fmaf(wgd * Jd[i], Jd[j], fmaf(wJ[i], J[j], hs[q2])); ++q2; }
#pragma unroll
        for (int i = 0; i < D; ++i) kadd(gs[i], gc[i], wJ[i] * r + (wgd * Jd[i]) * rd);
        kadd(es, ec, rho + wdep * rhod);
      }
    }

    // warp merge: the first 32 sums by reduce-scatter (lane l ends with sum l), the rest (Sim3: 4)
    // by butterfly; then a fixed-order merge over warps
    {
      float S[32], Cc[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int src = i;
        float sv = 0.f, cv = 0.f;
        if (src < NH) { sv = hs[src]; cv = hc[src]; }
        else if (src < NH + D) { sv = gs[src - NH]; cv = gc[src - NH]; }
        else if (src == NH + D) { sv = es; cv = ec; }
        S[i] = sv;
        Cc[i] = cv;
      }
      constexpr int EXTRA = NS > 32 ? NS - 32 : 1;
      float XS[EXTRA], XC[EXTRA];
#pragma unroll
      for (int i = 0; i < EXTRA; ++i) {
        const int src = 32 + i;
        float sv = 0.f, cv = 0.f;
        if (src < NH) { sv = hs[src]; cv = hc[src]; }
        else if (src < NH + D) { sv = gs[src - NH]; cv = gc[src - NH]; }
        else if (src == NH + D) { sv = es; cv = ec; }
        XS[i] = sv;
        XC[i] = cv;
      }
      warp_reduce_scatter(S, Cc, lane);
      if (NS > 32) warp_butterfly<EXTRA>(XS, XC);
      good = __reduce_add_sync(0xffffffffu, good);
      bad = __reduce_add_sync(0xffffffffu, bad);
      oob = __reduce_add_sync(0xffffffffu, oob);
      if (lane < NS && lane < 32) {
        ws[wid][lane] = S[0];
        wc[wid][lane] = Cc[0];
      }
      if (NS > 32 && lane == 0) {
#pragma unroll
        for (int i = 0; i < EXTRA; ++i) {
          if (32 + i < NS) {
            ws[wid][(32 + i) % NS] = XS[i];
            wc[wid][(32 + i) % NS] = XC[i];
          }
        }
      }
      if (lane == 31) {
        wn[wid][0] = good;
        wn[wid][1] = bad;
        wn[wid][2] = oob;
      }
    }
    __syncthreads();
    // this CTA's partial goes straight into rank 0's shared memory
    if (tid < NS) {
      float s = 0.f, c = 0.f;
      for (int k = 0; k < NW; ++k) kmerge(s, c, ws[k][tid], wc[k][tid]);
      CtaPart* dst = cluster.map_shared_rank(&allpart[rank], 0u);
      dst->s[tid] = s;
      dst->c[tid] = c;
    } else if (tid < NS + 3) {
      int v = 0;
      for (int k = 0; k < NW; ++k) v += wn[k][tid - NS];
      cluster.map_shared_rank(&allpart[rank], 0u)->cnt[tid - NS] = v;
    }
    cluster.sync();

    if (rank == 0) {
      if (tid < NS) {
        float s = 0.f, c = 0.f;
        for (unsigned r = 0; r < C; ++r) kmerge(s, c, allpart[r].s[tid], allpart[r].c[tid]);
        tot[tid] = (double)s - (double)c;
        totf[tid] = s - c;
      } else if (tid < NS + 3) {
        int v = 0;
        for (unsigned r = 0; r < C; ++r) v += allpart[r].cnt[tid - NS];
        tot[tid + 1] = (double)v;  // NS+1 inliers, NS+2 outliers, NS+3 left the image
      }
      __syncthreads();
      if (wid == 0) {
        if (lane == 0) tot[NS] = tot[NS + 1] + tot[NS + 2];
        __syncwarp();
        speculate<SIM3>(a, lm, tot, totf, sc, lane);
        __syncwarp();
        int act = 0;
        if (lane == 0) act = lm_decide<SIM3>(a, lm, tot);
        act = __shfl_sync(0xffffffffu, act, 0);
        __syncwarp();
        lm_copy<SIM3>(lm, tot, totf, act, lane);
        __syncwarp();
        if (lane == 0) lm_continue<SIM3>(a, lm, ctl, sc, act);
        __syncwarp();
        if (lm.need_exp) {
          if (SIM3) warp_exp_mul<true>(lm.dx, lm.T, lm.Ttry, lane);
          else warp_exp_mul_se3f(lm.dx, lm.T, lm.Ttry, lane);
          __syncwarp();
          if (lane < 12) {  // publish the trial pose as float, one element per lane
            const float f = (float)lm.Ttry[lane];
            if ((lane & 3) == 3) ctl.t[lane >> 2] = f;
            else ctl.R[3 * (lane >> 2) + (lane & 3)] = f;
          }
          __syncwarp();
          if (lane == 0) lm.need_exp = 0;
          __syncwarp();
        }
        push_ctl();
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
template <int NT, int MINB, bool SIM3>
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
  return cudaLaunchKernelEx(&cfg, track_kernel<NT, MINB, SIM3>, a);
}

template <int NT, int MINB, bool SIM3>
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
  if (cudaOccupancyMaxActiveClusters(&n, track_kernel<NT, MINB, SIM3>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

#define LSDG_TRACK_SHAPES(X) X(128, 4) X(128, 8) X(256, 2) X(256, 4) X(512, 1) X(512, 2)

// Per context, outside any stream capture: allows clusters of up to 16 CTAs (non-portable size)
// for every instantiation and uploads the sim(3) series coefficients.
cudaError_t track_prepare() {
  cudaError_t e = cudaSuccess;
#define X(nt, mb)                                                                                                      \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(track_kernel<nt, mb, false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1); \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(track_kernel<nt, mb, true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  LSDG_TRACK_SHAPES(X)
#undef X
  double tab[11][21];
  double fact[21];
  fact[0] = 1.0;
  for (int k = 1; k <= 20; ++k) fact[k] = fact[k - 1] * k;
  for (int sh = 1; sh <= 11; ++sh)
    for (int k = 0; k <= 20; ++k) tab[sh - 1][k] = 1.0 / (fact[k] * (double)(sh + k));
  const cudaError_t e2 = cudaMemcpyToSymbol(c_sim3_tab, tab, sizeof(tab));
  return e != cudaSuccess ? e : e2;
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

cudaError_t launch_track(const TrackArgs& a, int threads, int minblocks, int cluster, int n_clusters, cudaStream_t s,
                         bool sim3) {
#define X(nt, mb)                                                                                            \
  if (threads == nt && minblocks == mb)                                                                      \
    return sim3 ? launch_nt<nt, mb, true>(a, cluster, n_clusters, s) : launch_nt<nt, mb, false>(a, cluster, n_clusters, s);
  LSDG_TRACK_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

int track_max_clusters(int threads, int minblocks, int cluster, bool sim3) {
#define X(nt, mb) \
  if (threads == nt && minblocks == mb) return sim3 ? max_clusters_nt<nt, mb, true>(cluster) : max_clusters_nt<nt, mb, false>(cluster);
  LSDG_TRACK_SHAPES(X)
#undef X
  return 0;
}

}  // namespace lsdg

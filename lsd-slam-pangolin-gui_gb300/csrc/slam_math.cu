// slam_math.cu -- host-only: Sim3 algebra and the keyframe pose graph (see slam_math.h).
//
// Sim3 exponential: T = [[e^sigma R(omega), V v], [0, 1]] with V = a0 I + a1 K + a2 K^2 (K = [omega]x),
// a0 = int_0^1 e^(sigma t) dt, a1 = int e^(sigma t) sin(theta t) / theta, a2 = int e^(sigma t)
// (1 - cos(theta t)) / theta^2: closed forms, with series where they cancel (small theta: the theta
// series over I_n = int t^(n-1) e^(sigma t) dt, whose upward recurrence is stable for |sigma| >= 1e-3).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>

#include "slam_math.h"

namespace lsdg {
namespace slam {

M4 M4::identity() {
  M4 I;
  std::memset(I.a, 0, sizeof(I.a));
  I.a[0] = I.a[5] = I.a[10] = I.a[15] = 1.0;
  return I;
}

M4 mul(const M4& A, const M4& B) {
  M4 C;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double s = 0.0;
      for (int k = 0; k < 4; ++k) s += A(r, k) * B(k, c);
      C(r, c) = s;
    }
  return C;
}

M4 sim3_inv(const M4& T) {
  const double s2 = T(0, 0) * T(0, 0) + T(1, 0) * T(1, 0) + T(2, 0) * T(2, 0);  // column norm^2 = s^2
  M4 o = M4::identity();
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) o(i, j) = T(j, i) / s2;
  for (int i = 0; i < 3; ++i) o(i, 3) = -(o(i, 0) * T(0, 3) + o(i, 1) * T(1, 3) + o(i, 2) * T(2, 3));
  return o;
}

static double det3(const double M[9]) {
  return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
}

double sim3_scale(const M4& T) {
  const double M[9] = {T(0, 0), T(0, 1), T(0, 2), T(1, 0), T(1, 1), T(1, 2), T(2, 0), T(2, 1), T(2, 2)};
  return std::cbrt(det3(M));
}

static void hat(const double w[3], double K[9]) {
  K[0] = 0; K[1] = -w[2]; K[2] = w[1];
  K[3] = w[2]; K[4] = 0; K[5] = -w[0];
  K[6] = -w[1]; K[7] = w[0]; K[8] = 0;
}

static void mat3_mul(const double A[9], const double B[9], double C[9]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}

void so3_exp(const double w[3], double R[9]) {
  const double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  double K[9], K2[9];
  hat(w, K);
  mat3_mul(K, K, K2);
  double a, b;
  if (th < 1e-8) {
    a = 1.0;
    b = 0.5;
  } else {
    a = std::sin(th) / th;
    b = (1.0 - std::cos(th)) / (th * th);
  }
  for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0 ? 1.0 : 0.0) + a * K[i] + b * K2[i];
}

void so3_log(const double R[9], double w[3]) {
  const double c = std::max(-1.0, std::min(1.0, (R[0] + R[4] + R[8] - 1.0) * 0.5));
  const double th = std::acos(c);
  const double v[3] = {(R[7] - R[5]) * 0.5, (R[2] - R[6]) * 0.5, (R[3] - R[1]) * 0.5};
  if (th < 1e-6) {
    for (int i = 0; i < 3; ++i) w[i] = v[i];
    return;
  }
  if (M_PI - th < 1e-4) {  // near pi: the axis from the symmetric part
    double B[9];
    for (int i = 0; i < 9; ++i) B[i] = (R[i] + (i % 4 == 0 ? 1.0 : 0.0)) * 0.5;
    int k = 0;
    if (B[4] > B[0]) k = 1;
    if (B[8] > B[4 * k]) k = 2;
    const double n = std::sqrt(std::max(B[4 * k], 1e-300));
    double ax[3] = {B[k] / n, B[3 + k] / n, B[6 + k] / n};
    if (ax[0] * v[0] + ax[1] * v[1] + ax[2] * v[2] < 0) for (double& x : ax) x = -x;
    for (int i = 0; i < 3; ++i) w[i] = ax[i] * th;
    return;
  }
  const double f = th / std::sin(th);
  for (int i = 0; i < 3; ++i) w[i] = v[i] * f;
}

// V = a0 I + a1 K + a2 K^2 of the Sim3 exponential.
static void sim3_V(const double w[3], double sg, double V[9]) {
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double th = std::sqrt(th2);
  const double a0 = std::fabs(sg) < 1e-5 ? 1.0 + sg / 2.0 + sg * sg / 6.0 : std::expm1(sg) / sg;
  double a1, a2;
  if (th < 1e-3) {
    double I[6];
    if (std::fabs(sg) < 1e-3) {
      I[1] = 1.0; I[2] = 0.5 + sg / 3.0; I[3] = 1.0 / 3.0 + sg / 4.0; I[4] = 0.25 + sg / 5.0; I[5] = 0.2 + sg / 6.0;
    } else {
      const double es = std::exp(sg);
      I[1] = std::expm1(sg) / sg;
      for (int n = 2; n <= 5; ++n) I[n] = (es - (n - 1) * I[n - 1]) / sg;
    }
    a1 = I[2] - th2 * I[4] / 6.0;
    a2 = I[3] / 2.0 - th2 * I[5] / 24.0;
  } else {
    const double es = std::exp(sg);
    const double D = sg * sg + th2;
    const double S1 = (es * (sg * std::sin(th) - th * std::cos(th)) + th) / D;
    const double C1 = (es * (sg * std::cos(th) + th * std::sin(th)) - sg) / D;
    a1 = S1 / th;
    a2 = (a0 - C1) / th2;
  }
  double K[9], K2[9];
  hat(w, K);
  mat3_mul(K, K, K2);
  for (int i = 0; i < 9; ++i) V[i] = a0 * (i % 4 == 0 ? 1.0 : 0.0) + a1 * K[i] + a2 * K2[i];
}

M4 sim3_exp(const double xi[7]) {
  double R[9], V[9];
  so3_exp(xi + 3, R);
  sim3_V(xi + 3, xi[6], V);
  const double s = std::exp(xi[6]);
  M4 T = M4::identity();
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) T(i, j) = s * R[3 * i + j];
    T(i, 3) = V[3 * i] * xi[0] + V[3 * i + 1] * xi[1] + V[3 * i + 2] * xi[2];
  }
  return T;
}

static bool solve3(const double A[9], const double b[3], double x[3]) {
  const double d = det3(A);
  if (!(std::fabs(d) > 1e-300)) return false;
  for (int k = 0; k < 3; ++k) {
    double M[9];
    std::memcpy(M, A, sizeof(M));
    for (int i = 0; i < 3; ++i) M[3 * i + k] = b[i];
    x[k] = det3(M) / d;
  }
  return true;
}

void sim3_log(const M4& T, double xi[7]) {
  const double s = sim3_scale(T);
  double R[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = T(i, j) / s;
  so3_log(R, xi + 3);
  xi[6] = std::log(s);
  double V[9];
  sim3_V(xi + 3, xi[6], V);
  const double t[3] = {T(0, 3), T(1, 3), T(2, 3)};
  if (!solve3(V, t, xi)) xi[0] = xi[1] = xi[2] = NAN;
}

void adjoint(const M4& T, double A[49]) {
  const double s = sim3_scale(T);
  double R[9], K[9], KR[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = T(i, j) / s;
  const double t[3] = {T(0, 3), T(1, 3), T(2, 3)};
  hat(t, K);
  mat3_mul(K, R, KR);
  std::memset(A, 0, sizeof(double) * 49);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      A[7 * i + j] = s * R[3 * i + j];
      A[7 * i + 3 + j] = KR[3 * i + j];
      A[7 * (3 + i) + 3 + j] = R[3 * i + j];
    }
  for (int i = 0; i < 3; ++i) A[7 * i + 6] = -t[i];
  A[48] = 1.0;
}

// Nearest rotation to a 3x3 matrix that is close to one (polar decomposition by the Newton
// iteration R <- (R + R^-T) / 2, quadratic near SO(3); Higham 1986).  Poses that arrive from the
// float tracker, or are composed from such poses, drift off SO(3) by rounding; sim3_inv and the
// graph's residuals assume a rotation, and a chain of compositions and inverses of a non-rotation
// amplifies the drift, so every pose is brought back onto SO(3) where it enters.
void orthonormalize(double R[9]) {
  for (int it = 0; it < 4; ++it) {
    // cofactor matrix C: R^-T = C / det(R)
    double C[9];
    C[0] = R[4] * R[8] - R[5] * R[7];
    C[1] = R[5] * R[6] - R[3] * R[8];
    C[2] = R[3] * R[7] - R[4] * R[6];
    C[3] = R[2] * R[7] - R[1] * R[8];
    C[4] = R[0] * R[8] - R[2] * R[6];
    C[5] = R[1] * R[6] - R[0] * R[7];
    C[6] = R[1] * R[5] - R[2] * R[4];
    C[7] = R[2] * R[3] - R[0] * R[5];
    C[8] = R[0] * R[4] - R[1] * R[3];
    const double det = R[0] * C[0] + R[1] * C[1] + R[2] * C[2];
    if (!(det > 0.0)) return;  // not near a rotation: left as it is
    for (int k = 0; k < 9; ++k) R[k] = 0.5 * (R[k] + C[k] / det);
  }
}

M4 from13(const double p[13]) {
  double R[9];
  for (int k = 0; k < 9; ++k) R[k] = p[k];
  orthonormalize(R);
  M4 T = M4::identity();
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) T(i, j) = p[12] * R[3 * i + j];
    T(i, 3) = p[9 + i];
  }
  return T;
}

void to13(const M4& T, double p[13]) {
  const double s = sim3_scale(T);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) p[3 * i + j] = T(i, j) / s;
    p[9 + i] = T(i, 3);
  }
  p[12] = s;
}

M4 from12(const double p[12]) {
  M4 T = M4::identity();
  for (int i = 0; i < 12; ++i) T.a[i] = p[i];
  double R[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = p[4 * i + j];
  orthonormalize(R);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T(i, j) = R[3 * i + j];
  return T;
}

void to12(const M4& T, double p[12]) {
  for (int i = 0; i < 12; ++i) p[i] = T.a[i];
}

// ------------------------------------------------------------------------------------------
// Pose graph
// ------------------------------------------------------------------------------------------
void PoseGraph::add_edge(int i, int j, const M4& Z, const double W[49]) {
  Edge e;
  e.i = i;
  e.j = j;
  e.Z = Z;
  std::copy(W, W + 49, e.W.begin());
  edges.push_back(e);
}

void PoseGraph::residual(const Edge& e, double r[7]) const {
  sim3_log(mul(mul(sim3_inv(e.Z), sim3_inv(poses[e.i])), poses[e.j]), r);
}

static double maha2(const double r[7], const double* W) {
  double m = 0.0;
  for (int a = 0; a < 7; ++a)
    for (int b = 0; b < 7; ++b) m += r[a] * W[7 * a + b] * r[b];
  return m;
}

double PoseGraph::cost() const {
  double c = 0.0;
  for (const Edge& e : edges) {
    double r[7];
    residual(e, r);
    const double m2 = maha2(r, e.W.data());
    const double m = std::sqrt(std::max(m2, 0.0));
    c += m <= huber ? m2 : huber * (2.0 * m - huber);
  }
  return c;
}

// Blocked right-looking Cholesky (lower, in place), then forward and back substitution.  The
// trailing update of each block column is split by rows over `threads` host threads.
bool cholesky_solve(std::vector<double>& A, int m, std::vector<double>& b, int threads) {
  constexpr int NB = 64;
  bool ok = true;
  for (int k0 = 0; k0 < m && ok; k0 += NB) {
    const int k1 = std::min(m, k0 + NB);
    // factor the diagonal block and the panel below it, column by column
    for (int k = k0; k < k1 && ok; ++k) {
      double d = A[(size_t)k * m + k];
      for (int p = k0; p < k; ++p) d -= A[(size_t)k * m + p] * A[(size_t)k * m + p];
      if (!(d > 0.0)) {
        ok = false;
        break;
      }
      const double l = std::sqrt(d);
      A[(size_t)k * m + k] = l;
      for (int i = k + 1; i < m; ++i) {
        double v = A[(size_t)i * m + k];
        for (int p = k0; p < k; ++p) v -= A[(size_t)i * m + p] * A[(size_t)k * m + p];
        A[(size_t)i * m + k] = v / l;
      }
    }
    if (!ok) break;
    // trailing update: A[i][j] -= sum_p L[i][p] L[j][p] for i >= j >= k1, p in [k0, k1)
    const int rows = m - k1;
    if (rows <= 0) break;
    auto work = [&](int r0, int r1) {
      for (int i = k1 + r0; i < k1 + r1; ++i) {
        const double* Li = &A[(size_t)i * m + k0];
        for (int j = k1; j <= i; ++j) {
          const double* Lj = &A[(size_t)j * m + k0];
          double s = 0.0;
          for (int p = 0; p < k1 - k0; ++p) s += Li[p] * Lj[p];
          A[(size_t)i * m + j] -= s;
        }
      }
    };
    const int nt = std::max(1, std::min(threads, rows / 32));
    if (nt == 1) {
      work(0, rows);
    } else {
      // rows of equal work: row i costs ~ i, so split by the square root of the cumulative cost
      std::vector<std::thread> th;
      int prev = 0;
      for (int t = 1; t <= nt; ++t) {
        const double f = std::sqrt((double)t / nt);
        const int cut = t == nt ? rows : (int)(f * rows);
        th.emplace_back(work, prev, cut);
        prev = cut;
      }
      for (auto& x : th) x.join();
    }
  }
  if (!ok) return false;
  for (int i = 0; i < m; ++i) {  // L y = b
    double v = b[i];
    for (int p = 0; p < i; ++p) v -= A[(size_t)i * m + p] * b[p];
    b[i] = v / A[(size_t)i * m + i];
  }
  for (int i = m - 1; i >= 0; --i) {  // L^T x = y
    double v = b[i];
    for (int p = i + 1; p < m; ++p) v -= A[(size_t)p * m + i] * b[p];
    b[i] = v / A[(size_t)i * m + i];
  }
  return true;
}

// Cholesky factorisation and solve restricted to the lower envelope: row i of A has no entry left
// of column env[i] (env[i] <= i), and neither has L (fill stays inside the envelope), so the work is
// the sum over rows of (i - env[i])^2 / 2 instead of m^3 / 6.
bool envelope_cholesky_solve(std::vector<double>& A, int m, const std::vector<int>& env, std::vector<double>& b) {
  for (int i = 0; i < m; ++i) {
    double* Li = &A[(size_t)i * m];
    for (int j = env[i]; j <= i; ++j) {
      const double* Lj = &A[(size_t)j * m];
      double v = Li[j];
      for (int k = std::max(env[i], env[j]); k < j; ++k) v -= Li[k] * Lj[k];
      if (j < i) {
        Li[j] = v / Lj[j];
      } else {
        if (!(v > 0.0)) return false;
        Li[i] = std::sqrt(v);
      }
    }
  }
  for (int i = 0; i < m; ++i) {  // L y = b
    const double* Li = &A[(size_t)i * m];
    double v = b[i];
    for (int k = env[i]; k < i; ++k) v -= Li[k] * b[k];
    b[i] = v / Li[i];
  }
  for (int i = m - 1; i >= 0; --i) {  // L^T x = y, column-oriented
    const double* Li = &A[(size_t)i * m];
    b[i] /= Li[i];
    for (int k = env[i]; k < i; ++k) b[k] -= Li[k] * b[i];
  }
  return true;
}

// Reverse Cuthill-McKee order of the free nodes (1..n-1; node 0 is held) over the edges' node
// adjacency: pos[node] = its block position, pos[0] = -1.  Nodes that edges join end up near each
// other, so the normal equations' envelope stays narrow even when the second lap of a path is tied
// to the first.  Ties broken by degree, then index: the order depends on the graph alone.
std::vector<int> rcm_positions(int n, const std::vector<Edge>& edges) {
  std::vector<std::vector<int>> adj(n);
  for (const Edge& e : edges)
    if (e.i != e.j && e.i > 0 && e.j > 0) {
      adj[e.i].push_back(e.j);
      adj[e.j].push_back(e.i);
    }
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  auto less = [&](int a, int b) { return adj[a].size() != adj[b].size() ? adj[a].size() < adj[b].size() : a < b; };
  std::vector<int> order;
  order.reserve(n > 0 ? n - 1 : 0);
  std::vector<char> seen(n, 0);
  if (n > 0) seen[0] = 1;
  for (;;) {
    int start = -1;
    for (int k = 1; k < n; ++k)
      if (!seen[k] && (start < 0 || less(k, start))) start = k;
    if (start < 0) break;
    seen[start] = 1;
    size_t head = order.size();
    order.push_back(start);
    while (head < order.size()) {
      const int v = order[head++];
      std::vector<int> next;
      for (int u : adj[v])
        if (!seen[u]) {
          seen[u] = 1;
          next.push_back(u);
        }
      std::sort(next.begin(), next.end(), less);
      order.insert(order.end(), next.begin(), next.end());
    }
  }
  std::reverse(order.begin(), order.end());
  std::vector<int> pos(n, -1);
  for (size_t q = 0; q < order.size(); ++q) pos[order[q]] = (int)q;
  return pos;
}

double PoseGraph::optimize(int iterations, double lam) {
  const int n = (int)poses.size();
  const int m = 7 * (n - 1);  // node 0 is held
  double c = cost();
  if (m <= 0 || edges.empty()) return c;
  // block positions (reverse Cuthill-McKee) and the lower envelope of the normal equations
  const std::vector<int> pos = rcm_positions(n, edges);
  std::vector<int> envb(n - 1), env(m);
  for (int q = 0; q < n - 1; ++q) envb[q] = q;
  for (const Edge& e : edges) {
    if (e.i <= 0 || e.j <= 0) continue;
    const int a = pos[e.i], b2 = pos[e.j];
    const int lo = std::min(a, b2), hi = std::max(a, b2);
    envb[hi] = std::min(envb[hi], lo);
  }
  double env_work = 0.0;
  for (int r = 0; r < m; ++r) {
    env[r] = 7 * envb[r / 7];
    env_work += 0.5 * (double)(r - env[r] + 1) * (double)(r - env[r] + 1);
  }
  // the envelope solve when it saves most of the dense work, else the threaded dense one
  const bool use_env = env_work < 0.25 * (double)m * m * m / 6.0;
  std::vector<double> H((size_t)m * m), b(m), A, x;
  for (int it = 0; it < iterations; ++it) {
    std::fill(H.begin(), H.end(), 0.0);
    std::fill(b.begin(), b.end(), 0.0);
    for (const Edge& e : edges) {
      double r[7];
      residual(e, r);
      const double m2 = maha2(r, e.W.data());
      const double mm = std::sqrt(std::max(m2, 0.0));
      const double wgt = mm <= huber ? 1.0 : huber / mm;  // iteratively reweighted (Huber)
      double W[49];
      for (int q = 0; q < 49; ++q) W[q] = wgt * e.W[q];
      double Ji[49];
      adjoint(mul(sim3_inv(poses[e.j]), poses[e.i]), Ji);
      for (double& v : Ji) v = -v;
      static const double Id[49] = {1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0,
                                    0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1};
      const double* J[2] = {Ji, Id};
      const int col[2] = {e.i > 0 ? 7 * pos[e.i] : -1, e.j > 0 ? 7 * pos[e.j] : -1};
      double JtW[2][49];  // J^T W per block
      for (int q = 0; q < 2; ++q)
        for (int a = 0; a < 7; ++a)
          for (int c2 = 0; c2 < 7; ++c2) {
            double s = 0.0;
            for (int k = 0; k < 7; ++k) s += J[q][7 * k + a] * W[7 * k + c2];
            JtW[q][7 * a + c2] = s;
          }
      for (int qa = 0; qa < 2; ++qa) {
        if (col[qa] < 0) continue;
        for (int a = 0; a < 7; ++a) {
          double s = 0.0;
          for (int k = 0; k < 7; ++k) s += JtW[qa][7 * a + k] * r[k];
          b[col[qa] + a] += s;
        }
        for (int qb = 0; qb < 2; ++qb) {
          if (col[qb] < 0) continue;
          for (int a = 0; a < 7; ++a)
            for (int c2 = 0; c2 < 7; ++c2) {
              double s = 0.0;
              for (int k = 0; k < 7; ++k) s += JtW[qa][7 * a + k] * J[qb][7 * k + c2];
              H[(size_t)(col[qa] + a) * m + col[qb] + c2] += s;
            }
        }
      }
    }
    double cnew = c;
    for (;;) {
      A = H;
      for (int i = 0; i < m; ++i) A[(size_t)i * m + i] += lam * std::max(H[(size_t)i * m + i], 1e-12);
      x = b;
      for (double& v : x) v = -v;
      const std::vector<M4> old = poses;
      bool solved = use_env ? envelope_cholesky_solve(A, m, env, x) : cholesky_solve(A, m, x, threads);
      if (solved) {
        for (int k = 1; k < n; ++k) poses[k] = mul(poses[k], sim3_exp(&x[7 * pos[k]]));
        cnew = cost();
      }
      if (solved && std::isfinite(cnew) && cnew <= c) {
        lam = std::max(lam * 0.3, 1e-9);
        break;
      }
      poses = old;
      lam *= 10.0;
      if (lam > 1e8) return c;
    }
    const bool done = c - cnew < 1e-10 * std::max(c, 1e-30);
    c = cnew;
    if (done) break;
  }
  return c;
}

}  // namespace slam
}  // namespace lsdg

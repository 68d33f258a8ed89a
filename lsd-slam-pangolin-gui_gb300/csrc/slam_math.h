// slam_math.h -- Sim3 algebra and the keyframe pose graph of the full SLAM loop (host C++, double).
//
// The reference keeps its keyframe graph in g2o (KeyFrameGraph, inside the unvendored lsd-slam
// import; lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:148-168 shows the graph it hands the
// viewer: keyframe ids and Sim3 camToWorld poses).  g2o is absent, so this is the project's own
// small graph: nodes are camera-to-world Sim3 poses T = [[s R, t], [0, 1]], an edge (i, j, Z, W)
// says "pose j seen from pose i is Z" with 7x7 information W in the twist order (v, omega,
// log-scale), the cost is sum rho(r^T W r) with r = log(Z^-1 T_i^-1 T_j) and a Huber kernel rho on
// the Mahalanobis norm; perturbations act on the right (T <- T exp(d)), so to first order
// r(d) = r + d_j - Adj(T_j^-1 T_i) d_i.  Damped Gauss-Newton over the normal equations, with the
// nodes in reverse Cuthill-McKee order and factorised inside their lower envelope (or, when the
// envelope is wide, by a dense blocked Cholesky whose trailing updates run on several host threads).
#pragma once

#include <array>
#include <vector>

namespace lsdg {
namespace slam {

struct M4 {
  double a[16];  // row-major 4x4
  static M4 identity();
  double& operator()(int r, int c) { return a[4 * r + c]; }
  double operator()(int r, int c) const { return a[4 * r + c]; }
};

M4 mul(const M4& A, const M4& B);
M4 sim3_inv(const M4& T);
double sim3_scale(const M4& T);            // cube root of det(sR)
void so3_exp(const double w[3], double R[9]);
void so3_log(const double R[9], double w[3]);
M4 sim3_exp(const double xi[7]);
void sim3_log(const M4& T, double xi[7]);
void adjoint(const M4& T, double A[49]);
void orthonormalize(double R[9]);          // nearest rotation to a near-rotation (row-major 3x3)
M4 from13(const double p[13]);             // {R, t, s} -> [[s R, t], [0, 1]], R brought onto SO(3)
void to13(const M4& T, double p[13]);
M4 from12(const double p[12]);             // [R | t] row-major, R brought onto SO(3)
void to12(const M4& T, double p[12]);

struct Edge {
  int i, j;
  M4 Z;
  std::array<double, 49> W;
};

class PoseGraph {
 public:
  std::vector<M4> poses;
  std::vector<Edge> edges;
  double huber = 3.0;  // robust kernel on the Mahalanobis norm of an edge residual (in sigmas)
  int threads = 1;     // host threads of the Cholesky's trailing updates

  int add_node(const M4& T) {
    poses.push_back(T);
    return (int)poses.size() - 1;
  }
  void add_edge(int i, int j, const M4& Z, const double W[49]);
  void residual(const Edge& e, double r[7]) const;
  double cost() const;
  // Damped Gauss-Newton with node 0 held; returns the final cost.
  double optimize(int iterations, double lam = 1e-4);
};

// Cholesky factorisation in place of the m x m symmetric positive definite matrix A (row-major,
// lower triangle used) and the solve A x = b; false when a pivot is not positive.
bool cholesky_solve(std::vector<double>& A, int m, std::vector<double>& b, int threads);
// The same restricted to the lower envelope (row i starts at column env[i]); the optimiser orders the
// nodes by reverse Cuthill-McKee (rcm_positions) and uses it when it saves most of the dense work.
bool envelope_cholesky_solve(std::vector<double>& A, int m, const std::vector<int>& env, std::vector<double>& b);
std::vector<int> rcm_positions(int n, const std::vector<Edge>& edges);


}  // namespace slam
}  // namespace lsdg

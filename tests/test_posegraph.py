"""CPU tests of the Sim3 pose graph used by the sequence driver: exp/log round trip and the
adjoint identity, exact recovery from consistent measurements, drift correction by a loop edge,
and the Umeyama alignment of the trajectory error."""
import math

import numpy as np
import pytest

import posegraph as G


def rand_sim3(rng, scale_range=(0.7, 1.4), trans=1.0, angle=0.8):
    xi = np.concatenate([rng.normal(size=3) * trans, rng.normal(size=3) * angle / math.sqrt(3),
                         [math.log(rng.uniform(*scale_range))]])
    return G.sim3_exp(xi), xi


@pytest.mark.parametrize("seed", range(5))
def test_exp_log_round_trip_and_adjoint(seed):
    rng = np.random.default_rng(seed)
    T, xi = rand_sim3(rng)
    np.testing.assert_allclose(G.sim3_log(T), xi, atol=1e-10)
    S, _ = rand_sim3(rng)
    # S exp(xi) S^-1 = exp(Adj(S) xi)
    lhs = S @ G.sim3_exp(xi) @ G.sim3_inv(S)
    np.testing.assert_allclose(lhs, G.sim3_exp(G.adjoint(S) @ xi), atol=1e-10)
    np.testing.assert_allclose(G.from13(G.to13(T)), T, atol=1e-12)


def test_consistent_chain_is_recovered():
    rng = np.random.default_rng(1)
    truth = [np.eye(4)]
    for _ in range(6):
        truth.append(truth[-1] @ rand_sim3(rng, trans=0.3, angle=0.2)[0])
    g = G.PoseGraph()
    g.add_node(truth[0])
    for k in range(1, len(truth)):
        g.add_node(truth[k] @ rand_sim3(rng, (0.9, 1.1), 0.1, 0.05)[0])  # perturbed start
    for k in range(1, len(truth)):
        g.add_edge(k - 1, k, G.sim3_inv(truth[k - 1]) @ truth[k], np.eye(7))
    g.add_edge(0, 3, G.sim3_inv(truth[0]) @ truth[3], np.eye(7))
    cost = g.optimize(30)
    assert cost < 1e-16
    for k in range(len(truth)):
        np.testing.assert_allclose(g.poses[k], truth[k], atol=1e-7)


def test_loop_edge_spreads_drift():
    """A chain with scale drift in every odometry edge and one accurate loop edge back to the start:
    optimisation spreads the error and brings the last pose close to the truth."""
    n = 12
    truth = [np.eye(4)]
    step = G.sim3_exp(np.array([0.3, 0, 0, 0, 2 * math.pi / n, 0, 0]))
    for _ in range(n):
        truth.append(truth[-1] @ step)
    drift = G.sim3_exp(np.array([0.01, 0, 0, 0, 0.01, 0, 0.02]))
    g = G.PoseGraph()
    g.add_node(truth[0])
    for k in range(1, n + 1):
        Z = G.sim3_inv(truth[k - 1]) @ truth[k] @ drift
        g.add_node(g.poses[-1] @ Z)
        g.add_edge(k - 1, k, Z, np.eye(7))
    g.add_edge(0, n, G.sim3_inv(truth[0]) @ truth[n], 100 * np.eye(7))
    before = np.linalg.norm(g.poses[n][:3, 3] - truth[n][:3, 3])
    g.optimize(30)
    after = np.linalg.norm(g.poses[n][:3, 3] - truth[n][:3, 3])
    assert after < 0.1 * before


def test_ate_alignment():
    rng = np.random.default_rng(3)
    gt = rng.normal(size=(50, 3))
    R = G.so3_exp(np.array([0.3, -0.2, 0.5]))
    est = (2.5 * (R @ gt.T)).T + np.array([1.0, 2.0, 3.0])
    rmse, (s, R2, t) = G.ate_rmse(est, gt)
    assert rmse < 1e-10 and s == pytest.approx(1 / 2.5)
    noisy = est + 0.01 * rng.normal(size=est.shape)
    assert G.ate_rmse(noisy, gt)[0] < 0.01


@pytest.mark.parametrize("xi", [[0.1, 0.2, -0.3, 0, 0, 0, 0], [0.1, 0.2, -0.3, 1e-5, 2e-5, 0, 0.3],
                                [0.1, 0.2, -0.3, 0.4, -0.2, 0.1, 0], [0.1, 0.2, -0.3, 0.4, -0.2, 0.1, -1.2],
                                [0.1, 0.2, -0.3, 2e-4, 0, 0, 2.5], [0.1, 0.2, -0.3, 2.5, 0.3, 0.1, 1e-7]])
def test_closed_form_V_matches_quadrature(xi):
    w, s = np.array(xi[3:6]), xi[6]
    np.testing.assert_allclose(G._V(w, s), G._V_quadrature(w, s), rtol=0, atol=1e-11)


def test_huber_kernel_resists_a_bad_edge():
    rng = np.random.default_rng(5)
    truth = [np.eye(4)]
    for _ in range(5):
        truth.append(truth[-1] @ rand_sim3(rng, trans=0.3, angle=0.2)[0])
    g = G.PoseGraph()
    for T in truth:
        g.add_node(T)
    for k in range(1, 6):
        g.add_edge(k - 1, k, G.sim3_inv(truth[k - 1]) @ truth[k], 1e4 * np.eye(7))
    g.add_edge(0, 4, G.sim3_exp(np.array([3.0, 0, 0, 1.0, 0, 0, 0.5])), 1e4 * np.eye(7))  # wrong
    g2 = G.PoseGraph()
    g2.poses = [p.copy() for p in g.poses]
    g2.edges = list(g.edges)
    g2.huber = float("inf")                    # plain least squares
    g.optimize(20)
    g2.optimize(20)
    err = max(np.linalg.norm(g.poses[k][:3, 3] - truth[k][:3, 3]) for k in range(6))
    err_ls = max(np.linalg.norm(g2.poses[k][:3, 3] - truth[k][:3, 3]) for k in range(6))
    # the kernel bounds the outlier's pull to ~3 sigma (0.01 m) per edge of the chain it bends
    assert err < 0.2 and err_ls > 5 * err, (err, err_ls)

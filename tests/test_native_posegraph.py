"""CPU tests of the library's Sim3 pose graph (lsdg_posegraph_*, csrc/slam_math.cu) against the
independent numpy restatement in tests/posegraph.py: exp / log agree, and the same graphs converge
to the same poses (consistent chains recovered exactly, drift spread by a loop edge, a bad edge held
off by the Huber kernel)."""
import math

import numpy as np
import pytest

import lsdg
import posegraph as G


def rand_sim3(rng, scale_range=(0.7, 1.4), trans=1.0, angle=0.8):
    xi = np.concatenate([rng.normal(size=3) * trans, rng.normal(size=3) * angle / math.sqrt(3),
                         [math.log(rng.uniform(*scale_range))]])
    return G.sim3_exp(xi), xi


@pytest.mark.parametrize("seed", range(6))
def test_exp_log_match_numpy(seed):
    rng = np.random.default_rng(seed)
    T, xi = rand_sim3(rng)
    np.testing.assert_allclose(G.from13(lsdg.sim3_exp13(xi)), T, atol=1e-12)
    np.testing.assert_allclose(lsdg.sim3_log13(G.to13(T)), xi, atol=1e-10)


@pytest.mark.parametrize("xi", [[0.1, 0.2, -0.3, 0, 0, 0, 0], [0.1, 0.2, -0.3, 1e-5, 2e-5, 0, 0.3],
                                [0.1, 0.2, -0.3, 2e-4, 0, 0, 2.5], [0.1, 0.2, -0.3, 2.5, 0.3, 0.1, 1e-7],
                                [0.0, 0.0, 0.0, 3.1415, 0.0, 0.0, 0.0]])
def test_exp_log_branches(xi):
    T = G.sim3_exp(np.array(xi))
    np.testing.assert_allclose(G.from13(lsdg.sim3_exp13(xi)), T, atol=1e-11)
    np.testing.assert_allclose(G.sim3_exp(lsdg.sim3_log13(G.to13(T))), T, atol=1e-9)


def _both(truth_nodes, edges):
    py = G.PoseGraph()
    cg = lsdg.NativePoseGraph()
    for T in truth_nodes:
        py.add_node(T)
        cg.add_node(G.to13(T))
    for i, j, Z, W in edges:
        py.add_edge(i, j, Z, W)
        cg.add_edge(i, j, G.to13(Z), W)
    return py, cg


def test_consistent_chain_recovered_like_numpy():
    rng = np.random.default_rng(1)
    truth = [np.eye(4)]
    for _ in range(6):
        truth.append(truth[-1] @ rand_sim3(rng, trans=0.3, angle=0.2)[0])
    start = [truth[0]] + [truth[k] @ rand_sim3(rng, (0.9, 1.1), 0.1, 0.05)[0] for k in range(1, len(truth))]
    edges = [(k - 1, k, G.sim3_inv(truth[k - 1]) @ truth[k], np.eye(7)) for k in range(1, len(truth))]
    edges.append((0, 3, G.sim3_inv(truth[0]) @ truth[3], np.eye(7)))
    py, cg = _both(start, edges)
    assert cg.optimize(30) < 1e-16
    py.optimize(30)
    for k in range(len(truth)):
        np.testing.assert_allclose(G.from13(cg.pose(k)), truth[k], atol=1e-7)
        np.testing.assert_allclose(G.from13(cg.pose(k)), py.poses[k], atol=1e-7)
    cg.close()


def test_loop_edge_and_huber_like_numpy():
    n = 12
    truth = [np.eye(4)]
    step = G.sim3_exp(np.array([0.3, 0, 0, 0, 2 * math.pi / n, 0, 0]))
    for _ in range(n):
        truth.append(truth[-1] @ step)
    drift = G.sim3_exp(np.array([0.01, 0, 0, 0, 0.01, 0, 0.02]))
    nodes, edges = [truth[0]], []
    for k in range(1, n + 1):
        Z = G.sim3_inv(truth[k - 1]) @ truth[k] @ drift
        nodes.append(nodes[-1] @ Z)
        edges.append((k - 1, k, Z, np.eye(7)))
    edges.append((0, n, G.sim3_inv(truth[0]) @ truth[n], 100 * np.eye(7)))
    edges.append((0, 5, G.sim3_exp(np.array([3.0, 0, 0, 1.0, 0, 0, 0.5])), 1e2 * np.eye(7)))  # wrong
    py, cg = _both(nodes, edges)
    c_py = py.optimize(30)
    c_cg = cg.optimize(30)
    assert c_cg == pytest.approx(c_py, rel=1e-6)
    for k in range(n + 1):
        np.testing.assert_allclose(G.from13(cg.pose(k)), py.poses[k], atol=1e-6)
    before = np.linalg.norm(nodes[n][:3, 3] - truth[n][:3, 3])
    after = np.linalg.norm(G.from13(cg.pose(n))[:3, 3] - truth[n][:3, 3])
    assert after < 0.1 * before
    cg.close()


def test_large_chain_uses_the_envelope_factorisation():
    """A 200-node chain with edges that skip 7 nodes (1,393 unknowns): in reverse Cuthill-McKee order
    its envelope is a few blocks wide, so the envelope factorisation solves it."""
    rng = np.random.default_rng(7)
    truth = [np.eye(4)]
    for _ in range(199):
        truth.append(truth[-1] @ rand_sim3(rng, (0.98, 1.02), 0.1, 0.05)[0])
    start = [truth[0]] + [T @ rand_sim3(rng, (0.99, 1.01), 0.01, 0.01)[0] for T in truth[1:]]
    edges = [(k - 1, k, G.sim3_inv(truth[k - 1]) @ truth[k], np.eye(7)) for k in range(1, 200)]
    edges += [(k - 7, k, G.sim3_inv(truth[k - 7]) @ truth[k], np.eye(7)) for k in range(7, 200, 3)]
    _, cg = _both(start, edges)
    assert cg.optimize(20) < 1e-14
    for k in (50, 120, 199):
        np.testing.assert_allclose(G.from13(cg.pose(k)), truth[k], atol=1e-6)
    cg.close()


def test_poses_enter_on_so3():
    """A pose whose rotation has drifted off SO(3) (a tracker's rounding, compounded) enters the graph
    as the nearest rotation: the stored rotation is orthonormal with determinant 1 and the scale and
    translation are kept."""
    rng = np.random.default_rng(3)
    T, _ = rand_sim3(rng)
    p = G.to13(T)
    bent = p.copy()
    bent[:9] = (p[:9].reshape(3, 3) @ (np.eye(3) + 0.02 * rng.normal(size=(3, 3)))).ravel()
    g = lsdg.NativePoseGraph()
    g.add_node(bent)
    q = g.pose(0)
    R = q[:9].reshape(3, 3)
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
    assert abs(np.linalg.det(R) - 1.0) < 1e-12
    np.testing.assert_allclose(R, p[:9].reshape(3, 3), atol=0.05)
    assert q[12] == p[12] and np.array_equal(q[9:12], p[9:12])


def test_branch_kept_when_inputs_drift_off_so3():
    """A loop with a 12 % scale disagreement and a branch of 20 keyframes hanging off it, every pose
    and edge given with a rotation off SO(3) by 1e-3: the optimiser spreads the loop's disagreement
    and leaves the branch's relative scales at 1 (a chain of compositions of non-rotations once drove
    such a branch's scale up 10x)."""
    rng = np.random.default_rng(5)

    def bend(p):
        q = np.array(p, np.float64)
        q[:9] = (q[:9].reshape(3, 3) @ (np.eye(3) + 1e-3 * rng.normal(size=(3, 3)))).ravel()
        return q

    n = 24
    P = []
    for k in range(n):
        a = 2 * np.pi * k / n
        T = np.eye(4)
        T[:3, :3] = G.so3_exp(np.array([0, a, 0]))
        T[:3, 3] = [math.cos(a), 0.0, math.sin(a)]
        P.append(T)
    info = np.diag([1e6, 1e6, 1e6, 1e7, 1e7, 1e7, 1e7])
    g = lsdg.NativePoseGraph()
    for T in P:
        g.add_node(bend(G.to13(T)))
    for k in range(n - 1):
        g.add_edge(k, k + 1, bend(G.to13(G.sim3_inv(P[k]) @ P[k + 1])), info)
    Zl = G.sim3_inv(P[0]) @ P[n - 1]
    Zl[:3, :3] *= 0.88
    g.add_edge(0, n - 1, bend(G.to13(Zl)), info)
    Q = [P[3]]
    step = np.eye(4)
    step[:3, :3] = G.so3_exp(np.array([0, 0.05, 0]))
    step[:3, 3] = [0.05, 0, 0.01]
    idx = [3]
    for k in range(20):
        Q.append(Q[-1] @ step)
        idx.append(g.add_node(bend(G.to13(Q[-1]))))
        g.add_edge(idx[-2], idx[-1], bend(G.to13(step)), info)
    g.optimize(20)
    rel = [g.pose(idx[k])[12] / g.pose(idx[k - 1])[12] for k in range(1, len(idx))]
    np.testing.assert_allclose(rel, 1.0, atol=1e-6)


def test_densely_connected_graph_uses_the_threaded_factorisation():
    """80 nodes each tied to 12 random others (553 unknowns): no order keeps the envelope narrow, so
    the dense blocked Cholesky with threaded trailing updates solves it; consistent edges give the
    truth back."""
    rng = np.random.default_rng(11)
    n = 80
    truth = [np.eye(4)] + [rand_sim3(rng, (0.9, 1.1), 1.0, 0.5)[0] for _ in range(n - 1)]
    start = [truth[0]] + [T @ rand_sim3(rng, (0.99, 1.01), 0.01, 0.01)[0] for T in truth[1:]]
    edges = [(k - 1, k, G.sim3_inv(truth[k - 1]) @ truth[k], np.eye(7)) for k in range(1, n)]
    for k in range(n):
        for j in rng.choice(n, 12, replace=False):
            if j != k:
                edges.append((int(k), int(j), G.sim3_inv(truth[k]) @ truth[j], np.eye(7)))
    _, cg = _both(start, edges)
    assert cg.optimize(20) < 1e-14
    for k in (17, 45, 79):
        np.testing.assert_allclose(G.from13(cg.pose(k)), truth[k], atol=1e-6)
    cg.close()


def test_two_laps_like_numpy():
    """A path driven twice: the second lap's keyframes tied to the first lap's (far apart in creation
    order, neighbours in reverse Cuthill-McKee order), with drift on the odometry and a scale
    disagreement on the ties; the envelope solve converges to the numpy restatement's poses."""
    rng = np.random.default_rng(13)
    n = 24
    step = G.sim3_exp(np.array([0.25, 0, 0, 0, 2 * math.pi / n, 0, 0]))
    truth = [np.eye(4)]
    for _ in range(2 * n - 1):
        truth.append(truth[-1] @ step)
    drift = G.sim3_exp(np.array([0.004, 0.002, 0, 0.001, 0.003, 0, 0.003]))
    nodes, edges = [truth[0]], []
    for k in range(1, 2 * n):
        Z = G.sim3_inv(truth[k - 1]) @ truth[k] @ drift
        nodes.append(nodes[-1] @ Z)
        edges.append((k - 1, k, Z, np.eye(7) * 10))
    for k in range(n, 2 * n):  # second lap seen from the first, 5 % scale disagreement
        Z = G.sim3_inv(truth[k - n]) @ truth[k]
        Z[:3, :3] *= 1.05
        edges.append((k - n, k, Z, np.eye(7)))
    py, cg = _both(nodes, edges)
    c_py = py.optimize(30)
    c_cg = cg.optimize(30)
    assert c_cg == pytest.approx(c_py, rel=1e-6)
    for k in range(0, 2 * n, 5):
        np.testing.assert_allclose(G.from13(cg.pose(k)), py.poses[k], atol=1e-6)
    cg.close()

"""The oracle's soft-min against its definition assembled from its own
pair distances: L = m - tau log sum over waypoints and (link, object)
pairs with d < m + 30 tau of exp(-(d - m) / tau), m the trajectory's minimum
(the workload's truncation; geometry_ad.py:613-814 sums the same kind of
terms), and its gradient against central differences of L on a small arm.
CPU only."""

import numpy as np

from klampt_gb300 import scenes as sc


def _scene():
    from oracle.oracle_py import Oracle
    robot = sc.arm(3, rings=4, segments=8)
    rng = np.random.default_rng(11)
    spheres = [sc.icosphere_mesh(c, r, 1) for c, r in
               zip(rng.uniform([0.1, -0.4, 0.1], [0.5, 0.4, 0.8], (6, 3)), rng.uniform(0.03, 0.08, 6))]
    env = sc.env_from_objects("spheres", spheres)
    return robot, env, Oracle(robot, env)


def test_softmin_equals_its_definition():
    robot, env, o = _scene()
    rng = np.random.default_rng(12)
    T, W, tau = 3, 5, 0.01
    q = sc.noisy_trajectories(robot, T, W, rng)
    L, _ = o.softmin(q, tau)
    for t in range(T):
        dmin, _, _, _ = o.min_distance(q[t], 1e3, want_grad=False)
        m = float(dmin.min())
        terms = []
        for w in range(W):
            _, dist = o.pair_features(q[t, w], m + 30 * tau)
            terms.extend(dist.tolist())
        terms = np.asarray(terms)
        assert terms.size > 0 and abs(terms.min() - m) <= 1e-12
        ref = m - tau * np.log(np.exp(-(terms - m) / tau).sum())
        assert abs(L[t] - ref) <= 1e-12 * max(1.0, abs(ref)), (t, L[t], ref)


def test_softmin_gradient_matches_central_differences():
    robot, env, o = _scene()
    rng = np.random.default_rng(13)
    T, W, tau, h = 2, 3, 0.01, 1e-5
    q = sc.noisy_trajectories(robot, T, W, rng).astype(np.float64)
    _, G = o.softmin(q.astype(np.float32), tau)
    ok = 0
    for t in range(T):
        for w in range(W):
            for j in range(robot.num_links):
                qp, qm = q[t:t + 1].copy(), q[t:t + 1].copy()
                qp[0, w, j] += h
                qm[0, w, j] -= h
                qp32, qm32 = qp.astype(np.float32), qm.astype(np.float32)
                step = float(qp32[0, w, j]) - float(qm32[0, w, j])
                Lp, _ = o.softmin(qp32, tau, want_grad=False)
                Lm, _ = o.softmin(qm32, tau, want_grad=False)
                fd = (Lp[0] - Lm[0]) / step
                scale = max(np.abs(G[t]).max(), 1e-6)
                ok += abs(fd - G[t, w, j]) <= 1e-4 * scale
    # entries at a feature switch (a kink) may differ; they are rare
    assert ok >= 0.9 * T * W * robot.num_links, ok

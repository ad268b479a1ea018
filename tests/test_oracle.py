"""Pins the FP64 oracle: known-answer tests (including the rotation
convention vector of the reference's own tests/test_math_so3.py), independent
cross-checks of the canonical triangle predicates, and brute force vs BVH
culling.  CPU only."""

import math
import os

import numpy as np
import pytest

from klampt_gb300 import scenes as sc
from oracle import oracle_py as op

NT = os.cpu_count() or 2


def one_link_robot(mesh, axis=(0, 0, 1)):
    V, F = mesh
    return sc.RobotSpec(name="one", parents=np.array([-1], np.int32), joint_types=np.zeros(1, np.int32),
                        T0_parent=np.array([[1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0]], np.float64),
                        axes=np.array([axis], np.float64), qmin=np.array([-math.pi]), qmax=np.array([math.pi]),
                        meshes=[(V, F)])


def test_sincos_accuracy():
    x = np.random.default_rng(0).uniform(-100, 100, 200000)
    s, c = op.sincos(x)
    ulp = lambda a, b: np.max(np.abs(a - b) / np.spacing(np.maximum(np.abs(b), 1e-300)))
    assert ulp(s, np.sin(x)) <= 2 and ulp(c, np.cos(x)) <= 2
    s0, c0 = op.sincos(np.array([0.0, math.pi / 2, -math.pi]))
    assert s0[0] == 0.0 and c0[0] == 1.0
    assert abs(s0[1] - 1) < 1e-16 and abs(c0[2] + 1) < 1e-16


def test_rotation_convention_matches_reference_so3_vector():
    """tests/test_math_so3.py:15-19 of the reference: the quaternion
    (w,x,y,z) = (-4.32978e-17, -0.707107, 4.32978e-17, 0.707107) has
    roll, pitch, yaw = (0, pi/2, pi), i.e. R = Rz(yaw) Ry(pitch) Rx(roll).
    A z-y-x chain of revolute joints at those angles must give that matrix."""
    w, x, y, z = (-4.32978e-17, -0.707107, 4.32978e-17, 0.707107)
    n = math.sqrt(w * w + x * x + y * y + z * z)
    w, x, y, z = w / n, x / n, y / n, z / n
    Rq = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                   [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                   [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    I = [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0]
    box = sc.box_mesh((0, 0, 0), (0.1, 0.1, 0.1))
    robot = sc.RobotSpec(name="zyx", parents=np.array([-1, 0, 1], np.int32), joint_types=np.zeros(3, np.int32),
                         T0_parent=np.array([I, I, I], np.float64),
                         axes=np.array([[0, 0, 1], [0, 1, 0], [1, 0, 0]], np.float64),
                         qmin=np.full(3, -4.0), qmax=np.full(3, 4.0), meshes=[box, box, box])
    o = op.Oracle(robot, None)
    T = o.fk(np.array([math.pi, math.pi / 2, 0.0]))
    assert np.allclose(T[2, :9].reshape(3, 3), Rq, atol=2e-6)


def test_fk_planar_closed_form():
    L1, L2 = 0.4, 0.25
    I = [1, 0, 0, 0, 1, 0, 0, 0, 1]
    box = sc.box_mesh((0, 0, 0), (0.01, 0.01, 0.01))
    robot = sc.RobotSpec(name="planar", parents=np.array([-1, 0, 1], np.int32),
                         joint_types=np.array([0, 0, 2], np.int32),
                         T0_parent=np.array([I + [0, 0, 0], I + [L1, 0, 0], I + [L2, 0, 0]], np.float64),
                         axes=np.array([[0, 0, 1], [0, 0, 1], [0, 0, 1]], np.float64),
                         qmin=np.array([-4, -4, 0.0]), qmax=np.array([4, 4, 0.0]), meshes=[box, box, box])
    o = op.Oracle(robot, None)
    for q0, q1 in [(0.3, -1.1), (2.5, 0.7), (-3.0, 3.0)]:
        T = o.fk(np.array([q0, q1, 0.0]))
        ex = L1 * math.cos(q0) + L2 * math.cos(q0 + q1)
        ey = L1 * math.sin(q0) + L2 * math.sin(q0 + q1)
        assert abs(T[2, 9] - ex) < 1e-15 and abs(T[2, 10] - ey) < 1e-15
    # prismatic: translation along the axis by q
    robot.joint_types = np.array([1, 0, 2], np.int32)
    o = op.Oracle(robot, None)
    T = o.fk(np.array([0.2, 0.0, 0.0]))
    assert abs(T[0, 11] - 0.2) < 1e-16


@pytest.mark.parametrize("d,expect", [(0.5, 1), (0.999, 1), (1.0, 1), (1.0 + 1e-9, 0), (1.2, 0)])
def test_box_box_known_answers(d, expect):
    """Unit cubes (half extent 0.5) at centre distance d collide iff d <= 1;
    touching faces count as collision."""
    robot = one_link_robot(sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5)))
    env = sc.env_from_objects("b", [sc.box_mesh((d, 0.0, 0.0), (0.5, 0.5, 0.5))])
    o = op.Oracle(robot, env)
    eh, _, _ = o.check_configs(np.zeros((1, 1), np.float32))
    assert eh[0] == expect


def test_containment_is_not_collision():
    """Mesh-mesh collision tests surfaces (PQP semantics): a box strictly
    inside another does not collide."""
    robot = one_link_robot(sc.box_mesh((0, 0, 0), (0.1, 0.1, 0.1)))
    env = sc.env_from_objects("b", [sc.box_mesh((0, 0, 0), (1, 1, 1))])
    eh, _, _ = op.Oracle(robot, env).check_configs(np.zeros((1, 1), np.float32))
    assert eh[0] == 0


def test_margin_within_distance():
    robot = one_link_robot(sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5)))
    robot.margins = np.array([0.05])
    env = sc.env_from_objects("b", [sc.box_mesh((1.04, 0, 0), (0.5, 0.5, 0.5))])
    eh, _, _ = op.Oracle(robot, env).check_configs(np.zeros((1, 1), np.float32))
    assert eh[0] == 1
    env = sc.env_from_objects("b", [sc.box_mesh((1.06, 0, 0), (0.5, 0.5, 0.5))])
    eh, _, _ = op.Oracle(robot, env).check_configs(np.zeros((1, 1), np.float32))
    assert eh[0] == 0


def test_sphere_sphere_distance_and_penetration():
    """|c1-c2| - r1 - r2 (geometry_ad.py:160-163) within the icospheres'
    polyhedral tolerance; overlapping spheres give negative distance."""
    r1, r2 = 0.1, 0.2
    robot = one_link_robot(sc.icosphere_mesh((0, 0, 0), r1, 3))
    for D, tol in [(1.0, 2e-3), (0.25, 4e-3)]:
        env = sc.env_from_objects("s", [sc.icosphere_mesh((D, 0, 0), r2, 3)])
        o = op.Oracle(robot, env)
        res = o.pair_distance(np.zeros(1, np.float32), 0, 0)
        assert res["found"]
        assert abs(res["d"] - (D - r1 - r2)) < tol, res["d"]
        if D < r1 + r2:
            assert res["signed"] and res["d"] < 0
        else:
            assert abs(res["cp"][0] - r1) < tol and abs(res["cq"][0] - (D - r2)) < tol
            assert np.allclose(res["dir"], [-1, 0, 0], atol=0.05)


def _np_seg_tri(p0, p1, a, b, c):
    """Segment / triangle crossing (independent: Moller-Trumbore on the
    segment's line), returns (crosses, robust)."""
    e1, e2 = b - a, c - a
    d = p1 - p0
    h = np.cross(d, e2)
    det = e1 @ h
    if abs(det) < 1e-12:
        return False, False
    f = 1.0 / det
    s = p0 - a
    u = f * (s @ h)
    qv = np.cross(s, e1)
    v = f * (d @ qv)
    t = f * (e2 @ qv)
    m = 1e-9
    inside = u > m and v > m and u + v < 1 - m and t > m and t < 1 - m
    near = min(abs(u), abs(v), abs(1 - u - v), abs(t), abs(1 - t)) < 1e-7
    return inside, not near


def test_tri_tri_overlap_independent_crosscheck():
    rng = np.random.default_rng(5)
    agree = 0
    for _ in range(3000):
        P = rng.normal(size=(3, 3))
        Q = rng.normal(size=(3, 3)) * 0.8 + rng.normal(size=3) * 0.5
        hit, d2, cp, cq = op.tri_tri(P, Q)
        cross, robust = False, True
        for (X, Y) in ((P, Q), (Q, P)):
            for i in range(3):
                c, r = _np_seg_tri(X[i], X[(i + 1) % 3], Y[0], Y[1], Y[2])
                cross |= c
                robust &= r
        if not robust:
            continue
        assert hit == cross
        assert (d2 == 0.0) == hit
        agree += 1
    assert agree > 2500


def test_tri_tri_distance_vs_sampling():
    rng = np.random.default_rng(6)
    g = np.linspace(0, 1, 41)
    uu, vv = np.meshgrid(g, g)
    m = (uu + vv) <= 1
    bary = np.stack([1 - uu[m] - vv[m], uu[m], vv[m]], axis=1)
    for _ in range(60):
        P = rng.normal(size=(3, 3))
        Q = rng.normal(size=(3, 3)) + rng.normal(size=3) * 3
        hit, d2, cp, cq = op.tri_tri(P, Q)
        if hit:
            continue
        SP, SQ = bary @ P, bary @ Q
        dmin = np.sqrt(((SP[:, None, :] - SQ[None, :, :]) ** 2).sum(-1).min())
        d = math.sqrt(d2)
        assert d <= dmin + 1e-12
        assert dmin - d < 0.15 * max(np.ptp(P, 0).max(), np.ptp(Q, 0).max()) / 40 * 4
        assert abs(np.linalg.norm(cp - cq) - d) < 1e-12


def test_bvh_culling_matches_brute_force():
    """The oracle's BVH traversal returns exactly the all-pairs verdicts."""
    robot = sc.arm(6, rings=4, segments=12)
    env = sc.env_from_objects("boxes", sc.random_boxes(12, np.random.default_rng(3)))
    o = op.Oracle(robot, env)
    q = sc.uniform_configs(robot, 96, np.random.default_rng(4))
    eh, sh, _ = o.check_configs(q, nthreads=NT)
    eb, sb = o.check_configs_brute(q)
    assert np.array_equal(eh, eb) and np.array_equal(sh, sb)
    assert 0 < eh.sum() < len(q) and 0 < sh.sum() < len(q)


def test_edge_first_hit_semantics():
    """first_hit = first infeasible configuration a + (k/n)(b-a), k = 0..n."""
    robot, env, q = sc.scene_cfg0()
    o = op.Oracle(robot, env)
    qa, qb, ns = sc.random_edges(robot, 48, np.random.default_rng(9))
    fh, _ = o.check_edges(qa, qb, ns, nthreads=NT)
    for e in range(48):
        n = int(ns[e])
        ks = np.arange(n + 1)
        qs = (qa[e].astype(np.float64)[None, :] + (ks / n)[:, None] * (qb[e].astype(np.float64) - qa[e])[None, :])
        feas = o.is_feasible(qs.astype(np.float32))
        # the oracle interpolates in FP64 from the float endpoints; re-deriving
        # the configurations in float32 can only flip borderline steps
        bad = np.flatnonzero(feas == 0)
        expect = int(bad[0]) if bad.size else -1
        assert fh[e] == expect or abs(fh[e] - expect) <= 1


def test_masks_exclude_terrain_for_base_links():
    """PlannerSettings.cpp:34-41: links with parent -1 are not tested against
    terrains (group 1)."""
    robot = sc.arm(2, rings=4, segments=12)
    terrain = sc.box_mesh((0, 0, 0.05), (1.0, 1.0, 0.02))  # cuts through link 0 only
    env = sc.env_from_objects("t", [terrain], groups=[1], convex=[1])
    o = op.Oracle(robot, env)
    q = np.zeros((1, 2), np.float32)
    eh, _, _ = o.check_configs(q)
    assert eh[0] == 0
    env2 = sc.env_from_objects("o", [terrain], groups=[0], convex=[1])
    eh, _, _ = op.Oracle(robot, env2).check_configs(q)
    assert eh[0] == 1


def test_oracle_raycast_box_known_answers():
    """Ray casting on a unit box: face, edge and corner hits, a ray from
    inside, a scaled direction, a miss, a zero direction."""
    from oracle.oracle_py import Oracle, raycast
    box = sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5))
    env = sc.env_from_objects("box", [box])
    o = Oracle(sc.arm(2), env)
    s = np.array([[2, 0, 0], [2, 0.5, 0.5], [0, 0, 0], [2, 2, 2], [2, 0, 0], [2, 0, 0]], np.float32)
    d = np.array([[-1, 0, 0], [-1, 0, 0], [1, 0, 0], [1, 0, 0], [-2, 0, 0], [0, 0, 0]], np.float32)
    obj, tri, t, pt = raycast(o, s, d)
    assert obj.tolist() == [0, 0, 0, -1, 0, -1]
    assert t[0] == 1.5 and t[1] == 1.5 and t[2] == 0.5 and t[4] == 0.75
    assert np.isinf(t[3]) and np.isinf(t[5])
    assert np.array_equal(pt[0], [0.5, 0, 0]) and np.array_equal(pt[1], [0.5, 0.5, 0.5])


def test_oracle_jacobian_matches_finite_differences():
    """Oracle Jacobians (angular and linear rows) against central differences
    of the oracle's own FK on a tree robot with revolute, prismatic and weld
    joints."""
    from oracle.oracle_py import Oracle, jacobian
    robot = sc.humanoid()
    robot.joint_types = robot.joint_types.copy()
    robot.joint_types[3] = 1  # one prismatic joint
    box = sc.box_mesh((5, 5, 5), (0.1, 0.1, 0.1))
    o = Oracle(robot, sc.env_from_objects("far", [box]))
    rng = np.random.default_rng(3)
    L = robot.num_links
    q = rng.uniform(-1, 1, (4, L)).astype(np.float32)
    links = rng.integers(0, L, 4).astype(np.int32)
    pl = rng.uniform(-0.1, 0.1, (4, 3)).astype(np.float32)
    J = jacobian(o, q, links, pl)
    h = 1e-6
    for b in range(4):
        for j in range(L):
            qp = q[b].astype(np.float64).copy(); qm = qp.copy()
            qp[j] += h; qm[j] -= h
            Tp, Tm = o.fk(qp), o.fk(qm)
            li = links[b]
            pp = Tp[li, :9].reshape(3, 3) @ pl[b] + Tp[li, 9:]
            pm = Tm[li, :9].reshape(3, 3) @ pl[b] + Tm[li, 9:]
            assert np.allclose((pp - pm) / (2 * h), J[b, 3:, j], atol=1e-6)
            # angular velocity from dR R^T
            dR = (Tp[li, :9] - Tm[li, :9]).reshape(3, 3) / (2 * h)
            Om = dR @ o.fk(q[b].astype(np.float64))[li, :9].reshape(3, 3).T
            assert np.allclose([Om[2, 1], Om[0, 2], Om[1, 0]], J[b, :3, j], atol=1e-6)


def test_oracle_ik_reaches_reachable_targets():
    """The FP64 IK restatement: targets made by FK of random configurations
    are reached from perturbed starts (position, and position + rotation)."""
    from oracle.oracle_py import Oracle, ik_solve
    robot = sc.arm(7, rings=4, segments=8)
    o = Oracle(robot, sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))]))
    rng = np.random.default_rng(11)
    B = 64
    qt = rng.uniform(-2.5, 2.5, (B, 7))
    pl = np.tile([0.0, 0.0, 0.3], (B, 1))
    T = np.stack([o.fk(x)[6] for x in qt])
    pt = np.einsum("bij,bj->bi", T[:, :9].reshape(B, 3, 3), pl) + T[:, 9:]
    q0 = np.clip(qt + rng.normal(0, 0.3, qt.shape), -math.pi, math.pi)
    q, ok, res, its = ik_solve(o, q0, np.full(B, 6), pl, pt, tol=1e-6)
    assert ok.mean() > 0.9 and (res[ok == 1] <= 1e-6).all()
    for b in np.nonzero(ok)[0][:8]:
        Tb = o.fk(q[b])[6]
        assert np.abs(Tb[:9].reshape(3, 3) @ pl[b] + Tb[9:] - pt[b]).max() <= 1e-6
    q, ok, res, its = ik_solve(o, q0, np.full(B, 6), pl, pt, Rtarget=T[:, :9], tol=1e-6)
    assert ok.mean() > 0.8


def test_self_distance_brute_force():
    """Self distance of a small arm against all triangle pairs of its enabled
    self pairs (FP64 placements, canonical triangle distance): value, pair,
    contact as 0, cutoff, and the gradient against central differences."""
    from oracle.oracle_py import Oracle, self_distance, tri_tri
    robot = sc.arm(4, rings=2, segments=6)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    o = Oracle(robot, env)
    rng = np.random.default_rng(41)
    q = sc.uniform_configs(robot, 24, rng)
    d, pair, cp, g = self_distance(o, q, cutoff=10.0)
    L = robot.num_links
    mask = robot.packed()["self_mask"].astype(bool).reshape(L, L)
    for b in range(len(q)):
        T = o.fk(q[b].astype(np.float64))
        world = []
        for l, (V, F) in enumerate(robot.meshes):
            R, t = T[l, :9].reshape(3, 3), T[l, 9:]
            world.append((V.astype(np.float64) @ R.T + t)[np.asarray(F)])
        best, bp = np.inf, (-1, -1)
        for i in range(L):
            for j in range(i + 1, L):
                if not mask[i, j]:
                    continue
                m = min(tri_tri(world[i][a], world[j][c])[1] for a in range(len(world[i])) for c in range(len(world[j])))
                if np.sqrt(m) < best - 1e-12:
                    best, bp = np.sqrt(m), (i, j)
        assert abs(d[b] - best) <= 1e-9 * max(1.0, best), (b, d[b], best)
        if best > 1e-6:
            assert tuple(pair[b]) == bp, (b, pair[b], bp)
    # cutoff: nothing below it gives (cutoff, -1, -1)
    d2, p2, _, _ = self_distance(o, q[:4], cutoff=1e-9)
    assert np.all((d2 == 1e-9) == (p2[:, 0] < 0))
    # gradient against central differences (FP64 evaluation, steps where the
    # closest pair stays the same)
    h = 1e-5
    checked = 0
    for b in range(len(q)):
        if not (d[b] > 1e-3):
            continue
        for k in range(L):
            qp, qm = q[b].astype(np.float64).copy(), q[b].astype(np.float64).copy()
            qp[k] += h
            qm[k] -= h
            dp, pp, _, _ = self_distance(o, qp.astype(np.float32)[None], cutoff=10.0)
            dm, pm, _, _ = self_distance(o, qm.astype(np.float32)[None], cutoff=10.0)
            if tuple(pp[0]) != tuple(pair[b]) or tuple(pm[0]) != tuple(pair[b]):
                continue
            fd = (dp[0] - dm[0]) / (np.float32(qp[k]) - np.float32(qm[k]))
            assert abs(fd - g[b, k]) <= 2e-3 * max(1.0, abs(g[b, k])), (b, k, fd, g[b, k])
            checked += 1
    assert checked > 10


def test_self_pair_distances_consistent():
    """Per-pair self distances: the minimum over the enabled pairs is the self
    distance (the earliest pair on equal distances), each entry matches the
    brute force over the pair's triangles, disabled pairs read -1."""
    from oracle.oracle_py import Oracle, self_distance, self_pair_distances, tri_tri
    robot = sc.arm(4, rings=2, segments=6)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    o = Oracle(robot, env)
    q = sc.uniform_configs(robot, 12, np.random.default_rng(43))
    dp = self_pair_distances(o, q, cutoff=10.0)
    d, pair, _, _ = self_distance(o, q, cutoff=10.0)
    L = robot.num_links
    iu, ju = np.triu_indices(L, 1)
    mask = robot.packed()["self_mask"].astype(bool).reshape(L, L)[iu, ju]
    assert (dp[:, ~mask] == -1).all() and (dp[:, mask] >= 0).all()
    for b in range(len(q)):
        k = int(np.argmin(np.where(mask, dp[b], np.inf)))
        assert dp[b, k] == d[b] and (iu[k], ju[k]) == tuple(pair[b])
        T = o.fk(q[b].astype(np.float64))
        world = []
        for l, (V, F) in enumerate(robot.meshes):
            R, t = T[l, :9].reshape(3, 3), T[l, 9:]
            world.append((V.astype(np.float64) @ R.T + t)[np.asarray(F)])
        for k in np.flatnonzero(mask):
            i, j = iu[k], ju[k]
            m = min(tri_tri(a, c)[1] for a in world[i] for c in world[j])
            assert abs(dp[b, k] - np.sqrt(m)) <= 1e-12


def test_self_distance_pair_ties_keep_earlier_pair():
    """The 7-link arm's (3, 5) and (4, 6) pairs are mirror images: their
    distances are often the same double while the squared distances differ in
    the last bit.  The pair loop keeps the earlier pair unless a later one is
    strictly closer, so the result is (3, 5) whenever the two distances are
    equal."""
    from oracle.oracle_py import Oracle, self_distance, self_pair_distances
    robot = sc.arm(7, rings=8, segments=16)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    o = Oracle(robot, env)
    rng = np.random.default_rng(51)
    q = (sc.uniform_configs(robot, 256, rng) * rng.uniform(0, 1, (256, 1))).astype(np.float32)
    q = q[:32]
    d, pair, _, _ = self_distance(o, q, cutoff=1e3, nthreads=os.cpu_count() or 4)
    dp = self_pair_distances(o, q, cutoff=1e3, nthreads=os.cpu_count() or 4)
    L = robot.num_links
    k35 = 3 * L - 3 * 4 // 2 + (5 - 3 - 1)
    k46 = 4 * L - 4 * 5 // 2 + (6 - 4 - 1)
    tied = np.flatnonzero((dp[:, k35] == dp[:, k46]) & (dp[:, k35] == d) & (d > 0))
    assert len(tied) >= 2
    assert (pair[tied] == [3, 5]).all()

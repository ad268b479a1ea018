"""The Klamp't-facing layer (RobotModel / WorldCollider / RobotCSpace), the
autograd wrappers and the heterogeneous multi-robot batch, against the FP64
oracle, through the C ABI."""

import math
import os

import numpy as np
import pytest

from klampt_gb300 import scenes as sc

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 4


@pytest.fixture(scope="module")
def world0():
    from klampt_gb300 import build
    build.build()
    from klampt_gb300.klampt import WorldModel
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg0()
    W = WorldModel([robot], env)
    yield W, robot, env, q, Oracle(robot, env)
    W.close()


def test_robotmodel_set_config_and_transforms(world0):
    W, robot, env, q, o = world0
    r = W.robot(0)
    with pytest.raises(RuntimeError):
        r.setConfig([0.0, 1.0])
    r.setConfig(q[3].astype(np.float64))
    T64 = o.fk(q[3].astype(np.float64))
    for i in range(r.numLinks()):
        R, t = r.link(i).getTransform()
        Rr = np.asarray(R).reshape(3, 3).T  # column-major -> row-major
        assert np.allclose(Rr, T64[i, :9].reshape(3, 3), atol=1e-5)
        assert np.allclose(t, T64[i, 9:], atol=1e-5)
    eh, sh, _ = o.check_configs(q[3:4])
    assert r.selfCollides() == bool(sh[0])


def test_link_jacobian_methods(world0):
    from oracle.oracle_py import jacobian
    W, robot, env, q, o = world0
    r = W.robot(0)
    r.setConfig(q[7].astype(np.float64))
    pl = [0.01, -0.02, 0.15]
    J = r.link(4).getJacobian(pl)
    Jo = jacobian(o, q[7:8], [4], [pl])[0]
    assert J.shape == (6, r.numLinks()) and np.abs(J - Jo).max() < 2e-5
    assert np.array_equal(r.link(4).getPositionJacobian(pl), J[3:])
    Jb = r.getJacobians(q[:32], 4, np.tile(pl, (32, 1)))
    assert np.abs(Jb - jacobian(o, q[:32], np.full(32, 4), np.tile(pl, (32, 1)))).max() < 2e-5


def test_iksolver_facade(world0):
    from klampt_gb300.klampt import IKObjective, IKSolver
    W, robot, env, q, o = world0
    r = W.robot(0)
    target_q = np.clip(q[11].astype(np.float64), -2.5, 2.5)
    r.setConfig(target_q)
    goal = r.link(5).getWorldPosition([0, 0, 0.3])
    r.setConfig(np.clip(target_q + 0.2, -math.pi, math.pi))
    obj = IKObjective()
    obj.setFixedPoint(5, [0, 0, 0.3], goal)
    s = IKSolver(r)
    s.add(obj)
    s.setTolerance(1e-4)
    assert s.solve() and s.getResidualMax() <= 1e-4
    assert np.abs(np.asarray(r.link(5).getWorldPosition([0, 0, 0.3])) - goal).max() < 2e-4


def test_collider_and_cspace(world0):
    from klampt_gb300.klampt import RobotCSpace, WorldCollider
    W, robot, env, q, o = world0
    col = WorldCollider(W)
    eh, sh = col.check_configs(q[:512])
    eo, so, _ = o.check_configs(q[:512], nthreads=NT)
    assert np.array_equal(eh, eo.astype(bool)) and np.array_equal(sh, so.astype(bool))
    space = RobotCSpace(W.robot(0), col)
    f = space.isFeasibleBatch(q[:512])
    assert np.array_equal(f, o.is_feasible(q[:512], nthreads=NT).astype(bool))
    assert space.feasible(q[0]) == bool(f[0])
    space.setVisibilityEpsilon(1e-2)
    qa, qb, _ = sc.random_edges(robot, 64, np.random.default_rng(12))
    vis, fh = space.isVisibleBatch(qa, qb)
    n = space.steps(qa, qb)
    fh_o, _ = o.check_edges(qa, qb, n, nthreads=NT)
    assert np.array_equal(fh, fh_o) and np.array_equal(vis, fh_o < 0)
    assert space.isVisible(qa[0], qb[0]) == bool(vis[0])


def test_collider_distance_result(world0):
    from klampt_gb300.klampt import DistanceQuerySettings, WorldCollider
    W, robot, env, q, o = world0
    col = WorldCollider(W)
    W.robot(0).setConfig(q[5].astype(np.float64))
    res = col.distance(settings=DistanceQuerySettings(upperBound=2.0))
    d_o, p_o, cp_o, _ = o.min_distance(q[5:6], 2.0)
    assert abs(res.d - d_o[0]) <= 1e-9 * max(1.0, abs(d_o[0]))
    assert (res.elem1, res.elem2) == tuple(p_o[0])
    if res.hasGradients:
        assert abs(np.linalg.norm(res.grad1) - 1.0) < 1e-6


def test_world_and_collider_raycast(world0):
    from klampt_gb300.klampt import WorldCollider
    from oracle.oracle_py import raycast
    W, robot, env, q, o = world0
    col = WorldCollider(W)
    rng = np.random.default_rng(21)
    S = rng.uniform(-1.5, 1.5, (2048, 3)).astype(np.float32)
    D = rng.normal(size=(2048, 3)).astype(np.float32)
    obj, tri, t, pt = col.rayCastBatch(S, D)
    ro, rt, rtt, rp = raycast(o, S, D, nthreads=NT)
    assert np.array_equal(obj, ro) and np.array_equal(tri, rt) and np.array_equal(t, rtt) and np.array_equal(pt, rp)
    k = int(np.argmax(obj >= 0))
    assert col.rayCast(S[k], D[k]) == (int(ro[k]), rp[k].tolist())
    miss = int(np.argmax(obj < 0))
    assert col.rayCast(S[miss], D[miss]) is None
    assert W.rayCast(S[miss], D[miss])[0] == -1


def test_autograd_wrappers():
    import torch
    from klampt_gb300.autodiff import MinDistance, SoftMinDistance
    from klampt_gb300.engine import World
    robot, env, q = sc.scene_cfg2(T=8, W=4)
    w = World(env, [robot])
    qt = torch.as_tensor(q).cuda().requires_grad_(True)
    L = SoftMinDistance.apply(qt, w, 0.01)
    (2.0 * L).sum().backward()
    L2, G = w.softmin(q, 0.01)
    assert torch.allclose(L.detach(), L2)
    assert torch.allclose(qt.grad, 2.0 * G)
    qc = torch.as_tensor(q.reshape(-1, 7)[:16]).cuda().requires_grad_(True)
    d = MinDistance.apply(qc, w, 1.0)
    d.sum().backward()
    _, _, _, g = w.distance(q.reshape(-1, 7)[:16], 1.0)
    assert torch.allclose(qc.grad, g)
    w.close()


def test_autotuner_keeps_results(world0):
    from klampt_gb300 import autotune
    W, robot, env, q, o = world0
    w = W.engine
    before = w.check_configs(q[:512])
    best, table = autotune.tune_configs(w, q[:512], reps=1)
    assert len(table) == 36 and set(best) == {"blocks_per_sm", "grab", "job_flush", "fp64_inline"}
    assert all(w.get_option(k) == v for k, v in best.items())
    after = w.check_configs(q[:512])
    assert all(np.array_equal(x.cpu().numpy(), y.cpu().numpy()) for x, y in zip(before, after))


def test_edge_autotuner_graph_mode_keeps_results(world0):
    """Edge tuning with every setting timed as its CUDA-graph plan leaves the
    fastest setting in the world, destroys its plans, and changes no result."""
    from klampt_gb300 import autotune
    W, robot, env, q, o = world0
    w = W.engine
    qa, qb, ns = sc.random_edges(robot, 256, np.random.default_rng(77))
    before = w.check_edges(qa, qb, ns).cpu().numpy()
    best, table = autotune.tune_edges(w, qa, qb, ns, reps=1, graph=True, finalists=2, final_reps=2)
    assert len(table) == 54 and set(best) == {"blocks_per_sm", "grab", "job_flush", "fp64_inline", "edge_chunk"}
    assert all(w.get_option(k) == v for k, v in best.items())
    assert np.array_equal(w.check_edges(qa, qb, ns).cpu().numpy(), before)


def test_heterogeneous_batch_matches_oracle():
    """Four robots (6-DOF, 7-DOF, 12-DOF dual arm, 30-DOF humanoid) in one
    launch, every configuration checked against its own robot's oracle."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robots, env, (ids, q) = sc.scene_cfg3(total=1023, n_spheres=70, n_boxes=870)
    w = World(env, robots)
    ref = []
    for r, spec in enumerate(robots):
        sel = np.flatnonzero(ids == r)
        eo, so, _ = Oracle(spec, env).check_configs(q[sel, :spec.num_links], nthreads=NT)
        ref.append((sel, eo, so))
    # configurations sorted by robot into per-robot groups (FP64 deferred)
    # and one configuration per item (FP64 inline)
    for fp64_inline in (0, 1):
        w.set_option("fp64_inline", fp64_inline)
        eh, sh = w.check_configs_multi(ids, q)
        eh, sh = eh.cpu().numpy(), sh.cpu().numpy()
        for r, (sel, eo, so) in enumerate(ref):
            assert np.array_equal(eh[sel], eo), (fp64_inline, r)
            assert np.array_equal(sh[sel], so), (fp64_inline, r)
        assert 0 < eh.mean() < 1 and 0 < sh.mean() < 1
    w.close()


def test_jacobian_matches_oracle():
    """Batched full Jacobians (FP32) against the FP64 oracle on a 7-DOF arm
    and a 31-link tree with weld and prismatic joints."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle, jacobian
    box = sc.box_mesh((5, 5, 5), (0.1, 0.1, 0.1))
    env = sc.env_from_objects("far", [box])
    hum = sc.humanoid()
    hum.joint_types = hum.joint_types.copy()
    hum.joint_types[3] = 1
    rng = np.random.default_rng(9)
    for robot in (sc.arm(7, rings=8, segments=8), hum):
        w = World(env, [robot])
        o = Oracle(robot, env)
        L = robot.num_links
        B = 2048
        q = rng.uniform(-math.pi, math.pi, (B, L)).astype(np.float32)
        links = rng.integers(0, L, B).astype(np.int32)
        pl = rng.uniform(-0.2, 0.2, (B, 3)).astype(np.float32)
        J = w.jacobian(q, links, pl).cpu().numpy()
        Jo = jacobian(o, q, links, pl)
        scale = max(1.0, float(np.abs(Jo).max()))
        assert np.abs(J - Jo).max() <= 2e-5 * scale
        # one link for every configuration
        J1 = w.jacobian(q[:16], L - 1, pl[:16]).cpu().numpy()
        assert np.abs(J1 - jacobian(o, q[:16], np.full(16, L - 1), pl[:16])).max() <= 2e-5 * scale
        w.close()


def test_self_collision_pair_sampling():
    """Pairs colliding over a batch of samples: the engine's OR-accumulated
    pair mask equals the FP64 oracle's, for a 7-DOF arm and the humanoid."""
    from klampt_gb300.engine import World
    from klampt_gb300.klampt import RandomizedSelfCollisionPairs, WorldModel
    from oracle.oracle_py import Oracle, self_pairs
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    rng = np.random.default_rng(17)
    for robot in (sc.arm(7, rings=8, segments=8), sc.humanoid()):
        w = World(env, [robot])
        o = Oracle(robot, env)
        q = sc.uniform_configs(robot, 3000, rng)
        m = w.self_collision_pairs(q).cpu().numpy().astype(np.uint32)
        mo = self_pairs(o, q, nthreads=NT)
        assert np.array_equal(m, mo) and mo.any()
        # accumulation: two halves OR to the whole
        acc = w.self_collision_pairs(q[:1500])
        acc = w.self_collision_pairs(q[1500:], mask=acc).cpu().numpy().astype(np.uint32)
        assert np.array_equal(acc, mo)
        w.close()
    W = WorldModel([sc.arm(7, rings=8, segments=8)], env)
    col = RandomizedSelfCollisionPairs(W.robot(0), 500, seed=3)
    assert col.shape == (7, 7) and not col[0, 1] and col.any()
    W.close()


def test_independent_self_collision_pairs():
    """Candidate pairs that collide alone in a sample: engine against the FP64
    oracle (humanoid: many candidate pairs, most samples with several
    collisions), plus the Klamp't-facing two-pass function."""
    from klampt_gb300.engine import World
    from klampt_gb300.klampt import (RandomizedIndependentSelfCollisionPairs, RandomizedSelfCollisionPairs,
                                     WorldModel)
    from oracle.oracle_py import Oracle, indep_pairs, self_pairs
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    rng = np.random.default_rng(19)
    for robot in (sc.arm(7, rings=8, segments=8), sc.humanoid()):
        w = World(env, [robot])
        o = Oracle(robot, env)
        cand = self_pairs(o, sc.uniform_configs(robot, 2000, rng), nthreads=NT)
        q = sc.uniform_configs(robot, 3000, rng)
        m = w.independent_self_collision_pairs(q, cand).cpu().numpy().astype(np.uint32)
        mo = indep_pairs(o, q, cand, nthreads=NT)
        assert np.array_equal(m, mo) and mo.any()
        assert not (mo & ~cand).any()  # independent pairs are candidates
        w.close()
    W = WorldModel([sc.humanoid()], env)
    col = RandomizedSelfCollisionPairs(W.robot(0), 400, seed=5)
    ind = RandomizedIndependentSelfCollisionPairs(W.robot(0), 400, seed=5)
    # the two-pass function draws its candidate samples as the one-pass call does
    assert ind.any() and not (ind & ~col).any()
    W.close()


def test_batched_ik_matches_oracle_iteration():
    """Batched IK (FP32, one warp per problem) against the FP64 restatement of
    the same iteration: same convergence verdicts on almost every problem,
    every GPU solution verified in FP64, nearby solutions."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle, ik_solve
    robot = sc.arm(7, rings=4, segments=8)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    w = World(env, [robot])
    o = Oracle(robot, env)
    rng = np.random.default_rng(23)
    B = 2048
    qt = rng.uniform(-2.5, 2.5, (B, 7))
    pl = np.tile(np.array([0.0, 0.0, 0.3], np.float32), (B, 1))
    T = np.stack([o.fk(x)[6] for x in qt])
    pt = (np.einsum("bij,bj->bi", T[:, :9].reshape(B, 3, 3), pl) + T[:, 9:]).astype(np.float32)
    q0 = np.clip(qt + rng.normal(0, 0.3, qt.shape), -math.pi, math.pi).astype(np.float32)
    for Rt in (None, T[:, :9].astype(np.float32)):
        q, ok, res, its = (x.cpu().numpy() for x in w.ik_solve(q0, 6, pl, pt, Rtarget=Rt, tol=1e-4))
        qo, oko, reso, _ = ik_solve(o, q0, np.full(B, 6), pl, pt, Rtarget=Rt, tol=1e-4)
        assert ok.mean() > 0.85 and (ok == oko).mean() > 0.97
        good = np.nonzero(ok)[0]
        for b in good[:: max(1, len(good) // 64)]:
            Tb = o.fk(q[b].astype(np.float64))[6]
            assert np.abs(Tb[:9].reshape(3, 3) @ pl[b] + Tb[9:] - pt[b]).max() <= 1e-4 + 2e-5
        both = np.nonzero((ok == 1) & (oko == 1))[0]
        assert np.median(np.abs(q[both] - qo[both]).max(axis=1)) < 1e-2
    w.close()


def test_config_plans_replay_and_autotune():
    """Configuration batches replayed as CUDA graphs: one robot, and the
    four-robot heterogeneous batch autotuned first; every replay equals the
    eager call and the oracle."""
    import torch
    from klampt_gb300 import autotune
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robots, env, (ids, q) = sc.scene_cfg3(total=2048, n_spheres=70, n_boxes=870)
    w = World(env, robots)
    best, table = autotune.tune_configs_multi(w, ids, q, reps=1)
    assert set(best) == {"blocks_per_sm", "grab", "job_flush", "fp64_inline"} and len(table) == 36
    ids_d, q_d = torch.as_tensor(ids).cuda(), torch.as_tensor(q).cuda()
    eh = torch.empty(len(ids), dtype=torch.uint8, device="cuda")
    sh = torch.empty(len(ids), dtype=torch.uint8, device="cuda")
    plan = w.config_plan(q_d, eh, sh, robot_ids=ids_d)
    e_ref, s_ref = (x.cpu().numpy() for x in w.check_configs_multi(ids, q))
    for _ in range(3):
        eh.fill_(7)
        plan.launch()
        w.sync()
        assert np.array_equal(eh.cpu().numpy(), e_ref) and np.array_equal(sh.cpu().numpy(), s_ref)
    for r, spec in enumerate(robots):
        sel = np.flatnonzero(ids == r)
        eo, so, _ = Oracle(spec, env).check_configs(q[sel, :spec.num_links], nthreads=NT)
        assert np.array_equal(e_ref[sel], eo) and np.array_equal(s_ref[sel], so)
    plan.close()
    # one robot
    q1 = torch.as_tensor(q[ids == 1, :robots[1].num_links]).contiguous().cuda()
    e1 = torch.empty(q1.shape[0], dtype=torch.uint8, device="cuda")
    s1 = torch.empty(q1.shape[0], dtype=torch.uint8, device="cuda")
    p1 = w.config_plan(q1, e1, s1, robot=1)
    p1.launch()
    w.sync()
    ea, sa = w.check_configs(q1, robot=1)
    assert torch.equal(e1, ea) and torch.equal(s1, sa)
    p1.close()
    w.close()

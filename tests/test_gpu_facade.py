"""The Klamp't-named collider, C-space and planner surfaces on the GPU,
against the FP64 oracle: WorldCollider pair iterators (collide.py:379-698),
ignoreCollision / isCollisionEnabled, RobotCSpace selfCollision /
envCollision / feasibilityFailures (robotcspace.py:98-118), make_space
(robotplanning.py:23-90) and a batched lazy PRM whose milestone and edge
checks are one GPU call per round."""

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
    env.groups = env.groups.copy()
    env.groups[0] = 2          # object 0 alone in its group: it can be ignored on its own
    W = WorldModel([robot], env)
    yield W, robot, env, q, Oracle(robot, env)
    W.close()


def test_pair_iterators_match_oracle(world0):
    from klampt_gb300.klampt import RigidObjectModel, WorldCollider
    from oracle.oracle_py import GeomPairOracle, self_pairs
    W, robot, env, q, o = world0
    col = WorldCollider(W)
    r = W.robot(0)
    L = robot.num_links
    I12 = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)
    eo, so, _ = o.check_configs(q[:48], nthreads=NT)
    for b in range(48):
        r.setConfig(q[b].astype(np.float64))
        # self pairs
        got = {(a.index, c.index) for a, c in col.robotSelfCollisions(0)}
        words = self_pairs(o, q[b:b + 1])
        want = {(j, i) for i in range(L) for j in range(L) if (int(words[i]) >> j) & 1}
        assert got == want, (b, got, want)
        assert bool(got) == bool(so[b]) and r.selfCollides() == bool(so[b])
        # link-object pairs, each decided against the oracle's FP64 transforms
        pairs = list(col.robotObjectCollisions(0)) + list(col.robotTerrainCollisions(0))
        T = o.fk(q[b].astype(np.float64))
        got = {(l.index, ob.object) for l, ob in pairs}
        want = set()
        for l in range(L):
            for ob in range(env.num_objects):
                if GeomPairOracle(robot.meshes[l], env.meshes[ob]).collide(T[l], I12)[0]:
                    want.add((l, ob))
        assert got == want, (b, got ^ want)
        assert bool(got) == bool(eo[b]) == col.robotEnvCollides(0)
    # environment pairs (static): every overlapping pair of boxes
    objs = [col.world.rigidObject(i) for i in range(W.numRigidObjects())]
    got = set()
    for ob in objs:
        for a, c in col.objectObjectCollisions(ob):
            got.add(frozenset((a.object, c.object)))
    want = set()
    for i in range(env.num_objects):
        for j in range(i + 1, env.num_objects):
            if GeomPairOracle(env.meshes[i], env.meshes[j]).collide(I12, I12)[0]:
                want.add(frozenset((i, j)))
    assert got == want and want
    # collisions() = self pairs + link-object pairs + object pairs at the current configuration
    allp = list(col.collisions())
    assert {frozenset((a.object, c.object)) for a, c in allp
            if isinstance(a, RigidObjectModel) and isinstance(c, RigidObjectModel)} == want


def test_ignore_collision_and_masks(world0):
    from klampt_gb300.klampt import WorldCollider
    from oracle.oracle_py import Oracle, default_masks
    W, robot, env, q, o = world0
    col = WorldCollider(W)
    r = W.robot(0)
    link3, link5 = r.link(3), r.link(5)
    obj0 = W.rigidObject(0)     # group 2, alone
    obj1 = W.rigidObject(1)     # group 0, shared
    assert col.isCollisionEnabled((link3, link5)) and col.isCollisionEnabled((link3, obj0))
    assert not col.isCollisionEnabled((r.link(2), r.link(3)))   # adjacent links
    col.ignoreCollision((link3, link5))
    col.ignoreCollision((link5, obj0))
    assert not col.isCollisionEnabled((link3, link5)) and not col.isCollisionEnabled((link5, obj0))
    with pytest.raises(ValueError):
        col.ignoreCollision((link3, obj1))    # shares group 0 with 18 other boxes
    # the batched verdicts honour the same masks as the oracle with them
    mask = robot.default_self_mask().copy()
    mask[3, 5] = 0
    spec = sc.RobotSpec(**{**robot.__dict__, "self_mask": mask})
    masks = default_masks(robot, env).copy()
    masks[5] &= np.uint32(~(1 << 2) & 0xFFFFFFFF)
    o2 = Oracle(spec, env, masks=masks)
    eh, sh = col.check_configs(q[:1024])
    eo, so, _ = o2.check_configs(q[:1024], nthreads=NT)
    assert np.array_equal(eh, eo.astype(bool)) and np.array_equal(sh, so.astype(bool))
    col.ignoreCollision(link3)
    assert not col.isCollisionEnabled(link3)
    eh, sh = col.check_configs(q[:256])
    r.enableSelfCollision(3, 5, True)   # restore the world for the other tests
    for j in range(r.numLinks()):
        if abs(j - 3) > 1:
            r.enableSelfCollision(3, j, True)
    col.setLinkEnvMask(0, 3, 0xFFFFFFFF)
    col.setLinkEnvMask(0, 5, 0xFFFFFFFF)


def test_cspace_queries_and_failures(world0):
    from klampt_gb300.klampt import RobotCSpace, WorldCollider
    W, robot, env, q, o = world0
    col = WorldCollider(W)
    space = RobotCSpace(W.robot(0), col)
    eo, so, _ = o.check_configs(q[:64], nthreads=NT)
    for b in range(64):
        x = q[b].astype(np.float64).tolist()
        assert space.selfCollision(x) == bool(so[b])
        assert space.envCollision(x) == bool(eo[b])
        f = space.feasibilityFailures(x)
        assert ("self collision" in f) == bool(so[b]) and ("env collision" in f) == bool(eo[b])
    # without a collider only limits and self collision count (robotcspace.py:68-70)
    bare = RobotCSpace(W.robot(0))
    _, so512, _ = o.check_configs(q[:512], nthreads=NT, want_env=False)
    assert np.array_equal(bare.isFeasibleBatch(q[:512]), ~so512.astype(bool))
    # an extra host constraint applies after the GPU tests
    space.addConstraint(lambda x: x[0] > 0.0, "q0 positive")
    f = space.isFeasibleBatch(q[:512])
    ref = o.is_feasible(q[:512], nthreads=NT).astype(bool) & (q[:512, 0] > 0)
    assert np.array_equal(f, ref)


def test_make_space_and_batched_lazy_prm(world0):
    from klampt_gb300.klampt import make_space
    from klampt_gb300.plan import BatchedLazyPRM
    W, robot, env, q, o = world0
    space = make_space(W, W.robot(0), edgeCheckResolution=0.02)
    feas = o.is_feasible(q, nthreads=NT).astype(bool)
    free = q[feas].astype(np.float64)
    start = free[0]
    d = np.linalg.norm(free - start, axis=1)
    goal = free[np.flatnonzero(d > 0.8)[np.argmin(d[d > 0.8])]]  # a nearby free configuration
    planner = BatchedLazyPRM(space, k=12, seed=3)
    path = planner.plan(start, goal, n_milestones=1500, max_rounds=200)
    assert path is not None
    P = np.asarray(path, np.float32)
    assert np.array_equal(P[0], start.astype(np.float32)) and np.array_equal(P[-1], goal.astype(np.float32))
    assert o.is_feasible(P, nthreads=NT).all()
    n = space.steps(P[:-1], P[1:])
    fh, _ = o.check_edges(P[:-1], P[1:], n, nthreads=NT)
    assert (fh < 0).all()
    # every milestone verdict the planner saw equals the oracle's
    Q = planner.milestones.astype(np.float32)
    assert o.is_feasible(Q, nthreads=NT).all()
    st = planner.stats
    assert st["feasibility_batches"] == 2 and st["visibility_batches"] >= 1
    assert st["edges_checked"] >= len(path) - 1

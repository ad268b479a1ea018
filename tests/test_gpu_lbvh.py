"""Environments whose trees are built on the GPU (linear BVH): every query
through them gives the oracle's results bit for bit (collision verdicts,
edge first hits, closest pairs, ray hits), on the icosphere field, boxes, a
terrain in its own group, and edge cases of the build (a one-triangle
object, an object of identical triangles, whose keys all tie, flat objects,
sparse group numbers)."""

import os

import numpy as np
import pytest

from klampt_gb300 import scenes as sc

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 4


@pytest.fixture(scope="module")
def built():
    from klampt_gb300 import build
    build.build()
    from oracle import oracle_py
    oracle_py.build()
    return True


def _world(env, robots):
    from klampt_gb300.engine import World
    return World(env, robots, gpu_build=True)


def _rays_match(w, o, s, d):
    from oracle.oracle_py import raycast
    obj, tri, t, pt = (x.cpu().numpy() for x in w.raycast(s, d))
    ro, rt, rtt, rp = raycast(o, s, d, nthreads=NT)
    assert np.array_equal(obj, ro), np.nonzero(obj != ro)[0][:10]
    assert np.array_equal(tri, rt) and np.array_equal(t, rtt) and np.array_equal(pt, rp)
    return obj


def _configs_match(w, o, q):
    eh_o, sh_o, _ = o.check_configs(q, nthreads=NT)
    eh, sh = (x.cpu().numpy() for x in w.check_configs(q))
    assert np.array_equal(eh, eh_o), np.flatnonzero(eh != eh_o)[:10]
    assert np.array_equal(sh, sh_o)
    return eh


def test_lbvh_boxes_configs(built):
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg0()
    w = _world(env, [robot])
    o = Oracle(robot, env)
    eh = _configs_match(w, o, q)
    assert 0.1 < eh.mean() < 0.9
    w.close()


def test_lbvh_sphere_field_edges_and_rays(built):
    from oracle.oracle_py import Oracle
    robot, env, (qa, qb, ns) = sc.scene_cfg1(n_edges=2048)
    w = _world(env, [robot])
    o = Oracle(robot, env)
    fh_o, _ = o.check_edges(qa, qb, ns, nthreads=NT)
    fh = w.check_edges(qa, qb, ns).cpu().numpy()
    assert np.array_equal(fh, fh_o), np.flatnonzero(fh != fh_o)[:10]
    assert (fh_o < 0).any() and (fh_o > 0).any()
    _configs_match(w, o, sc.uniform_configs(robot, 2048, np.random.default_rng(7)))
    s, d = sc.camera_rays(sc.CAMERA_EYES[1], sc.SPHERE_FIELD_CENTER, 96, 64)
    obj = _rays_match(w, o, s, d)
    assert 0.2 < (obj >= 0).mean() < 1.0
    w.close()


def test_lbvh_sphere_field_distance(built):
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg2(T=16, W=8)
    w = _world(env, [robot])
    o = Oracle(robot, env)
    qq = q.reshape(-1, robot.num_links)[:64]
    d_o, p_o, cp_o, _ = o.min_distance(qq, 1e3, nthreads=NT)
    d, p, cp, _ = (x.cpu().numpy() for x in w.distance(qq, 1e3))
    assert np.array_equal(p, p_o)
    assert (np.abs(d - d_o) <= 1e-6 * np.maximum(np.abs(d_o), 1e-12)).all()
    nz = d_o != 0
    assert np.allclose(cp[nz], cp_o[nz], rtol=0, atol=1e-9)
    w.close()


def test_lbvh_terrain_groups(built):
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg4(n_configs=256, nx=128, ny=256, spacing=0.016)
    w = _world(env, [robot])
    o = Oracle(robot, env)
    _configs_match(w, o, q)
    d_o, p_o, _, _ = o.min_distance(q[:32], 0.2, nthreads=NT)
    d, p, _, _ = (x.cpu().numpy() for x in w.distance(q[:32], 0.2))
    assert np.array_equal(p, p_o)
    assert np.allclose(d, d_o, rtol=1e-6, atol=1e-12)
    rng = np.random.default_rng(3)
    n = 4096
    s = np.stack([rng.uniform(-1, 1, n), rng.uniform(-2, 2, n), np.full(n, 1.5)], 1).astype(np.float32)
    dd = np.stack([rng.normal(0, 0.2, n), rng.normal(0, 0.2, n), -np.ones(n)], 1).astype(np.float32)
    _rays_match(w, o, s, dd)
    w.close()


def test_lbvh_build_edge_cases(built):
    """One-triangle objects, an object of 64 copies of one triangle (all keys
    equal), flat quads (zero-extent centroid axes), a five-triangle object,
    objects in groups 0, 5 and 31."""
    from oracle.oracle_py import Oracle
    tri1 = (np.array([[0.3, 0.0, 0.2], [0.6, 0.1, 0.2], [0.4, 0.4, 0.5]]), np.array([[0, 1, 2]]))
    tri2 = (np.array([[-0.4, 0.2, 0.5], [-0.2, 0.2, 0.5], [-0.3, 0.5, 0.5]]), np.array([[0, 1, 2]]))
    dup = (np.array([[0.0, -0.4, 0.3], [0.3, -0.4, 0.3], [0.1, -0.2, 0.6]]), np.tile([[0, 1, 2]], (64, 1)))
    quad = (np.array([[-1, -1, -0.6], [1, -1, -0.6], [1, 1, -0.6], [-1, 1, -0.6]]), np.array([[0, 1, 2], [0, 2, 3]]))
    wall = (np.array([[0.9, -1, 0], [0.9, 1, 0], [0.9, 1, 1.0], [0.9, -1, 1.0]]), np.array([[0, 1, 2], [0, 2, 3]]))
    fan_v = np.array([[-0.5, -0.5, 0.8]] + [[-0.5 + 0.2 * np.cos(a), -0.5 + 0.2 * np.sin(a), 0.8]
                                            for a in np.linspace(0, 2 * np.pi, 6, endpoint=False)])
    fan = (fan_v, np.array([[0, k, k % 5 + 1] for k in range(1, 6)]))
    boxes = sc.random_boxes(6, np.random.default_rng(11), half_lo=0.05, half_hi=0.15)
    meshes = [tri1, tri2, dup, quad, wall, fan] + boxes
    groups = [0, 5, 5, 31, 31, 0] + [0, 5, 0, 5, 0, 31]
    convex = [0, 0, 0, 0, 0, 0] + [1] * 6
    env = sc.env_from_objects("edge_cases", meshes, groups, convex)
    robot = sc.arm(6, rings=16)
    w = _world(env, [robot])
    o = Oracle(robot, env)
    q = sc.uniform_configs(robot, 2048, np.random.default_rng(12))
    eh = _configs_match(w, o, q)
    assert 0.05 < eh.mean() < 0.95
    d_o, p_o, _, _ = o.min_distance(q[:64], 1e3, nthreads=NT)
    d, p, _, _ = (x.cpu().numpy() for x in w.distance(q[:64], 1e3))
    assert np.array_equal(p, p_o)
    assert (np.abs(d - d_o) <= 1e-6 * np.maximum(np.abs(d_o), 1e-12)).all()
    rng = np.random.default_rng(13)
    s = rng.uniform(-1.2, 1.2, (8192, 3)).astype(np.float32)
    dd = rng.normal(size=(8192, 3)).astype(np.float32)
    obj = _rays_match(w, o, s, dd)
    assert len(set(obj.tolist())) > 6
    w.close()


def test_lbvh_matches_host_built_world(built):
    """The GPU-built and host-built worlds agree on a larger batch, where the
    oracle would be slow; both are parity-tested above."""
    from klampt_gb300.engine import World
    robot, env, (qa, qb, ns) = sc.scene_cfg1(n_edges=8192)
    wg = _world(env, [robot])
    wh = World(env, [robot])
    assert np.array_equal(wg.check_edges(qa, qb, ns).cpu().numpy(), wh.check_edges(qa, qb, ns).cpu().numpy())
    q = sc.uniform_configs(robot, 32768, np.random.default_rng(21))
    for a, b in zip(wg.check_configs(q), wh.check_configs(q)):
        assert np.array_equal(a.cpu().numpy(), b.cpu().numpy())
    wg.close()
    wh.close()

"""GPU parity of batched ray casting against the FP64 oracle: hit object,
triangle, parameter t and hit point bit for bit, on the icosphere field, a
terrain with boxes, and known answers on a box (edges, corners, in-plane
rays, rays from inside, zero direction)."""

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


def _compare(w, o, s, d):
    from oracle.oracle_py import raycast
    obj, tri, t, pt = w.raycast(s, d)
    ro, rt, rtt, rp = raycast(o, s, d, nthreads=NT)
    obj, tri, t, pt = (x.cpu().numpy() for x in (obj, tri, t, pt))
    assert np.array_equal(obj, ro), np.nonzero(obj != ro)[0][:10]
    assert np.array_equal(tri, rt)
    assert np.array_equal(t, rtt)
    assert np.array_equal(pt, rp)
    return obj


def test_ray_sphere_field(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, _ = sc.scene_cfg1(n_edges=2)
    w = World(env, [robot])
    o = Oracle(robot, env)
    s, d = sc.camera_rays(sc.CAMERA_EYES[0], sc.SPHERE_FIELD_CENTER, 128, 96)
    obj = _compare(w, o, s, d)
    assert 0.2 < (obj >= 0).mean() < 1.0
    rng = np.random.default_rng(5)
    s2 = (np.asarray(sc.SPHERE_FIELD_CENTER) + rng.uniform(-1.2, 1.2, (8192, 3))).astype(np.float32)
    d2 = rng.normal(size=(8192, 3)).astype(np.float32) * rng.uniform(0.1, 3.0, (8192, 1)).astype(np.float32)
    _compare(w, o, s2, d2)
    w.close()


def test_ray_terrain_and_boxes(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, _ = sc.scene_cfg4(n_configs=4, nx=128, ny=256)
    w = World(env, [robot])
    o = Oracle(robot, env)
    rng = np.random.default_rng(7)
    n = 8192
    s = np.stack([rng.uniform(-0.25, 0.25, n), rng.uniform(-0.5, 0.5, n), np.full(n, 1.5)], 1).astype(np.float32)
    d = np.stack([rng.normal(0, 0.05, n), rng.normal(0, 0.05, n), -np.ones(n)], 1).astype(np.float32)
    obj = _compare(w, o, s, d)
    assert (obj >= 0).mean() > 0.5
    w.close()


def test_ray_box_known_answers(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    box = sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5))
    env = sc.env_from_objects("box", [box])
    robot = sc.arm(2)
    w = World(env, [robot])
    o = Oracle(robot, env)
    s = np.array([[2, 0, 0], [2, 0.5, 0.5], [0, 0, 0], [2, 2, 2], [2, 0, 0], [2, 0.5, 0], [0.5, 2, 0],
                  [0.5, 0, 0], [2, 0, 0]], np.float32)
    d = np.array([[-1, 0, 0], [-1, 0, 0], [1, 0, 0], [1, 0, 0], [-2, 0, 0], [-1, 0, 0], [0, -1, 0],
                  [1, 0, 0], [0, 0, 0]], np.float32)
    obj, tri, t, pt = (x.cpu().numpy() for x in w.raycast(s, d))
    _compare(w, o, s, d)
    assert obj.tolist() == [0, 0, 0, -1, 0, 0, 0, 0, -1]
    assert t[0] == 1.5 and t[1] == 1.5 and t[2] == 0.5 and t[4] == 0.75 and t[7] == 0.0
    assert np.array_equal(pt[0], [0.5, 0, 0])
    assert np.isinf(t[3]) and np.isinf(t[8])
    w.close()


def test_ray_nonfinite_rejected(built):
    from klampt_gb300.engine import World
    from klampt_gb300._kgpu import KgpuError
    box = sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5))
    w = World(sc.env_from_objects("box", [box]), [sc.arm(2)])
    s = np.array([[np.nan, 0, 0]], np.float32)
    d = np.array([[1, 0, 0]], np.float32)
    with pytest.raises(KgpuError):
        w.raycast(s, d)
    # the context stays usable
    obj, _, t, _ = w.raycast(np.array([[2, 0, 0]], np.float32), np.array([[-1, 0, 0]], np.float32))
    assert int(obj.cpu()[0]) == 0 and float(t.cpu()[0]) == 1.5
    w.close()

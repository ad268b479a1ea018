"""GPU parity of the free-geometry pair queries (kgpu_geom_collide /
kgpu_geom_distance, the batched Geometry3D collides / withinDistance /
distance_ext) against the FP64 oracle, through the C ABI: verdicts bit-exact,
distances, closest points and closest triangles bit-exact (both sides
finalise in the canonical FP64 arithmetic)."""

import os
import zlib

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


def _random_transforms(rng, n, spread):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                  2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                  2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], 1)
    t = rng.uniform(-spread, spread, (n, 3))
    return np.ascontiguousarray(np.concatenate([R, t], 1))


PAIRS = {
    "cylinder_cylinder": (lambda: sc.cylinder_mesh(0.05, 0.3, 32, 16), lambda: sc.cylinder_mesh(0.05, 0.3, 32, 16),
                          0.25),
    "cylinder_icosphere": (lambda: sc.cylinder_mesh(0.05, 0.3, 32, 32), lambda: sc.icosphere_mesh((0, 0, 0), 0.1, 3),
                           0.22),
    "box_terrain": (lambda: sc.box_mesh((0, 0, 0), (0.1, 0.05, 0.2)),
                    lambda: sc.heightfield_mesh(64, 64, 0.02, np.random.default_rng(5).uniform(0, 0.05, (64, 64)),
                                                (-0.63, -0.63, 0.0)), 0.5),
}


@pytest.mark.parametrize("name", sorted(PAIRS))
def test_geom_pairs_match_oracle(built, name):
    from klampt_gb300.engine import Geometry
    from oracle.oracle_py import GeomPairOracle
    ma, mb, spread = PAIRS[name]
    A, B = ma(), mb()
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    n = 4096
    Ta = _random_transforms(rng, n, spread)
    Tb = _random_transforms(rng, n, spread)
    if name == "box_terrain":
        Tb[:] = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)
        Ta[:, 11] = rng.uniform(-0.15, 0.3, n)
    ga, gb = Geometry(*A), Geometry(*B)
    o = GeomPairOracle(A, B)
    for tol in (0.0, 0.01):
        hit = ga.collide(gb, Ta, Tb, tol=tol).cpu().numpy()
        ho = o.collide(Ta, Tb, tol=tol, nthreads=NT)
        assert np.array_equal(hit, ho), (tol, np.flatnonzero(hit != ho)[:8])
        assert 0.05 < ho.mean() < 0.95
    for ub in (np.inf, 0.05):
        d, cp, elem, dr = (x.cpu().numpy() for x in ga.distance(gb, Ta, Tb, upper_bound=ub))
        do, cpo, eo, dro = o.distance(Ta, Tb, upper_bound=ub, nthreads=NT)
        assert np.array_equal(elem, eo), (ub, np.flatnonzero((elem != eo).any(1))[:8])
        assert np.array_equal(d, do), (ub, np.abs(d - do).max())
        assert np.array_equal(cp, cpo) and np.allclose(dr, dro, rtol=0, atol=1e-15)
        assert (do == 0).any() and (do > 0).any()
    # margins fatten both geometries
    ga.set_margin(0.01)
    gb.set_margin(0.02)
    om = GeomPairOracle(A, B, margin_a=0.01, margin_b=0.02)
    assert np.array_equal(ga.collide(gb, Ta, Tb).cpu().numpy(), om.collide(Ta, Tb, nthreads=NT))
    d, _, elem, _ = (x.cpu().numpy() for x in ga.distance(gb, Ta, Tb))
    do, _, eo, _ = om.distance(Ta, Tb, nthreads=NT)
    assert np.array_equal(elem, eo) and np.array_equal(d, do)
    ga.close()
    gb.close()


def test_geom_fixed_transform_and_errors(built):
    import torch
    from klampt_gb300.engine import Geometry
    from klampt_gb300._kgpu import KgpuError
    from oracle.oracle_py import GeomPairOracle
    A, B = sc.cylinder_mesh(0.05, 0.3, 16, 8), sc.box_mesh((0, 0, 0.1), (0.1, 0.1, 0.1))
    ga, gb = Geometry(*A), Geometry(*B)
    rng = np.random.default_rng(7)
    Ta = _random_transforms(rng, 512, 0.3)
    Tb = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0.05, 0, 0], np.float64)
    o = GeomPairOracle(A, B)
    assert np.array_equal(ga.collide(gb, Ta, Tb).cpu().numpy(), o.collide(Ta, Tb[None]))
    d, _, e, _ = (x.cpu().numpy() for x in ga.distance(gb, Tb, Ta))
    do, _, eo, _ = GeomPairOracle(A, B).distance(Tb[None], Ta)
    assert np.array_equal(e, eo) and np.array_equal(d, do)
    # a non-finite transform is reported on sync; the geometry stays usable
    bad = Ta.copy()
    bad[3, 4] = np.nan
    with pytest.raises(KgpuError):
        ga.collide(gb, bad, Tb)
    assert np.array_equal(ga.collide(gb, Ta, Tb).cpu().numpy(), o.collide(Ta, Tb[None]))
    # empty geometries: no collision; distance is an error (robotsim.cpp:1786-1787)
    ge = Geometry(np.zeros((0, 3)), np.zeros((0, 3), np.int32))
    assert not ge.collide(gb, Ta, Tb).cpu().numpy().any()
    with pytest.raises(KgpuError):
        ge.distance(gb, Ta, Tb)
    for g in (ga, gb, ge):
        g.close()
    torch.cuda.synchronize()


def test_geometry3d_facade(built):
    """Klamp't-named Geometry3D: se3 column-major transforms, margins,
    DistanceQueryResult fields, batched overloads."""
    from klampt_gb300.klampt import DistanceQuerySettings, Geometry3D, TriangleMesh
    from oracle.oracle_py import GeomPairOracle
    A, B = sc.cylinder_mesh(0.05, 0.3, 16, 8), sc.icosphere_mesh((0, 0, 0), 0.1, 2)
    g1, g2 = Geometry3D(TriangleMesh(*A)), Geometry3D(TriangleMesh(*B))
    o = GeomPairOracle(A, B)
    c, s = np.cos(0.3), np.sin(0.3)
    Rrow = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    g1.setCurrentTransform(Rrow.T.reshape(-1).tolist(), [0.0, 0.0, 0.0])  # so3: column-major
    for x in (0.12, 0.16, 0.4):
        g2.setCurrentTransform([1, 0, 0, 0, 1, 0, 0, 0, 1], [x, 0.0, 0.1])
        Ta = np.concatenate([Rrow.reshape(-1), [0, 0, 0]])
        Tb = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, x, 0.0, 0.1])
        assert g1.collides(g2) == bool(o.collide(Ta, Tb)[0])
        assert g1.withinDistance(g2, 0.05) == bool(o.collide(Ta, Tb, tol=0.05)[0])
        r = g1.distance(g2)
        do, cpo, eo, dro = o.distance(Ta, Tb)
        assert r.d == do[0] and (r.elem1, r.elem2) == tuple(eo[0])
        assert r.hasClosestPoints and np.array_equal(r.cp1, cpo[0, :3])
        if do[0] > 0:
            assert r.hasGradients and np.allclose(r.grad1, dro[0]) and np.allclose(r.grad2, -dro[0])
        ru = g1.distance_ext(g2, DistanceQuerySettings(upperBound=0.01))
        assert ru.d == (0.01 if do[0] >= 0.01 else do[0])
    g1.setCollisionMargin(0.3)  # the sphere at x = 0.4 is ~0.25 from the cylinder
    assert g1.getCollisionMargin() == 0.3 and g1.collides(g2)
    Ts = np.tile(np.concatenate([Rrow.T.reshape(-1), [0, 0, 0]]), (3, 1))
    Tb3 = np.array([[1, 0, 0, 0, 1, 0, 0, 0, 1, x, 0, 0.1] for x in (0.12, 0.4, 0.7)], np.float64)
    assert g1.collides_batch(g2, Ts, Tb3).tolist() == [True, True, False]
    assert Geometry3D().collides(g2) is False
    with pytest.raises(RuntimeError):
        Geometry3D().distance(g2)

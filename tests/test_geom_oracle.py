"""The FP64 oracle of the free-geometry pair queries (Geometry3D collides /
withinDistance / distance_ext) on known answers: unit cubes at known
offsets (touching counts as contact, as PQP's TriContact does), margins and
tolerances as distance thresholds, upper bounds, fixed transforms."""

import numpy as np

from klampt_gb300 import scenes as sc
from oracle.oracle_py import GeomPairOracle

I12 = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)


def _at(x, y=0.0, z=0.0):
    T = I12.copy()
    T[9:] = (x, y, z)
    return T


def test_cube_pair_known_answers():
    cube = sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5))
    o = GeomPairOracle(cube, cube)
    offs = np.array([0.5, 0.999, 1.0, 1.001, 1.5, 3.0])
    Tb = np.stack([_at(x) for x in offs])
    hit = o.collide(I12[None], Tb)
    assert hit.tolist() == [1, 1, 1, 0, 0, 0]
    d, cp, elem, dr = o.distance(I12[None], Tb)
    assert np.allclose(d, np.maximum(offs - 1.0, 0.0), atol=1e-12)
    sep = d > 0
    assert np.allclose(dr[sep], [[-1, 0, 0]] * int(sep.sum()))    # grad1 points from b to a
    assert np.allclose(cp[sep, 0], 0.5) and np.allclose(cp[sep, 3], offs[sep] - 0.5)
    assert (elem >= 0).all()
    # tolerance and margins: within (m_a + tol) + m_b
    assert o.collide(I12[None], Tb, tol=0.5).tolist() == [1, 1, 1, 1, 1, 0]
    om = GeomPairOracle(cube, cube, margin_a=0.2, margin_b=0.3)
    assert om.collide(I12[None], Tb).tolist() == [1, 1, 1, 1, 1, 0]
    dm, _, _, _ = om.distance(I12[None], Tb)
    assert np.allclose(dm, np.maximum(offs - 1.0, 0.0) - 0.5, atol=1e-12)
    # upper bound: nothing closer than 0.2 beyond the margins -> (upper, -1)
    du, _, eu, _ = o.distance(I12[None], Tb, upper_bound=0.2)
    assert np.allclose(du[offs - 1.0 >= 0.2], 0.2) and (eu[offs - 1.0 >= 0.2] == -1).all()
    assert np.allclose(du[offs - 1.0 < 0.2], np.maximum(offs - 1.0, 0.0)[offs - 1.0 < 0.2])


def test_rotated_cube_corner_gap():
    """A cube turned 45 degrees about z: its edge faces the other cube's face
    at a gap of x - 0.5 - sqrt(2)/2."""
    cube = sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5))
    o = GeomPairOracle(cube, cube)
    c, s = np.cos(np.pi / 4), np.sin(np.pi / 4)
    Tb = np.array([c, -s, 0, s, c, 0, 0, 0, 1, 2.0, 0.1, 0.0])
    d, cp, _, _ = o.distance(I12, Tb)
    assert abs(d[0] - (2.0 - 0.5 - np.sqrt(0.5))) < 1e-12
    assert abs(cp[0, 3] - (2.0 - np.sqrt(0.5))) < 1e-12

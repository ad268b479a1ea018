"""Robot and mesh ingestion (.rob, URDF, OFF / OBJ / STL) on CPU: parsed
fields, FK through the oracle, round trips through the .rob writer."""

import math
import os
import struct

import numpy as np
import pytest

from klampt_gb300 import model_io as mio
from klampt_gb300 import scenes as sc


def test_mesh_formats_round_trip(tmp_path):
    V, F = sc.box_mesh((0.1, 0.2, 0.3), (0.5, 0.25, 0.125))
    mio.save_off(str(tmp_path / "b.off"), (V, F))
    V2, F2 = mio.load_off(str(tmp_path / "b.off"))
    assert np.array_equal(V, V2) and np.array_equal(F, F2)
    # OBJ with a quad and a negative index
    (tmp_path / "q.obj").write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\n# quad\nf 1/1 2/2 3/3 -1\n")
    V3, F3 = mio.load_obj(str(tmp_path / "q.obj"))
    assert V3.shape == (4, 3) and F3.tolist() == [[0, 1, 2], [0, 2, 3]]
    # binary and ASCII STL of the same triangles
    tris = V[F].astype(np.float32)
    with open(tmp_path / "b.stl", "wb") as f:
        f.write(b"\0" * 80 + struct.pack("<I", len(tris)))
        for t in tris:
            f.write(struct.pack("<3f", 0, 0, 0) + t.tobytes() + b"\0\0")
    Vb, Fb = mio.load_stl(str(tmp_path / "b.stl"))
    assert Vb.shape == (8, 3) and np.allclose(Vb[Fb], tris, atol=0)
    lines = ["solid b"] + [f"facet normal 0 0 0\nouter loop\n" + "".join(f"vertex {x} {y} {z}\n" for x, y, z in t)
                           + "endloop\nendfacet" for t in tris] + ["endsolid b"]
    (tmp_path / "a.stl").write_text("\n".join(lines))
    Va, Fa = mio.load_stl(str(tmp_path / "a.stl"))
    assert Va.shape == (8, 3) and np.allclose(Va[Fa], tris)


def test_rob_round_trip_and_items(tmp_path):
    robot = sc.arm(4, rings=4, segments=8)
    mio.save_rob(str(tmp_path / "arm.rob"), robot)
    r2 = mio.load_rob(str(tmp_path / "arm.rob"))
    assert np.array_equal(r2.parents, robot.parents) and np.array_equal(r2.joint_types, robot.joint_types)
    assert np.array_equal(r2.T0_parent, robot.T0_parent) and np.array_equal(r2.axes, robot.axes)
    assert np.array_equal(r2.qmin, robot.qmin) and np.array_equal(r2.qmax, robot.qmax)
    for (Va, Fa), (Vb, Fb) in zip(robot.meshes, r2.meshes):
        assert np.array_equal(Va, Vb) and np.array_equal(Fa, Fb)
    assert np.array_equal(r2.self_mask, robot.default_self_mask())
    # items: names, degrees, base translation, geomscale, selfcollision subset, noselfcollision, weld
    mio.save_off(str(tmp_path / "unit.off"), sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5)))
    (tmp_path / "r.rob").write_text(
        "# three links\n"
        "links base 'mid link' tip\n"
        "parents -1 0 1\n"
        "jointtype r p r\n"
        "tparent 1 0 0 0 1 0 0 0 1 0 0 0 \\\n  1 0 0 0 1 0 0 0 1 0 0 1   1 0 0 0 1 0 0 0 1 0 0 1\n"
        "axis 0 0 1 1 0 0 0 1 0\n"
        "qmindeg -90 0 -45\nqmaxdeg 90 0.5 45\n"
        "translation 1 2 3\n"
        "geometry unit.off \"\" unit.off\n"
        "geomscale 0.2\n"
        "geomtransform 2 1 0 0 0.5 0 1 0 0 0 0 1 0 0 0 0 1\n"
        "selfcollision base tip 0 1\n"
        "noselfcollision 0 1\n"
        "joint weld 1\n")
    r = mio.load_rob(str(tmp_path / "r.rob"))
    assert r.joint_types.tolist() == [0, 1, 0]
    assert np.allclose(r.qmin, [-math.pi / 2, 0, -math.pi / 4]) and r.qmax[1] == 0.0  # weld pins the DOF
    assert np.array_equal(r.T0_parent[0][9:], [1, 2, 3])
    assert len(r.meshes[1][1]) == 0
    assert np.allclose(r.meshes[0][0].max(axis=0), 0.1)
    assert np.allclose(r.meshes[2][0].max(axis=0), [0.6, 0.1, 0.1])
    assert r.self_mask[0, 2] == 1 and r.self_mask.sum() == 1


def test_rob_denavit_hartenberg_fk(tmp_path):
    """A 2-link planar DH arm: link frames follow T0_Parent * Rz(q)."""
    from oracle.oracle_py import Oracle
    (tmp_path / "dh.rob").write_text("parents -1 0\nalpha 0 0\na 0 1.0\nd 0 0\ntheta 0 0\nqmin -3 -3\nqmax 3 3\n")
    r = mio.load_rob(str(tmp_path / "dh.rob"))
    r.meshes = [sc.box_mesh((0.5, 0, 0), (0.5, 0.05, 0.05))] * 2
    o = Oracle(r, sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))]))
    q = np.array([0.3, 0.4])
    T = o.fk(q)
    assert np.allclose(T[1, 9:], [math.cos(0.3), math.sin(0.3), 0.0], atol=1e-12)
    ang = math.atan2(T[1, 3], T[1, 0])
    assert abs(ang - 0.7) < 1e-12


def test_urdf_tree_limits_and_geometry(tmp_path):
    from oracle.oracle_py import Oracle
    mio.save_off(str(tmp_path / "m.off"), sc.box_mesh((0, 0, 0), (0.5, 0.5, 0.5)))
    (tmp_path / "r.urdf").write_text("""<?xml version="1.0"?>
<robot name="t">
  <link name="world"/>
  <link name="base"><collision><origin xyz="0 0 0.1"/><geometry><box size="0.2 0.2 0.2"/></geometry></collision></link>
  <link name="upper"><collision><geometry><cylinder radius="0.05" length="0.4"/></geometry></collision></link>
  <link name="hand"><collision><geometry><mesh filename="m.off" scale="0.1 0.1 0.1"/></geometry></collision>
                     <collision><origin xyz="0.1 0 0"/><geometry><sphere radius="0.03"/></geometry></collision></link>
  <link name="slider"/>
  <joint name="fix" type="fixed"><parent link="world"/><child link="base"/></joint>
  <joint name="j1" type="revolute"><parent link="base"/><child link="upper"/>
    <origin xyz="0 0 0.2" rpy="0 0 1.5707963267948966"/><axis xyz="0 1 0"/><limit lower="-1" upper="2"/></joint>
  <joint name="j2" type="continuous"><parent link="upper"/><child link="hand"/><origin xyz="0 0 0.4"/></joint>
  <joint name="j3" type="prismatic"><parent link="base"/><child link="slider"/><axis xyz="2 0 0"/>
    <limit lower="0" upper="0.3"/></joint>
  <klampt><noselfcollision pairs="base hand"/></klampt>
</robot>""")
    r = mio.load_urdf(str(tmp_path / "r.urdf"))
    assert r.num_links == 4 and r.parents.tolist() == [-1, 0, 1, 0]
    assert r.joint_types.tolist() == [0, 0, 0, 1]
    assert r.qmin[0] == r.qmax[0] == 0.0
    assert (r.qmin[1], r.qmax[1]) == (-1.0, 2.0) and math.isinf(r.qmin[2])
    assert np.allclose(r.axes[3], [1, 0, 0])
    assert len(r.meshes[2][1]) == 12 + 320 and len(r.meshes[3][1]) == 0
    assert r.self_mask[0, 2] == 0 and r.self_mask[1, 3] == 0  # noselfcollision; slider has no geometry
    o = Oracle(r, sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))]))
    T = o.fk(np.array([0.0, 0.0, 0.0, 0.2]))
    assert np.allclose(T[2, 9:], [0, 0, 0.6], atol=1e-12)
    assert np.allclose(T[3, 9:], [0.2, 0, 0], atol=1e-12)


def test_load_robot_dispatch(tmp_path):
    with pytest.raises(ValueError):
        mio.load_robot(str(tmp_path / "x.dae"))


def test_rob_item_names_are_case_insensitive(tmp_path):
    """The reference lower-cases item names (Cpp/Modeling/Robot.cpp:313); its
    moving-base generator writes TParent, qMin, qMax
    (Python/klampt/model/create/moving_base_robot.py:30-39)."""
    mio.save_off(str(tmp_path / "c.off"), sc.box_mesh((0, 0, 0), (0.05, 0.05, 0.05)))
    (tmp_path / "m.rob").write_text(
        "### a floating base in the generator's spelling\n"
        "TParent 1 0 0   0 1 0   0 0 1   0 0 0  \\\n"
        "1 0 0   0 1 0   0 0 1   0 0 0  \\\n"
        "1 0 0   0 1 0   0 0 1   0 0 0  \\\n"
        "1 0 0   0 1 0   0 0 1   0 0 0  \\\n"
        "1 0 0   0 1 0   0 0 1   0 0 0  \\\n"
        "1 0 0   0 1 0   0 0 1   0 0 0\n"
        "Parents -1 0 1 2 3 4\n"
        "axis 1 0 0   0 1 0    0 0 1     0 0 1     0 1 0     1 0 0\n"
        "JointType p p p r r r\n"
        "qMin -1 -1 -1  -inf -inf -inf\n"
        "qMax  1  1  1   inf  inf  inf\n"
        "Geometry \"\" \"\" \"\" \"\" \"\" \"c.off\"\n")
    r = mio.load_rob(str(tmp_path / "m.rob"))
    assert r.num_links == 6 and r.parents.tolist() == [-1, 0, 1, 2, 3, 4]
    assert r.joint_types.tolist() == [1, 1, 1, 0, 0, 0]
    assert r.qmin.tolist()[:3] == [-1, -1, -1] and r.qmax.tolist()[:3] == [1, 1, 1]
    assert np.isinf(r.qmin[3:]).all() and np.isinf(r.qmax[3:]).all()
    assert len(r.meshes[5][1]) == 12 and all(len(m[1]) == 0 for m in r.meshes[:5])


REF_OBJECTS = "/root/reference/tests/objects"


@pytest.mark.skipif(not os.path.isdir(REF_OBJECTS), reason="the reference's test fixtures are not mounted")
def test_reference_fixtures_known_answers():
    """The reference's own test objects: cube.off (the unit cube) and
    block.obj (a rigid object: cube.off scaled by 0.4, moved by -0.2 and
    placed at (1, 0, 0.3), tests/test_ODERigidObject.cpp:17), with known
    overlap and distance answers from the oracle's pair queries."""
    from oracle.oracle_py import GeomPairOracle
    V, F = mio.load_off(os.path.join(REF_OBJECTS, "cube.off"))
    assert V.shape == (8, 3) and F.shape == (12, 3)
    assert V.min(0).tolist() == [0, 0, 0] and V.max(0).tolist() == [1, 1, 1]
    (W, Fb), T = mio.load_rigid_object(os.path.join(REF_OBJECTS, "block.obj"))
    assert np.allclose(T[9:], [1.0, 0.0, 0.3]) and np.allclose(T[:9], np.eye(3).reshape(-1))
    assert np.allclose(W.min(0), [0.8, -0.2, 0.1]) and np.allclose(W.max(0), [1.2, 0.2, 0.5])
    I12 = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)
    o = GeomPairOracle((V, F), (W, Fb))
    offs = [-0.3, -0.2, -0.1, 0.0, 0.25]   # the unit cube moved along x
    Ta = np.stack([np.concatenate([I12[:9], [x, 0, 0]]) for x in offs])
    hit = o.collide(Ta, I12[None])
    assert hit.tolist() == [0, 1, 1, 1, 1]   # x = -0.2 touches the block's face at 0.8
    d, _, _, _ = o.distance(Ta, I12[None])
    assert np.allclose(d, [0.1, 0, 0, 0, 0], atol=1e-12)

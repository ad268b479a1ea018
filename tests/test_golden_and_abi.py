"""CPU checks: the oracle reproduces the committed golden vectors; the C-ABI
library builds, loads and exports every entry point include/kgpu.h declares;
scene generators honour the workload definitions."""

import math
import os
import re

import numpy as np
import pytest

from klampt_gb300 import scenes as sc
from oracle import oracle_py as op

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "oracle_golden.npz")
NT = os.cpu_count() or 2


def test_oracle_reproduces_goldens():
    g = np.load(GOLDEN)
    robot, env, _ = sc.scene_cfg0()
    o = op.Oracle(robot, env)
    eh, sh, _ = o.check_configs(g["cfg0_q"], nthreads=NT)
    assert np.array_equal(eh, g["cfg0_env"]) and np.array_equal(sh, g["cfg0_self"])
    robot1, env1, _ = sc.scene_cfg1(n_edges=8)
    o1 = op.Oracle(robot1, env1)
    fh, _ = o1.check_edges(g["cfg1_qa"], g["cfg1_qb"], g["cfg1_ns"], nthreads=NT)
    assert np.array_equal(fh, g["cfg1_first_hit"])
    for q, T in zip(g["fk_q"], g["fk_T"]):
        assert np.array_equal(o1.fk(q.astype(np.float64)), T)


def header_symbols():
    with open(os.path.join(ROOT, "include", "kgpu.h")) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(kgpu_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    import ctypes
    from klampt_gb300 import build, _kgpu
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = header_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding declares exactly the header's entry points
    assert sorted(_kgpu.exported_symbols()) == syms
    L = _kgpu.load(path)
    assert L.kgpu_version().decode().startswith("kgpu")


def test_invalid_arguments_are_rejected_without_gpu():
    """Host-side validation fails before any device work."""
    import ctypes
    from klampt_gb300 import build, _kgpu
    build.build()
    L = _kgpu.load()
    h = ctypes.c_void_p()
    d = _kgpu.RobotDesc(num_links=0)
    assert L.kgpu_robot_create(ctypes.byref(d), ctypes.byref(h)) == _kgpu.KGPU_ERR_INVALID
    assert "num_links" in _kgpu.last_error()
    d = _kgpu.RobotDesc(num_links=40)
    assert L.kgpu_robot_create(ctypes.byref(d), ctypes.byref(h)) == _kgpu.KGPU_ERR_INVALID
    assert L.kgpu_fk(None, 0, None, 0, None, None, None) == _kgpu.KGPU_ERR_INVALID


def test_robot_description_validation():
    """Bad parent order and non-unit axes are refused (host only)."""
    import ctypes
    from klampt_gb300 import build, _kgpu
    build.build()
    L = _kgpu.load()
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)

    def desc(spec):
        p = spec.packed()
        d = _kgpu.RobotDesc(num_links=spec.num_links, parents=ptr(p["parents"]), joint_types=ptr(p["joint_types"]),
                            T0_parent=ptr(p["T0_parent"]), axes=ptr(p["axes"]), qmin=ptr(p["qmin"]),
                            qmax=ptr(p["qmax"]), vert_offset=ptr(p["vert_offset"]), verts=ptr(p["verts"]),
                            tri_offset=ptr(p["tri_offset"]), tris=ptr(p["tris"]), margins=ptr(p["margins"]),
                            self_mask=ptr(p["self_mask"]))
        return d, p  # keep p alive with d

    h = ctypes.c_void_p()
    spec = sc.arm(3, rings=2, segments=6)
    spec.parents = np.array([-1, 2, 1], np.int32)  # parent after child
    d, keep = desc(spec)
    assert L.kgpu_robot_create(ctypes.byref(d), ctypes.byref(h)) == _kgpu.KGPU_ERR_INVALID
    spec = sc.arm(3, rings=2, segments=6)
    spec.axes[1] = [0, 2, 0]
    d, keep = desc(spec)
    assert L.kgpu_robot_create(ctypes.byref(d), ctypes.byref(h)) == _kgpu.KGPU_ERR_INVALID
    assert "unit" in _kgpu.last_error()
    spec = sc.arm(3, rings=2, segments=6)
    spec.meshes[1] = (spec.meshes[1][0], spec.meshes[1][1] + 1000)  # vertex index out of range
    d, keep = desc(spec)
    assert L.kgpu_robot_create(ctypes.byref(d), ctypes.byref(h)) == _kgpu.KGPU_ERR_INVALID


def signed_volume(V, F):
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    return np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0


def test_meshes_closed_and_outward():
    V, F = sc.cylinder_mesh(0.05, 0.3, 32, 16)
    assert len(F) == 1088
    assert abs(signed_volume(V, F) - math.pi * 0.05 ** 2 * 0.3) < 0.01 * math.pi * 0.05 ** 2 * 0.3
    assert len(sc.cylinder_mesh(0.05, 0.3, 32, 32)[1]) == 2112
    V, F = sc.box_mesh((0, 0, 0), (0.1, 0.2, 0.3))
    assert abs(signed_volume(V, F) - 0.2 * 0.4 * 0.6) < 1e-12
    V, F = sc.icosphere_mesh((1, 2, 3), 0.1, 2)
    assert len(F) == 320 and signed_volume(V, F) > 0
    # every edge shared by exactly two triangles (closed manifold)
    for V, F in (sc.cylinder_mesh(), sc.icosphere_mesh((0, 0, 0), 1, 2), sc.box_mesh((0, 0, 0), (1, 1, 1))):
        e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
        _, cnt = np.unique(e, axis=0, return_counts=True)
        assert (cnt == 2).all()


def test_workload_generators():
    robot, env, (qa, qb, ns) = sc.scene_cfg1(n_edges=2000)
    assert env.num_tris == 640000 and robot.num_links == 7
    assert ns.min() >= 2 and ns.max() <= 400
    step = np.abs(qb.astype(np.float64) - qa) / ns[:, None]
    assert np.all(step.max(axis=1) <= 0.01 + 1e-5)
    assert np.all(qa >= -math.pi) and np.all(qb <= math.pi)
    robots, env3, (ids, q3) = sc.scene_cfg3(total=1000, n_spheres=7, n_boxes=87)
    assert [r.num_links for r in robots] == [6, 7, 12, 31]
    assert np.bincount(ids).tolist() == [400, 300, 200, 100]
    h = sc.humanoid()
    assert sum(1 for t in h.joint_types if t != 2) == 30
    assert all(p < i for i, p in enumerate(h.parents))

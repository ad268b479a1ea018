"""Robot and mesh ingestion: Klamp't .rob files, URDF files and OFF / OBJ /
STL meshes into the descriptors the engine takes (scenes.RobotSpec, whose
`packed()` is kgpu_robot_desc's layout), plus a .rob writer.

Semantics follow the reference's loaders for the items that matter to this
path (kinematics, joint limits, collision geometry, self-collision pairs):

  .rob      Cpp/Modeling/Robot.cpp:216-1080 (RobotModel::Load) and the item
            list of Cpp/docs/Manual-FileTypes.md:163-238: links, parents,
            jointtype (r/p), tparent (row-major R, then t) or Denavit-
            Hartenberg parameters, axis (default z), qmin/qmax (and the
            *deg forms), q, translation/rotation of the base (applied to
            every root link, Robot.cpp:971-975), geometry (paths relative
            to the file), geomscale (one value or one per link),
            geomtransform (4x4, applied after the scale), geommargin,
            selfcollision (when present, only those pairs; otherwise every
            pair except link-parent, Robot.cpp:1277-1296), noselfcollision,
            joint weld (the DOF is pinned: qmin = qmax = its initial value).
            Dynamics, drivers, sensors and `scale` (rejected by the reference
            too, Robot.cpp:1017-1018) are not read.
  URDF      Cpp/IO/URDFConverter.cpp, Manual-FileTypes.md:240-275: every
            URDF link becomes a link whose parent is its joint's parent link;
            T0_parent = the joint origin (xyz, rpy as fixed-axis roll, pitch,
            yaw), axis = the joint axis; revolute / continuous -> r (continuous
            without limits), prismatic -> p, fixed -> a pinned DOF; collision
            geometry = every <collision> element (mesh with scale, box,
            cylinder, sphere) merged in the link frame; `package://` URIs
            resolve against <klampt package_root>; <klampt><noselfcollision>
            and <selfcollision> as for .rob.  Links are numbered depth-first
            from the root; primitives are tessellated (box 12 triangles,
            cylinder 32 segments, sphere a subdivision-2 icosphere), where
            the reference may keep them analytic.
  meshes    OFF (Klamp't's native format), OBJ (polygon faces fan-
            triangulated), STL (ASCII and binary; identical vertices merged).
"""

from __future__ import annotations

import math
import os
import shlex
import struct
import xml.etree.ElementTree as ET
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .scenes import Mesh, RobotSpec, box_mesh, cylinder_mesh, icosphere_mesh

# --------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------


def _tokens_no_comments(text: str) -> List[str]:
    out = []
    for line in text.splitlines():
        line = line.split("#", 1)[0].strip()
        if line:
            out.extend(line.split())
    return out


def load_off(path: str) -> Mesh:
    """Object File Format: 'OFF', counts (V F E), V vertices, F polygons
    ('n i0 ... in-1'), polygons fan-triangulated."""
    with open(path, "r") as f:
        tok = _tokens_no_comments(f.read())
    if not tok or not tok[0].upper().endswith("OFF"):
        raise ValueError(f"{path}: not an OFF file")
    k = 1
    nv, nf = int(tok[k]), int(tok[k + 1])
    k += 3
    V = np.array([float(x) for x in tok[k:k + 3 * nv]], np.float64).reshape(nv, 3)
    k += 3 * nv
    F = []
    for _ in range(nf):
        n = int(tok[k])
        idx = [int(x) for x in tok[k + 1:k + 1 + n]]
        k += 1 + n
        F.extend((idx[0], idx[i], idx[i + 1]) for i in range(1, n - 1))
    return V, np.asarray(F, np.int32).reshape(-1, 3)


def load_obj(path: str) -> Mesh:
    """Wavefront OBJ: 'v x y z' and 'f a b c ...' (indices 1-based or
    negative, 'v/vt/vn' forms accepted), polygons fan-triangulated."""
    V, F = [], []
    with open(path, "r") as f:
        for line in f:
            p = line.split("#", 1)[0].split()
            if not p:
                continue
            if p[0] == "v":
                V.append([float(x) for x in p[1:4]])
            elif p[0] == "f":
                idx = []
                for t in p[1:]:
                    i = int(t.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(V) + i)
                F.extend((idx[0], idx[i], idx[i + 1]) for i in range(1, len(idx) - 1))
    return np.asarray(V, np.float64).reshape(-1, 3), np.asarray(F, np.int32).reshape(-1, 3)


def _merge_vertices(tri_verts: np.ndarray) -> Mesh:
    flat = tri_verts.reshape(-1, 3)
    V, inv = np.unique(flat, axis=0, return_inverse=True)
    return V.astype(np.float64), inv.reshape(-1, 3).astype(np.int32)


def load_stl(path: str) -> Mesh:
    """STL, binary or ASCII; identical vertex coordinates are merged."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) >= 84:
        n = struct.unpack("<I", data[80:84])[0]
        if 84 + 50 * n == len(data):
            rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]),
                                count=n, offset=84)
            return _merge_vertices(rec["v"].astype(np.float64))
    text = data.decode("ascii", errors="replace")
    verts = [[float(x) for x in line.split()[1:4]] for line in text.splitlines() if line.strip().startswith("vertex")]
    if len(verts) % 3:
        raise ValueError(f"{path}: malformed ASCII STL")
    return _merge_vertices(np.asarray(verts, np.float64).reshape(-1, 3, 3))


def load_mesh(path: str) -> Mesh:
    ext = os.path.splitext(path)[1].lower()
    if ext == ".off":
        return load_off(path)
    if ext == ".obj":
        return load_obj(path)
    if ext == ".stl":
        return load_stl(path)
    raise ValueError(f"{path}: unsupported mesh format {ext!r} (OFF, OBJ, STL)")


def save_off(path: str, mesh: Mesh):
    V, F = mesh
    with open(path, "w") as f:
        f.write(f"OFF\n{len(V)} {len(F)} 0\n")
        for v in V:
            f.write(" ".join(repr(float(x)) for x in v) + "\n")
        for t in F:
            f.write(f"3 {int(t[0])} {int(t[1])} {int(t[2])}\n")


def _transform_mesh(mesh: Mesh, M: np.ndarray) -> Mesh:
    """Applies a 4x4 (or 3x4) transform to the vertices."""
    V, F = mesh
    M = np.asarray(M, np.float64)
    return V @ M[:3, :3].T + M[:3, 3], F


def _merge_meshes(meshes: Sequence[Mesh]) -> Mesh:
    Vs, Fs, off = [], [], 0
    for V, F in meshes:
        Vs.append(np.asarray(V, np.float64).reshape(-1, 3))
        Fs.append(np.asarray(F, np.int32).reshape(-1, 3) + off)
        off += len(V)
    if not Vs:
        return np.zeros((0, 3)), np.zeros((0, 3), np.int32)
    return np.concatenate(Vs), np.concatenate(Fs)


# --------------------------------------------------------------------------
# transforms
# --------------------------------------------------------------------------


def _rpy_matrix(r: float, p: float, y: float) -> np.ndarray:
    """URDF rpy: fixed-axis roll (x), pitch (y), yaw (z): R = Rz(y) Ry(p) Rx(r)."""
    cr, sr, cp, sp, cy, sy = math.cos(r), math.sin(r), math.cos(p), math.sin(p), math.cos(y), math.sin(y)
    return np.array([[cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr],
                     [sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr],
                     [-sp, cp * sr, cp * cr]], np.float64)


def _T12(R: np.ndarray, t: Sequence[float]) -> np.ndarray:
    return np.concatenate([np.asarray(R, np.float64).reshape(-1), np.asarray(t, np.float64)])


def _compose12(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    RA, tA = A[:9].reshape(3, 3), A[9:]
    RB, tB = B[:9].reshape(3, 3), B[9:]
    return _T12(RA @ RB, RA @ tB + tA)


def _dh_transform(alpha: float, a: float, d: float, theta: float) -> np.ndarray:
    """T0_Parent from Denavit-Hartenberg parameters in the modified (Craig)
    convention, T = Rx(alpha) Tx(a) Rz(theta) Tz(d): with the joint rotating
    about the link's own z axis, T * Rz(q) = Rx(alpha) Tx(a) Rz(theta + q)
    Tz(d), the convention that maps exactly onto Klamp't's
    T0_Parent * J(q) link model.  (The reference's DH helper lives in
    KrisLibrary, absent here; this convention is an assumption.)"""
    ct, st, ca, sa = math.cos(theta), math.sin(theta), math.cos(alpha), math.sin(alpha)
    Rx = np.array([[1.0, 0.0, 0.0], [0.0, ca, -sa], [0.0, sa, ca]])
    Rz = np.array([[ct, -st, 0.0], [st, ct, 0.0], [0.0, 0.0, 1.0]])
    R = Rx @ Rz
    t = np.array([a, 0.0, 0.0]) + R @ np.array([0.0, 0.0, d])
    return _T12(R, t)


# --------------------------------------------------------------------------
# self-collision pairs
# --------------------------------------------------------------------------


def _link_index(names: List[str], item: str) -> int:
    if item in names:
        return names.index(item)
    try:
        i = int(item)
    except ValueError:
        raise ValueError(f"unknown link {item!r}") from None
    if not 0 <= i < len(names):
        raise ValueError(f"link index {i} out of range")
    return i


def _self_mask(names, parents, meshes, on_pairs, off_pairs) -> np.ndarray:
    L = len(names)
    m = np.zeros((L, L), np.uint8)
    if on_pairs:
        for a, b in on_pairs:
            i, j = sorted((_link_index(names, a), _link_index(names, b)))
            if i == j:
                raise ValueError(f"invalid self-collision pair {a}, {b}")
            m[i, j] = 1
    else:
        for i in range(L):
            for j in range(i + 1, L):
                if parents[j] != i and parents[i] != j:
                    m[i, j] = 1
    for a, b in off_pairs:
        i, j = sorted((_link_index(names, a), _link_index(names, b)))
        m[i, j] = 0
    # pairs with an empty geometry never collide
    for i in range(L):
        if len(meshes[i][1]) == 0:
            m[i, :] = 0
            m[:, i] = 0
    return np.triu(m, 1)


def _pairs(tokens: Sequence[str]) -> List[Tuple[str, str]]:
    if len(tokens) % 2:
        raise ValueError("self-collision items come in pairs")
    return [(tokens[i], tokens[i + 1]) for i in range(0, len(tokens), 2)]


# --------------------------------------------------------------------------
# .rob
# --------------------------------------------------------------------------


def _rob_items(path: str) -> List[Tuple[str, List[str]]]:
    with open(path, "r") as f:
        text = f.read().replace("\\\n", " ")
    items = []
    for line in text.splitlines():
        line = line.split("#", 1)[0].strip()
        if not line:
            continue
        tok = shlex.split(line)
        # item names are case-insensitive: the reference lower-cases them
        # (Cpp/Modeling/Robot.cpp:313), and its own generators write TParent,
        # qMin, qMax (Python/klampt/model/create/moving_base_robot.py:30-39)
        items.append((tok[0].lower(), tok[1:]))
    return items


def load_rob(path: str, name: Optional[str] = None) -> RobotSpec:
    """Loads a Klamp't .rob file (kinematic and geometric items)."""
    items = _rob_items(path)
    base_dir = os.path.dirname(os.path.abspath(path))
    vals: Dict[str, List[str]] = {}
    geomtransform: List[Tuple[int, np.ndarray]] = []
    on_pairs: List[Tuple[str, str]] = []
    off_pairs: List[Tuple[str, str]] = []
    welds: List[int] = []
    for key, args in items:
        if key == "geomtransform":
            geomtransform.append((int(args[0]), np.array([float(x) for x in args[1:17]]).reshape(4, 4)))
        elif key == "selfcollision":
            on_pairs += _pairs(args)
        elif key == "noselfcollision":
            off_pairs += _pairs(args)
        elif key == "joint":
            if args and args[0] == "weld":
                welds.append(int(args[1]))
        elif key == "scale":
            if float(args[0]) != 1.0:
                raise ValueError(f"{path}: 'scale' is not supported (Robot.cpp:1017-1018)")
        elif key == "mount":
            raise ValueError(f"{path}: 'mount' is not supported by this loader")
        else:
            vals.setdefault(key, []).extend(args)

    def floats(key, scale=1.0):
        return [float(x) * scale for x in vals[key]] if key in vals else None

    names = vals.get("links")
    parents = [int(x) for x in vals["parents"]]
    L = len(parents)
    if names is None:
        names = [str(i) for i in range(L)]
    if len(names) != L:
        raise ValueError(f"{path}: {len(names)} link names for {L} parents")
    deg = math.pi / 180.0
    jt = vals.get("jointtype", ["r"] * L)
    joint_types = np.array([0 if t == "r" else 1 for t in jt], np.int32)
    qmin = floats("qmin") or ([x for x in floats("qmindeg", deg)] if "qmindeg" in vals else [-math.inf] * L)
    qmax = floats("qmax") or ([x for x in floats("qmaxdeg", deg)] if "qmaxdeg" in vals else [math.inf] * L)
    q0 = floats("q") or (floats("qdeg", deg) if "qdeg" in vals else [0.0] * L)
    axes = np.array(floats("axis") or [0.0, 0.0, 1.0] * L, np.float64).reshape(L, 3)
    if "tparent" in vals:
        T0 = np.array(floats("tparent"), np.float64).reshape(L, 12)
    else:
        alpha = floats("alpha") or floats("alphadeg", deg)
        a, d = floats("a"), floats("d")
        theta = floats("theta") or floats("thetadeg", deg)
        if None in (alpha, a, d, theta):
            raise ValueError(f"{path}: neither tparent nor Denavit-Hartenberg parameters")
        T0 = np.stack([_dh_transform(alpha[i], a[i], d[i], theta[i]) for i in range(L)])
        axes = np.tile([0.0, 0.0, 1.0], (L, 1))
    base = _T12(np.array(floats("rotation") or [1, 0, 0, 0, 1, 0, 0, 0, 1]).reshape(3, 3),
                floats("translation") or [0, 0, 0])
    for i in range(L):
        if parents[i] < 0:
            T0[i] = _compose12(base, T0[i])
    qmin, qmax = np.array(qmin, np.float64), np.array(qmax, np.float64)
    for i in welds:
        qmin[i] = qmax[i] = q0[i]
    geom = vals.get("geometry", [""] * L)
    gs = floats("geomscale") or [1.0]
    gs = gs * L if len(gs) == 1 else gs
    gm = floats("geommargin") or [0.0]
    gm = gm * L if len(gm) == 1 else gm
    meshes: List[Mesh] = []
    for i in range(L):
        if i < len(geom) and geom[i]:
            fn = geom[i] if os.path.isabs(geom[i]) else os.path.join(base_dir, geom[i])
            V, F = load_mesh(fn)
            V = V * gs[i]
        else:
            V, F = np.zeros((0, 3)), np.zeros((0, 3), np.int32)
        meshes.append((V, F))
    for i, M in geomtransform:
        if len(meshes[i][1]):
            meshes[i] = _transform_mesh(meshes[i], M)
    mask = _self_mask(names, parents, meshes, on_pairs, off_pairs)
    return RobotSpec(name=name or os.path.splitext(os.path.basename(path))[0],
                     parents=np.array(parents, np.int32), joint_types=joint_types, T0_parent=T0, axes=axes,
                     qmin=qmin, qmax=qmax, meshes=meshes, margins=np.array(gm[:L], np.float64),
                     self_mask=mask)


def save_rob(path: str, robot: RobotSpec, names: Optional[Sequence[str]] = None):
    """Writes `robot` as a .rob file with one OFF mesh per link beside it."""
    L = robot.num_links
    names = list(names) if names else [f"link{i}" for i in range(L)]
    stem = os.path.splitext(os.path.basename(path))[0]
    d = os.path.dirname(os.path.abspath(path))
    geoms = []
    for i, mesh in enumerate(robot.meshes):
        if len(mesh[1]):
            fn = f"{stem}_link{i}.off"
            save_off(os.path.join(d, fn), mesh)
            geoms.append(fn)
        else:
            geoms.append('""')

    def row(v):
        return " ".join(repr(float(x)) for x in np.asarray(v).reshape(-1))

    lines = ["links " + " ".join(shlex.quote(n) for n in names),
             "parents " + " ".join(str(int(p)) for p in robot.parents),
             "jointtype " + " ".join("r" if t == 0 else "p" for t in robot.joint_types),
             "tparent " + "  ".join(row(T) for T in robot.T0_parent),
             "axis " + "  ".join(row(a) for a in robot.axes),
             "qmin " + row(robot.qmin), "qmax " + row(robot.qmax),
             "geometry " + " ".join(geoms)]
    if robot.margins is not None:
        lines.append("geommargin " + row(robot.margins))
    mask = robot.self_mask if robot.self_mask is not None else robot.default_self_mask()
    pairs = [(i, j) for i in range(L) for j in range(i + 1, L) if mask[i, j]]
    if pairs:
        lines.append("selfcollision " + " ".join(f"{i} {j}" for i, j in pairs))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# --------------------------------------------------------------------------
# URDF
# --------------------------------------------------------------------------


def _origin(el) -> np.ndarray:
    o = el.find("origin") if el is not None else None
    xyz = [float(x) for x in (o.get("xyz", "0 0 0") if o is not None else "0 0 0").split()]
    rpy = [float(x) for x in (o.get("rpy", "0 0 0") if o is not None else "0 0 0").split()]
    return _T12(_rpy_matrix(*rpy), xyz)


def _geometry_mesh(g, base_dir: str, package_root: str) -> Mesh:
    if g.find("box") is not None:
        sx, sy, sz = (float(x) for x in g.find("box").get("size").split())
        return box_mesh((0, 0, 0), (sx / 2, sy / 2, sz / 2))
    if g.find("cylinder") is not None:
        c = g.find("cylinder")
        r, length = float(c.get("radius")), float(c.get("length"))
        V, F = cylinder_mesh(r, length, 32, 4)
        return V - np.array([0, 0, length / 2]), F  # URDF cylinders are centred
    if g.find("sphere") is not None:
        return icosphere_mesh((0, 0, 0), float(g.find("sphere").get("radius")), 2)
    m = g.find("mesh")
    if m is None:
        raise ValueError("unsupported URDF geometry")
    fn = m.get("filename")
    if fn.startswith("package://"):
        fn = os.path.join(package_root, fn[len("package://"):].split("/", 1)[-1])
    elif fn.startswith("file://"):
        fn = fn[len("file://"):]
    if not os.path.isabs(fn):
        fn = os.path.join(base_dir, fn)
    V, F = load_mesh(fn)
    s = [float(x) for x in m.get("scale", "1 1 1").split()]
    return V * np.asarray(s if len(s) == 3 else s * 3, np.float64), F


def load_urdf(path: str, name: Optional[str] = None) -> RobotSpec:
    """Loads a URDF file's kinematic tree, joint limits and collision
    geometry (plus the Klamp't self-collision elements)."""
    root = ET.parse(path).getroot()
    base_dir = os.path.dirname(os.path.abspath(path))
    kl = root.find("klampt")
    package_root = os.path.join(base_dir, kl.get("package_root", ".")) if kl is not None else base_dir
    world = kl.get("world_frame", "world") if kl is not None else "world"
    links = [l.get("name") for l in root.findall("link") if l.get("name") != world]
    joints = root.findall("joint")
    child_joint = {j.find("child").get("link"): j for j in joints}
    # order links so that parents come first (depth-first from the roots)
    kids: Dict[str, List[str]] = {}
    for j in joints:
        p = j.find("parent").get("link")
        kids.setdefault(p, []).append(j.find("child").get("link"))
    roots = [l for l in links if l not in child_joint or child_joint[l].find("parent").get("link") == world]
    order: List[str] = []
    stack = list(reversed(roots))
    while stack:
        l = stack.pop()
        order.append(l)
        stack.extend(reversed(kids.get(l, [])))
    index = {l: i for i, l in enumerate(order)}
    L = len(order)
    parents = np.full(L, -1, np.int32)
    jt = np.zeros(L, np.int32)
    T0 = np.tile(_T12(np.eye(3), [0, 0, 0]), (L, 1))
    axes = np.tile([0.0, 0.0, 1.0], (L, 1))
    qmin, qmax = np.zeros(L), np.zeros(L)
    link_el = {l.get("name"): l for l in root.findall("link")}
    meshes: List[Mesh] = []
    for i, l in enumerate(order):
        j = child_joint.get(l)
        if j is not None:
            p = j.find("parent").get("link")
            parents[i] = index[p] if p in index else -1
            T0[i] = _origin(j)
            ax = j.find("axis")
            if ax is not None:
                a = np.array([float(x) for x in ax.get("xyz").split()])
                axes[i] = a / np.linalg.norm(a)
            t = j.get("type")
            lim = j.find("limit")
            if t in ("revolute", "prismatic"):
                jt[i] = 0 if t == "revolute" else 1
                qmin[i] = float(lim.get("lower", "-inf")) if lim is not None else -math.inf
                qmax[i] = float(lim.get("upper", "inf")) if lim is not None else math.inf
            elif t == "continuous":
                qmin[i], qmax[i] = -math.inf, math.inf
            elif t == "fixed":
                pass  # pinned DOF: qmin = qmax = 0
            else:
                raise ValueError(f"{path}: unsupported joint type {t!r}")
        parts = []
        for c in link_el[l].findall("collision"):
            parts.append(_transform_mesh(_geometry_mesh(c.find("geometry"), base_dir, package_root),
                                         np.vstack([np.hstack([_origin(c)[:9].reshape(3, 3),
                                                               _origin(c)[9:, None]]), [0, 0, 0, 1]])))
        meshes.append(_merge_meshes(parts))
    on_pairs, off_pairs = [], []
    if kl is not None:
        for tag, dst in (("selfcollision", on_pairs), ("noselfcollision", off_pairs)):
            for el in kl.findall(tag):
                if el.get("pairs"):
                    dst += _pairs(el.get("pairs").split())
                if el.get("group1") and el.get("group2"):
                    dst += [(a, b) for a in el.get("group1").split() for b in el.get("group2").split()]
    mask = _self_mask(order, list(parents), meshes, on_pairs, off_pairs)
    return RobotSpec(name=name or root.get("name", os.path.splitext(os.path.basename(path))[0]),
                     parents=parents, joint_types=jt, T0_parent=T0, axes=axes, qmin=qmin, qmax=qmax,
                     meshes=meshes, margins=np.zeros(L), self_mask=mask)


def load_rigid_object(path: str) -> Tuple[Mesh, np.ndarray]:
    """Loads a Klamp't rigid-object file (Cpp/Modeling/RigidObject.cpp:
    34-125): `mesh` (a geometry file relative to the object file),
    `geomscale` (1 or 3 values) and `geomtranslate` applied to the geometry,
    and the object's transform `T` (12 values: R row-major then t, or a 4x4
    row-major matrix) or `position`.  Returns (the mesh in the world frame,
    T as 12 numbers R row-major then t); mass and contact items are not
    read."""
    base_dir = os.path.dirname(os.path.abspath(path))
    items: Dict[str, List[str]] = {}
    with open(path, "r") as f:
        for line in f.read().splitlines():
            line = line.split("#", 1)[0].strip()
            if line:
                tok = shlex.split(line)
                items[tok[0]] = tok[1:]
    if "mesh" not in items or len(items["mesh"]) != 1:
        raise ValueError(f"{path}: a rigid object needs one 'mesh' item")
    V, F = load_mesh(os.path.join(base_dir, items["mesh"][0]))
    V = np.asarray(V, np.float64)
    if "geomscale" in items:
        sc = [float(x) for x in items["geomscale"]]
        if len(sc) not in (1, 3):
            raise ValueError(f"{path}: geomscale needs 1 or 3 values")
        V = V * np.asarray(sc if len(sc) == 3 else sc * 3)
    if "geomtranslate" in items:
        V = V + np.asarray([float(x) for x in items["geomtranslate"]], np.float64)
    T = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)
    if "T" in items:
        v = [float(x) for x in items["T"]]
        if len(v) == 12:
            T = np.asarray(v, np.float64)
        elif len(v) == 16:
            M = np.asarray(v, np.float64).reshape(4, 4)
            T = np.concatenate([M[:3, :3].reshape(-1), M[:3, 3]])
        else:
            raise ValueError(f"{path}: T needs 12 or 16 values")
    if "position" in items:
        T[9:] = [float(x) for x in items["position"]]
    W = V @ T[:9].reshape(3, 3).T + T[9:]
    return (W, np.asarray(F, np.int32)), T


def load_robot(path: str) -> RobotSpec:
    """.rob or .urdf by extension."""
    ext = os.path.splitext(path)[1].lower()
    if ext == ".rob":
        return load_rob(path)
    if ext == ".urdf":
        return load_urdf(path)
    raise ValueError(f"{path}: unsupported robot format {ext!r}")

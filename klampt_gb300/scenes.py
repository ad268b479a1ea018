"""Synthetic robots, environments and query batches for the five benchmark
workloads of the configuration-validity and proximity path.

No public benchmark suite exists for this path (the reference ships no robot
or world data for it: ``tests/test_types.py:7-8`` needs the absent
Klampt-examples repository), so every workload is generated here from a
seeded ``numpy.random.default_rng`` with the shapes, sizes and value
distributions of the workload definitions:

* ``arm(ndof)``: serial revolute arm, link length 0.3 m, joint axes
  alternating z/y, each link a closed cylinder of radius 0.05 m along its
  local z in [0, 0.3]; ``rings=16`` gives 1,088 triangles per link and
  ``rings=32`` 2,112.  Joint limits [-pi, pi].  This follows the .rob model
  semantics: ``T0_Parent`` translation (0,0,0.3) for every link after the
  first (``Cpp/Modeling/Robot.cpp:961-965``), self-collision on every pair
  except link-parent (``Cpp/docs/Manual-FileTypes.md:212``).
* boxes, icospheres (subdivision s gives 20*4**s triangles), a heightfield
  terrain, and the dual-arm / humanoid robots of the heterogeneous batch.

Geometry is FP64; the engine keeps FP64 copies for its band re-test and FP32
copies for traversal.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

PI = math.pi

Mesh = Tuple[np.ndarray, np.ndarray]  # (V float64 [n,3], F int32 [m,3])


# --------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------

def cylinder_mesh(radius: float = 0.05, length: float = 0.3, segments: int = 32,
                  rings: int = 16) -> Mesh:
    """Closed cylinder along local z in [0, length]: ``segments`` around,
    ``rings`` bands of quads along the axis, fan caps.  Outward winding.
    Triangles: 2*segments*rings + 2*segments."""
    ang = 2.0 * PI * np.arange(segments) / segments
    ring_xy = np.stack([radius * np.cos(ang), radius * np.sin(ang)], axis=1)
    V = []
    for j in range(rings + 1):
        z = length * j / rings
        V.append(np.concatenate([ring_xy, np.full((segments, 1), z)], axis=1))
    V = np.concatenate(V, axis=0)
    c0 = V.shape[0]
    V = np.concatenate([V, [[0.0, 0.0, 0.0], [0.0, 0.0, length]]], axis=0)
    F = []
    for j in range(rings):
        for i in range(segments):
            i1 = (i + 1) % segments
            v00 = j * segments + i
            v10 = j * segments + i1
            v01 = (j + 1) * segments + i
            v11 = (j + 1) * segments + i1
            F.append((v00, v10, v11))
            F.append((v00, v11, v01))
    top = rings * segments
    for i in range(segments):
        i1 = (i + 1) % segments
        F.append((c0, i1, i))                # bottom cap, normal -z
        F.append((c0 + 1, top + i, top + i1))  # top cap, normal +z
    return V.astype(np.float64), np.asarray(F, dtype=np.int32)


def box_mesh(center: Sequence[float], half: Sequence[float]) -> Mesh:
    """Axis-aligned box as 8 vertices / 12 outward triangles."""
    c = np.asarray(center, dtype=np.float64)
    h = np.asarray(half, dtype=np.float64)
    s = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)
    V = c + s * h
    F = np.array([[0, 2, 1], [0, 3, 2],   # -z
                  [4, 5, 6], [4, 6, 7],   # +z
                  [0, 1, 5], [0, 5, 4],   # -y
                  [2, 3, 7], [2, 7, 6],   # +y
                  [1, 2, 6], [1, 6, 5],   # +x
                  [0, 4, 7], [0, 7, 3]],  # -x
                 dtype=np.int32)
    return V, F


_ICO_CACHE = {}


def _unit_icosphere(subdiv: int) -> Mesh:
    if subdiv in _ICO_CACHE:
        return _ICO_CACHE[subdiv]
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
         (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
         (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
         (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                mid[key] = len(V) - 1
            return mid[key]

        F2 = []
        for (a, b, c) in F:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            F2 += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = F2
    out = (np.asarray(V, dtype=np.float64), np.asarray(F, dtype=np.int32))
    # orient outward
    Vv, Ff = out
    cen = Vv[Ff].mean(axis=1)
    n = np.cross(Vv[Ff[:, 1]] - Vv[Ff[:, 0]], Vv[Ff[:, 2]] - Vv[Ff[:, 0]])
    flip = (n * cen).sum(axis=1) < 0
    Ff[flip] = Ff[flip][:, [0, 2, 1]]
    _ICO_CACHE[subdiv] = (Vv, Ff)
    return Vv, Ff


def icosphere_mesh(center: Sequence[float], radius: float, subdiv: int = 2) -> Mesh:
    V, F = _unit_icosphere(subdiv)
    return np.asarray(center, dtype=np.float64) + radius * V, F.copy()


def heightfield_mesh(nx: int, ny: int, spacing: float, heights: np.ndarray,
                     origin: Sequence[float]) -> Mesh:
    """Grid of nx*ny vertices (2*(nx-1)*(ny-1) triangles), upward normals."""
    ox, oy, oz = origin
    xs = ox + spacing * np.arange(nx)
    ys = oy + spacing * np.arange(ny)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    V = np.stack([X.ravel(), Y.ravel(), oz + heights.ravel()], axis=1)
    i = np.arange(nx - 1)[:, None]
    j = np.arange(ny - 1)[None, :]
    v00 = (i * ny + j).ravel()
    v10 = ((i + 1) * ny + j).ravel()
    v01 = (i * ny + j + 1).ravel()
    v11 = ((i + 1) * ny + j + 1).ravel()
    F = np.empty((2 * v00.size, 3), dtype=np.int32)
    F[0::2] = np.stack([v00, v10, v11], axis=1)
    F[1::2] = np.stack([v00, v11, v01], axis=1)
    return V.astype(np.float64), F


# --------------------------------------------------------------------------
# robots
# --------------------------------------------------------------------------

def _translation(x: float, y: float, z: float) -> np.ndarray:
    return np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, x, y, z], dtype=np.float64)


@dataclass
class RobotSpec:
    name: str
    parents: np.ndarray          # int32 [L]
    joint_types: np.ndarray      # int32 [L]
    T0_parent: np.ndarray        # float64 [L,12]
    axes: np.ndarray             # float64 [L,3]
    qmin: np.ndarray             # float64 [L]
    qmax: np.ndarray             # float64 [L]
    meshes: List[Mesh]           # per link, link-local
    margins: Optional[np.ndarray] = None
    self_mask: Optional[np.ndarray] = None  # uint8 [L,L]

    @property
    def num_links(self) -> int:
        return int(self.parents.shape[0])

    def default_self_mask(self) -> np.ndarray:
        """Every pair except link-parent (Cpp/docs/Manual-FileTypes.md:212)."""
        L = self.num_links
        m = np.ones((L, L), dtype=np.uint8)
        np.fill_diagonal(m, 0)
        for i in range(L):
            p = int(self.parents[i])
            if p >= 0:
                m[i, p] = m[p, i] = 0
        return np.triu(m, 1)

    def packed(self):
        """Flat arrays in the layout of kgpu_robot_desc."""
        vo, to, V, F = [0], [0], [], []
        for (v, f) in self.meshes:
            V.append(np.asarray(v, np.float64))
            F.append(np.asarray(f, np.int32))
            vo.append(vo[-1] + len(v))
            to.append(to[-1] + len(f))
        mask = self.self_mask if self.self_mask is not None else self.default_self_mask()
        margins = self.margins if self.margins is not None else np.zeros(self.num_links)
        return dict(
            parents=np.ascontiguousarray(self.parents, np.int32),
            joint_types=np.ascontiguousarray(self.joint_types, np.int32),
            T0_parent=np.ascontiguousarray(self.T0_parent, np.float64).reshape(-1),
            axes=np.ascontiguousarray(self.axes, np.float64).reshape(-1),
            qmin=np.ascontiguousarray(self.qmin, np.float64),
            qmax=np.ascontiguousarray(self.qmax, np.float64),
            vert_offset=np.asarray(vo, np.int32),
            verts=np.ascontiguousarray(np.concatenate(V) if V else np.zeros((0, 3)), np.float64).reshape(-1),
            tri_offset=np.asarray(to, np.int32),
            tris=np.ascontiguousarray(np.concatenate(F) if F else np.zeros((0, 3), np.int32), np.int32).reshape(-1),
            margins=np.ascontiguousarray(margins, np.float64),
            self_mask=np.ascontiguousarray(mask, np.uint8).reshape(-1),
        )


def arm(ndof: int, rings: int = 16, segments: int = 32, radius: float = 0.05,
        length: float = 0.3, base=(0.0, 0.0, 0.0), name: Optional[str] = None) -> RobotSpec:
    L = ndof
    T0 = np.stack([_translation(*base)] + [_translation(0, 0, length)] * (L - 1))
    axes = np.array([[0, 0, 1] if i % 2 == 0 else [0, 1, 0] for i in range(L)], dtype=np.float64)
    mesh = cylinder_mesh(radius, length, segments, rings)
    return RobotSpec(
        name=name or f"arm{ndof}",
        parents=np.arange(-1, L - 1, dtype=np.int32),
        joint_types=np.zeros(L, np.int32),
        T0_parent=T0, axes=axes,
        qmin=np.full(L, -PI), qmax=np.full(L, PI),
        meshes=[(mesh[0].copy(), mesh[1].copy()) for _ in range(L)],
    )


def dual_arm(rings: int = 16, segments: int = 16) -> RobotSpec:
    """12-DOF: two 6-DOF arms on a fixed torso (the world frame), bases at
    y = +-0.3 m; 544-triangle links by default."""
    a = arm(6, rings=rings, segments=segments, base=(0.0, 0.3, 0.0))
    b = arm(6, rings=rings, segments=segments, base=(0.0, -0.3, 0.0))
    parents = np.concatenate([a.parents, np.where(b.parents >= 0, b.parents + 6, -1)]).astype(np.int32)
    return RobotSpec(
        name="dual_arm12", parents=parents,
        joint_types=np.zeros(12, np.int32),
        T0_parent=np.concatenate([a.T0_parent, b.T0_parent]),
        axes=np.concatenate([a.axes, b.axes]),
        qmin=np.full(12, -PI), qmax=np.full(12, PI),
        meshes=a.meshes + b.meshes,
    )


def humanoid() -> RobotSpec:
    """30-DOF tree: a welded torso (link 0, one zero-range DOF as Klamp't
    models fixed links) branching into two 7-DOF arms, two 6-DOF legs and a
    4-DOF head/neck.  Link meshes span ~500 to ~5k triangles."""
    parents, T0, axes, meshes, jt = [-1], [_translation(0, 0, 0)], [[0, 0, 1]], [], [2]
    meshes.append(cylinder_mesh(0.15, 0.5, 48, 50))  # torso ~4.9k tris
    limb_mesh = {"arm": cylinder_mesh(0.04, 0.25, 24, 12),   # 624
                 "leg": cylinder_mesh(0.06, 0.35, 32, 24),   # 1600
                 "neck": cylinder_mesh(0.05, 0.12, 24, 10)}  # 528

    def chain(n, root_off, kind, first_axis, down=False):
        first = True
        for k in range(n):
            parents.append(0 if first else len(parents) - 1)
            if first:
                T = _translation(*root_off)
                if down:  # rotate the chain root by pi about x so the limb hangs down
                    T[:9] = [1, 0, 0, 0, -1, 0, 0, 0, -1]
                T0.append(T)
            else:
                T0.append(_translation(0, 0, {"arm": 0.25, "leg": 0.35, "neck": 0.12}[kind]))
            ax = [[0, 0, 1], [0, 1, 0], [1, 0, 0]][(k + first_axis) % 3]
            axes.append(ax)
            v, f = limb_mesh[kind]
            meshes.append((v.copy(), f.copy()))
            jt.append(0)
            first = False

    chain(7, (0.0, 0.2, 0.45), "arm", 1)
    chain(7, (0.0, -0.2, 0.45), "arm", 1)
    chain(6, (0.0, 0.1, 0.0), "leg", 2, down=True)
    chain(6, (0.0, -0.1, 0.0), "leg", 2, down=True)
    chain(4, (0.0, 0.0, 0.5), "neck", 0)
    L = len(parents)
    qmin = np.full(L, -PI)
    qmax = np.full(L, PI)
    qmin[0] = qmax[0] = 0.0
    T0 = np.stack(T0)
    return RobotSpec(name="humanoid30", parents=np.asarray(parents, np.int32),
                     joint_types=np.asarray(jt, np.int32), T0_parent=T0,
                     axes=np.asarray(axes, np.float64), qmin=qmin, qmax=qmax, meshes=meshes)


# --------------------------------------------------------------------------
# environments
# --------------------------------------------------------------------------

@dataclass
class EnvSpec:
    name: str
    meshes: List[Mesh]
    groups: np.ndarray            # int32 [N]
    convex: np.ndarray            # uint8 [N]
    margins: Optional[np.ndarray] = None
    info: dict = field(default_factory=dict)

    @property
    def num_objects(self) -> int:
        return len(self.meshes)

    @property
    def num_tris(self) -> int:
        return int(sum(len(f) for _, f in self.meshes))

    def packed(self):
        vo, to = [0], [0]
        for (v, f) in self.meshes:
            vo.append(vo[-1] + len(v))
            to.append(to[-1] + len(f))
        V = np.concatenate([v for v, _ in self.meshes]).astype(np.float64)
        F = np.concatenate([f for _, f in self.meshes]).astype(np.int32)
        margins = self.margins if self.margins is not None else np.zeros(self.num_objects)
        return dict(vert_offset=np.asarray(vo, np.int32), verts=np.ascontiguousarray(V).reshape(-1),
                    tri_offset=np.asarray(to, np.int32), tris=np.ascontiguousarray(F).reshape(-1),
                    groups=np.ascontiguousarray(self.groups, np.int32),
                    convex=np.ascontiguousarray(self.convex, np.uint8),
                    margins=np.ascontiguousarray(margins, np.float64))


def random_boxes(n: int, rng: np.random.Generator, lo=-1.0, hi=1.0,
                 half_lo=0.05, half_hi=0.2) -> List[Mesh]:
    c = rng.uniform(lo, hi, size=(n, 3))
    h = rng.uniform(half_lo, half_hi, size=(n, 3))
    return [box_mesh(c[i], h[i]) for i in range(n)]


def random_icospheres(n: int, rng: np.random.Generator, center, side: float,
                      r_lo=0.02, r_hi=0.1, subdiv=2) -> List[Mesh]:
    c = np.asarray(center) + rng.uniform(-side / 2, side / 2, size=(n, 3))
    r = rng.uniform(r_lo, r_hi, size=n)
    return [icosphere_mesh(c[i], r[i], subdiv) for i in range(n)]


def env_from_objects(name, meshes, groups=None, convex=None, info=None) -> EnvSpec:
    n = len(meshes)
    return EnvSpec(name=name, meshes=meshes,
                   groups=np.zeros(n, np.int32) if groups is None else np.asarray(groups, np.int32),
                   convex=np.ones(n, np.uint8) if convex is None else np.asarray(convex, np.uint8),
                   info=info or {})


# --------------------------------------------------------------------------
# query batches
# --------------------------------------------------------------------------

def uniform_configs(robot: RobotSpec, n: int, rng: np.random.Generator) -> np.ndarray:
    q = rng.uniform(robot.qmin, robot.qmax, size=(n, robot.num_links))
    return q.astype(np.float32)


def random_edges(robot: RobotSpec, n: int, rng: np.random.Generator, step: float = 0.01,
                 min_steps: int = 2, max_steps: int = 400):
    """Straight-line planner edges with log-uniform step counts: n_e =
    round(exp(U[ln min, ln max])), a direction d with max|d_i| = 1, and
    qb = qa + step*n_e*d (resampled until inside the joint limits), so the
    largest joint step between consecutive configurations is ``step``."""
    L = robot.num_links
    lo = robot.qmin.astype(np.float64)
    hi = robot.qmax.astype(np.float64)
    span = hi - lo
    nsteps = np.rint(np.exp(rng.uniform(math.log(min_steps), math.log(max_steps), size=n))).astype(np.int32)
    qa = np.empty((n, L))
    qb = np.empty((n, L))
    for e in range(n):
        for _ in range(1000):
            d = rng.normal(size=L)
            d /= np.abs(d).max()
            a = rng.uniform(lo, hi)
            b = a + step * nsteps[e] * d
            if np.all(b >= lo) and np.all(b <= hi):
                break
        qa[e], qb[e] = a, b
    # float32 inputs, and qb clipped into the limits after rounding
    qa32 = qa.astype(np.float32)
    qb32 = np.clip(qb, lo + 1e-6 * span, hi - 1e-6 * span).astype(np.float32)
    return qa32, qb32, nsteps


def noisy_trajectories(robot: RobotSpec, T: int, W: int, rng: np.random.Generator,
                       sigma: float = 0.05) -> np.ndarray:
    L = robot.num_links
    q = rng.uniform(robot.qmin, robot.qmax, size=(T, W, L)) + rng.normal(0.0, sigma, size=(T, W, L))
    q = np.clip(q, robot.qmin, robot.qmax)
    return q.astype(np.float32)


# --------------------------------------------------------------------------
# the five workloads
# --------------------------------------------------------------------------

SPHERE_FIELD_CENTER = (1.4, 0.0, 0.6)


def scene_cfg0(seed: int = 1000):
    """6-DOF arm (1,088 tris/link), 20 random boxes (240 tris), 4,096 configs."""
    rng = np.random.default_rng(seed)
    robot = arm(6, rings=16)
    env = env_from_objects("boxes20", random_boxes(20, rng))
    q = uniform_configs(robot, 4096, rng)
    return robot, env, q


def sphere_field(rng: np.random.Generator, n: int = 2000, subdiv: int = 2,
                 center=SPHERE_FIELD_CENTER, side: float = 2.0) -> EnvSpec:
    meshes = random_icospheres(n, rng, center, side, subdiv=subdiv)
    return env_from_objects(f"icospheres{n}", meshes,
                            info=dict(center=list(center), side=side, subdiv=subdiv))


def camera_rays(eye: Sequence[float], target: Sequence[float], w: int, h: int, fov: float = 1.0):
    """Pinhole-camera rays (sources [w*h, 3], unnormalised directions
    [w*h, 3], FP32) from `eye` looking at `target`, vertical field of view
    `fov` radians, z up."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, [0, 0, 1.0])
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    xs = (np.arange(w) + 0.5) / w * 2 - 1
    ys = (np.arange(h) + 0.5) / h * 2 - 1
    X, Y = np.meshgrid(xs * np.tan(fov / 2) * w / h, ys * np.tan(fov / 2), indexing="xy")
    d = f[None, None] + X[..., None] * r + Y[..., None] * u
    s = np.broadcast_to(eye, d.shape)
    return s.reshape(-1, 3).astype(np.float32), d.reshape(-1, 3).astype(np.float32)


CAMERA_EYES = ((-1.0, -1.5, 1.2), (-1.2, 1.5, 1.0), (0.2, 0.1, 2.6), (3.6, 0.3, 0.8))


def scene_cfg1(seed: int = 1001, n_edges: int = 16384):
    """7-DOF arm (2,112 tris/link), 2,000 icospheres (subdivision 2 = 320
    tris each, 640k tris), 16,384 edges of 2..400 steps at 0.01 rad."""
    rng = np.random.default_rng(seed)
    robot = arm(7, rings=32)
    env = sphere_field(rng)
    qa, qb, ns = random_edges(robot, n_edges, rng)
    return robot, env, (qa, qb, ns)


def scene_cfg2(seed: int = 1002, T: int = 8192, W: int = 32):
    rng = np.random.default_rng(seed)
    robot = arm(7, rings=32)
    env = sphere_field(np.random.default_rng(1001))
    q = noisy_trajectories(robot, T, W, rng)
    return robot, env, q


def scene_cfg3(seed: int = 1003, total: int = 65536, n_spheres: int = 700, n_boxes: int = 8700):
    rng = np.random.default_rng(seed)
    robots = [arm(6, rings=16, segments=16), arm(7, rings=32), dual_arm(), humanoid()]
    meshes = random_icospheres(n_spheres, rng, SPHERE_FIELD_CENTER, 2.0, subdiv=3)
    meshes += random_boxes(n_boxes, rng, lo=-1.0, hi=1.0, half_lo=0.01, half_hi=0.04)
    env = env_from_objects("boxes_spheres_1M", meshes)
    counts = [int(total * f) for f in (0.4, 0.3, 0.2)]
    counts.append(total - sum(counts))
    ids = np.concatenate([np.full(c, i, np.int32) for i, c in enumerate(counts)])
    rng.shuffle(ids)
    Lmax = max(r.num_links for r in robots)
    q = np.zeros((total, Lmax), np.float32)
    for i, r in enumerate(robots):
        sel = ids == i
        q[sel, :r.num_links] = uniform_configs(r, int(sel.sum()), rng)
    return robots, env, (ids, q)


def terrain_heights(nx, ny, spacing, rng, n_bumps=8):
    xs = spacing * np.arange(nx)
    ys = spacing * np.arange(ny)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    H = np.zeros_like(X)
    for _ in range(n_bumps):
        A = rng.uniform(0.1, 0.5)
        s = rng.uniform(0.1, 0.5)
        cx = rng.uniform(0, xs[-1])
        cy = rng.uniform(0, ys[-1])
        H += A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    return H


def scene_cfg4(seed: int = 1004, n_configs: int = 1048576, nx: int = 512, ny: int = 1024,
               spacing: float = 0.004):
    rng = np.random.default_rng(seed)
    robot = arm(7, rings=32)
    H = terrain_heights(nx, ny, spacing, rng)
    origin = (-spacing * (nx - 1) / 2, -spacing * (ny - 1) / 2, -1.0)
    terrain = heightfield_mesh(nx, ny, spacing, H, origin)
    boxes = random_boxes(500, rng)
    meshes = [terrain] + boxes
    groups = [1] + [0] * len(boxes)
    convex = [0] + [1] * len(boxes)
    env = env_from_objects("terrain_boxes", meshes, groups, convex)
    q = uniform_configs(robot, n_configs, rng)
    return robot, env, q

"""Klamp't-facing classes over the engine: the calls planners and trajectory
optimisers make on this path keep their names and meaning, and gain batched
overloads.

Mirrors (paths relative to the Klamp't tree):
  RobotModel.setConfig / getConfig / link(i).getTransform / selfCollides /
      enableSelfCollision          Python/klampt/src/robotsim.cpp:5311-5321,
                                   5513-5539; robotmodel.h:537-855
  DistanceQuerySettings / DistanceQueryResult
                                   Python/klampt/src/geometry.h:631-673
  WorldCollider                    Python/klampt/model/collide.py:246-630
  RobotCSpace.feasible / isFeasible / isVisible / eps
                                   Python/klampt/plan/robotcspace.py:31-118,
                                   cspace.py:81,185-200, motionplanning.cpp:789-809
  WorldModel.rayCast, WorldCollider.rayCast
                                   Cpp/Modeling/World.cpp:465-515 (environment
                                   part), Python/klampt/model/collide.py:219-243
  RobotModelLink.getJacobian / getPositionJacobian / getOrientationJacobian
                                   Python/klampt/src/robotsim.cpp:4817-4860
  IKObjective / IKSolver (one objective)
                                   Python/klampt/src/robotik.h:21-260
  RandomizedSelfCollisionPairs     Cpp/Modeling/RandomizedSelfCollisions.h:24
  RandomizedIndependentSelfCollisionPairs  Cpp/Modeling/RandomizedSelfCollisions.h:33
  Geometry3D (triangle mesh) collides / withinDistance / distance /
      distance_ext / setCollisionMargin
                                   Python/klampt/src/geometry.h:810-1110,
                                   robotsim.cpp:1656-1690, 1782-1819
Batched overloads: RobotModel.setConfigs / getJacobians, WorldCollider.check_configs /
distance_batch / rayCastBatch, RobotCSpace.isFeasibleBatch / isVisibleBatch,
Geometry3D.collides_batch / withinDistance_batch / distance_batch.

Rotations follow Klamp't's so3 convention in this layer (9 numbers,
column-major); the engine's ABI uses row-major.  Errors raise RuntimeError, as
the reference's SWIG layer does (robotsim.i:41-53).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import engine
from ._kgpu import GROUP_RIGID_OBJECT, GROUP_TERRAIN
from .model_io import load_robot


@dataclass
class DistanceQuerySettings:
    """geometry.h:631-638 (defaults robotsim.cpp:1725-1727)."""
    relErr: float = 0.0
    absErr: float = 0.0
    upperBound: float = math.inf


@dataclass
class DistanceQueryResult:
    """geometry.h:641-673.  d < 0 is penetration; cp1/cp2 are the closest
    points on self and other in world coordinates; grad1 is the gradient of
    the distance w.r.t. moving cp1 and grad2 = -grad1.  elem1 / elem2: the
    closest triangles for Geometry3D.distance; the (link, object) pair for
    WorldCollider.distance."""
    d: float = math.inf
    hasClosestPoints: bool = False
    hasGradients: bool = False
    cp1: List[float] = field(default_factory=list)
    cp2: List[float] = field(default_factory=list)
    grad1: List[float] = field(default_factory=list)
    grad2: List[float] = field(default_factory=list)
    elem1: int = -1
    elem2: int = -1


class TriangleMesh:
    """vertices [N, 3] and triangle vertex indices [M, 3] (Klamp't's
    TriangleMesh, Python/klampt/src/geometry.h)."""

    def __init__(self, vertices=None, indices=None):
        self.vertices = np.zeros((0, 3)) if vertices is None else np.asarray(vertices, np.float64).reshape(-1, 3)
        self.indices = np.zeros((0, 3), np.int32) if indices is None else np.asarray(indices, np.int32).reshape(-1, 3)


def _se3_rows(T) -> np.ndarray:
    """Klamp't se3 element(s) (R column-major 9, t 3) -> the engine's
    row-major [B, 12]."""
    T = np.asarray(T, np.float64).reshape(-1, 12)
    R = T[:, :9].reshape(-1, 3, 3).transpose(0, 2, 1).reshape(-1, 9)
    return np.ascontiguousarray(np.concatenate([R, T[:, 9:]], 1))


class Geometry3D:
    """A triangle-mesh geometry with a current transform and a collision
    margin (Python/klampt/src/geometry.h:810-1110): collides (:1020),
    withinDistance (:1031), distance / distance_ext (:1103-1108),
    setCurrentTransform / getCurrentTransform, setCollisionMargin /
    getCollisionMargin (:930-932).  Batched overloads take [B, 12] arrays of
    se3 elements (R column-major, then t) for both geometries (or one
    transform for either): collides_batch, withinDistance_batch,
    distance_batch.  Triangle-mesh pairs give unsigned distances (0 when
    they touch), as the reference's do (geometry.h:1077-1092)."""

    def __init__(self, mesh: Optional[TriangleMesh] = None):
        self._mesh = None
        self._geom = None
        self._margin = 0.0
        self._T = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)  # se3 order
        if mesh is not None:
            self.setTriangleMesh(mesh)

    def setTriangleMesh(self, mesh: TriangleMesh):
        if self._geom is not None:
            self._geom.close()
        self._mesh = mesh
        self._geom = engine.Geometry(mesh.vertices, mesh.indices, self._margin)

    def getTriangleMesh(self) -> Optional[TriangleMesh]:
        return self._mesh

    def type(self) -> str:
        return "TriangleMesh" if self._mesh is not None else ""

    def empty(self) -> bool:
        return self._mesh is None or len(self._mesh.indices) == 0

    def setCurrentTransform(self, R: Sequence[float], t: Sequence[float]):
        self._T = np.concatenate([np.asarray(R, np.float64).reshape(9), np.asarray(t, np.float64).reshape(3)])

    def getCurrentTransform(self) -> Tuple[List[float], List[float]]:
        return self._T[:9].tolist(), self._T[9:].tolist()

    def setCollisionMargin(self, margin: float):
        if not margin >= 0:
            raise RuntimeError("collision margin must be non-negative")
        self._margin = float(margin)
        if self._geom is not None:
            self._geom.set_margin(margin)

    def getCollisionMargin(self) -> float:
        return self._margin

    def close(self):
        if self._geom is not None:
            self._geom.close()
            self._geom = None

    # ---- single queries at the current transforms -------------------------
    def collides(self, other: "Geometry3D") -> bool:
        """robotsim.cpp:1656-1662 (False when either geometry is empty)."""
        return bool(self.collides_batch(other, self._T, other._T)[0])

    def withinDistance(self, other: "Geometry3D", tol: float) -> bool:
        """robotsim.cpp:1685-1690."""
        return bool(self.withinDistance_batch(other, tol, self._T, other._T)[0])

    def distance(self, other: "Geometry3D") -> DistanceQueryResult:
        return self.distance_ext(other, DistanceQuerySettings())

    def distance_ext(self, other: "Geometry3D", settings: DistanceQuerySettings) -> DistanceQueryResult:
        """robotsim.cpp:1782-1819 (the dir1 / grad2 swap there gives grad1 =
        (cp1 - cp2) / |cp1 - cp2|)."""
        d, cp, elem, dr = self.distance_batch(other, self._T, other._T, settings)
        res = DistanceQueryResult(d=float(d[0]), elem1=int(elem[0, 0]), elem2=int(elem[0, 1]))
        if elem[0, 0] >= 0:
            res.hasClosestPoints = True
            res.cp1 = cp[0, :3].tolist()
            res.cp2 = cp[0, 3:].tolist()
            if np.any(dr[0] != 0):
                res.hasGradients = True
                res.grad1 = dr[0].tolist()
                res.grad2 = (-dr[0]).tolist()
        return res

    # ---- batched overloads -------------------------------------------------
    def collides_batch(self, other: "Geometry3D", T_self, T_other) -> np.ndarray:
        return self.withinDistance_batch(other, 0.0, T_self, T_other)

    def withinDistance_batch(self, other: "Geometry3D", tol: float, T_self, T_other) -> np.ndarray:
        A, B = _se3_rows(T_self), _se3_rows(T_other)
        n = max(len(A), len(B))
        if self._geom is None or other._geom is None:
            return np.zeros(n, bool)
        return self._geom.collide(other._geom, A, B, tol).cpu().numpy().astype(bool)

    def distance_batch(self, other: "Geometry3D", T_self, T_other, settings: Optional[DistanceQuerySettings] = None):
        """(d [B], closest points [B, 6], closest triangles [B, 2],
        grad1 [B, 3]); raises RuntimeError for an empty geometry
        (robotsim.cpp:1786-1787)."""
        settings = settings or DistanceQuerySettings()
        if self._geom is None or other._geom is None:
            raise RuntimeError("Geometry3D.distance: Geometry is empty")
        d, cp, elem, dr = self._geom.distance(other._geom, _se3_rows(T_self), _se3_rows(T_other),
                                              settings.upperBound)
        return d.cpu().numpy(), cp.cpu().numpy(), elem.cpu().numpy(), dr.cpu().numpy()


class WorldModel:
    """Robots and a static environment resident on the current CUDA device.
    Robots may be given as specs or as .rob / .urdf file names
    (WorldModel::LoadRobot, Cpp/Modeling/World.cpp; model_io.load_robot)."""

    def __init__(self, robots: Sequence, env):
        robots = [load_robot(r) if isinstance(r, str) else r for r in robots]
        self.env_spec = env
        self.robot_specs = list(robots)
        self._world = engine.World(env, self.robot_specs)
        self._robots = [RobotModel(self, i) for i in range(len(self.robot_specs))]

    @property
    def engine(self) -> engine.World:
        return self._world

    def numRobots(self) -> int:
        return len(self._robots)

    def robot(self, i: int) -> "RobotModel":
        return self._robots[i]

    def numRigidObjects(self) -> int:
        return int(np.sum(self.env_spec.groups == GROUP_RIGID_OBJECT)) if self.env_spec is not None else 0

    def numTerrains(self) -> int:
        return int(np.sum(self.env_spec.groups == GROUP_TERRAIN)) if self.env_spec is not None else 0

    def _objects_of(self, terrain: bool) -> List[int]:
        if self.env_spec is None:
            return []
        g = np.asarray(self.env_spec.groups)
        sel = g == GROUP_TERRAIN if terrain else g != GROUP_TERRAIN
        return [int(i) for i in np.flatnonzero(sel)]

    def rigidObject(self, i: int) -> "RigidObjectModel":
        """The i-th environment object that is not a terrain (group != 1)."""
        objs = self._objects_of(False)
        if not (0 <= i < len(objs)):
            raise RuntimeError("Invalid rigid object index")
        return RigidObjectModel(self, i, objs[i])

    def terrain(self, i: int) -> "TerrainModel":
        """The i-th environment object of the terrain group (1)."""
        objs = self._objects_of(True)
        if not (0 <= i < len(objs)):
            raise RuntimeError("Invalid terrain index")
        return TerrainModel(self, i, objs[i])

    def _object_geometry(self, obj: int) -> "Geometry3D":
        """Geometry3D of environment object obj (world frame, identity
        transform, its collision margin), created once."""
        cache = self.__dict__.setdefault("_obj_geoms", {})
        if obj not in cache:
            V, F = self.env_spec.meshes[obj]
            g = Geometry3D(TriangleMesh(V, F))
            m = self.env_spec.margins
            if m is not None and m[obj] > 0:
                g.setCollisionMargin(float(m[obj]))
            cache[obj] = g
        return cache[obj]

    def rayCast(self, s: Sequence[float], d: Sequence[float]) -> Tuple[int, List[float]]:
        """WorldModel::RayCast over the environment: (object index, world hit
        point), or (-1, [0, 0, 0]) when nothing is hit."""
        obj, _, _, pt = self._world.raycast(np.asarray(s, np.float32)[None], np.asarray(d, np.float32)[None])
        return int(obj.cpu()[0]), pt.cpu().numpy()[0].tolist()

    def close(self):
        for g in self.__dict__.get("_obj_geoms", {}).values():
            g.close()
        for r in self._robots:
            for g in r.__dict__.get("_link_geoms", {}).values():
                g.close()
        self._world.close()


class _EnvBody:
    """An environment object seen as a world body (RigidObjectModel /
    TerrainModel): `index` counts within its kind, `object` is its index in
    the environment description."""

    def __init__(self, world: "WorldModel", index: int, obj: int):
        self.world = world
        self.index = index
        self.object = obj

    def getID(self) -> int:
        return self.object

    def getName(self) -> str:
        return f"{type(self).__name__}[{self.index}]"

    def geometry(self) -> "Geometry3D":
        return self.world._object_geometry(self.object)

    def __eq__(self, other) -> bool:
        return type(self) is type(other) and self.world is other.world and self.object == other.object

    def __hash__(self) -> int:
        return hash((type(self).__name__, id(self.world), self.object))


class RigidObjectModel(_EnvBody):
    """robotmodel.h RigidObjectModel: a static environment object here."""


class TerrainModel(_EnvBody):
    """robotmodel.h TerrainModel: an environment object of the terrain group."""


class RobotModelLink:
    def __init__(self, robot: "RobotModel", index: int):
        self.robot = robot
        self.index = index

    def getIndex(self) -> int:
        return self.index

    def getID(self) -> Tuple[int, int]:
        return (self.robot.index, self.index)

    def getName(self) -> str:
        return f"link[{self.robot.index}:{self.index}]"

    def getParent(self) -> int:
        return int(self.robot.spec.parents[self.index])

    def geometry(self) -> "Geometry3D":
        """The link's Geometry3D placed at the robot's current configuration
        (FP64 transform, Klamp't so3 order)."""
        g = self.robot._link_geometry(self.index)
        T = self.robot._current_transforms64()[self.index]
        g.setCurrentTransform(np.asarray(T[:9]).reshape(3, 3).T.reshape(-1), T[9:])
        return g

    def __eq__(self, other) -> bool:
        return isinstance(other, RobotModelLink) and self.robot is other.robot and self.index == other.index

    def __hash__(self) -> int:
        return hash(("link", id(self.robot), self.index))

    def getTransform(self) -> Tuple[List[float], List[float]]:
        """(R, t) of the link in the world frame at the robot's current
        configuration, R column-major (Klamp't so3)."""
        T = self.robot._current_transforms()[self.index]
        R = np.asarray(T[:9], np.float64).reshape(3, 3)
        return R.T.reshape(-1).tolist(), [float(x) for x in T[9:]]

    def getWorldPosition(self, plocal: Sequence[float]) -> List[float]:
        T = self.robot._current_transforms()[self.index]
        R = np.asarray(T[:9], np.float64).reshape(3, 3)
        return (R @ np.asarray(plocal, np.float64) + np.asarray(T[9:], np.float64)).tolist()

    def getJacobian(self, plocal: Sequence[float]) -> np.ndarray:
        """6 x n Jacobian of the point plocal at the current configuration,
        orientation rows first (robotsim.cpp:4817-4825)."""
        r = self.robot
        J = r.world.engine.jacobian(r._q[None], self.index, np.asarray(plocal, np.float32)[None], robot=r.index)
        return J.cpu().numpy()[0].astype(np.float64)

    def getPositionJacobian(self, plocal: Sequence[float]) -> np.ndarray:
        """3 x n position Jacobian (robotsim.cpp:4837-4845)."""
        return self.getJacobian(plocal)[3:]

    def getOrientationJacobian(self) -> np.ndarray:
        """3 x n orientation Jacobian."""
        return self.getJacobian([0.0, 0.0, 0.0])[:3]


class RobotModel:
    """robotmodel.h:537; one DOF per link."""

    def __init__(self, world: WorldModel, index: int):
        self.world = world
        self.index = index
        self.spec = world.robot_specs[index]
        self._q = np.zeros(self.spec.num_links, np.float32)
        self._T = None
        self._T64 = None
        m = self.spec.self_mask if self.spec.self_mask is not None else self.spec.default_self_mask()
        m = np.asarray(m, bool).reshape(self.spec.num_links, self.spec.num_links)
        self._self_enabled = np.triu(m, 1) | np.triu(m, 1).T

    def numLinks(self) -> int:
        return self.spec.num_links

    def link(self, i: int) -> RobotModelLink:
        if not (0 <= i < self.numLinks()):
            raise RuntimeError("Invalid link index")
        return RobotModelLink(self, i)

    def getJointLimits(self) -> Tuple[List[float], List[float]]:
        return self.spec.qmin.tolist(), self.spec.qmax.tolist()

    def getConfig(self) -> List[float]:
        return self._q.astype(np.float64).tolist()

    def setConfig(self, q: Sequence[float]):
        """robotsim.cpp:5311-5321 (size mismatch is an error)."""
        q = np.asarray(q, np.float64)
        if q.shape != (self.numLinks(),):
            raise RuntimeError("Invalid size of configuration")
        self._q = q.astype(np.float32)
        self._T = None
        self._T64 = None

    def setConfigs(self, Q) -> np.ndarray:
        """Batched FK: world transforms [B, L, 12] (R row-major, t)."""
        return self.world.engine.fk(Q, robot=self.index).cpu().numpy()

    def getJacobians(self, Q, links, plocal) -> np.ndarray:
        """Batched full Jacobians [B, 6, n] of points plocal [B, 3] on links
        [B] (or one link) at configurations Q [B, n]."""
        return self.world.engine.jacobian(Q, links, plocal, robot=self.index).cpu().numpy()

    def _current_transforms(self) -> np.ndarray:
        if self._T is None:
            self._T = self.setConfigs(self._q[None])[0]
        return self._T

    def _current_transforms64(self) -> np.ndarray:
        """[L, 12] canonical FP64 transforms (R row-major, t) at the current
        configuration: the ones the engine's FP64 decisions use."""
        if self._T64 is None:
            self._T64 = self.world.engine.fk64(self._q[None], robot=self.index).cpu().numpy()[0]
        return self._T64

    def _link_geometry(self, i: int) -> "Geometry3D":
        cache = self.__dict__.setdefault("_link_geoms", {})
        if i not in cache:
            V, F = self.spec.meshes[i]
            g = Geometry3D(TriangleMesh(V, F))
            m = self.spec.margins
            if m is not None and m[i] > 0:
                g.setCollisionMargin(float(m[i]))
            cache[i] = g
        return cache[i]

    def enableSelfCollision(self, link1: int, link2: int, value: bool = True):
        """robotsim.cpp:5513-5527."""
        self.world.engine.enable_self_pair(self.index, link1, link2, value)
        self._self_enabled[link1, link2] = self._self_enabled[link2, link1] = bool(value)

    def selfCollisionEnabled(self, link1: int, link2: int) -> bool:
        """robotsim.cpp (RobotModel::selfCollisionEnabled)."""
        return bool(self._self_enabled[link1, link2])

    def selfCollides(self) -> bool:
        """robotsim.cpp:5529-5539 at the current configuration."""
        _, sh = self.world.engine.check_configs(self._q[None], robot=self.index, env=False)
        return bool(sh.cpu().numpy()[0])

    def selfCollidesBatch(self, Q) -> np.ndarray:
        _, sh = self.world.engine.check_configs(Q, robot=self.index, env=False)
        return sh.cpu().numpy().astype(bool)


class WorldCollider:
    """collide.py:246-700.  The collision mask starts at Klamp't's defaults
    (collide.py:314-359, PlannerSettings.cpp:16-42): robot links against
    rigid objects, non-base links against terrains, rigid objects against
    each other and against terrains, links of different robots, and each
    robot's enabled self pairs.  Link-level masks live in the engine (per
    link and environment group, and the self pairs), so the batched
    verdicts honour them; pairs the engine cannot mask (one object of a
    group shared with others, robot-robot and object-object pairs) are kept
    here and honoured by the pair iterators.

    Pair iterators (collisions, robotSelfCollisions, robotObjectCollisions,
    robotTerrainCollisions, objectTerrainCollisions, objectObjectCollisions)
    decide each pair on the GPU: self pairs through the engine's per-pair
    self-collision query, every other pair through the Geometry3D pair query
    on FP64 transforms, after a bounding-box quick reject (collide.py:467)."""

    def __init__(self, world: WorldModel, ignore=()):
        self.world = world
        self._ignored = set()        # frozenset pairs of bodies, and single bodies
        self._env_mask = {}          # (robot, link) -> group mask held by the engine
        for r in range(world.numRobots()):
            spec = world.robot(r).spec
            for l in range(spec.num_links):
                self._env_mask[(r, l)] = 0xFFFFFFFF & ~((1 << GROUP_TERRAIN) if spec.parents[l] < 0 else 0)
        self.terrains = [world.terrain(i) for i in range(world.numTerrains())]
        self.rigidObjects = [world.rigidObject(i) for i in range(world.numRigidObjects())]
        self.robots = [[world.robot(r).link(l) for l in range(world.robot(r).numLinks())]
                       for r in range(world.numRobots())]
        for i in ignore:
            self.ignoreCollision(i)

    # ---- masks --------------------------------------------------------------
    def _group(self, body: _EnvBody) -> int:
        return int(self.world.env_spec.groups[body.object])

    def _alone_in_group(self, body: _EnvBody) -> bool:
        g = np.asarray(self.world.env_spec.groups)
        return int(np.sum(g == g[body.object])) == 1

    def _set_link_mask(self, link: RobotModelLink, mask: int):
        key = (link.robot.index, link.index)
        self._env_mask[key] = mask & 0xFFFFFFFF
        self.world.engine.set_link_env_mask(key[0], key[1], mask & 0xFFFFFFFF)

    def _link_env_enabled(self, link: RobotModelLink, body: _EnvBody) -> bool:
        if link in self._ignored or body in self._ignored or frozenset((link, body)) in self._ignored:
            return False
        return bool((self._env_mask[(link.robot.index, link.index)] >> self._group(body)) & 1)

    def _pair_enabled(self, a, b) -> bool:
        """Whether the pair (a, b) is checked (collide.py:314-359 defaults,
        with the ignores applied)."""
        if a == b or a in self._ignored or b in self._ignored or frozenset((a, b)) in self._ignored:
            return False
        la, lb = isinstance(a, RobotModelLink), isinstance(b, RobotModelLink)
        if la and lb:
            if a.robot is b.robot:
                return a.robot.selfCollisionEnabled(a.index, b.index)
            return True
        if la or lb:
            link, body = (a, b) if la else (b, a)
            return self._link_env_enabled(link, body)
        # environment pairs: terrain-object and object-object (not terrain-terrain)
        return not (isinstance(a, TerrainModel) and isinstance(b, TerrainModel))

    def ignoreCollision(self, ign):
        """collide.py:379-404: a body, or a pair of bodies, removed from
        consideration.  A link-object pair whose object shares its
        environment group with other objects cannot be masked by the engine
        for the batched verdicts: it is then ignored by the pair iterators
        and a ValueError says so unless the object is alone in its group."""
        if isinstance(ign, (tuple, list)):
            a, b = ign
            la, lb = isinstance(a, RobotModelLink), isinstance(b, RobotModelLink)
            if la and lb and a.robot is b.robot:
                a.robot.enableSelfCollision(a.index, b.index, False)
            elif la != lb:
                link, body = (a, b) if la else (b, a)
                if not isinstance(body, _EnvBody):
                    raise ValueError("Invalid ignore collision item, must be a pair of bodies in the world")
                if not self._alone_in_group(body):
                    raise ValueError("the engine masks links against whole environment groups: give this object "
                                     "a group of its own when the environment is created to ignore it alone")
                self._set_link_mask(link, self._env_mask[(link.robot.index, link.index)] & ~(1 << self._group(body)))
            self._ignored.add(frozenset((a, b)))
            return
        if isinstance(ign, RobotModelLink):
            self._set_link_mask(ign, 0)
            r = ign.robot
            for j in range(r.numLinks()):
                if j != ign.index and r.selfCollisionEnabled(ign.index, j):
                    r.enableSelfCollision(ign.index, j, False)
        elif isinstance(ign, _EnvBody):
            if not self._alone_in_group(ign):
                raise ValueError("the engine masks links against whole environment groups: give this object "
                                 "a group of its own when the environment is created to ignore it alone")
            for links in self.robots:
                for link in links:
                    self._set_link_mask(link, self._env_mask[(link.robot.index, link.index)] & ~(1 << self._group(ign)))
        else:
            raise ValueError("Invalid ignore collision item, must be a body in the world")
        self._ignored.add(ign)

    def isCollisionEnabled(self, obj_or_pair) -> bool:
        """collide.py:406-427."""
        if isinstance(obj_or_pair, (tuple, list)):
            a, b = obj_or_pair
            return self._pair_enabled(a, b)
        return any(self._pair_enabled(obj_or_pair, other) for other in self._bodies() if other != obj_or_pair)

    def setLinkEnvMask(self, robot: int, link: int, group_mask: int):
        self._set_link_mask(self.world.robot(robot).link(link), group_mask)

    # ---- pair iterators ---------------------------------------------------------
    def _bodies(self):
        out = list(self.terrains) + list(self.rigidObjects)
        for links in self.robots:
            out += [l for l in links if len(l.robot.spec.meshes[l.index][1]) > 0]
        return out

    def _geom(self, body):
        return body.robot._link_geometry(body.index) if isinstance(body, RobotModelLink) else body.geometry()

    def _transform(self, body) -> np.ndarray:
        if isinstance(body, RobotModelLink):
            return body.robot._current_transforms64()[body.index]
        return np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)

    def _bb(self, body):
        """World bounding box of a body, widened by its margin."""
        g = self._geom(body)
        V = g.getTriangleMesh().vertices
        T = self._transform(body)
        W = V @ T[:9].reshape(3, 3).T + T[9:]
        m = g.getCollisionMargin() + 1e-9
        return W.min(0) - m, W.max(0) + m

    def _collide_pairs(self, pairs):
        """Colliding pairs among `pairs` (each (a, b)), in order."""
        if not pairs:
            return []
        bbs = {}
        hits = []
        self_cache = {}
        for a, b in pairs:
            if isinstance(a, RobotModelLink) and isinstance(b, RobotModelLink) and a.robot is b.robot:
                r = a.robot
                if r.index not in self_cache:
                    words = self.world.engine.self_collision_pairs(r._q[None], robot=r.index)
                    self_cache[r.index] = words.cpu().numpy().astype(np.uint32)
                i, j = min(a.index, b.index), max(a.index, b.index)
                if (int(self_cache[r.index][i]) >> j) & 1:
                    hits.append((a, b))
                continue
            for x in (a, b):
                if x not in bbs:
                    bbs[x] = self._bb(x)
            (alo, ahi), (blo, bhi) = bbs[a], bbs[b]
            if np.any(alo > bhi) or np.any(blo > ahi):
                continue
            ga, gb = self._geom(a), self._geom(b)
            hit = ga._geom.collide(gb._geom, self._transform(a)[None], self._transform(b)[None])
            if bool(hit.cpu().numpy()[0]):
                hits.append((a, b))
        return hits

    def collisionTests(self, filter1=None, filter2=None):
        """collide.py:429-499 (without the quick reject: the pairs to test)."""
        bodies = self._bodies()
        out = []
        for i, a in enumerate(bodies):
            for b in bodies[i + 1:]:
                if not self._pair_enabled(a, b):
                    continue
                if filter1 is None:
                    out.append((a, b))
                elif filter2 is None:
                    if filter1(a) and filter1(b):
                        out.append((a, b))
                elif filter1(a) and filter2(b):
                    out.append((a, b))
                elif filter2(a) and filter1(b):
                    out.append((b, a))
        return out

    def collisions(self, filter1=None, filter2=None):
        """collide.py:501-529: yields the colliding (body, body) pairs."""
        for a, b in self._collide_pairs(self.collisionTests(filter1, filter2)):
            yield (a, b)

    def robotSelfCollisions(self, robot=None):
        """collide.py:531-560: colliding (link, link) pairs of a robot (or of
        every robot)."""
        if isinstance(robot, RobotModel):
            robot = robot.index
        robots = range(self.world.numRobots()) if robot is None else [robot]
        for r in robots:
            links = self.robots[r]
            pairs = [(links[i], links[j]) for i in range(len(links)) for j in range(i)
                     if self._pair_enabled(links[i], links[j])]
            for c in self._collide_pairs(pairs):
                yield c

    def _robot_env(self, robot, bodies):
        if isinstance(robot, RobotModel):
            robot = robot.index
        pairs = [(l, o) for o in bodies for l in self.robots[robot] if self._pair_enabled(l, o)]
        return self._collide_pairs(pairs)

    def robotObjectCollisions(self, robot, object=None):
        """collide.py:562-595: colliding (link, rigid object) pairs."""
        objs = self.rigidObjects if object is None else [
            object if isinstance(object, RigidObjectModel) else self.rigidObjects[object]]
        for c in self._robot_env(robot, objs):
            yield c

    def robotTerrainCollisions(self, robot, terrain=None):
        """collide.py:597-630: colliding (link, terrain) pairs."""
        ters = self.terrains if terrain is None else [
            terrain if isinstance(terrain, TerrainModel) else self.terrains[terrain]]
        for c in self._robot_env(robot, ters):
            yield c

    def objectTerrainCollisions(self, object, terrain=None):
        """collide.py:632-664."""
        o = object if isinstance(object, RigidObjectModel) else self.rigidObjects[object]
        ters = self.terrains if terrain is None else [
            terrain if isinstance(terrain, TerrainModel) else self.terrains[terrain]]
        for c in self._collide_pairs([(o, t) for t in ters if self._pair_enabled(o, t)]):
            yield c

    def objectObjectCollisions(self, object, object2=None):
        """collide.py:666-698."""
        o = object if isinstance(object, RigidObjectModel) else self.rigidObjects[object]
        others = [x for x in self.rigidObjects if x != o] if object2 is None else [
            object2 if isinstance(object2, RigidObjectModel) else self.rigidObjects[object2]]
        for c in self._collide_pairs([(o, x) for x in others if self._pair_enabled(o, x)]):
            yield c

    def robotSelfCollides(self, robot: int = 0) -> bool:
        return self.world.robot(robot).selfCollides()

    def robotEnvCollides(self, robot: int = 0) -> bool:
        """Any link against any enabled object or terrain at the current
        configuration (robotObjectCollisions + robotTerrainCollisions)."""
        q = self.world.robot(robot)._q[None]
        eh, _ = self.world.engine.check_configs(q, robot=robot, self_collision=False)
        return bool(eh.cpu().numpy()[0])

    def check_configs(self, Q, robot: int = 0) -> Tuple[np.ndarray, np.ndarray]:
        """Batched environment / self verdicts of configurations Q [B, L]."""
        eh, sh = self.world.engine.check_configs(Q, robot=robot)
        return eh.cpu().numpy().astype(bool), sh.cpu().numpy().astype(bool)

    def check_configs_multi(self, robot_ids, Q) -> Tuple[np.ndarray, np.ndarray]:
        """Heterogeneous batch: configuration b belongs to robot_ids[b]
        (Q [B, max links], padded)."""
        eh, sh = self.world.engine.check_configs_multi(robot_ids, Q)
        return eh.cpu().numpy().astype(bool), sh.cpu().numpy().astype(bool)

    def distance(self, robot: int = 0,
                 settings: Optional[DistanceQuerySettings] = None) -> DistanceQueryResult:
        """Minimum signed link-object distance at the current configuration
        (distance_ext over every enabled pair, robotsim.cpp:1782-1819)."""
        settings = settings or DistanceQuerySettings()
        cutoff = settings.upperBound if math.isfinite(settings.upperBound) else 1e3
        q = self.world.robot(robot)._q[None]
        d, pair, cp, g = self.world.engine.distance(q, cutoff, robot=robot, want_grad=False)
        d = float(d.cpu().numpy()[0])
        pair = pair.cpu().numpy()[0]
        cp = cp.cpu().numpy()[0]
        res = DistanceQueryResult(d=d, elem1=int(pair[0]), elem2=int(pair[1]))
        if pair[0] >= 0:
            res.hasClosestPoints = True
            res.cp1 = cp[:3].tolist()
            res.cp2 = cp[3:].tolist()
            if d != 0.0:
                # separated: (cp1-cp2)/d; penetrating: cp2 = cp1 + depth n and
                # d = -depth, so the same expression gives the face normal n
                u = (cp[:3] - cp[3:]) / d
                res.hasGradients = True
                res.grad1 = u.tolist()
                res.grad2 = (-u).tolist()
        return res

    def rayCast(self, s: Sequence[float], d: Sequence[float]) -> Optional[Tuple[int, List[float]]]:
        """collide.ray_cast over the environment's objects: (object index,
        hit point) of the first hit, or None."""
        o, p = self.world.rayCast(s, d)
        return None if o < 0 else (o, p)

    def rayCastBatch(self, S, D):
        """Rays S[i] + t D[i]: (object [R] (-1 = none), triangle [R], t [R],
        hit point [R, 3])."""
        obj, tri, t, pt = self.world.engine.raycast(S, D)
        return obj.cpu().numpy(), tri.cpu().numpy(), t.cpu().numpy(), pt.cpu().numpy()

    def distance_batch(self, Q, cutoff: float = 1.0, robot: int = 0):
        """(d [B], (link, object) [B, 2], closest points [B, 6], dd/dq [B, L])."""
        d, pair, cp, g = self.world.engine.distance(Q, cutoff, robot=robot)
        return d.cpu().numpy(), pair.cpu().numpy(), cp.cpu().numpy(), g.cpu().numpy()


class IKObjective:
    """One point (or point + rotation) constraint on a link
    (robotik.h:21-60: setFixedPoint, setFixedTransform)."""

    def __init__(self):
        self.link = -1
        self.plocal = [0.0, 0.0, 0.0]
        self.pworld = [0.0, 0.0, 0.0]
        self.R = None  # row-major 3x3 when the rotation is constrained

    def setFixedPoint(self, link: int, plocal: Sequence[float], pworld: Sequence[float]):
        self.link, self.plocal, self.pworld, self.R = int(link), list(plocal), list(pworld), None

    def setFixedTransform(self, link: int, R: Sequence[float], t: Sequence[float]):
        """R in Klamp't's so3 order (column-major), t the link origin."""
        Rm = np.asarray(R, np.float64).reshape(3, 3).T
        self.link, self.plocal, self.pworld, self.R = int(link), [0.0, 0.0, 0.0], list(t), Rm.reshape(-1).tolist()


class IKSolver:
    """IKSolver (robotik.h:151-260) for one objective: solve() starts from
    the robot's current configuration and leaves the result in it."""

    def __init__(self, robot: "RobotModel"):
        self.robot = robot
        self.objectives: List[IKObjective] = []
        self.maxIters = 100
        self.tol = 1e-3
        self._residual = None

    def add(self, objective: IKObjective):
        if self.objectives:
            raise RuntimeError("one objective per solver on this path")
        self.objectives.append(objective)

    def setMaxIters(self, iters: int):
        self.maxIters = int(iters)

    def setTolerance(self, tol: float):
        self.tol = float(tol)

    def solve(self) -> bool:
        obj = self.objectives[0]
        r = self.robot
        Rt = None if obj.R is None else np.asarray(obj.R, np.float32)[None]
        q, ok, res, _ = r.world.engine.ik_solve(r._q[None], obj.link, np.asarray(obj.plocal, np.float32)[None],
                                                np.asarray(obj.pworld, np.float32)[None], Rtarget=Rt,
                                                max_iters=self.maxIters, tol=self.tol, robot=r.index)
        r.setConfig(q.cpu().numpy()[0].astype(np.float64))
        self._residual = float(res.cpu().numpy()[0])
        return bool(ok.cpu().numpy()[0])

    def getResidualMax(self) -> float:
        return self._residual


def _sample_configs(robot: "RobotModel", numSamples: int, rng: np.random.Generator) -> np.ndarray:
    """Configurations uniform within the finite joint limits; DOFs with an
    infinite limit keep their current value (SampleRobot,
    Cpp/Modeling/RandomizedSelfCollisions.cpp:9-17)."""
    spec = robot.spec
    Q = np.tile(robot._q, (numSamples, 1)).astype(np.float32)
    fin = np.isfinite(spec.qmin) & np.isfinite(spec.qmax)
    Q[:, fin] = rng.uniform(spec.qmin[fin], spec.qmax[fin], (numSamples, int(fin.sum())))
    return Q


def _words_to_matrix(words: np.ndarray, L: int) -> np.ndarray:
    return np.array([[bool((int(words[i]) >> j) & 1) for j in range(L)] for i in range(L)])


def RandomizedSelfCollisionPairs(robot: "RobotModel", numSamples: int, seed: int = 0) -> np.ndarray:
    """collision[i, j] = True iff enabled pair (i, j) collided in one of
    numSamples configurations drawn uniformly within the finite joint limits
    (Cpp/Modeling/RandomizedSelfCollisions.cpp:9-38)."""
    Q = _sample_configs(robot, numSamples, np.random.default_rng(seed))
    words = robot.world.engine.self_collision_pairs(Q, robot=robot.index).cpu().numpy().astype(np.uint32)
    return _words_to_matrix(words, robot.spec.num_links)


def RandomizedIndependentSelfCollisionPairs(robot: "RobotModel", numSamples: int, seed: int = 0) -> np.ndarray:
    """collision[i, j] = True iff enabled pair (i, j) was, in one of numSamples
    further samples, the only colliding pair among those found colliding in
    a first numSamples samples (Cpp/Modeling/RandomizedSelfCollisions.cpp:
    42-66 and 114-140: TestCollisions, then TestIndependentCollisions)."""
    rng = np.random.default_rng(seed)
    eng = robot.world.engine
    cand = eng.self_collision_pairs(_sample_configs(robot, numSamples, rng), robot=robot.index)
    words = eng.independent_self_collision_pairs(_sample_configs(robot, numSamples, rng), cand,
                                                 robot=robot.index).cpu().numpy().astype(np.uint32)
    return _words_to_matrix(words, robot.spec.num_links)


def RandomizedSelfCollisionDistances(robot: "RobotModel", numSamples: int, seed: int = 0,
                                     cutoff: float = 1e3):
    """(minDistance, maxDistance) [L, L]: for every pair i < j whose links
    both have geometry, enabled for self collision or not, the smallest and
    largest distance over numSamples configurations drawn like SampleRobot;
    the lower triangle mirrors the upper one and the diagonal is 0; pairs
    without geometry keep +inf / -inf
    (Cpp/Modeling/RandomizedSelfCollisions.cpp:142-180).  Distances are exact
    (the reference asks its geometry backend for 0.001 absolute / 1% relative
    accuracy)."""
    L = robot.spec.num_links
    Q = _sample_configs(robot, numSamples, np.random.default_rng(seed))
    lo = np.full((L, L), np.inf)
    hi = np.full((L, L), -np.inf)
    iu, ju = np.triu_indices(L, 1)
    if numSamples > 0:
        dp = robot.world.engine.self_pair_distances(Q, cutoff, robot=robot.index, all_pairs=True).cpu().numpy()
        valid = (dp >= 0).all(0)
        lo[iu[valid], ju[valid]] = dp[:, valid].min(0)
        hi[iu[valid], ju[valid]] = dp[:, valid].max(0)
    lo[ju, iu] = lo[iu, ju]
    hi[ju, iu] = hi[iu, ju]
    np.fill_diagonal(lo, 0.0)
    np.fill_diagonal(hi, 0.0)
    return lo, hi


class RobotCSpace:
    """robotcspace.py:31-118: feasibility = joint limits, then environment
    (when a collider is given), then self collision, then the extra
    constraints (RobotCSpace.cpp:786-823); visibility = every configuration
    a + (k/n)(b-a), k = 0..n, feasible, with n = max(1, ceil(|b - a|_2 / eps))
    in the L2 configuration metric (RobotCSpace.cpp:48,212-218) at
    resolution eps (cspace.py:81).  The CSpaceInterface queries
    (isFeasible / isVisible, motionplanning.cpp:789-809) gain batched
    overloads that send a planner's milestones or edges to the GPU in one
    call (isFeasibleBatch / isVisibleBatch)."""

    def __init__(self, robot: RobotModel, collider: Optional[WorldCollider] = None):
        self.robot = robot
        self.collider = collider
        self.eps = 1e-3
        lo, hi = robot.getJointLimits()
        self.bound = list(zip(lo, hi))
        self._extra = []  # (name, f(x) -> bool)
        self.properties = {"geodesic": 1}

    def setVisibilityEpsilon(self, eps: float):
        if not eps > 0:
            raise RuntimeError("Invalid visibility epsilon")
        self.eps = float(eps)

    def addConstraint(self, checker, name: Optional[str] = None):
        """robotcspace.py:75 / CSpaceInterface.addFeasibilityTest: a host
        predicate f(x) -> bool applied after the GPU tests."""
        self._extra.append((name or f"constraint {len(self._extra)}", checker))

    addFeasibilityTest = addConstraint

    def inJointLimits(self, x) -> bool:
        return all(lo <= xi <= hi for xi, (lo, hi) in zip(x, self.bound))

    def sample(self) -> List[float]:
        """Uniform within the joint limits (CSpace.sample)."""
        return [float(np.random.uniform(lo, hi)) for lo, hi in self.bound]

    def distance(self, a, b) -> float:
        return float(np.linalg.norm(np.asarray(b, np.float64) - np.asarray(a, np.float64)))

    def interpolate(self, a, b, u: float) -> List[float]:
        a = np.asarray(a, np.float64)
        return (a + u * (np.asarray(b, np.float64) - a)).tolist()

    def _gpu_feasible(self, Q) -> np.ndarray:
        eng = self.robot.world.engine
        Q = np.asarray(Q, np.float32).reshape(-1, self.robot.numLinks())
        if self.collider is not None:
            return eng.is_feasible(Q, robot=self.robot.index).cpu().numpy().astype(bool)
        lo = np.array([b[0] for b in self.bound])
        hi = np.array([b[1] for b in self.bound])
        inl = ((Q >= lo) & (Q <= hi)).all(1)
        _, sh = eng.check_configs(Q, robot=self.robot.index, env=False)
        return inl & ~sh.cpu().numpy().astype(bool)

    def isFeasibleBatch(self, Q) -> np.ndarray:
        """Feasibility of configurations Q [B, n]: one GPU call (limits,
        environment, self collision), then the extra constraints on the
        configurations that passed."""
        f = self._gpu_feasible(Q)
        if self._extra:
            for i in np.flatnonzero(f):
                x = np.asarray(Q[i], np.float64).tolist()
                f[i] = all(fn(x) for _, fn in self._extra)
        return f

    def feasible(self, x) -> bool:
        return bool(self.isFeasibleBatch(np.asarray(x, np.float32)[None])[0])

    isFeasible = feasible

    def selfCollision(self, x=None) -> bool:
        """robotcspace.py:98-105."""
        if x is not None:
            self.robot.setConfig(x)
        return self.robot.selfCollides()

    def envCollision(self, x=None) -> bool:
        """robotcspace.py:107-118: the robot against the collider's objects
        and terrains (False without a collider)."""
        if self.collider is None:
            return False
        if x is not None:
            self.robot.setConfig(x)
        return self.collider.robotEnvCollides(self.robot.index)

    def feasibilityFailures(self, x) -> List[str]:
        """CSpaceInterface.feasibilityFailures (motionplanning.cpp): names of
        the failed tests."""
        out = []
        if not self.inJointLimits(x):
            out.append("joint limits")
        if self.envCollision(x):
            out.append("env collision")
        if self.selfCollision(x):
            out.append("self collision")
        out += [name for name, fn in self._extra if not fn(list(map(float, x)))]
        return out

    def steps(self, A, B) -> np.ndarray:
        A = np.asarray(A, np.float64).reshape(-1, self.robot.numLinks())
        B = np.asarray(B, np.float64).reshape(-1, self.robot.numLinks())
        return np.maximum(1, np.ceil(np.linalg.norm(B - A, axis=1) / self.eps)).astype(np.int32)

    def isVisibleBatch(self, A, B) -> Tuple[np.ndarray, np.ndarray]:
        """(visible [E] bool, first infeasible step index [E], -1 if none):
        one GPU call for all E edges; extra constraints, if any, are checked
        on the host along the edges the GPU found free."""
        A = np.asarray(A, np.float32).reshape(-1, self.robot.numLinks())
        B = np.asarray(B, np.float32).reshape(-1, self.robot.numLinks())
        n = self.steps(A, B)
        eng = self.robot.world.engine
        if self.collider is not None:
            fh = eng.check_edges(A, B, n, robot=self.robot.index).cpu().numpy()
        else:
            fh = np.full(len(n), -1, np.int32)
            for e in range(len(n)):
                u = np.arange(n[e] + 1)[:, None] / float(n[e])
                Q = (A[e].astype(np.float64) + u * (B[e].astype(np.float64) - A[e])).astype(np.float32)
                bad = np.flatnonzero(~self._gpu_feasible(Q))
                fh[e] = bad[0] if len(bad) else -1
        if self._extra:
            for e in np.flatnonzero(fh < 0):
                for k in range(n[e] + 1):
                    if not all(fn(self.interpolate(A[e], B[e], k / n[e])) for _, fn in self._extra):
                        fh[e] = k
                        break
        return fh < 0, fh

    def isVisible(self, a, b) -> bool:
        vis, _ = self.isVisibleBatch(np.asarray(a)[None], np.asarray(b)[None])
        return bool(vis[0])


def make_space(world: WorldModel, robot: RobotModel, edgeCheckResolution: float = 1e-2,
               extraConstraints: Sequence = (), ignoreCollisions: Sequence = ()) -> RobotCSpace:
    """robotplanning.py:23-90 (make_space) for the unconstrained case: a
    RobotCSpace over a WorldCollider of the world (ignoring the listed
    bodies or pairs), edge resolution edgeCheckResolution, extra host
    constraints.  Planners built on it check milestones and edges in
    batches (isFeasibleBatch / isVisibleBatch; klampt_gb300.plan)."""
    collider = WorldCollider(world, ignore=list(ignoreCollisions))
    space = RobotCSpace(robot, collider)
    space.eps = float(edgeCheckResolution)
    for c in extraConstraints:
        space.addConstraint(c)
    return space

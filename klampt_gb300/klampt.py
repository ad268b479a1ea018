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
Batched overloads: RobotModel.setConfigs / getJacobians, WorldCollider.check_configs /
distance_batch / rayCastBatch, RobotCSpace.isFeasibleBatch / isVisibleBatch.

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
    points on self (the link) and other (the object) in world coordinates;
    grad1 is the gradient of the distance w.r.t. moving cp1 and grad2 =
    -grad1; elem1 = link index, elem2 = object index."""
    d: float = math.inf
    hasClosestPoints: bool = False
    hasGradients: bool = False
    cp1: List[float] = field(default_factory=list)
    cp2: List[float] = field(default_factory=list)
    grad1: List[float] = field(default_factory=list)
    grad2: List[float] = field(default_factory=list)
    elem1: int = -1
    elem2: int = -1


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

    def rayCast(self, s: Sequence[float], d: Sequence[float]) -> Tuple[int, List[float]]:
        """WorldModel::RayCast over the environment: (object index, world hit
        point), or (-1, [0, 0, 0]) when nothing is hit."""
        obj, _, _, pt = self._world.raycast(np.asarray(s, np.float32)[None], np.asarray(d, np.float32)[None])
        return int(obj.cpu()[0]), pt.cpu().numpy()[0].tolist()

    def close(self):
        self._world.close()


class RobotModelLink:
    def __init__(self, robot: "RobotModel", index: int):
        self.robot = robot
        self.index = index

    def getIndex(self) -> int:
        return self.index

    def getParent(self) -> int:
        return int(self.robot.spec.parents[self.index])

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

    def enableSelfCollision(self, link1: int, link2: int, value: bool = True):
        """robotsim.cpp:5513-5527."""
        self.world.engine.enable_self_pair(self.index, link1, link2, value)

    def selfCollides(self) -> bool:
        """robotsim.cpp:5529-5539 at the current configuration."""
        _, sh = self.world.engine.check_configs(self._q[None], robot=self.index, env=False)
        return bool(sh.cpu().numpy()[0])

    def selfCollidesBatch(self, Q) -> np.ndarray:
        _, sh = self.world.engine.check_configs(Q, robot=self.index, env=False)
        return sh.cpu().numpy().astype(bool)


class WorldCollider:
    """collide.py:246: the collision mask follows Klamp't's defaults
    (links vs rigid objects, non-base links vs terrains, robot self pairs);
    ignoreCollision-style edits go through setLinkEnvMask /
    RobotModel.enableSelfCollision."""

    def __init__(self, world: WorldModel):
        self.world = world

    def setLinkEnvMask(self, robot: int, link: int, group_mask: int):
        self.world.engine.set_link_env_mask(robot, link, group_mask)

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
    """(minDistance, maxDistance) [L, L]: for each enabled self pair i < j the
    smallest and largest distance over numSamples configurations drawn like
    SampleRobot (Cpp/Modeling/RandomizedSelfCollisions.cpp:142-180); +inf /
    -inf for pairs that are not enabled (the reference's initial values).
    Distances are exact (the reference asks its geometry backend for 0.001
    absolute / 1% relative accuracy)."""
    L = robot.spec.num_links
    Q = _sample_configs(robot, numSamples, np.random.default_rng(seed))
    dp = robot.world.engine.self_pair_distances(Q, cutoff, robot=robot.index).cpu().numpy()
    lo = np.full((L, L), np.inf)
    hi = np.full((L, L), -np.inf)
    iu, ju = np.triu_indices(L, 1)
    valid = (dp >= 0).all(0) if len(dp) else np.zeros(len(iu), bool)
    if len(dp):
        lo[iu[valid], ju[valid]] = dp[:, valid].min(0)
        hi[iu[valid], ju[valid]] = dp[:, valid].max(0)
    return lo, hi


class RobotCSpace:
    """robotcspace.py:31: feasibility = joint limits, then environment, then
    self collision (RobotCSpace.cpp:786-823); visibility = every
    configuration a + (k/n)(b-a), k = 0..n, feasible, with
    n = max(1, ceil(|b - a|_2 / eps)) in the L2 configuration metric
    (RobotCSpace.cpp:48,212-218) at resolution eps (cspace.py:81)."""

    def __init__(self, robot: RobotModel, collider: Optional[WorldCollider] = None):
        self.robot = robot
        self.collider = collider
        self.eps = 1e-3
        lo, hi = robot.getJointLimits()
        self.bound = list(zip(lo, hi))

    def setVisibilityEpsilon(self, eps: float):
        if not eps > 0:
            raise RuntimeError("Invalid visibility epsilon")
        self.eps = float(eps)

    def inJointLimits(self, x) -> bool:
        return all(lo <= xi <= hi for xi, (lo, hi) in zip(x, self.bound))

    def isFeasibleBatch(self, Q) -> np.ndarray:
        f = self.robot.world.engine.is_feasible(Q, robot=self.robot.index)
        return f.cpu().numpy().astype(bool)

    def feasible(self, x) -> bool:
        return bool(self.isFeasibleBatch(np.asarray(x, np.float32)[None])[0])

    isFeasible = feasible

    def steps(self, A, B) -> np.ndarray:
        A = np.asarray(A, np.float64).reshape(-1, self.robot.numLinks())
        B = np.asarray(B, np.float64).reshape(-1, self.robot.numLinks())
        return np.maximum(1, np.ceil(np.linalg.norm(B - A, axis=1) / self.eps)).astype(np.int32)

    def isVisibleBatch(self, A, B) -> Tuple[np.ndarray, np.ndarray]:
        """(visible [E] bool, first infeasible step index [E], -1 if none)."""
        n = self.steps(A, B)
        fh = self.robot.world.engine.check_edges(np.asarray(A, np.float32), np.asarray(B, np.float32), n,
                                                 robot=self.robot.index).cpu().numpy()
        return fh < 0, fh

    def isVisible(self, a, b) -> bool:
        vis, _ = self.isVisibleBatch(np.asarray(a)[None], np.asarray(b)[None])
        return bool(vis[0])

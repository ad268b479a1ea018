"""Host logic of the batched lazy PRM (klampt_gb300.plan), on the CPU: the
C-space is a stand-in whose batched queries are answered by the FP64
oracle, so only the planner's own roadmap, search and batching are under
test (the engine behind the real C-space is parity-tested on the GPU)."""

import os

import numpy as np

from klampt_gb300 import scenes as sc
from klampt_gb300.plan import BatchedLazyPRM

NT = os.cpu_count() or 4


class OracleSpace:
    def __init__(self, robot, env, eps=0.02):
        from oracle.oracle_py import Oracle
        self.o = Oracle(robot, env)
        self.bound = list(zip(robot.qmin, robot.qmax))
        self.eps = eps
        self.calls = []

    def isFeasibleBatch(self, Q):
        self.calls.append(("feasible", len(Q)))
        return self.o.is_feasible(np.asarray(Q, np.float32), nthreads=NT).astype(bool)

    def steps(self, A, B):
        return np.maximum(1, np.ceil(np.linalg.norm(np.asarray(B, np.float64) - A, axis=1) / self.eps)).astype(np.int32)

    def isVisibleBatch(self, A, B):
        self.calls.append(("visible", len(A)))
        fh, _ = self.o.check_edges(A, B, self.steps(A, B), nthreads=NT)
        return fh < 0, fh


def test_lazy_prm_batches_and_path():
    robot, env, q = sc.scene_cfg0()
    space = OracleSpace(robot, env)
    feas = space.o.is_feasible(q, nthreads=NT).astype(bool)
    free = q[feas].astype(np.float64)
    d = np.linalg.norm(free - free[0], axis=1)
    goal = free[np.flatnonzero(d > 0.8)[np.argmin(d[d > 0.8])]]
    planner = BatchedLazyPRM(space, k=12, seed=3)
    path = planner.plan(free[0], goal, n_milestones=1500, max_rounds=200)
    assert path is not None
    P = np.asarray(path, np.float32)
    assert space.o.is_feasible(P).all()
    fh, _ = space.o.check_edges(P[:-1], P[1:], space.steps(P[:-1], P[1:]))
    assert (fh < 0).all()
    kinds = [k for k, _ in space.calls]
    # two milestone batches (the ends, then all samples); one edge batch per round
    assert kinds[:2] == ["feasible", "feasible"] and set(kinds[2:]) == {"visible"}
    assert planner.stats["visibility_batches"] == len(kinds) - 2


def test_lazy_prm_infeasible_goal():
    robot, env, q = sc.scene_cfg0()
    space = OracleSpace(robot, env)
    feas = space.o.is_feasible(q, nthreads=NT).astype(bool)
    start = q[np.flatnonzero(feas)[0]].astype(np.float64)
    goal = q[np.flatnonzero(~feas)[0]].astype(np.float64)
    assert BatchedLazyPRM(space, seed=1).plan(start, goal, n_milestones=50) is None

"""A lazy probabilistic roadmap whose collision checks go to the GPU in
batches: the planner-side use of the batched CSpaceInterface queries
(CSpaceInterface.isFeasible / isVisible, Python/klampt/src/motionplanning.cpp:
789-809, as reached through robotplanning.make_space,
Python/klampt/plan/robotplanning.py:23-90).

Klamp't's lazy PRM (KrisLibrary LazyPRM*, selected by MotionPlan type
"lazyprm*") checks one milestone and one edge per callback.  Here every
round sends all new milestones to RobotCSpace.isFeasibleBatch in one call,
and all unchecked edges of the current shortest roadmap path to
RobotCSpace.isVisibleBatch in one call; the graph search stays on the host.
"""

from __future__ import annotations

import heapq
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np


class BatchedLazyPRM:
    """Lazy PRM over a RobotCSpace (or anything with isFeasibleBatch,
    isVisibleBatch and bound): k-nearest-neighbour roadmap in the L2 metric,
    shortest path by Dijkstra, edges of that path checked in one batch,
    failed edges removed, repeated until a path survives."""

    def __init__(self, space, k: int = 10, seed: int = 0):
        self.space = space
        self.k = int(k)
        self.rng = np.random.default_rng(seed)
        self.milestones = np.zeros((0, len(space.bound)))
        self.adj: List[Dict[int, float]] = []
        self.checked: Dict[Tuple[int, int], bool] = {}
        self.stats = {"feasibility_batches": 0, "visibility_batches": 0, "milestones_checked": 0,
                      "edges_checked": 0}

    def _sample(self, n: int) -> np.ndarray:
        lo = np.array([b[0] for b in self.space.bound])
        hi = np.array([b[1] for b in self.space.bound])
        return self.rng.uniform(lo, hi, (n, len(lo))).astype(np.float32).astype(np.float64)

    def add_milestones(self, Q: np.ndarray) -> np.ndarray:
        """Checks Q [n, d] in one GPU call, keeps the feasible ones and
        connects each to its k nearest roadmap neighbours (edges unchecked).
        Returns the roadmap indices of the kept milestones."""
        Q = np.asarray(Q, np.float64).reshape(-1, self.milestones.shape[1])
        ok = self.space.isFeasibleBatch(Q.astype(np.float32))
        self.stats["feasibility_batches"] += 1
        self.stats["milestones_checked"] += len(Q)
        new = []
        for q in Q[ok]:
            i = len(self.milestones)
            self.milestones = np.vstack([self.milestones, q[None]])
            self.adj.append({})
            new.append(i)
        for i in new:
            d = np.linalg.norm(self.milestones - self.milestones[i], axis=1)
            d[i] = np.inf
            for j in np.argsort(d)[:self.k]:
                if np.isfinite(d[j]):
                    self.adj[i][int(j)] = float(d[j])
                    self.adj[int(j)][i] = float(d[j])
        return np.asarray(new, np.int64)

    def _shortest(self, s: int, g: int) -> Optional[List[int]]:
        dist = {s: 0.0}
        prev = {}
        pq = [(0.0, s)]
        while pq:
            du, u = heapq.heappop(pq)
            if u == g:
                path = [g]
                while path[-1] != s:
                    path.append(prev[path[-1]])
                return path[::-1]
            if du > dist.get(u, np.inf):
                continue
            for v, w in self.adj[u].items():
                nd = du + w
                if nd < dist.get(v, np.inf):
                    dist[v] = nd
                    prev[v] = u
                    heapq.heappush(pq, (nd, v))
        return None

    def plan(self, start: Sequence[float], goal: Sequence[float], n_milestones: int = 500,
             max_rounds: int = 50) -> Optional[List[List[float]]]:
        """A collision-free path start -> goal (list of configurations), or
        None when the roadmap has none after max_rounds path checks."""
        d = len(self.space.bound)
        self.milestones = np.zeros((0, d))
        self.adj, self.checked = [], {}
        ends = self.add_milestones(np.asarray([start, goal], np.float64))
        if len(ends) < 2:
            return None
        s, g = 0, 1
        self.add_milestones(self._sample(n_milestones))
        for _ in range(max_rounds):
            path = self._shortest(s, g)
            if path is None:
                return None
            edges = [(min(a, b), max(a, b)) for a, b in zip(path[:-1], path[1:])]
            todo = [e for e in edges if e not in self.checked]
            if todo:
                A = self.milestones[[e[0] for e in todo]]
                B = self.milestones[[e[1] for e in todo]]
                vis, _ = self.space.isVisibleBatch(A.astype(np.float32), B.astype(np.float32))
                self.stats["visibility_batches"] += 1
                self.stats["edges_checked"] += len(todo)
                for e, v in zip(todo, vis):
                    self.checked[e] = bool(v)
                    if not v:
                        self.adj[e[0]].pop(e[1], None)
                        self.adj[e[1]].pop(e[0], None)
            if all(self.checked.get(e, False) for e in edges):
                return [self.milestones[i].tolist() for i in path]
        return None

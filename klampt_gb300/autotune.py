"""Autotuner for the engine's launch shape and work split.

Tries, on a sample of the caller's own workload, every combination of
  blocks_per_sm  2, 3, 4   (8-warp blocks per SM; selects the register budget
                            of the engine instantiation: 128 / 80 / 64)
  grab           1, 2, 4   (work items a warp takes per queue atomic)
  job_flush      32, 64    (triangle-pair jobs collected before testing)
and, for configuration batches,
  fp64_inline    0, 1      (FP64 triangle tests deferred to a second kernel,
                            or inline in the traversal)
or, for edge batches (FP64 tests always deferred there),
  edge_chunk     8, 16, 32 (consecutive steps of an edge per work item)
times each with CUDA events (median of `reps` after one warm-up), re-times
the few fastest with more repetitions and leaves the fastest setting in the
world.  Results are identical for every setting; only
the time changes.
"""

from __future__ import annotations

import itertools
from typing import Callable, Dict, List, Optional, Tuple

import torch

from .engine import World

_BASE = {"blocks_per_sm": (2, 3, 4), "grab": (1, 2, 4), "job_flush": (32, 64)}
GRID = dict(_BASE, fp64_inline=(0, 1))
GRID_EDGES = dict(_BASE, fp64_inline=(0,), edge_chunk=(8, 16, 32))


def _time(fn: Callable[[], None], reps: int, prep: Optional[Callable[[], None]] = None) -> float:
    fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        if prep is not None:
            prep()  # outside the timed region (e.g. an L2 flush)
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        torch.cuda.synchronize()
        times.append(s.elapsed_time(e))
    return sorted(times)[len(times) // 2]


def tune(world: World, run: Callable[[], None], reps: int = 3,
         grid: Dict[str, tuple] = GRID, prep: Optional[Callable[[], None]] = None,
         finalists: int = 4, final_reps: int = 9) -> Tuple[Dict[str, int], List[Tuple[Dict[str, int], float]]]:
    """Times `run` (a closure launching the workload on `world`) under every
    setting of `grid` (median of `reps`; `prep` runs before each repetition,
    untimed), re-times the `finalists` fastest with `final_reps` repetitions
    so that one noisy sample does not decide, applies and returns the best
    plus the full table (ms)."""
    def timed(cfg):
        for k, v in cfg.items():
            world.set_option(k, v)
        return _time(run, reps, prep)

    keys = list(grid)
    table = [(cfg, timed(cfg)) for cfg in (dict(zip(keys, values))
                                           for values in itertools.product(*(grid[k] for k in keys)))]
    final = []
    for cfg, _ in sorted(table, key=lambda x: x[1])[:max(1, finalists)]:
        for k, v in cfg.items():
            world.set_option(k, v)
        final.append((cfg, _time(run, final_reps, prep)))
    best = min(final, key=lambda x: x[1])[0]
    for k, v in best.items():
        world.set_option(k, v)
    world.sync()
    return best, table


def tune_edges(world: World, qa, qb, nsteps, robot: int = 0, reps: int = 3,
               prep: Optional[Callable[[], None]] = None, graph: bool = False,
               finalists: int = 4, final_reps: int = 9):
    """The edge grid on a sample batch.  graph=True times each setting as the
    CUDA-graph edge plan it would be replayed as (one plan per setting,
    recorded on first use and destroyed afterwards) instead of eager calls."""
    a = torch.as_tensor(qa).cuda()
    b = torch.as_tensor(qb).cuda()
    n = torch.as_tensor(nsteps).cuda()
    if not graph:
        return tune(world, lambda: world.check_edges(a, b, n, robot=robot, sync=False), reps, GRID_EDGES, prep,
                    finalists, final_reps)
    out = torch.empty(a.shape[0], dtype=torch.int32, device="cuda")
    plans = {}

    def run():
        key = tuple(world.get_option(k) for k in GRID_EDGES)
        if key not in plans:
            plans[key] = world.edge_plan(a, b, n, out, robot=robot)
        plans[key].launch()

    try:
        return tune(world, run, reps, GRID_EDGES, prep, finalists, final_reps)
    finally:
        world.sync()
        for p in plans.values():
            p.close()


def tune_configs(world: World, q, robot: int = 0, reps: int = 3):
    qd = torch.as_tensor(q).cuda()
    return tune(world, lambda: world.check_configs(qd, robot=robot, sync=False), reps)


def tune_configs_multi(world: World, robot_ids, q, reps: int = 3, prep: Optional[Callable[[], None]] = None):
    """The grid on a heterogeneous batch (robot_ids [B], q [B, max links])."""
    ids = torch.as_tensor(robot_ids).cuda()
    qd = torch.as_tensor(q).cuda()
    return tune(world, lambda: world.check_configs_multi(ids, qd, sync=False), reps, GRID, prep)

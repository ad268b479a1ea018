"""Host logic of the Klamp't-named facade, run on the CPU: the engine is
replaced by the FP64 oracle so only the facade's own sampling and reduction
are under test (the engine itself is parity-tested on the GPU)."""

import os
from types import SimpleNamespace

import numpy as np
import torch

from klampt_gb300 import klampt as kl
from klampt_gb300 import scenes as sc

NT = os.cpu_count() or 4


def _robot_with_oracle_engine(spec, env):
    from oracle.oracle_py import Oracle, self_pair_distances
    o = Oracle(spec, env)
    calls = []

    def pair_distances(Q, cutoff, robot=0):
        calls.append((np.array(Q), cutoff, robot))
        return torch.from_numpy(self_pair_distances(o, Q, cutoff=cutoff, nthreads=NT))

    engine = SimpleNamespace(self_pair_distances=pair_distances)
    robot = SimpleNamespace(spec=spec, _q=np.zeros(spec.num_links, np.float32), index=0,
                            world=SimpleNamespace(engine=engine))
    return robot, o, calls


def test_randomized_self_collision_distances_reduction():
    """Per-pair minima and maxima over the samples; +inf / -inf for pairs
    that are not queried; the samples are SampleRobot's (uniform within the
    finite limits, seeded)."""
    from oracle.oracle_py import self_pair_distances
    spec = sc.arm(5, rings=4, segments=8)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    robot, o, calls = _robot_with_oracle_engine(spec, env)
    lo, hi = kl.RandomizedSelfCollisionDistances(robot, 40, seed=7)
    assert len(calls) == 1
    Q = calls[0][0]
    assert Q.shape == (40, 5)
    assert np.array_equal(Q, kl._sample_configs(robot, 40, np.random.default_rng(7)))
    assert (Q >= spec.qmin.astype(np.float32)).all() and (Q <= spec.qmax.astype(np.float32)).all()
    ref = self_pair_distances(o, Q, cutoff=1e3, nthreads=NT)
    L = spec.num_links
    iu, ju = np.triu_indices(L, 1)
    mask = spec.packed()["self_mask"].astype(bool).reshape(L, L)[iu, ju]
    assert np.array_equal(lo[iu[mask], ju[mask]], ref[:, mask].min(0))
    assert np.array_equal(hi[iu[mask], ju[mask]], ref[:, mask].max(0))
    assert np.isposinf(lo[iu[~mask], ju[~mask]]).all() and np.isneginf(hi[iu[~mask], ju[~mask]]).all()
    assert np.isposinf(np.tril(lo)[np.tril_indices(L)]).all()
    assert (lo[iu[mask], ju[mask]] <= hi[iu[mask], ju[mask]]).all()


def test_randomized_self_collision_distances_no_samples():
    spec = sc.arm(3, rings=4, segments=8)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    robot, _, _ = _robot_with_oracle_engine(spec, env)
    lo, hi = kl.RandomizedSelfCollisionDistances(robot, 0)
    assert np.isposinf(lo).all() and np.isneginf(hi).all()

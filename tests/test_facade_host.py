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

    def pair_distances(Q, cutoff, robot=0, all_pairs=False):
        calls.append((np.array(Q), cutoff, robot, all_pairs))
        return torch.from_numpy(self_pair_distances(o, Q, cutoff=cutoff, nthreads=NT, all_pairs=all_pairs))

    engine = SimpleNamespace(self_pair_distances=pair_distances)
    robot = SimpleNamespace(spec=spec, _q=np.zeros(spec.num_links, np.float32), index=0,
                            world=SimpleNamespace(engine=engine))
    return robot, o, calls


def test_randomized_self_collision_distances_reduction():
    """Per-pair minima and maxima over the samples for every pair with
    geometry, self-collision mask or not (RandomizedSelfCollisions.cpp:
    145-151); the lower triangle mirrors the upper one and the diagonal is 0
    (:171-178); the samples are SampleRobot's (uniform within the finite
    limits, seeded)."""
    from oracle.oracle_py import self_pair_distances
    spec = sc.arm(5, rings=4, segments=8)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    robot, o, calls = _robot_with_oracle_engine(spec, env)
    lo, hi = kl.RandomizedSelfCollisionDistances(robot, 40, seed=7)
    assert len(calls) == 1 and calls[0][3] is True
    Q = calls[0][0]
    assert Q.shape == (40, 5)
    assert np.array_equal(Q, kl._sample_configs(robot, 40, np.random.default_rng(7)))
    assert (Q >= spec.qmin.astype(np.float32)).all() and (Q <= spec.qmax.astype(np.float32)).all()
    ref = self_pair_distances(o, Q, cutoff=1e3, nthreads=NT, all_pairs=True)
    enabled_only = self_pair_distances(o, Q, cutoff=1e3, nthreads=NT)
    L = spec.num_links
    iu, ju = np.triu_indices(L, 1)
    mask = spec.packed()["self_mask"].astype(bool).reshape(L, L)[iu, ju]
    assert (~mask).any() and (ref >= 0).all()                     # adjacent pairs are queried too
    assert np.array_equal(ref[:, mask], enabled_only[:, mask])
    assert (enabled_only[:, ~mask] == -1).all()
    assert np.array_equal(lo[iu, ju], ref.min(0)) and np.array_equal(hi[iu, ju], ref.max(0))
    assert np.array_equal(lo, lo.T) and np.array_equal(hi, hi.T)
    assert (np.diag(lo) == 0).all() and (np.diag(hi) == 0).all()
    assert (lo[iu, ju] <= hi[iu, ju]).all()
    # adjacent links touch at their shared joint
    assert (lo[iu[~mask], ju[~mask]] == 0).all()


def test_randomized_self_collision_distances_no_samples():
    spec = sc.arm(3, rings=4, segments=8)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    robot, _, calls = _robot_with_oracle_engine(spec, env)
    lo, hi = kl.RandomizedSelfCollisionDistances(robot, 0)
    assert not calls
    off = ~np.eye(3, dtype=bool)
    assert np.isposinf(lo[off]).all() and np.isneginf(hi[off]).all()
    assert (np.diag(lo) == 0).all() and (np.diag(hi) == 0).all()

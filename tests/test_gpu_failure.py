"""Failure paths of the collision engine, driven on the GPU without a fault:
world options cap the undecided-pair list (the FP64 fallback pass re-checks
every step), the traversal spill stack (KGPU_ERR_OVERFLOW), and the
work-sharing hand-over wait (a donor that claims a waiting warp and never
hands work over, with a one-poll wait limit: KGPU_ERR_TIMEOUT).  Each case
checks the status the host reads and that the world answers correctly
afterwards; every wait in the kernel is bounded, nothing hangs or traps."""

import os

import numpy as np
import pytest

from klampt_gb300 import scenes as sc

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 4


@pytest.fixture(scope="module")
def cfg1():
    from klampt_gb300 import build
    build.build()
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, (qa, qb, ns) = sc.scene_cfg1(n_edges=2048)
    w = World(env, [robot])
    fo, _ = Oracle(robot, env).check_edges(qa, qb, ns, nthreads=NT)
    yield w, (qa, qb, ns), fo
    w.close()


def test_pair_list_overflow_takes_the_fallback_pass(cfg1):
    w, (qa, qb, ns), fo = cfg1
    w.reset_stats()
    w.set_option("pend_cap", 1)
    try:
        fh = w.check_edges(qa, qb, ns).cpu().numpy()
    finally:
        w.set_option("pend_cap", 0)
    assert np.array_equal(fh, fo)
    assert w.stats()["band_pairs"] > 1  # more undecided pairs than the list held


def test_spill_exhaustion_is_reported(cfg1):
    from klampt_gb300._kgpu import KGPU_ERR_OVERFLOW, KgpuError
    w, (qa, qb, ns), fo = cfg1
    w.reset_stats()
    w.check_edges(qa, qb, ns)
    assert w.stats()["spills"] > 0  # the workload spills its traversal stacks
    w.set_option("spill_cap", 1)
    try:
        with pytest.raises(KgpuError) as ex:
            w.check_edges(qa, qb, ns)
        assert ex.value.code == KGPU_ERR_OVERFLOW
    finally:
        w.set_option("spill_cap", 0)
    assert np.array_equal(w.check_edges(qa, qb, ns).cpu().numpy(), fo)


def test_share_wait_timeout_is_reported(cfg1):
    from klampt_gb300._kgpu import KGPU_ERR_TIMEOUT, KgpuError
    w, (qa, qb, ns), fo = cfg1
    idx = np.argsort(-ns)[:64]  # few long edges: warps run dry while siblings hold deep stacks
    w.set_option("share_no_release", 1)
    w.set_option("share_wait_polls", 1)
    try:
        with pytest.raises(KgpuError) as ex:
            w.check_edges(qa[idx], qb[idx], ns[idx])
        assert ex.value.code == KGPU_ERR_TIMEOUT
    finally:
        w.set_option("share_no_release", 0)
        w.set_option("share_wait_polls", 0)
    # the donor kept its entries, the context is usable, results are exact
    assert np.array_equal(w.check_edges(qa[idx], qb[idx], ns[idx]).cpu().numpy(), fo[idx])
    assert np.array_equal(w.check_edges(qa, qb, ns).cpu().numpy(), fo)


def test_failure_options_validated(cfg1):
    from klampt_gb300._kgpu import KgpuError
    w = cfg1[0]
    for name, bad in (("pend_cap", -1), ("spill_cap", float("nan")), ("share_wait_polls", 2.0 ** 21),
                      ("share_no_release", 2)):
        with pytest.raises(KgpuError):
            w.set_option(name, bad)
    assert w.get_option("pend_cap") == 0 and w.get_option("share_no_release") == 0

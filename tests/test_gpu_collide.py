"""GPU parity of the collision engine against the FP64 oracle (bit-exact
booleans / indices), through the C ABI."""

import os

import numpy as np
import pytest

from klampt_gb300 import scenes as sc

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 4


@pytest.fixture(scope="module")
def built():
    from klampt_gb300 import build
    build.build()
    from oracle import oracle_py
    oracle_py.build()
    return True


@pytest.fixture(scope="module")
def cfg0(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg0()
    w = World(env, [robot])
    o = Oracle(robot, env)
    yield robot, env, q, w, o
    w.close()


@pytest.fixture(scope="module")
def cfg1(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, (qa, qb, ns) = sc.scene_cfg1(n_edges=2048)
    w = World(env, [robot])
    o = Oracle(robot, env)
    yield robot, env, (qa, qb, ns), w, o
    w.close()


def _check_fk_bounds(w, o, robot, q):
    """Every vertex placed with the FP32 transform lies within the reported
    per-link bound of its FP64 placement."""
    T, err = w.fk(q, with_error=True)
    T = T.cpu().numpy().astype(np.float64)
    err = err.cpu().numpy().astype(np.float64)
    worst_ratio = 0.0
    for b in range(len(q)):
        T64 = o.fk(q[b].astype(np.float64))
        for l, (V, _) in enumerate(robot.meshes):
            R32, t32 = T[b, l, :9].reshape(3, 3), T[b, l, 9:]
            R64, t64 = T64[l, :9].reshape(3, 3), T64[l, 9:]
            d = np.linalg.norm(V @ R32.T + t32 - (V @ R64.T + t64), axis=1).max()
            assert d <= err[b, l], (b, l, d, err[b, l])
            worst_ratio = max(worst_ratio, d / err[b, l])
    return worst_ratio, err


def test_fk_error_bounds_hold(cfg0):
    robot, env, q, w, o = cfg0
    ratio, err = _check_fk_bounds(w, o, robot, q[:256])
    # bounds are rigorous (ratio <= 1) and tight enough to be useful
    assert ratio <= 1.0 and err.max() < 5e-5


def test_fk_error_bounds_tree_robot(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot = sc.humanoid()
    env = sc.env_from_objects("one_box", [sc.box_mesh((2, 2, 2), (0.1, 0.1, 0.1))])
    w = World(env, [robot])
    o = Oracle(robot, env)
    q = sc.uniform_configs(robot, 64, np.random.default_rng(11))
    ratio, err = _check_fk_bounds(w, o, robot, q)
    assert ratio <= 1.0
    w.close()


def test_cfg0_verdicts_bit_exact(cfg0):
    robot, env, q, w, o = cfg0
    eh_o, sh_o, _ = o.check_configs(q, nthreads=NT)
    eh, sh = w.check_configs(q)
    eh, sh = eh.cpu().numpy(), sh.cpu().numpy()
    assert np.array_equal(eh, eh_o), np.flatnonzero(eh != eh_o)[:10]
    assert np.array_equal(sh, sh_o), np.flatnonzero(sh != sh_o)[:10]
    assert 0.1 < eh.mean() < 0.9 and 0.1 < sh.mean() < 0.9


def test_cfg0_plain64_bit_exact(cfg0):
    robot, env, q, w, o = cfg0
    eh_o, sh_o, _ = o.check_configs(q[:1024], nthreads=NT)
    eh, sh = w.check_configs_plain64(q[:1024])
    assert np.array_equal(eh.cpu().numpy(), eh_o)
    assert np.array_equal(sh.cpu().numpy(), sh_o)


def test_cfg0_env_only_and_self_only(cfg0):
    robot, env, q, w, o = cfg0
    eh_o, sh_o, _ = o.check_configs(q[:512], nthreads=NT)
    eh, sh = w.check_configs(q[:512], env=True, self_collision=False)
    assert sh is None and np.array_equal(eh.cpu().numpy(), eh_o)
    eh, sh = w.check_configs(q[:512], env=False, self_collision=True)
    assert eh is None and np.array_equal(sh.cpu().numpy(), sh_o)


def test_cfg0_host_buffers(cfg0):
    robot, env, q, w, o = cfg0
    eh_d, sh_d = w.check_configs(q[:1000])
    eh_h, sh_h = w.check_configs_host(q[:1000])
    assert np.array_equal(eh_h, eh_d.cpu().numpy()) and np.array_equal(sh_h, sh_d.cpu().numpy())


def test_feasibility_matches_oracle(cfg0):
    robot, env, q, w, o = cfg0
    qq = q[:1024].copy()
    qq[::7, 2] = 3.5  # outside the joint limits
    f_o = o.is_feasible(qq, nthreads=NT)
    f = w.is_feasible(qq).cpu().numpy()
    assert np.array_equal(f, f_o)
    assert f[::7].sum() == 0


@pytest.mark.parametrize("which", ["dual_arm", "humanoid"])
def test_config_groups_other_link_counts(built, which):
    """Configuration batches are checked in groups of 32 / L configurations
    (L = link count rounded up to 8, 16 or 32): the 12-link dual arm runs in
    pairs, the 31-link humanoid alone.  A batch size that is not a multiple
    of the group, joint-limit violations at every position of a group, and
    environment, self and feasibility verdicts against the oracle."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot = sc.dual_arm() if which == "dual_arm" else sc.humanoid()
    env = sc.sphere_field(np.random.default_rng(1001), n=400)
    w = World(env, [robot])
    o = Oracle(robot, env)
    q = sc.uniform_configs(robot, 1001, np.random.default_rng(31))
    eh_o, sh_o, _ = o.check_configs(q, nthreads=NT)
    eh, sh = (x.cpu().numpy() for x in w.check_configs(q))
    assert np.array_equal(eh, eh_o) and np.array_equal(sh, sh_o)
    assert 0.02 < eh.mean() < 0.98
    qq = q.copy()
    span = robot.qmax - robot.qmin
    for k in range(0, len(qq), 5):
        j = (k // 5) % robot.num_links
        if span[j] > 0:
            qq[k, j] = robot.qmax[j] + 0.25
    f_o = o.is_feasible(qq, nthreads=NT)
    f = w.is_feasible(qq).cpu().numpy()
    assert np.array_equal(f, f_o)
    w.close()


def test_cfg1_configs_bit_exact(cfg1):
    robot, env, (qa, qb, ns), w, o = cfg1
    q = sc.uniform_configs(robot, 2048, np.random.default_rng(7))
    eh_o, sh_o, _ = o.check_configs(q, nthreads=NT)
    eh, sh = w.check_configs(q)
    assert np.array_equal(eh.cpu().numpy(), eh_o)
    assert np.array_equal(sh.cpu().numpy(), sh_o)


def test_cfg1_edges_first_hit_exact(cfg1):
    robot, env, (qa, qb, ns), w, o = cfg1
    fh_o, _ = o.check_edges(qa, qb, ns, nthreads=NT)
    fh = w.check_edges(qa, qb, ns).cpu().numpy()
    bad = np.flatnonzero(fh != fh_o)
    assert bad.size == 0, (bad[:10], fh[bad[:10]], fh_o[bad[:10]])
    assert (fh_o < 0).any() and (fh_o > 0).any()


def test_cfg1_edges_plain64_exact(cfg1):
    robot, env, (qa, qb, ns), w, o = cfg1
    sel = slice(0, 512)
    fh_o, _ = o.check_edges(qa[sel], qb[sel], ns[sel], nthreads=NT)
    fh = w.check_edges_plain64(qa[sel], qb[sel], ns[sel]).cpu().numpy()
    assert np.array_equal(fh, fh_o)
    # one thread per (edge, step): the same first hits
    fs = w.check_edges_plain64(qa[sel], qb[sel], ns[sel], per_step=True).cpu().numpy()
    assert np.array_equal(fs, fh_o)
    # one thread per (edge, step, query)
    fp = w.check_edges_plain64(qa[sel], qb[sel], ns[sel], per_pair=True).cpu().numpy()
    assert np.array_equal(fp, fh_o)


def test_cfg1_edges_host_and_graph(cfg1):
    import torch
    robot, env, (qa, qb, ns), w, o = cfg1
    ref = w.check_edges(qa, qb, ns).cpu().numpy()
    host = w.check_edges_host(qa, qb, ns)
    assert np.array_equal(host, ref)
    a = torch.as_tensor(qa).cuda()
    b = torch.as_tensor(qb).cuda()
    n = torch.as_tensor(ns).cuda()
    out = torch.empty(len(ns), dtype=torch.int32, device="cuda")
    plan = w.edge_plan(a, b, n, out)
    for _ in range(3):
        out.fill_(-7)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.launch()
        e1.record()
        w.sync()
        assert np.array_equal(out.cpu().numpy(), ref)
        # the main pass's own time, from the events inside the graph, lies
        # within the whole launch's
        main_ms = plan.main_pass_ms()
        assert 0.0 < main_ms <= e0.elapsed_time(e1)
    plan.close()


def test_edge_plan_survives_scratch_growth(cfg1):
    """An edge plan recorded for a small batch keeps working after a larger
    edge batch and a mixed-robot batch have grown the world's scratch."""
    import torch
    robot, env, (qa, qb, ns), w, o = cfg1
    small = slice(0, 100)
    ref = w.check_edges(qa[small], qb[small], ns[small]).cpu().numpy()
    a, b, n = (torch.as_tensor(x[small]).cuda() for x in (qa, qb, ns))
    out = torch.empty(100, dtype=torch.int32, device="cuda")
    plan = w.edge_plan(a, b, n, out)
    plan.launch()
    w.sync()
    assert np.array_equal(out.cpu().numpy(), ref)
    big = np.concatenate([qa] * 3), np.concatenate([qb] * 3), np.concatenate([ns] * 3)
    fh_big = w.check_edges(*big).cpu().numpy()
    assert np.array_equal(fh_big[:len(ns)], w.check_edges(qa, qb, ns).cpu().numpy())
    out.fill_(-7)
    plan.launch()
    w.sync()
    assert np.array_equal(out.cpu().numpy(), ref)
    plan.close()


def test_edges_full_batch_repeatable(built):
    """The full 16,384-edge batch (deep traversals handed between warps at
    the end of every launch) gives the oracle's first hits in each of 42
    launches (14 for each of three edge chunk sizes): hand-over races show
    up as rare, launch-dependent first hits one step late."""
    import torch
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, (qa, qb, ns) = sc.scene_cfg1()
    w = World(env, [robot])
    o = Oracle(robot, env)
    fh_o, _ = o.check_edges(qa, qb, ns, nthreads=NT)
    a, b, n = (torch.as_tensor(x).cuda() for x in (qa, qb, ns))
    for chunk in (8, 16, 32):
        w.set_option("edge_chunk", chunk)
        for _ in range(14):
            fh = w.check_edges(a, b, n).cpu().numpy()
            bad = np.flatnonzero(fh != fh_o)
            assert bad.size == 0, (chunk, bad[:5], fh[bad[:5]], fh_o[bad[:5]])
    w.close()


def test_edges_single_step_and_limits(cfg1):
    """n = 1 edges (two configurations) and an edge leaving the limits."""
    robot, env, (qa, qb, ns), w, o = cfg1
    a = qa[:64].copy()
    b = qb[:64].copy()
    n = np.ones(64, np.int32)
    b[5, 1] = 3.3  # endpoint outside [-pi, pi]
    fh_o, _ = o.check_edges(a, b, n, nthreads=NT)
    fh = w.check_edges(a, b, n).cpu().numpy()
    assert np.array_equal(fh, fh_o)
    assert fh[5] in (0, 1)


def test_bad_step_count_reports_error(cfg1):
    from klampt_gb300._kgpu import KgpuError, KGPU_ERR_INVALID
    robot, env, (qa, qb, ns), w, o = cfg1
    n = ns[:8].copy()
    n[3] = 0
    with pytest.raises(KgpuError) as ei:
        w.check_edges(qa[:8], qb[:8], n)
    assert ei.value.code == KGPU_ERR_INVALID
    # the world stays usable afterwards
    fh = w.check_edges(qa[:8], qb[:8], ns[:8]).cpu().numpy()
    fh_o, _ = o.check_edges(qa[:8], qb[:8], ns[:8])
    assert np.array_equal(fh, fh_o)


def test_nonfinite_config_reports_error(cfg0):
    from klampt_gb300._kgpu import KgpuError, KGPU_ERR_NOT_FINITE
    robot, env, q, w, o = cfg0
    qq = q[:16].copy()
    qq[4, 0] = np.nan
    with pytest.raises(KgpuError) as ei:
        w.check_configs(qq)
    assert ei.value.code == KGPU_ERR_NOT_FINITE
    # the host-buffer calls report the device status with their results, and
    # the world stays usable
    with pytest.raises(KgpuError) as ei:
        w.check_configs_host(qq)
    assert ei.value.code == KGPU_ERR_NOT_FINITE
    qb = q[16:32].copy()
    ns = np.full(16, 5, np.int32)
    with pytest.raises(KgpuError) as ei:
        w.check_edges_host(qq, qb, ns)
    assert ei.value.code == KGPU_ERR_NOT_FINITE
    eo, so, _ = o.check_configs(q[:16], nthreads=NT)
    eh, sh = w.check_configs_host(q[:16])
    assert np.array_equal(eh, eo.astype(bool)) and np.array_equal(sh, so.astype(bool))
    fo, _ = o.check_edges(q[:16], qb, ns, nthreads=NT)
    assert np.array_equal(w.check_edges_host(q[:16], qb, ns), fo)


@pytest.mark.parametrize("per_sm", [2, 3, 4])
def test_every_residency_bit_exact(cfg1, per_sm):
    """Each instantiation of the main pass (2, 3 or 4 blocks per SM: 128, 80
    or 64 registers, more spilled stack at the lower budgets) gives the
    oracle's edge and configuration results."""
    robot, env, (qa, qb, ns), w, o = cfg1
    fh_o, _ = o.check_edges(qa, qb, ns, nthreads=NT)
    eo, so, _ = o.check_configs(qa, nthreads=NT)
    w.set_option("blocks_per_sm", per_sm)
    try:
        assert np.array_equal(w.check_edges(qa, qb, ns).cpu().numpy(), fh_o)
        eh, sh = (x.cpu().numpy() for x in w.check_configs(qa))
        assert np.array_equal(eh, eo) and np.array_equal(sh, so)
    finally:
        w.set_option("blocks_per_sm", 3)


@pytest.mark.parametrize("stage", [256, 1024])
def test_staged_environment_levels_bit_exact(cfg1, stage):
    """With the top levels of the environment tree staged in shared memory
    (stage_nodes, the 2-blocks-per-SM kernels), edges and configurations
    give the oracle's results."""
    robot, env, (qa, qb, ns), w, o = cfg1
    fh_o, _ = o.check_edges(qa, qb, ns, nthreads=NT)
    eo, so, _ = o.check_configs(qa, nthreads=NT)
    w.set_option("blocks_per_sm", 2)
    w.set_option("stage_nodes", stage)
    try:
        assert w.get_option("stage_nodes") == stage
        assert np.array_equal(w.check_edges(qa, qb, ns).cpu().numpy(), fh_o)
        eh, sh = (x.cpu().numpy() for x in w.check_configs(qa))
        assert np.array_equal(eh, eo) and np.array_equal(sh, so)
    finally:
        w.set_option("stage_nodes", 0)
        w.set_option("blocks_per_sm", 3)

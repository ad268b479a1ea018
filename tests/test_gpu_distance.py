"""GPU parity of signed distance, its gradient and the trajectory soft-min
against the FP64 oracle, plus central finite differences (h = 1e-5)."""

import os

import numpy as np
import pytest

from klampt_gb300 import scenes as sc

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 4
GRAD_RTOL = 1e-4


@pytest.fixture(scope="module")
def built():
    from klampt_gb300 import build
    build.build()
    from oracle import oracle_py
    oracle_py.build()
    return True


@pytest.fixture(scope="module")
def cfg2(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg2(T=16, W=8)
    w = World(env, [robot])
    o = Oracle(robot, env)
    yield robot, env, q, w, o
    w.close()


def _grad_close(g, g_ref, rtol=GRAD_RTOL):
    g = np.asarray(g, np.float64)
    g_ref = np.asarray(g_ref, np.float64)
    scale = max(np.abs(g_ref).max(), 1e-6)
    return np.abs(g - g_ref).max() <= rtol * scale + 1e-7


def test_min_distance_matches_oracle(cfg2):
    robot, env, q, w, o = cfg2
    qq = q.reshape(-1, robot.num_links)[:96]
    d_o, p_o, cp_o, g_o = o.min_distance(qq, 1e3, nthreads=NT)
    d, p, cp, g = w.distance(qq, 1e3)
    d, p, cp, g = d.cpu().numpy(), p.cpu().numpy(), cp.cpu().numpy(), g.cpu().numpy()
    assert np.array_equal(p, p_o), np.flatnonzero((p != p_o).any(1))[:5]
    rel = np.abs(d - d_o) / np.maximum(np.abs(d_o), 1e-12)
    assert rel.max() <= 1e-6, (rel.max(), np.argmax(rel))
    nz = d_o != 0
    assert np.allclose(cp[nz], cp_o[nz], rtol=0, atol=1e-9)
    for b in range(len(qq)):
        assert _grad_close(g[b], g_o[b]), (b, g[b], g_o[b])
    assert (d_o < 0).any() and (d_o > 0).any()


def test_min_distance_cutoff_terrain(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg4(n_configs=64, nx=128, ny=256, spacing=0.016)
    w = World(env, [robot])
    o = Oracle(robot, env)
    d_o, p_o, cp_o, g_o = o.min_distance(q, 0.2, nthreads=NT)
    d, p, cp, g = w.distance(q, 0.2)
    d, p, g = d.cpu().numpy(), p.cpu().numpy(), g.cpu().numpy()
    assert np.array_equal(p, p_o)
    assert np.allclose(d, d_o, rtol=1e-6, atol=1e-12)
    for b in range(len(q)):
        assert _grad_close(g[b], g_o[b])
    w.close()


def test_softmin_matches_oracle(cfg2):
    robot, env, q, w, o = cfg2
    qt = q[:4]
    L_o, G_o = o.softmin(qt, 0.01, nthreads=NT)
    L, G = w.softmin(qt, 0.01)
    L, G = L.cpu().numpy(), G.cpu().numpy()
    assert np.allclose(L, L_o, rtol=1e-6, atol=1e-12), (L, L_o)
    for t in range(len(qt)):
        assert _grad_close(G[t], G_o[t]), (t, np.abs(G[t] - G_o[t]).max(), np.abs(G_o[t]).max())


@pytest.mark.parametrize("which", ["arm", "dual_arm", "humanoid"])
def test_self_distance_matches_oracle(built, which):
    """Link-link minimum distance over the enabled self pairs: closest pair
    exact, distance within 1e-6 relative, closest points within 1e-9,
    gradient within 1e-4 of the FP64 oracle; contacts give 0 on the smallest
    colliding pair."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle, self_distance
    robot = {"arm": lambda: sc.arm(7, rings=8, segments=16), "dual_arm": sc.dual_arm,
             "humanoid": sc.humanoid}[which]()
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    w = World(env, [robot])
    o = Oracle(robot, env)
    rng = np.random.default_rng(51)
    # configurations scaled towards zero by a random factor: a mix of
    # contacts and separated links (uniform humanoid configurations all
    # self-collide)
    q = (sc.uniform_configs(robot, 256, rng) * rng.uniform(0, 1, (256, 1))).astype(np.float32)
    d_o, p_o, cp_o, g_o = self_distance(o, q, cutoff=1e3, nthreads=NT)
    d, p, cp, g = (x.cpu().numpy() for x in w.self_distance(q, 1e3))
    assert np.array_equal(p, p_o), np.flatnonzero((p != p_o).any(1))[:5]
    rel = np.abs(d - d_o) / np.maximum(np.abs(d_o), 1e-12)
    assert rel.max() <= 1e-6, (rel.max(), np.argmax(rel))
    assert np.array_equal(d == 0, d_o == 0)
    nz = d_o != 0
    assert np.allclose(cp[nz], cp_o[nz], rtol=0, atol=1e-9)
    assert (cp[~nz] == 0).all()
    for b in range(len(q)):
        assert _grad_close(g[b], g_o[b]), (b, g[b], g_o[b])
    assert nz.any()
    # cutoff below most distances: (cutoff, -1, -1) where nothing is closer
    c = float(np.quantile(d_o[nz], 0.3))
    d_c, p_c, _, _ = self_distance(o, q, cutoff=c, nthreads=NT)
    d2, p2, _, g2 = (x.cpu().numpy() if x is not None else None for x in w.self_distance(q, c, want_grad=False))
    assert g2 is None
    assert np.array_equal(p2, p_c) and np.allclose(d2, d_c, rtol=1e-6, atol=0)
    assert (p_c[:, 0] < 0).any() and (p_c[:, 0] >= 0).any()
    w.close()


def test_self_distance_finite_differences(built):
    """d/dq of the self distance against central differences of the oracle
    (h = 1e-3 on FP32 configurations, where the closest pair is unchanged)."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle, self_distance
    robot = sc.arm(7, rings=8, segments=16)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    w = World(env, [robot])
    o = Oracle(robot, env)
    q = sc.uniform_configs(robot, 32, np.random.default_rng(52))
    d, p, _, g = (x.cpu().numpy() for x in w.self_distance(q, 1e3))
    h = 1e-3
    checked = 0
    for b in np.flatnonzero(d > 1e-2)[:12]:
        for k in range(robot.num_links):
            qp, qm = q[b].copy(), q[b].copy()
            qp[k] += h
            qm[k] -= h
            dp, pp, _, _ = self_distance(o, qp[None], cutoff=1e3)
            dm, pm, _, _ = self_distance(o, qm[None], cutoff=1e3)
            if tuple(pp[0]) != tuple(p[b]) or tuple(pm[0]) != tuple(p[b]):
                continue
            fd = (dp[0] - dm[0]) / (float(qp[k]) - float(qm[k]))
            assert abs(fd - g[b, k]) <= 2e-2 * max(1.0, abs(g[b, k])), (b, k, fd, g[b, k])
            checked += 1
    assert checked > 20
    w.close()


def test_self_distance_empty_and_errors(built):
    from klampt_gb300.engine import World
    robot = sc.arm(3, rings=4, segments=8)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    w = World(env, [robot])
    d, p, cp, g = w.self_distance(np.zeros((0, 3), np.float32), 1.0)
    assert d.shape == (0,) and p.shape == (0, 2)
    with pytest.raises(Exception):
        w.self_distance(np.zeros((4, 3), np.float32), -1.0)
    with pytest.raises(Exception):
        w.self_distance(np.zeros((4, 3), np.float32), float("nan"))
    w.close()


def test_self_pair_distances_matches_oracle(built):
    """Every queried pair's own minimum bit for bit (enabled pairs, and every
    pair with geometry), unqueried pairs -1, and the sampled per-pair minima
    and maxima of RandomizedSelfCollisionDistances."""
    from klampt_gb300.engine import World
    from klampt_gb300 import klampt as kl
    from oracle.oracle_py import Oracle, self_pair_distances
    robot = sc.dual_arm()
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    w = World(env, [robot])
    o = Oracle(robot, env)
    rng = np.random.default_rng(53)
    q = (sc.uniform_configs(robot, 128, rng) * rng.uniform(0, 1, (128, 1))).astype(np.float32)
    for all_pairs in (False, True):
        for cutoff in (1e3, 0.2):
            dp_o = self_pair_distances(o, q, cutoff=cutoff, nthreads=NT, all_pairs=all_pairs)
            dp = w.self_pair_distances(q, cutoff, all_pairs=all_pairs).cpu().numpy()
            assert np.array_equal(dp, dp_o), (all_pairs, np.argwhere(dp != dp_o)[:5])
        assert (dp_o == 0).any() and (dp_o == 0.2).any() and ((dp_o > 0) & (dp_o < 0.2)).any()
        assert (dp_o < 0).any() != all_pairs
    w.close()
    wm = kl.WorldModel([robot], env)
    lo, hi = kl.RandomizedSelfCollisionDistances(wm.robot(0), 64, seed=3)
    Q = kl._sample_configs(wm.robot(0), 64, np.random.default_rng(3))
    ref = self_pair_distances(o, Q, cutoff=1e3, nthreads=NT, all_pairs=True)
    L = robot.num_links
    iu, ju = np.triu_indices(L, 1)
    ok = (ref >= 0).all(0)
    assert ok.all()
    assert np.array_equal(lo[iu, ju], ref.min(0)) and np.array_equal(lo[ju, iu], ref.min(0))
    assert np.array_equal(hi[iu, ju], ref.max(0)) and np.array_equal(hi[ju, iu], ref.max(0))
    assert (np.diag(lo) == 0).all() and (np.diag(hi) == 0).all()
    wm.close()


def test_self_min_distance_autograd(built):
    """The autograd Function's backward applies the kernel's gradient."""
    import torch
    from klampt_gb300.autodiff import SelfMinDistance
    from klampt_gb300.engine import World
    robot = sc.arm(7, rings=8, segments=16)
    env = sc.env_from_objects("far", [sc.box_mesh((9, 9, 9), (0.1, 0.1, 0.1))])
    w = World(env, [robot])
    rng = np.random.default_rng(54)
    q = (sc.uniform_configs(robot, 64, rng) * rng.uniform(0, 1, (64, 1))).astype(np.float32)
    d_ref, _, _, g_ref = w.self_distance(q, 1e3)
    qt = torch.tensor(q, device="cuda", requires_grad=True)
    d = SelfMinDistance.apply(qt, w, 1e3)
    assert torch.allclose(d.detach(), d_ref, rtol=1e-12, atol=0)
    (2.0 * d).sum().backward()
    assert torch.allclose(qt.grad, 2.0 * g_ref)
    w.close()

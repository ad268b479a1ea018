"""GPU parity at the workloads' stated sizes, against the FP64 oracle:

* collision margins (links and objects) on the box scene and the icosphere
  field, configuration batches and edges, both FP64 placements;
* the heterogeneous four-robot batch on the full 1M-triangle scene;
* clamped signed distance with gradient on the full 512 x 1024 terrain;
* the trajectory soft-min on 64 trajectories x 32 waypoints, and central
  finite differences (h = 1e-5) of all 64 x 32 x 7 gradient entries, where the
  only entries left out are those whose closest feature pair switches inside
  +-h (found by the oracle, listed, not a tolerated fraction).
"""

import os

import numpy as np
import pytest

from klampt_gb300 import scenes as sc

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 4
TAU = 0.01
GRAD_RTOL = 1e-4   # gradient error relative to the largest entry of its trajectory / configuration
DIST_RTOL = 1e-6   # distance and soft-min relative error


@pytest.fixture(scope="module")
def built():
    from klampt_gb300 import build
    build.build()
    from oracle import oracle_py
    oracle_py.build()
    return True


def _grad_close(g, g_ref, rtol=GRAD_RTOL):
    g = np.asarray(g, np.float64)
    g_ref = np.asarray(g_ref, np.float64)
    scale = max(np.abs(g_ref).max(), 1e-6)
    return np.abs(g - g_ref).max() <= rtol * scale + 1e-7


# ---------------------------------------------------------------------------
# margins
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("scene", ["boxes", "icospheres"])
def test_margins_bit_exact(built, scene):
    """Link margins and object margins in [0.01, 0.05] m: every verdict of a
    configuration batch (FP64 deferred and inline) and every edge's first hit
    equal the oracle's, which decides dist <= m_a + m_b in FP64."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    rng = np.random.default_rng(77)
    if scene == "boxes":
        robot, env, q = sc.scene_cfg0()
        n_edges = 512
    else:
        robot, env, _ = sc.scene_cfg1(n_edges=2)
        q = sc.uniform_configs(robot, 4096, rng)
        n_edges = 1024
    robot.margins = rng.uniform(0.01, 0.05, robot.num_links)
    env.margins = rng.uniform(0.01, 0.05, env.num_objects)
    # the base link never moves: objects within reach of its margin would
    # make every configuration collide, so those keep margin 0 (and so does
    # the base link)
    robot.margins[0] = 0.0
    base_lo, base_hi = np.array([-0.05, -0.05, 0.0]), np.array([0.05, 0.05, 0.3])
    for k, (V, _) in enumerate(env.meshes):
        gap = np.maximum(0.0, np.maximum(V.min(0) - base_hi, base_lo - V.max(0)))
        if np.linalg.norm(gap) < 0.15:
            env.margins[k] = 0.0
    w = World(env, [robot])
    o = Oracle(robot, env)
    eo, so, _ = o.check_configs(q, nthreads=NT)
    # margins widen contacts: more configurations collide than without
    e0, s0, _ = Oracle(sc.scene_cfg0()[0] if scene == "boxes" else sc.arm(7, rings=32),
                       env.__class__(env.name, env.meshes, env.groups, env.convex)).check_configs(q, nthreads=NT)
    assert eo.sum() > e0.sum() and so.sum() > s0.sum()
    for fp64_inline in (0, 1):
        w.set_option("fp64_inline", fp64_inline)
        eh, sh = (x.cpu().numpy() for x in w.check_configs(q))
        assert np.array_equal(eh, eo), (scene, fp64_inline, np.flatnonzero(eh != eo)[:8])
        assert np.array_equal(sh, so), (scene, fp64_inline, np.flatnonzero(sh != so)[:8])
        f = w.is_feasible(q).cpu().numpy()
        assert np.array_equal(f, o.is_feasible(q, nthreads=NT))
    w.set_option("fp64_inline", -1)
    qa, qb, ns = sc.random_edges(robot, n_edges, np.random.default_rng(78))
    fh = w.check_edges(qa, qb, ns).cpu().numpy()
    fh_o, _ = o.check_edges(qa, qb, ns, nthreads=NT)
    assert np.array_equal(fh, fh_o), np.flatnonzero(fh != fh_o)[:8]
    assert (fh_o >= 0).any() and (fh_o < 0).any()
    w.close()


# ---------------------------------------------------------------------------
# heterogeneous batch, full 1M-triangle scene
# ---------------------------------------------------------------------------

def test_hetero_full_scene(built):
    """All 65,536 configurations of the four robots in one launch on the full
    1.0M-triangle scene; 4,096 of them (stratified by robot) checked against
    each robot's oracle, for both FP64 placements."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robots, env, (ids, q) = sc.scene_cfg3()
    assert env.num_tris >= 1_000_000 and len(ids) == 65536
    w = World(env, robots)
    rng = np.random.default_rng(79)
    ref = []
    for r, spec in enumerate(robots):
        members = np.flatnonzero(ids == r)
        sel = np.sort(rng.choice(members, 1024, replace=False))
        eo, so, _ = Oracle(spec, env).check_configs(q[sel, :spec.num_links], nthreads=NT)
        ref.append((sel, eo, so))
    for fp64_inline in (0, 1):
        w.set_option("fp64_inline", fp64_inline)
        eh, sh = (x.cpu().numpy() for x in w.check_configs_multi(ids, q))
        for r, (sel, eo, so) in enumerate(ref):
            assert np.array_equal(eh[sel], eo), (fp64_inline, r, np.flatnonzero(eh[sel] != eo)[:8])
            assert np.array_equal(sh[sel], so), (fp64_inline, r, np.flatnonzero(sh[sel] != so)[:8])
    # the 1M-triangle field (8,700 boxes and 700 spheres in a 2 m cube) meets
    # every sampled configuration; the self verdicts are mixed
    allo = np.concatenate([x[2] for x in ref])
    assert 0 < allo.mean() < 1
    w.close()


# ---------------------------------------------------------------------------
# clamped signed distance on the full terrain
# ---------------------------------------------------------------------------

def test_min_distance_full_terrain(built):
    """Clamped signed distance (cutoff 0.2 m) with d/dq on the 512 x 1024
    terrain (1,045,506 triangles) plus 500 boxes: 2,048 configurations, the
    closest (link, object) pair identical, d within 1e-6 relative, closest
    points within 1e-9 m, gradient within 1e-4."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg4(n_configs=2048)
    assert env.meshes[0][1].shape[0] == 2 * 511 * 1023
    w = World(env, [robot])
    o = Oracle(robot, env)
    d_o, p_o, cp_o, g_o = o.min_distance(q, 0.2, nthreads=NT)
    d, p, cp, g = (x.cpu().numpy() for x in w.distance(q, 0.2))
    assert np.array_equal(p, p_o), np.flatnonzero((p != p_o).any(1))[:8]
    rel = np.abs(d - d_o) / np.maximum(np.abs(d_o), 1e-12)
    assert rel.max() <= DIST_RTOL, (rel.max(), int(np.argmax(rel)))
    hit = p_o[:, 0] >= 0
    nz = hit & (d_o != 0)
    assert np.allclose(cp[nz], cp_o[nz], rtol=0, atol=1e-9)
    bad = [b for b in range(len(q)) if not _grad_close(g[b], g_o[b])]
    assert not bad, bad[:8]
    # among the 500 boxes in the 2 m cube every configuration has an obstacle
    # within the cutoff (most are in contact); the closest is always a box
    assert (d_o < 0).any()
    # the terrain alone (links masked to group 1): every closest pair is the
    # 1M-triangle terrain, parity as above
    from oracle.oracle_py import default_masks
    masks = default_masks(robot, env) & np.uint32(1 << 1)
    for l in range(robot.num_links):
        w.set_link_env_mask(0, l, int(masks[l]))
    o_t = Oracle(robot, env, masks=masks)
    d_o, p_o, cp_o, g_o = o_t.min_distance(q, 0.2, nthreads=NT)
    d, p, cp, g = (x.cpu().numpy() for x in w.distance(q, 0.2))
    assert np.array_equal(p, p_o), np.flatnonzero((p != p_o).any(1))[:8]
    rel = np.abs(d - d_o) / np.maximum(np.abs(d_o), 1e-12)
    assert rel.max() <= DIST_RTOL, (rel.max(), int(np.argmax(rel)))
    nz = (p_o[:, 0] >= 0) & (d_o != 0)
    assert np.allclose(cp[nz], cp_o[nz], rtol=0, atol=1e-9)
    bad = [b for b in range(len(q)) if not _grad_close(g[b], g_o[b])]
    assert not bad, bad[:8]
    # terrain pairs within the cutoff, and clamped configurations
    assert (p_o[:, 1] == 0).sum() > 50 and nz.any() and (p_o[:, 0] < 0).any()
    w.close()


# ---------------------------------------------------------------------------
# soft-min, 64 trajectories x 32 waypoints
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def cfg2_64(built):
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg2(T=64, W=32)
    w = World(env, [robot])
    o = Oracle(robot, env)
    yield robot, env, q, w, o
    w.close()


def test_softmin_64x32_matches_oracle(cfg2_64):
    robot, env, q, w, o = cfg2_64
    L_o, G_o = o.softmin(q, TAU, nthreads=NT)
    L, G = (x.cpu().numpy() for x in w.softmin(q, TAU))
    rel = np.abs(L - L_o) / np.maximum(np.abs(L_o), 1e-12)
    assert rel.max() <= DIST_RTOL, (rel.max(), int(np.argmax(rel)))
    bad = [t for t in range(len(q)) if not _grad_close(G[t], G_o[t])]
    assert not bad, bad[:8]


def _feature_set(o, qw, bound):
    feats, _ = o.pair_features(qw, bound)
    return {(int(r[0]), int(r[1])): (int(r[2]), int(r[3]), int(r[4])) for r in feats}


def test_softmin_finite_differences_64x32(cfg2_64):
    """Central differences (h = 1e-5) of the soft-min against the adjoint
    gradient on every entry of 64 trajectories x 32 waypoints x 7 joints.
    An entry may miss 1e-4 only where the oracle shows that a pair's closest
    feature (triangle pair, or vertex/face of a penetration) differs between
    q - h, q and q + h, i.e. the central difference straddles a kink."""
    robot, env, q, w, o = cfg2_64
    T, Wn, L = q.shape
    _, G = w.softmin(q, TAU)
    G = G.cpu().numpy().astype(np.float64)
    h = 1e-5
    plus = np.repeat(q[:, None, None], Wn * L, axis=1).reshape(T, Wn, L, Wn, L).copy()
    minus = plus.copy()
    steps = np.zeros((T, Wn, L))
    for wp in range(Wn):
        for j in range(L):
            plus[:, wp, j, wp, j] = (q[:, wp, j].astype(np.float64) + h).astype(np.float32)
            minus[:, wp, j, wp, j] = (q[:, wp, j].astype(np.float64) - h).astype(np.float32)
            steps[:, wp, j] = plus[:, wp, j, wp, j].astype(np.float64) - minus[:, wp, j, wp, j]
    Lp, _ = w.softmin(plus.reshape(T * Wn * L, Wn, L), TAU, want_grad=False)
    Lm, _ = w.softmin(minus.reshape(T * Wn * L, Wn, L), TAU, want_grad=False)
    fd = ((Lp.cpu().numpy() - Lm.cpu().numpy()).reshape(T, Wn, L)) / steps
    scale = np.maximum(np.abs(G).reshape(T, -1).max(1), 1e-6)[:, None, None]
    err = np.abs(fd - G) / scale
    failing = np.argwhere(err > GRAD_RTOL)
    # explain every failing entry by a feature switch inside +-h
    unexplained = []
    m_traj = {}
    for t, wp, j in failing:
        if t not in m_traj:
            d_o, _, _, _ = o.min_distance(q[t], 1e3, want_grad=False)
            m_traj[t] = float(d_o.min())
        bound = m_traj[t] + 31 * TAU
        base = _feature_set(o, q[t, wp], bound)
        fp = _feature_set(o, plus[t, wp, j, wp], bound)
        fm = _feature_set(o, minus[t, wp, j, wp], bound)
        common = set(base) & set(fp) & set(fm)
        if not any(base[k] != fp[k] or base[k] != fm[k] for k in common):
            unexplained.append((int(t), int(wp), int(j), float(err[t, wp, j])))
    assert not unexplained, unexplained[:8]
    # the kinks are a small set (a sanity check on the test, not a tolerance)
    assert len(failing) <= 0.02 * err.size, (len(failing), err.size)


def test_penetration_gradient_finite_differences(built):
    """Penetrating configurations of the box field (d < 0: a link vertex
    inside a convex box, depth to the box's nearest face plane): central
    differences (h = 1e-5 on FP32 joint values) of the engine's distance
    against its d/dq, every entry where the oracle shows the same deciding
    feature (link, box, vertex, face) at q - h, q and q + h."""
    from klampt_gb300.engine import World
    from oracle.oracle_py import Oracle
    robot, env, q = sc.scene_cfg4(n_configs=256, nx=64, ny=64, spacing=0.032)
    w = World(env, [robot])
    o = Oracle(robot, env)
    d, p, _, g = (x.cpu().numpy() for x in w.distance(q, 0.2))
    pen = np.flatnonzero(d < -1e-4)[:48]
    assert len(pen) >= 24
    L = robot.num_links
    h = 1e-5
    checked = 0
    for b in pen:
        qp = np.repeat(q[b][None], L, 0)
        qm = qp.copy()
        for j in range(L):
            qp[j, j] = np.float32(q[b, j] + h)
            qm[j, j] = np.float32(q[b, j] - h)
        dp, pp, _, _ = (x.cpu().numpy() for x in w.distance(qp, 0.2))
        dm, pm, _, _ = (x.cpu().numpy() for x in w.distance(qm, 0.2))
        base = o.pair_features(q[b], 0.0)
        for j in range(L):
            if tuple(pp[j]) != tuple(p[b]) or tuple(pm[j]) != tuple(p[b]):
                continue
            fp, fm = o.pair_features(qp[j], 0.0), o.pair_features(qm[j], 0.0)
            key = lambda F: {(int(r[0]), int(r[1])): tuple(int(x) for x in r[2:]) for r in F[0]}
            kb, kp, km = key(base), key(fp), key(fm)
            pair = (int(p[b, 0]), int(p[b, 1]))
            if kb.get(pair) != kp.get(pair) or kb.get(pair) != km.get(pair):
                continue  # the deciding vertex or face switches inside +-h
            fd = (dp[j] - dm[j]) / (float(qp[j, j]) - float(qm[j, j]))
            assert abs(fd - g[b, j]) <= 1e-4 * max(np.abs(g[b]).max(), 1e-6) + 1e-7, (b, j, fd, g[b, j])
            checked += 1
    assert checked >= 100
    w.close()

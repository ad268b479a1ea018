"""The canonical FP64 triangle predicate (kx_tri_tri_overlap: 17-axis
separating-axis test, touching = contact, the restatement of PQP's
TriContact) against an independent exact method (oracle/exact_tri.cpp:
feasibility of the barycentric intersection system in integer arithmetic).

Over 10^6 integer triangle pairs built to hit the degenerate cases where
implementations differ — coplanar pairs, shared edges, shared vertices, a
vertex on a face or an edge, crossing edges that exactly touch — the FP64
predicate evaluates exactly (|coordinates| <= 1024 keep every product below
2^53), so it must agree with the exact test on every pair of non-degenerate
triangles.  Zero-area triangles are reported apart: the separating-axis set
loses its normals there (the listed disagreements are all of that kind).
Rotated copies of pairs whose verdict is robust under a quarter-unit shift
then check the predicate on general FP64 inputs."""

import os

import numpy as np

NT = os.cpu_count() or 4


def _unimodular(rng, n):
    """n random integer 3x3 matrices with determinant +-1 (products of
    elementary shears and a permutation), entries small."""
    M = np.tile(np.eye(3, dtype=np.int64), (n, 1, 1))
    for _ in range(3):
        i = rng.integers(0, 3, n)
        j = (i + rng.integers(1, 3, n)) % 3
        k = rng.integers(-1, 2, n)
        E = np.tile(np.eye(3, dtype=np.int64), (n, 1, 1))
        E[np.arange(n), i, j] = k
        M = E @ M
    perm = np.array([rng.permutation(3) for _ in range(n)])
    return M[np.arange(n)[:, None], perm]


def _apply(M, T):
    return np.einsum("nij,nkj->nki", M, T.reshape(-1, 3, 3)).reshape(-1, 9)


def _pairs(rng, n_each):
    """(P, Q, label) integer triangle pairs of the degenerate families."""
    out = []

    def add(P, Q, label):
        out.append((np.asarray(P, np.int64).reshape(-1, 9), np.asarray(Q, np.int64).reshape(-1, 9), label))

    n = n_each
    # small lattices: many coincidences of every kind
    add(rng.integers(-2, 3, (n, 9)), rng.integers(-2, 3, (n, 9)), "lattice5")
    add(rng.integers(-4, 5, (n, 9)), rng.integers(-4, 5, (n, 9)), "lattice9")
    # coplanar pairs in z = 0, then in slanted integer planes
    P = rng.integers(-6, 7, (n, 3, 3)); P[:, :, 2] = 0
    Q = rng.integers(-6, 7, (n, 3, 3)); Q[:, :, 2] = 0
    add(P, Q, "coplanar_z0")
    M = _unimodular(rng, n)
    add(_apply(M, P), _apply(M, Q), "coplanar_slanted")
    # shared edge (same and opposite orientation), shared vertex
    P = rng.integers(-8, 9, (n, 9))
    Q = rng.integers(-8, 9, (n, 9))
    Q[:, 0:3], Q[:, 3:6] = P[:, 0:3], P[:, 3:6]
    add(P, Q, "shared_edge")
    Q2 = Q.copy(); Q2[:, 0:3], Q2[:, 3:6] = P[:, 3:6], P[:, 0:3]
    add(P, Q2, "shared_edge_reversed")
    Q3 = rng.integers(-8, 9, (n, 9))
    Q3[:, 0:3] = P[np.arange(n)[:, None], 3 * (np.arange(n) % 3)[:, None] + np.arange(3)[None]]
    add(P, Q3, "shared_vertex")
    # a vertex of Q on P's face, on P's edge, or at a lattice point next to
    # it; P = (0,0,0), (2a,0,0), (0,2b,0) under a unimodular map
    a = rng.integers(1, 6, n); b = rng.integers(1, 6, n)
    P = np.zeros((n, 3, 3), np.int64); P[:, 1, 0] = 2 * a; P[:, 2, 1] = 2 * b
    u = rng.integers(0, 2 * a + 1); v = (rng.integers(0, 2 * b + 1))
    tip = np.stack([u, v, rng.integers(-1, 2, n)], 1)
    Q = rng.integers(-8, 9, (n, 3, 3)); Q[:, 0] = tip
    M = _unimodular(rng, n)
    add(_apply(M, P), _apply(M, Q), "vertex_on_face")
    # crossing edges at heights -1, 0 (touching) and +1
    c = rng.integers(-1, 2, n)
    ea = rng.integers(1, 7, n); eb = rng.integers(1, 7, n)
    P = np.zeros((n, 3, 3), np.int64); P[:, 0, 0] = -ea; P[:, 1, 0] = ea
    P[:, 2] = np.stack([rng.integers(-6, 7, n), rng.integers(-6, 7, n), rng.integers(-6, -1, n)], 1)
    Q = np.zeros((n, 3, 3), np.int64); Q[:, 0, 1] = -eb; Q[:, 1, 1] = eb; Q[:, 0, 2] = c; Q[:, 1, 2] = c
    Q[:, 2] = np.stack([rng.integers(-6, 7, n), rng.integers(-6, 7, n), c + rng.integers(1, 6, n)], 1)
    M = _unimodular(rng, n)
    add(_apply(M, P), _apply(M, Q), "edge_cross")
    # large coordinates: Q a translate of P by a short lattice vector
    P = rng.integers(-900, 901, (n, 9))
    add(P, P + np.tile(rng.integers(-3, 4, (n, 3)), 3) + rng.integers(-1, 2, (n, 9)), "large_near")
    return out


def _nondegenerate(T):
    T = T.reshape(-1, 3, 3)
    n = np.cross(T[:, 1] - T[:, 0], T[:, 2] - T[:, 0])
    return (n != 0).any(1)


def test_exact_method_known_answers():
    from oracle.oracle_py import tri_tri_exact
    P = np.array([[0, 0, 0, 4, 0, 0, 0, 4, 0]] * 6)
    Q = np.array([
        [1, 1, -1, 1, 1, 5, 2, 1, 5],    # pierces the face
        [1, 1, 0, 1, 1, 5, 2, 1, 5],     # vertex on the face
        [1, 1, 1, 1, 1, 5, 2, 1, 5],     # above it
        [4, 0, 0, 9, 9, 9, 9, 0, 9],     # shares a vertex
        [2, 2, 0, 5, 5, 0, 2, 5, 0],     # coplanar, touching at (2, 2, 0) on the hypotenuse
        [3, 3, 0, 5, 5, 0, 2, 5, 0],     # coplanar, apart
    ])
    assert tri_tri_exact(P, Q).tolist() == [1, 1, 0, 1, 1, 0]


def test_fp64_predicate_matches_exact_on_a_million_degenerate_pairs():
    from oracle.oracle_py import tri_tri_batch, tri_tri_exact
    rng = np.random.default_rng(4242)
    families = _pairs(rng, 112_000)
    total = 0
    report = {}
    for P, Q, label in families:
        ex = tri_tri_exact(P, Q, nthreads=NT)
        fp = tri_tri_batch(P.astype(np.float64), Q.astype(np.float64))
        good = _nondegenerate(P) & _nondegenerate(Q)
        bad = np.flatnonzero(good & (ex != fp))
        assert bad.size == 0, (label, [(P[i].tolist(), Q[i].tolist(), int(ex[i]), int(fp[i])) for i in bad[:4]])
        if label.startswith("shared"):
            assert ex.all(), label      # a shared vertex or edge is a contact
        else:
            assert 0 < ex[good].mean() < 1, label  # both answers occur
        deg = np.flatnonzero(~good & (ex != fp))
        report[label] = (int(good.sum()), int((~good).sum()), int(deg.size), int((fp[deg] == 1).sum()))
        total += int(good.sum())
    assert total >= 1_000_000, total
    # zero-area triangles: the only disagreements, and always "contact"
    # reported for a pair that is apart (the normals vanish, so fewer axes
    # can separate), never a missed contact
    for label, (_, _, ndeg, nfp1) in report.items():
        assert nfp1 == ndeg, (label, report[label])


def test_fp64_predicate_on_rotated_robust_pairs():
    """General FP64 inputs: lattice pairs whose exact verdict survives every
    quarter-unit shift of Q (scaled by 4, shifted by +-1 along each axis)
    keep it under a random rotation, evaluated by the FP64 predicate."""
    from oracle.oracle_py import tri_tri_batch, tri_tri_exact
    rng = np.random.default_rng(4343)
    P = rng.integers(-60, 61, (60_000, 9)) * 4
    Q = P + np.tile(rng.integers(-40, 41, (60_000, 3)), 3) + rng.integers(-30, 31, (60_000, 9))
    Q = np.clip(Q, -1024, 1024)
    base = tri_tri_exact(P, Q, nthreads=NT)
    robust = np.ones(len(P), bool)
    for ax in range(3):
        for s in (-1, 1):
            sh = np.zeros(9, np.int64); sh[ax::3] = s
            robust &= tri_tri_exact(P, Q + sh, nthreads=NT) == base
    keep = np.flatnonzero(robust & _nondegenerate(P) & _nondegenerate(Q))
    assert len(keep) > 20_000 and 0.1 < base[keep].mean() < 0.9
    A = rng.normal(size=(len(keep), 3, 3))
    R, _ = np.linalg.qr(A)
    t = rng.uniform(-50, 50, (len(keep), 1, 3))
    Pr = (np.einsum("nij,nkj->nki", R, P[keep].reshape(-1, 3, 3) / 4.0) + t).reshape(-1, 9)
    Qr = (np.einsum("nij,nkj->nki", R, Q[keep].reshape(-1, 3, 3) / 4.0) + t).reshape(-1, 9)
    fp = tri_tri_batch(Pr, Qr)
    assert np.array_equal(fp, base[keep]), np.flatnonzero(fp != base[keep])[:8]

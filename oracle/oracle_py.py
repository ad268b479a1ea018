"""ctypes driver of the FP64 CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py`` as the checker.  The engine never
imports this module.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compiles the oracle (make in oracle/); returns the library path."""
    srcs = [os.path.join(HERE, f) for f in ("oracle.cpp", "exact_tri.cpp", "Makefile")]
    srcs.append(os.path.join(HERE, "..", "include", "kgpu_exact.h"))
    stale = (not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(f) for f in srcs))
    if force or stale:
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "all"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.orc_robot_create.restype = P
        L.orc_env_create.restype = P
        for name in ("orc_check_configs", "orc_check_edges", "orc_is_feasible", "orc_pair_distance",
                     "orc_min_distance", "orc_softmin", "orc_tri_tri", "orc_raycast", "orc_jacobian", "orc_self_pairs", "orc_ik",
                     "orc_indep_pairs", "orc_self_distance", "orc_self_pair_distances", "orc_pair_features", "orc_tri_tri_batch",
                     "orc_tri_tri_exact", "orc_geom_collide", "orc_geom_distance"):
            getattr(L, name).restype = ctypes.c_int
        L.orc_robot_destroy.argtypes = [P]
        L.orc_env_destroy.argtypes = [P]
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def default_masks(robot_spec, env_spec) -> np.ndarray:
    """Klamp't default masks (PlannerSettings.cpp:16-42): every link against
    rigid objects (group 0) and other groups, links with parent -1 not
    against terrains (group 1)."""
    L = robot_spec.num_links
    m = np.full(ORC_MAXL, 0xFFFFFFFF, dtype=np.uint32)
    for i in range(L):
        if int(robot_spec.parents[i]) < 0:
            m[i] &= np.uint32(~(1 << 1) & 0xFFFFFFFF)
    return m


ORC_MAXL = 32


class Oracle:
    """FP64 oracle over one robot and one environment."""

    def __init__(self, robot_spec, env_spec, masks: Optional[np.ndarray] = None):
        L = lib()
        self.robot_spec = robot_spec
        self.env_spec = env_spec
        self.nl = robot_spec.num_links
        r = robot_spec.packed()
        self._keep = [r]
        self.robot = L.orc_robot_create(
            ctypes.c_int(self.nl), _p(r["parents"]), _p(r["joint_types"]), _p(r["T0_parent"]),
            _p(r["axes"]), _p(r["qmin"]), _p(r["qmax"]), _p(r["vert_offset"]), _p(r["verts"]),
            _p(r["tri_offset"]), _p(r["tris"]), _p(r["margins"]), _p(r["self_mask"]))
        self.env = None
        if env_spec is not None:
            e = env_spec.packed()
            self._keep.append(e)
            self.env = L.orc_env_create(
                ctypes.c_int(env_spec.num_objects), _p(e["vert_offset"]), _p(e["verts"]),
                _p(e["tri_offset"]), _p(e["tris"]), _p(e["groups"]), _p(e["convex"]),
                _p(e["margins"]))
        self.masks = np.ascontiguousarray(
            masks if masks is not None else default_masks(robot_spec, env_spec), dtype=np.uint32)

    def close(self):
        L = lib()
        if self.robot:
            L.orc_robot_destroy(ctypes.c_void_p(self.robot))
            self.robot = None
        if self.env:
            L.orc_env_destroy(ctypes.c_void_p(self.env))
            self.env = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fk(self, q) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float64)
        T = np.empty((self.nl, 12), np.float64)
        lib().orc_fk(ctypes.c_void_p(self.robot), _p(q), _p(T))
        return T

    def check_configs(self, q, nthreads: int = 1, want_env=True, want_self=True):
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, self.nl)
        B = q.shape[0]
        env_hit = np.zeros(B, np.uint8) if want_env else None
        self_hit = np.zeros(B, np.uint8) if want_self else None
        cnt = np.zeros(3, np.int64)
        lib().orc_check_configs(ctypes.c_void_p(self.robot), ctypes.c_void_p(self.env), _p(self.masks),
                                _p(q), ctypes.c_int(B), _p(env_hit), _p(self_hit),
                                ctypes.c_int(nthreads), _p(cnt))
        return env_hit, self_hit, cnt

    def check_configs_brute(self, q):
        """Verdicts by testing every triangle pair (no BVH culling)."""
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, self.nl)
        B = q.shape[0]
        eh = np.zeros(B, np.uint8)
        sh = np.zeros(B, np.uint8)
        lib().orc_check_configs_brute(ctypes.c_void_p(self.robot), ctypes.c_void_p(self.env), _p(self.masks),
                                      _p(q), ctypes.c_int(B), _p(eh), _p(sh))
        return eh, sh

    def is_feasible(self, q, nthreads: int = 1) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, self.nl)
        out = np.zeros(q.shape[0], np.uint8)
        lib().orc_is_feasible(ctypes.c_void_p(self.robot), ctypes.c_void_p(self.env), _p(self.masks),
                              _p(q), ctypes.c_int(q.shape[0]), _p(out), ctypes.c_int(nthreads))
        return out

    def check_edges(self, qa, qb, nsteps, nthreads: int = 1):
        qa = np.ascontiguousarray(qa, dtype=np.float32).reshape(-1, self.nl)
        qb = np.ascontiguousarray(qb, dtype=np.float32).reshape(-1, self.nl)
        ns = np.ascontiguousarray(nsteps, dtype=np.int32)
        E = qa.shape[0]
        out = np.zeros(E, np.int32)
        cnt = np.zeros(3, np.int64)
        lib().orc_check_edges(ctypes.c_void_p(self.robot), ctypes.c_void_p(self.env), _p(self.masks),
                              _p(qa), _p(qb), _p(ns), ctypes.c_int(E), _p(out),
                              ctypes.c_int(nthreads), _p(cnt))
        return out, cnt

    def pair_distance(self, q, link: int, obj: int, bound: float = 1e300):
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(self.nl)
        out = np.zeros(10, np.float64)
        feat = np.zeros(3, np.int32)
        found = lib().orc_pair_distance(ctypes.c_void_p(self.robot), ctypes.c_void_p(self.env), _p(q),
                                        ctypes.c_int(link), ctypes.c_int(obj), ctypes.c_double(bound),
                                        _p(out), _p(feat))
        return dict(found=bool(found), d=out[0], cp=out[1:4], cq=out[4:7], dir=out[7:10],
                    feat=feat[:2].copy(), signed=bool(feat[2]))

    def pair_features(self, q, bound: float, max_pairs: int = 4096):
        """Enabled (link, object) pairs of configuration q closer than
        `bound`: int array [n, 5] of (link, object, feature a, feature b,
        signed flag) and their distances [n]."""
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(self.nl)
        out = np.zeros((max_pairs, 5), np.int32)
        dist = np.zeros(max_pairs, np.float64)
        n = lib().orc_pair_features(ctypes.c_void_p(self.robot), ctypes.c_void_p(self.env), _p(self.masks),
                                    _p(q), ctypes.c_double(bound), _p(out), _p(dist), ctypes.c_int(max_pairs))
        assert n <= max_pairs, n
        return out[:n].copy(), dist[:n].copy()

    def min_distance(self, q, cutoff: float, nthreads: int = 1, want_grad=True, counts=None):
        """(d, pair, cp, grad); `counts`, an int64 array of 3, receives the
        canonical traversal's (node pairs, triangle pairs, configurations)."""
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, self.nl)
        B = q.shape[0]
        d = np.zeros(B, np.float64)
        pair = np.zeros((B, 2), np.int32)
        cp = np.zeros((B, 6), np.float64)
        grad = np.zeros((B, self.nl), np.float64) if want_grad else None
        lib().orc_min_distance(ctypes.c_void_p(self.robot), ctypes.c_void_p(self.env), _p(self.masks),
                               _p(q), ctypes.c_int(B), ctypes.c_double(cutoff), _p(d), _p(pair),
                               _p(cp), _p(grad), ctypes.c_int(nthreads), _p(counts))
        return d, pair, cp, grad

    def softmin(self, q, tau: float, nthreads: int = 1, want_grad=True, counts=None):
        """(L, dL/dq); `counts` as for min_distance (items = waypoints)."""
        q = np.ascontiguousarray(q, dtype=np.float32)
        T, W = q.shape[0], q.shape[1]
        Lout = np.zeros(T, np.float64)
        grad = np.zeros((T, W, self.nl), np.float64) if want_grad else None
        lib().orc_softmin(ctypes.c_void_p(self.robot), ctypes.c_void_p(self.env), _p(self.masks),
                          _p(q), ctypes.c_int(T), ctypes.c_int(W), ctypes.c_double(tau),
                          _p(Lout), _p(grad), ctypes.c_int(nthreads), _p(counts))
        return Lout, grad


def ik_solve(oracle: "Oracle", q0, links, plocal, ptarget, Rtarget=None, max_iters=100, tol=1e-3):
    """FP64 restatement of the engine's IK iteration: (q, ok, residual, iters)."""
    L = oracle.nl
    q = np.ascontiguousarray(q0, dtype=np.float64).reshape(-1, L).copy()
    B = q.shape[0]
    links = np.ascontiguousarray(links, np.int32).reshape(B)
    pl = np.ascontiguousarray(plocal, np.float64).reshape(B, 3)
    pt = np.ascontiguousarray(ptarget, np.float64).reshape(B, 3)
    Rt = None if Rtarget is None else np.ascontiguousarray(Rtarget, np.float64).reshape(B, 9)
    ok = np.zeros(B, np.uint8)
    res = np.zeros(B, np.float64)
    its = np.zeros(B, np.int32)
    lib().orc_ik(ctypes.c_void_p(oracle.robot), ctypes.c_int(B), _p(q), _p(links), _p(pl), _p(pt), _p(Rt),
                 ctypes.c_int(max_iters), ctypes.c_double(tol), _p(ok), _p(res), _p(its))
    return q, ok, res, its


def self_pairs(oracle: "Oracle", q, nthreads: int = 1, mask=None) -> np.ndarray:
    """OR over configurations of the enabled self pairs' verdicts: uint32
    words, bit j of word i set when pair (i, j) collides somewhere."""
    L = oracle.nl
    q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, L)
    m = np.zeros(L, np.uint32) if mask is None else np.ascontiguousarray(mask, np.uint32).copy()
    lib().orc_self_pairs(ctypes.c_void_p(oracle.robot), ctypes.c_void_p(oracle.env), _p(q), ctypes.c_int(q.shape[0]),
                         _p(m), ctypes.c_int(nthreads))
    return m


def indep_pairs(oracle: "Oracle", q, cand, nthreads: int = 1, mask=None) -> np.ndarray:
    """Candidate pairs (uint32 words) that collide alone in some configuration."""
    L = oracle.nl
    q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, L)
    c = np.ascontiguousarray(cand, np.uint32).reshape(L)
    m = np.zeros(L, np.uint32) if mask is None else np.ascontiguousarray(mask, np.uint32).copy()
    lib().orc_indep_pairs(ctypes.c_void_p(oracle.robot), ctypes.c_void_p(oracle.env), _p(q), ctypes.c_int(q.shape[0]),
                          _p(c), _p(m), ctypes.c_int(nthreads))
    return m


def self_distance(oracle: "Oracle", q, cutoff: float = 1e3, nthreads: int = 1):
    """Minimum distance between the robot's own links over its enabled self
    pairs: (d [B], pair [B, 2], cp [B, 6], grad [B, L])."""
    L = oracle.nl
    q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, L)
    B = q.shape[0]
    d = np.zeros(B, np.float64)
    pair = np.zeros((B, 2), np.int32)
    cp = np.zeros((B, 6), np.float64)
    g = np.zeros((B, L), np.float64)
    lib().orc_self_distance(ctypes.c_void_p(oracle.robot), ctypes.c_void_p(oracle.env), _p(q), ctypes.c_int(B),
                            ctypes.c_double(cutoff), _p(d), _p(pair), _p(cp), _p(g), ctypes.c_int(nthreads))
    return d, pair, cp, g


def self_pair_distances(oracle: "Oracle", q, cutoff: float = 1e3, nthreads: int = 1, all_pairs: bool = False):
    """Each self pair's own minimum distance: [B, L (L - 1) / 2] in
    upper-triangle order, clamped at cutoff; -1 for pairs not queried (the
    enabled self pairs, or with all_pairs every pair with geometry)."""
    L = oracle.nl
    q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, L)
    B = q.shape[0]
    out = np.zeros((B, L * (L - 1) // 2), np.float64)
    lib().orc_self_pair_distances(ctypes.c_void_p(oracle.robot), ctypes.c_void_p(oracle.env), _p(q), ctypes.c_int(B),
                                  ctypes.c_double(cutoff), _p(out), ctypes.c_int(int(all_pairs)),
                                  ctypes.c_int(nthreads))
    return out


def jacobian(oracle: "Oracle", q, links, plocal):
    """Full 6 x L Jacobians (angular rows first) of points plocal[b] on links[b]."""
    L = oracle.nl
    q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, L)
    B = q.shape[0]
    links = np.ascontiguousarray(links, dtype=np.int32).reshape(B)
    plocal = np.ascontiguousarray(plocal, dtype=np.float32).reshape(B, 3)
    J = np.zeros((B, 6, L), np.float64)
    lib().orc_jacobian(ctypes.c_void_p(oracle.robot), _p(q), ctypes.c_int(B), _p(links), _p(plocal), _p(J))
    return J


def raycast(oracle: "Oracle", s, d, nthreads: int = 1):
    """Environment ray casting: (obj, tri, t, point) per ray (obj -1: no hit)."""
    s = np.ascontiguousarray(s, dtype=np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(d, dtype=np.float32).reshape(-1, 3)
    R = s.shape[0]
    obj = np.zeros(R, np.int32)
    tri = np.zeros(R, np.int32)
    t = np.zeros(R, np.float64)
    pt = np.zeros((R, 3), np.float64)
    lib().orc_raycast(ctypes.c_void_p(oracle.env), _p(s), _p(d), ctypes.c_int(R), _p(obj), _p(tri), _p(t),
                      _p(pt), ctypes.c_int(nthreads))
    return obj, tri, t, pt


def sincos(x) -> tuple:
    x = np.ascontiguousarray(x, dtype=np.float64)
    s = np.empty_like(x)
    c = np.empty_like(x)
    lib().orc_sincos(_p(x), ctypes.c_int(x.size), _p(s), _p(c))
    return s, c


def tri_tri(P, Q):
    P = np.ascontiguousarray(P, dtype=np.float64).reshape(9)
    Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(9)
    d2 = np.zeros(1, np.float64)
    cp = np.zeros(3, np.float64)
    cq = np.zeros(3, np.float64)
    hit = lib().orc_tri_tri(_p(P), _p(Q), _p(d2), _p(cp), _p(cq))
    return bool(hit), float(d2[0]), cp, cq


def tri_tri_batch(P, Q) -> np.ndarray:
    """The canonical FP64 separating-axis predicate on n pairs [n, 9]."""
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 9)
    Q = np.ascontiguousarray(Q, np.float64).reshape(-1, 9)
    out = np.zeros(len(P), np.uint8)
    lib().orc_tri_tri_batch(_p(P), _p(Q), ctypes.c_int(len(P)), _p(out))
    return out


def tri_tri_exact(P, Q, nthreads: int = 1) -> np.ndarray:
    """Independent exact test (oracle/exact_tri.cpp: feasibility of the
    barycentric system in integer arithmetic) on n pairs of integer
    triangles [n, 9], |coordinate| <= 1024."""
    P = np.ascontiguousarray(P, np.int32).reshape(-1, 9)
    Q = np.ascontiguousarray(Q, np.int32).reshape(-1, 9)
    out = np.zeros(len(P), np.uint8)
    r = lib().orc_tri_tri_exact(_p(P), _p(Q), ctypes.c_int(len(P)), _p(out), ctypes.c_int(nthreads))
    if r != 0:
        raise ValueError("coordinates must be integers of magnitude <= 1024")
    return out


class GeomPairOracle:
    """FP64 oracle of the free-geometry pair queries: a two-link oracle robot
    holding geometry a (link 0) and geometry b (link 1) with their margins,
    placed by the caller's transforms."""

    def __init__(self, mesh_a, mesh_b, margin_a: float = 0.0, margin_b: float = 0.0):
        Va, Fa = (np.asarray(x) for x in mesh_a)
        Vb, Fb = (np.asarray(x) for x in mesh_b)
        eye = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], np.float64)
        self._keep = dict(
            parents=np.array([-1, -1], np.int32), jt=np.array([2, 2], np.int32), T0=np.concatenate([eye, eye]),
            axes=np.array([0, 0, 1, 0, 0, 1], np.float64), qmin=np.zeros(2), qmax=np.zeros(2),
            vo=np.array([0, len(Va), len(Va) + len(Vb)], np.int32),
            V=np.ascontiguousarray(np.concatenate([Va, Vb]), np.float64).reshape(-1),
            to=np.array([0, len(Fa), len(Fa) + len(Fb)], np.int32),
            F=np.ascontiguousarray(np.concatenate([Fa, Fb]), np.int32).reshape(-1),
            m=np.array([margin_a, margin_b], np.float64))
        k = self._keep
        self.robot = lib().orc_robot_create(ctypes.c_int(2), _p(k["parents"]), _p(k["jt"]), _p(k["T0"]), _p(k["axes"]),
                                            _p(k["qmin"]), _p(k["qmax"]), _p(k["vo"]), _p(k["V"]), _p(k["to"]),
                                            _p(k["F"]), _p(k["m"]), None)

    def close(self):
        if self.robot:
            lib().orc_robot_destroy(ctypes.c_void_p(self.robot))
            self.robot = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _tf(Ta, Tb):
        A = np.ascontiguousarray(Ta, np.float64).reshape(-1, 12)
        B = np.ascontiguousarray(Tb, np.float64).reshape(-1, 12)
        n = max(len(A), len(B))
        flags = (1 if len(A) == 1 and n > 1 else 0) | (2 if len(B) == 1 and n > 1 else 0)
        return A, B, n, flags

    def collide(self, Ta, Tb, tol: float = 0.0, nthreads: int = 1) -> np.ndarray:
        A, B, n, flags = self._tf(Ta, Tb)
        hit = np.zeros(n, np.uint8)
        lib().orc_geom_collide(ctypes.c_void_p(self.robot), _p(A), _p(B), ctypes.c_int(n), ctypes.c_int(flags),
                               ctypes.c_double(tol), _p(hit), ctypes.c_int(nthreads))
        return hit

    def distance(self, Ta, Tb, upper_bound: float = float("inf"), nthreads: int = 1):
        A, B, n, flags = self._tf(Ta, Tb)
        d = np.zeros(n, np.float64)
        cp = np.zeros((n, 6), np.float64)
        elem = np.zeros((n, 2), np.int32)
        dr = np.zeros((n, 3), np.float64)
        lib().orc_geom_distance(ctypes.c_void_p(self.robot), _p(A), _p(B), ctypes.c_int(n), ctypes.c_int(flags),
                                ctypes.c_double(upper_bound), _p(d), _p(cp), _p(elem), _p(dr), ctypes.c_int(nthreads))
        return d, cp, elem, dr

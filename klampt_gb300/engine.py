"""World handle over the C ABI: batched FK, collision verdicts, feasibility,
edge checks, signed distance and soft-min gradients on one GPU.

Device buffers are torch tensors (torch is used for device memory and streams
only); every query goes through libkgpu.so.  Inputs may be numpy arrays
(copied to the device) or CUDA tensors (used in place).
"""

from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _kgpu
from ._kgpu import check, lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _dptr(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(x, dtype) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x.to(device="cuda", dtype=dtype)
    else:
        t = torch.as_tensor(np.ascontiguousarray(x), dtype=dtype).cuda()
    return t.contiguous()


class Robot:
    """Robot handle built from a scenes.RobotSpec-like object (links, parents,
    T0_parent, axes, joint types, limits, link meshes, margins, self mask)."""

    def __init__(self, spec):
        self.spec = spec
        self.num_links = spec.num_links
        p = spec.packed()
        self._arrays = p
        d = _kgpu.RobotDesc(
            num_links=self.num_links, parents=_ptr(p["parents"]), joint_types=_ptr(p["joint_types"]),
            T0_parent=_ptr(p["T0_parent"]), axes=_ptr(p["axes"]), qmin=_ptr(p["qmin"]), qmax=_ptr(p["qmax"]),
            vert_offset=_ptr(p["vert_offset"]), verts=_ptr(p["verts"]), tri_offset=_ptr(p["tri_offset"]),
            tris=_ptr(p["tris"]), margins=_ptr(p["margins"]), self_mask=_ptr(p["self_mask"]))
        h = ctypes.c_void_p()
        check(lib().kgpu_robot_create(ctypes.byref(d), ctypes.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().kgpu_robot_destroy(self.handle)
            self.handle = None


class Environment:
    """Static environment handle from a scenes.EnvSpec-like object.

    ``gpu_build`` builds the environment trees on the GPU (linear BVH) instead
    of the host builder; every query gives the same results with either."""

    def __init__(self, spec, gpu_build: bool = False):
        self.spec = spec
        p = spec.packed()
        self._arrays = p
        d = _kgpu.EnvDesc(num_objects=spec.num_objects, vert_offset=_ptr(p["vert_offset"]),
                          verts=_ptr(p["verts"]), tri_offset=_ptr(p["tri_offset"]), tris=_ptr(p["tris"]),
                          groups=_ptr(p["groups"]), convex=_ptr(p["convex"]), margins=_ptr(p["margins"]))
        h = ctypes.c_void_p()
        check(lib().kgpu_env_create_ex(ctypes.byref(d), 1 if gpu_build else 0, ctypes.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().kgpu_env_destroy(self.handle)
            self.handle = None


class Geometry:
    """A free triangle mesh (kgpu_geom) with its collision margin: the
    engine side of a TriangleMesh Geometry3D.  Pair queries place two
    geometries by a transform each, batched over transforms."""

    def __init__(self, verts, tris, margin: float = 0.0):
        v = np.ascontiguousarray(verts, np.float64).reshape(-1, 3)
        f = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
        d = _kgpu.GeomDesc(num_verts=len(v), verts=v.ctypes.data, num_tris=len(f), tris=f.ctypes.data,
                           margin=float(margin))
        h = ctypes.c_void_p()
        check(lib().kgpu_geom_create(ctypes.byref(d), ctypes.byref(h)))
        self.handle = h
        self.num_tris = len(f)

    def close(self):
        if getattr(self, "handle", None):
            lib().kgpu_geom_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_margin(self, margin: float):
        check(lib().kgpu_geom_set_margin(self.handle, float(margin)))

    def margin(self) -> float:
        v = ctypes.c_double()
        check(lib().kgpu_geom_get_margin(self.handle, ctypes.byref(v)))
        return v.value

    @staticmethod
    def _transforms(Ta, Tb):
        A = _dev(Ta, torch.float64).reshape(-1, 12).contiguous()
        B = _dev(Tb, torch.float64).reshape(-1, 12).contiguous()
        n = max(A.shape[0], B.shape[0])
        flags = 0
        if A.shape[0] == 1 and n > 1:
            flags |= _kgpu.GEOM_FIXED_A
        if B.shape[0] == 1 and n > 1:
            flags |= _kgpu.GEOM_FIXED_B
        if A.shape[0] not in (1, n) or B.shape[0] not in (1, n):
            raise ValueError("transform batches must have equal sizes (or one transform)")
        return A, B, n, flags

    def collide(self, other: "Geometry", Ta, Tb, tol: float = 0.0, sync: bool = True) -> torch.Tensor:
        """[B] uint8: 1 where this geometry at Ta[b] and `other` at Tb[b] are
        within (margin + tol) + other.margin (touching counts).  Ta / Tb:
        [B, 12] (R row-major, t) or one transform."""
        A, B, n, flags = self._transforms(Ta, Tb)
        hit = torch.empty(n, dtype=torch.uint8, device="cuda")
        check(lib().kgpu_geom_collide(self.handle, other.handle, _dptr(A), _dptr(B), n, flags, float(tol),
                                      _dptr(hit), _stream()))
        if sync:
            self.sync()
        return hit

    def distance(self, other: "Geometry", Ta, Tb, upper_bound: float = float("inf"), sync: bool = True):
        """(d [B], cp [B, 6], elem [B, 2], dir [B, 3]) as kgpu_geom_distance."""
        A, B, n, flags = self._transforms(Ta, Tb)
        d = torch.empty(n, dtype=torch.float64, device="cuda")
        cp = torch.empty((n, 6), dtype=torch.float64, device="cuda")
        elem = torch.empty((n, 2), dtype=torch.int32, device="cuda")
        dr = torch.empty((n, 3), dtype=torch.float64, device="cuda")
        check(lib().kgpu_geom_distance(self.handle, other.handle, _dptr(A), _dptr(B), n, flags, float(upper_bound),
                                       _dptr(d), _dptr(cp), _dptr(elem), _dptr(dr), _stream()))
        if sync:
            self.sync()
        return d, cp, elem, dr

    def sync(self):
        check(lib().kgpu_geom_sync(self.handle, _stream()))


class EdgePlan:
    """A captured CUDA graph of one edge-check batch over fixed device buffers."""

    def __init__(self, world: "World", robot: int, qa: torch.Tensor, qb: torch.Tensor, nsteps: torch.Tensor,
                 first_hit: torch.Tensor):
        self.world = world
        self._keep = (qa, qb, nsteps, first_hit)
        h = ctypes.c_void_p()
        check(lib().kgpu_edge_plan_create(world.handle, robot, _dptr(qa), _dptr(qb), _dptr(nsteps), qa.shape[0],
                                          _dptr(first_hit), ctypes.byref(h)))
        self.handle = h

    def launch(self):
        check(lib().kgpu_edge_plan_launch(self.handle, _stream()))

    def main_pass_ms(self) -> float:
        """Device time of the last launch's main traversal pass (call after
        that launch has completed)."""
        ms = ctypes.c_float()
        check(lib().kgpu_edge_plan_main_pass_ms(self.handle, ctypes.byref(ms)))
        return float(ms.value)

    def close(self):
        if self.handle:
            lib().kgpu_edge_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ConfigPlan:
    """A captured CUDA graph of one configuration-batch check over fixed
    device buffers (one robot, or robot_ids for a heterogeneous batch)."""

    def __init__(self, world: "World", q: torch.Tensor, env_hit: torch.Tensor, self_hit: torch.Tensor,
                 robot: int = 0, robot_ids: Optional[torch.Tensor] = None):
        self.world = world
        self._keep = (q, env_hit, self_hit, robot_ids)
        h = ctypes.c_void_p()
        B = env_hit.shape[0]
        stride = q.shape[-1] if q.dim() > 1 else 0
        check(lib().kgpu_config_plan_create(world.handle, -1 if robot_ids is not None else robot, _dptr(robot_ids),
                                            _dptr(q), stride, B, _dptr(env_hit), _dptr(self_hit), ctypes.byref(h)))
        self.handle = h

    def launch(self):
        check(lib().kgpu_config_plan_launch(self.handle, _stream()))

    def close(self):
        if self.handle:
            lib().kgpu_config_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class World:
    """An environment plus robots on the current CUDA device."""

    def __init__(self, env_spec, robot_specs: Sequence, gpu_build: bool = False):
        self.env = Environment(env_spec, gpu_build=gpu_build) if env_spec is not None else None
        self.robots: List[Robot] = [Robot(s) for s in robot_specs]
        arr = (ctypes.c_void_p * len(self.robots))(*[r.handle.value for r in self.robots])
        h = ctypes.c_void_p()
        check(lib().kgpu_world_create(self.env.handle if self.env else None, arr, len(self.robots),
                                      ctypes.byref(h)))
        self.handle = h

    # ---- lifetime --------------------------------------------------------
    def close(self):
        if getattr(self, "handle", None):
            lib().kgpu_world_destroy(self.handle)
            self.handle = None
        for r in getattr(self, "robots", []):
            r.close()
        if getattr(self, "env", None):
            self.env.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- settings ----------------------------------------------------------
    def set_option(self, name: str, value: float):
        check(lib().kgpu_world_set_option(self.handle, name.encode(), float(value)))

    def get_option(self, name: str) -> float:
        v = ctypes.c_double()
        check(lib().kgpu_world_get_option(self.handle, name.encode(), ctypes.byref(v)))
        return v.value

    def set_link_env_mask(self, robot: int, link: int, mask: int):
        check(lib().kgpu_world_set_link_env_mask(self.handle, robot, link, ctypes.c_uint32(mask & 0xFFFFFFFF)))

    def enable_self_pair(self, robot: int, i: int, j: int, enabled: bool):
        check(lib().kgpu_world_enable_self_pair(self.handle, robot, i, j, 1 if enabled else 0))

    def sync(self):
        check(lib().kgpu_world_sync(self.handle, _stream()))

    def stats(self) -> dict:
        s = _kgpu.Stats()
        check(lib().kgpu_world_get_stats(self.handle, ctypes.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in _kgpu.Stats._fields_}

    def reset_stats(self):
        check(lib().kgpu_world_reset_stats(self.handle))

    # ---- queries (device) ----------------------------------------------------
    def fk(self, q, robot: int = 0, sync: bool = True, with_error: bool = False):
        """World transforms [B, L, 12] (R row-major, t); with_error also
        returns [B, L] bounds on the world-position error of any link vertex
        against FP64 forward kinematics."""
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L)
        T = torch.empty((qd.shape[0], L, 12), dtype=torch.float32, device="cuda")
        err = torch.empty((qd.shape[0], L), dtype=torch.float32, device="cuda") if with_error else None
        check(lib().kgpu_fk(self.handle, robot, _dptr(qd), qd.shape[0], _dptr(T), _dptr(err), _stream()))
        if sync:
            self.sync()
        return (T, err) if with_error else T

    def fk64(self, q, robot: int = 0, sync: bool = True) -> torch.Tensor:
        """World transforms [B, L, 12] (FP64, R row-major, t) in the
        canonical arithmetic the engine's FP64 decisions use."""
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L).contiguous()
        T = torch.empty((qd.shape[0], L, 12), dtype=torch.float64, device="cuda")
        check(lib().kgpu_fk64(self.handle, robot, _dptr(qd), qd.shape[0], _dptr(T), _stream()))
        if sync:
            self.sync()
        return T

    def check_configs(self, q, robot: int = 0, env: bool = True, self_collision: bool = True,
                      sync: bool = True):
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L)
        B = qd.shape[0]
        eh = torch.zeros(B, dtype=torch.uint8, device="cuda") if env else None
        sh = torch.zeros(B, dtype=torch.uint8, device="cuda") if self_collision else None
        check(lib().kgpu_check_configs(self.handle, robot, _dptr(qd), B, _dptr(eh), _dptr(sh), _stream()))
        if sync:
            self.sync()
        return eh, sh

    def check_configs_multi(self, robot_ids, q, sync: bool = True):
        ids = _dev(robot_ids, torch.int32).reshape(-1)
        qd = _dev(q, torch.float32)
        B = ids.shape[0]
        qd = qd.reshape(B, -1)
        eh = torch.zeros(B, dtype=torch.uint8, device="cuda")
        sh = torch.zeros(B, dtype=torch.uint8, device="cuda")
        check(lib().kgpu_check_configs_multi(self.handle, _dptr(ids), _dptr(qd), qd.shape[1], B, _dptr(eh),
                                             _dptr(sh), _stream()))
        if sync:
            self.sync()
        return eh, sh

    def is_feasible(self, q, robot: int = 0, sync: bool = True) -> torch.Tensor:
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L)
        out = torch.zeros(qd.shape[0], dtype=torch.uint8, device="cuda")
        check(lib().kgpu_is_feasible(self.handle, robot, _dptr(qd), qd.shape[0], _dptr(out), _stream()))
        if sync:
            self.sync()
        return out

    def check_edges(self, qa, qb, nsteps, robot: int = 0, sync: bool = True) -> torch.Tensor:
        L = self.robots[robot].num_links
        a = _dev(qa, torch.float32).reshape(-1, L)
        b = _dev(qb, torch.float32).reshape(-1, L)
        n = _dev(nsteps, torch.int32).reshape(-1)
        out = torch.empty(a.shape[0], dtype=torch.int32, device="cuda")
        check(lib().kgpu_check_edges(self.handle, robot, _dptr(a), _dptr(b), _dptr(n), a.shape[0], _dptr(out),
                                     _stream()))
        if sync:
            self.sync()
        return out

    def check_configs_plain64(self, q, robot: int = 0, sync: bool = True):
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L)
        B = qd.shape[0]
        eh = torch.zeros(B, dtype=torch.uint8, device="cuda")
        sh = torch.zeros(B, dtype=torch.uint8, device="cuda")
        check(lib().kgpu_check_configs_plain64(self.handle, robot, _dptr(qd), B, _dptr(eh), _dptr(sh), _stream()))
        if sync:
            self.sync()
        return eh, sh

    def check_edges_plain64(self, qa, qb, nsteps, robot: int = 0, sync: bool = True,
                            per_step: bool = False, per_pair: bool = False) -> torch.Tensor:
        """The plain FP64 method: one thread per edge (in order), with
        per_step one thread per (edge, step), with per_pair one thread per
        (edge, step, query)."""
        L = self.robots[robot].num_links
        a = _dev(qa, torch.float32).reshape(-1, L)
        b = _dev(qb, torch.float32).reshape(-1, L)
        n = _dev(nsteps, torch.int32).reshape(-1)
        out = torch.empty(a.shape[0], dtype=torch.int32, device="cuda")
        fn = (lib().kgpu_check_edges_plain64_pairs if per_pair else
              lib().kgpu_check_edges_plain64_steps if per_step else lib().kgpu_check_edges_plain64)
        check(fn(self.handle, robot, _dptr(a), _dptr(b), _dptr(n), a.shape[0], _dptr(out), _stream()))
        if sync:
            self.sync()
        return out

    def config_plan(self, q: torch.Tensor, env_hit: torch.Tensor, self_hit: torch.Tensor, robot: int = 0,
                    robot_ids: Optional[torch.Tensor] = None) -> ConfigPlan:
        """A CUDA-graph plan of check_configs (or, with robot_ids, of
        check_configs_multi) over these device buffers."""
        return ConfigPlan(self, q, env_hit, self_hit, robot, robot_ids)

    def edge_plan(self, qa: torch.Tensor, qb: torch.Tensor, nsteps: torch.Tensor, first_hit: torch.Tensor,
                  robot: int = 0) -> EdgePlan:
        return EdgePlan(self, robot, qa, qb, nsteps, first_hit)

    def distance(self, q, cutoff: float, robot: int = 0, want_grad: bool = True, sync: bool = True):
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L)
        B = qd.shape[0]
        d = torch.empty(B, dtype=torch.float64, device="cuda")
        pair = torch.empty((B, 2), dtype=torch.int32, device="cuda")
        cp = torch.empty((B, 6), dtype=torch.float64, device="cuda")
        g = torch.empty((B, L), dtype=torch.float32, device="cuda") if want_grad else None
        check(lib().kgpu_distance(self.handle, robot, _dptr(qd), B, float(cutoff), _dptr(d), _dptr(pair), _dptr(cp),
                                  _dptr(g), _stream()))
        if sync:
            self.sync()
        return d, pair, cp, g

    def self_distance(self, q, cutoff: float, robot: int = 0, want_grad: bool = True, sync: bool = True):
        """Minimum distance between the robot's own links over its enabled self
        pairs: (d [B], pair [B, 2] (i, j), cp [B, 6], grad [B, L] or None)."""
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L).contiguous()
        B = qd.shape[0]
        d = torch.empty(B, dtype=torch.float64, device="cuda")
        pair = torch.empty((B, 2), dtype=torch.int32, device="cuda")
        cp = torch.empty((B, 6), dtype=torch.float64, device="cuda")
        g = torch.empty((B, L), dtype=torch.float32, device="cuda") if want_grad else None
        check(lib().kgpu_self_distance(self.handle, robot, _dptr(qd), B, float(cutoff), _dptr(d), _dptr(pair),
                                       _dptr(cp), _dptr(g), _stream()))
        if sync:
            self.sync()
        return d, pair, cp, g

    def self_pair_distances(self, q, cutoff: float, robot: int = 0, all_pairs: bool = False, sync: bool = True):
        """Each self pair's own minimum distance: [B, L (L - 1) / 2] in
        upper-triangle order (i < j), clamped at cutoff; -1 for pairs not
        queried (the enabled self pairs, or with all_pairs every pair whose
        links have geometry)."""
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L).contiguous()
        B = qd.shape[0]
        out = torch.empty((B, L * (L - 1) // 2), dtype=torch.float64, device="cuda")
        check(lib().kgpu_self_pair_distances(self.handle, robot, _dptr(qd), B, float(cutoff), int(all_pairs),
                                             _dptr(out), _stream()))
        if sync:
            self.sync()
        return out

    def softmin(self, q, tau: float, robot: int = 0, want_grad: bool = True, sync: bool = True):
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32)
        T, W = qd.shape[0], qd.shape[1]
        qd = qd.reshape(T, W, L).contiguous()
        out = torch.empty(T, dtype=torch.float64, device="cuda")
        g = torch.empty((T, W, L), dtype=torch.float32, device="cuda") if want_grad else None
        check(lib().kgpu_softmin_grad(self.handle, robot, _dptr(qd), T, W, float(tau), _dptr(out), _dptr(g),
                                      _stream()))
        if sync:
            self.sync()
        return out, g

    def ik_solve(self, q0, links, plocal, ptarget, Rtarget=None, max_iters: int = 100, tol: float = 1e-3,
                 robot: int = 0, sync: bool = True):
        """Batched IK from initial guesses q0 [B, L]: (q [B, L], ok [B],
        residual [B], iters [B]).  Rtarget [B, 9] (row-major) adds the
        orientation constraint."""
        L = self.robots[robot].num_links
        q = _dev(q0, torch.float32).reshape(-1, L).clone()
        B = q.shape[0]
        pl = _dev(plocal, torch.float32).reshape(-1, 3)
        pl = (pl.expand(B, 3) if pl.shape[0] == 1 else pl).contiguous()
        pt = _dev(ptarget, torch.float32).reshape(B, 3).contiguous()
        Rt = None if Rtarget is None else _dev(Rtarget, torch.float32).reshape(B, 9).contiguous()
        ok = torch.empty(B, dtype=torch.uint8, device="cuda")
        res = torch.empty(B, dtype=torch.float32, device="cuda")
        its = torch.empty(B, dtype=torch.int32, device="cuda")
        if isinstance(links, (int, np.integer)):
            ld, lk = None, int(links)
        else:
            ld, lk = _dev(links, torch.int32).reshape(B).contiguous(), 0
        check(lib().kgpu_ik_solve(self.handle, robot, B, _dptr(q), None if ld is None else _dptr(ld), lk, _dptr(pl),
                                  _dptr(pt), None if Rt is None else _dptr(Rt), int(max_iters), float(tol),
                                  _dptr(ok), _dptr(res), _dptr(its), _stream()))
        if sync:
            self.sync()
        return q, ok, res, its

    def self_collision_pairs(self, q, robot: int = 0, mask=None, sync: bool = True):
        """Self pairs colliding in some configuration of q [B, L]: uint32
        words [L] (bit j of word i: pair (i, j)), OR-accumulated into `mask`
        (a CUDA int32 tensor) when given."""
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L).contiguous()
        m = torch.zeros(L, dtype=torch.int32, device="cuda") if mask is None else mask
        check(lib().kgpu_self_collision_pairs(self.handle, robot, _dptr(qd), qd.shape[0], _dptr(m), _stream()))
        if sync:
            self.sync()
        return m

    def independent_self_collision_pairs(self, q, candidates, robot: int = 0, mask=None, sync: bool = True):
        """Candidate self pairs (uint32 words [L], as self_collision_pairs
        returns them) that collide alone in some configuration of q [B, L]:
        uint32 words [L], OR-accumulated into `mask` when given."""
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L).contiguous()
        if isinstance(candidates, torch.Tensor):
            c = candidates.to(device="cuda", dtype=torch.int32).reshape(L).contiguous()
        else:  # uint32 words: reinterpret, bit 31 included
            c = torch.as_tensor(np.ascontiguousarray(candidates, dtype=np.uint32).view(np.int32)).cuda().reshape(L)
        m = torch.zeros(L, dtype=torch.int32, device="cuda") if mask is None else mask
        check(lib().kgpu_independent_self_collision_pairs(self.handle, robot, _dptr(qd), qd.shape[0], _dptr(c),
                                                          _dptr(m), _stream()))
        if sync:
            self.sync()
        return m

    def jacobian(self, q, links, plocal, robot: int = 0, sync: bool = True):
        """Full Jacobians [B, 6, L] (angular rows, then linear) of points
        plocal [B, 3] (link frame) on links [B] (or one int for all)."""
        L = self.robots[robot].num_links
        qd = _dev(q, torch.float32).reshape(-1, L).contiguous()
        B = qd.shape[0]
        pd = _dev(plocal, torch.float32).reshape(-1, 3)
        if pd.shape[0] == 1 and B > 1:
            pd = pd.expand(B, 3)
        pd = pd.contiguous()
        J = torch.empty((B, 6, L), dtype=torch.float32, device="cuda")
        if isinstance(links, (int, np.integer)):
            check(lib().kgpu_jacobian(self.handle, robot, _dptr(qd), B, None, int(links), _dptr(pd), _dptr(J),
                                      _stream()))
        else:
            ld = _dev(links, torch.int32).reshape(B).contiguous()
            check(lib().kgpu_jacobian(self.handle, robot, _dptr(qd), B, _dptr(ld), 0, _dptr(pd), _dptr(J), _stream()))
        if sync:
            self.sync()
        return J

    def raycast(self, s, d, sync: bool = True):
        """Rays s[i] + t d[i] (t >= 0) against the environment: (obj, tri, t,
        point) per ray; obj -1 and t = inf on a miss."""
        sd = _dev(s, torch.float32).reshape(-1, 3).contiguous()
        dd = _dev(d, torch.float32).reshape(-1, 3).contiguous()
        R = sd.shape[0]
        if dd.shape[0] != R:
            raise ValueError("s and d must hold the same number of rays")
        obj = torch.empty(R, dtype=torch.int32, device="cuda")
        tri = torch.empty(R, dtype=torch.int32, device="cuda")
        t = torch.empty(R, dtype=torch.float64, device="cuda")
        pt = torch.empty((R, 3), dtype=torch.float64, device="cuda")
        check(lib().kgpu_raycast(self.handle, _dptr(sd), _dptr(dd), R, _dptr(obj), _dptr(tri), _dptr(t), _dptr(pt),
                                 _stream()))
        if sync:
            self.sync()
        return obj, tri, t, pt

    # ---- queries (host buffers, through the C ABI's pinned staging) -----------
    def check_configs_host(self, q: np.ndarray, robot: int = 0):
        L = self.robots[robot].num_links
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, L)
        B = q.shape[0]
        eh = np.zeros(B, np.uint8)
        sh = np.zeros(B, np.uint8)
        check(lib().kgpu_check_configs_host(self.handle, robot, _ptr(q), B, _ptr(eh), _ptr(sh)))
        return eh, sh

    def check_edges_host(self, qa: np.ndarray, qb: np.ndarray, nsteps: np.ndarray, robot: int = 0) -> np.ndarray:
        L = self.robots[robot].num_links
        qa = np.ascontiguousarray(qa, dtype=np.float32).reshape(-1, L)
        qb = np.ascontiguousarray(qb, dtype=np.float32).reshape(-1, L)
        n = np.ascontiguousarray(nsteps, dtype=np.int32).reshape(-1)
        out = np.zeros(qa.shape[0], np.int32)
        check(lib().kgpu_check_edges_host(self.handle, robot, _ptr(qa), _ptr(qb), _ptr(n), qa.shape[0], _ptr(out)))
        return out

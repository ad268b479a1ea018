"""ctypes binding of the C ABI in include/kgpu.h (libkgpu.so, built in-tree).

This is the same boundary a C++ host or any other FFI binds; the Python
layer adds nothing but argument marshalling and the mapping of status codes
to exceptions (RuntimeError, as the reference's SWIG layer does in
Python/klampt/src/robotsim.i:41-53).  There is no fallback: if the library
is missing or cannot be loaded, importing this module raises.
"""

from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB

KGPU_OK = 0
KGPU_ERR_INVALID = 1
KGPU_ERR_CUDA = 2
KGPU_ERR_OOM = 3
KGPU_ERR_OVERFLOW = 4
KGPU_ERR_TIMEOUT = 5
KGPU_ERR_NOT_FINITE = 6
KGPU_ERR_EMPTY = 7
KGPU_ERR_UNSUPPORTED = 8

GEOM_FIXED_A = 1
GEOM_FIXED_B = 2

GROUP_RIGID_OBJECT = 0
GROUP_TERRAIN = 1
MAX_LINKS = 32

_c_p = ctypes.c_void_p
_i32 = ctypes.c_int32


class RobotDesc(ctypes.Structure):
    _fields_ = [("num_links", _i32), ("parents", _c_p), ("joint_types", _c_p), ("T0_parent", _c_p),
                ("axes", _c_p), ("qmin", _c_p), ("qmax", _c_p), ("vert_offset", _c_p), ("verts", _c_p),
                ("tri_offset", _c_p), ("tris", _c_p), ("margins", _c_p), ("self_mask", _c_p)]


class EnvDesc(ctypes.Structure):
    _fields_ = [("num_objects", _i32), ("vert_offset", _c_p), ("verts", _c_p), ("tri_offset", _c_p),
                ("tris", _c_p), ("groups", _c_p), ("convex", _c_p), ("margins", _c_p)]


class GeomDesc(ctypes.Structure):
    _fields_ = [("num_verts", ctypes.c_int32), ("verts", ctypes.c_void_p), ("num_tris", ctypes.c_int32),
                ("tris", ctypes.c_void_p), ("margin", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("items", ctypes.c_uint64), ("node_pairs", ctypes.c_uint64), ("tri_pairs", ctypes.c_uint64),
                ("band_pairs", ctypes.c_uint64), ("spills", ctypes.c_uint64), ("certified", ctypes.c_uint64),
                ("fp64_hits", ctypes.c_uint64), ("dist_pairs", ctypes.c_uint64),
                ("dist_node_pairs", ctypes.c_uint64), ("dist_tri_pairs", ctypes.c_uint64),
                ("dist_fp64", ctypes.c_uint64)]


class KgpuError(RuntimeError):
    """A non-zero status from the engine; ``code`` holds the KGPU_ERR_* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"kgpu error {code}: {msg}")
        self.code = code


# (name, argtypes); every function returns kgpu_status unless listed below
_SIGS = {
    "kgpu_robot_create": [_c_p, _c_p],
    "kgpu_robot_destroy": [_c_p],
    "kgpu_env_create": [_c_p, _c_p],
    "kgpu_env_create_ex": [_c_p, _i32, _c_p],
    "kgpu_env_destroy": [_c_p],
    "kgpu_world_create": [_c_p, _c_p, _i32, _c_p],
    "kgpu_world_destroy": [_c_p],
    "kgpu_world_set_link_env_mask": [_c_p, _i32, _i32, ctypes.c_uint32],
    "kgpu_world_enable_self_pair": [_c_p, _i32, _i32, _i32, _i32],
    "kgpu_world_set_option": [_c_p, ctypes.c_char_p, ctypes.c_double],
    "kgpu_world_get_option": [_c_p, ctypes.c_char_p, _c_p],
    "kgpu_world_sync": [_c_p, _c_p],
    "kgpu_world_get_stats": [_c_p, _c_p],
    "kgpu_world_reset_stats": [_c_p],
    "kgpu_fk": [_c_p, _i32, _c_p, _i32, _c_p, _c_p, _c_p],
    "kgpu_fk64": [_c_p, _i32, _c_p, _i32, _c_p, _c_p],
    "kgpu_check_configs": [_c_p, _i32, _c_p, _i32, _c_p, _c_p, _c_p],
    "kgpu_check_configs_multi": [_c_p, _c_p, _c_p, _i32, _i32, _c_p, _c_p, _c_p],
    "kgpu_is_feasible": [_c_p, _i32, _c_p, _i32, _c_p, _c_p],
    "kgpu_check_edges": [_c_p, _i32, _c_p, _c_p, _c_p, _i32, _c_p, _c_p],
    "kgpu_check_configs_plain64": [_c_p, _i32, _c_p, _i32, _c_p, _c_p, _c_p],
    "kgpu_check_edges_plain64": [_c_p, _i32, _c_p, _c_p, _c_p, _i32, _c_p, _c_p],
    "kgpu_check_edges_plain64_steps": [_c_p, _i32, _c_p, _c_p, _c_p, _i32, _c_p, _c_p],
    "kgpu_check_edges_plain64_pairs": [_c_p, _i32, _c_p, _c_p, _c_p, _i32, _c_p, _c_p],
    "kgpu_distance": [_c_p, _i32, _c_p, _i32, ctypes.c_double, _c_p, _c_p, _c_p, _c_p, _c_p],
    "kgpu_self_distance": [_c_p, _i32, _c_p, _i32, ctypes.c_double, _c_p, _c_p, _c_p, _c_p, _c_p],
    "kgpu_self_pair_distances": [_c_p, _i32, _c_p, _i32, ctypes.c_double, _i32, _c_p, _c_p],
    "kgpu_softmin_grad": [_c_p, _i32, _c_p, _i32, _i32, ctypes.c_double, _c_p, _c_p, _c_p],
    "kgpu_ik_solve": [_c_p, _i32, _i32, _c_p, _c_p, _i32, _c_p, _c_p, _c_p, _i32, ctypes.c_float, _c_p, _c_p, _c_p,
                      _c_p],
    "kgpu_self_collision_pairs": [_c_p, _i32, _c_p, _i32, _c_p, _c_p],
    "kgpu_independent_self_collision_pairs": [_c_p, _i32, _c_p, _i32, _c_p, _c_p, _c_p],
    "kgpu_jacobian": [_c_p, _i32, _c_p, _i32, _c_p, _i32, _c_p, _c_p, _c_p],
    "kgpu_raycast": [_c_p, _c_p, _c_p, _i32, _c_p, _c_p, _c_p, _c_p, _c_p],
    "kgpu_geom_create": [_c_p, _c_p],
    "kgpu_geom_destroy": [_c_p],
    "kgpu_geom_set_margin": [_c_p, ctypes.c_double],
    "kgpu_geom_get_margin": [_c_p, _c_p],
    "kgpu_geom_collide": [_c_p, _c_p, _c_p, _c_p, _i32, _i32, ctypes.c_double, _c_p, _c_p],
    "kgpu_geom_distance": [_c_p, _c_p, _c_p, _c_p, _i32, _i32, ctypes.c_double, _c_p, _c_p, _c_p, _c_p, _c_p],
    "kgpu_geom_sync": [_c_p, _c_p],
    "kgpu_check_configs_host": [_c_p, _i32, _c_p, _i32, _c_p, _c_p],
    "kgpu_check_edges_host": [_c_p, _i32, _c_p, _c_p, _c_p, _i32, _c_p],
    "kgpu_check_edges_noalloc": [_c_p, _i32, _c_p, _c_p, _c_p, _i32, _c_p, _c_p],
    "kgpu_edge_plan_create": [_c_p, _i32, _c_p, _c_p, _c_p, _i32, _c_p, _c_p],
    "kgpu_edge_plan_launch": [_c_p, _c_p],
    "kgpu_edge_plan_main_pass_ms": [_c_p, _c_p],
    "kgpu_edge_plan_destroy": [_c_p],
    "kgpu_config_plan_create": [_c_p, _i32, _c_p, _c_p, _i32, _i32, _c_p, _c_p, _c_p],
    "kgpu_config_plan_launch": [_c_p, _c_p],
    "kgpu_config_plan_destroy": [_c_p],
}
_STR_FUNCS = ("kgpu_last_error", "kgpu_version")

_lib = None


def exported_symbols():
    """Names of every entry point declared in include/kgpu.h."""
    return list(_SIGS) + list(_STR_FUNCS)


def load(path: str = LIB_PATH):
    """Loads libkgpu.so (no compilation here; call klampt_gb300.build.build()
    first).  Raises OSError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"libkgpu.so not found at {path}; run klampt_gb300.build.build()")
    L = ctypes.CDLL(path)
    for name, args in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = _i32
    for name in _STR_FUNCS:
        f = getattr(L, name)
        f.argtypes = []
        f.restype = ctypes.c_char_p
    _lib = L
    return L


def lib():
    return _lib if _lib is not None else load()


def last_error() -> str:
    return lib().kgpu_last_error().decode()


def check(status: int):
    if status != KGPU_OK:
        raise KgpuError(status, last_error())

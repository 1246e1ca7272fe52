"""ctypes binding of the C ABI in include/xdgcu.h (libxdgcu.so).

The shared library is built in-tree by xdg_gb300.build.  Loading fails
loudly when it is missing: there is no CPU fallback for the engine.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
_VP = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_int = ctypes.c_int
_dbl = ctypes.c_double

# status / enums (xdgcu.h)
OK = 0
RAY_OK, RAY_INVALID, RAY_STACK_OVERFLOW, RAY_WALK_LIMIT, RAY_NO_EXIT_FACE = 0, 1, 2, 4, 5
RAY_OUTPUT_FULL = 6
RAY_EVENT_LIMIT, RAY_LOST, RAY_STUCK = 7, 8, 9
BC_TRANSMISSION, BC_VACUUM, BC_REFLECTING = 0, 1, 2
ANY, EXITING, ENTERING = -1, 0, 1
FP64, MIXED = 0, 1
QUERY_RAY_FIRE, QUERY_POINT_IN_VOLUME, QUERY_OCCLUDED, QUERY_FIND_VOLUME = 0, 1, 2, 3

# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "xdgcu_version": (_int, []),
    "xdgcu_create": (_int, [ctypes.POINTER(_VP), _int]),
    "xdgcu_destroy": (_int, [_VP]),
    "xdgcu_last_error": (ctypes.c_char_p, [_VP]),
    "xdgcu_register_surface": (_int, [_VP, _i32, _i64, _VP, _VP]),
    "xdgcu_create_surface_tree": (_int, [_VP, _VP, _VP, _i32, _dbl, _I]),
    "xdgcu_create_global_surface_tree": (_int, [_VP, _I]),
    "xdgcu_set_tet_mesh": (_int, [_VP, _i64, _VP, _i64, _VP, _VP, _VP, _VP]),
    "xdgcu_create_element_tree": (_int, [_VP, _VP, _i64, _I]),
    "xdgcu_create_global_element_tree": (_int, [_VP, _I]),
    "xdgcu_num_surface_trees": (_int, [_VP]),
    "xdgcu_num_element_trees": (_int, [_VP]),
    "xdgcu_ray_fire": (_int, [_VP, _i32, _VP, _i64, _VP, _VP, _VP, _i32, _VP, _VP, _VP, _VP,
                              _VP, _VP, _i32, _VP]),
    "xdgcu_point_in_volume": (_int, [_VP, _i32, _VP, _i64, _VP, _VP, _VP, _VP, _VP, _VP, _i32,
                                     _VP]),
    "xdgcu_occluded": (_int, [_VP, _i32, _VP, _i64, _VP, _VP, _VP, _VP, _VP, _i32, _VP]),
    "xdgcu_set_volume_map": (_int, [_VP, _i32, _VP, _VP, _i32]),
    "xdgcu_find_volume": (_int, [_VP, _i64, _VP, _VP, _VP, _VP, _i32, _VP]),
    "xdgcu_closest": (_int, [_VP, _i32, _VP, _i64, _VP, _VP, _VP, _VP, _i32, _VP]),
    "xdgcu_find_element": (_int, [_VP, _i32, _VP, _i64, _VP, _VP, _VP, _VP, _i32, _VP]),
    "xdgcu_next_element": (_int, [_VP, _i64, _VP, _VP, _VP, _VP, _VP, _VP, _i32, _VP]),
    "xdgcu_walk_elements": (_int, [_VP, _i64, _VP, _VP, _VP, _VP, _i32, _VP, _VP, _VP, _VP,
                                   _i32, _VP]),
    "xdgcu_walk_elements_packed": (_int, [_VP, _i64, _VP, _VP, _VP, _VP, _i32, _i64, _VP, _VP,
                                          _VP, _VP, _i32, _VP]),
    "xdgcu_walk_elements_packed_noalloc": (_int, [_VP, _i64, _VP, _VP, _VP, _VP, _i32, _i64,
                                                  _VP, _VP, _VP, _VP, _i32, _VP]),
    "xdgcu_set_boundary_face_elements": (_int, [_VP, _i64, _VP, _VP]),
    "xdgcu_segments_global": (_int, [_VP, _i32, _i32, _i64, _VP, _VP, _i32, _i32, _i64, _VP, _VP,
                                     _VP, _VP, _i32, _VP]),
    "xdgcu_point_in_volumes": (_int, [_VP, _i64, _VP, _VP, _i32, _VP, _VP, _VP, _i32, _VP]),
    "xdgcu_set_surface_boundary": (_int, [_VP, _i32, _VP, _VP]),
    "xdgcu_transport_surfaces": (_int, [_VP, _i64, _VP, _VP, _VP, _VP, _dbl, _i32, _i32, _i32,
                                        _VP, _VP, _VP, _VP, _VP, _VP, _i32, _VP]),
    "xdgcu_seed_streams": (_int, [ctypes.c_uint64, _i64, _VP]),
    "xdgcu_transport_elements": (_int, [_VP, _i64, _VP, _VP, _VP, _VP, _dbl, _i32, _VP, _VP,
                                        _VP, _VP, _i32, _VP]),
    "xdgcu_set_tuning": (_int, [_VP, ctypes.c_char_p, _i64]),
    "xdgcu_get_tuning": (_int, [_VP, ctypes.c_char_p, _I64]),
    "xdgcu_autotune_trace": (_int, [_VP, _i32, _i32, _VP, _i64, _VP, _VP, _i32, _i32, _i32, _D]),
    "xdgcu_rebuild_trees": (_int, [_VP, _i32]),
    "xdgcu_autotune_walk": (_int, [_VP, _i64, _VP, _VP, _VP, _VP, _i32, _i32, _i32, _D]),
    "xdgcu_set_counting": (_int, [_VP, _i32]),
    "xdgcu_get_counters": (_int, [_VP, _I64]),
    "xdgcu_surface_tree_info": (_int, [_VP, _i32, _I64]),
    "xdgcu_element_tree_info": (_int, [_VP, _i32, _I64]),
}

_lib = None


class EngineError(RuntimeError):
    pass


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libxdgcu.so (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise EngineError(f"{_build.LIB} is missing; run xdg_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc: int, ctx=None, what: str = ""):
    if rc != OK:
        msg = _lib.xdgcu_last_error(ctx).decode() if _lib is not None else ""
        raise EngineError(f"{what} failed (status {rc}): {msg}")

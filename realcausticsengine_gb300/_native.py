"""ctypes binding of librealcaustics.so (the C ABI in include/realcaustics.h).

The library is built in-tree by realcausticsengine_gb300.build (or
__graft_entry__.build()).  There is no CPU fallback: if the library is missing or
fails to load, `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import abi

LIB_PATH = Path(__file__).resolve().parent / "librealcaustics.so"
_lib = None


class NativeError(RuntimeError):
    pass


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise NativeError(f"{LIB_PATH} is missing: run realcausticsengine_gb300.build.build() first")
    L = C.CDLL(str(LIB_PATH))
    L.init.argtypes = abi.INIT_ARGTYPES
    L.init.restype = None
    L.main.argtypes = []
    L.main.restype = C.c_int
    L.rc_default_config.argtypes = [C.POINTER(abi.RcConfig)]
    L.rc_set_config.argtypes = [C.POINTER(abi.RcConfig)]
    L.rc_prepare.argtypes = []
    L.rc_prepare_host.argtypes = [C.POINTER(C.c_float)]
    L.rc_host_mesh_bvh.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_float)]
    L.rc_host_world_bvh.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
    L.rc_render.argtypes = [C.c_int]
    L.rc_read_image.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.rc_release.argtypes = []
    L.rc_last_error.restype = C.c_char_p
    L.rc_get_stats.argtypes = [C.c_void_p, C.c_int]
    L.rc_trace_rays.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
    L.rc_trace_rays_full.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
    L.rc_trace_rays_shape.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_int]
    L.rc_kd_query.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p,
                              C.c_longlong, C.POINTER(C.c_longlong)]
    L.rc_gather_query.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_void_p,
                                  C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]
    L.rc_gather_variants.argtypes = []
    L.rc_device_bus_id.argtypes = [C.c_char_p, C.c_int]
    L.rc_light_photons_shape.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]
    L.rc_tc_gemm_selftest.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.rc_tc_wait_selftest.argtypes = [C.c_uint]
    L.rc_camera_queries.argtypes = [C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]
    L.rc_kd_build_nodes.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]
    L.rc_render_timed.argtypes = [C.c_int, C.c_void_p]
    L.rc_kd_build_noalloc.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]
    L.rc_kd_noalloc_last_error.restype = C.c_char_p
    L.rc_light_photons.argtypes = [C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]
    L.rc_proposal_state.argtypes = [C.c_longlong, C.c_void_p, C.c_void_p]
    L.rc_render_debug.argtypes = [C.c_int]
    L.rc_save_state.argtypes = [C.c_char_p]
    L.rc_load_state.argtypes = [C.c_char_p]
    L.rc_scene_dump.argtypes = [C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]
    L.rc_prepare_stats.argtypes = [C.c_void_p, C.c_int]
    L.rc_context_create.restype = C.c_void_p
    L.rc_context_create.argtypes = []
    L.rc_context_bind.argtypes = [C.c_void_p]
    L.rc_context_destroy.argtypes = [C.c_void_p]
    L.rc_batch_render.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.rc_mlt_photons.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong), C.c_void_p]
    _lib = L
    return L


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = lib().rc_last_error().decode(errors="replace")
        raise NativeError(f"{what} failed ({rc}): {msg}")


EXPORTS = ["init", "main", "rc_default_config", "rc_set_config", "rc_prepare", "rc_prepare_host",
           "rc_host_mesh_bvh", "rc_host_world_bvh", "rc_render", "rc_read_image", "rc_release",
           "rc_last_error", "rc_get_stats", "rc_trace_rays", "rc_trace_rays_full", "rc_trace_rays_shape", "rc_kd_query",
           "rc_kd_build_nodes", "rc_light_photons", "rc_render_timed", "rc_kd_build_noalloc",
           "rc_kd_noalloc_last_error", "rc_proposal_state", "rc_render_debug",
           "rc_save_state", "rc_load_state", "rc_scene_dump", "rc_prepare_stats",
           "rc_context_create", "rc_context_bind", "rc_context_destroy", "rc_gather_query",
           "rc_gather_variants", "rc_camera_queries", "rc_device_bus_id", "rc_tc_gemm_selftest",
           "rc_tc_wait_selftest", "rc_light_photons_shape", "rc_batch_render",
           "rc_mlt_photons"]

"""CPU oracle - test infrastructure only.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; the product (realcausticsengine_gb300) never imports it.

Two libraries:
  _build/liboracle.so   the restatement in vm_oracle.cpp (built on every host)
  _ref/libref_oracle.so the reference's own sources + ref_harness.cpp, built by
                        build_ref.sh only where the reference sources exist
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_oracle.so"


def build() -> Path:
    BUILD.mkdir(exist_ok=True)
    src = HERE / "vm_oracle.cpp"
    if LIB.exists() and LIB.stat().st_mtime > src.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", str(src), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_reference() -> Path | None:
    """Compile the reference with build_ref.sh (the recipe locates its sources; the
    REF_ROOT environment variable overrides where).  None where the sources are absent
    (exit status 3), as on the GPU hosts."""
    r = subprocess.run(["bash", str(HERE / "build_ref.sh")], capture_output=True, text=True)
    if r.returncode == 3:
        return None
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    return REF_LIB


_oracle = None
_ref = None


def oracle() -> C.CDLL:
    global _oracle
    if _oracle is None:
        build()
        lib = C.CDLL(str(LIB))
        from realcausticsengine_gb300 import abi
        lib.oracle_init.argtypes = abi.INIT_ARGTYPES
        lib.oracle_init.restype = None
        lib.oracle_prepare.argtypes = [C.POINTER(C.c_float)]
        lib.oracle_trace.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_int]
        lib.oracle_kd_query.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_longlong]
        lib.oracle_kd_query.restype = C.c_longlong
        lib.oracle_bsdf.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_light_sample.argtypes = [C.c_void_p, C.c_void_p]
        lib.oracle_render_reference.argtypes = [C.c_void_p, C.c_int]
        lib.oracle_render_plain.argtypes = [C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.c_longlong, C.c_int, C.c_int,
                                            C.c_void_p, C.c_void_p]
        lib.oracle_light_photons.argtypes = [C.c_int, C.c_ulonglong, C.c_longlong, C.c_int, C.c_void_p, C.c_longlong, C.c_int]
        lib.oracle_light_photons.restype = C.c_longlong
        lib.oracle_mesh_bvh.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_float)]
        lib.oracle_world_bvh.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        lib.oracle_scene_info.argtypes = [C.c_void_p]
        lib.oracle_last_error.restype = C.c_char_p
        lib.oracle_debug_view.argtypes = [C.c_int, C.c_float, C.c_void_p]
        _oracle = lib
    return _oracle


def reference() -> C.CDLL | None:
    """The reference itself, or None where it cannot be built (no sources)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            if build_reference() is None:
                return None
        lib = C.CDLL(str(REF_LIB))
        from realcausticsengine_gb300 import abi
        lib.init.argtypes = abi.INIT_ARGTYPES
        lib.init.restype = None
        lib.ref_prepare.argtypes = [C.POINTER(C.c_float)]
        lib.ref_trace.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
        lib.ref_kd_build.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        lib.ref_kd_query.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_longlong]
        lib.ref_kd_query.restype = C.c_longlong
        lib.ref_bsdf.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ref_light_sample.argtypes = [C.c_void_p, C.c_void_p]
        lib.ref_render.argtypes = [C.c_void_p]
        lib.ref_mesh_bvh.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_float)]
        lib.ref_world_bvh.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        lib.ref_layout.argtypes = [C.c_void_p]
        lib.ref_debug.argtypes = [C.c_int, C.c_void_p]
        lib.ref_debug_bvh.argtypes = []
        _ref = lib
    return _ref

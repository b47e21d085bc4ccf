"""ctypes mirrors of the structs the reference's init() takes.

Layouts (LP64, x86-64 and aarch64) of Real Caustics/src:
  vec3             12 B   (vec3.h:13-19)
  Debug_stuff      24 B   (Vertex_Merging.h:13-19)
  PythonMatrix4x4  64 B   (matrix.h:151-170)
  Python_Light     64 B   (Lights.h:15-36)
  Python_Material  28 B   (materials.h:21-32)
  Blender Mesh     mpoly @200, mloop @208, mvert @256 (Blender_definitions.h:214-311);
                   MVert 20 B, MPoly 12 B, MLoop 8 B
"""
from __future__ import annotations

import ctypes as C

MESH_BLENDER_SIZE = 1776
OFF_MPOLY, OFF_MLOOP, OFF_MVERT = 200, 208, 256


class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class DebugStuff(C.Structure):
    _fields_ = [("number_of_points", C.c_int), ("direction", Vec3), ("roughness", C.c_float),
                ("specular", C.c_float)]


class Matrix4x4(C.Structure):
    _fields_ = [("t", C.c_float * 16)]


class PythonLight(C.Structure):
    _fields_ = [("type", C.c_char), ("color", C.c_float * 3), ("position", Vec3), ("width", C.c_float),
                ("height", C.c_float), ("spread", C.c_float), ("rotation", Vec3), ("power", C.c_float),
                ("angle", C.c_float), ("radius", C.c_float)]


class PythonMaterial(C.Structure):
    _fields_ = [("type", C.c_char), ("ior", C.c_float), ("roughness", C.c_float), ("specular", C.c_float),
                ("color", C.c_float * 3)]


class RcConfig(C.Structure):
    _fields_ = [("max_path_length", C.c_int), ("photons_per_iter", C.c_longlong), ("sampler", C.c_int),
                ("mlt_chains", C.c_int), ("large_step_prob", C.c_float), ("seed", C.c_ulonglong),
                ("write_exr", C.c_int), ("exr_path", C.c_char * 256), ("verbose", C.c_int),
                ("learned_proposal", C.c_int), ("train_iterations", C.c_int), ("train_steps", C.c_int),
                ("learning_rate", C.c_float), ("camera_seed", C.c_ulonglong),
                ("autotune", C.c_int), ("graph_replay", C.c_int), ("gpu_bvh", C.c_int)]


SAMPLER_UNIFORM, SAMPLER_HYBRID, SAMPLER_PSSMLT = 0, 1, 2

assert C.sizeof(Vec3) == 12 and C.sizeof(DebugStuff) == 24 and C.sizeof(Matrix4x4) == 64
assert C.sizeof(PythonLight) == 64 and C.sizeof(PythonMaterial) == 28

INIT_ARGTYPES = [C.c_int, C.c_float, C.c_float, C.POINTER(C.c_longlong), C.c_uint, C.POINTER(Matrix4x4),
                 C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.c_uint, C.c_uint, Vec3, Vec3, Vec3, Vec3, Vec3,
                 C.POINTER(PythonLight), C.c_uint, C.POINTER(PythonMaterial), C.c_uint,
                 C.POINTER(C.POINTER(C.c_int)), C.c_int, DebugStuff]


def vec3(v) -> Vec3:
    return Vec3(float(v[0]), float(v[1]), float(v[2]))

"""Scene description and its Blender-layout encoding for init().

A `Scene` holds triangle meshes (object-space vertices, int16 vertex normals as
Blender stores them, one material slot per triangle), world matrices, materials,
lights and the camera.  `InitArgs` encodes it into exactly the bytes the Blender
add-on hands to init(): Blender `Mesh` structs whose mpoly/mloop/mvert pointers
point at MPoly/MLoop/MVert arrays, PythonMatrix4x4 / Python_Light / Python_Material
arrays, and the per-mesh material index tables.  The same InitArgs drives this
library, the reference compiled as an oracle and the CPU restatement.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

MVERT_DT = np.dtype([("co", "<f4", 3), ("no", "<i2", 3), ("flag", "i1"), ("bweight", "i1")])
MPOLY_DT = np.dtype([("loopstart", "<i4"), ("totloop", "<i4"), ("mat_nr", "<i2"), ("flag", "i1"), ("pad", "i1")])
MLOOP_DT = np.dtype([("v", "<u4"), ("e", "<u4")])
assert MVERT_DT.itemsize == 20 and MPOLY_DT.itemsize == 12 and MLOOP_DT.itemsize == 8


@dataclass
class Mesh:
    verts: np.ndarray            # (V, 3) float32, object space
    normals: np.ndarray          # (V, 3) int16 (unit normal * 32767)
    tris: np.ndarray             # (T, 3) uint32 vertex indices
    mat_slot: np.ndarray         # (T,) int16 material slot per triangle
    slot_materials: list         # slot -> global material index
    matrix: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))


@dataclass
class Light:
    kind: str                    # 'A' area, 'S' sun, 'P' point
    color: tuple = (1.0, 1.0, 1.0)
    position: tuple = (0.0, 0.0, 0.0)
    width: float = 1.0
    height: float = 1.0
    rotation: tuple = (0.0, 0.0, 0.0)   # degrees (area), radians (sun)
    power: float = 1.0
    angle: float = 0.0
    radius: float = 0.0


@dataclass
class Material:
    kind: str                    # 'P' plastic, 'G' glass, 'M' metal, 'R' rough dielectric
    color: tuple = (1.0, 1.0, 1.0)
    ior: float = 1.5
    roughness: float = 0.0
    specular: float = 0.0


@dataclass
class Camera:
    width: int
    height: int
    position: tuple
    corners: tuple               # (top-right, bottom-right, bottom-left, top-left)


@dataclass
class Scene:
    meshes: list
    materials: list
    lights: list
    camera: Camera
    samples: int = 1
    base_radius: float = 0.01
    radius_reduction: float = 0.75
    name: str = "scene"

    def num_tris(self) -> int:
        return int(sum(len(m.tris) for m in self.meshes))


def look_at_camera(width, height, eye, target, up, fov_deg) -> Camera:
    """Pinhole camera with vertical field of view fov_deg, image plane at distance 1."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    h = np.tan(np.radians(fov_deg) / 2.0)
    w = h * width / height
    c = eye + fwd
    tr = c + right * w + upv * h
    br = c + right * w - upv * h
    bl = c - right * w - upv * h
    tl = c - right * w + upv * h
    return Camera(width, height, tuple(eye), (tuple(tr), tuple(br), tuple(bl), tuple(tl)))


class InitArgs:
    """The argument list of init(), with every buffer kept alive by this object."""

    def __init__(self, scene: Scene, debug_test: int = 1, debug_ior: float = 0.0):
        self.scene = scene
        n = len(scene.meshes)
        self._keep = []
        self.blobs = []
        ptrs = (C.c_longlong * max(n, 1))()
        mats = (abi.Matrix4x4 * max(n, 1))()
        nverts = (C.c_uint * max(n, 1))()
        ntris = (C.c_uint * max(n, 1))()
        midx = (C.POINTER(C.c_int) * max(n, 1))()
        for i, m in enumerate(scene.meshes):
            V = len(m.verts)
            T = len(m.tris)
            mv = np.zeros(max(V, 1), MVERT_DT)
            mv["co"][:V] = np.asarray(m.verts, np.float32)
            mv["no"][:V] = np.asarray(m.normals, np.int16)
            mp = np.zeros(max(T, 1), MPOLY_DT)
            mp["loopstart"][:T] = np.arange(T, dtype=np.int32) * 3
            mp["totloop"][:T] = 3
            mp["mat_nr"][:T] = np.asarray(m.mat_slot, np.int16)
            ml = np.zeros(max(3 * T, 1), MLOOP_DT)
            ml["v"][: 3 * T] = np.asarray(m.tris, np.uint32).reshape(-1)
            blob = np.zeros(abi.MESH_BLENDER_SIZE, np.uint8)
            for off, arr in ((abi.OFF_MPOLY, mp), (abi.OFF_MLOOP, ml), (abi.OFF_MVERT, mv)):
                blob[off:off + 8] = np.frombuffer(np.uint64(arr.ctypes.data).tobytes(), np.uint8)
            self._keep += [mv, mp, ml, blob]
            self.blobs.append(blob)
            ptrs[i] = blob.ctypes.data
            mats[i].t[:] = [float(v) for v in np.asarray(m.matrix, np.float32).reshape(-1)]
            nverts[i] = V
            ntris[i] = T
            slots = np.asarray(m.slot_materials, np.int32)
            self._keep.append(slots)
            midx[i] = slots.ctypes.data_as(C.POINTER(C.c_int))
        nl = len(scene.lights)
        lights = (abi.PythonLight * max(nl, 1))()
        for i, l in enumerate(scene.lights):
            L = lights[i]
            L.type = l.kind.encode()
            L.color[:] = [float(c) for c in l.color]
            L.position = abi.vec3(l.position)
            L.width, L.height, L.spread = float(l.width), float(l.height), 0.0
            L.rotation = abi.vec3(l.rotation)
            L.power, L.angle, L.radius = float(l.power), float(l.angle), float(l.radius)
        nm = len(scene.materials)
        mats_py = (abi.PythonMaterial * max(nm, 1))()
        for i, m in enumerate(scene.materials):
            P = mats_py[i]
            P.type = m.kind.encode()
            P.ior, P.roughness, P.specular = float(m.ior), float(m.roughness), float(m.specular)
            P.color[:] = [float(c) for c in m.color]
        cam = scene.camera
        self._keep += [ptrs, mats, nverts, ntris, midx, lights, mats_py]
        self.args = (
            int(scene.samples), float(scene.base_radius), float(scene.radius_reduction),
            ptrs, n, mats, nverts, ntris, int(cam.width), int(cam.height),
            abi.vec3(cam.position), abi.vec3(cam.corners[0]), abi.vec3(cam.corners[1]),
            abi.vec3(cam.corners[2]), abi.vec3(cam.corners[3]),
            lights, nl, mats_py, nm, midx, int(debug_test), abi.DebugStuff(specular=float(debug_ior)),
        )

    def call(self, init_fn):
        init_fn.argtypes = abi.INIT_ARGTYPES
        init_fn.restype = None
        init_fn(*self.args)

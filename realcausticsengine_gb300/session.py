"""Host-side session over the C ABI, shaped like the Blender add-on's use of the
reference DLL: init(...) with the scene's Blender data, then render, then read the
image.  All work runs in librealcaustics.so on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from ._native import check, lib
from .scene import InitArgs, Scene

STAT_NAMES = ["light_paths", "photons", "queries", "merged", "light_ms", "kd_ms", "camera_ms", "gather_ms",
              "accum_ms", "device_ms", "iterations", "scene_radius", "radius", "launches", "photon_tests",
              "chunks_tested", "light_rays"]


class Context:
    """A library context (rc_context_create).  Bound on a thread (`with ctx:` or
    bind()), it holds that thread's scene, settings, last error and device buffers, so
    scenes in different contexts render concurrently from different threads; threads
    that bind nothing share the default context."""

    def __init__(self):
        self.L = lib()
        self.handle = self.L.rc_context_create()
        if not self.handle:
            raise MemoryError("rc_context_create failed")

    def bind(self):
        check(self.L.rc_context_bind(self.handle), "rc_context_bind")

    @staticmethod
    def unbind():
        lib().rc_context_bind(None)

    def __enter__(self):
        self.bind()
        return self

    def __exit__(self, *exc):
        self.unbind()

    def destroy(self):
        if self.handle:
            check(self.L.rc_context_destroy(self.handle), "rc_context_destroy")
            self.handle = None


def batch_render(contexts, iterations: int) -> np.ndarray:
    """rc_batch_render: `iterations` more iterations of every scene held by `contexts`
    (Context objects, each with a scene loaded while it was bound) as one launch set per
    iteration.  Returns the call's timing record (device ms, batch iterations, kernel
    launches, iterations rendered again, light and camera pass ms of the last one)."""
    L = lib()
    handles = (C.c_void_p * len(contexts))(*[c.handle for c in contexts])
    out = np.zeros(6, np.float64)
    check(L.rc_batch_render(handles, len(contexts), iterations, out.ctypes.data), "rc_batch_render")
    return out


class Renderer:
    """One scene loaded into the library (the library holds one scene at a time,
    like the reference's global `scene`)."""

    def __init__(self, scene: Scene, max_path_length: int = 6, photons_per_iter: int = 0, seed: int = 0,
                 sampler: int = abi.SAMPLER_UNIFORM, verbose: bool = False, learned_proposal: bool = False,
                 train_iterations: int = 8, train_steps: int = 64, learning_rate: float = 1e-3,
                 camera_seed: int = 0, autotune: bool = True, graph_replay: bool = True, gpu_bvh: bool = True):
        self.scene = scene
        self.L = lib()
        cfg = abi.RcConfig()
        check(self.L.rc_default_config(C.byref(cfg)), "rc_default_config")
        cfg.max_path_length = max_path_length
        cfg.photons_per_iter = photons_per_iter
        cfg.seed = seed
        cfg.sampler = sampler
        cfg.write_exr = 0
        cfg.verbose = int(verbose)
        cfg.learned_proposal = int(learned_proposal)
        cfg.train_iterations = train_iterations
        cfg.train_steps = train_steps
        cfg.learning_rate = learning_rate
        cfg.camera_seed = camera_seed
        cfg.autotune = int(autotune)
        cfg.graph_replay = int(graph_replay)
        cfg.gpu_bvh = int(gpu_bvh)
        check(self.L.rc_set_config(C.byref(cfg)), "rc_set_config")
        self.args = InitArgs(scene)
        self.args.call(self.L.init)
        err = self.L.rc_last_error().decode()
        if err:
            raise RuntimeError(f"init failed: {err}")

    def prepare(self):
        check(self.L.rc_prepare(), "rc_prepare")

    def prepare_host(self) -> np.ndarray:
        info = (C.c_float * 9)()
        check(self.L.rc_prepare_host(info), "rc_prepare_host")
        return np.array(info, np.float32)

    def scene_dump(self, which: int) -> np.ndarray:
        """The scene arrays the kernels read (rc_scene_dump) as uint32 words."""
        n = C.c_longlong(0)
        check(self.L.rc_scene_dump(which, None, 0, C.byref(n)), "rc_scene_dump")
        out = np.zeros(n.value, np.uint32)
        check(self.L.rc_scene_dump(which, out.ctypes.data, n.value, C.byref(n)), "rc_scene_dump")
        return out

    def prepare_stats(self) -> dict:
        a = np.zeros(5, np.float64)
        self.L.rc_prepare_stats(a.ctypes.data, 5)
        return {"mesh_bvh_ms": a[0], "device_bvh": bool(a[1]), "rest_ms": a[2], "mesh_nodes": int(a[3]),
                "level_passes": int(a[4])}

    def render(self, iterations: int):
        check(self.L.rc_render(int(iterations)), "rc_render")

    def image(self) -> np.ndarray:
        W, H = self.scene.camera.width, self.scene.camera.height
        out = np.zeros((H, W, 3), np.float32)
        check(self.L.rc_read_image(out.ctypes.data, W, H), "rc_read_image")
        return out

    def stats(self) -> dict:
        a = np.zeros(len(STAT_NAMES), np.float64)
        check(self.L.rc_get_stats(a.ctypes.data, len(STAT_NAMES)), "rc_get_stats")
        return dict(zip(STAT_NAMES, a.tolist()))

    def trace(self, origins: np.ndarray, dirs: np.ndarray, tmin: float = 0.001, shape: int = 0) -> np.ndarray:
        """Closest hits (n, 16) through traversal `shape`: 0 the persistent passes',
        1 the wavefront pass's warp-stepped one, 2 pop-and-test (the reference's form)."""
        o = np.ascontiguousarray(origins, np.float32)
        d = np.ascontiguousarray(dirs, np.float32)
        n = len(o)
        out = np.zeros((n, 16), np.float32)
        check(self.L.rc_trace_rays_shape(n, o.ctypes.data, d.ctypes.data, C.c_float(tmin), out.ctypes.data,
                                         int(shape)), "rc_trace_rays_shape")
        return out

    def camera_queries(self, iteration: int) -> np.ndarray:
        """Merge queries of one camera pass: (n, 4) float32 [position xyz, camera dVM]."""
        n = C.c_longlong()
        check(self.L.rc_camera_queries(int(iteration), None, 0, C.byref(n)), "rc_camera_queries")
        out = np.zeros((max(n.value, 1), 4), np.float32)
        check(self.L.rc_camera_queries(int(iteration), out.ctypes.data, len(out), C.byref(n)), "rc_camera_queries")
        return out[:n.value]

    def light_photons_shape(self, shape: int, iteration: int) -> np.ndarray:
        """Photons of one light pass in launch shape `shape` (6: the wavefront pass)."""
        n = C.c_longlong()
        check(self.L.rc_light_photons_shape(shape, int(iteration), None, 0, C.byref(n)), "rc_light_photons_shape")
        out = np.zeros((max(n.value, 1), 12), np.float32)
        check(self.L.rc_light_photons_shape(shape, int(iteration), out.ctypes.data, len(out), C.byref(n)),
              "rc_light_photons_shape")
        return out[:n.value]

    def mlt_photons(self, variant: int, iteration: int):
        """Photons of one Metropolis light pass (PSSMLT variant 0: the render's chains, one
        path segment per loop iteration; 1: one step at a time) and its (visible large
        steps, large steps)."""
        n = C.c_longlong()
        st = np.zeros(2, np.uint64)
        check(self.L.rc_mlt_photons(variant, int(iteration), None, 0, C.byref(n), st.ctypes.data), "rc_mlt_photons")
        out = np.zeros((max(n.value, 1), 12), np.float32)
        check(self.L.rc_mlt_photons(variant, int(iteration), out.ctypes.data, len(out), C.byref(n), st.ctypes.data),
              "rc_mlt_photons")
        return out[:n.value], (int(st[0]), int(st[1]))

    def light_photons(self, iteration: int) -> np.ndarray:
        n = C.c_longlong()
        check(self.L.rc_light_photons(int(iteration), None, 0, C.byref(n)), "rc_light_photons")
        out = np.zeros((max(n.value, 1), 12), np.float32)
        check(self.L.rc_light_photons(int(iteration), out.ctypes.data, n.value, C.byref(n)), "rc_light_photons")
        return out[: n.value]

    def host_mesh_bvh(self, mesh: int, cap: int = 1 << 22, with_index: bool = False):
        nodes = np.zeros((cap, 8), np.uint32)
        idx = np.zeros(cap + 1, np.int32)
        cost = C.c_float()
        n = self.L.rc_host_mesh_bvh(mesh, nodes.ctypes.data, cap, idx.ctypes.data, cap + 1, C.byref(cost))
        if n < 0:
            check(n, "rc_host_mesh_bvh")
        if with_index:
            return nodes[:n], cost.value, idx
        return nodes[:n], cost.value

    def release(self):
        self.L.rc_release()


def kd_query(positions: np.ndarray, queries: np.ndarray, r2: float, with_indices: bool = True, variant: int = -1):
    """Radius query on caller-chosen photons through the render's own gather kernel
    (launch shape `variant`, -1 = default): (counts, [photon id arrays])."""
    L = lib()
    p = np.ascontiguousarray(positions, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    counts = np.zeros(len(q), np.int32)
    total = C.c_longlong()
    check(L.rc_gather_query(int(variant), len(p), p.ctypes.data, len(q), q.ctypes.data, C.c_float(r2),
                            counts.ctypes.data, None, 0, C.byref(total)), "rc_gather_query")
    if not with_indices:
        return counts, None
    idx = np.zeros(max(total.value, 1), np.int32)
    check(L.rc_gather_query(int(variant), len(p), p.ctypes.data, len(q), q.ctypes.data, C.c_float(r2),
                            counts.ctypes.data, idx.ctypes.data, len(idx), C.byref(total)), "rc_gather_query")
    offs = np.concatenate([[0], np.cumsum(counts)])
    return counts, [idx[offs[j]:offs[j + 1]] for j in range(len(q))]


def gather_variants() -> int:
    return int(lib().rc_gather_variants())


def kd_build_nodes(positions: np.ndarray) -> np.ndarray:
    L = lib()
    p = np.ascontiguousarray(positions, np.float32)
    nn = C.c_longlong()
    check(L.rc_kd_build_nodes(len(p), p.ctypes.data, None, 0, C.byref(nn)), "rc_kd_build_nodes")
    out = np.zeros((max(nn.value, 1), 2), np.uint32)
    check(L.rc_kd_build_nodes(len(p), p.ctypes.data, out.ctypes.data, nn.value, C.byref(nn)), "rc_kd_build_nodes")
    return out[:nn.value]

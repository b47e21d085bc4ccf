"""Generate tests/golden/reference_golden.npz from the reference itself.

Runs the reference compiled from its own sources (oracle/build_ref.sh ->
oracle/_ref/libref_oracle.so) on seeded synthetic inputs and stores its outputs:
  scene prep info, every mesh BVH and the world BVH, closest hits of random rays,
  KD-tree radius sets, BSDF sample/evaluate/pdf probes, light samples, the debug
  views (debug_test 2-4), and a full reference render (its own estimator and RNG
  stream).
Run in a fresh process (the reference keeps process-global RNG state):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from realcausticsengine_gb300 import abi, scenes  # noqa: E402
from realcausticsengine_gb300.scene import InitArgs  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_golden.npz"

MATERIALS = [("P", (0.8, 0.8, 0.8), 1.5, 1.0, 0.0), ("P", (0.3, 0.6, 0.9), 1.5, 0.05, 0.5),
             ("P", (0.9, 0.4, 0.3), 1.5, 0.6, 0.4), ("G", (1, 1, 1), 1.5, 0.0, 0.0),
             ("G", (1, 1, 1), 1.33, 0.0, 0.0), ("M", (0.9, 0.8, 0.6), 1.5, 0.3, 0.0),
             ("M", (1, 1, 1), 1.5, 0.0, 0.0), ("X", (1, 1, 1), 1.0, 0.0, 0.0)]


def scene_hash(args: InitArgs) -> str:
    h = hashlib.sha256()
    for b in args._keep:
        if isinstance(b, np.ndarray):
            if b.dtype == np.uint8 and b.size == abi.MESH_BLENDER_SIZE:
                continue   # holds pointers
            h.update(b.tobytes())
    return h.hexdigest()


def bsdf_inputs(rng, n):
    ng = rng.normal(size=(n, 3)); ng /= np.linalg.norm(ng, axis=1, keepdims=True)
    ns = ng + 0.1 * rng.normal(size=(n, 3)); ns /= np.linalg.norm(ns, axis=1, keepdims=True)
    ns *= rng.uniform(0.97, 1.0, (n, 1))
    d = rng.normal(size=(n, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True)
    isect = np.concatenate([ng, ns, d], 1).astype(np.float32)
    u = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    we = rng.normal(size=(n, 3)); we /= np.linalg.norm(we, axis=1, keepdims=True)
    return isect, u, we.astype(np.float32)


def main():
    ref = oracle.reference()
    if ref is None:
        raise SystemExit("reference sources not available; cannot generate fixtures")
    os.chdir(tempfile.mkdtemp())   # the reference writes D:\*.obj / .exr into the cwd
    rng = np.random.default_rng(20261203)
    g = {}
    # --- scene, BVHs, hits
    sc = scenes.test_scene(48, 36, subdiv=2, samples=2)
    args = InitArgs(sc)
    g["scene_hash"] = np.frombuffer(bytes.fromhex(scene_hash(args)), np.uint8)
    args.call(ref.init)
    info = (C.c_float * 9)()
    ref.ref_prepare(info)
    g["prep_info"] = np.array(info, np.float32)
    for m in range(len(sc.meshes)):
        cap = 1 << 14
        nodes = np.zeros((cap, 8), np.uint32); idx = np.zeros(cap, np.int32); cost = C.c_float()
        n = ref.ref_mesh_bvh(m, nodes.ctypes.data, cap, idx.ctypes.data, cap, C.byref(cost))
        g[f"mesh{m}_nodes"] = nodes[:n]
        g[f"mesh{m}_index"] = idx[:len(sc.meshes[m].tris) + 1]
        g[f"mesh{m}_cost"] = np.array([cost.value], np.float32)
    wn = np.zeros((256, 8), np.uint32); wi = np.zeros(256, np.int32)
    n = ref.ref_world_bvh(wn.ctypes.data, 256, wi.ctypes.data, 256)
    g["world_nodes"] = wn[:n]
    g["world_index"] = wi[:len(sc.meshes) + 1]
    nr = 4000
    o = rng.uniform(-4, 4, (nr, 3)).astype(np.float32); o[:, 2] = rng.uniform(0.2, 5, nr)
    d = rng.normal(size=(nr, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True); d = d.astype(np.float32)
    # half of the rays aimed at scene points, so most hit something
    tgt = rng.uniform(-2.5, 2.5, (nr // 2, 3)); tgt[:, 2] = rng.uniform(0.0, 1.6, nr // 2)
    dd = tgt - o[: nr // 2]; dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    d[: nr // 2] = dd.astype(np.float32)
    hits = np.zeros((nr, 16), np.float32)
    ref.ref_trace(nr, o.ctypes.data, d.ctypes.data, C.c_float(0.001), hits.ctypes.data)
    g["ray_o"], g["ray_d"], g["ray_hits"] = o, d, hits
    # --- light samples (primary samples in the reference's storage order)
    nl = 400
    lu = rng.uniform(0, 1, (nl, 8)).astype(np.float32)
    lo = np.zeros((nl, 10), np.float32)
    for i in range(nl):
        ref.ref_light_sample(lu[i].ctypes.data, lo[i].ctypes.data)
    g["light_u"], g["light_out"] = lu, lo
    # --- BSDF probes
    for k, (t, col, ior, rough, spec) in enumerate(MATERIALS):
        pm = abi.PythonMaterial(); pm.type = t.encode(); pm.ior = ior; pm.roughness = rough; pm.specular = spec
        pm.color[:] = col
        isect, u, we = bsdf_inputs(rng, 300)
        out = np.zeros((300, 2, 23), np.float32)
        for i in range(300):
            for mode in (0, 1):
                ref.ref_bsdf(C.byref(pm), isect[i].ctypes.data, mode, u[i].ctypes.data, we[i].ctypes.data,
                             out[i, mode].ctypes.data)
        g[f"bsdf{k}_mat"] = np.frombuffer(bytes(pm), np.uint8).copy()
        g[f"bsdf{k}_isect"], g[f"bsdf{k}_u"], g[f"bsdf{k}_we"], g[f"bsdf{k}_out"] = isect, u, we, out
    ref.ref_release()
    # --- KD radius sets (tree order as the reference visits; sets compared sorted)
    for k, (n, q, r) in enumerate([(1, 8, 0.5), (2, 8, 0.5), (7, 16, 0.4), (600, 100, 0.12), (6000, 200, 0.05)]):
        pos = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
        if n >= 600:
            pos[: n // 10] = np.round(pos[: n // 10] * 8) / 8   # duplicated coordinates (ties)
        qp = rng.uniform(-1.1, 1.1, (q, 3)).astype(np.float32)
        cnt = np.zeros(q, np.int32); idx = np.zeros(n * q, np.int32)
        tot = ref.ref_kd_query(n, pos.ctypes.data, q, qp.ctypes.data, C.c_float(np.float32(r * r)), cnt.ctypes.data,
                               idx.ctypes.data, len(idx))
        g[f"kd{k}_pos"], g[f"kd{k}_q"], g[f"kd{k}_r2"] = pos, qp, np.array([r * r], np.float32)
        g[f"kd{k}_counts"], g[f"kd{k}_idx"] = cnt, idx[:tot]
    # --- debug views (debug_test 2-4, Debug_stuff::specular = 1.5)
    for mode in (2, 3, 4):
        args = InitArgs(sc, debug_test=mode, debug_ior=1.5)
        args.call(ref.init)
        ref.ref_prepare(None)
        img = np.zeros(3 * 48 * 36, np.float32)
        assert ref.ref_debug(mode, img.ctypes.data) == 0
        g[f"debug{mode}_image"] = img
    # --- full render by the reference integrator (fresh RNG state matters: do it last
    # in a process whose earlier calls consumed the stream? no - re-init resets nothing,
    # so the render runs in a child process)
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


def render_child():
    ref = oracle.reference()
    os.chdir(tempfile.mkdtemp())
    sc = scenes.test_scene(48, 36, subdiv=2, samples=2)
    args = InitArgs(sc)
    args.call(ref.init)
    ref.ref_prepare(None)
    img = np.zeros(3 * 48 * 36, np.float32)
    ref.ref_render(img.ctypes.data)
    return img


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--render":
        img = render_child()
        np.save(sys.argv[2], img)
    else:
        main()
        import subprocess
        tmp = Path(tempfile.mkdtemp()) / "render.npy"
        subprocess.run([sys.executable, __file__, "--render", str(tmp)], check=True, stdout=subprocess.DEVNULL)
        g = dict(np.load(OUT))
        g["render_image"] = np.load(tmp)
        np.savez_compressed(OUT, **g)
        print(f"added reference render; {OUT.stat().st_size} bytes")

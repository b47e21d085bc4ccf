"""Closest hits at the workloads' own sizes, bit for bit against the oracle's
restatement of Scene::hit (src/Scene.cpp:154-189, world leaves src/BVH/BVH_world.cpp:267-283,
Möller-Trumbore src/Triangle.cpp:20-88), which is pinned to the compiled reference.

The GPU path builds the mesh BVHs on the device (word-for-word the host build) and
traverses them with each of its traversals; the oracle builds its own host BVH.  Every field of every ray's hit
record must match: t, u, v, Ng, Ns, position, front face, material, triangle id.
"""
import ctypes as C

import numpy as np
import pytest

from realcausticsengine_gb300 import scenes
from realcausticsengine_gb300.scene import InitArgs
from realcausticsengine_gb300.session import Renderer

pytestmark = pytest.mark.gpu


def _rays(rng, n, lo, hi, zlo, zhi, aim_lo, aim_hi, aim_z):
    """Origins in a box; half the rays aimed at random points of a target box, the rest
    in uniformly random directions."""
    o = np.stack([rng.uniform(lo, hi, n), rng.uniform(lo, hi, n), rng.uniform(zlo, zhi, n)], 1)
    d = rng.normal(size=(n, 3))
    t = np.stack([rng.uniform(aim_lo, aim_hi, n // 2), rng.uniform(aim_lo, aim_hi, n // 2),
                  rng.uniform(aim_z[0], aim_z[1], n // 2)], 1)
    d[: n // 2] = t - o[: n // 2]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def _compare(orc, sc, o, d, min_hit_frac):
    """Every GPU traversal (0: the persistent passes', 1: the wavefront pass's
    warp-stepped one, 2: pop-and-test) against the oracle."""
    r = Renderer(sc)
    got = [r.trace(o, d, shape=k) for k in (0, 1, 2)]
    r.release()
    InitArgs(sc).call(orc.oracle_init)
    assert orc.oracle_prepare(None) == 0
    want = np.zeros((len(o), 16), np.float32)
    orc.oracle_trace(len(o), o.ctypes.data, d.ctypes.data, C.c_float(0.001), want.ctypes.data, 32)
    assert want[:, 0].mean() > min_hit_frac
    for k, g in enumerate(got):
        mism = (g.view(np.uint32) != want.view(np.uint32)).any(1)
        assert not mism.any(), f"traversal {k}: {int(mism.sum())} of {len(o)} rays differ"


def test_hits_water_pool_full_grid(orc):
    """The 512x512-vertex water height field (522,242 triangles) and its floor."""
    sc = scenes.water_pool(64, 36, grid=512)
    rng = np.random.default_rng(31)
    o, d = _rays(rng, 60000, -5.0, 5.0, -1.4, 4.0, -5.0, 5.0, (-1.5, 0.1))
    _compare(orc, sc, o, d, 0.5)


@pytest.mark.parametrize("groups", [1, 16])
def test_hits_gem_cluster(orc, groups):
    """2,000 faceted gems (2,001 materials) in one mesh, and grouped into 16 meshes, so
    that the world BVH has many leaves and the reference's world-leaf overwrite (the
    last-visited mesh's own closest hit wins) decides many rays."""
    sc = scenes.gem_cluster(64, 36, groups=groups)
    rng = np.random.default_rng(40 + groups)
    o, d = _rays(rng, 60000, -3.5, 3.5, 0.02, 3.0, -3.2, 3.2, (0.0, 0.3))
    _compare(orc, sc, o, d, 0.5)


@pytest.mark.parametrize("seed", [1, 34])
def test_hits_batch_scenes(orc, seed):
    """Two scenes of the 64-scene batch: displaced glass spheres of 107k and 1.7M
    triangles over a plane."""
    sc, _ = scenes.batch_scene(seed, 32, 32)
    rng = np.random.default_rng(50 + seed)
    o, d = _rays(rng, 60000, -3.0, 3.0, 0.05, 4.0, -1.2, 1.2, (0.2, 2.6))
    _compare(orc, sc, o, d, 0.5)

"""Device SAH BVH build (bvh_build.cu) against the host build.

The host build is pinned to the reference's own build (tests/test_abi.py compares
node arrays, triangle lists and traversal costs with the compiled reference); here the
scene arrays the kernels read - mesh nodes, triangle records in leaf order, the world
BVH built from the device's mesh bounds and costs, mesh roots - must be word-for-word
the same whichever side built the mesh BVHs.
"""
import numpy as np
import pytest

from realcausticsengine_gb300 import scenes
from realcausticsengine_gb300.scene import Camera, Light, Material, Mesh, Scene, look_at_camera

pytestmark = pytest.mark.gpu


def _dumps(sc, gpu_bvh):
    from realcausticsengine_gb300.session import Renderer
    r = Renderer(sc, max_path_length=4, photons_per_iter=4096, gpu_bvh=gpu_bvh)
    r.prepare()
    out = [r.scene_dump(w) for w in range(4)]
    st = r.prepare_stats()
    r.release()
    return out, st


def _mesh(V, F, mat=0, matrix=None):
    V = np.asarray(V, np.float32)
    F = np.asarray(F, np.uint32)
    N = np.tile(np.array([[0, 0, 32767]], np.int16), (len(V), 1))
    return Mesh(V, N, F, np.zeros(len(F), np.int16), [mat],
                np.eye(4, dtype=np.float32) if matrix is None else np.asarray(matrix, np.float32))


def _scene(meshes):
    mats = [Material("P", color=(0.8, 0.8, 0.8), roughness=1.0), Material("G", ior=1.5)]
    lights = [Light("A", position=(0.0, 0.0, 6.0), width=2.0, height=2.0, power=10.0)]
    cam = look_at_camera(32, 24, (0.0, -6.0, 5.0), (0.0, 0.0, 0.0), (0, 0, 1), 40.0)
    return Scene(meshes, mats, lights, cam, samples=1, name="bvh_edges")


def _edge_scene():
    rng = np.random.default_rng(7)
    one = _mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])
    two = _mesh([[0, 0, 1], [1, 0, 1], [0, 1, 1], [1, 1, 1]], [[0, 1, 2], [1, 3, 2]])
    three = _mesh(rng.uniform(-1, 1, (9, 3)), np.arange(9).reshape(3, 3))
    # 5000 copies of one triangle: flat centroid bounds, a 5000-triangle leaf decided
    # in the level passes
    same = _mesh([[0, 0, 2], [0.5, 0, 2], [0, 0.5, 2]], np.tile([[0, 1, 2]], (5000, 1)))
    # two clusters of coincident triangles: bucket ties and duplicated centroids
    V = np.concatenate([rng.uniform(-2, -1.9, (3000, 3)), rng.uniform(1.9, 2, (3000, 3))]).astype(np.float32)
    F = np.arange(6000).reshape(2000, 3)
    F = np.concatenate([F, F, F])
    clusters = _mesh(V, F, 1)
    # random soup above the segment size handled per warp
    soup_v = rng.uniform(-3, 3, (3 * 20000, 3)).astype(np.float32)
    soup_v = soup_v.reshape(20000, 3, 3)
    soup_v = (soup_v[:, :1] + 0.05 * (soup_v - soup_v[:, :1])).reshape(-1, 3)
    soup = _mesh(soup_v, np.arange(60000).reshape(20000, 3))
    # axis-aligned flat grid (zero extent in z, equal centroid coordinates in rows)
    g = 120
    xs, ys = np.meshgrid(np.linspace(-4, 4, g), np.linspace(-4, 4, g))
    Vg = np.stack([xs.ravel(), ys.ravel(), np.full(g * g, -0.5)], 1)
    Fg = []
    for i in range(g - 1):
        for j in range(g - 1):
            a = i * g + j
            Fg += [[a, a + 1, a + g], [a + 1, a + g + 1, a + g]]
    grid = _mesh(Vg, Fg)
    return _scene([one, two, three, same, clusters, soup, grid])


def _random_meshes_scene(seed=3, count=40):
    """Many meshes of random sizes (1 to 30,000 triangles): soups of small random
    triangles, random grids and stretched slabs, so that segments cross the per-warp size
    at every depth and the world BVH has many leaves."""
    rng = np.random.default_rng(seed)
    meshes = []
    for m in range(count):
        n = int(np.exp(rng.uniform(0.0, np.log(30000.0))))
        centre = rng.uniform(-4, 4, 3)
        scale = rng.uniform(0.05, 2.0, 3)
        kind = m % 3
        if kind == 0:   # soup
            base = centre + rng.uniform(-1, 1, (n, 1, 3)) * scale
            V = (base + rng.normal(0, 0.02, (n, 3, 3))).reshape(-1, 3)
            F = np.arange(3 * n).reshape(n, 3)
        elif kind == 1:  # grid with random heights
            g = max(2, int(np.sqrt(n / 2)) + 1)
            xs, ys = np.meshgrid(np.linspace(-1, 1, g), np.linspace(-1, 1, g))
            V = np.stack([xs.ravel(), ys.ravel(), rng.normal(0, 0.05, g * g)], 1) * scale + centre
            F = []
            for i in range(g - 1):
                for j in range(g - 1):
                    a = i * g + j
                    F += [[a, a + 1, a + g], [a + 1, a + g + 1, a + g]]
            F = np.asarray(F)
        else:            # thin slab: flat on one axis
            V = rng.uniform(-1, 1, (3 * n, 3)) * scale + centre
            V[:, m % 3 - 1] = centre[m % 3 - 1]
            F = np.arange(3 * n).reshape(n, 3)
        meshes.append(_mesh(V, F, m % 2))
    return _scene(meshes)


SCENES = {
    "test_scene": lambda: scenes.test_scene(),
    "glass_sphere": lambda: scenes.glass_sphere_point(64, 64, subdiv=5),
    "water_pool_256": lambda: scenes.water_pool(64, 36, grid=256),
    "gem_cluster_4": lambda: scenes.gem_cluster(64, 36, n_gems=300, groups=4),
    "batch_0": lambda: scenes.batch_scene(0, 32, 32)[0],
    "batch_5": lambda: scenes.batch_scene(5, 32, 32)[0],
    "edges": _edge_scene,
    "random_meshes": _random_meshes_scene,
}


@pytest.mark.parametrize("name", list(SCENES))
def test_device_bvh_matches_host(name):
    sc = SCENES[name]()
    dev, st_dev = _dumps(sc, True)
    host, st_host = _dumps(sc, False)
    assert st_dev["device_bvh"] and not st_host["device_bvh"]
    for w, (a, b) in enumerate(zip(dev, host)):
        assert a.shape == b.shape, (w, a.shape, b.shape)
        diff = np.nonzero(a != b)[0]
        assert len(diff) == 0, (w, diff[:8], a[diff[:8]], b[diff[:8]])


def test_device_bvh_water_pool_full():
    """The 522,242-triangle water pool (the benchmark scene), level passes included."""
    sc = scenes.water_pool(64, 36, grid=512)
    dev, st_dev = _dumps(sc, True)
    host, _ = _dumps(sc, False)
    assert st_dev["device_bvh"] and st_dev["level_passes"] > 0
    for a, b in zip(dev, host):
        assert a.shape == b.shape and (a == b).all()


def test_negative_zero_falls_back_to_host():
    """A triangle box coordinate of -0.0 (translation -0.0 keeps the sign) is outside
    the device build's domain: the host builds that scene, with the same arrays."""
    m = np.eye(4, dtype=np.float32)
    m[0, 3] = -0.0
    tri = _mesh([[-0.0, -1, -1], [1, -1, -1], [1, 1, -1]], [[0, 1, 2]], matrix=m)
    sc = _scene([tri, _mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])])
    dev, st_dev = _dumps(sc, True)
    host, _ = _dumps(sc, False)
    assert not st_dev["device_bvh"]
    for a, b in zip(dev, host):
        assert (a == b).all()

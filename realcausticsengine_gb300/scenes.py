"""Seeded synthetic scenes (z-up, as the reference's area lights emit along -z).

Workloads (sizes as specified; coordinates mapped from the y-up wording by
(x, y, z) -> (x, -z, y)):
  glass_sphere_point   glass icosphere subdiv 5 (20,480 tris, r=1, IOR 1.5) 1.2 above a
                       10x10 diffuse plane (albedo 0.8), point light 5 above, 512x512,
                       fov 40, camera at (0,-4,4); 1M photons/iter, 16 iters, merge
                       radius 0.005 x scene diameter, max depth 8
  water_pool           512x512-vertex heightfield over [-5,5]^2 (522,242 tris), sum of
                       32 sines (wavelength log-uniform [0.2,3], amplitude ~ wl^1.5, max
                       0.05), GGX dielectric roughness 0.02 IOR 1.33, diffuse floor 1.5
                       below, 2x2 area light at height 6, 1920x1080, 16M photons/iter
  gem_cluster          2,000 convex polyhedra of 60-200 facets (~260k triangles), IOR
                       U(1.5,2.4), roughness U(0,0.05), per-channel IOR spread 0.02, 8 area
                       lights of random size and colour, 3840x2160; 65,536 PSSMLT chains,
                       large-step probability 0.3, 32M photons/iter
  small test scenes    the same ingredients at sizes the CPU oracle finishes in seconds
"""
from __future__ import annotations

import numpy as np

from .scene import Camera, Light, Material, Mesh, Scene, look_at_camera


def _normals_i16(n: np.ndarray) -> np.ndarray:
    n = n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-20)
    return np.round(n * 32767.0).astype(np.int16)


def icosphere(subdiv: int, radius: float = 1.0):
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = f
    for _ in range(subdiv):
        cache = {}
        nf = []

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[k] = len(verts) - 1
            return cache[k]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts)
    return (V * radius).astype(np.float32), _normals_i16(V), np.array(faces, np.uint32)


def plane(size: float, z: float = 0.0):
    h = size / 2.0
    V = np.array([(-h, -h, z), (h, -h, z), (h, h, z), (-h, h, z)], np.float32)
    N = _normals_i16(np.tile([[0.0, 0.0, 1.0]], (4, 1)))
    F = np.array([(0, 1, 2), (0, 2, 3)], np.uint32)
    return V, N, F


def box(sx, sy, sz):
    """Axis-aligned box with flat faces (4 vertices per face)."""
    V, N, F = [], [], []
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            n = np.zeros(3); n[axis] = sgn
            u = np.zeros(3); u[(axis + 1) % 3] = 1.0
            w = np.cross(n, u)
            half = np.array([sx, sy, sz]) / 2.0
            c = n * half
            corners = [c + (a * u + b * w) * half for a, b in ((-1, -1), (1, -1), (1, 1), (-1, 1))]
            base = len(V)
            V += corners
            N += [n] * 4
            F += [(base, base + 1, base + 2), (base, base + 2, base + 3)]
    return np.array(V, np.float32), _normals_i16(np.array(N)), np.array(F, np.uint32)


def translate(x, y, z, s=1.0):
    m = np.eye(4, dtype=np.float32) * np.float32(s)
    m[3, 3] = 1.0
    m[:3, 3] = (x, y, z)
    return m


def rotation_xyz(rx, ry, rz):
    cx, sx, cy, sy, cz, sz = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry), np.cos(rz), np.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    m = np.eye(4)
    m[:3, :3] = Rz @ Ry @ Rx
    return m.astype(np.float32)


def _mesh(V, N, F, mat_index, matrix=None):
    return Mesh(V, N, F, np.zeros(len(F), np.int16), [mat_index],
                np.eye(4, dtype=np.float32) if matrix is None else np.asarray(matrix, np.float32))


def glass_sphere_point(width=512, height=512, subdiv=5, samples=16, light="point") -> Scene:
    """Glass icosphere over a diffuse plane, lit by a point light (or an area light,
    which the reference can render, when light='area')."""
    mats = [Material("G", color=(1, 1, 1), ior=1.5), Material("P", color=(0.8, 0.8, 0.8), roughness=1.0, specular=0.0)]
    Vs, Ns, Fs = icosphere(subdiv, 1.0)
    Vp, Np, Fp = plane(10.0, 0.0)
    meshes = [_mesh(Vs, Ns, Fs, 0, translate(0, 0, 1.2)), _mesh(Vp, Np, Fp, 1)]
    if light == "point":
        lights = [Light("P", color=(1, 1, 1), position=(0, 0, 5), power=40.0)]
    else:
        lights = [Light("A", color=(1, 1, 1), position=(0, 0, 5), width=1.0, height=1.0, power=40.0)]
    cam = look_at_camera(width, height, (0, -4, 4), (0, 0, 0.8), (0, 0, 1), 40.0)
    return Scene(meshes, mats, lights, cam, samples=samples, base_radius=0.01, radius_reduction=0.75,
                 name=f"glass_sphere_{light}")


def water_heightfield(n=512, size=10.0, waves=32, seed=0):
    rng = np.random.default_rng(seed)
    lam = np.exp(rng.uniform(np.log(0.2), np.log(3.0), waves))
    amp = 0.05 * (lam / lam.max()) ** 1.5
    ang = rng.uniform(0, 2 * np.pi, waves)
    ph = rng.uniform(0, 2 * np.pi, waves)
    xs = np.linspace(-size / 2, size / 2, n)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    H = np.zeros_like(X)
    dHx = np.zeros_like(X)
    dHy = np.zeros_like(X)
    for k in range(waves):
        kx, ky = np.cos(ang[k]) * 2 * np.pi / lam[k], np.sin(ang[k]) * 2 * np.pi / lam[k]
        arg = kx * X + ky * Y + ph[k]
        H += amp[k] * np.sin(arg)
        dHx += amp[k] * kx * np.cos(arg)
        dHy += amp[k] * ky * np.cos(arg)
    V = np.stack([X, Y, H], -1).reshape(-1, 3).astype(np.float32)
    N = _normals_i16(np.stack([-dHx, -dHy, np.ones_like(H)], -1).reshape(-1, 3))
    i = np.arange(n - 1)
    a = (i[None, :] + n * i[:, None]).reshape(-1)
    F = np.concatenate([np.stack([a, a + 1, a + n + 1], -1), np.stack([a, a + n + 1, a + n], -1)]).astype(np.uint32)
    return V, N, F


def water_pool(width=1920, height=1080, grid=512, samples=64, roughness=0.02) -> Scene:
    mats = [Material("R", color=(1, 1, 1), ior=1.33, roughness=roughness),
            Material("P", color=(0.8, 0.8, 0.8), roughness=1.0, specular=0.0)]
    Vw, Nw, Fw = water_heightfield(grid)
    Vf, Nf, Ff = plane(10.0, -1.5)
    meshes = [_mesh(Vw, Nw, Fw, 0), _mesh(Vf, Nf, Ff, 1)]
    lights = [Light("A", color=(1, 1, 1), position=(0, 0, 6), width=2.0, height=2.0, power=30.0)]
    cam = look_at_camera(width, height, (0, -7.5, 5.5), (0, 0, -1.5), (0, 0, 1), 50.0)
    return Scene(meshes, mats, lights, cam, samples=samples, base_radius=0.0015, radius_reduction=0.75,
                 name="water_pool")


def test_scene(width=64, height=48, subdiv=2, samples=2, rough_glass=False, dispersion=0.0) -> Scene:
    """Small scene for CPU parity: glass sphere, rough metal sphere, smooth and rough
    plastic boxes with rotations, a diffuse floor, an area light (reference-renderable
    unless rough_glass or dispersion; dispersion > 0 makes the sphere an 'R' dielectric
    with that per-channel IOR spread)."""
    glass = "R" if (rough_glass or dispersion > 0) else "G"
    mats = [Material(glass, color=(1, 1, 1), ior=1.5, roughness=0.1 if rough_glass else 0.0, specular=dispersion),
            Material("P", color=(0.8, 0.8, 0.8), roughness=1.0, specular=0.0),
            Material("M", color=(0.9, 0.8, 0.6), roughness=0.3),
            Material("P", color=(0.3, 0.6, 0.9), roughness=0.05, specular=0.5),
            Material("M", color=(1.0, 1.0, 1.0), roughness=0.0),
            Material("P", color=(0.9, 0.4, 0.3), roughness=0.6, specular=0.4)]
    Vs, Ns, Fs = icosphere(subdiv, 1.0)
    Vp, Np, Fp = plane(8.0, 0.0)
    Vb, Nb, Fb = box(1.0, 1.0, 1.0)
    meshes = [
        _mesh(Vs, Ns, Fs, 0, translate(0.0, 0.0, 1.1)),
        _mesh(Vp, Np, Fp, 1),
        _mesh(Vs, Ns, Fs, 2, translate(-2.0, 0.8, 0.6) @ np.diag([0.6, 0.6, 0.6, 1]).astype(np.float32)),
        _mesh(Vb, Nb, Fb, 3, translate(2.0, 0.5, 0.5) @ rotation_xyz(0.3, 0.2, 0.7)),
        _mesh(Vb, Nb, Fb, 4, translate(1.2, -1.5, 0.35) @ rotation_xyz(0.0, 0.0, 0.4) @ np.diag([1.5, 0.2, 0.7, 1]).astype(np.float32)),
        _mesh(Vs, Ns, Fs, 5, translate(-1.0, -1.6, 0.4) @ np.diag([0.4, 0.4, 0.4, 1]).astype(np.float32)),
    ]
    lights = [Light("A", color=(1, 1, 1), position=(0.5, 0.3, 4.0), width=1.0, height=0.8, rotation=(10.0, -15.0, 5.0),
                    power=25.0),
              Light("A", color=(1.0, 0.8, 0.6), position=(-2.0, 1.0, 3.5), width=0.5, height=0.5, power=8.0)]
    cam = look_at_camera(width, height, (0.3, -5.5, 3.8), (0, 0, 0.6), (0, 0, 1), 45.0)
    return Scene(meshes, mats, lights, cam, samples=samples, base_radius=0.03, radius_reduction=0.75, name="test_scene")


def sun_scene(width=48, height=32) -> Scene:
    s = test_scene(width, height, subdiv=1)
    s.lights = [Light("S", color=(1, 1, 0.9), rotation=(0.3, -0.2, 0.5), power=3.0)]
    s.name = "sun_scene"
    return s


def _convex_gem(rng, n_points: int):
    """A convex polyhedron: the hull of random points on an ellipsoid, flat-shaded
    (vertices repeated per facet, normals = outward facet normals)."""
    from scipy.spatial import ConvexHull
    axes = np.array([1.0, rng.uniform(0.6, 1.0), rng.uniform(0.4, 0.8)])
    p = rng.normal(size=(n_points, 3))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    p *= axes
    hull = ConvexHull(p)
    tris = hull.simplices.copy()
    a, b, c = p[tris[:, 0]], p[tris[:, 1]], p[tris[:, 2]]
    n = np.cross(b - a, c - a)
    flip = (n * hull.equations[:, :3]).sum(1) < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]
    n[flip] = -n[flip]
    V = p[tris.reshape(-1)]
    N = np.repeat(n, 3, axis=0)
    F = np.arange(len(V), dtype=np.uint32).reshape(-1, 3)
    return V, N, F


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def gem_cluster(width=3840, height=2160, n_gems=2000, groups=1, seed=0, dispersion=0.02, samples=128) -> Scene:
    """Faceted gem cluster: `n_gems` randomly rotated and scaled convex polyhedra of
    60-200 triangular facets (hulls of 32-102 points on random ellipsoids), IOR
    U(1.5, 2.4), roughness U(0, 0.05), per-channel IOR spread `dispersion` (material 'R'),
    on a 12x12 diffuse plane, lit by 8 area lights of random size and colour; the gems
    are grouped into `groups` meshes by square tiles of the cluster (one mesh by
    default: with several world leaves the reference's world-leaf overwrite makes the
    last leaf's hit win, so grouping changes the image as well as the traversal cost)."""
    rng = np.random.default_rng(seed)
    mats = [Material("P", color=(0.8, 0.8, 0.8), roughness=1.0, specular=0.0)]
    meshes = []
    Vp, Np, Fp = plane(12.0, 0.0)
    meshes.append(_mesh(Vp, Np, Fp, 0))
    # positions first, then spatially coherent groups (tiles of a square grid, so the
    # group meshes' boxes do not all overlap)
    rad = 3.2 * np.sqrt(rng.uniform(size=n_gems))
    ang = rng.uniform(0, 2 * np.pi, n_gems)
    xy = np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1)
    side = max(1, int(round(np.sqrt(groups))))
    cell = np.clip(((xy + 3.2) / 6.4 * side).astype(int), 0, side - 1)
    gid = cell[:, 0] * side + cell[:, 1]
    for g in range(side * side):
        members = np.nonzero(gid == g)[0]
        if len(members) == 0:
            continue
        Vs, Ns, Fs, Ms = [], [], [], []
        base = 0
        slots = []
        for k in members:
            V, N, F = _convex_gem(rng, int(rng.integers(32, 103)))
            R = _rotation(rng)
            scale = rng.uniform(0.06, 0.22)
            pos = np.array([xy[k, 0], xy[k, 1], 0.0])
            V = (V @ R.T) * scale
            pos[2] = -V[:, 2].min() + 0.002
            Vs.append((V + pos).astype(np.float32))
            Ns.append(N @ R.T)
            Fs.append(F + base)
            base += len(V)
            mats.append(Material("R", color=(1, 1, 1), ior=float(rng.uniform(1.5, 2.4)),
                                 roughness=float(rng.uniform(0.0, 0.05)), specular=dispersion))
            slots.append(len(mats) - 1)
            Ms.append(np.full(len(F), len(slots) - 1, np.int16))
        V = np.concatenate(Vs)
        N = _normals_i16(np.concatenate(Ns))
        F = np.concatenate(Fs).astype(np.uint32)
        meshes.append(Mesh(V, N, F, np.concatenate(Ms), slots, np.eye(4, dtype=np.float32)))
    lights = []
    for i in range(8):
        a = 2 * np.pi * i / 8 + rng.uniform(-0.2, 0.2)
        rr = rng.uniform(1.5, 4.0)
        hue = rng.uniform(0, 1)
        col = tuple(float(0.6 + 0.4 * np.cos(2 * np.pi * (hue + o))) for o in (0.0, 1 / 3, 2 / 3))
        w = rng.uniform(0.3, 1.5)
        lights.append(Light("A", color=col, position=(rr * np.cos(a), rr * np.sin(a), rng.uniform(4.5, 6.5)),
                            width=w, height=w * rng.uniform(0.5, 1.5), power=float(rng.uniform(6.0, 14.0))))
    cam = look_at_camera(width, height, (0.0, -8.5, 6.0), (0.0, 0.0, 0.0), (0, 0, 1), 42.0)
    return Scene(meshes, mats, lights, cam, samples=samples, base_radius=0.0012, radius_reduction=0.75,
                 name="gem_cluster")


def geodesic_sphere(freq: int):
    """Unit sphere from the icosahedron with every face cut into freq^2 triangles
    (20 freq^2 in all), vertices shared between faces."""
    V0, _, F0 = icosphere(0, 1.0)
    V0 = V0.astype(np.float64)
    V0 /= np.linalg.norm(V0, axis=1, keepdims=True)
    i, j = np.meshgrid(np.arange(freq + 1), np.arange(freq + 1), indexing="ij")
    keep = i + j <= freq
    i, j = i[keep], j[keep]
    index = -np.ones((freq + 1, freq + 1), np.int64)
    index[i, j] = np.arange(len(i))
    # the triangles of one face in local (i, j) grid indices
    ti, tj = np.meshgrid(np.arange(freq), np.arange(freq), indexing="ij")
    up = ti + tj < freq
    down = ti + tj < freq - 1
    local = np.concatenate([
        np.stack([index[ti[up], tj[up]], index[ti[up] + 1, tj[up]], index[ti[up], tj[up] + 1]], 1),
        np.stack([index[ti[down] + 1, tj[down]], index[ti[down] + 1, tj[down] + 1], index[ti[down], tj[down] + 1]], 1)])
    Vs, Fs = [], []
    for f, (a_, b_, c_) in enumerate(F0):
        A, B, C = V0[a_], V0[b_], V0[c_]
        P = (A[None] * (freq - i - j)[:, None] + B[None] * i[:, None] + C[None] * j[:, None]) / freq
        Vs.append(P / np.linalg.norm(P, axis=1, keepdims=True))
        Fs.append(local + f * len(i))
    V = np.concatenate(Vs)
    F = np.concatenate(Fs)
    # weld the copies of edge and corner vertices
    key = np.round(V * 1e7).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    return V[first], inv.reshape(-1)[F]


def displaced_glass_sphere(rng, tris: float, amplitude: float, radius: float = 1.0):
    """Geodesic sphere of about `tris` triangles whose vertices move along the normal by
    amplitude x a smooth noise in [-1, 1] (a sum of 6 random sinusoids of the unit
    position); smooth normals from the displaced faces."""
    freq = max(2, int(round(np.sqrt(tris / 20.0))))
    U, F = geodesic_sphere(freq)
    k = rng.normal(size=(6, 3)) * rng.uniform(2.0, 6.0, (6, 1))
    ph = rng.uniform(0, 2 * np.pi, 6)
    noise = np.sin(U @ k.T + ph).sum(1)
    noise /= max(np.abs(noise).max(), 1e-12)
    V = U * (radius * (1.0 + amplitude * noise))[:, None]
    fn = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    N = np.zeros_like(V)
    for c in range(3):
        np.add.at(N, F[:, c], fn)
    return V.astype(np.float32), _normals_i16(N), F.astype(np.uint32)


def batch_scene(seed: int, width=512, height=512):
    """One scene of the 64-scene batch: a displaced glass sphere (vertex noise amplitude
    U(0, 0.2)) of log-uniform [1k, 2M] triangles, IOR U(1.3, 1.8), roughness U(0, 0.1),
    over a diffuse plane, lit by 1-4 lights, each a point or an area light; photons per
    iteration log-uniform [256k, 8M], 512x512.  Returns (scene, photons_per_iter)."""
    rng = np.random.default_rng(1000 + seed)
    tris = float(np.exp(rng.uniform(np.log(1e3), np.log(2e6))))
    photons = int(np.exp(rng.uniform(np.log(256 * 1024), np.log(8 * 1024 * 1024))))
    roughness = float(rng.uniform(0.0, 0.1))
    mats = [Material("R", color=(1, 1, 1), ior=float(rng.uniform(1.3, 1.8)), roughness=roughness),
            Material("P", color=(0.8, 0.8, 0.8), roughness=1.0, specular=0.0)]
    Vs, Ns, Fs = displaced_glass_sphere(rng, tris, float(rng.uniform(0.0, 0.2)))
    Vp, Np, Fp = plane(8.0, 0.0)
    meshes = [_mesh(Vs, Ns, Fs, 0, translate(0.0, 0.0, 1.4)), _mesh(Vp, Np, Fp, 1)]
    lights = []
    for i in range(int(rng.integers(1, 5))):
        col = tuple(float(c) for c in rng.uniform(0.6, 1.0, 3))
        pos = (float(rng.uniform(-1.5, 1.5)), float(rng.uniform(-1.5, 1.5)), float(rng.uniform(4.0, 6.0)))
        if rng.uniform() < 0.5:
            lights.append(Light("P", color=col, position=pos, power=float(rng.uniform(15.0, 40.0))))
        else:
            w = float(rng.uniform(0.5, 2.0))
            lights.append(Light("A", color=col, position=pos, width=w, height=w, power=float(rng.uniform(10.0, 30.0))))
    cam = look_at_camera(width, height, (0.0, -5.0, 4.0), (0.0, 0.0, 0.6), (0, 0, 1), 45.0)
    sc = Scene(meshes, mats, lights, cam, samples=4, base_radius=0.004, radius_reduction=0.75, name=f"batch{seed}")
    return sc, photons


WORKLOADS = {
    "glass_sphere_point": dict(scene=glass_sphere_point, photons_per_iter=1 << 20, iterations=16, max_path_length=8),
    "water_pool": dict(scene=water_pool, photons_per_iter=16 << 20, iterations=64, max_path_length=8),
}

"""Seeded synthetic scenes for the benchmark workloads and the radial test
volumes Galaxy's own gold-image tests render.

* radial_volume: the analytic fields of Galaxy's `radial` generator at T=1
  (src/apps/radial.cpp:154-231), on the grid `vti2vol` writes
  (scripts/vti2vol:69-80: origin -1, spacing 2/(n-1) printed with "%f").
* triangle_spheres_scene: 9 displaced UV spheres, ~200k triangles, 512x512,
  one directional light, shadows (the small triangle workload).
* blob_volume / volume_scene: Gaussian-blob fp32 field with value noise,
  1024x1024, 0.5-voxel steps, opacity ramp 0 -> 0.8 over [0.2, 1], early
  termination at alpha 0.99 (the volume workload).
* mixed_scene: 512^3 blob field in 2x2x2 bricks plus 4M spheres of radius
  0.002, 2048x2048, shadows plus 4 AO rays per hit (the partitioned mixed
  workload).

Every generator takes a seed and uses numpy's counter-based Philox bit
generator, so a (seed, size) pair always gives the same scene.
"""
import numpy as np

from .scene import (Camera, Lighting, Particles, ParticlesVis, PathLines, PathLinesVis, Triangles,
                    TrianglesVis, Visualization, Volume, VolumeVis)

f32 = np.float32

COOLWARM = [(0.0, 0.23, 0.30, 0.75), (0.25, 0.55, 0.69, 1.0), (0.5, 0.87, 0.87, 0.87),
            (0.75, 0.96, 0.60, 0.48), (1.0, 0.71, 0.02, 0.15)]
RADIAL_COLORMAP = [(0.0, 1.0, 0.5, 0.5), (0.25, 0.5, 1.0, 0.5), (0.5, 0.5, 0.5, 1.0),
                   (0.75, 1.0, 1.0, 0.5), (1.0, 1.0, 0.5, 1.0)]


def rng(seed):
    return np.random.Generator(np.random.Philox(int(seed)))


# ------------------------------------------------------------------ radial
def radial_fields(n=256):
    """float32 arrays (n,n,n) indexed [z,y,x]: xramp, yramp, zramp, oneBall,
    eightBalls, computed in single precision as radial.cpp:208-231 does."""
    d = f32(2.0 / (n - 1))
    c = f32(-1) + np.arange(n, dtype=f32) * d
    X = c[None, None, :]
    Y = c[None, :, None]
    Z = c[:, None, None]
    one = np.sqrt((X * X + Y * Y) + Z * Z).astype(f32)
    ax = (np.abs(X) - f32(0.5)).astype(f32)
    ay = (np.abs(Y) - f32(0.5)).astype(f32)
    az = (np.abs(Z) - f32(0.5)).astype(f32)
    eight = np.sqrt((ax * ax + ay * ay) + az * az).astype(f32)
    shp = (n, n, n)
    return {"xramp": np.broadcast_to(X, shp).astype(f32), "yramp": np.broadcast_to(Y, shp).astype(f32),
            "zramp": np.broadcast_to(Z, shp).astype(f32), "oneBall": one, "eightBalls": eight}


def radial_volume(name, n=256, fields=None):
    f = fields if fields is not None else radial_fields(n)
    spacing = float("%f" % (2.0 / (n - 1)))
    return Volume(f[name], origin=(-1.0, -1.0, -1.0), deltas=(spacing,) * 3)


# ----------------------------------------------------------- blob volumes
def blob_field(n, n_blobs, seed, noise=0.05, lattice=16):
    """n^3 float32 field on [0,1]^3 (spacing 1/(n-1)), indexed [z,y,x]:
    sum of n_blobs Gaussians (centres U[0.1,0.9]^3, sigma U[0.03,0.12],
    amplitude U[0.5,1]) plus trilinear value noise of the given amplitude on
    a lattice every `lattice` voxels.  The Gaussians are separable, so the
    field is one (n x B) @ (B x n^2) product."""
    g = rng(seed)
    cen = g.uniform(0.1, 0.9, size=(n_blobs, 3))
    sig = g.uniform(0.03, 0.12, size=n_blobs)
    amp = g.uniform(0.5, 1.0, size=n_blobs)
    x = np.linspace(0.0, 1.0, n)
    gx = np.exp(-((x[None, :] - cen[:, 0:1]) ** 2) / (2 * sig[:, None] ** 2)).astype(f32)
    gy = np.exp(-((x[None, :] - cen[:, 1:2]) ** 2) / (2 * sig[:, None] ** 2)).astype(f32)
    gz = (np.exp(-((x[None, :] - cen[:, 2:3]) ** 2) / (2 * sig[:, None] ** 2)) * amp[:, None]).astype(f32)
    field = np.empty((n, n, n), f32)
    yx = (gy[:, :, None] * gx[:, None, :]).reshape(n_blobs, n * n)     # B x n^2
    zc = 64
    for z0 in range(0, n, zc):
        z1 = min(n, z0 + zc)
        field[z0:z1] = (gz[:, z0:z1].T @ yx).reshape(z1 - z0, n, n)
    if noise > 0:
        m = (n - 1) // lattice + 2
        lat = g.uniform(-1.0, 1.0, size=(m, m, m)).astype(f32) * f32(noise)
        pos = np.arange(n, dtype=np.float64) / lattice
        i0 = np.minimum(pos.astype(np.int64), m - 2)
        fr = (pos - i0).astype(f32)
        # separable trilinear upsampling, one axis at a time
        W = np.zeros((n, m), f32)
        W[np.arange(n), i0] = 1 - fr
        W[np.arange(n), i0 + 1] += fr
        t = (W @ lat.reshape(m, m * m)).reshape(n, m, m)          # z
        t = np.matmul(W[None], t)                                  # y: (n, n, m)
        for z0 in range(0, n, 64):
            field[z0:z0 + 64] += np.matmul(t[z0:z0 + 64], W.T)     # x
    return field


def blob_volume(n=256, n_blobs=16, seed=1):
    return Volume(blob_field(n, n_blobs, seed), origin=(0.0, 0.0, 0.0), deltas=(1.0 / (n - 1),) * 3)


def volume_vis(vol):
    return VolumeVis(vol, volume_rendering=True, colormap=COOLWARM,
                     opacitymap=[(0.0, 0.0), (0.2, 0.0), (1.0, 0.8)])


def volume_scene(n=256, width=1024, height=1024, seed=1, partitions=(1, 1, 1)):
    """Volume workload: (camera, visualization)."""
    vol = blob_volume(n, 16, seed)
    vis = Visualization([volume_vis(vol)], Lighting(), partitions=partitions,
                        sampling_rate=2.0, opaque_alpha=0.99)
    cam = Camera(eye=(0.5, 0.5, 2.3), direction=(0.0, 0.0, -1.0), up=(0, 1, 0), aov=40.0,
                 width=width, height=height)
    return cam, vis


# ------------------------------------------------------ triangle spheres
def uv_sphere(n_lat, n_lon):
    """Unit UV sphere: vertices (poles + (n_lat-1) rings of n_lon) and
    2*n_lon*(n_lat-1) triangles."""
    th = np.pi * np.arange(1, n_lat) / n_lat
    ph = 2 * np.pi * np.arange(n_lon) / n_lon
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    ring = np.stack([st * np.cos(ph)[None, :], st * np.sin(ph)[None, :],
                     np.broadcast_to(ct, (n_lat - 1, n_lon))], -1).reshape(-1, 3)
    verts = np.concatenate([[[0.0, 0.0, 1.0]], ring, [[0.0, 0.0, -1.0]]])
    south = len(verts) - 1

    def rv(i, j):
        return 1 + i * n_lon + (j % n_lon)

    tris = []
    j = np.arange(n_lon)
    tris.append(np.stack([np.zeros(n_lon, int), rv(0, j), rv(0, j + 1)], -1))
    for i in range(n_lat - 2):
        a, b, c, d = rv(i, j), rv(i + 1, j), rv(i + 1, j + 1), rv(i, j + 1)
        tris.append(np.stack([a, b, c], -1))
        tris.append(np.stack([a, c, d], -1))
    tris.append(np.stack([np.full(n_lon, south), rv(n_lat - 2, j + 1), rv(n_lat - 2, j)], -1))
    return verts, np.concatenate(tris)


def vertex_normals(v, t):
    """Area-weighted vertex normals of a triangle mesh."""
    fn = np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]])
    n = np.zeros_like(v)
    for a in range(3):
        for k in range(3):
            n[:, a] += np.bincount(t[:, k], weights=fn[:, a], minlength=len(v))
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return n


def displaced_sphere_mesh(n_triangles=10_000_000, seed=5, amplitude=0.01, center=(0.5, 0.5, 0.5), radius=0.4):
    """One displaced UV sphere with about n_triangles triangles (the serving
    workload's large mesh), per-vertex data = displacement."""
    n = max(8, int(round(np.sqrt(n_triangles / 2.0))))
    sv, st = uv_sphere(n, n)
    g = rng(seed)
    disp = g.uniform(-amplitude, amplitude, size=len(sv))
    v = sv * (radius * (1.0 + disp))[:, None] + np.asarray(center)
    return Triangles(v.astype(f32), st.astype(np.int32), vertex_normals(v, st).astype(f32),
                     (0.5 + disp / (2 * amplitude)).astype(f32))


def triangle_spheres(seed=0, n_seg=105, grid=3, spacing=2.5, amplitude=0.01):
    """grid x grid displaced unit UV spheres in the z=0 plane."""
    g = rng(seed)
    sv, st = uv_sphere(n_seg, n_seg)
    V, T, D = [], [], []
    k = 0
    off = (grid - 1) / 2.0
    for j in range(grid):
        for i in range(grid):
            disp = g.uniform(-amplitude, amplitude, size=len(sv))
            v = sv * (1.0 + disp)[:, None] + np.array([(i - off) * spacing, (j - off) * spacing, 0.0])
            T.append(st + sum(len(x) for x in V))
            V.append(v)
            D.append((k + 0.5) / (grid * grid) + 10.0 * disp)
            k += 1
    v = np.concatenate(V)
    t = np.concatenate(T)
    return Triangles(v.astype(f32), t.astype(np.int32), vertex_normals(v, t).astype(f32),
                     np.concatenate(D).astype(f32))


def triangle_spheres_scene(width=512, height=512, seed=0, n_seg=105, partitions=(1, 1, 1)):
    """Triangle workload: (camera, visualization)."""
    mesh = triangle_spheres(seed, n_seg)
    L = Lighting()
    L.lights, L.types = [tuple(float(x) for x in -np.ones(3, f32) / f32(np.sqrt(3)))], [0]
    L.shadows, L.n_ao, L.Ka, L.Kd = True, 0, 0.5, 0.5
    vis = Visualization([TrianglesVis(mesh, colormap=COOLWARM)], L, partitions=partitions,
                        box=(-6.0, -6.0, -2.0, 6.0, 6.0, 2.0))
    cam = Camera(eye=(0, 0, 10), direction=(0, 0, -10), up=(0, 1, 0), aov=45.0, width=width, height=height)
    return cam, vis


# --------------------------------------------------------------- mixed
def sphere_cloud(n, seed=2, radius_box=(0.0, 1.0), clusters=32, sigma=0.02):
    """n sphere centres: half uniform in the box, half in `clusters` Gaussian
    clusters of the given sigma (clipped to the box); per-sphere data U[0,1]."""
    g = rng(seed)
    lo, hi = radius_box
    nu = n // 2
    a = g.uniform(lo, hi, size=(nu, 3))
    cc = g.uniform(lo + 0.1, hi - 0.1, size=(clusters, 3))
    which = g.integers(0, clusters, size=n - nu)
    b = np.clip(cc[which] + g.normal(0.0, sigma, size=(n - nu, 3)), lo, hi)
    data = g.uniform(0.0, 1.0, size=n)
    return Particles(np.concatenate([a, b]).astype(f32), data.astype(f32))


def mixed_scene(n=512, n_spheres=4_000_000, width=2048, height=2048, seed=3, partitions=(2, 2, 2),
                n_ao=4, ao_radius=0.1):
    """Partitioned mixed workload: (camera, visualization)."""
    vol = Volume(blob_field(n, 64, seed), origin=(0.0, 0.0, 0.0), deltas=(1.0 / (n - 1),) * 3)
    parts = sphere_cloud(n_spheres, seed + 1)
    L = Lighting()
    L.lights, L.types = [tuple(float(x) for x in -np.ones(3, f32) / f32(np.sqrt(3)))], [0]
    L.shadows, L.n_ao, L.ao_radius, L.Ka, L.Kd = True, n_ao, ao_radius, 0.5, 0.5
    vis = Visualization([volume_vis(vol),
                         ParticlesVis(parts, radius0=0.002, radius1=0.002, value0=0.0, value1=0.0,
                                      colormap=[(0.0, 0.9, 0.8, 0.2), (1.0, 0.2, 0.8, 0.9)])],
                        L, partitions=partitions, sampling_rate=2.0, opaque_alpha=0.99)
    cam = Camera(eye=(1.9, 1.4, 2.6), direction=(0.5 - 1.9, 0.5 - 1.4, 0.5 - 2.6), up=(0, 1, 0), aov=35.0,
                 width=width, height=height)
    return cam, vis


# ---------------------------------------------------------------- path lines
def abc_pathlines(n_lines=2000, n_vertices=64, seed=5, step=0.004, box=(0.1, 0.9)):
    """Seeded path lines: forward-Euler streamlines of the ABC flow
    (A, B, C) = (1, 0.7, 0.43) on the unit cube from uniform seed points;
    per-vertex data = flow speed scaled to [0, 1]."""
    g = rng(seed)
    p = g.uniform(box[0], box[1], size=(n_lines, 3))
    a, b, c = 1.0, 0.7, 0.43
    pts = np.empty((n_lines, n_vertices, 3), np.float64)
    spd = np.empty((n_lines, n_vertices), np.float64)
    for k in range(n_vertices):
        x, y, z = (2.0 * np.pi * p).T
        v = np.stack([a * np.sin(z) + c * np.cos(y), b * np.sin(x) + a * np.cos(z), c * np.sin(y) + b * np.cos(x)], 1)
        pts[:, k] = p
        spd[:, k] = np.linalg.norm(v, axis=1)
        p = p + step * v
    spd = spd / (a + b + c)
    return PathLines.from_polylines(list(pts.astype(f32)), list(spd.astype(f32)))


def pathlines_scene(n_lines=2000, n_vertices=64, width=512, height=512, seed=5, partitions=(1, 1, 1),
                    n_ao=2, ao_radius=0.05, radius0=0.003, radius1=0.008, volume=False):
    """Path-line workload: (camera, visualization).  volume=True adds a 64^3
    blob volume, so path lines and the volume march interleave."""
    lines = abc_pathlines(n_lines, n_vertices, seed)
    L = Lighting()
    L.lights, L.types = [tuple(float(x) for x in -np.ones(3, f32) / f32(np.sqrt(3)))], [0]
    L.shadows, L.n_ao, L.ao_radius, L.Ka, L.Kd = True, n_ao, ao_radius, 0.5, 0.5
    ops = [PathLinesVis(lines, radius0=radius0, radius1=radius1, value0=0.0, value1=1.0, colormap=COOLWARM)]
    kw = {}
    if volume:
        n = 64
        vol = Volume(blob_field(n, 16, seed + 1), origin=(0.0, 0.0, 0.0), deltas=(1.0 / (n - 1),) * 3)
        ops.insert(0, volume_vis(vol))
        kw = dict(sampling_rate=2.0, opaque_alpha=0.99)
    else:
        kw = dict(box=(0.0, 0.0, 0.0, 1.0, 1.0, 1.0))
    vis = Visualization(ops, L, partitions=partitions, **kw)
    cam = Camera(eye=(1.9, 1.4, 2.6), direction=(0.5 - 1.9, 0.5 - 1.4, 0.5 - 2.6), up=(0, 1, 0), aov=35.0,
                 width=width, height=height)
    return cam, vis

"""Empty-space skipping in the march passes (GXY_TUNE_SKIP_CLEAR, and
GXY_TUNE_SKIP_MODE for the passes that skip and run through clear bricks).

Bricks whose trilinear samples all lie below the transfer function's
zero-opacity threshold are flagged at commit; an interval between two
positions in such bricks composites nothing, so the march reads no voxels
for it.  Every frame and every counter except samples_skipped must equal
those of the same scene committed without the flags (up to the order of the
float atomics that add several contributions into one pixel), and the
oracle's."""
import numpy as np
import pytest

import oracle_lib as O
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

pytestmark = pytest.mark.gpu

ATOMIC_ORDER_TOL = 1e-6


@pytest.fixture(scope="module")
def gpu():
    from galaxy_gb300 import gpu as g
    g.init(0)
    return g


def commit(gpu, vis, skip):
    gpu.set_tuning(gpu.TUNE_SKIP_CLEAR, skip)
    try:
        return gpu.Scene(vis)
    finally:
        gpu.set_tuning(gpu.TUNE_SKIP_CLEAR, 1)


def render_pair(gpu, cam, vis, level):
    """Level 1: clear flags, per-position skipping in the camera-ray march
    and superbrick jumps in the shadow/AO march; level 2: per-position
    skipping and brick runs in both passes; level 3: level 1 plus the
    occlusion shortcut of the shadow/AO query.  Against the scene without
    flags."""
    L = S.resolve_lights(vis.lighting, cam)
    on, off = commit(gpu, vis, 1), commit(gpu, vis, 0)
    before = gpu.get_tuning(gpu.TUNE_SKIP_MODE)
    gpu.set_tuning(gpu.TUNE_SKIP_MODE, {1: 2, 2: 7, 3: 11}[level])
    try:
        a = on.render_host(cam, L)
        ca = on.counters()
    finally:
        gpu.set_tuning(gpu.TUNE_SKIP_MODE, before)
    b = off.render_host(cam, L)
    cb = off.counters()
    return a, b, ca, cb, L


# Counters the occlusion shortcut changes: the rays it ends are neither
# marched nor traversed past their first hit.
SHORTCUT_COUNTERS = ("samples", "nodes", "prim_tests", "sph_tests", "tri_tests")


def same_frames(a, b, ca, cb, level=1):
    assert float(np.abs(a - b).max()) <= ATOMIC_ORDER_TOL
    for k in ca:
        if k != "samples_skipped" and not (level == 3 and k in SHORTCUT_COUNTERS):
            assert ca[k] == cb[k], k


def image_close(img, ref, rmse_tol=1e-3, ch_tol=2.0 / 255, frac=0.999):
    d = np.abs(img[..., :3] - ref[..., :3])
    assert float(np.sqrt(np.mean(d ** 2))) <= rmse_tol
    assert float(np.mean(d <= ch_tol)) >= frac


@pytest.mark.parametrize("level", [1, 2, 3])
def test_volume_scene_skips_and_matches(gpu, level):
    cam, vis = scenes.volume_scene(n=96, width=128, height=128)
    a, b, ca, cb, L = render_pair(gpu, cam, vis, level)
    same_frames(a, b, ca, cb, level)
    # the blob field is mostly below the opacity ramp's start (0.2)
    assert ca["samples_skipped"] > 0.3 * ca["samples"]
    assert cb["samples_skipped"] < 0.05 * cb["samples"]
    ref, cnt = O.OracleScene(vis).render(cam, L, nthreads=8)
    image_close(a, ref)
    if level != 3:
        assert ca["samples"] == cnt["samples"]


@pytest.mark.parametrize("level", [1, 2, 3])
def test_shadow_and_ao_marches_skip_and_match(gpu, level):
    """Partitioned volume + particles with shadows and AO: the secondary
    march pass skips as the primary one does."""
    cam, vis = scenes.mixed_scene(n=64, n_spheres=4000, width=96, height=96, partitions=(2, 1, 1), n_ao=2)
    a, b, ca, cb, L = render_pair(gpu, cam, vis, level)
    same_frames(a, b, ca, cb, level)
    assert ca["samples_skipped"] > 0
    ref, cnt = O.OracleScene(vis).render(cam, L, nthreads=8)
    image_close(a, ref)
    # (sample totals are not compared here: the device path drops shadow/AO
    # rays whose payload is zero before marching them, the oracle marches
    # them; the frames agree either way)
    assert ca["shadow_rays"] == cnt["shadow"]


def _threshold_volume(n=48, seed=7):
    """Values just below the lookup's last zero-opacity point 127/255 of a
    TF whose opacity steps from 0 to ~1 between 0.5 and 0.502, with a few
    voxels above it (opacity ~0.6), placed on brick boundaries so the
    neighbouring bricks see them only through their apron."""
    g = np.random.default_rng(seed)
    edge = np.float32(127.0 / 255.0)
    f = (edge - np.float32(2e-3) * g.random((n, n, n), dtype=np.float32)).astype(np.float32)
    # voxels at the exact edge and a hair below: non-zero or zero opacity
    # by a few ulps, bricks with them must not be flagged
    f[8, 8, 8:40] = edge
    f[20, 24, 8:40] = np.nextafter(edge, np.float32(0))
    hot = g.integers(1, n // 4 - 1, size=(24, 3)) * 4
    f[hot[:, 0], hot[:, 1], hot[:, 2]] = np.float32(0.5005)
    return S.Volume(f, origin=(0.0, 0.0, 0.0), deltas=(1.0 / (n - 1),) * 3)


@pytest.mark.parametrize("level", [1, 2, 3])
def test_threshold_edge_and_apron(gpu, level):
    vol = _threshold_volume()
    vv = S.VolumeVis(vol, volume_rendering=True, colormap=[(0.0, 0.2, 0.3, 0.9), (1.0, 0.9, 0.3, 0.2)],
                     opacitymap=[(0.0, 0.0), (0.5, 0.0), (0.502, 1.0), (1.0, 1.0)])
    vis = S.Visualization([vv], S.Lighting(), sampling_rate=2.0, opaque_alpha=0.99)
    cam = S.Camera((0.5, 0.45, 2.2), (0.0, 0.05, -1.0), (0, 1, 0), 35.0, 96, 96)
    a, b, ca, cb, L = render_pair(gpu, cam, vis, level)
    same_frames(a, b, ca, cb, level)
    assert ca["samples_skipped"] > 0
    assert float(a[..., 3].max()) > 0.05      # the hot voxels are visible
    ref, cnt = O.OracleScene(vis).render(cam, L, nthreads=8)
    image_close(a, ref)
    if level != 3:
        assert ca["samples"] == cnt["samples"]


@pytest.mark.parametrize("level", [1, 2, 3])
def test_opaque_floor_tf_skips_nothing(gpu, level):
    """A transfer function with opacity at its low end has no zero-opacity
    threshold: no brick is flagged, and only march positions that end a
    march before any interval composites stay unread."""
    cam, vis = scenes.volume_scene(n=64, width=64, height=64)
    vis.operators[0].opacitymap = [(0.0, 0.05), (1.0, 0.8)]
    a, b, ca, cb, L = render_pair(gpu, cam, vis, level)
    same_frames(a, b, ca, cb, level)
    assert ca["samples_skipped"] == cb["samples_skipped"]


@pytest.mark.parametrize("block", [8, 16])
@pytest.mark.parametrize("eye", [(1.7, 1.3, 2.1), (-0.9, 0.52, 0.47), (0.5, 0.5, 2.5)])
@pytest.mark.parametrize("level", [1, 2, 3])
def test_checkerboard_brick_boundaries(gpu, eye, block, level):
    """A checkerboard of dense and empty blocks: rays cross brick boundaries
    between clear and non-clear bricks at every angle, including an
    axis-aligned view (direction components exactly 0)."""
    n = 64
    i = np.arange(n)
    chk = ((i[:, None, None] // block + i[None, :, None] // block + i[None, None, :] // block) % 2).astype(np.float32)
    g = np.random.default_rng(3)
    f = (0.1 + 0.7 * chk * g.random((n, n, n), dtype=np.float32)).astype(np.float32)
    vol = S.Volume(f, origin=(0.0, 0.0, 0.0), deltas=(1.0 / (n - 1),) * 3)
    vv = S.VolumeVis(vol, volume_rendering=True, colormap=scenes.COOLWARM,
                     opacitymap=[(0.0, 0.0), (0.3, 0.0), (1.0, 0.3)])
    vis = S.Visualization([vv], S.Lighting(), sampling_rate=2.0, opaque_alpha=0.99)
    d = tuple(0.5 - e for e in eye)
    cam = S.Camera(eye, d, (0, 1, 0), 40.0, 80, 80)
    a, b, ca, cb, L = render_pair(gpu, cam, vis, level)
    same_frames(a, b, ca, cb, level)
    assert ca["samples_skipped"] > 0.02 * ca["samples"]
    ref, cnt = O.OracleScene(vis).render(cam, L, nthreads=8)
    image_close(a, ref)


@pytest.mark.parametrize("level", [1, 2, 3])
@pytest.mark.parametrize("eye", [(2.2, 1.6, 2.9), (0.5, 0.5, 2.5), (-1.3, 0.9, 0.2)])
def test_superbrick_runs(gpu, eye, level):
    """A 160^3 volume, clear except for a dense ball and a dense slab: most
    rays cross runs of clear 32^3 superbricks (the DDA path) before, between
    and after the dense parts, at oblique and axis-aligned angles, with
    shadows and AO so both march passes run."""
    n = 160
    g = np.random.default_rng(11)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ball = ((x - 80) ** 2 + (y - 70) ** 2 + (z - 90) ** 2) < 22 ** 2
    slab = (x > 120) & (x < 131) & (y < 60)
    f = np.where(ball | slab, 0.35 + 0.6 * g.random((n, n, n), dtype=np.float32),
                 0.25 * g.random((n, n, n), dtype=np.float32)).astype(np.float32)
    vol = S.Volume(f, origin=(0.0, 0.0, 0.0), deltas=(1.0 / (n - 1),) * 3)
    vv = S.VolumeVis(vol, volume_rendering=True, colormap=scenes.COOLWARM,
                     opacitymap=[(0.0, 0.0), (0.3, 0.0), (1.0, 0.4)])
    parts = S.Particles(g.uniform(0.05, 0.95, size=(400, 3)).astype(np.float32), np.zeros(400, np.float32))
    L = S.Lighting()
    L.lights, L.types = [(-0.577, -0.577, -0.577)], [0]
    L.shadows, L.n_ao, L.ao_radius, L.Ka, L.Kd = True, 2, 0.3, 0.5, 0.5
    vis = S.Visualization([vv, S.ParticlesVis(parts, radius0=0.02, radius1=0.02)], L, partitions=(2, 1, 1),
                          sampling_rate=2.0, opaque_alpha=0.99)
    d = tuple(0.5 - e for e in eye)
    cam = S.Camera(eye, d, (0, 1, 0), 40.0, 96, 96)
    a, b, ca, cb, L = render_pair(gpu, cam, vis, level)
    same_frames(a, b, ca, cb, level)
    assert ca["samples_skipped"] > 0.5 * ca["samples"]
    if level == 3:   # some shadow/AO rays ended at their first hit, unmarched
        assert ca["samples"] < cb["samples"] and ca["nodes"] < cb["nodes"]
    ref, cnt = O.OracleScene(vis).render(cam, L, nthreads=8)
    image_close(a, ref)


@pytest.mark.parametrize("level", [1, 2, 3])
def test_offset_anisotropic_volume(gpu, level):
    """A volume away from the origin, with a different spacing on each axis
    and counts that are multiples of neither the brick (4 cells) nor the
    superbrick (32 cells): partial bricks and superbricks at the far faces,
    rays crossing them obliquely, shadows and AO across two partitions."""
    nx, ny, nz = 70, 83, 45
    org, dl = (-1.3, 0.4, 2.0), (0.02, 0.015, 0.03)
    g = np.random.default_rng(17)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    f = 0.2 * g.random((nz, ny, nx), dtype=np.float32)
    for cx, cy, cz, r in ((20, 30, 12, 9.0), (55, 70, 35, 7.0), (66, 10, 40, 6.0)):
        f += np.exp(-((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2) / (2 * r * r)).astype(np.float32)
    vol = S.Volume(f.astype(np.float32), origin=org, deltas=dl)
    lo = np.array(org, np.float32)
    hi = lo + np.array(dl, np.float32) * (np.array((nx, ny, nz), np.float32) - 1)
    vv = S.VolumeVis(vol, volume_rendering=True, colormap=scenes.COOLWARM,
                     opacitymap=[(0.0, 0.0), (0.3, 0.0), (1.2, 0.6)])
    pts = (lo + (hi - lo) * g.uniform(0.05, 0.95, size=(300, 3))).astype(np.float32)
    parts = S.Particles(pts, np.zeros(300, np.float32))
    L = S.Lighting()
    L.lights, L.types = [(-0.577, -0.577, -0.577)], [0]
    L.shadows, L.n_ao, L.ao_radius, L.Ka, L.Kd = True, 2, 0.2, 0.5, 0.5
    vis = S.Visualization([vv, S.ParticlesVis(parts, radius0=0.03, radius1=0.03)], L, partitions=(2, 1, 1),
                          sampling_rate=2.0, opaque_alpha=0.99)
    c = (lo + hi) / 2
    eye = tuple(float(v) for v in c + np.array([1.6, 0.9, 2.3], np.float32))
    cam = S.Camera(eye, tuple(float(v) for v in c - np.array(eye, np.float32)), (0, 1, 0), 40.0, 80, 80)
    a, b, ca, cb, L = render_pair(gpu, cam, vis, level)
    same_frames(a, b, ca, cb, level)
    assert ca["samples_skipped"] > 0.1 * ca["samples"]
    ref, cnt = O.OracleScene(vis).render(cam, L, nthreads=8)
    image_close(a, ref)


@pytest.mark.parametrize("parts", [(2, 2, 2), (4, 1, 1)])
def test_handed_off_primaries_split_same_frames(gpu, parts):
    """Primaries handed to the next brick traced as a query pass plus the
    skipping camera-ray march (GXY_TUNE_SPLIT_HANDOFF 1) or in one pass per
    ray (0): the same frames and ray counters, and the oracle's image."""
    cam, vis = scenes.mixed_scene(n=96, n_spheres=20000, width=128, height=128, partitions=parts, n_ao=2)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    out = {}
    try:
        for v in (0, 1):
            gpu.set_tuning(gpu.TUNE_SPLIT_HANDOFF, v)
            out[v] = (sc.render_host(cam, L), sc.counters())
    finally:
        gpu.set_tuning(gpu.TUNE_SPLIT_HANDOFF, 1)
    (a, ca), (b, cb) = out[1], out[0]
    assert ca["handoffs"] > 0
    assert float(np.abs(a - b).max()) <= ATOMIC_ORDER_TOL
    for k in ("primary_rays", "shadow_rays", "ao_rays", "segments", "handoffs", "terminated", "dropped", "samples"):
        assert ca[k] == cb[k], k
    ref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(a, ref)


@pytest.mark.parametrize("shortcut", [1, 9])
def test_warp_packet_shadow_query_same_frames(gpu, shortcut):
    """Shadow/AO rays queried one lane per ray (GXY_TUNE_SEC_PACKET 0) or one
    warp per 32-ray packet (1), with and without the occlusion shortcut: the
    same frames and ray counters, and the oracle's image."""
    cam, vis = scenes.mixed_scene(n=96, n_spheres=20000, width=128, height=128, partitions=(2, 2, 2), n_ao=4)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    before = gpu.get_tuning(gpu.TUNE_SKIP_MODE)
    out = {}
    try:
        gpu.set_tuning(gpu.TUNE_SKIP_MODE, shortcut)
        for v in (0, 1):
            gpu.set_tuning(gpu.TUNE_SEC_PACKET, v)
            out[v] = (sc.render_host(cam, L), sc.counters())
    finally:
        gpu.set_tuning(gpu.TUNE_SEC_PACKET, 0)
        gpu.set_tuning(gpu.TUNE_SKIP_MODE, before)
    (a, ca), (b, cb) = out[1], out[0]
    assert float(np.abs(a - b).max()) <= ATOMIC_ORDER_TOL
    for k in ("primary_rays", "shadow_rays", "ao_rays", "segments", "handoffs", "terminated", "dropped", "samples"):
        assert ca[k] == cb[k], k
    ref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(a, ref)

"""Frame generations launched ahead of the host's count reads
(GXY_TUNE_RUNAHEAD).

After the camera generation the frame path reads the three queue counts once
per block of generations; a block runs to the generation count of the
scene's previous frame, its later generations take their input counts from a
ring in device memory, and its queues were grown to the block's worst case
beforehand.  Whatever the block length, a frame must be the frame of one
read per generation (the loop Galaxy's Renderer runs per received RayList,
Renderer.cpp:674-690): the same image (to the order of float atomics), the
same counters and generation count, the same rays in per generation in the
profile -- and the oracle's image.  A frame longer than the previous one
goes on past the block; a shorter one ends inside it.  Where the queue limit
keeps a block's queues from growing, the block is shortened, not the frame
broken.
"""
import numpy as np
import pytest

import oracle_lib as O
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

COUNTERS = ("primary_rays", "shadow_rays", "ao_rays", "segments", "handoffs", "terminated", "samples",
            "samples_skipped", "nodes", "prim_tests", "bounces", "overflow")


def image_close(img, ref, rmse_tol=1e-3, ch_tol=2.0 / 255, frac=0.999):
    d = np.abs(img[..., :3] - ref[..., :3])
    assert float(np.sqrt(np.mean(d ** 2))) <= rmse_tol
    assert float(np.mean(d <= ch_tol)) >= frac


def deep_scene(width=64, height=48, along_x=True):
    """A 64^3 blob volume in 16 bricks along x, viewed along +x: every camera
    ray crosses all 16 bricks (16 generations); viewed along +y, one brick."""
    vol = S.Volume(scenes.blob_field(64, 8, 4), origin=(0.0, 0.0, 0.0), deltas=(1.0 / 63,) * 3)
    L = S.Lighting()
    L.lights, L.types, L.shadows, L.n_ao = [(-0.577, -0.577, -0.577)], [0], True, 2
    vis = S.Visualization([scenes.volume_vis(vol)], L, partitions=(16, 1, 1), sampling_rate=2.0, opaque_alpha=0.99)
    if along_x:
        cam = S.Camera(eye=(-1.5, 0.5, 0.5), direction=(1.0, 0.0, 0.0), up=(0, 1, 0), aov=20.0, width=width,
                       height=height)
    else:
        cam = S.Camera(eye=(0.53, -1.5, 0.5), direction=(0.0, 1.0, 0.0), up=(0, 0, 1), aov=2.0, width=width,
                       height=height)
    return cam, vis


SCENES = {
    "mixed": lambda: scenes.mixed_scene(n=96, n_spheres=20000, width=128, height=128, partitions=(2, 2, 2), n_ao=2),
    "deep": deep_scene,
    "triangles": lambda: scenes.triangle_spheres_scene(width=128, height=128, n_seg=24),
}


@pytest.fixture(scope="module")
def gpu():
    from galaxy_gb300 import gpu as g
    g.init(0)
    return g


def frame(gpu, sc, cam, L, runahead):
    gpu.set_tuning(gpu.TUNE_RUNAHEAD, runahead)
    try:
        img = sc.render_host(cam, L)
    finally:
        gpu.set_tuning(gpu.TUNE_RUNAHEAD, 4)
    c = sc.counters()
    # rays in per (generation, kind) of the query/trace launches; a block's
    # generations after the queues ran dry launch with no rays
    per_gen = {}
    for g in sc.generations():
        if g["kind"] in (1, 2, 5) and g["rays_in"]:
            per_gen[(g["generation"], g["kind"])] = g["rays_in"]
    return img, {k: c[k] for k in COUNTERS}, per_gen


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SCENES))
def test_runahead_same_frames(gpu, name):
    cam, vis = SCENES[name]()
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    sc.set_profiling(True)
    ref = frame(gpu, sc, cam, L, 1)
    assert ref[1]["overflow"] == 0
    if name == "deep":
        assert ref[1]["bounces"] >= 16
    for k in (2, 3, 4, 16):
        got = frame(gpu, sc, cam, L, k)
        np.testing.assert_allclose(got[0], ref[0], atol=1e-5)
        assert got[1] == ref[1], k
        assert got[2] == ref[2], k
    oref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(ref[0], oref)
    assert ref[1]["primary_rays"] == cnt["primary"]


@pytest.mark.gpu
def test_runahead_under_queue_limit(gpu):
    """Queues held below a block's worst case: the blocks shorten to what the
    queues hold, the frame is unchanged."""
    cam, vis = deep_scene(96, 64)
    L = S.resolve_lights(vis.lighting, cam)
    ref = frame(gpu, gpu.Scene(vis), cam, L, 1)
    gpu.set_tuning(gpu.TUNE_QUEUE_LIMIT, 30000)
    try:
        sc = gpu.Scene(vis)
        first = frame(gpu, sc, cam, L, 16)    # no previous frame: a read per generation
        got = frame(gpu, sc, cam, L, 16)
    finally:
        gpu.set_tuning(gpu.TUNE_QUEUE_LIMIT, 0)
    for f in (first, got):
        np.testing.assert_allclose(f[0], ref[0], atol=1e-5)
        assert f[1] == ref[1]


@pytest.mark.gpu
def test_runahead_longer_and_shorter_frames(gpu):
    """A view through one brick (a couple of generations) before a view
    through all 16 bricks, and back: the longer frame goes on past its first
    block, the shorter one ends inside it; each equals its frame on a scene
    with no history."""
    cam_x, vis = deep_scene(64, 48, along_x=True)
    cam_y, _ = deep_scene(64, 48, along_x=False)
    Lx, Ly = S.resolve_lights(vis.lighting, cam_x), S.resolve_lights(vis.lighting, cam_y)
    want_x = frame(gpu, gpu.Scene(vis), cam_x, Lx, 1)
    want_y = frame(gpu, gpu.Scene(vis), cam_y, Ly, 1)
    assert want_x[1]["bounces"] >= 16 > want_y[1]["bounces"]
    sc = gpu.Scene(vis)
    sc.set_profiling(True)
    for cam, L, want in ((cam_y, Ly, want_y), (cam_x, Lx, want_x), (cam_y, Ly, want_y), (cam_x, Lx, want_x)):
        got = frame(gpu, sc, cam, L, 16)
        np.testing.assert_allclose(got[0], want[0], atol=1e-5)
        assert got[1] == want[1]


def test_runahead_knob_range():
    """Host side only: the knob takes 1-16 generations and refuses the rest."""
    from galaxy_gb300 import gpu
    old = gpu.get_tuning(gpu.TUNE_RUNAHEAD)
    try:
        for bad in (0, -1, 17):
            with pytest.raises(gpu.GxyError):
                gpu.set_tuning(gpu.TUNE_RUNAHEAD, bad)
        gpu.set_tuning(gpu.TUNE_RUNAHEAD, 16)
        assert gpu.get_tuning(gpu.TUNE_RUNAHEAD) == 16
    finally:
        gpu.set_tuning(gpu.TUNE_RUNAHEAD, old)

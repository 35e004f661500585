"""Failure paths of the device path, made on the host side (no GPU fault):

  * queue room: the frame path grows its queues to the worst case of each
    launch; a frame whose camera rays do not fit the HBM budget or the
    queue limit (GXY_TUNE_QUEUE_LIMIT) is rendered in bands of image rows,
    as Galaxy splits an over-large ray list (Renderer.cpp:674-690), with the
    same image as in one piece; a limit below one row's rays is refused with
    GXY_ERR_OOM before anything is launched, and the next frame is correct;
  * the HBM budget of gxy_gpu_init refuses a commit that does not fit;
  * a batch whose rays outlast its generations per submission is continued
    from its queues until they are empty (a ray crossing 16 bricks needs 16
    generations), so no ray is lost;
  * the serving loop cancels a waiting request and reports it.
"""
import numpy as np
import pytest

import oracle_lib as O
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    from galaxy_gb300 import gpu
    gpu.init(0)
    return torch, gpu


def image_close(img, ref, rmse_tol=1e-3, ch_tol=2.0 / 255, frac=0.999):
    d = np.abs(img[..., :3] - ref[..., :3])
    assert float(np.sqrt(np.mean(d ** 2))) <= rmse_tol
    assert float(np.mean(d <= ch_tol)) >= frac


def small_mixed(width=96, height=96, partitions=(2, 2, 1)):
    return scenes.mixed_scene(n=64, n_spheres=20000, width=width, height=height, partitions=partitions, n_ao=2)


def test_queue_limit_renders_in_bands(env):
    torch, gpu = env
    cam, vis = small_mixed()
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    ref = sc.render_host(cam, L)
    c0 = sc.counters()
    assert c0["bands"] == 1
    gpu.set_tuning(gpu.TUNE_QUEUE_LIMIT, 6000)
    try:
        sc2 = gpu.Scene(vis)
        got = sc2.render_host(cam, L)
        c1 = sc2.counters()
    finally:
        gpu.set_tuning(gpu.TUNE_QUEUE_LIMIT, 0)
    assert c1["bands"] > 1 and c1["overflow"] == 0
    np.testing.assert_allclose(got, ref, atol=1e-5)
    for k in ("primary_rays", "shadow_rays", "ao_rays", "terminated", "segments"):
        assert c1[k] == c0[k], k
    oref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(got, oref)
    assert c1["primary_rays"] == cnt["primary"]


def test_queue_limit_below_one_row_is_refused(env):
    torch, gpu = env
    cam, vis = small_mixed()
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    ref = sc.render_host(cam, L)
    sc2 = gpu.Scene(vis)
    gpu.set_tuning(gpu.TUNE_QUEUE_LIMIT, 50)    # one row emits ~96 camera rays, 2 AO each
    try:
        with pytest.raises(gpu.GxyError) as e:
            sc2.render_host(cam, L)
        assert e.value.code == gpu.A.GXY_ERR_OOM
    finally:
        gpu.set_tuning(gpu.TUNE_QUEUE_LIMIT, 0)
    np.testing.assert_allclose(sc2.render_host(cam, L), ref, atol=1e-5)


def test_hbm_budget_bands_and_refusals(env):
    torch, gpu = env
    cam, vis = small_mixed(width=128, height=128)
    L = S.resolve_lights(vis.lighting, cam)
    ref = gpu.Scene(vis).render_host(cam, L)
    sc = gpu.Scene(vis)
    used = gpu.hbm_in_use()
    try:
        # room for about a quarter of the frame's queues: rendered in bands
        gpu.init(0, used + (3 << 20))
        got = sc.render_host(cam, L)
        c = sc.counters()
        assert c["bands"] > 1 and c["overflow"] == 0
        np.testing.assert_allclose(got, ref, atol=1e-5)
        # a commit beyond the budget is refused
        with pytest.raises(gpu.GxyError) as e:
            gpu.Scene(vis)
        assert e.value.code == gpu.A.GXY_ERR_OOM
        # a batch beyond the budget is refused at admission
        with pytest.raises(gpu.GxyError) as e:
            gpu.Batch(max_pixels=4 << 20, max_jobs=4, max_shadow=1, max_ao=2)
        assert e.value.code == gpu.A.GXY_ERR_ADMISSION
    finally:
        gpu.init(0, 0)
    np.testing.assert_allclose(sc.render_host(cam, L), ref, atol=1e-5)


def deep_scene(width=64, height=48):
    """A 64^3 blob volume in 16 bricks along x, viewed along +x: every camera
    ray crosses all 16 bricks, so a frame takes 16 generations."""
    vol = S.Volume(scenes.blob_field(64, 8, 4), origin=(0.0, 0.0, 0.0), deltas=(1.0 / 63,) * 3)
    L = S.Lighting()
    L.lights, L.types, L.shadows, L.n_ao = [(-0.577, -0.577, -0.577)], [0], True, 0
    vis = S.Visualization([scenes.volume_vis(vol)], L, partitions=(16, 1, 1), sampling_rate=2.0, opaque_alpha=0.99)
    cam = S.Camera(eye=(-1.5, 0.5, 0.5), direction=(1.0, 0.0, 0.0), up=(0, 1, 0), aov=20.0, width=width,
                   height=height)
    return cam, vis


@pytest.mark.parametrize("graph", [False, True])
def test_batch_continues_past_its_generation_limit(env, graph):
    torch, gpu = env
    cam, vis = deep_scene()
    L = S.resolve_lights(vis.lighting, cam).c()
    a, b = gpu.Scene(vis), gpu.Scene(vis)
    ref = a.render_host(cam, L)
    assert a.counters()["bounces"] > 12
    for uniform in (True, False):
        bt = gpu.Batch(max_pixels=2 * cam.width * cam.height, max_jobs=4, max_shadow=1, max_ao=0)
        fbs = [torch.zeros((cam.height, cam.width, 4), device="cuda") for _ in range(2)]
        torch.cuda.synchronize()
        bt.submit([(a, cam, L, fbs[0].data_ptr()), ((a if uniform else b), cam, L, fbs[1].data_ptr())],
                  use_graph=graph)
        bt.wait(60000)
        c = bt.counters()
        assert c["bounces"] > 10 and c["overflow"] == 0
        for fb in fbs:
            np.testing.assert_allclose(fb.cpu().numpy(), ref, atol=1e-5)
        bt.release()


def test_server_cancel(env):
    """A request still waiting behind a large one is cancelled: it is never
    rendered, take() reports GXY_ERR_CANCELLED, the others are unaffected."""
    torch, gpu = env
    cam0, vis = small_mixed()
    sc = gpu.Scene(vis)
    big = S.Camera(cam0.eye, cam0.dir, cam0.up, cam0.aov, 1024, 1024)
    srv = gpu.NativeServer(n_slots=1, slot_pixels=1024 * 1024, max_jobs=1, max_shadow=1, max_ao=2,
                           fb_budget=1 << 28, small_pixels=0, small_batch_pixels=1024 * 1024)
    try:
        reqs = [big] + [S.Camera((cam0.eye[0] + 0.05 * k,) + tuple(cam0.eye[1:]), cam0.dir, cam0.up, cam0.aov, 96,
                                 96) for k in range(5)]
        lights = [S.resolve_lights(vis.lighting, c) for c in reqs]
        ids = [srv.submit(sc, c, L) for c, L in zip(reqs, lights)]
        was_running = srv.cancel(ids[-1])
        assert not was_running
        srv.drain(60000)
        for rid, cam, L in zip(ids, reqs, lights):
            if rid == ids[-1]:
                with pytest.raises(gpu.GxyError) as e:
                    srv.take(rid)
                assert e.value.code == gpu.A.GXY_ERR_CANCELLED
                continue
            img, lat, rays = srv.take(rid)
            assert rays > 0
            np.testing.assert_allclose(img, sc.render_host(cam, L), atol=1e-5)
    finally:
        srv.release()

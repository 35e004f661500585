"""Batched frames (one persistent wavefront launch for many jobs) and the
continuous-batching serving loop: every job's image equals the same frame
rendered alone through the plain path (within float-atomic ordering), and
served requests match the oracle's render of the same camera and lighting."""
import numpy as np
import pytest

from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    from galaxy_gb300 import gpu
    gpu.init(0)
    cam_m, vis_m = scenes.mixed_scene(n=64, n_spheres=20000, width=96, height=96, partitions=(2, 2, 1), n_ao=2)
    cam_t, vis_t = scenes.triangle_spheres_scene(width=80, height=64, n_seg=24)
    return torch, gpu, {"mixed": (gpu.Scene(vis_m), cam_m, vis_m), "tri": (gpu.Scene(vis_t), cam_t, vis_t)}


def alone(torch, sc, cam, L):
    fb = torch.zeros((cam.height, cam.width, 4), dtype=torch.float32, device="cuda")
    sc.render(cam, L, fb.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return fb.cpu().numpy()


def jobs_for(env, n, seed=0):
    torch, gpu, sc = env
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(n):
        key = ["mixed", "tri"][k % 2]
        scene, cam0, vis = sc[key]
        cam = S.Camera(cam0.eye, cam0.dir, cam0.up, cam0.aov, int(rng.integers(16, 97)), int(rng.integers(16, 97)))
        ang = rng.uniform(-0.3, 0.3)
        cam.eye = (cam0.eye[0] + ang, cam0.eye[1], cam0.eye[2])
        L = S.resolve_lights(vis.lighting, cam)
        jobs.append((key, scene, cam, L.c()))
    return jobs


@pytest.mark.parametrize("coop", [False, True])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("uniform", [False, True])
def test_batch_equals_alone(env, graph, uniform, coop):
    torch, gpu, sc = env
    jobs = jobs_for(env, 12)
    if uniform:
        jobs = [j for j in jobs if j[0] == "mixed"]
    b = gpu.Batch(max_pixels=200000, max_jobs=64, max_shadow=1, max_ao=2)
    fbs = [torch.zeros((c.height, c.width, 4), dtype=torch.float32, device="cuda") for _, _, c, _ in jobs]
    torch.cuda.synchronize()
    b.submit([(s, c, L, fb.data_ptr()) for (_, s, c, L), fb in zip(jobs, fbs)], use_graph=graph, cooperative=coop)
    b.wait(60000)
    cnt = b.counters()
    total_primary = 0
    for (_, s, c, L), fb in zip(jobs, fbs):
        ref = alone(torch, s, c, L)
        total_primary += s.counters()["primary_rays"]
        got = fb.cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-5
    assert cnt["primary_rays"] == total_primary
    # resubmission of the same slot (graph update path) gives the same images
    for fb in fbs:
        fb.zero_()
    torch.cuda.synchronize()
    b.submit([(s, c, L, fb.data_ptr()) for (_, s, c, L), fb in zip(jobs, fbs)], use_graph=graph, cooperative=coop)
    b.wait(60000)
    for (_, s, c, L), fb in zip(jobs, fbs):
        assert np.abs(fb.cpu().numpy() - alone(torch, s, c, L)).max() <= 1e-5
    b.release()


def test_batch_admission_and_errors(env):
    torch, gpu, sc = env
    from galaxy_gb300.gpu import GxyError
    jobs = jobs_for(env, 4)
    b = gpu.Batch(max_pixels=1000, max_jobs=2, max_shadow=1, max_ao=2)
    fb = torch.zeros((100, 100, 4), device="cuda")
    with pytest.raises(GxyError):   # too many pixels
        b.submit([(jobs[0][1], jobs[0][2], jobs[0][3], fb.data_ptr())])
    with pytest.raises(GxyError):   # too many jobs
        b.submit([(j[1], j[2], j[3], fb.data_ptr()) for j in jobs[:3]])
    b.release()


def test_serving_results_match_alone(env):
    """Requests served by the continuous-batching loop produce the same image
    alone and in the mix."""
    torch, gpu, sc = env
    from galaxy_gb300 import serve
    table = {k: v[0] for k, v in sc.items()}
    jobs = jobs_for(env, 24, seed=3)
    reqs = [serve.Request(i, 0.0005 * i, key, cam, L) for i, (key, _, cam, L) in enumerate(jobs)]
    srv = serve.Server(table, n_slots=3, slot_pixels=30000, max_jobs=8, max_shadow=1, max_ao=2,
                       fb_budget=1 << 28, use_graph=True, keep_results=True, small_pixels=4000,
                       small_batch_pixels=20000)
    st = srv.run(reqs, time_limit=60)
    assert st["completed"] == len(reqs) and st["refused"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0
    for r in reqs:
        ref = alone(torch, table[r.scene], r.camera, r.lighting)
        assert np.abs(r.fb - ref).max() <= 1e-5
    srv.release()
    # and against the oracle: a request served in the mix is the reference
    # path's image of its camera and lighting
    import oracle_lib as O
    for r in reqs[:6]:
        vis = sc[r.scene][2]
        ref, cnt = O.OracleScene(vis).render(r.camera, S.resolve_lights(vis.lighting, r.camera))
        d = np.abs(r.fb[..., :3] - ref[..., :3])
        assert float(np.sqrt(np.mean(d ** 2))) <= 1e-3
        assert float(np.mean(d <= 2.0 / 255)) >= 0.999


def test_native_server_contract(env):
    """gxy_server_*: refusals at submission, poll/drain/take, one take per
    request, images equal to rendering alone."""
    torch, gpu, sc = env
    A = gpu.A
    srv = gpu.NativeServer(n_slots=2, slot_pixels=10000, max_jobs=4, max_shadow=1, max_ao=2, fb_budget=1 << 24,
                           small_pixels=3000, small_batch_pixels=8000)
    try:
        scene, cam0, vis = sc["tri"]
        big = S.Camera(cam0.eye, cam0.dir, cam0.up, cam0.aov, 200, 100)      # 20000 pixels > slot
        with pytest.raises(gpu.GxyError) as e:
            srv.submit(scene, big, S.resolve_lights(vis.lighting, big))
        assert e.value.code == A.GXY_ERR_ADMISSION
        ids = []
        for k, (key, sce, cam, L) in enumerate(jobs_for(env, 6, seed=9)):
            ids.append((srv.submit(sce, cam, L), sce, cam, L))
        srv.drain(60000)
        for rid, sce, cam, L in ids:
            assert srv.poll(rid)
            img, lat, rays = srv.take(rid)
            assert lat > 0 and rays > 0
            assert np.abs(img - alone(torch, sce, cam, L)).max() <= 1e-5
            with pytest.raises(gpu.GxyError):
                srv.poll(rid)   # taken: no longer known
    finally:
        srv.release()

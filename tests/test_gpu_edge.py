"""Edge cases of the device path against the oracle: an empty scene, tiny
and odd image sizes, empty ray lists, degenerate path-line segments,
invalid arguments, a whole 4096x4096 frame; and the autotuner's
coordinate descent."""
import numpy as np
import pytest

import oracle_lib as O
from galaxy_gb300 import _abi as A
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from galaxy_gb300 import gpu as g
    g.init(0)
    return g


def close(img, ref, rmse_tol=1e-3, ch_tol=2.0 / 255, frac=0.999):
    d = np.abs(img[..., :3] - ref[..., :3])
    assert float(np.sqrt(np.mean(d ** 2))) <= rmse_tol
    assert float(np.mean(d <= ch_tol)) >= frac


def both(gpu, cam, vis):
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    img = sc.render_host(cam, L)
    ref, cnt = O.OracleScene(vis).render(cam, L, nthreads=8)
    return img, ref, sc.counters(), cnt


def test_empty_scene(gpu):
    vis = S.Visualization([], S.Lighting())
    cam = S.Camera((0, 0, 5), (0, 0, -1), (0, 1, 0), 45.0, 64, 48)
    img, ref, c, cnt = both(gpu, cam, vis)
    assert np.array_equal(img, ref) and not img.any()
    assert c["primary_rays"] == cnt["primary"] and c["shadow_rays"] == 0 and c["ao_rays"] == 0


@pytest.mark.parametrize("w,h", [(1, 1), (2, 1), (127, 33), (33, 127)])
def test_tiny_and_odd_images(gpu, w, h):
    cam, vis = scenes.pathlines_scene(n_lines=300, n_vertices=32, width=w, height=h, partitions=(2, 1, 1))
    img, ref, c, cnt = both(gpu, cam, vis)
    close(img, ref)
    assert c["primary_rays"] == cnt["primary"] and c["shadow_rays"] == cnt["shadow"]


def test_empty_ray_lists(gpu):
    cam, vis = scenes.pathlines_scene(n_lines=50, n_vertices=16, width=16, height=16)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    empty = A.RayListArrays(0)
    traced, sec = sc.trace(0, L, empty, capacity=1)
    assert traced.n == 0 and sec.n == 0
    assert gpu.classify(empty).n == 0
    assert sc.assign_destinations(0, empty).n == 0
    fb = np.zeros((4, 4, 4), np.float32)
    gpu.accumulate_terminated(empty, fb)
    assert not fb.any()


def test_degenerate_path_line_segments(gpu):
    """Zero-length segments (repeated vertices) are two coincident spheres:
    the cylinder term drops out (a == 0, DataDrivenPathLines.ispc:132)."""
    pts = np.array([[0.3, 0.5, 0.5], [0.3, 0.5, 0.5], [0.6, 0.55, 0.5], [0.6, 0.55, 0.5], [0.7, 0.3, 0.4]], np.float32)
    lines = S.PathLines(pts, [0, 1, 2, 3], data=[0.0, 0.2, 0.5, 0.8, 1.0])
    L = S.Lighting()
    L.lights, L.types, L.shadows, L.n_ao = [(-0.577, -0.577, -0.577)], [0], True, 2
    vis = S.Visualization([S.PathLinesVis(lines, radius0=0.04, radius1=0.08, value0=0.0, value1=1.0,
                                          colormap=scenes.COOLWARM)], L, box=(0, 0, 0, 1, 1, 1))
    cam = S.Camera((0.5, 0.5, 2.0), (0, 0, -1), (0, 1, 0), 30.0, 96, 96)
    img, ref, c, cnt = both(gpu, cam, vis)
    close(img, ref)
    assert cnt["shadow"] > 50 and c["shadow_rays"] == cnt["shadow"]


def test_invalid_arguments_are_refused(gpu):
    cam, vis = scenes.pathlines_scene(n_lines=20, n_vertices=8, width=16, height=16)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    bad = cam.c()
    bad.width = 0
    with pytest.raises(gpu.GxyError) as e:
        sc.render_host(bad, L, out=np.zeros((16, 16, 4), np.float32))
    assert e.value.code == A.GXY_ERR_INVALID
    none = L.c() if hasattr(L, "c") else L
    none.n_lights = 0
    with pytest.raises(gpu.GxyError) as e:
        sc.render_host(cam, none)
    assert e.value.code == A.GXY_ERR_INVALID
    with pytest.raises(gpu.GxyError) as e:
        sc.generate_initial_rays(5, cam)
    assert e.value.code == A.GXY_ERR_INVALID
    # a segment index past the last vertex is refused at commit
    lines = S.PathLines(np.zeros((3, 3), np.float32), [0, 2])
    with pytest.raises(gpu.GxyError) as e:
        gpu.Scene(S.Visualization([S.PathLinesVis(lines, radius0=0.01, radius1=0.01)], box=(0, 0, 0, 1, 1, 1)))
    assert e.value.code == A.GXY_ERR_INVALID


def test_largest_frame_matches_oracle(gpu):
    """4096x4096 (16.8 M camera rays, the serving workload's largest image)
    of the ~197k-triangle scene with hard shadows: the whole frame on the
    GPU and in the oracle."""
    cam, vis = scenes.triangle_spheres_scene(width=4096, height=4096)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    img = sc.render_host(cam, L)
    ref, cnt = O.OracleScene(vis).render(cam, L)
    close(img, ref)
    c = sc.counters()
    assert c["primary_rays"] == cnt["primary"] == 4096 * 4096
    assert c["shadow_rays"] == cnt["shadow"]


def test_autotuner_coordinate_descent(gpu):
    """The tuner measures one knob at a time, returns a setting for every
    knob (one of the settings it measured), and leaves the library set to
    it."""
    from galaxy_gb300 import autotune
    cam, vis = scenes.mixed_scene(n=48, n_spheres=4000, width=96, height=96, partitions=(2, 1, 1), n_ao=2)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    before = autotune.current()
    try:
        res = autotune.tune(sc, cam, L, frames=1, passes=1)
        best = res["best"]
        assert set(n for n, _, _ in autotune.KNOBS) <= set(best)
        assert autotune.current() == {n: best[n] for n, _, _ in autotune.KNOBS}
        assert len(res["candidates"]) >= 1 + sum(len(v) - 1 for _, _, v in autotune.KNOBS) - 1
        # the kept setting is one of those measured, timed over >= 30 ms of frames
        assert {n: best[n] for n, _, _ in autotune.KNOBS} in [{n: c[n] for n, _, _ in autotune.KNOBS}
                                                              for c in res["candidates"]]
        assert res["frames_per_setting"] >= 1 and best["ms_per_frame"] > 0
        # every setting renders the same image (within the parity tolerance)
        img = sc.render_host(cam, L)
        autotune.apply(before)
        ref = sc.render_host(cam, L)
        close(img, ref)
    finally:
        autotune.apply(before)


def test_carried_hits_same_frames(gpu):
    """Shadow/AO rays that move to the next partition carry their query's
    closest hit (GXY_TUNE_CARRY_HITS): the frames and ray counters equal
    those with a fresh query in every partition; only node visits and
    primitive tests drop."""
    cam, vis = scenes.mixed_scene(n=64, n_spheres=20000, width=128, height=128, partitions=(2, 2, 2), n_ao=4)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    before = gpu.get_tuning(gpu.TUNE_CARRY_HITS)
    cont = gpu.get_tuning(gpu.TUNE_CONTINUE)
    try:
        # rays carried through the queues (continuing them in the march
        # kernel, GXY_TUNE_CONTINUE, also changes the generation counts)
        gpu.set_tuning(gpu.TUNE_CONTINUE, 0)
        gpu.set_tuning(gpu.TUNE_CARRY_HITS, 1)
        a = sc.render_host(cam, L)
        ca = sc.counters()
        gpu.set_tuning(gpu.TUNE_CARRY_HITS, 0)
        b = sc.render_host(cam, L)
        cb = sc.counters()
    finally:
        gpu.set_tuning(gpu.TUNE_CARRY_HITS, before)
        gpu.set_tuning(gpu.TUNE_CONTINUE, cont)
    assert float(np.abs(a - b).max()) <= 1e-6
    for k in ca:
        if k not in ("nodes", "prim_tests", "sph_tests", "tri_tests"):
            assert ca[k] == cb[k], k
    assert ca["handoffs"] > 0 and ca["nodes"] < cb["nodes"]

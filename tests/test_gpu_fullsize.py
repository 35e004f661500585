"""The benchmark workloads at their full sizes, GPU path against the oracle.

Same seeded scenes, same sizes as the timed workloads:
  * triangles: 9 displaced UV spheres (~197k triangles), 512x512, hard
    shadows -- image level, and RayList level over all 262,144 camera rays
    and every shadow ray they spawn;
  * volume: 256^3 blob field, 1024x1024, 0.5-voxel steps, early termination
    at alpha 0.99 (and at Galaxy's 0.999) -- image level, and the composited
    colour of every camera ray against the oracle's FP64 re-evaluation;
  * mixed: 512^3 blob field in 2x2x2 bricks + 4M spheres, 2048x2048, shadows
    + 4 AO rays per hit -- the whole frame;
  * every image of Galaxy's gold states at Galaxy's own 512x512 over 256^3
    radial volumes, against the oracle and against the gold PNG.

Tolerances (stated by the workloads): hit/miss agreement >= 99.99 %, hit
distance within 1e-5 relative, images within 2/255 per channel on 99.9 % of
channels with RMSE <= 1e-3, composited samples within 1e-4 of FP64.
"""
import numpy as np
import pytest

import gold_scenes as G
import oracle_lib as O
import pngio
from galaxy_gb300 import _abi as A
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

pytestmark = pytest.mark.gpu

RMSE_TOL = 1e-3
CH_TOL = 2.0 / 255
HIT_AGREE = 0.9999
T_RTOL = 1e-5
F64_TOL = 1e-4


@pytest.fixture(scope="module")
def gpu():
    from galaxy_gb300 import gpu as g
    g.init(0)
    return g


def image_close(img, ref):
    d = np.abs(img[..., :3] - ref[..., :3])
    rmse = float(np.sqrt(np.mean(d ** 2)))
    within = float(np.mean(d <= CH_TOL))
    assert rmse <= RMSE_TOL, ("rmse", rmse)
    assert within >= 0.999, ("fraction within 2/255", within, float(d.max()))
    return rmse


def hits(r):
    return (r.term & A.RAY_SURFACE) != 0


def check_trace(ta, tb):
    """Hit/miss agreement and hit distance of two traced RayLists."""
    ha, hb = hits(ta), hits(tb)
    agree = float(np.mean(ha == hb))
    assert agree >= HIT_AGREE, agree
    both = ha & hb
    np.testing.assert_allclose(ta.t[both], tb.t[both], rtol=T_RTOL)
    return agree, int(both.sum())


def test_triangles_full(gpu):
    cam, vis = scenes.triangle_spheres_scene()
    assert cam.width == cam.height == 512
    assert len(vis.operators[0].dataset.indices) > 190_000
    L = S.resolve_lights(vis.lighting, cam)
    g = gpu.Scene(vis)
    o = O.OracleScene(vis)
    img = g.render_host(cam, L)
    ref, cnt = o.render(cam, L)
    image_close(img, ref)
    c = g.counters()
    assert c["primary_rays"] == cnt["primary"] == 512 * 512
    assert c["shadow_rays"] == cnt["shadow"] > 100_000
    # RayList level: every camera ray, then every shadow ray it spawns
    rays = o.generate_initial_rays(0, cam)
    assert rays.n == 512 * 512
    ta, sa = g.trace(0, L, rays)
    tb, sb = o.trace(0, L, rays)
    check_trace(ta, tb)
    assert sa.n == sb.n == cnt["shadow"]
    np.testing.assert_array_equal(sa.x, sb.x)
    np.testing.assert_array_equal(sa.y, sb.y)
    np.testing.assert_allclose(np.stack([sa.dx, sa.dy, sa.dz]), np.stack([sb.dx, sb.dy, sb.dz]), rtol=1e-5,
                               atol=1e-6)
    ua, _ = g.trace(0, L, sb)
    ub, _ = o.trace(0, L, sb)
    agree, n_hit = check_trace(ua, ub)
    assert n_hit > 1000   # the spheres shadow each other


@pytest.mark.parametrize("alpha", [0.99, 0.999])
def test_volume_full(gpu, alpha):
    cam, vis = scenes.volume_scene()
    vis.opaque_alpha = alpha
    assert (cam.width, cam.height) == (1024, 1024)
    assert vis.operators[0].dataset.samples.shape == (256, 256, 256)
    L = S.resolve_lights(vis.lighting, cam)
    g = gpu.Scene(vis)
    o = O.OracleScene(vis)
    img = g.render_host(cam, L)
    ref, cnt = o.render(cam, L)
    image_close(img, ref)
    c = g.counters()
    assert c["primary_rays"] == cnt["primary"] > 500_000
    assert c["samples"] == cnt["samples"]
    if alpha == 0.99:
        # composited colour of every camera ray against FP64
        rays = o.generate_initial_rays(0, cam)
        ta, _ = g.trace(0, L, rays)
        ref64 = o.trace_f64(0, rays)
        got = np.stack([ta.r, ta.g, ta.b, ta.o], -1).astype(np.float64)
        err = np.abs(got - ref64)
        assert float(np.quantile(err, 0.9999)) <= F64_TOL, float(err.max())


def test_mixed_full(gpu):
    cam, vis = scenes.mixed_scene()
    assert (cam.width, cam.height) == (2048, 2048)
    assert vis.operators[1].dataset.centers.shape[0] == 4_000_000
    L = S.resolve_lights(vis.lighting, cam)
    g = gpu.Scene(vis)
    img = g.render_host(cam, L)
    c = g.counters()
    ref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(img, ref)
    assert c["handoffs"] > 0 and c["overflow"] == 0
    assert c["primary_rays"] == cnt["primary"]
    for k in ("shadow", "ao"):
        assert abs(c[k + "_rays"] - cnt[k]) <= 1e-4 * cnt[k] + 8, (k, c[k + "_rays"], cnt[k])


GOLD_CASES = [(name, k) for name in G.STATES for k in range(3 if name == "nineBalls" else 1)]


@pytest.mark.parametrize("name,k", GOLD_CASES)
def test_gold_states_full(gpu, name, k):
    """Galaxy's gold states as gxywriter renders them (512x512, 256^3 radial
    volumes): the GPU image against the oracle, and against Galaxy's gold
    PNG with the criteria the oracle is pinned by."""
    cam, vis, gold = G.load_gold_state(name)[k]
    assert (cam.width, cam.height) == (512, 512)
    L = S.resolve_lights(vis.lighting, cam)
    g = gpu.Scene(vis)
    img = g.render_host(cam, L)
    ref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(img, ref)
    c = g.counters()
    assert c["primary_rays"] == cnt["primary"]
    assert c["shadow_rays"] == cnt["shadow"] and c["ao_rays"] == cnt["ao"]
    q = O.quantize(img)
    png = pngio.read_png(gold)
    d = np.abs(q[..., :3].astype(int) - png[..., :3].astype(int))
    px = d.max(-1)
    assert d.mean() < 0.5, d.mean()
    assert (px > 2).mean() < 0.03, (px > 2).mean()
    assert (px > 8).mean() < 0.001, (px > 8).mean()

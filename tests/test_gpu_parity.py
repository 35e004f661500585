"""GPU path against the CPU oracle on the same seeded scenes.

Tolerances (floating-point path; the GPU kernels and the oracle evaluate the
same IEEE single-precision expressions in the same order, so most results are
bit-identical; differences come from the order of float atomics in the
framebuffer and from the rare primitive whose hit distance ties):
  * primary and shadow hit/miss agreement >= 99.99 %,
  * hit distance t within 1e-5 relative,
  * images: max 2/255 per channel on 99.9 % of channels and RMSE <= 1e-3,
  * composited volume samples within 1e-4 of the oracle's FP64 re-evaluation.
"""
import numpy as np
import pytest

import gold_scenes as G
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


def image_close(img, ref, rmse_tol=1e-3, ch_tol=2.0 / 255, frac=0.999):
    d = np.abs(img[..., :3] - ref[..., :3])
    rmse = float(np.sqrt(np.mean(d ** 2)))
    ok = float(np.mean(d <= ch_tol))
    assert rmse <= rmse_tol, ("rmse", rmse)
    assert ok >= frac, ("fraction within %g" % ch_tol, ok, float(d.max()))
    return rmse, float(d.max())


def render_both(gpu, cam, vis, threads=8):
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    img = sc.render_host(cam, L)
    ref, cnt = O.OracleScene(vis).render(cam, L, nthreads=threads)
    return img, ref, sc, cnt


@pytest.mark.parametrize("name", ["absolute", "absolute-shadow", "camera-shadow", "infinite", "nineBalls",
                                  "oneBall", "xyz"])
def test_gold_scenes_match_oracle(gpu, name):
    for cam, vis, _ in G.load_gold_state(name, size=192, n=128)[:2]:
        img, ref, sc, cnt = render_both(gpu, cam, vis)
        image_close(img, ref)
        c = sc.counters()
        assert c["primary_rays"] == cnt["primary"]
        assert c["shadow_rays"] == cnt["shadow"] and c["ao_rays"] == cnt["ao"]


def test_partitioned_gold_scene(gpu):
    cam, vis, _ = G.load_gold_state("absolute-shadow", size=160, n=96, partitions=(2, 2, 1))[0]
    img, ref, sc, cnt = render_both(gpu, cam, vis)
    image_close(img, ref)
    c = sc.counters()
    assert c["handoffs"] > 0 and c["primary_rays"] == cnt["primary"]


def test_triangle_scene(gpu):
    cam, vis = scenes.triangle_spheres_scene(width=160, height=160, n_seg=24)
    img, ref, sc, cnt = render_both(gpu, cam, vis)
    image_close(img, ref)
    c = sc.counters()
    assert c["primary_rays"] == 160 * 160 == cnt["primary"]
    assert c["shadow_rays"] == cnt["shadow"]


@pytest.mark.parametrize("split", [(0, 0, 1), (1, 0, 1), (0, 1, 1), (1, 1, 1), (1, 1, 0)])
def test_mixed_partitioned_scene(gpu, split):
    """Every tracing variant: one pass, split shadow/AO, split camera rays
    with the warp-cooperative (third flag 1) or the per-lane camera query."""
    gpu.set_tuning(gpu.TUNE_SPLIT_SECONDARY, split[0])
    gpu.set_tuning(gpu.TUNE_SPLIT_PRIMARY, split[1])
    gpu.set_tuning(gpu.TUNE_CAMERA_PACKET, split[2])
    cam, vis = scenes.mixed_scene(n=64, n_spheres=20000, width=128, height=128, partitions=(2, 2, 2), n_ao=4)
    try:
        img, ref, sc, cnt = render_both(gpu, cam, vis)
    finally:
        gpu.set_tuning(gpu.TUNE_SPLIT_SECONDARY, 1)
        gpu.set_tuning(gpu.TUNE_SPLIT_PRIMARY, 1)
        gpu.set_tuning(gpu.TUNE_CAMERA_PACKET, 1)
    image_close(img, ref)
    c = sc.counters()
    assert c["primary_rays"] == cnt["primary"]
    assert abs(c["ao_rays"] - cnt["ao"]) <= 0.001 * cnt["ao"] + 8


def test_query_and_march_register_budgets_same_frames(gpu):
    """The shadow/AO query at 2, 3 or 4 resident blocks per SM
    (GXY_TUNE_QUERY_BLOCKS), the camera-ray march at 2 or 3
    (GXY_TUNE_PMARCH_BLOCKS) and the camera and handed-off primary queries
    at 2 or 4 (GXY_TUNE_PQUERY_BLOCKS): the same frames and counters, equal
    to the oracle."""
    cam, vis = scenes.mixed_scene(n=64, n_spheres=20000, width=128, height=128, partitions=(2, 2, 2), n_ao=4)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    out = []
    try:
        for qb, pb, cb in ((3, 2, 2), (4, 3, 4), (3, 3, 2), (4, 2, 4), (2, 2, 2)):
            gpu.set_tuning(gpu.TUNE_QUERY_BLOCKS, qb)
            gpu.set_tuning(gpu.TUNE_PMARCH_BLOCKS, pb)
            gpu.set_tuning(gpu.TUNE_PQUERY_BLOCKS, cb)
            out.append((sc.render_host(cam, L), sc.counters()))
    finally:
        gpu.set_tuning(gpu.TUNE_QUERY_BLOCKS, 3)
        gpu.set_tuning(gpu.TUNE_PMARCH_BLOCKS, 2)
        gpu.set_tuning(gpu.TUNE_PQUERY_BLOCKS, 2)
    for img, c in out[1:]:
        assert float(np.abs(img - out[0][0]).max()) <= 1e-6
        for k in ("primary_rays", "shadow_rays", "ao_rays", "terminated", "samples", "nodes"):
            assert c[k] == out[0][1][k], k
    ref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(out[0][0], ref)
    with pytest.raises(gpu.GxyError):
        gpu.set_tuning(gpu.TUNE_QUERY_BLOCKS, 5)
    with pytest.raises(gpu.GxyError):
        gpu.set_tuning(gpu.TUNE_PMARCH_BLOCKS, 4)
    with pytest.raises(gpu.GxyError):
        gpu.set_tuning(gpu.TUNE_PQUERY_BLOCKS, 3)


@pytest.mark.parametrize("split_primary", [0, 1])
@pytest.mark.parametrize("blocks", [2, 3])
def test_volume_scene(gpu, split_primary, blocks):
    gpu.set_tuning(gpu.TUNE_SPLIT_PRIMARY, split_primary)
    gpu.set_tuning(gpu.TUNE_BLOCKS_PER_SM, blocks)
    cam, vis = scenes.volume_scene(n=96, width=128, height=128)
    try:
        img, ref, sc, cnt = render_both(gpu, cam, vis)
    finally:
        gpu.set_tuning(gpu.TUNE_SPLIT_PRIMARY, 1)
        gpu.set_tuning(gpu.TUNE_BLOCKS_PER_SM, 3)
    image_close(img, ref)
    assert sc.counters()["samples"] == cnt["samples"]


# ------------------------------------------------------------ RayList level
def _fields_equal(a, b, names, rtol=0.0):
    for f in names:
        x, y = getattr(a, f), getattr(b, f)
        if rtol == 0.0:
            assert np.array_equal(x, y), f
        else:
            np.testing.assert_allclose(x, y, rtol=rtol, atol=1e-6, err_msg=f)


def test_raylist_camera_rays_identical(gpu):
    cam, vis = scenes.mixed_scene(n=64, n_spheres=5000, width=96, height=80, partitions=(2, 2, 1))
    g = gpu.Scene(vis)
    o = O.OracleScene(vis)
    for p in range(4):
        a = g.generate_initial_rays(p, cam)
        b = o.generate_initial_rays(p, cam)
        assert a.n == b.n
        _fields_equal(a, b, ("x", "y", "type", "ox", "oy", "oz", "dx", "dy", "dz", "t", "tMax"))


def _hit_agreement(a, b):
    ha = (a.term & A.RAY_SURFACE) != 0
    hb = (b.term & A.RAY_SURFACE) != 0
    return float(np.mean(ha == hb)), ha & hb


@pytest.mark.parametrize("which", ["triangles", "mixed", "iso", "pathlines"])
def test_raylist_trace_matches_oracle(gpu, which):
    if which == "triangles":
        cam, vis = scenes.triangle_spheres_scene(width=128, height=128, n_seg=32)
    elif which == "pathlines":
        cam, vis = scenes.pathlines_scene(n_lines=600, n_vertices=48, width=128, height=128)
    elif which == "mixed":
        cam, vis = scenes.mixed_scene(n=64, n_spheres=20000, width=96, height=96, partitions=(1, 1, 1), n_ao=4)
    else:
        cam, vis, _ = G.load_gold_state("oneBall", size=96, n=96)[0]
    L = S.resolve_lights(vis.lighting, cam)
    g = gpu.Scene(vis)
    o = O.OracleScene(vis)
    rays = o.generate_initial_rays(0, cam)
    ta, sa = g.trace(0, L, rays)
    tb, sb = o.trace(0, L, rays)
    agree, both = _hit_agreement(ta, tb)
    assert agree >= 0.9999, agree
    np.testing.assert_allclose(ta.t[both], tb.t[both], rtol=1e-5)
    assert sa.n == sb.n
    np.testing.assert_allclose(np.stack([ta.r, ta.g, ta.b, ta.o]), np.stack([tb.r, tb.g, tb.b, tb.o]), atol=2e-6)
    # secondary rays: same order (AO block, then shadow block), same payloads
    _fields_equal(sa, sb, ("x", "y", "type"))
    _fields_equal(sa, sb, ("ox", "oy", "oz", "dx", "dy", "dz", "r", "g", "b", "tMax"), rtol=1e-5)
    # trace the secondaries: shadow/AO hit/miss agreement
    ua, _ = g.trace(0, L, sb)
    ub, _ = o.trace(0, L, sb)
    agree2, _ = _hit_agreement(ua, ub)
    assert agree2 >= 0.9999, agree2
    # classify and destinations
    ca = gpu.classify(ua)
    cb = o.classify(ub)
    assert np.mean(ca.classification == cb.classification) >= 0.9999


@pytest.mark.parametrize("case", ["lines", "lines_bricks", "lines_volume", "lines_volume_refill"])
def test_pathlines_match_oracle(gpu, case):
    """PathLinesVis: capsule segments (DataDrivenPathLines.ispc:100-203) with
    the post-intersect colour mapping, alone, across 2x2x1 bricks, and inside
    a volume (split passes)."""
    if case == "lines":
        cam, vis = scenes.pathlines_scene(n_lines=800, n_vertices=48, width=128, height=128)
    elif case == "lines_bricks":
        cam, vis = scenes.pathlines_scene(n_lines=800, n_vertices=48, width=128, height=128, partitions=(2, 2, 1))
    else:
        cam, vis = scenes.pathlines_scene(n_lines=800, n_vertices=48, width=128, height=128, volume=True,
                                          partitions=(2, 1, 1))
    gpu.set_tuning(gpu.TUNE_CAMERA_PACKET, 0 if case.endswith("refill") else 1)
    try:
        img, ref, sc, cnt = render_both(gpu, cam, vis)
    finally:
        gpu.set_tuning(gpu.TUNE_CAMERA_PACKET, 1)
    image_close(img, ref)
    c = sc.counters()
    assert c["primary_rays"] == cnt["primary"]
    assert c["shadow_rays"] == cnt["shadow"] and c["ao_rays"] == cnt["ao"]
    assert c["shadow_rays"] > 100   # the lines are hit


def test_partition_document_render(gpu):
    """Bricks from a Galaxy partition document: uneven bricks match the
    oracle, and a document equal to the 2x2x1 grid renders the grid's image."""
    doc = {"parts": [{"extent": [0, 0.3, 0, 1, 0, 1]}, {"extent": [0.3, 0.7, 0, 1, 0, 1]},
                     {"extent": [0.7, 1, 0, 0.5, 0, 1]}, {"extent": [0.7, 1, 0.5, 1, 0, 1]}]}
    cam, vis = scenes.pathlines_scene(n_lines=800, n_vertices=48, width=128, height=128)
    vis.partition_extents = S.partition_document(doc)
    img, ref, sc, cnt = render_both(gpu, cam, vis)
    image_close(img, ref)
    assert sc.counters()["primary_rays"] == cnt["primary"]
    grid = {"parts": [{"extent": [x0, x1, y0, y1, 0, 1]} for (y0, y1) in ((0, 0.5), (0.5, 1))
                      for (x0, x1) in ((0, 0.5), (0.5, 1))]}
    cam, vis = scenes.pathlines_scene(n_lines=800, n_vertices=48, width=128, height=128, partitions=(2, 2, 1))
    L = S.resolve_lights(vis.lighting, cam)
    a = gpu.Scene(vis).render_host(cam, L)
    vis.partition_extents = S.partition_document(grid)
    b = gpu.Scene(vis).render_host(cam, L)
    np.testing.assert_allclose(a, b, atol=1e-6)


def test_assign_destinations_identical(gpu):
    cam, vis = scenes.mixed_scene(n=64, n_spheres=2000, width=64, height=64, partitions=(2, 2, 2))
    L = S.resolve_lights(vis.lighting, cam)
    g = gpu.Scene(vis)
    o = O.OracleScene(vis)
    for p in range(8):
        rays = o.generate_initial_rays(p, cam)
        if rays.n == 0:
            continue
        tb, _ = o.trace(p, L, rays)
        cb = o.classify(tb)
        da = g.assign_destinations(p, cb)
        db = o.assign_destinations(p, cb)
        assert np.array_equal(da.classification, db.classification)


def test_accumulate_terminated(gpu):
    rng = np.random.default_rng(5)
    n = 5000
    r = A.RayListArrays(n, x=rng.integers(0, 32, n), y=rng.integers(0, 16, n),
                        r=rng.normal(size=n), g=rng.normal(size=n), b=rng.normal(size=n), o=rng.normal(size=n),
                        classification=rng.choice([A.TERMINATED, A.DROP_ON_FLOOR, 3], n))
    fb = np.zeros((16, 32, 4), np.float32)
    gpu.accumulate_terminated(r, fb)
    ref = np.zeros((16, 32, 4), np.float64)
    m = r.classification == A.TERMINATED
    np.add.at(ref, (r.y[m], r.x[m]), np.stack([r.r, r.g, r.b, r.o], -1)[m])
    np.testing.assert_allclose(fb, ref, atol=1e-4)


def test_volume_composite_fp64(gpu):
    """Composited primary-ray colour against the oracle's FP64 re-evaluation
    of the same sample positions."""
    cam, vis = scenes.volume_scene(n=128, width=96, height=96)
    L = S.resolve_lights(vis.lighting, cam)
    g = gpu.Scene(vis)
    o = O.OracleScene(vis)
    rays = o.generate_initial_rays(0, cam)
    ta, _ = g.trace(0, L, rays)
    ref64 = o.trace_f64(0, rays)
    got = np.stack([ta.r, ta.g, ta.b, ta.o], -1).astype(np.float64)
    err = np.abs(got - ref64)
    assert float(np.quantile(err, 0.9999)) <= 1e-4, float(err.max())


def test_bvh_stats(gpu):
    cam, vis = scenes.triangle_spheres_scene(width=64, height=64, n_seg=40)
    g = gpu.Scene(vis)
    info = g.bvh_info()
    n = len(vis.operators[0].dataset.indices)
    assert info["prim_refs"] == n
    assert n / 32 <= info["nodes"] <= n


def test_errors_are_reported(gpu):
    from galaxy_gb300.gpu import GxyError
    cam, vis = scenes.triangle_spheres_scene(width=32, height=32, n_seg=8)
    g = gpu.Scene(vis)
    L = vis.lighting.c()
    L.n_lights = 99
    with pytest.raises(GxyError):
        g.render_host(cam, L)
    bad = vis.lighting.c()
    bad.types[0] = 1    # unresolved camera light
    with pytest.raises(GxyError):
        g.render_host(cam, bad)


@pytest.mark.parametrize("which", ["triangles", "mixed", "pathlines"])
def test_sah_top_bvh_matches_oracle(gpu, which):
    """BVH with the binned-SAH top over radix-tree clusters (small clusters,
    so the top tree is deep): same images as the oracle."""
    gpu.set_tuning(gpu.TUNE_BVH_SAH, 16)
    try:
        if which == "triangles":
            cam, vis = scenes.triangle_spheres_scene(width=128, height=128, n_seg=24)
        elif which == "mixed":
            cam, vis = scenes.mixed_scene(n=64, n_spheres=20000, width=112, height=112, partitions=(2, 2, 1), n_ao=2)
        else:
            cam, vis = scenes.pathlines_scene(n_lines=500, n_vertices=32, width=112, height=112)
        img, ref, sc, cnt = render_both(gpu, cam, vis)
        assert sc.bvh_info()["nodes"] > 0
    finally:
        gpu.set_tuning(gpu.TUNE_BVH_SAH, 0)
    image_close(img, ref)
    c = sc.counters()
    assert c["primary_rays"] == cnt["primary"] and c["shadow_rays"] == cnt["shadow"]


@pytest.mark.parametrize("shortcut", [0, 8])
@pytest.mark.parametrize("which", ["mixed", "pathlines"])
def test_continued_shadow_ao_rays_same_frames(gpu, which, shortcut):
    """Shadow/AO rays that move to the next brick march on in the same lane
    (GXY_TUNE_CONTINUE 1) or wait for the next generation (0), with and
    without the occlusion shortcut: the same frames and ray counts, fewer
    generations, equal to the oracle."""
    if which == "mixed":
        cam, vis = scenes.mixed_scene(n=64, n_spheres=20000, width=128, height=128, partitions=(2, 2, 2), n_ao=4)
    else:
        cam, vis = scenes.pathlines_scene(n_lines=600, n_vertices=48, width=112, height=112, volume=True,
                                          partitions=(2, 2, 1))
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    mode = gpu.get_tuning(gpu.TUNE_SKIP_MODE)
    out = {}
    try:
        gpu.set_tuning(gpu.TUNE_SKIP_MODE, (mode & ~8) | shortcut)
        for v in (0, 1):
            gpu.set_tuning(gpu.TUNE_CONTINUE, v)
            out[v] = (sc.render_host(cam, L), sc.counters())
    finally:
        gpu.set_tuning(gpu.TUNE_CONTINUE, 1)
        gpu.set_tuning(gpu.TUNE_SKIP_MODE, mode)
    (a, ca), (b, cb) = out[1], out[0]
    assert float(np.abs(a - b).max()) <= 1e-6
    for k in ("primary_rays", "shadow_rays", "ao_rays", "terminated", "dropped", "handoffs", "segments", "samples"):
        assert ca[k] == cb[k], k
    assert cb["handoffs"] > 0 and ca["bounces"] <= cb["bounces"]
    ref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(a, ref)


@pytest.mark.parametrize("sah", [0, 16])
@pytest.mark.parametrize("which", ["triangles", "mixed"])
def test_cost_collapse_same_frames_fewer_nodes(gpu, which, sah):
    """BVH8 nodes grouped by the surface-area cost programme
    (GXY_TUNE_BVH_COLLAPSE 1) or greedily (0), under the radix tree alone and
    under a binned-SAH top: the same frames and ray counts (the closest hit
    does not depend on the tree), fewer wide nodes."""
    if which == "triangles":
        cam, vis = scenes.triangle_spheres_scene(width=128, height=128, n_seg=32)
    else:
        cam, vis = scenes.mixed_scene(n=64, n_spheres=20000, width=112, height=112, partitions=(2, 2, 1), n_ao=2)
    L = S.resolve_lights(vis.lighting, cam)
    out = {}
    try:
        gpu.set_tuning(gpu.TUNE_BVH_SAH, sah)
        for v in (0, 1):
            gpu.set_tuning(gpu.TUNE_BVH_COLLAPSE, v)
            sc = gpu.Scene(vis)
            out[v] = (sc.render_host(cam, L), sc.counters(), sc.bvh_info())
    finally:
        gpu.set_tuning(gpu.TUNE_BVH_COLLAPSE, 1)
        gpu.set_tuning(gpu.TUNE_BVH_SAH, 0)
    (a, ca, ia), (b, cb, ib) = out[1], out[0]
    assert float(np.abs(a - b).max()) <= 1e-6
    for k in ("primary_rays", "shadow_rays", "ao_rays", "terminated", "samples"):
        assert ca[k] == cb[k], k
    assert ia["prim_refs"] == ib["prim_refs"]
    assert ia["nodes"] < ib["nodes"]
    ref, cnt = O.OracleScene(vis).render(cam, L)
    image_close(a, ref)

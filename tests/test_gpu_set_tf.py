"""Transfer-function changes on a committed scene (gxy_gpu_scene_set_tf) and
scene views (gxy_gpu_scene_view).

MappedVis_set_transferFunction (MappedVis.ispc:35) replaces an operator's
transfer function without touching its data.  Here a frame after set_tf
must equal a frame of a fresh commit with that transfer function -- the
same images (to the order of float atomics) and the same counters,
including the samples whose voxels the empty-space skipping leaves unread,
so the recomputed clear-brick flags are exactly the fresh commit's -- and
must match the oracle.  A view renders its own transfer function while the
scene it came from keeps the old one.
"""
import copy

import numpy as np
import pytest

import oracle_lib as O
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

pytestmark = pytest.mark.gpu

COUNTERS = ("primary_rays", "shadow_rays", "ao_rays", "segments", "handoffs", "terminated", "samples",
            "samples_skipped", "nodes", "prim_tests")


@pytest.fixture(scope="module")
def gpu():
    from galaxy_gb300 import gpu as g
    g.init(0)
    return g


def image_close(img, ref, rmse_tol=1e-3, ch_tol=2.0 / 255, frac=0.999):
    d = np.abs(img[..., :3] - ref[..., :3])
    assert float(np.sqrt(np.mean(d ** 2))) <= rmse_tol
    assert float(np.mean(d <= ch_tol)) >= frac


def with_tfs(vis, vol_opacity=None, vol_colormap=None, sph_colormap=None):
    """A copy of vis with other transfer functions for the volume (operator
    0) and the particles (operator 1)."""
    v = copy.copy(vis)
    v.operators = [copy.copy(op) for op in vis.operators]
    if vol_opacity is not None:
        v.operators[0].opacitymap = vol_opacity
    if vol_colormap is not None:
        v.operators[0].colormap = vol_colormap
    if sph_colormap is not None:
        v.operators[1].colormap = sph_colormap
    return v


OPAC_B = [(0.0, 0.0), (0.45, 0.0), (1.0, 0.95)]          # higher threshold: more clear bricks
OPAC_C = [(0.0, 0.02), (0.3, 0.1), (1.0, 0.6)]           # no zero-opacity range: no clear bricks
CMAP_B = [(0.0, 0.9, 0.1, 0.1), (1.0, 0.1, 0.1, 0.9)]
SPH_B = [(0.0, 0.1, 0.9, 0.1), (1.0, 0.9, 0.9, 0.1)]


def frame(sc, cam, L):
    img = sc.render_host(cam, L)
    c = sc.counters()
    return img, {k: c[k] for k in COUNTERS}


def assert_same_frame(a, b):
    np.testing.assert_allclose(a[0], b[0], atol=2e-6)
    assert a[1] == b[1]


@pytest.mark.parametrize("opacity", [OPAC_B, OPAC_C])
def test_set_tf_equals_fresh_commit(gpu, opacity):
    cam, vis = scenes.mixed_scene(n=96, n_spheres=20000, width=128, height=128, partitions=(2, 2, 2), n_ao=2)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    before = frame(sc, cam, L)
    new = with_tfs(vis, vol_opacity=opacity, vol_colormap=CMAP_B, sph_colormap=SPH_B)
    sc.set_tf(gpu.VIS_VOLUME, 0, new.operators[0])
    sc.set_tf(gpu.VIS_PARTICLES, 0, new.operators[1])
    after = frame(sc, cam, L)
    fresh = frame(gpu.Scene(new), cam, L)
    assert_same_frame(after, fresh)
    assert not np.allclose(after[0], before[0])
    ref, cnt = O.OracleScene(new).render(cam, L)
    image_close(after[0], ref)
    assert after[1]["primary_rays"] == cnt["primary"]
    # and back: the original transfer functions give the original frame
    sc.set_tf(gpu.VIS_VOLUME, 0, vis.operators[0])
    sc.set_tf(gpu.VIS_PARTICLES, 0, vis.operators[1])
    assert_same_frame(frame(sc, cam, L), before)


def test_view_keeps_the_base_scene(gpu):
    cam, vis = scenes.mixed_scene(n=96, n_spheres=20000, width=112, height=112, partitions=(2, 1, 1), n_ao=2)
    L = S.resolve_lights(vis.lighting, cam)
    base = gpu.Scene(vis)
    a = frame(base, cam, L)
    new = with_tfs(vis, vol_opacity=OPAC_B, vol_colormap=CMAP_B)
    view = base.view()
    view.set_tf(gpu.VIS_VOLUME, 0, new.operators[0])
    v = frame(view, cam, L)
    assert_same_frame(v, frame(gpu.Scene(new), cam, L))
    assert_same_frame(frame(base, cam, L), a)
    # a view outlives its base: the shared datasets stay until the last handle
    base.release()
    assert_same_frame(frame(view, cam, L), v)
    view.release()


def test_set_tf_triangles(gpu):
    cam, vis = scenes.triangle_spheres_scene(width=128, height=128, n_seg=24)
    L = S.resolve_lights(vis.lighting, cam)
    sc = gpu.Scene(vis)
    new = copy.copy(vis)
    new.operators = [copy.copy(vis.operators[0])]
    new.operators[0].colormap = CMAP_B
    sc.set_tf(gpu.VIS_TRIANGLES, 0, new.operators[0])
    got = frame(sc, cam, L)
    assert_same_frame(got, frame(gpu.Scene(new), cam, L))
    ref, _ = O.OracleScene(new).render(cam, L)
    image_close(got[0], ref)


def test_set_tf_refuses_unknown_operator(gpu):
    from galaxy_gb300.gpu import GxyError
    cam, vis = scenes.triangle_spheres_scene(width=32, height=32, n_seg=8)
    sc = gpu.Scene(vis)
    with pytest.raises(GxyError):
        sc.set_tf(gpu.VIS_VOLUME, 0, vis.operators[0])
    with pytest.raises(GxyError):
        sc.set_tf(gpu.VIS_TRIANGLES, 1, vis.operators[0])

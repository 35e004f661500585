"""Pin the CPU oracle against Galaxy's own gold images.

Galaxy's gold tests (tests/image-gold-tests.sh in the Galaxy tree) render each
state file with gxywriter at 512x512 and accept an image when perceptualdiff
-fov 85 passes.  Here the oracle renders the same states (radial volumes
regenerated analytically) and each image must agree with its gold:
mean absolute difference below 0.5/255 per channel, fewer than 3% of pixels
off by more than 2/255 and fewer than 0.1% off by more than 8/255 (edge
pixels of isosurfaces, where OSPRay's gradient and our stated central
difference differ).
"""
import numpy as np
import pytest

import gold_scenes as G
import oracle_lib as O
import pngio
from galaxy_gb300 import scene as S

CASES = [(name, k) for name in G.STATES for k in range(3 if name == "nineBalls" else 1)]


@pytest.mark.parametrize("name,k", CASES)
def test_oracle_matches_gold(name, k):
    cam, vis, gold = G.load_gold_state(name)[k]
    sc = O.OracleScene(vis)
    fb, cnt = sc.render(cam, S.resolve_lights(vis.lighting, cam), nthreads=8)
    img = O.quantize(fb)
    g = pngio.read_png(gold)
    d = np.abs(img[..., :3].astype(int) - g[..., :3].astype(int))
    px = d.max(-1)
    assert d.mean() < 0.5, d.mean()
    assert (px > 2).mean() < 0.03, (px > 2).mean()
    assert (px > 8).mean() < 0.001, (px > 8).mean()
    assert (img[..., 3] == 255).all()


def test_partitioned_oracle_matches_gold():
    """Galaxy runs the gold tests at np=1 and np=2 against the same golds: a
    2-brick partition must also pass."""
    cam, vis, gold = G.load_gold_state("absolute-shadow", partitions=(2, 1, 1))[0]
    sc = O.OracleScene(vis)
    fb, cnt = sc.render(cam, S.resolve_lights(vis.lighting, cam), nthreads=8)
    img = O.quantize(fb)
    g = pngio.read_png(gold)
    d = np.abs(img[..., :3].astype(int) - g[..., :3].astype(int))
    assert d.mean() < 0.5 and (d.max(-1) > 8).mean() < 0.001


def test_ao_tables_match_uv_ih():
    """The AO tables are regenerated (float32 radical inverse rounded to 6
    significant digits); they must equal UV.ih's printed tables entry by
    entry."""
    import json
    import os
    t = json.load(open(os.path.join(G.ROOT, "tests", "golden", "ao_tables.json")))
    u, v = O.ao_tables()
    assert np.array_equal(u, np.array([float(x) for x in t["randomU"]], np.float32))
    assert np.array_equal(v, np.array([float(x) for x in t["randomV"]], np.float32))


def test_tf_resample_matches_oracle():
    """Host MappedVis resampling (galaxy_gb300.scene.resample_tf) against the
    oracle's restatement of MappedVis::local_commit."""
    import ctypes as C
    from galaxy_gb300 import _abi as A
    cm = np.array([[0.0, 1.0, 0.5, 0.5], [0.25, 0.5, 1.0, 0.5], [0.5, 0.5, 0.5, 1.0], [1.0, 1.0, 0.5, 1.0]],
                  np.float32)
    om = np.array([[0.0, 0.05], [0.2, 0.02], [0.21, 0.0], [1.0, 0.0]], np.float32)
    for rng in (None, (0.1, 0.9)):
        a = S.resample_tf(cm, om, rng)
        b = A.gxy_tf()
        O.lib().oracle_tf_resample(A.fptr(cm), len(cm), A.fptr(om), len(om), rng is not None,
                                   *(rng or (0, 0)), C.byref(b))
        assert np.array_equal(np.ctypeslib.as_array(a.colors), np.ctypeslib.as_array(b.colors))
        assert np.array_equal(np.ctypeslib.as_array(a.opacities), np.ctypeslib.as_array(b.opacities))
        assert list(a.range) == list(b.range)

"""Host-side logic without a GPU: Galaxy's JSON semantics for lights and
cameras, light resolution, brick partitions (product vs oracle), state-file
loading, scene generators and the AO tables."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle_lib as O
from galaxy_gb300 import _abi as A
from galaxy_gb300 import gpu, scenes
from galaxy_gb300 import scene as S


def test_lighting_json_defaults_and_normalisation():
    L = S.Lighting.from_json({"Sources": [[0, 3, 4], [1, 2, 3, 2]], "shadows": True})
    assert L.types == [0, 2]
    np.testing.assert_allclose(L.lights[0], (0, 0.6, 0.8), rtol=1e-6)   # directional normalised (Lighting.cpp:76-90)
    assert L.lights[1] == (1.0, 2.0, 3.0)
    assert (L.Ka, L.Kd, L.n_ao, L.ao_radius, L.shadows) == (0.5, 0.5, 0, 1.0, True)
    Z = S.Lighting.from_json({"Sources": [[0, 0, 0]]})
    np.testing.assert_allclose(Z.lights[0], (0.57735,) * 3, rtol=1e-5)


def test_camera_json_quirks():
    c = S.Camera.from_json({"viewpoint": [1, 2, 3], "viewcenter": [0, 0, 0], "viewup": [0, 1, 0], "aov": 30,
                            "dimensions": [640, 480]})
    assert c.dir == (-1.0, -2.0, -3.0)
    assert (c.width, c.height) == (640, 640)   # height from dimensions[0] (Camera.cpp:267-271)
    with pytest.raises(ValueError):
        S.Camera.from_json({"viewpoint": [0, 0, 1], "viewup": [0, 1, 0], "aov": 30})


def test_resolve_lights_python_matches_c_abi():
    L = S.Lighting.from_json({"Sources": [[1, 2, 3, 1], [-1, -1, 0, 0], [4, 5, 6, 2]]})
    cam = S.Camera((1, 3, -3), (-1, -3, 3), (0, 1, 0), 30)
    a = S.resolve_lights(L, cam).c()
    b = gpu.resolve_lights(L, cam)
    assert list(a.types)[:3] == list(b.types)[:3] == [2, 0, 2]
    for i in range(3):
        assert list(a.lights[i]) == list(b.lights[i])


def test_register_budget_and_continue_knobs():
    """Host side only: the per-kernel register-budget knobs take the block
    counts their kernels are built for and refuse the rest; the knobs read
    back what was set; GXY_TUNE_CONTINUE is an on/off switch."""
    knobs = {gpu.TUNE_QUERY_BLOCKS: ((2, 3, 4), (1, 5)), gpu.TUNE_PMARCH_BLOCKS: ((2, 3), (1, 4)),
             gpu.TUNE_PQUERY_BLOCKS: ((2, 4), (3, 5))}
    for knob, (good, bad) in knobs.items():
        before = gpu.get_tuning(knob)
        try:
            for v in good:
                gpu.set_tuning(knob, v)
                assert gpu.get_tuning(knob) == v
            for v in bad:
                with pytest.raises(gpu.GxyError):
                    gpu.set_tuning(knob, v)
                assert gpu.get_tuning(knob) == good[-1]
        finally:
            gpu.set_tuning(knob, before)
    before = gpu.get_tuning(gpu.TUNE_CONTINUE)
    try:
        gpu.set_tuning(gpu.TUNE_CONTINUE, 0)
        assert gpu.get_tuning(gpu.TUNE_CONTINUE) == 0
        gpu.set_tuning(gpu.TUNE_CONTINUE, 7)
        assert gpu.get_tuning(gpu.TUNE_CONTINUE) == 1
    finally:
        gpu.set_tuning(gpu.TUNE_CONTINUE, before)
    assert (gpu.get_tuning(gpu.TUNE_QUERY_BLOCKS), gpu.get_tuning(gpu.TUNE_PMARCH_BLOCKS),
            gpu.get_tuning(gpu.TUNE_PQUERY_BLOCKS), gpu.get_tuning(gpu.TUNE_CONTINUE)) == (3, 2, 2, 1)


@pytest.mark.parametrize("parts", [(1, 1, 1), (2, 1, 1), (2, 2, 2), (3, 2, 1)])
def test_partitions_product_equals_oracle(parts):
    vol = scenes.radial_volume("oneBall", 40)
    vis = S.Visualization([S.VolumeVis(vol, isovalues=[0.3])], partitions=parts)
    osc = O.OracleScene(vis)
    n = parts[0] * parts[1] * parts[2]
    for p in range(n):
        a = gpu.partition_layout(vis, p)
        b = osc.partition_info(p)
        assert list(a.local_box) == list(b.local_box)
        assert list(a.global_box) == list(b.global_box)
        assert list(a.neighbors) == list(b.neighbors)
        assert a.n_partitions == n


def test_geometry_partitions_product_equals_oracle():
    cam, vis = scenes.triangle_spheres_scene(width=8, height=8, n_seg=8, partitions=(2, 1, 2))
    vis.box = None
    osc = O.OracleScene(vis)
    for p in range(4):
        a, b = gpu.partition_layout(vis, p), osc.partition_info(p)
        assert list(a.local_box) == list(b.local_box) and list(a.neighbors) == list(b.neighbors)


def test_load_state_file(tmp_path):
    f = scenes.radial_fields(16)["oneBall"]
    f.tofile(str(tmp_path / "ball.raw"))
    (tmp_path / "ball.vol").write_text("float\n-1 -1 -1\n16 16 16\n0.133333 0.133333 0.133333\nball.raw\n")
    state = {"Datasets": [{"name": "b", "type": "Volume", "filename": "ball.vol"}],
             "Renderer": {"epsilon": 0.002},
             "Visualizations": [{"Lighting": {"Sources": [[1, 0, 0, 1]], "ao count": 2},
                                 "operators": [{"type": "Volume", "dataset": "b", "isovalues": [0.5],
                                                "colormap": [[0, 1, 0, 0], [1, 0, 0, 1]]}]}],
             "Cameras": [{"viewpoint": [0, 0, 4], "viewcenter": [0, 0, 0], "viewup": [0, 1, 0], "aov": 30},
                         {"viewpoint": [4, 0, 0], "viewdirection": [-1, 0, 0], "viewup": [0, 1, 0], "aov": 45}]}
    (tmp_path / "s.state").write_text(json.dumps(state))
    rend, eps = S.load_state(str(tmp_path / "s.state"))
    assert eps == 0.002 and len(rend) == 2
    cam, vis = rend[1]
    assert vis.epsilon == 0.002 and vis.lighting.n_ao == 2 and vis.lighting.types == [1]
    d = vis.desc()
    assert d.n_volumes == 1 and d.volumes[0].n_isovalues == 1 and list(d.volumes[0].counts) == [16, 16, 16]
    assert np.array_equal(vis.operators[0].dataset.samples.reshape(-1), f.reshape(-1))


def test_generators_are_seeded():
    a = scenes.sphere_cloud(1000, seed=4)
    b = scenes.sphere_cloud(1000, seed=4)
    assert np.array_equal(a.centers, b.centers) and np.array_equal(a.data, b.data)
    v1 = scenes.blob_field(24, 5, 9)
    v2 = scenes.blob_field(24, 5, 9)
    assert np.array_equal(v1, v2)
    m = scenes.triangle_spheres(seed=0, n_seg=12)
    assert len(m.indices) == 9 * 2 * 12 * 11 and np.isfinite(m.normals).all()


def test_tf_resample_edges():
    tf = S.resample_tf([(0.0, 0, 0, 0), (1.0, 1, 1, 1)], [(0.0, 0.0), (0.5, 1.0), (1.0, 0.0)])
    op = np.ctypeslib.as_array(tf.opacities)
    assert op[0] == 0.0 and op[-1] == 0.0 and abs(op[127] - 0.996) < 0.01
    assert list(tf.range) == [0.0, 1.0]


def test_autotune_descent_finds_the_separable_optimum():
    """The autotuner's search (autotune.descend) on a synthetic cost with a
    known optimum: a sum of one term per knob reaches it in one sweep plus
    a confirming one, measures each setting once, and reports the best."""
    from galaxy_gb300 import autotune
    knobs = (("a", 1, (1, 2, 3)), ("b", 2, (8, 16, 32)), ("c", 3, (0, 1)))
    target = {"a": 3, "b": 8, "c": 1}
    calls = []

    def measure(s):
        calls.append(dict(s))
        return sum(abs(knobs[i][2].index(s[n]) - knobs[i][2].index(target[n])) + 1.0
                   for i, (n, _, _) in enumerate(knobs))

    best, ms, results = autotune.descend(measure, {"a": 1, "b": 16, "c": 0}, knobs, passes=3)
    assert best == target and ms == 3.0
    keys = [tuple(sorted(c.items())) for c in calls]
    assert len(keys) == len(set(keys)) == len(results)
    assert min(r["ms_per_frame"] for r in results) == ms


def test_autotune_descent_keeps_start_when_nothing_is_faster():
    from galaxy_gb300 import autotune
    knobs = (("a", 1, (1, 2)), ("b", 2, (4, 8)))
    best, ms, results = autotune.descend(lambda s: 5.0 if s == {"a": 2, "b": 8} else 9.0,
                                         {"a": 2, "b": 8}, knobs)
    assert best == {"a": 2, "b": 8} and ms == 5.0 and len(results) == 3


def test_autotune_descent_ignores_gains_within_the_noise_margin():
    """With min_gain, a setting faster by less than that fraction does not
    replace the current one; a larger gain still does."""
    from galaxy_gb300 import autotune
    knobs = (("a", 1, (1, 2)), ("b", 2, (4, 8)))
    cost = {(1, 4): 10.0, (2, 4): 9.97, (1, 8): 9.0, (2, 8): 8.99}
    best, ms, _ = autotune.descend(lambda s: cost[(s["a"], s["b"])], {"a": 1, "b": 4}, knobs, passes=3,
                                   min_gain=0.005)
    assert best == {"a": 1, "b": 8} and ms == 9.0
    best0, ms0, _ = autotune.descend(lambda s: cost[(s["a"], s["b"])], {"a": 1, "b": 4}, knobs, passes=3)
    assert best0 == {"a": 2, "b": 8} and ms0 == 8.99


def test_poisson_requests_are_seeded_and_shaped():
    """Serving arrivals: Poisson at the given rate (mean gap 1/rate),
    image sides log-uniform within the range, deterministic per seed."""
    from galaxy_gb300 import serve

    def make(rng, rid, t, key, side):
        return (rid, t, key, side)

    a = serve.poisson_requests(200.0, 4000, ["x", "y"], make, seed=3, side_range=(256, 4096))
    b = serve.poisson_requests(200.0, 4000, ["x", "y"], make, seed=3, side_range=(256, 4096))
    assert a == b
    t = np.array([r[1] for r in a])
    assert np.all(np.diff(t) > 0)
    assert abs(np.mean(np.diff(t)) - 1 / 200.0) < 0.1 / 200.0
    sides = np.array([r[3] for r in a])
    assert sides.min() >= 256 and sides.max() <= 4096
    # log-uniform: about half the sides below the geometric mean 1024
    assert 0.45 < np.mean(sides < 1024) < 0.55
    assert {r[2] for r in a} == {"x", "y"}


def test_serving_summary():
    from types import SimpleNamespace as R
    from galaxy_gb300 import serve
    reqs = [R(arrival=0.0, t_done=0.010 * (i + 1), rays=100, refused=False) for i in range(100)]
    reqs.append(R(arrival=0.0, t_done=None, rays=0, refused=True))
    s = serve.summarize(reqs, makespan=2.0)
    assert s["requests"] == 101 and s["completed"] == 100 and s["refused"] == 1
    assert s["rays"] == 10000 and s["rays_per_s"] == 5000.0
    assert abs(s["p50_ms"] - 505.0) < 1e-6 and abs(s["p99_ms"] - 990.1) < 1e-6


def test_algorithmic_bytes_of_a_generation():
    """The roofline's per-launch byte model: 64 B per record read and
    written, 128 B per node line, 48 B per triangle and 16 B per sphere
    tested, 4 B per sample read (positions in clear bricks read nothing),
    32 B per framebuffer contribution."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "bench_mod", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    g = {"rays_in": 10, "enqueued": 3, "nodes": 7, "tri_tests": 2, "sph_tests": 5, "samples": 100,
         "samples_skipped": 60, "terminated": 4}
    assert bench.algorithmic_bytes(g) == 64 * 13 + 128 * 7 + 48 * 2 + 16 * 5 + 4 * 40 + 32 * 4
    g.pop("samples_skipped")
    assert bench.algorithmic_bytes(g) == 64 * 13 + 128 * 7 + 48 * 2 + 16 * 5 + 4 * 100 + 32 * 4


def test_dram_roofline_is_taken_per_frame():
    """The DRAM-measured roofline divides a frame's measured bytes by the
    kernel's time per frame, so the same frame split into more or fewer
    launches gives the same figure."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "bench_mod", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    # two frames of 3 launches (4 ms per frame) against two frames of 5 launches (same 4 ms)
    a = bench.dram_roofline(2.0e9, [3.0, 0.5, 0.5] * 2, [3e9, 5e8, 5e8] * 2, 2, 1000.0)
    b = bench.dram_roofline(2.0e9, [2.0, 1.0, 0.5, 0.25, 0.25] * 2, [2e9, 1e9, 5e8, 2.5e8, 2.5e8] * 2, 2, 1000.0)
    assert abs(a["achieved"] - 500.0) < 1e-9 and abs(b["achieved"] - 500.0) < 1e-9
    assert abs(a["frac"] - 0.5) < 1e-12
    assert a["bytes_per_launch"] == 2.0e9 / 3 and b["bytes_per_launch"] == 2.0e9 / 5
    assert abs(a["traffic_over_algorithmic"] - 0.5) < 1e-12 and abs(b["traffic_over_algorithmic"] - 0.5) < 1e-12

"""The C++ host layer (galaxy_gb300/host: Galaxy's Camera, Lighting,
MappedVis/VolumeVis, Visualization, Rendering, RenderingSet and RayList over
the C ABI, and gxywriter) on Galaxy's gold state files, with the radial
volumes written as .vol files as Galaxy's own tests read them.

  * without a GPU: what gxywriter -n makes of each state file -- cameras,
    resolved lights, 256-entry transfer functions -- equals, bit for bit,
    what the Python object model makes of it;
  * on the GPU: gxywriter's images equal the oracle's renders of the same
    scenes, and its RayList pass (camera rays, TraceRays::Trace, the
    secondaries traced again) counts what the oracle counts.
"""
import json
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

import gold_scenes as G
import oracle_lib as O
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def gxywriter():
    from galaxy_gb300 import build
    build.build()
    return build.GXYWRITER


def write_state_dir(tmp, name, n):
    """The state file and its radial-*.vol datasets (header as vti2vol writes
    it: type, origin, counts, spacing printed with %f, raw file name)."""
    doc = json.load(open(os.path.join(G.GOLD_DIR, name + ".state")))
    fields = scenes.radial_fields(n)
    spacing = "%f" % (2.0 / (n - 1))
    for d in doc["Datasets"]:
        fn = d["filename"]
        key = fn[len("radial-"):-4]
        raw = fn[:-4] + ".raw"
        fields[key].astype(np.float32).tofile(os.path.join(tmp, raw))
        with open(os.path.join(tmp, fn), "w") as f:
            f.write("float\n-1 -1 -1\n%d %d %d\n%s %s %s\n%s\n" % (n, n, n, spacing, spacing, spacing, raw))
    path = os.path.join(tmp, name + ".state")
    shutil.copy(os.path.join(G.GOLD_DIR, name + ".state"), path)
    return path


def hexf(v):
    return np.array([float.fromhex(x) for x in v], np.float32)


@pytest.mark.parametrize("name", ["oneBall", "nineBalls", "camera-shadow", "xyz"])
def test_state_parsing_matches_python(tmp_path, name):
    exe = gxywriter()
    path = write_state_dir(str(tmp_path), name, 16)
    out = subprocess.run([exe, "-n", "-s", "96", "80", path], capture_output=True, text=True, check=True).stdout
    got = [json.loads(line) for line in out.splitlines() if line.strip()]
    want, eps = S.load_state(path)
    assert len(got) == len(want)
    for g, (cam, vis) in zip(got, want):
        cam.width, cam.height = 96, 80
        c = cam.c()
        for k in ("eye", "dir", "up"):
            assert np.array_equal(hexf(g["camera"][k]), np.array(getattr(c, k)[:], np.float32)), k
        assert float.fromhex(g["camera"]["aov"]) == np.float32(c.aov)
        assert (g["camera"]["width"], g["camera"]["height"]) == (96, 80)
        L = S.resolve_lights(vis.lighting, cam).c()
        gl = g["lighting"]
        assert gl["n"] == L.n_lights and gl["types"] == list(L.types[:L.n_lights])
        lights = np.array([L.lights[i][k] for i in range(L.n_lights) for k in range(3)], np.float32)
        assert np.array_equal(hexf(gl["lights"]), lights)
        assert (float.fromhex(gl["Ka"]), float.fromhex(gl["Kd"])) == (np.float32(L.Ka), np.float32(L.Kd))
        assert (gl["n_ao"], gl["shadows"]) == (L.n_ao, L.shadows)
        assert float.fromhex(g["epsilon"]) == np.float32(vis.epsilon)
        assert len(g["volumes"]) == len(vis.operators)
        for gv, op in zip(g["volumes"], vis.operators):
            tf = op.tf()
            assert np.array_equal(hexf(gv["colors"]), np.ctypeslib.as_array(tf.colors))
            assert np.array_equal(hexf(gv["opacities"]), np.ctypeslib.as_array(tf.opacities))
            assert np.array_equal(hexf(gv["range"]), np.array(tf.range[:], np.float32))
            assert (gv["slices"], gv["isovalues"], gv["volume_rendering"]) == (
                len(op.slices), len(op.isovalues), int(op.volume_rendering))


@pytest.mark.gpu
@pytest.mark.parametrize("name,parts", [("oneBall", (1, 1, 1)), ("nineBalls", (1, 1, 1)),
                                        ("absolute-shadow", (2, 1, 1)), ("camera", (1, 1, 1))])
def test_gxywriter_images_match_oracle(tmp_path, name, parts):
    exe = gxywriter()
    path = write_state_dir(str(tmp_path), name, 128)
    prefix = os.path.join(str(tmp_path), "img")
    cmd = [exe, "-s", "256", "256", "-p"] + [str(p) for p in parts] + ["-o", prefix, "-R", "0", path]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    lines = [json.loads(line) for line in res.stdout.splitlines() if line.strip()]
    want, eps = S.load_state(path, partitions=parts)
    assert len(lines) == len(want)
    for line, (cam, vis) in zip(lines, want):
        cam.width = cam.height = 256
        img = np.fromfile(line["image"], np.float32).reshape(256, 256, 4)
        L = S.resolve_lights(vis.lighting, cam)
        osc = O.OracleScene(vis)
        ref, cnt = osc.render(cam, L)
        d = np.abs(img[..., :3] - ref[..., :3])
        assert float(np.sqrt(np.mean(d ** 2))) <= 1e-3
        assert float(np.mean(d <= 2.0 / 255)) >= 0.999
        assert (line["primary"], line["shadow"], line["ao"]) == (cnt["primary"], cnt["shadow"], cnt["ao"])
        # RayList level on partition 0
        rays = osc.generate_initial_rays(0, cam)
        traced, sec = osc.trace(0, L, rays)
        again, _ = osc.trace(0, L, sec)
        rl = line["raylist"]
        assert rl["rays"] == rays.n and rl["secondary"] == sec.n
        hits = int(((traced.term & 1) != 0).sum())
        sec_hits = int(((again.term & 1) != 0).sum())
        assert abs(rl["hits"] - hits) <= 1e-4 * max(1, rays.n)
        assert abs(rl["secondary_hits"] - sec_hits) <= 1e-4 * max(1, sec.n)

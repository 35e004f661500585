"""The viewer command protocol (ViewerClientServer::handle,
multiserver/ViewerClientServer.cpp:62-253) over the device path: replies
and errors on the CPU, a rendered frame streamed as pixel messages on the
GPU."""
import json

import numpy as np
import pytest

from galaxy_gb300 import serve
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes


def test_command_replies_and_errors():
    s = serve.CommandSession()
    assert s.handle("permute_pixels off") == (True, "ok") and not s.permute
    assert s.handle("permute_pixels sideways") == (True, "error permute_pixels needs on or off")
    assert s.handle("max_rays_per_packet 4096") == (True, "ok") and s.max_rays_per_packet == 4096
    assert s.handle("window 64 x") == (True, "error window command needs width and height as integers")
    assert s.handle("window 64 48") == (True, "ok") and (s.camera.width, s.camera.height) == (64, 48)
    assert s.handle("json {not json") == (True, "error parsing json command")
    cam = {"viewpoint": [0, 0, 3], "viewdirection": [0, 0, -1], "viewup": [0, 1, 0], "aov": 30}
    assert s.handle("json " + json.dumps({"Camera": cam})) == (True, "ok")
    assert (s.camera.width, s.camera.height) == (64, 48)   # the window size stays
    assert s.handle("json " + json.dumps({"Renderer": {"epsilon": 0.002}})) == (True, "ok") and s.epsilon == 0.002
    bad = {"Datasets": [{"name": "v", "type": "Volume", "filename": "missing.vol"}]}
    assert s.handle("json " + json.dumps(bad)) == (True, "error loading datasets from json command")
    assert s.handle("frobnicate") == (False, None)
    assert s.render() is None   # nothing committed yet


@pytest.mark.gpu
def test_render_streams_the_frame(tmp_path):
    from galaxy_gb300 import gpu
    gpu.init(0)
    vol = scenes.blob_volume(48, 8, 3)
    vol.samples.tofile(str(tmp_path / "blob.raw"))
    (tmp_path / "blob.vol").write_text("float 0 0 0 48 48 48 %r %r %r blob.raw\n" % tuple(vol.deltas))
    got = []
    s = serve.CommandSession(base_dir=str(tmp_path), on_pixels=lambda n, f, snd, px: got.append((n, f, snd, px)),
                             chunk=1000)
    doc = {"Datasets": [{"name": "blob", "type": "Volume", "filename": "blob.vol"}],
           "Visualization": {"Lighting": {"Sources": [[-1, -1, -1, 0]], "shadows": False},
                             "operators": [{"type": "Volume", "dataset": "blob", "volume rendering": True,
                                            "transfer function": [[0, 0.1, 0.2, 0.9], [1, 1, 0.8, 0.2]],
                                            "opacitymap": [[0, 0], [0.3, 0], [1, 0.9]]}]},
           "Camera": {"viewpoint": [0.5, 0.5, 2.5], "viewdirection": [0, 0, -1], "viewup": [0, 1, 0], "aov": 35,
                      "dimensions": [80, 80]}}
    assert s.handle("json " + json.dumps(doc)) == (True, "ok")
    assert s.handle("renderMany 2") == (True, "ok")
    assert s.frame == 2 and got and {f for _, f, _, _ in got} == {0, 1}
    assert all(n <= 1000 and n == len(px) for n, _, _, px in got)
    # frame 0 re-assembled from its pixel messages equals a direct render
    fb = np.zeros((80, 80, 4), np.float32)
    for n, f, _, px in got:
        if f == 0:
            fb[px["y"], px["x"]] = np.stack([px["r"], px["g"], px["b"], px["o"]], -1)
    ref = s.scene.render_host(s.camera, S.resolve_lights(s.visualization.lighting, s.camera))
    assert fb.any() and np.array_equal(fb, ref)

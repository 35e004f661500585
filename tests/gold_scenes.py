"""Galaxy's gold-image scenes (tests/*.state in the Galaxy tree) rebuilt from
the fixtures in tests/golden/golds: the radial volumes are regenerated
analytically instead of being read from .vol files."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from galaxy_gb300 import scene as S  # noqa: E402
from galaxy_gb300 import scenes  # noqa: E402

GOLD_DIR = os.path.join(ROOT, "tests", "golden", "golds")
STATES = ["absolute", "absolute-shadow", "camera", "camera-shadow", "infinite", "infinite-shadow",
          "nineBalls", "oneBall", "xyz"]

_fields = {}


def radial(name, n=256):
    if n not in _fields:
        _fields[n] = scenes.radial_fields(n)
    return scenes.radial_volume(name, n, _fields[n])


def load_gold_state(name, size=512, partitions=(1, 1, 1), n=256):
    """-> list of (camera, visualization, gold_png_path) in gxywriter order."""
    doc = json.load(open(os.path.join(GOLD_DIR, name + ".state")))
    eps = float(doc.get("Renderer", {}).get("epsilon", 0.001))
    datasets = {}
    for d in doc["Datasets"]:
        fn = d["filename"]
        assert fn.startswith("radial-") and fn.endswith(".vol"), fn
        datasets[d["name"]] = radial(fn[len("radial-"):-4], n)
    out = []
    viss = []
    for v in doc["Visualizations"]:
        L = S.Lighting.from_json(v.get("Lighting", v.get("lighting", {})))
        ops = []
        for o in v["operators"]:
            t = o["type"] if o["type"].endswith("Vis") else o["type"] + "Vis"
            assert t == "VolumeVis", t
            ops.append(S.VolumeVis.from_json(o, datasets))
        viss.append(S.Visualization(ops, L, partitions=partitions, epsilon=eps))
    k = 0
    for c in doc["Cameras"]:
        for vis in viss:
            cam = S.Camera.from_json(c)
            cam.width, cam.height = size, size
            out.append((cam, vis, os.path.join(GOLD_DIR, "%s_%05d.png" % (name, k))))
            k += 1
    return out

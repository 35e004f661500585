"""Copy Galaxy's gold-image fixtures into tests/golden/.

Run once, in a checkout that has the Galaxy source tree, with its path as the
only argument.  Copies tests/golds/*.png (512x512 RGBA images rendered by
Galaxy's gxywriter) and the tests/*.state files that produced them, and
writes ao_tables.json with the randomU/randomV tables of
src/renderer/UV.ih parsed as text.  The data-driven state is skipped: its
inputs need VTK.
"""
import json
import os
import re
import shutil
import sys


def main(galaxy_root):
    here = os.path.dirname(os.path.abspath(__file__))
    out = os.path.join(here, "golds")
    os.makedirs(out, exist_ok=True)
    tdir = os.path.join(galaxy_root, "tests")
    for f in sorted(os.listdir(os.path.join(tdir, "golds"))):
        if f.endswith(".png") and not f.startswith("data-driven"):
            shutil.copy(os.path.join(tdir, "golds", f), os.path.join(out, f))
    for f in sorted(os.listdir(tdir)):
        if f.endswith(".state") and not f.startswith("data-driven"):
            shutil.copy(os.path.join(tdir, f), os.path.join(out, f))
    src = open(os.path.join(galaxy_root, "src", "renderer", "UV.ih")).read()
    tabs = {}
    for name in ("randomU", "randomV"):
        body = re.search(name + r"\[256\]\s*=\s*\{([^}]*)\}", src).group(1)
        tabs[name] = [t.strip() for t in body.replace("\n", " ").split(",") if t.strip()]
    json.dump(tabs, open(os.path.join(here, "ao_tables.json"), "w"))


if __name__ == "__main__":
    main(sys.argv[1])

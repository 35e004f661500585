"""On-disk formats: volume headers (.vol / .json, Volume.cpp:195-297), the
partition document (Geometry.cpp:279-350) and the image writers
(ImageWriter.cpp:30-48 PNG, :80-151 FITS)."""
import json
import os

import numpy as np
import pytest

import oracle_lib as O
import pngio
from galaxy_gb300 import gpu, image
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes

DOC = {"parts": [{"extent": [0, 0.3, 0, 1, 0, 1]}, {"extent": [0.3, 0.7, 0, 1, 0, 1]},
                 {"extent": [0.7, 1, 0, 0.5, 0, 1]}, {"extent": [0.7, 1, 0.5, 1, 0, 1]}]}


def test_partition_document_layout():
    ext = S.partition_document(json.dumps(DOC))
    cam, vis = scenes.pathlines_scene(n_lines=50, n_vertices=16, width=8, height=8)
    vis.partition_extents = ext
    osc = O.OracleScene(vis)
    # Galaxy's rule: a face neighbour starts where this brick starts on the
    # other two axes, so brick 1's +x neighbour is 2 and brick 3 has none in -x
    want = [[-1, 1, -1, -1, -1, -1], [0, 2, -1, -1, -1, -1], [1, -1, -1, 3, -1, -1], [-1, -1, 2, -1, -1, -1]]
    for p in range(4):
        a, b = gpu.partition_layout(vis, p), osc.partition_info(p)
        assert list(a.neighbors) == list(b.neighbors) == want[p]
        assert list(a.local_box) == list(b.local_box) == [float(np.float32(x)) for x in
                                                          np.asarray(DOC["parts"][p]["extent"])[[0, 2, 4, 1, 3, 5]]]
        assert list(a.global_box) == list(b.global_box) == [0, 0, 0, 1, 1, 1]
        assert a.n_partitions == 4


def test_partition_document_errors():
    with pytest.raises(ValueError):
        S.partition_document({"nope": []})
    with pytest.raises(ValueError):
        S.partition_document({"parts": [{"extent": [0, 1, 0, 1]}]})


@pytest.mark.parametrize("kind", ["vol-float", "vol-uchar", "json-float", "json-uchar"])
def test_volume_headers(tmp_path, kind):
    rng = np.random.default_rng(3)
    counts = (5, 4, 3)
    fmt, dt = kind.split("-")
    a = (rng.uniform(0, 1, counts[::-1]).astype(np.float32) if dt == "float"
         else rng.integers(0, 256, counts[::-1]).astype(np.uint8))
    a.tofile(str(tmp_path / "raw.bin"))
    if fmt == "vol":
        hdr = tmp_path / "v.vol"
        hdr.write_text("%s 0.5 1 2 %d %d %d 0.1 0.2 0.3 raw.bin\n" % (dt, *counts))
    else:
        hdr = tmp_path / "v.json"
        hdr.write_text(json.dumps({"type": dt, "origin": [0.5, 1, 2], "counts": list(counts),
                                   "delta": [0.1, 0.2, 0.3], "rawdata": "raw.bin"}))
    v = S.Volume.load_vol(str(hdr))
    assert v.counts == counts and v.origin == (0.5, 1.0, 2.0)
    assert np.allclose(v.deltas, (0.1, 0.2, 0.3))
    assert v.samples.dtype == np.float32 and np.array_equal(v.samples, a.astype(np.float32))


def test_color_writer_quantises_like_the_oracle(tmp_path):
    rng = np.random.default_rng(4)
    fb = rng.uniform(-0.5, 1.7, (7, 9, 4)).astype(np.float32)
    path = image.ColorImageWriter(str(tmp_path / "img")).write(fb)
    got = pngio.read_png(path)
    assert got.shape == (7, 9, 4) and np.all(got[..., 3] == 255)
    q = image.quantize(fb)
    assert np.array_equal(got, q)
    assert np.array_equal(q, O.quantize(fb))
    # row order: the framebuffer's row 0 (bottom) is the file's last row
    v = np.float32(255) * fb[0, :, :3]
    assert np.array_equal(got[-1, :, :3], (np.trunc(v).astype(np.int64) & 255).astype(np.uint8))


@pytest.mark.parametrize("w,h", [(9, 7), (36, 20)])   # 36*20*4 = 2880: a whole block of padding
def test_fits_writer(tmp_path, w, h):
    rng = np.random.default_rng(5)
    fb = rng.normal(size=(h, w, 4)).astype(np.float32)
    paths = image.FloatImageWriter(str(tmp_path / "img")).write(fb)
    assert [os.path.basename(p) for p in paths] == ["img_r.fits", "img_g.fits", "img_b.fits", "img_a.fits"]
    for k, p in enumerate(paths):
        data = open(p, "rb").read()
        assert len(data) == 2880 + 4 * w * h + (2880 - (4 * w * h) % 2880)
        hdr = data[:2880].decode("ascii")
        assert hdr.startswith("SIMPLE  = T") and "BITPIX  = -32" in hdr and "NAXIS1  = %d" % w in hdr
        assert np.array_equal(image.read_fits_channel(p), fb[..., k])

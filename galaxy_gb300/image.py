"""Image writers for rendered framebuffers (fp32 RGBA, pixel (x, y) at
row y, y = 0 the bottom row).

ColorImageWriter follows Galaxy's ColorImageWriter::Write
(src/renderer/ImageWriter.cpp:30-48): each channel becomes
(unsigned char)(255 * v) with no clamp, alpha is forced to 0xff, rows are
flipped so the top row is written first, and the result goes to
<name>.png.  The cast of an out-of-range value is undefined behaviour in
C++; it is defined here, as in the oracle, as truncation toward zero to a
32-bit integer followed by its low 8 bits.

FloatImageWriter follows FloatImageWriter::Write (ImageWriter.cpp:80-151):
one FITS file per channel, <name>_r.fits ... <name>_a.fits, each a
2880-byte header of 80-character cards (SIMPLE, BITPIX -32, NAXIS 2, NAXIS1
w, NAXIS2 h, EXTEND, END), the channel as big-endian float32 in the
framebuffer's row order, and 2880 - (4wh mod 2880) bytes of space padding
(a whole block when 4wh is a multiple of 2880, as Galaxy writes it).
"""
import os
import struct
import zlib

import numpy as np


def quantize(rgba):
    """fp32 (h, w, 4) -> uint8 (h, w, 4) as ColorImageWriter (flipped rows)."""
    rgba = np.asarray(rgba, np.float32)
    v = np.float32(255.0) * rgba[..., :3]
    with np.errstate(invalid="ignore", over="ignore"):
        q = np.where(np.isfinite(v) & (np.abs(v) < 2.0 ** 31), np.trunc(v), 0).astype(np.int64) & 0xFF
    out = np.empty(rgba.shape[:2] + (4,), np.uint8)
    out[..., :3] = q.astype(np.uint8)
    out[..., 3] = 0xFF
    return out[::-1].copy()


def png_bytes(rgba8):
    """8-bit RGBA (h, w, 4), top row first -> PNG file bytes."""
    h, w, _ = rgba8.shape
    raw = b"".join(b"\x00" + rgba8[y].tobytes() for y in range(h))

    def chunk(tag, body):
        return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


class ColorImageWriter:
    def __init__(self, basename="image"):
        self.basename = basename

    def write(self, rgba, name=None):
        path = "%s.png" % (name if name else self.basename)
        with open(path, "wb") as f:
            f.write(png_bytes(quantize(rgba)))
        return path


def _card(key, value):
    s = "%s%s" % (key, value)
    if len(s) > 80:
        raise ValueError("FITS card longer than 80 characters")
    return s + " " * (80 - len(s))


def fits_header(w, h):
    hdr = "".join([_card("SIMPLE  = ", "T"), _card("BITPIX  = ", -32), _card("NAXIS   = ", 2),
                   _card("NAXIS1  = ", w), _card("NAXIS2  = ", h), _card("EXTEND  = ", "T"), _card("END", "")])
    return (hdr + " " * (2880 - len(hdr))).encode("ascii")


class FloatImageWriter:
    def __init__(self, basename="image"):
        self.basename = basename
        self.frame = 0

    def write(self, rgba, name=None):
        rgba = np.asarray(rgba, np.float32)
        h, w, _ = rgba.shape
        fn = name if name else self.basename
        hdr = fits_header(w, h)
        pad = b" " * (2880 - (w * h * 4) % 2880)
        paths = []
        for k, c in enumerate("rgba"):
            path = "%s_%c.fits" % (fn, c)
            with open(path, "wb") as f:
                f.write(hdr)
                f.write(np.ascontiguousarray(rgba[..., k]).astype(">f4").tobytes())
                f.write(pad)
            paths.append(path)
        self.frame += 1
        return paths


def read_fits_channel(path):
    """(h, w) float32 of a file written by FloatImageWriter."""
    data = open(path, "rb").read()
    cards = [data[i:i + 80].decode("ascii") for i in range(0, 2880, 80)]
    kv = {}
    for c in cards:
        if "=" in c[:10]:
            kv[c[:8].strip()] = c[10:].strip()
    w, h = int(kv["NAXIS1"]), int(kv["NAXIS2"])
    return np.frombuffer(data, ">f4", w * h, 2880).astype(np.float32).reshape(h, w)

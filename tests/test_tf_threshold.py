"""The zero-opacity threshold behind the empty-space skipping
(gxy_tf_clear_below, host code of the device library) against the oracle's
transfer-function lookup: every value below the threshold has opacity
exactly 0, and the threshold lies within 2e-4 of the range below the last
value that does (values between interpolate two zero entries).  Random
transfer functions over random ranges, plus the edge cases: no zero
entry, one, all."""
import ctypes as C

import numpy as np

import oracle_lib as O
from galaxy_gb300 import _abi as A
from galaxy_gb300 import gpu


def make_tf(opac, r0, r1):
    tf = A.gxy_tf()
    col = np.linspace(0, 1, 768, dtype=np.float32)
    C.memmove(tf.colors, col.ctypes.data, col.nbytes)
    op = np.ascontiguousarray(opac, np.float32)
    C.memmove(tf.opacities, op.ctypes.data, op.nbytes)
    tf.range[0], tf.range[1] = float(r0), float(r1)
    return tf


def opacity(tf, v):
    return O.lib().oracle_tf_opacity(C.byref(tf), C.c_float(float(v)))


def below(t, n, span, g):
    """Values below t: the float just below, and a spread down to t - span."""
    out = [np.nextafter(np.float32(t), np.float32(-np.inf))]
    out += list((np.float32(t) - np.float32(span) * g.random(n, dtype=np.float32)).astype(np.float32))
    return [v for v in out if v < t]


def test_values_below_threshold_have_zero_opacity():
    g = np.random.default_rng(5)
    checked = 0
    for trial in range(300):
        z = int(g.integers(1, 256))                        # opac[0 .. z-1] zero
        opac = np.zeros(256, np.float32)
        opac[z:] = g.uniform(1e-4, 1.0, size=256 - z).astype(np.float32)
        r0 = float(g.uniform(-5, 5))
        r1 = r0 + float(g.choice([1e-3, 0.5, 1.0, 7.0, 300.0]))
        tf = make_tf(opac, r0, r1)
        t = gpu.tf_clear_below(tf)
        assert np.isfinite(t)
        for v in below(t, 40, (r1 - r0) * 0.3 + 1e-3, g):
            assert opacity(tf, v) == 0.0, (trial, z, r0, r1, t, v)
            checked += 1
        # tight: within 2e-4 of the range below the last zero-opacity value
        last_zero = r0 + (z - 1) * (r1 - r0) / 255.0
        assert t >= last_zero - 2e-4 * (r1 - r0) - 1e-6 * abs(r0), (z, r0, r1, t)
        # and the first entry past the zero run is reached with positive opacity
        assert opacity(tf, np.float32(r0 + (z + 0.5) * (r1 - r0) / 255.0)) > 0.0
    assert checked > 5000


def test_threshold_edge_cases():
    inf = float("inf")
    # lowest entry positive: nothing is transparent
    assert gpu.tf_clear_below(make_tf(np.full(256, 0.1), 0.0, 1.0)) == -inf
    # all zero: everything is
    assert gpu.tf_clear_below(make_tf(np.zeros(256), 0.0, 1.0)) == inf
    # only the lowest entry zero: values at or below r0 read it
    opac = np.full(256, 0.5)
    opac[0] = 0.0
    tf = make_tf(opac, 0.25, 0.75)
    t = gpu.tf_clear_below(tf)
    assert t == np.float32(0.25)
    assert opacity(tf, np.nextafter(np.float32(0.25), np.float32(-1))) == 0.0
    assert opacity(tf, np.float32(0.2505)) > 0.0

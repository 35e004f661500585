"""Path lines in the oracle (CPU): the capsule restatement of
DataDrivenPathLines_intersect_kernel (DataDrivenPathLines.ispc:100-203)
checked against its geometric meaning, and the brick layout of a path-line
scene against the C ABI's host-side layout."""
import numpy as np

import oracle_lib as O
from galaxy_gb300 import _abi as A
from galaxy_gb300 import gpu
from galaxy_gb300 import scene as S
from galaxy_gb300 import scenes


def seg_distance(p, a, b):
    """Distance from points p (n, 3) to segment a-b (float64)."""
    ab = b - a
    s = np.clip(((p - a) @ ab) / (ab @ ab), 0.0, 1.0)
    return np.linalg.norm(p - (a + s[:, None] * ab), axis=1)


def line_segment_min_distance(o, d, a, b, n=4001):
    """Smallest distance between rays (o, d) and segment a-b, by dense
    sampling of the segment (float64)."""
    s = np.linspace(0.0, 1.0, n)
    q = a[None, :] + s[:, None] * (b - a)[None, :]
    best = np.full(len(o), np.inf)
    for k in range(0, n, 500):
        qq = q[k:k + 500]
        w = qq[None, :, :] - o[:, None, :]
        t = np.maximum((w * d[:, None, :]).sum(-1) / (d * d).sum(-1)[:, None], 0.0)
        dist = np.linalg.norm(w - t[..., None] * d[:, None, :], axis=-1)
        best = np.minimum(best, dist.min(1))
    return best


def one_segment_scene(r=0.05):
    a, b = np.array([0.3, 0.45, 0.5]), np.array([0.7, 0.55, 0.45])
    lines = S.PathLines(np.stack([a, b]), [0])
    vis = S.Visualization([S.PathLinesVis(lines, radius0=r, radius1=r, value0=0.0, value1=0.0)],
                          box=(0.0, 0.0, 0.0, 1.0, 1.0, 1.0))
    cam = S.Camera(eye=(0.5, 0.5, 2.0), direction=(0, 0, -1), up=(0, 1, 0), aov=20.0, width=64, height=64)
    return cam, vis, a, b, r


def test_capsule_hits_lie_on_the_capsule_and_misses_pass_outside():
    cam, vis, a, b, r = one_segment_scene()
    osc = O.OracleScene(vis)
    L = S.resolve_lights(vis.lighting, cam)
    rays = osc.generate_initial_rays(0, cam)
    traced, _ = osc.trace(0, L, rays)
    o = np.stack([rays.ox, rays.oy, rays.oz], 1).astype(np.float64)
    d = np.stack([rays.dx, rays.dy, rays.dz], 1).astype(np.float64)
    hit = (traced.term & A.RAY_SURFACE) != 0
    assert 50 < hit.sum() < rays.n
    p = o[hit] + traced.t[hit, None].astype(np.float64) * d[hit]
    assert np.max(np.abs(seg_distance(p, a, b) - r)) < 1e-4 * (1 + r)
    miss = line_segment_min_distance(o[~hit], d[~hit], a, b)
    assert miss.min() > r - 1e-4


def test_pathline_partitions_equal_oracle():
    cam, vis = scenes.pathlines_scene(n_lines=50, n_vertices=16, width=8, height=8, partitions=(2, 1, 2))
    vis.box = None   # layout from the path lines' own bounds (vertices grown by their radius)
    osc = O.OracleScene(vis)
    for p in range(4):
        ga, ob = gpu.partition_layout(vis, p), osc.partition_info(p)
        assert list(ga.global_box) == list(ob.global_box)
        assert list(ga.local_box) == list(ob.local_box) and list(ga.neighbors) == list(ob.neighbors)


def test_polylines_to_segments():
    lines = S.PathLines.from_polylines([np.zeros((4, 3)), np.ones((3, 3))], [np.arange(4), np.arange(3)])
    assert list(lines.indices) == [0, 1, 2, 4, 5]
    assert lines.vertices.shape == (7, 3) and lines.data.shape == (7,)

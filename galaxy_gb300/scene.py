"""Galaxy's scene objects on the host side of the C ABI.

Class names and JSON semantics follow Galaxy's renderer/data layer:
Lighting (src/renderer/Lighting.cpp:58-115), Camera (Camera.cpp:165-281),
MappedVis transfer-function resampling (MappedVis.cpp:86-203, 277-338),
VolumeVis (VolumeVis.cpp:119-163), ParticlesVis (ParticlesVis.cpp:104-118),
PathLinesVis (PathLinesVis.cpp:29-112), TrianglesVis, Volume (.vol import,
Volume.cpp:195-214), PathLines (polylines) and Visualization
(Visualization.cpp:293-340).  A Visualization turns into the gxy_scene_desc
the device path consumes; numpy arrays referenced by the descriptor are kept
alive by the Python objects.
"""
import ctypes as C
import math
import os

import numpy as np

from . import _abi as A


# --------------------------------------------------------------- Lighting
class Lighting:
    """Lighting_ispc defaults (Lighting.ispc:29-44) and JSON loading
    (Lighting.cpp:58-115)."""

    def __init__(self):
        self.lights = [(1.0, 1.0, 1.0)]
        self.types = [2]
        self.Ka, self.Kd = 0.5, 0.5
        self.n_ao, self.ao_radius = 0, 1.0
        self.shadows = False

    @classmethod
    def from_json(cls, v):
        L = cls()
        if "Sources" in v:
            lights, types = [], []
            for s in v["Sources"]:
                x, y, z = float(s[0]), float(s[1]), float(s[2])
                t = 0 if len(s) == 3 else int(s[3])
                if t == 0:
                    # single-precision arithmetic as Lighting.cpp:76-90
                    x, y, z = np.float32(x), np.float32(y), np.float32(z)
                    d = np.float32(np.sqrt(np.float32(x * x + y * y) + z * z))
                    if d == 0:
                        x = y = z = np.float32(0.577350)
                    else:
                        x, y, z = x / d, y / d, z / d
                lights.append((float(x), float(y), float(z)))
                types.append(t)
            L.lights, L.types = lights, types
        if "shadows" in v:
            L.shadows = bool(v["shadows"])
        L.n_ao = int(v.get("ao count", 0))
        L.ao_radius = float(v.get("ao radius", 1))
        L.Ka = float(v.get("Ka", 0.5))
        L.Kd = float(v.get("Kd", 0.5))
        return L

    def to_json(self):
        return {"Sources": [list(l) + [t] for l, t in zip(self.lights, self.types)],
                "Ka": self.Ka, "Kd": self.Kd, "ao count": self.n_ao,
                "ao radius": self.ao_radius, "shadows": self.shadows}

    def c(self):
        L = A.gxy_lighting()
        if len(self.lights) > A.MAX_LIGHTS:
            raise ValueError("at most %d lights" % A.MAX_LIGHTS)
        L.n_lights = len(self.lights)
        for i, (l, t) in enumerate(zip(self.lights, self.types)):
            L.lights[i][0], L.lights[i][1], L.lights[i][2] = l
            L.types[i] = t
        L.Ka, L.Kd = self.Ka, self.Kd
        L.n_ao, L.ao_radius = self.n_ao, self.ao_radius
        L.shadows = 1 if self.shadows else 0
        return L


# ----------------------------------------------------------------- Camera
class Camera:
    """Camera::LoadFromJSON (Camera.cpp:237-278).  Note the reference sets
    the height from dimensions[0] (Camera.cpp:267-271); kept."""

    def __init__(self, eye=(0, 0, 1), direction=(0, 0, -1), up=(0, 1, 0), aov=45.0,
                 width=512, height=512):
        self.eye, self.dir, self.up = tuple(eye), tuple(direction), tuple(up)
        self.aov, self.width, self.height = float(aov), int(width), int(height)

    @classmethod
    def from_json(cls, v):
        eye = [float(x) for x in v["viewpoint"]]
        if "viewdirection" in v:
            d = [float(x) for x in v["viewdirection"]]
        elif "viewcenter" in v:
            d = [float(v["viewcenter"][k]) - eye[k] for k in range(3)]
        else:
            raise ValueError("need either viewdirection or viewcenter")
        cam = cls(eye, d, [float(x) for x in v["viewup"]], float(v["aov"]))
        if "dimensions" in v:
            cam.width = int(v["dimensions"][0])
            cam.height = int(v["dimensions"][0])
        return cam

    def c(self):
        c = A.gxy_camera()
        c.eye[:] = [float(np.float32(x)) for x in self.eye]
        c.dir[:] = [float(np.float32(x)) for x in self.dir]
        c.up[:] = [float(np.float32(x)) for x in self.up]
        c.aov, c.width, c.height = self.aov, self.width, self.height
        return c


def resolve_lights(lighting, camera):
    """Rendering::resolve_lights (Rendering.cpp:157-216): type-1 lights are
    camera-relative offsets (right, up, viewdir) that become point lights."""
    f = np.float32

    def nrm(v):
        l = f(np.sqrt(f(f(v[0] * v[0]) + f(v[1] * v[1])) + f(v[2] * v[2])))
        if l == 0:
            return v
        d = f(1.0 / float(l))
        return np.array([v[0] * d, v[1] * d, v[2] * d], f)

    def cross(a, b):
        return np.array([f(a[1] * b[2]) - f(a[2] * b[1]), f(a[2] * b[0]) - f(a[0] * b[2]),
                         f(a[0] * b[1]) - f(a[1] * b[0])], f)

    vp = np.array(camera.eye, f)
    vu = nrm(np.array(camera.up, f))
    vd = nrm(np.array(camera.dir, f))
    right = nrm(cross(vd, vu))
    up = cross(vd, right)
    out = Lighting()
    out.Ka, out.Kd, out.n_ao, out.ao_radius, out.shadows = (
        lighting.Ka, lighting.Kd, lighting.n_ao, lighting.ao_radius, lighting.shadows)
    out.lights, out.types = [], []
    for l, t in zip(lighting.lights, lighting.types):
        if t == 1:
            l = np.array(l, f)
            p = vp + right * l[0] + up * l[1] + vd * l[2]
            out.lights.append(tuple(float(x) for x in p.astype(f)))
            out.types.append(2)
        else:
            out.lights.append(tuple(l))
            out.types.append(t)
    return out


# ------------------------------------------------------- transfer function
def resample_tf(colormap, opacitymap, data_range=None):
    """MappedVis::local_commit (MappedVis.cpp:286-333) -> gxy_tf.  colormap is
    a list of (x, r, g, b); opacitymap of (x, a)."""
    cm = np.asarray(colormap, np.float32).reshape(-1, 4)
    om = np.asarray(opacitymap, np.float32).reshape(-1, 2)
    tf = A.gxy_tf()
    colors = np.zeros((256, 3), np.float32)
    i0, i1 = 0, 1
    xmin, xmax = float(cm[0, 0]), float(cm[-1, 0])
    for i in range(256):
        x = np.float32(xmin + (i / 255.0) * (xmax - xmin))
        if x > cm[-1, 0]:
            x = cm[-1, 0]
        while i1 < len(cm) - 1 and cm[i1, 0] < x:
            i0, i1 = i0 + 1, i1 + 1
        d = np.float32(x - cm[i0, 0]) / np.float32(cm[i1, 0] - cm[i0, 0])
        for k in range(3):
            colors[i, k] = cm[i0, k + 1] + d * np.float32(cm[i1, k + 1] - cm[i0, k + 1])
    opac = np.zeros(256, np.float32)
    i0, i1 = 0, 1
    xmin, xmax = float(om[0, 0]), float(om[-1, 0])
    for i in range(256):
        x = np.float32(xmin + (i / 255.0) * (xmax - xmin))
        if x > om[-1, 0]:
            x = om[-1, 0]
        while i1 < len(om) - 1 and om[i1, 0] < x:
            i0, i1 = i0 + 1, i1 + 1
        d = np.float32(x - om[i0, 0]) / np.float32(om[i1, 0] - om[i0, 0])
        opac[i] = om[i0, 1] + d * np.float32(om[i1, 1] - om[i0, 1])
    C.memmove(tf.colors, colors.ctypes.data, colors.nbytes)
    C.memmove(tf.opacities, opac.ctypes.data, opac.nbytes)
    if data_range is not None:
        tf.range[0], tf.range[1] = float(data_range[0]), float(data_range[1])
    else:
        tf.range[0], tf.range[1] = float(cm[0, 0]), float(cm[-1, 0])
    return tf


DEFAULT_COLORMAP = [(0.0, 0.4, 0.4, 0.4), (1.0, 1.0, 1.0, 1.0)]   # MappedVis.cpp:58-59
DEFAULT_OPACITYMAP = [(0.0, 1.0), (1.0, 1.0)]                     # MappedVis.cpp:61-62


class MappedVis:
    def __init__(self, dataset=None, colormap=None, opacitymap=None, data_range=None):
        self.dataset = dataset
        self.colormap = list(colormap) if colormap is not None else list(DEFAULT_COLORMAP)
        self.opacitymap = list(opacitymap) if opacitymap is not None else list(DEFAULT_OPACITYMAP)
        self.data_range = data_range

    def load_mapped_json(self, v):
        # MappedVis::LoadFromJSON (MappedVis.cpp:86-203), inline maps only
        if "data range" in v:
            self.data_range = (float(v["data range"][0]), float(v["data range"][1]))
        m = v.get("transfer function", v.get("colormap"))
        if m is not None and not isinstance(m, str):
            self.colormap = [tuple(float(x) for x in e) for e in m]
            if "opacitymap" in v:
                self.opacitymap = [tuple(float(x) for x in e) for e in v["opacitymap"]]

    def tf(self):
        return resample_tf(self.colormap, self.opacitymap, self.data_range)


class VolumeVis(MappedVis):
    def __init__(self, dataset=None, isovalues=(), slices=(), volume_rendering=False, **kw):
        super().__init__(dataset, **kw)
        self.isovalues = list(isovalues)
        self.slices = [tuple(s) for s in slices]
        self.volume_rendering = bool(volume_rendering)

    @classmethod
    def from_json(cls, v, datasets):
        vis = cls(datasets[v["dataset"]])
        vis.load_mapped_json(v)
        vis.isovalues = [float(x) for x in v.get("isovalues", [])]
        if "slices" in v:
            vis.slices = [tuple(float(x) for x in s) for s in v["slices"]]
        elif "plane" in v:
            vis.slices = [tuple(float(x) for x in v["plane"])]
        vis.volume_rendering = bool(v.get("volume rendering", False))
        return vis


class TrianglesVis(MappedVis):
    @classmethod
    def from_json(cls, v, datasets):
        vis = cls(datasets[v["dataset"]])
        vis.load_mapped_json(v)
        return vis


class ParticlesVis(MappedVis):
    def __init__(self, dataset=None, radius0=0.02, radius1=0.02, value0=0.0, value1=0.0, **kw):
        super().__init__(dataset, **kw)
        self.radius0, self.radius1, self.value0, self.value1 = radius0, radius1, value0, value1

    @classmethod
    def from_json(cls, v, datasets):
        vis = cls(datasets[v["dataset"]])
        # ParticlesVis::LoadFromJSON (ParticlesVis.cpp:104-118)
        for k, a in (("radius0", "radius0"), ("radius1", "radius1"), ("value0", "value0"),
                     ("value1", "value1")):
            if k in v:
                setattr(vis, a, float(v[k]))
        if "radius" in v:
            vis.radius0 = float(v["radius"])
            vis.value0 = vis.value1 = vis.radius1 = 0.0
        vis.load_mapped_json(v)
        return vis


class PathLinesVis(MappedVis):
    """PathLinesVis (PathLinesVis.cpp:29-36 defaults, :104-112 LoadFromJSON):
    radius mapped from data between (value0, radius0) and (value1, radius1)."""

    def __init__(self, dataset=None, radius0=-1.0, radius1=1.0, value0=0.0, value1=1.0, **kw):
        super().__init__(dataset, **kw)
        self.radius0, self.radius1, self.value0, self.value1 = radius0, radius1, value0, value1

    @classmethod
    def from_json(cls, v, datasets):
        vis = cls(datasets[v["dataset"]])
        for k in ("radius0", "radius1", "value0", "value1"):
            if k in v:
                setattr(vis, k, float(v[k]))
        vis.load_mapped_json(v)
        return vis


# ---------------------------------------------------------------- datasets
class Volume:
    """Structured fp32 grid, x fastest (Volume.cpp:195-214 for .vol)."""

    def __init__(self, samples, origin=(0, 0, 0), deltas=(1, 1, 1)):
        self.samples = np.ascontiguousarray(samples, np.float32)
        assert self.samples.ndim == 3, "samples are (nz, ny, nx)"
        nz, ny, nx = self.samples.shape
        self.counts = (nx, ny, nz)
        self.origin = tuple(float(x) for x in origin)
        self.deltas = tuple(float(x) for x in deltas)

    @classmethod
    def load_vol(cls, path):
        """Volume header as Volume::local_import reads it (Volume.cpp:195-297):
        a .vol text header -- type, origin, counts, deltas, raw file name --
        or a .json header with "type", "origin", "counts", "delta",
        "rawdata" and optional "number of components".  Raw data are float32
        or uchar (read as their float values); the raw file name is
        relative to the header's directory.  Multi-component volumes are
        not rendered."""
        if path.endswith(".json"):
            import json
            doc = json.load(open(path))
            for k in ("type", "origin", "counts", "delta", "rawdata"):
                if k not in doc:
                    raise ValueError("volume JSON has no %s field: %s" % (k, path))
            kind = doc["type"]
            origin = [float(x) for x in doc["origin"]]
            counts = [int(x) for x in doc["counts"]]
            deltas = [float(x) for x in doc["delta"]]
            raw = doc["rawdata"]
            if int(doc.get("number of components", 1)) != 1:
                raise ValueError("multi-component volumes are not rendered")
        else:
            toks = open(path).read().split()
            kind = toks[0]
            origin = [float(x) for x in toks[1:4]]
            counts = [int(x) for x in toks[4:7]]
            deltas = [float(x) for x in toks[7:10]]
            raw = toks[10]
        if not raw.startswith("/"):
            raw = os.path.join(os.path.dirname(path), raw)
        n = counts[0] * counts[1] * counts[2]
        a = np.fromfile(raw, np.float32 if kind == "float" else np.uint8, count=n)
        if a.size != n:
            raise ValueError("raw data file %s holds %d of %d samples" % (raw, a.size, n))
        return cls(a.astype(np.float32).reshape(counts[2], counts[1], counts[0]), origin, deltas)


class Triangles:
    def __init__(self, vertices, indices, normals=None, data=None):
        self.vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(indices, np.int32).reshape(-1, 3)
        self.normals = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        self.data = None if data is None else np.ascontiguousarray(data, np.float32).reshape(-1)


class Particles:
    def __init__(self, centers, data=None):
        self.centers = np.ascontiguousarray(centers, np.float32).reshape(-1, 3)
        self.data = None if data is None else np.ascontiguousarray(data, np.float32).reshape(-1)


class PathLines:
    """Polylines: vertices (n, 3), per-vertex data and segment first-vertex
    indices (segment i joins indices[i] and indices[i] + 1), as
    PathLines::load_from_vtkPointSet builds them from polyline cells
    (PathLines.cpp:74-126)."""

    def __init__(self, vertices, indices, data=None):
        self.vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(indices, np.int32).reshape(-1)
        self.data = None if data is None else np.ascontiguousarray(data, np.float32).reshape(-1)

    @classmethod
    def from_polylines(cls, lines, data=None):
        """lines: list of (k_i, 3) vertex arrays; data: matching list of (k_i,)
        arrays or None.  Each polyline contributes its k_i - 1 segments."""
        verts, idx, dat, base = [], [], [], 0
        for j, ln in enumerate(lines):
            ln = np.asarray(ln, np.float32).reshape(-1, 3)
            verts.append(ln)
            idx.append(np.arange(base, base + len(ln) - 1, dtype=np.int32))
            if data is not None:
                dat.append(np.asarray(data[j], np.float32).reshape(-1))
            base += len(ln)
        return cls(np.concatenate(verts), np.concatenate(idx), np.concatenate(dat) if data is not None else None)


# ----------------------------------------------------------- Visualization
class Visualization:
    """A Visualization (Visualization.cpp:293-340): operators plus lighting,
    with the device-path knobs: brick partitions, sampling rate, opacity
    threshold and Renderer.epsilon."""

    def __init__(self, operators=(), lighting=None, partitions=(1, 1, 1), box=None,
                 sampling_rate=1.0, opaque_alpha=0.999, epsilon=0.001, partition_extents=None):
        self.operators = list(operators)
        self.lighting = lighting if lighting is not None else Lighting()
        self.partitions = tuple(int(p) for p in partitions)
        # explicit bricks from a partition document (see partition_document);
        # when given they replace the brick grid
        self.partition_extents = (None if partition_extents is None
                                  else np.ascontiguousarray(partition_extents, np.float32).reshape(-1, 6))
        self.box = box
        self.sampling_rate = float(sampling_rate)
        self.opaque_alpha = float(opaque_alpha)
        self.epsilon = float(epsilon)

    def desc(self):
        """Build the gxy_scene_desc; the returned object keeps every array
        it points at alive (attribute _keep)."""
        vols, tris, parts, lines = [], [], [], []
        keep = []
        for op in self.operators:
            if isinstance(op, VolumeVis):
                v = A.gxy_volume_vis()
                ds = op.dataset
                v.samples = A.fptr(ds.samples)
                keep.append(ds.samples)
                v.counts[:] = list(ds.counts)
                v.origin[:] = list(ds.origin)
                v.deltas[:] = list(ds.deltas)
                v.tf = op.tf()
                if len(op.slices) > A.MAX_SLICES or len(op.isovalues) > A.MAX_ISOVALUES:
                    raise ValueError("too many slices or isovalues")
                v.n_slices = len(op.slices)
                for i, s in enumerate(op.slices):
                    for k in range(4):
                        v.slices[i][k] = s[k]
                v.n_isovalues = len(op.isovalues)
                for i, s in enumerate(op.isovalues):
                    v.isovalues[i] = s
                v.volume_render = 1 if op.volume_rendering else 0
                vols.append(v)
            elif isinstance(op, TrianglesVis):
                ds = op.dataset
                t = A.gxy_triangles_vis()
                t.vertices, t.n_vertices = A.fptr(ds.vertices), len(ds.vertices)
                t.indices, t.n_triangles = A.iptr(ds.indices), len(ds.indices)
                t.normals = A.fptr(ds.normals)
                t.data = A.fptr(ds.data)
                t.tf = op.tf()
                keep += [ds.vertices, ds.indices, ds.normals, ds.data]
                tris.append(t)
            elif isinstance(op, ParticlesVis):
                ds = op.dataset
                p = A.gxy_particles_vis()
                p.centers, p.data, p.n = A.fptr(ds.centers), A.fptr(ds.data), len(ds.centers)
                p.radius0, p.radius1, p.value0, p.value1 = op.radius0, op.radius1, op.value0, op.value1
                p.tf = op.tf()
                keep += [ds.centers, ds.data]
                parts.append(p)
            elif isinstance(op, PathLinesVis):
                ds = op.dataset
                q = A.gxy_pathlines_vis()
                q.vertices, q.n_vertices = A.fptr(ds.vertices), len(ds.vertices)
                q.indices, q.n_segments = A.iptr(ds.indices), len(ds.indices)
                q.data = A.fptr(ds.data)
                q.radius0, q.radius1, q.value0, q.value1 = op.radius0, op.radius1, op.value0, op.value1
                q.tf = op.tf()
                keep += [ds.vertices, ds.indices, ds.data]
                lines.append(q)
            else:
                raise TypeError("unknown operator %r" % (op,))
        if len(vols) > A.MAX_VOLUMES:
            raise ValueError("at most %d volumes" % A.MAX_VOLUMES)
        d = A.gxy_scene_desc()
        va = (A.gxy_volume_vis * max(1, len(vols)))(*vols)
        ta = (A.gxy_triangles_vis * max(1, len(tris)))(*tris)
        pa = (A.gxy_particles_vis * max(1, len(parts)))(*parts)
        d.n_volumes, d.volumes = len(vols), C.cast(va, C.POINTER(A.gxy_volume_vis))
        d.n_triangle_sets, d.triangles = len(tris), C.cast(ta, C.POINTER(A.gxy_triangles_vis))
        d.n_particle_sets, d.particles = len(parts), C.cast(pa, C.POINTER(A.gxy_particles_vis))
        la = (A.gxy_pathlines_vis * max(1, len(lines)))(*lines)
        d.n_pathline_sets, d.pathlines = len(lines), C.cast(la, C.POINTER(A.gxy_pathlines_vis))
        d.partitions[:] = list(self.partitions)
        if self.partition_extents is not None:
            d.n_partition_extents = len(self.partition_extents)
            d.partition_extents = A.fptr(self.partition_extents)
            keep.append(self.partition_extents)
        if self.box is not None:
            d.has_box = 1
            d.box[:] = [float(x) for x in self.box]
        d.sampling_rate = self.sampling_rate
        d.opaque_alpha = self.opaque_alpha
        d.epsilon = self.epsilon
        d._keep = (keep, va, ta, pa, la)
        return d


def partition_document(doc):
    """Brick extents of a Galaxy partition document (a dict, JSON text or a
    path): {"parts": [{"extent": [xmin, xmax, ymin, ymax, zmin, zmax], ...},
    ...]}, one part per brick, as Geometry::get_partitioning reads it
    (Geometry.cpp:279-312).  Returns a float32 (n, 6) array for
    Visualization(partition_extents=...)."""
    import json
    if isinstance(doc, str):
        doc = json.load(open(doc)) if os.path.exists(doc) else json.loads(doc)
    if "parts" not in doc:
        raise ValueError("partition document does not have parts")
    parts = doc["parts"]
    if not isinstance(parts, list) or not parts:
        raise ValueError("invalid partition document")
    ext = np.array([[float(x) for x in p["extent"]] for p in parts], np.float32)
    if ext.shape[1] != 6:
        raise ValueError("a partition extent has 6 numbers")
    return ext


def datasets_from_json(doc, base="."):
    """The "Datasets" block of a state document (Datasets.cpp:99-125):
    name -> dataset.  Volumes load from .vol/.json headers relative to
    base; other types need VTK readers and are refused."""
    datasets = {}
    for d in doc.get("Datasets", []):
        t = d["type"]
        if t == "Volume":
            fn = d["filename"]
            if not fn.startswith("/"):
                fn = os.path.join(base, fn)
            datasets[d["name"]] = Volume.load_vol(fn)
        else:
            raise ValueError("dataset type %s needs VTK, which is not supported" % t)
    return datasets


def visualization_from_json(v, datasets, partitions=(1, 1, 1), epsilon=0.001):
    """One Visualization object (Visualization.cpp:293-340): lighting and
    operators; an operator type gets "Vis" appended when it lacks it
    (Visualization.cpp:318-322)."""
    lighting = Lighting()
    if "Lighting" in v:
        lighting = Lighting.from_json(v["Lighting"])
    elif "lighting" in v:
        lighting = Lighting.from_json(v["lighting"])
    ops = []
    for o in v["operators"]:
        t = o["type"]
        if not t.endswith("Vis"):
            t = t + "Vis"
        cls = {"VolumeVis": VolumeVis, "TrianglesVis": TrianglesVis,
               "ParticlesVis": ParticlesVis, "PathLinesVis": PathLinesVis}.get(t)
        if cls is None:
            raise ValueError("unknown operator type %s" % t)
        ops.append(cls.from_json(o, datasets))
    return Visualization(ops, lighting, partitions=partitions, epsilon=epsilon)


def renderer_epsilon(doc, default=0.001):
    """Renderer.epsilon of a state document (Renderer.cpp:289-296)."""
    if "Renderer" in doc and "epsilon" in doc["Renderer"]:
        return float(doc["Renderer"]["epsilon"])
    return default


def load_state(path, partitions=(1, 1, 1)):
    """Read a Galaxy state file (docs/state_files.md as implemented by
    gxywriter.cpp:181-219, Datasets.cpp:99-125, Visualization.cpp:293-340,
    Camera.cpp:165-281, Renderer.cpp:289-296).  Returns (renderings, epsilon):
    one (camera, visualization) pair per camera x visualization."""
    import json
    doc = json.load(open(path))
    base = os.path.dirname(os.path.abspath(path))
    eps = renderer_epsilon(doc)
    datasets = datasets_from_json(doc, base)
    viss = [visualization_from_json(v, datasets, partitions, eps) for v in doc.get("Visualizations", [])]
    cams = [Camera.from_json(c) for c in doc.get("Cameras", [])]
    return [(c, v) for c in cams for v in viss], eps

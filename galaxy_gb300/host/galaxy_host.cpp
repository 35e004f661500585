// galaxy_host.cpp -- Galaxy's renderer-side object model over the C ABI (see
// galaxy_host.hpp).  Host code only: it builds gxy_* descriptors and calls
// libgxy_gpu.so; every number follows the single-precision arithmetic of the
// Galaxy source each function cites (compiled with -ffp-contract=off).
#include "galaxy_host.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

namespace gxyhost {

int check(int rc) {
    if (rc == GXY_OK) return rc;
    char msg[1024] = {0};
    gxy_gpu_last_error(msg, sizeof msg);
    throw GxyError(rc, msg);
}

static std::string read_file(const std::string &path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    std::ostringstream ss;
    ss << in.rdbuf();
    return ss.str();
}

static std::string dir_of(const std::string &path) {
    size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string(".") : path.substr(0, k);
}

// ----------------------------------------------------------------- Lighting
// Lighting::LoadStateFromValue (Lighting.cpp:58-115): "Sources" of [x,y,z]
// (directional) or [x,y,z,type]; directional vectors normalised in single
// precision (a zero vector becomes (0.577350, 0.577350, 0.577350)).
void Lighting::LoadStateFromValue(const Json &v) {
    if (v.has("Sources")) {
        const Json &s = v["Sources"];
        sources.clear();
        types.clear();
        for (size_t k = 0; k < s.size(); k++) {
            const Json &e = s[k];
            float x = (float)e[0].num(), y = (float)e[1].num(), z = (float)e[2].num();
            int t = e.size() == 3 ? GXY_LIGHT_DIRECTIONAL : (int)e[3].num();
            if (t == GXY_LIGHT_DIRECTIONAL) {
                float d = std::sqrt((x * x + y * y) + z * z);
                if (d == 0.0f) x = y = z = 0.577350f;
                else {
                    x = x / d;
                    y = y / d;
                    z = z / d;
                }
            }
            sources.push_back({x, y, z});
            types.push_back(t);
        }
    }
    if (v.has("shadows")) shadows = v["shadows"].boolean();
    n_ao = v.has("ao count") ? (int)v["ao count"].num() : 0;
    ao_radius = v.has("ao radius") ? (float)v["ao radius"].num() : 1.0f;
    Ka = v.has("Ka") ? (float)v["Ka"].num() : 0.5f;
    Kd = v.has("Kd") ? (float)v["Kd"].num() : 0.5f;
}

gxy_lighting Lighting::c() const {
    gxy_lighting L;
    memset(&L, 0, sizeof L);
    if (sources.size() > GXY_MAX_LIGHTS) throw std::runtime_error("too many lights");
    L.n_lights = (int)sources.size();
    for (size_t k = 0; k < sources.size(); k++) {
        for (int a = 0; a < 3; a++) L.lights[k][a] = sources[k][a];
        L.types[k] = types[k];
    }
    L.Ka = Ka;
    L.Kd = Kd;
    L.n_ao = n_ao;
    L.ao_radius = ao_radius;
    L.shadows = shadows ? 1 : 0;
    return L;
}

// ------------------------------------------------------------------- Camera
// Camera::LoadFromJSON (Camera.cpp:237-278): viewpoint, viewdirection or
// viewcenter (direction = center - point, in double), viewup, aov; the
// reference takes both width and height from dimensions[0] (Camera.cpp:
// 267-271), kept.
void Camera::LoadFromJSON(const Json &v) {
    double vp[3], d[3];
    for (int a = 0; a < 3; a++) vp[a] = v["viewpoint"][a].num();
    if (v.has("viewdirection")) {
        for (int a = 0; a < 3; a++) d[a] = v["viewdirection"][a].num();
    } else if (v.has("viewcenter")) {
        for (int a = 0; a < 3; a++) d[a] = v["viewcenter"][a].num() - vp[a];
    } else {
        throw std::runtime_error("camera needs either viewdirection or viewcenter");
    }
    for (int a = 0; a < 3; a++) {
        eye[a] = (float)vp[a];
        dir[a] = (float)d[a];
        up[a] = (float)v["viewup"][a].num();
    }
    aov = (float)v["aov"].num();
    if (v.has("dimensions")) width = height = (int)v["dimensions"][0].num();
}

gxy_camera Camera::c() const {
    gxy_camera g;
    for (int a = 0; a < 3; a++) {
        g.eye[a] = eye[a];
        g.dir[a] = dir[a];
        g.up[a] = up[a];
    }
    g.aov = aov;
    g.width = width;
    g.height = height;
    return g;
}

// ----------------------------------------------------------------- datasets
// Volume::local_import header (Volume.cpp:195-297): a .vol text header --
// type, origin, counts, deltas, raw file -- or a .json header with "type",
// "origin", "counts", "delta", "rawdata"; float or uchar samples, the raw
// file relative to the header's directory.
std::shared_ptr<Volume> Volume::Load(const std::string &path) {
    auto v = std::make_shared<Volume>();
    std::string type, raw;
    const bool is_json = path.size() > 5 && path.compare(path.size() - 5, 5, ".json") == 0;
    if (is_json) {
        Json doc = Json::parse(read_file(path));
        type = doc["type"].str();
        for (int a = 0; a < 3; a++) {
            v->origin[a] = (float)doc["origin"][a].num();
            v->counts[a] = (int)doc["counts"][a].num();
            v->deltas[a] = (float)doc["delta"][a].num();
        }
        raw = doc["rawdata"].str();
        if (doc.has("number of components") && (int)doc["number of components"].num() != 1)
            throw std::runtime_error("multi-component volumes are not rendered");
    } else {
        std::istringstream in(read_file(path));
        in >> type >> v->origin[0] >> v->origin[1] >> v->origin[2] >> v->counts[0] >> v->counts[1] >> v->counts[2] >>
            v->deltas[0] >> v->deltas[1] >> v->deltas[2] >> raw;
        if (!in) throw std::runtime_error("bad volume header " + path);
    }
    if (raw.empty() || raw[0] != '/') raw = dir_of(path) + "/" + raw;
    const size_t n = (size_t)v->counts[0] * v->counts[1] * v->counts[2];
    v->samples.resize(n);
    std::ifstream in(raw, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open raw data " + raw);
    if (type == "float") {
        in.read(reinterpret_cast<char *>(v->samples.data()), (std::streamsize)(n * sizeof(float)));
    } else {
        std::vector<unsigned char> b(n);
        in.read(reinterpret_cast<char *>(b.data()), (std::streamsize)n);
        for (size_t k = 0; k < n; k++) v->samples[k] = (float)b[k];
    }
    if (!in) throw std::runtime_error("raw data file " + raw + " is short");
    return v;
}

// ---------------------------------------------------------------- operators
// MappedVis::LoadFromJSON (MappedVis.cpp:86-203), inline maps.
void MappedVis::LoadMappedJSON(const Json &v) {
    if (v.has("data range")) {
        has_range = true;
        range[0] = (float)v["data range"][0].num();
        range[1] = (float)v["data range"][1].num();
    }
    const Json *m = v.has("transfer function") ? &v["transfer function"] : v.has("colormap") ? &v["colormap"] : nullptr;
    if (m && m->is_array()) {
        colormap.clear();
        for (size_t k = 0; k < m->size(); k++)
            colormap.push_back({(float)(*m)[k][0].num(), (float)(*m)[k][1].num(), (float)(*m)[k][2].num(),
                                (float)(*m)[k][3].num()});
        if (v.has("opacitymap")) {
            const Json &o = v["opacitymap"];
            opacitymap.clear();
            for (size_t k = 0; k < o.size(); k++) opacitymap.push_back({(float)o[k][0].num(), (float)o[k][1].num()});
        }
    }
}

// MappedVis::local_commit (MappedVis.cpp:286-333): colour and opacity maps
// resampled to 256 entries over their own x spans; valueRange the data
// range if given, else the colormap's span.
gxy_tf MappedVis::local_commit() const {
    gxy_tf tf;
    memset(&tf, 0, sizeof tf);
    if (colormap.size() < 2 || opacitymap.size() < 2) throw std::runtime_error("a map needs two control points");
    {
        size_t i0 = 0, i1 = 1;
        const double xmin = colormap.front()[0], xmax = colormap.back()[0];
        for (int i = 0; i < GXY_TF_SIZE; i++) {
            float x = (float)(xmin + (i / 255.0) * (xmax - xmin));
            if (x > colormap.back()[0]) x = colormap.back()[0];
            while (i1 < colormap.size() - 1 && colormap[i1][0] < x) {
                i0++;
                i1++;
            }
            const float d = (x - colormap[i0][0]) / (colormap[i1][0] - colormap[i0][0]);
            for (int k = 0; k < 3; k++)
                tf.colors[3 * i + k] = colormap[i0][k + 1] + d * (colormap[i1][k + 1] - colormap[i0][k + 1]);
        }
    }
    {
        size_t i0 = 0, i1 = 1;
        const double xmin = opacitymap.front()[0], xmax = opacitymap.back()[0];
        for (int i = 0; i < GXY_TF_SIZE; i++) {
            float x = (float)(xmin + (i / 255.0) * (xmax - xmin));
            if (x > opacitymap.back()[0]) x = opacitymap.back()[0];
            while (i1 < opacitymap.size() - 1 && opacitymap[i1][0] < x) {
                i0++;
                i1++;
            }
            const float d = (x - opacitymap[i0][0]) / (opacitymap[i1][0] - opacitymap[i0][0]);
            tf.opacities[i] = opacitymap[i0][1] + d * (opacitymap[i1][1] - opacitymap[i0][1]);
        }
    }
    tf.range[0] = has_range ? range[0] : colormap.front()[0];
    tf.range[1] = has_range ? range[1] : colormap.back()[0];
    return tf;
}

// VolumeVis::LoadFromJSON (VolumeVis.cpp:119-163).
void VolumeVis::LoadFromJSON(const Json &v,
                             const std::vector<std::pair<std::string, std::shared_ptr<Volume>>> &ds) {
    const std::string &name = v["dataset"].str();
    for (auto &d : ds)
        if (d.first == name) volume = d.second;
    if (!volume) throw std::runtime_error("no dataset named " + name);
    LoadMappedJSON(v);
    if (v.has("isovalues"))
        for (size_t k = 0; k < v["isovalues"].size(); k++) isovalues.push_back((float)v["isovalues"][k].num());
    const Json *s = v.has("slices") ? &v["slices"] : nullptr;
    if (s) {
        for (size_t k = 0; k < s->size(); k++)
            slices.push_back({(float)(*s)[k][0].num(), (float)(*s)[k][1].num(), (float)(*s)[k][2].num(),
                              (float)(*s)[k][3].num()});
    } else if (v.has("plane")) {
        const Json &p = v["plane"];
        slices.push_back({(float)p[0].num(), (float)p[1].num(), (float)p[2].num(), (float)p[3].num()});
    }
    volume_rendering = v.has("volume rendering") && v["volume rendering"].boolean();
}

// ------------------------------------------------------------ Visualization
// Visualization::LoadFromJSON (Visualization.cpp:293-340): lighting and the
// operators; an operator type gets "Vis" appended when it lacks it
// (Visualization.cpp:318-322).  Volume operators only: the other types read
// VTK datasets.
void Visualization::LoadFromJSON(const Json &v,
                                 const std::vector<std::pair<std::string, std::shared_ptr<Volume>>> &ds) {
    if (v.has("Lighting")) lighting.LoadStateFromValue(v["Lighting"]);
    else if (v.has("lighting")) lighting.LoadStateFromValue(v["lighting"]);
    const Json &ops = v["operators"];
    for (size_t k = 0; k < ops.size(); k++) {
        std::string t = ops[k]["type"].str();
        if (t.size() < 3 || t.compare(t.size() - 3, 3, "Vis") != 0) t += "Vis";
        if (t != "VolumeVis") throw std::runtime_error("operator type " + t + " needs VTK datasets");
        VolumeVis vv;
        vv.LoadFromJSON(ops[k], ds);
        volumes.push_back(vv);
    }
}

Visualization::~Visualization() {
    if (scene_) gxy_gpu_scene_release(scene_);
}

gxy_scene Visualization::Commit() {
    if (scene_) return scene_;
    if (volumes.size() > GXY_MAX_VOLUMES) throw std::runtime_error("too many volumes");
    std::vector<gxy_volume_vis> vv(volumes.size());
    for (size_t m = 0; m < volumes.size(); m++) {
        const VolumeVis &s = volumes[m];
        gxy_volume_vis &d = vv[m];
        memset(&d, 0, sizeof d);
        d.samples = s.volume->samples.data();
        for (int a = 0; a < 3; a++) {
            d.counts[a] = s.volume->counts[a];
            d.origin[a] = s.volume->origin[a];
            d.deltas[a] = s.volume->deltas[a];
        }
        d.tf = s.local_commit();
        if (s.slices.size() > GXY_MAX_SLICES || s.isovalues.size() > GXY_MAX_ISOVALUES)
            throw std::runtime_error("too many slices or isovalues");
        d.n_slices = (int)s.slices.size();
        for (size_t k = 0; k < s.slices.size(); k++)
            for (int a = 0; a < 4; a++) d.slices[k][a] = s.slices[k][a];
        d.n_isovalues = (int)s.isovalues.size();
        for (size_t k = 0; k < s.isovalues.size(); k++) d.isovalues[k] = s.isovalues[k];
        d.volume_render = s.volume_rendering ? 1 : 0;
    }
    gxy_scene_desc desc;
    memset(&desc, 0, sizeof desc);
    desc.n_volumes = (int)vv.size();
    desc.volumes = vv.data();
    for (int a = 0; a < 3; a++) desc.partitions[a] = partitions[a];
    desc.sampling_rate = sampling_rate;
    desc.opaque_alpha = opaque_alpha;
    desc.epsilon = epsilon;
    check(gxy_gpu_scene_commit(&desc, &scene_));
    return scene_;
}

// ------------------------------------------------------------------ RayList
void RayList::Resize(int n) {
    n_ = n;
    const size_t cap = n > 0 ? (size_t)n : 1;
    for (auto &v : f) v.assign(cap, 0.0f);
    for (auto &v : i) v.assign(cap, 0);
}

gxy_raylist RayList::view() {
    gxy_raylist r;
    float **fp[20] = {&r.ox, &r.oy, &r.oz, &r.dx, &r.dy, &r.dz, &r.nx, &r.ny, &r.nz, &r.sample,
                      &r.r,  &r.g,  &r.b,  &r.o,  &r.sr, &r.sg, &r.sb, &r.so, &r.t,  &r.tMax};
    int32_t **ip[5] = {&r.x, &r.y, &r.type, &r.term, &r.classification};
    for (int k = 0; k < 20; k++) *fp[k] = f[k].data();
    for (int k = 0; k < 5; k++) *ip[k] = i[k].data();
    r.n = n_;
    return r;
}

RayList GenerateInitialRays(Visualization &vis, const Camera &cam, int partition) {
    gxy_camera c = cam.c();
    RayList out(cam.width * cam.height);
    gxy_raylist o = out.view();
    int32_t n = 0;
    check(gxy_gpu_generate_initial_rays(vis.Commit(), partition, &c, &o, &n));
    out.Truncate(n);
    return out;
}

// TraceRays::Trace (TraceRays.cpp:68-146): at most n_ao + n_lights
// secondaries per ray.
RayList Trace(const Lighting &lighting, Visualization &vis, int partition, RayList &in) {
    gxy_lighting L = lighting.c();
    const int cap = in.GetRayCount() * (L.n_ao + L.n_lights);
    RayList out(cap);
    gxy_raylist i = in.view(), o = out.view();
    int32_t n = 0;
    check(gxy_gpu_trace_raylist(vis.Commit(), partition, &L, &i, &o, &n));
    out.Truncate(n);
    return out;
}

// ----------------------------------------------------------------- Rendering
void Rendering::Render() {
    gxy_camera c = camera.c();
    gxy_lighting in = vis->lighting.c(), L;
    check(gxy_resolve_lights(&in, &c, &L));   // Rendering::resolve_lights (Rendering.cpp:157-216)
    framebuffer.assign((size_t)camera.width * camera.height * 4, 0.0f);
    check(gxy_gpu_render_host(vis->Commit(), &c, &L, framebuffer.data(), nullptr));
    check(gxy_gpu_query_counters(vis->scene(), &counters));
}

void RenderingSet::Render() {
    for (auto &r : renderings) r->Render();
}

// gxywriter (gxywriter.cpp:181-219) over a state file: Datasets (volumes),
// Renderer epsilon (Renderer.cpp:289-296), Visualizations, Cameras; one
// Rendering per camera x visualization, cameras outermost.
std::vector<std::shared_ptr<Rendering>> LoadState(const std::string &path, const int partitions[3],
                                                  int width_override, int height_override) {
    Json doc = Json::parse(read_file(path));
    const std::string base = dir_of(path);
    float eps = 0.001f;
    if (doc.has("Renderer") && doc["Renderer"].has("epsilon")) eps = (float)doc["Renderer"]["epsilon"].num();
    std::vector<std::pair<std::string, std::shared_ptr<Volume>>> ds;
    if (doc.has("Datasets")) {
        const Json &d = doc["Datasets"];
        for (size_t k = 0; k < d.size(); k++) {
            if (d[k]["type"].str() != "Volume")
                throw std::runtime_error("dataset type " + d[k]["type"].str() + " needs VTK");
            std::string fn = d[k]["filename"].str();
            if (fn.empty() || fn[0] != '/') fn = base + "/" + fn;
            ds.emplace_back(d[k]["name"].str(), Volume::Load(fn));
        }
    }
    std::vector<std::shared_ptr<Visualization>> viss;
    if (doc.has("Visualizations")) {
        const Json &vs = doc["Visualizations"];
        for (size_t k = 0; k < vs.size(); k++) {
            auto v = std::make_shared<Visualization>();
            v->epsilon = eps;
            for (int a = 0; a < 3; a++) v->partitions[a] = partitions[a];
            v->LoadFromJSON(vs[k], ds);
            viss.push_back(v);
        }
    }
    std::vector<std::shared_ptr<Rendering>> out;
    if (doc.has("Cameras")) {
        const Json &cs = doc["Cameras"];
        for (size_t k = 0; k < cs.size(); k++) {
            Camera c;
            c.LoadFromJSON(cs[k]);
            if (width_override > 0) c.width = width_override;
            if (height_override > 0) c.height = height_override;
            for (auto &v : viss) out.push_back(std::make_shared<Rendering>(c, v));
        }
    }
    return out;
}

}  // namespace gxyhost

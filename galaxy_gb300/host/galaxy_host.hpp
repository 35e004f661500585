// galaxy_host.hpp -- Galaxy's renderer-side object model in C++ over the C
// ABI of libgxy_gpu.so (include/gxy_gpu.h): the classes a Galaxy host keeps
// -- Lighting, Camera, the MappedVis operators, Visualization, Rendering,
// RenderingSet, RayList -- with their JSON state-file loading, each calling
// the device path through the thin C layer (no CUDA or torch types here).
//
// Reference classes (paths inside the Galaxy tree):
//   Lighting        src/renderer/Lighting.cpp:58-115 (LoadStateFromValue)
//   Camera          src/renderer/Camera.cpp:165-281 (LoadFromJSON)
//   MappedVis       src/renderer/MappedVis.cpp:86-203, 277-338 (TF resampling)
//   VolumeVis       src/renderer/VolumeVis.cpp:119-163
//   ParticlesVis    src/renderer/ParticlesVis.cpp:104-118
//   Visualization   src/renderer/Visualization.cpp:293-340
//   Volume          src/data/Volume.cpp:195-297 (.vol / .json headers)
//   Rendering       src/renderer/Rendering.h:54-136, Rendering.cpp:157-216
//   RenderingSet    src/renderer/RenderingSet.h:53, RenderingSet.cpp:700-738
//   RayList         src/renderer/Rays.h:43-227
//   TraceRays       src/renderer/TraceRays.cpp:68-146
//   gxywriter       src/apps/gxywriter.cpp:181-219 (camera x visualization)
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gxy_gpu.h"
#include "json.hpp"

namespace gxyhost {

// A C-ABI status other than GXY_OK, with the library's message.
struct GxyError : std::runtime_error {
    int code;
    GxyError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
int check(int rc);   // throws GxyError unless rc == GXY_OK

// ----------------------------------------------------------------- Lighting
class Lighting {
  public:
    std::vector<std::array<float, 3>> sources{{1.f, 1.f, 1.f}};
    std::vector<int> types{GXY_LIGHT_POINT};
    float Ka = 0.5f, Kd = 0.5f;
    int n_ao = 0;
    float ao_radius = 1.0f;
    bool shadows = false;
    void LoadStateFromValue(const Json &v);
    gxy_lighting c() const;
};

// ------------------------------------------------------------------- Camera
class Camera {
  public:
    float eye[3] = {0, 0, 1}, dir[3] = {0, 0, -1}, up[3] = {0, 1, 0};
    float aov = 45.0f;
    int width = 512, height = 512;
    void LoadFromJSON(const Json &v);
    gxy_camera c() const;
};

// ----------------------------------------------------------------- datasets
class Volume {
  public:
    std::vector<float> samples;   // x fastest
    int counts[3] = {0, 0, 0};
    float origin[3] = {0, 0, 0}, deltas[3] = {1, 1, 1};
    static std::shared_ptr<Volume> Load(const std::string &path);
};

// ---------------------------------------------------------------- operators
class MappedVis {
  public:
    std::vector<std::array<float, 4>> colormap{{0.0f, 0.4f, 0.4f, 0.4f}, {1.0f, 1.0f, 1.0f, 1.0f}};
    std::vector<std::array<float, 2>> opacitymap{{0.0f, 1.0f}, {1.0f, 1.0f}};
    bool has_range = false;
    float range[2] = {0, 0};
    void LoadMappedJSON(const Json &v);
    gxy_tf local_commit() const;   // the 256-entry resampled table
};

class VolumeVis : public MappedVis {
  public:
    std::shared_ptr<Volume> volume;
    std::vector<float> isovalues;
    std::vector<std::array<float, 4>> slices;
    bool volume_rendering = false;
    void LoadFromJSON(const Json &v, const std::vector<std::pair<std::string, std::shared_ptr<Volume>>> &ds);
};

// ------------------------------------------------------------ Visualization
class Visualization {
  public:
    std::vector<VolumeVis> volumes;
    Lighting lighting;
    int partitions[3] = {1, 1, 1};
    float epsilon = 0.001f, sampling_rate = 1.0f, opaque_alpha = 0.999f;
    ~Visualization();
    void LoadFromJSON(const Json &v, const std::vector<std::pair<std::string, std::shared_ptr<Volume>>> &ds);
    // Visualization_commit + ospCommit(model): the device scene (once)
    gxy_scene Commit();
    gxy_scene scene() const { return scene_; }

  private:
    gxy_scene scene_ = nullptr;
};

// ------------------------------------------------------------------ RayList
// The 25 SoA arrays of Rays.h in host memory, with the gxy_raylist view.
class RayList {
  public:
    explicit RayList(int n = 0) { Resize(n); }
    void Resize(int n);
    int GetRayCount() const { return n_; }
    void Truncate(int n) { n_ = n; }
    gxy_raylist view();
    std::vector<float> f[20];
    std::vector<int32_t> i[5];

  private:
    int n_ = 0;
};

// TraceRays::Trace (TraceRays.cpp:68-146): traces `in` in place for
// `partition` and returns the secondary list (AO block, then shadow block).
RayList Trace(const Lighting &lighting, Visualization &vis, int partition, RayList &in);
// Camera::generate_initial_rays for one partition.
RayList GenerateInitialRays(Visualization &vis, const Camera &cam, int partition);

// ----------------------------------------------------------------- Rendering
class Rendering {
  public:
    Rendering(const Camera &c, std::shared_ptr<Visualization> v) : camera(c), vis(std::move(v)) {}
    Camera camera;
    std::shared_ptr<Visualization> vis;
    std::vector<float> framebuffer;   // height x width x RGBA, y = 0 bottom row
    gxy_counters counters{};
    // Rendering::resolve_lights then one frame of Renderer::Start
    void Render();
};

// RenderingSet: the Renderings of one state file, rendered in turn through
// the device frame path (RenderingSet.cpp:700-738 enqueues each Rendering's
// camera rays with the same Renderer).
class RenderingSet {
  public:
    std::vector<std::shared_ptr<Rendering>> renderings;
    void Render();
};

// gxywriter's reading of a state file: every camera x visualization.
std::vector<std::shared_ptr<Rendering>> LoadState(const std::string &path, const int partitions[3],
                                                  int width_override = 0, int height_override = 0);

}  // namespace gxyhost

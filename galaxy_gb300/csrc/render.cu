// render.cu -- scene commit, the fused wavefront kernels and the C ABI of
// libgxy_gpu.so.
//
// Frame path (gxy_gpu_render): one launch per queue generation.
//   generation 0: k_frame<primary> -- one thread per pixel builds the camera
//     ray (Camera::generate_initial_rays, Camera.cpp:528-829) for every
//     partition whose box the ray enters first, then traces it.
//   generation g>0: k_frame<queue> over the previous generation's queue.
// In both, each ray is traced (trace_core), shaded if it is a primary
// surface hit (ambient, AO spawn, diffuse, shadow spawn), classified and
// routed in the same thread: a TERMINATED contribution is added to the
// framebuffer with one float4 atomic, a ray handed to a neighbour partition
// or kept for re-tracing and every spawned secondary is appended to the next
// generation's queue through one warp-aggregated atomic per warp.  This is
// the device form of processRays_task::work (Renderer.cpp:511-651), where
// Galaxy's MPI partitions become partitions of one device-resident scene.
//
// RayList path (gxy_gpu_trace_raylist etc.): the same per-ray code over the
// 25-array RayList layout, one kernel per ISPC export, for ray-level parity.
#include <cooperative_groups.h>
#include <cub/cub.cuh>

#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "gxy_dev.cuh"
#include "gxy_host.h"
#include "trace.cuh"

namespace gxy {

// ================================================================ errors
static thread_local std::string g_err;
int set_error(int code, const std::string &msg) {
    g_err = msg;
    return code;
}
const std::string &last_error() { return g_err; }

// ================================================================= arena
int DeviceArena::alloc(void **p, size_t bytes) {
    std::lock_guard<std::mutex> lk(mu_);
    if (budget_ && in_use_ + bytes > budget_)
        return set_error(GXY_ERR_OOM, "HBM budget exceeded: " + std::to_string(in_use_ + bytes) + " > " +
                                          std::to_string(budget_));
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(GXY_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    in_use_ += bytes;
    live_.emplace_back(*p, bytes);
    return GXY_OK;
}
void DeviceArena::free(void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu_);
    for (size_t i = 0; i < live_.size(); i++)
        if (live_[i].first == p) {
            in_use_ -= live_[i].second;
            live_[i] = live_.back();
            live_.pop_back();
            cudaFree(p);
            return;
        }
}
size_t DeviceArena::in_use() const {
    std::lock_guard<std::mutex> lk(mu_);
    return in_use_;
}
size_t DeviceArena::budget() const {
    std::lock_guard<std::mutex> lk(mu_);
    return budget_;
}
void DeviceArena::set_budget(size_t b) {
    std::lock_guard<std::mutex> lk(mu_);
    budget_ = b;
}
bool DeviceArena::would_fit(size_t bytes) const {
    std::lock_guard<std::mutex> lk(mu_);
    return !budget_ || in_use_ + bytes <= budget_;
}
DeviceArena &arena() {
    static DeviceArena a;
    return a;
}

static bool g_init = false;
static int g_device = 0;

// ========================================================== host helpers
struct F3h {
    float x, y, z;
};
static inline F3h h3(float x, float y, float z) { return {x, y, z}; }
static inline F3h hadd(F3h a, F3h b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline F3h hmul(float s, F3h a) { return {s * a.x, s * a.y, s * a.z}; }
static inline F3h hcross(F3h a, F3h b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// Galaxy's vec3f normalize (src/data/dtypes.h:164): len in float, 1.0/len in double.
static inline F3h gnorm(F3h a) {
    float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    if (l != 0.0f) {
        float d = (float)(1.0 / (double)l);
        a.x *= d; a.y *= d; a.z *= d;
    }
    return a;
}

// Camera set-up of Camera::generate_initial_rays (Camera.cpp:542-582).
static DevCamera setup_camera(const gxy_camera &c) {
    DevCamera C;
    F3h veye = h3(c.eye[0], c.eye[1], c.eye[2]);
    F3h vu = h3(c.up[0], c.up[1], c.up[2]);
    F3h vdir = h3(c.dir[0], c.dir[1], c.dir[2]);
    F3h center;
    C.ortho = c.aov == 0.0f;
    if (C.ortho) {
        center = hadd(veye, vdir);
        vdir = gnorm(vdir);
    } else {
        float d = (float)(1.0 / tan(2 * 3.1415926 * (c.aov / 2.0) / 360.0));
        vdir = gnorm(vdir);
        center = hadd(veye, hmul(d, vdir));
    }
    F3h vr = gnorm(hcross(vdir, vu));
    vu = gnorm(hcross(vr, vdir));
    int w = c.width, h = c.height;
    float pixel_scaling = (float)((((w < h) ? w : h) - 1.0) / 2.0);
    C.off_x = (float)((w - 1) / 2.0);
    C.off_y = (float)((h - 1) / 2.0);
    C.scaling = (float)(1.0 / pixel_scaling);
    C.eye = make_float3(veye.x, veye.y, veye.z);
    C.center = make_float3(center.x, center.y, center.z);
    C.vr = make_float3(vr.x, vr.y, vr.z);
    C.vu = make_float3(vu.x, vu.y, vu.z);
    C.vdir = make_float3(vdir.x, vdir.y, vdir.z);
    C.width = w;
    C.height = h;
    return C;
}

static int setup_lights(const gxy_lighting &l, DevLights &L) {
    if (l.n_lights < 0 || l.n_lights > GXY_MAX_LIGHTS) return set_error(GXY_ERR_INVALID, "bad light count");
    memset(&L, 0, sizeof L);
    L.n = l.n_lights;
    for (int i = 0; i < l.n_lights; i++) {
        if (l.types[i] == GXY_LIGHT_CAMERA)
            return set_error(GXY_ERR_INVALID, "camera-relative light not resolved (gxy_resolve_lights)");
        L.l[i] = make_float3(l.lights[i][0], l.lights[i][1], l.lights[i][2]);
        L.type[i] = l.types[i];
    }
    L.Ka = l.Ka;
    L.Kd = l.Kd;
    L.n_ao = l.n_ao < 0 ? 0 : l.n_ao;
    L.ao_radius = l.ao_radius;
    L.shadows = l.shadows ? 1 : 0;
    if (L.n_ao > 64) return set_error(GXY_ERR_INVALID, "at most 64 AO rays per hit");
    return GXY_OK;
}

// AO tables: radical inverse base 2 / base 3 in float32 rounded through
// "%.6g" (the 256-entry randomU / randomV tables of src/renderer/UV.ih),
// stored with the derived quantities the AO direction needs.
static void ao_tables(float4 *out) {
    char buf[64];
    for (int i = 0; i < 256; i++) {
        float r[2];
        for (int b = 0; b < 2; b++) {
            int base = b ? 3 : 2;
            float inv = 1.0f / (float)base, f = inv, acc = 0.0f;
            int k = i;
            while (k > 0) {
                acc = acc + f * (float)(k % base);
                f = f * inv;
                k /= base;
            }
            snprintf(buf, sizeof buf, "%.6g", (double)acc);
            r[b] = strtof(buf, nullptr);
        }
        float a = 6.28318530717958647692f * r[0];
        out[i] = make_float4(cosf(a), sinf(a), sqrtf(1.0f - r[1]), sqrtf(r[1]));
    }
}

// ================================================================ scene
// Device buffers of the datasets and the BVH, shared by a committed scene and
// the views made from it (gxy_gpu_scene_view); freed with the last of them.
struct SharedBuffers {
    std::vector<void *> ptrs;
    ~SharedBuffers() {
        for (void *p : ptrs) arena().free(p);
    }
};

struct Scene {
    DevScene S;
    gxy_partition_info pinfo;
    std::shared_ptr<SharedBuffers> heavy = std::make_shared<SharedBuffers>();
    std::vector<void *> light;               // this handle's own buffers (TF table, flags, device copy)
    std::vector<DevTF> tf_host;              // host copy of the TF table S.tfs
    float *bmax[kMaxVol] = {};               // per volume brick: largest voxel + margin (shared)
    int64_t n_bricks[kMaxVol] = {};
    int nbz[kMaxVol] = {};
    BVHInfo bvh;
    static constexpr int kMaxLaunch = 256;   // counter slots per frame
    DevScene *d_scene = nullptr;             // device copy of S (batches)
    DRay *qmarch = nullptr;                  // split-path march queue
    float *qmarch_hit = nullptr;             // per march record: the query's closest hit (0: none)
    size_t qmarch_cap = 0;
    DRay *pmarch = nullptr;                  // split primary march queue
    float4 *pmarch_hit = nullptr;
    size_t pmarch_cap = 0;
    DRay *q[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};   // ping-pong x (primary, shadow, AO)
    size_t qcap[2][3] = {{0, 0, 0}, {0, 0, 0}};
    unsigned *rowx = nullptr;           // per image row: camera rays emitted beyond one per pixel
    size_t rowx_cap = 0;
    static constexpr int kRing = 64;    // generations of queue counts kept in device memory
    unsigned int *qcount = nullptr;     // [8..15] split-pass cursors, then kRing x 3 per-generation queue counts
    DevCounters *ctr = nullptr;         // kMaxLaunch slots, one per launch
    DevCounters last{};
    int64_t bounces = 0;
    int bands = 1;                      // image-row bands of the last frame
    float *fbtmp = nullptr;
    size_t fbtmp_elems = 0;
    int profile = 0;
    std::vector<gxy_generation_stats> gens;
    std::vector<cudaEvent_t> events;
    // continuing primaries of a generation run on `side`, beside the
    // shadow/AO passes of the same generation (fork/join events)
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    std::mutex mu;                      // one render at a time per scene
    ~Scene() {
        for (void *p : light) arena().free(p);
        for (int b = 0; b < 2; b++)
            for (int k = 0; k < 3; k++) arena().free(q[b][k]);
        arena().free(qmarch);
        arena().free(qmarch_hit);
        arena().free(pmarch);
        arena().free(pmarch_hit);
        arena().free(qcount);
        arena().free(ctr);
        arena().free(fbtmp);
        arena().free(rowx);
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (side) cudaStreamDestroy(side);
    }
    // dataset buffers (shared with views)
    int upload(const void *src, size_t bytes, void **dst) {
        int rc = arena().alloc(dst, bytes ? bytes : 16);
        if (rc) return rc;
        heavy->ptrs.push_back(*dst);
        if (bytes) CK(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
        return GXY_OK;
    }
    // this handle's own buffers
    int alloc_light(void **dst, size_t bytes) {
        int rc = arena().alloc(dst, bytes ? bytes : 16);
        if (rc) return rc;
        light.push_back(*dst);
        return GXY_OK;
    }
    int upload_light(const void *src, size_t bytes, void **dst) {
        int rc = alloc_light(dst, bytes);
        if (rc) return rc;
        if (bytes) CK(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
        return GXY_OK;
    }
};

// Brick partitions and neighbours: Volume::partition (Volume.cpp:133-172,
// 371-390) on the first volume's grid, or an even split of the geometry box.
// Bricks of a scene: a partition document's extents, else the brick grid.
static int desc_partition_count(const gxy_scene_desc &d) {
    if (d.n_partition_extents > 0) return d.n_partition_extents;
    return (d.partitions[0] < 1 ? 1 : d.partitions[0]) * (d.partitions[1] < 1 ? 1 : d.partitions[1]) *
           (d.partitions[2] < 1 ? 1 : d.partitions[2]);
}
static int check_partition_extents(const gxy_scene_desc &d) {
    if (d.n_partition_extents < 0 || d.n_partition_extents > kMaxPart)
        return set_error(GXY_ERR_INVALID, "bad partition extent count");
    if (d.n_partition_extents > 0 && !d.partition_extents)
        return set_error(GXY_ERR_INVALID, "partition extents missing");
    for (int p = 0; p < d.n_partition_extents; p++)
        for (int a = 0; a < 3; a++)
            if (!(d.partition_extents[6 * p + 2 * a] <= d.partition_extents[6 * p + 2 * a + 1]))
                return set_error(GXY_ERR_INVALID, "partition extent with min > max");
    return GXY_OK;
}

static void make_partitions(const gxy_scene_desc &d, const std::vector<float> &geo_box, DevScene &S) {
    if (d.n_partition_extents > 0) {
        // Geometry::get_partitioning (Geometry.cpp:279-350): boxes from the
        // document, global box their union, neighbour i of brick p on a face
        // when i's extent touches that face and starts where p starts on the
        // other two axes (a later match wins, as in Galaxy's loop)
        const int n = d.n_partition_extents;
        const float *E = d.partition_extents;
        S.np = n;
        float g[6] = {FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX};
        for (int i = 0; i < n; i++) {
            const float *e = E + 6 * i;
            if (e[0] < g[0]) g[0] = e[0];
            if (e[1] > g[1]) g[1] = e[1];
            if (e[2] < g[2]) g[2] = e[2];
            if (e[3] > g[3]) g[3] = e[3];
            if (e[4] < g[4]) g[4] = e[4];
            if (e[5] > g[5]) g[5] = e[5];
        }
        for (int a = 0; a < 3; a++) {
            S.glo[a] = g[2 * a];
            S.ghi[a] = g[2 * a + 1];
        }
        for (int p = 0; p < n; p++) {
            const float *l = E + 6 * p;
            DevPartition &P = S.part[p];
            for (int a = 0; a < 3; a++) {
                P.lo[a] = l[2 * a];
                P.hi[a] = l[2 * a + 1];
            }
            for (int k = 0; k < 6; k++) P.nb[k] = -1;
            for (int i = 0; i < n; i++) {
                const float *e = E + 6 * i;
                auto last = [&](int a) { return e[2 * a + 1] == l[2 * a]; };
                auto next = [&](int a) { return e[2 * a] == l[2 * a + 1]; };
                auto eq = [&](int a) { return e[2 * a] == l[2 * a]; };
                if (last(0) && eq(1) && eq(2)) P.nb[0] = i;
                if (next(0) && eq(1) && eq(2)) P.nb[1] = i;
                if (eq(0) && last(1) && eq(2)) P.nb[2] = i;
                if (eq(0) && next(1) && eq(2)) P.nb[3] = i;
                if (eq(0) && eq(1) && last(2)) P.nb[4] = i;
                if (eq(0) && eq(1) && next(2)) P.nb[5] = i;
            }
        }
        return;
    }
    int PX = d.partitions[0] < 1 ? 1 : d.partitions[0];
    int PY = d.partitions[1] < 1 ? 1 : d.partitions[1];
    int PZ = d.partitions[2] < 1 ? 1 : d.partitions[2];
    S.np = PX * PY * PZ;
    for (int k = 0; k < PZ; k++)
        for (int j = 0; j < PY; j++)
            for (int i = 0; i < PX; i++) {
                int p = i + j * PX + k * PX * PY;
                DevPartition &P = S.part[p];
                if (d.n_volumes > 0) {
                    const gxy_volume_vis &v = d.volumes[0];
                    int ni = v.counts[0] - 2, nj = v.counts[1] - 2, nk = v.counts[2] - 2;
                    int di = ni / PX, dj = nj / PY, dk = nk / PZ;
                    int off[3] = {1 + i * di, 1 + j * dj, 1 + k * dk};
                    int cnt[3] = {1 + ((i == PX - 1) ? ni - off[0] : di), 1 + ((j == PY - 1) ? nj - off[1] : dj),
                                  1 + ((k == PZ - 1) ? nk - off[2] : dk)};
                    for (int a = 0; a < 3; a++) {
                        P.lo[a] = v.origin[a] + (off[a] * v.deltas[a]);
                        P.hi[a] = P.lo[a] + (cnt[a] - 1) * v.deltas[a];
                    }
                    if (p == 0) {
                        int gc[3] = {ni, nj, nk};
                        for (int a = 0; a < 3; a++) {
                            S.glo[a] = v.origin[a] + v.deltas[a];
                            S.ghi[a] = S.glo[a] + (gc[a] - 1) * v.deltas[a];
                        }
                    }
                } else {
                    const float *g = geo_box.data();
                    float ex = (g[3] - g[0]) / PX, ey = (g[4] - g[1]) / PY, ez = (g[5] - g[2]) / PZ;
                    P.lo[0] = g[0] + i * ex; P.lo[1] = g[1] + j * ey; P.lo[2] = g[2] + k * ez;
                    P.hi[0] = i == PX - 1 ? g[3] : g[0] + (i + 1) * ex;
                    P.hi[1] = j == PY - 1 ? g[4] : g[1] + (j + 1) * ey;
                    P.hi[2] = k == PZ - 1 ? g[5] : g[2] + (k + 1) * ez;
                    for (int a = 0; a < 3; a++) { S.glo[a] = g[a]; S.ghi[a] = g[3 + a]; }
                }
                P.nb[0] = (i > 0) ? p - 1 : -1;
                P.nb[1] = (i < PX - 1) ? p + 1 : -1;
                P.nb[2] = (j > 0) ? p - PX : -1;
                P.nb[3] = (j < PY - 1) ? p + PX : -1;
                P.nb[4] = (k > 0) ? p - PX * PY : -1;
                P.nb[5] = (k < PZ - 1) ? p + PX * PY : -1;
            }
}

static float sphere_radius(const gxy_particles_vis &p, int64_t i) {   // DataDrivenSpheres.ispc:104-116
    if (p.value0 != p.value1 && p.data) {
        float d = (p.data[i] - p.value0) / (p.value1 - p.value0);
        if (d > 1) return p.radius1;
        else if (d < 0) return p.radius0;
        else return p.radius0 + d * (p.radius1 - p.radius0);
    }
    return p.radius0;
}
static float sphere_epsilon(float r0) {   // DataDrivenSpheres.ispc:211-220
    float e = logf(r0);
    if (e < 0.f) e = -1.f / e;
    if (e > r0 / 100.0f) e = r0 / 100.0f;
    return e;
}

// MAP_RADIUS (DataDrivenPathLines.cpp:11-19): per-vertex path-line radius.
static float pathline_radius(const gxy_pathlines_vis &q, int64_t i) {
    if (q.value0 == q.value1 || !q.data) return q.radius0;
    float R = (q.data[i] - q.value0) / (q.value1 - q.value0);
    return (R <= 0.0f) ? q.radius0 : (R >= 1.0f) ? q.radius1 : q.radius0 + R * (q.radius1 - q.radius0);
}

static void tf_to_dev(const gxy_tf &t, DevTF &d) {
    memcpy(d.colors, t.colors, sizeof d.colors);
    memcpy(d.opac, t.opacities, sizeof d.opac);
    d.r0 = t.range[0];
    d.r1 = t.range[1];
    d.k = 255.0f / (t.range[1] - t.range[0]);
    d.pad = 0;
}

// Linear x-fastest volume -> bricked layout (DevVolume): one thread per
// output float; voxel indices past the grid (apron of the last brick, pad
// floats) read the clamped edge voxel and are never sampled.
__global__ void k_brick_volume(const float *lin, int nx, int ny, int nz, int nbx, int nby, int64_t n_out,
                               float *out) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_out) return;
    int64_t brick = e / kBrickFloats;
    int o = (int)(e % kBrickFloats);
    if (o >= kBrickSide * kBrickSide * kBrickSide) o = 0;
    int lx = o % kBrickSide, ly = (o / kBrickSide) % kBrickSide, lz = o / (kBrickSide * kBrickSide);
    int bx = (int)(brick % nbx), by = (int)((brick / nbx) % nby), bz = (int)(brick / ((int64_t)nbx * nby));
    int x = min(bx * kBrick + lx, nx - 1), y = min(by * kBrick + ly, ny - 1), z = min(bz * kBrick + lz, nz - 1);
    out[e] = lin[((int64_t)z * ny + y) * nx + x];
}

// Per brick of a bricked volume: an upper bound of every trilinear sample
// inside it.  A sample is a convex combination of the brick's voxels, so it
// exceeds their maximum by at most a few ulps of rounding in the weights
// (margin 1e-5 relative); NaN voxels are left out of the maximum because a
// sample touching one is NaN, whose opacity is zero.  -inf for a brick of
// NaN voxels only.  One warp per brick; computed once at commit.
__global__ void k_brick_max(const float *bricked, int64_t n_bricks, float *bmax) {
    const int64_t b = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (b >= n_bricks) return;       // uniform per warp: blockDim is a multiple of 32
    const float *p = bricked + b * kBrickFloats;
    float m = -INFINITY;
    for (int o = lane; o < kBrickSide * kBrickSide * kBrickSide; o += 32) m = fmaxf(m, p[o]);
    for (int s = 16; s > 0; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
    if (lane == 0) bmax[b] = (m == -INFINITY) ? m : m + fabsf(m) * 1e-5f;
}

// Per brick: 1 when no sample inside it can reach `below` (the transfer
// function's zero-opacity threshold), i.e. its bound lies below it; a brick
// of NaN voxels is clear whenever the threshold is above -inf.  Recomputed
// whenever the volume's transfer function changes.
__global__ void k_brick_flags(const float *bmax, int64_t n_bricks, float below, unsigned char *clear) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b < n_bricks) clear[b] = bmax[b] < below;
}

// Threshold T of a transfer function such that tf_lookup gives opacity
// exactly 0 for every value v < T (and for NaN): values at or below r0 read
// opac[0]; inside the range, floor((v - r0) * k) = i interpolates opac[i]
// and opac[i + 1].  With opac[0 .. z-1] zero, every v below
// r0 + (z - 1) / k interpolates two zeros; the bound is pulled in by 1e-4
// relative to cover the rounding of (v - r0) * k.  -inf when opac[0] > 0.
// Per superbrick: the AND of the clear flags of its bricks and of the bricks
// one brick around it (clamped to the grid).  One thread per superbrick.
__global__ void k_superbrick_clear(const unsigned char *clear, int nbx, int nby, int nbz, int nsx, int nsy, int nsz,
                                   unsigned char *sclear) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsx * nsy * nsz) return;
    const int sx = s % nsx, sy = (s / nsx) % nsy, sz = s / (nsx * nsy);
    unsigned char all = 1;
    for (int bz = max(sz * kSuper - 1, 0); bz <= min(sz * kSuper + kSuper, nbz - 1) && all; bz++)
        for (int by = max(sy * kSuper - 1, 0); by <= min(sy * kSuper + kSuper, nby - 1) && all; by++)
            for (int bx = max(sx * kSuper - 1, 0); bx <= min(sx * kSuper + kSuper, nbx - 1); bx++)
                if (!clear[((int64_t)bz * nby + by) * nbx + bx]) {
                    all = 0;
                    break;
                }
    sclear[s] = all;
}

static float tf_clear_below(const DevTF &t) {
    int z = 0;
    while (z < GXY_TF_SIZE && t.opac[z] == 0.0f) z++;
    if (z == 0) return -INFINITY;
    if (z == GXY_TF_SIZE) return INFINITY;
    float T = t.r0;
    if (z >= 2 && t.k > 0.0f && std::isfinite(t.k)) {
        double lim = (double)t.r0 + (double)(z - 1) / (double)t.k * (1.0 - 1e-4);
        float f = (float)lim;
        if ((double)f > lim) f = nextafterf(f, -INFINITY);
        if (f > T) T = f;
    }
    return T;
}

// Clear-brick and superbrick flags of volume V for zero-opacity threshold
// `below`, from the per-brick bounds, on stream st.
static int volume_flags(const DevVolume &V, const float *bm, int64_t nb, int nbz, float below, cudaStream_t st) {
    k_brick_flags<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(bm, nb, below, const_cast<unsigned char *>(V.clear));
    CK(cudaGetLastError());
    const int ns = V.nsx * V.nsy * V.nsz;
    k_superbrick_clear<<<(ns + 127) / 128, 128, 0, st>>>(V.clear, V.nbx, V.nby, nbz, V.nsx, V.nsy, V.nsz,
                                                         const_cast<unsigned char *>(V.sclear));
    CK(cudaGetLastError());
    return GXY_OK;
}

// Commit-time knob GXY_TUNE_SKIP_CLEAR: build the per-brick clear flags
// (empty-space skipping in the march passes) or leave them out.
static int g_tune_skip_clear = 1;

static int commit(const gxy_scene_desc *d, Scene *sc) {
    DevScene &S = sc->S;
    memset(&S, 0, sizeof S);
    if (d->n_volumes < 0 || d->n_volumes > kMaxVol) return set_error(GXY_ERR_INVALID, "bad volume count");
    if (d->n_triangle_sets < 0 || d->n_triangle_sets > 4 || d->n_particle_sets < 0 || d->n_particle_sets > 4 ||
        d->n_pathline_sets < 0 || d->n_pathline_sets > 4)
        return set_error(GXY_ERR_INVALID, "at most 4 triangle, 4 particle and 4 path-line sets");
    int rc = check_partition_extents(*d);
    if (rc) return rc;
    int np = desc_partition_count(*d);
    if (np > kMaxPart) return set_error(GXY_ERR_INVALID, "too many partitions");
    float rate = d->sampling_rate > 0 ? d->sampling_rate : 1.0f;
    S.rate = rate;
    {
        int e;
        float m = frexpf(rate, &e);
        S.rate_pow2 = (m == 0.5f) ? 1 : 0;
        S.inv_rate = 1.0f / rate;
    }
    S.opaque_alpha = d->opaque_alpha > 0 ? d->opaque_alpha : 0.999f;
    S.epsilon = d->epsilon;
    std::vector<DevTF> tfs;
    S.step = -1;
    for (int m = 0; m < d->n_volumes; m++) {
        const gxy_volume_vis &v = d->volumes[m];
        if (!v.samples || v.counts[0] < 2 || v.counts[1] < 2 || v.counts[2] < 2)
            return set_error(GXY_ERR_INVALID, "volume needs samples and counts >= 2");
        if (v.n_slices < 0 || v.n_slices > GXY_MAX_SLICES || v.n_isovalues < 0 || v.n_isovalues > GXY_MAX_ISOVALUES)
            return set_error(GXY_ERR_INVALID, "too many slices or isovalues");
        DevVolume &V = S.vol[m];
        size_t nvox = (size_t)v.counts[0] * v.counts[1] * v.counts[2];
        V.nx = v.counts[0]; V.ny = v.counts[1]; V.nz = v.counts[2];
        // cells 0 .. n-2 per axis, kBrick cells per brick
        V.nbx = (V.nx - 2) / kBrick + 1;
        V.nby = (V.ny - 2) / kBrick + 1;
        const int nbz = (V.nz - 2) / kBrick + 1;
        const int64_t n_out = (int64_t)V.nbx * V.nby * nbz * kBrickFloats;
        {
            ScratchList tmp(arena());
            float *lin;
            if ((rc = tmp.alloc((void **)&lin, nvox * sizeof(float)))) return rc;
            CK(cudaMemcpy(lin, v.samples, nvox * sizeof(float), cudaMemcpyHostToDevice));
            float *bricked;
            if ((rc = arena().alloc((void **)&bricked, (size_t)n_out * sizeof(float)))) return rc;
            sc->heavy->ptrs.push_back(bricked);
            k_brick_volume<<<(unsigned)((n_out + 255) / 256), 256>>>(lin, V.nx, V.ny, V.nz, V.nbx, V.nby, n_out,
                                                                     bricked);
            CK(cudaGetLastError());
            CK(cudaDeviceSynchronize());
            V.data = bricked;
        }
        V.ox = v.origin[0]; V.oy = v.origin[1]; V.oz = v.origin[2];
        V.dx = v.deltas[0]; V.dy = v.deltas[1]; V.dz = v.deltas[2];
        V.ux = nextafterf((float)(V.nx - 1), 0.0f);
        V.uy = nextafterf((float)(V.ny - 1), 0.0f);
        V.uz = nextafterf((float)(V.nz - 1), 0.0f);
        V.ix = 1.0f / V.dx;
        V.iy = 1.0f / V.dy;
        V.iz = 1.0f / V.dz;
        V.tf = (int)tfs.size();
        DevTF t;
        tf_to_dev(v.tf, t);
        tfs.push_back(t);
        if (g_tune_skip_clear) {
            const int64_t nb = n_out / kBrickFloats;
            float *bm;
            if ((rc = arena().alloc((void **)&bm, (size_t)nb * sizeof(float)))) return rc;
            sc->heavy->ptrs.push_back(bm);
            k_brick_max<<<(unsigned)((nb * 32 + 255) / 256), 256>>>(V.data, nb, bm);
            CK(cudaGetLastError());
            sc->bmax[m] = bm;
            sc->n_bricks[m] = nb;
            sc->nbz[m] = nbz;
            V.nsx = (V.nbx + kSuper - 1) / kSuper;
            V.nsy = (V.nby + kSuper - 1) / kSuper;
            V.nsz = (nbz + kSuper - 1) / kSuper;
            unsigned char *clear, *sclear;
            if ((rc = sc->alloc_light((void **)&clear, (size_t)nb))) return rc;
            if ((rc = sc->alloc_light((void **)&sclear, (size_t)V.nsx * V.nsy * V.nsz))) return rc;
            V.clear = clear;
            V.sclear = sclear;
            if ((rc = volume_flags(V, bm, nb, nbz, tf_clear_below(t), 0))) return rc;
            CK(cudaDeviceSynchronize());
        }
        V.n_slices = v.n_slices;
        for (int k = 0; k < v.n_slices; k++)
            V.slices[k] = make_float4(v.slices[k][0], v.slices[k][1], v.slices[k][2], v.slices[k][3]);
        V.n_iso = v.n_isovalues;
        for (int k = 0; k < v.n_isovalues; k++) V.iso[k] = v.isovalues[k];
        V.volume_render = v.volume_render ? 1 : 0;
        if (v.volume_render || v.n_isovalues > 0) S.integrate = 1;
        if (v.n_isovalues > 0) S.has_iso = 1;
        // samplingStep = smallest spacing; step = samplingStep / rate (TraceRays.ispc:342-361)
        float ss = fminf(v.deltas[0], fminf(v.deltas[1], v.deltas[2]));
        float st = ss / rate;
        if (S.step < 0 || S.step > st) {
            S.step = st;
            S.march_eps = d->epsilon * st;
        }
    }
    S.n_vol = d->n_volumes;
    // geometry
    std::vector<float> gbox = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    int64_t prim = 0;
    for (int s = 0; s < d->n_triangle_sets; s++) {
        const gxy_triangles_vis &t = d->triangles[s];
        DevTriSet &T = S.tri_sets[s];
        T.prim_base = prim;
        T.n = t.n_triangles;
        void *p;
        if ((rc = sc->upload(t.vertices, sizeof(float) * 3 * t.n_vertices, &p))) return rc;
        T.vertices = (const float *)p;
        if ((rc = sc->upload(t.indices, sizeof(int32_t) * 3 * t.n_triangles, &p))) return rc;
        T.indices = (const int32_t *)p;
        for (int64_t i = 0; i < 3 * t.n_triangles; i++)
            if (t.indices[i] < 0 || t.indices[i] >= t.n_vertices)
                return set_error(GXY_ERR_INVALID, "triangle index out of range");
        if (t.normals) {
            if ((rc = sc->upload(t.normals, sizeof(float) * 3 * t.n_vertices, &p))) return rc;
            T.normals = (const float *)p;
        }
        if (t.data) {
            if ((rc = sc->upload(t.data, sizeof(float) * t.n_vertices, &p))) return rc;
            T.data = (const float *)p;
        }
        T.tf = (int)tfs.size();
        DevTF tt;
        tf_to_dev(t.tf, tt);
        tfs.push_back(tt);
        for (int64_t i = 0; i < t.n_vertices; i++)
            for (int a = 0; a < 3; a++) {
                gbox[a] = fminf(gbox[a], t.vertices[3 * i + a]);
                gbox[3 + a] = fmaxf(gbox[3 + a], t.vertices[3 * i + a]);
            }
        prim += t.n_triangles;
    }
    S.n_tri = prim;
    S.n_tri_sets = d->n_triangle_sets;
    std::vector<float> radius;
    for (int s = 0; s < d->n_particle_sets; s++) {
        const gxy_particles_vis &q = d->particles[s];
        DevSphSet &P = S.sph_sets[s];
        P.prim_base = prim;
        P.n = q.n;
        void *p;
        if ((rc = sc->upload(q.centers, sizeof(float) * 3 * q.n, &p))) return rc;
        P.centers = (const float *)p;
        if (q.data) {
            if ((rc = sc->upload(q.data, sizeof(float) * q.n, &p))) return rc;
            P.data = (const float *)p;
        }
        P.tf = (int)tfs.size();
        DevTF tt;
        tf_to_dev(q.tf, tt);
        tfs.push_back(tt);
        P.eps = sphere_epsilon(q.radius0);
        for (int64_t i = 0; i < q.n; i++) {
            float r = sphere_radius(q, i);
            radius.push_back(r);
            for (int a = 0; a < 3; a++) {
                gbox[a] = fminf(gbox[a], q.centers[3 * i + a] - r);
                gbox[3 + a] = fmaxf(gbox[3 + a], q.centers[3 * i + a] + r);
            }
        }
        prim += q.n;
    }
    S.n_sph = prim - S.n_tri;
    S.n_sph_sets = d->n_particle_sets;
    for (int s = 0; s < d->n_pathline_sets; s++) {
        const gxy_pathlines_vis &q = d->pathlines[s];
        if (!q.vertices || q.n_vertices < 2 || q.n_segments < 0 || (q.n_segments > 0 && !q.indices))
            return set_error(GXY_ERR_INVALID, "path lines need vertices and segment indices");
        for (int64_t i = 0; i < q.n_segments; i++)
            if (q.indices[i] < 0 || (int64_t)q.indices[i] + 1 >= q.n_vertices)
                return set_error(GXY_ERR_INVALID, "path-line segment index out of range");
        DevLineSet &L = S.line_sets[s];
        L.prim_base = prim;
        L.n = q.n_segments;
        void *p;
        if ((rc = sc->upload(q.vertices, sizeof(float) * 3 * q.n_vertices, &p))) return rc;
        L.vertices = (const float *)p;
        if ((rc = sc->upload(q.indices, sizeof(int32_t) * q.n_segments, &p))) return rc;
        L.indices = (const int32_t *)p;
        std::vector<float> rv((size_t)q.n_vertices);
        for (int64_t i = 0; i < q.n_vertices; i++) {
            rv[i] = pathline_radius(q, i);
            // DataDrivenPathLines::finalize bounds (DataDrivenPathLines.cpp:79-86)
            for (int a = 0; a < 3; a++) {
                gbox[a] = fminf(gbox[a], q.vertices[3 * i + a] - rv[i]);
                gbox[3 + a] = fmaxf(gbox[3 + a], q.vertices[3 * i + a] + rv[i]);
            }
        }
        if ((rc = sc->upload(rv.data(), rv.size() * sizeof(float), &p))) return rc;
        L.radius = (const float *)p;
        L.radius0 = q.radius0;
        L.radius1 = q.radius1;
        L.value0 = q.value0;
        L.value1 = q.value1;
        L.tf = (int)tfs.size();
        DevTF tt;
        tf_to_dev(q.tf, tt);
        tfs.push_back(tt);
        prim += q.n_segments;
    }
    S.n_seg = prim - S.n_tri - S.n_sph;
    S.n_line_sets = d->n_pathline_sets;
    if (d->has_box) gbox.assign(d->box, d->box + 6);
    else if (prim == 0) gbox = {-1, -1, -1, 1, 1, 1};
    make_partitions(*d, gbox, S);
    void *p;
    if (tfs.empty()) tfs.resize(1);
    if ((rc = sc->upload_light(tfs.data(), tfs.size() * sizeof(DevTF), &p))) return rc;
    S.tfs = (const DevTF *)p;
    sc->tf_host = tfs;
    float4 ao[256];
    ao_tables(ao);
    if ((rc = sc->upload(ao, sizeof ao, &p))) return rc;
    S.ao = (const float4 *)p;
    float *drad = nullptr;
    if (!radius.empty()) {
        if ((rc = sc->upload(radius.data(), radius.size() * sizeof(float), &p))) return rc;
        drad = (float *)p;
    }
    if ((rc = build_bvh8(S, drad, arena(), 0, sc->bvh))) return rc;
    if (sc->bvh.nodes_ptr) sc->heavy->ptrs.push_back(sc->bvh.nodes_ptr);
    if (sc->bvh.slots_ptr) sc->heavy->ptrs.push_back(sc->bvh.slots_ptr);
    sc->bvh.nodes_ptr = sc->bvh.slots_ptr = nullptr;
    CK(cudaDeviceSynchronize());
    if ((rc = sc->upload_light(&S, sizeof S, &p))) return rc;
    sc->d_scene = (DevScene *)p;
    if ((rc = arena().alloc((void **)&sc->qcount, (16 + 3 * Scene::kRing) * sizeof(unsigned int)))) return rc;
    if ((rc = arena().alloc((void **)&sc->ctr, Scene::kMaxLaunch * sizeof(DevCounters)))) return rc;
    return GXY_OK;
}

// ------------------------------------------------ transfer functions, views
// MappedVis_set_transferFunction (MappedVis.ispc:35) on a committed scene:
// the operator's 4 KB table entry is replaced in device memory; for a volume
// the clear-brick and superbrick flags are recomputed from the per-brick
// bounds (no BVH rebuild, no re-bricking).  The device pointers in DevScene
// do not change, so launches that take the scene by value and batches that
// read its device copy both see the new table.
static int scene_set_tf(Scene *sc, int kind, int index, const gxy_tf &tf, cudaStream_t st) {
    DevScene &S = sc->S;
    int slot = -1, vol = -1;
    if (kind == GXY_VIS_VOLUME && index >= 0 && index < S.n_vol) {
        slot = S.vol[index].tf;
        vol = index;
    } else if (kind == GXY_VIS_TRIANGLES && index >= 0 && index < S.n_tri_sets) {
        slot = S.tri_sets[index].tf;
    } else if (kind == GXY_VIS_PARTICLES && index >= 0 && index < S.n_sph_sets) {
        slot = S.sph_sets[index].tf;
    } else if (kind == GXY_VIS_PATHLINES && index >= 0 && index < S.n_line_sets) {
        slot = S.line_sets[index].tf;
    }
    if (slot < 0 || slot >= (int)sc->tf_host.size())
        return set_error(GXY_ERR_INVALID, "no such operator for a transfer function");
    tf_to_dev(tf, sc->tf_host[slot]);
    CK(cudaMemcpyAsync(const_cast<DevTF *>(S.tfs) + slot, &sc->tf_host[slot], sizeof(DevTF),
                       cudaMemcpyHostToDevice, st));
    if (vol >= 0 && S.vol[vol].clear) {
        int rc = volume_flags(S.vol[vol], sc->bmax[vol], sc->n_bricks[vol], sc->nbz[vol],
                              tf_clear_below(sc->tf_host[slot]), st);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(st));
    return GXY_OK;
}

// A second handle on a committed scene: the datasets and the BVH are shared,
// the transfer-function table, the clear flags and the device copy of the
// scene are its own (copies of the base's current ones), so set_tf on the
// view leaves the base -- and frames in flight on it -- untouched.
static int scene_view(Scene *base, Scene *v) {
    v->S = base->S;
    v->pinfo = base->pinfo;
    v->heavy = base->heavy;
    v->bvh = base->bvh;
    v->tf_host = base->tf_host;
    for (int m = 0; m < kMaxVol; m++) {
        v->bmax[m] = base->bmax[m];
        v->n_bricks[m] = base->n_bricks[m];
        v->nbz[m] = base->nbz[m];
    }
    DevScene &S = v->S;
    void *p;
    int rc;
    if ((rc = v->upload_light(v->tf_host.data(), v->tf_host.size() * sizeof(DevTF), &p))) return rc;
    S.tfs = (const DevTF *)p;
    for (int m = 0; m < S.n_vol; m++) {
        DevVolume &V = S.vol[m];
        if (!V.clear) continue;
        const size_t ns = (size_t)V.nsx * V.nsy * V.nsz;
        unsigned char *clear, *sclear;
        if ((rc = v->alloc_light((void **)&clear, (size_t)v->n_bricks[m]))) return rc;
        if ((rc = v->alloc_light((void **)&sclear, ns))) return rc;
        CK(cudaMemcpy(clear, base->S.vol[m].clear, (size_t)v->n_bricks[m], cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(sclear, base->S.vol[m].sclear, ns, cudaMemcpyDeviceToDevice));
        V.clear = clear;
        V.sclear = sclear;
    }
    if ((rc = v->upload_light(&S, sizeof S, &p))) return rc;
    v->d_scene = (DevScene *)p;
    if ((rc = arena().alloc((void **)&v->qcount, (16 + 3 * Scene::kRing) * sizeof(unsigned int)))) return rc;
    if ((rc = arena().alloc((void **)&v->ctr, Scene::kMaxLaunch * sizeof(DevCounters)))) return rc;
    return GXY_OK;
}

// ============================================================== kernels
constexpr int kThreads = 256;

__device__ __forceinline__ void load_tfs(const DevScene &S, DevTF *sh) {
    for (int m = 0; m < S.n_vol; m++) {
        const float4 *src = reinterpret_cast<const float4 *>(S.tfs + S.vol[m].tf);
        float4 *dst = reinterpret_cast<float4 *>(sh + m);
        for (int i = threadIdx.x; i < (int)(sizeof(DevTF) / 16); i += blockDim.x) dst[i] = __ldg(src + i);
    }
    __syncthreads();
}

// The transfer function of volume 0 into shared memory: the split passes
// run only on scenes with one volume, so they hold one 4 KB table (a block
// that holds all kMaxVol tables takes 16 KB of the SM's L1/shared space).
__device__ __forceinline__ void load_tf0(const DevScene &S, DevTF *sh) {
    if (S.n_vol > 0) {
        const float4 *src = reinterpret_cast<const float4 *>(S.tfs + S.vol[0].tf);
        float4 *dst = reinterpret_cast<float4 *>(sh);
        for (int i = threadIdx.x; i < (int)(sizeof(DevTF) / 16); i += blockDim.x) dst[i] = __ldg(src + i);
    }
    __syncthreads();
}

// Box::intersect (src/data/Box.cpp:107-150).
__device__ __forceinline__ bool box_intersect(const float lo[3], const float hi[3], V3 org, V3 dir, float &tmin,
                                              float &tmax) {
    tmin = (lo[0] - org.x) / dir.x;
    tmax = (hi[0] - org.x) / dir.x;
    if (tmin > tmax) { float t = tmin; tmin = tmax; tmax = t; }
    if (tmax < 0) return false;
    float tymin = (lo[1] - org.y) / dir.y;
    float tymax = (hi[1] - org.y) / dir.y;
    if (tymin > tymax) { float t = tymin; tymin = tymax; tymax = t; }
    if (tymax < 0) return false;
    if ((tmin > tymax) || (tymin > tmax)) return false;
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = (lo[2] - org.z) / dir.z;
    float tzmax = (hi[2] - org.z) / dir.z;
    if (tzmin > tzmax) { float t = tzmin; tzmin = tzmax; tzmax = t; }
    if (tzmax < 0) return false;
    if ((tmin > tzmax) || (tzmin > tmax)) return false;
    if (tzmin > tmin) tmin = tzmin;
    if (tzmax < tmax) tmax = tzmax;
    if (tmin < 0) tmin = 0;
    return true;
}

// SpawnRays (Camera.cpp:403-441) for pixel (x, y): the ray and the mask of
// partitions that emit it.
__device__ __forceinline__ uint64_t camera_ray(const DevScene &S, const DevCamera &C, int x, int y, V3 &org, V3 &dir) {
    float fx = ((float)x - C.off_x) * C.scaling;
    float fy = ((float)y - C.off_y) * C.scaling;
    V3 xy = v3(C.center.x + fx * C.vr.x + fy * C.vu.x, C.center.y + fx * C.vr.y + fy * C.vu.y,
               C.center.z + fx * C.vr.z + fy * C.vu.z);
    if (C.ortho) {
        org = xy - v3(C.vdir.x, C.vdir.y, C.vdir.z);
        dir = v3(C.vdir.x, C.vdir.y, C.vdir.z);
    } else {
        org = v3(C.eye.x, C.eye.y, C.eye.z);
        V3 d = xy - org;
        float l = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        if (l != 0.0f) {
            float s = (float)(1.0 / (double)l);
            d.x *= s; d.y *= s; d.z *= s;
        }
        dir = d;
    }
    float gmin, gmax;
    if (!box_intersect(S.glo, S.ghi, org, dir, gmin, gmax)) return 0;
    uint64_t mask = 0;
    for (int p = 0; p < S.np; p++) {
        float lmin, lmax;
        if (!box_intersect(S.part[p].lo, S.part[p].hi, org, dir, lmin, lmax)) continue;
        float dd = fabsf(lmin) - fabsf(gmin);
        if ((lmax >= 0) && (dd < 0.000001f) && (dd > -0.000001f)) mask |= 1ull << p;
    }
    return mask;
}

// Inclusive warp scan of v; returns the exclusive prefix, total in *tot.
__device__ __forceinline__ unsigned warp_excl_scan(unsigned v, unsigned &tot) {
    int lane = threadIdx.x & 31;
    unsigned s = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += t;
    }
    tot = __shfl_sync(0xffffffffu, s, 31);
    return s - v;
}

__device__ __forceinline__ void put_ray(DRay *q, unsigned idx, V3 o, float t, V3 d, float tmax, float r, float g,
                                        float b, float a, int x, int y, int meta, int spare = 0) {
    DRay *p = q + idx;
    p->o = make_float4(o.x, o.y, o.z, t);
    p->d = make_float4(d.x, d.y, d.z, tmax);
    p->c = make_float4(r, g, b, a);
    p->m = make_int4(x, y, meta, spare);
}

enum { Q_PRIM = 0, Q_SHADOW = 1, Q_AO = 2, NQ = 3 };
enum { K_CAMERA = 0, K_PRIMARY = 1, K_SECONDARY = 2, K_MARCH = 3, K_PMARCH = 4, K_PQUERY = 5 };
constexpr int kMaxJobs = 1024;

// One render job (a camera x visualization of a RenderingSet).
struct DevJob {
    DevCamera cam;
    DevLights L;
    float *fb;
    const DevScene *scene;             // device copy of the job's scene (batches)
    long long pix0;                    // first global pixel index of the job
    long long tile0;                   // first 8x4 pixel tile of the job among all jobs' tiles
};

struct FrameArgs {
    DevJob job0;                       // single-job launches
    const DevJob *jobs;                // batch launches
    int n_jobs;
    long long total_pix;
    long long total_tiles;             // batches: 8x4 pixel tiles of all jobs (warp-cooperative camera query)
    // single-frame camera passes: the band of image rows [band_y0,
    // band_y0 + band_rows) this launch generates (the whole image unless the
    // frame is split into bands to fit its queues)
    int band_y0, band_rows;
    const DRay *qin[NQ];
    unsigned nin[NQ];
    const unsigned *nin_dev;           // batch split passes: input queue counts in device memory
    DRay *qout[NQ];
    unsigned *qout_count;              // NQ counters
    unsigned qcap[NQ];
    DevCounters *ctr;                  // this launch's counter slot
    // split shadow/AO tracing (volume scenes): query pass -> march queue -> march pass
    int split;
    DRay *qmarch;
    // Frame path: the query pass's closest hit per march record, handed on
    // in the spare word of a shadow/AO record that moves to the next
    // partition, where the query then reuses it (null: no hand-on).
    float *qmarch_hit;
    unsigned *qmarch_count;            // [0] records, [1] fetch cursor of the march pass
    unsigned qmarch_cap;
    // split primary tracing: camera query pass -> primary march queue -> march pass
    int trav_steps;                    // refill query passes: BVH8 node visits per refill round
    int queue_chunk;                   // shadow/AO query: records a warp takes from the queue at once (0: as needed)
    int march_steps;                   // refill march passes: samples per refill round
    int skip_mode;                     // GXY_TUNE_SKIP_MODE bits
    int split_prim;
    DRay *pmarch;
    float4 *pmarch_hit;                // 2 per record: (n, c.x), (c.y, c.z, -, -)
    unsigned *pmarch_count;            // [0] records, [1] fetch cursor, [2] camera query cursor, [3] extras
    unsigned pmarch_cap;
};

// Input count of queue k for a single-frame launch: the host's count, or --
// for generations launched ahead without a host read -- the count the
// previous generation left in device memory, bounded by nin[k] (the input
// queue's capacity then).
__device__ __forceinline__ unsigned frame_nin(const FrameArgs &A, int k) {
    return A.nin_dev ? min(__ldg(A.nin_dev + k), A.nin[k]) : A.nin[k];
}

// Reserve cnt consecutive queue records for this thread: one warp-wide scan
// and one atomic per warp.  Returns the first index (or ~0u if the queue is
// full; the overflow flag is then set).  All 32 lanes must call it.
__device__ __forceinline__ unsigned warp_reserve(unsigned cnt, unsigned *counter, unsigned cap, int &ovf) {
    unsigned tot;
    unsigned pre = warp_excl_scan(cnt, tot);
    unsigned base = 0;
    if (tot) {
        if ((threadIdx.x & 31) == 0) base = atomicAdd(counter, tot);
        base = __shfl_sync(0xffffffffu, base, 0);
    }
    if (!cnt) return 0;
    unsigned idx = base + pre;
    if (idx + cnt > cap) {
        ovf = 1;
        return 0xffffffffu;
    }
    return idx;
}

// Per-thread counts (32 bits: a thread handles far fewer than 2^32 rays in
// one launch, and the warp sums in flush_counters are 64-bit).
struct LocalCounters {
    unsigned prim = 0, sh = 0, ao = 0, seg = 0, hand = 0, term = 0, drop = 0, keep = 0, enq = 0, march = 0;
    int ovf = 0;
};

// Warp-level reduction of the counters, one atomic per counter per warp (no
// block barrier, so warps retire as soon as their own rays are done).
__device__ __forceinline__ void flush_counters(DevCounters *ctr, const LocalCounters &c, const RayStats &st) {
    const int lane = threadIdx.x & 31;
    unsigned long long vals[16] = {c.prim, c.sh,  c.ao,  c.seg, c.hand,  c.term,  c.drop,  c.keep,
                                   st.samples, st.nodes, st.tris, st.sphs, c.enq, c.march, st.skipped,
                                   (unsigned long long)(c.ovf | st.ovf)};
#pragma unroll
    for (int k = 0; k < 16; k++) {
        unsigned long long v = vals[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && v) {
            if (k < 15) atomicAdd(&(&ctr->primary)[k], v);
            else atomicExch(&ctr->overflow, 1);
        }
    }
}

__device__ __forceinline__ void add_pixel(float *fb, int width, int x, int y, float r, float g, float b, float o) {
    if (r != 0.0f || g != 0.0f || b != 0.0f || o != 0.0f) {
        float4 *px = reinterpret_cast<float4 *>(fb) + ((size_t)y * width + x);
        atomicAdd(px, make_float4(r, g, b, o));
    }
}

__device__ __forceinline__ void load_ray(const DRay *q, int64_t i, TraceIn &in, int &x, int &y, int &job) {
    const float4 *src = reinterpret_cast<const float4 *>(q + i);
    float4 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2);
    int4 m = __ldg(reinterpret_cast<const int4 *>(src + 3));
    in.org = v3(a.x, a.y, a.z);
    in.t = a.w;
    in.dir = v3(b.x, b.y, b.z);
    in.tmax = b.w;
    in.r = c.x; in.g = c.y; in.b = c.z; in.o = c.w;
    x = m.x;
    y = m.y;
    in.type = ray_type(m.z);
    in.part = ray_part(m.z);
    job = ray_job(m.z);
}

// Result of tracing one primary ray segment.
struct PrimOut {
    TraceOut T;
    int dest;
    bool spawn;
    float ar, ag, ab, o_post;
};

// Shade (reverse-lighting order of TraceRays.cpp:124-131), classify, route
// and accumulate one traced primary ray segment (P.T holds the trace).
__device__ __forceinline__ void primary_finish(const DevScene &S, const DevJob &J, const TraceIn &in, int x, int y,
                                               PrimOut &P, LocalCounters &c) {
    const DevLights &L = J.L;
    P.spawn = false;
    P.ar = P.ag = P.ab = P.o_post = 0.0f;
    TraceOut &T = P.T;
    if (in.type == GXY_RAY_PRIMARY && T.surface) {
        // ambient (TraceRays.ispc:735-761)
        float s = L.Ka * (1.0f - T.o);
        float ka_ao = L.n_ao ? -L.Ka / L.n_ao : 0.0f;
        float as = ka_ao * (1.0f - T.o);
        P.ar = as * T.sc.x; P.ag = as * T.sc.y; P.ab = as * T.sc.z;
        T.r += s * T.sc.x;
        T.g += s * T.sc.y;
        T.b += s * T.sc.z;
        // diffuse (TraceRays.ispc:859-923)
        float Kd = L.Kd / L.n;
        float tr = 0, tg = 0, tb = 0;
        for (int k = 0; k < L.n; k++) {
            V3 lv;
            if (L.type[k]) {
                float t = T.t;
                V3 sp = v3(in.org.x + t * in.dir.x, in.org.y + t * in.dir.y, in.org.z + t * in.dir.z);
                lv = nrm(v3(L.l[k].x, L.l[k].y, L.l[k].z) - sp);
            } else {
                lv = neg(v3(L.l[k].x, L.l[k].y, L.l[k].z));
            }
            float dd = dot(T.n, lv);
            if (dd > 0) {
                float dff = (1.0f - T.o) * dd;
                tr += dff * T.sc.x;
                tg += dff * T.sc.y;
                tb += dff * T.sc.z;
            }
        }
        float f = Kd * (1 - T.o);
        T.r = T.r + f * tr;
        T.g = T.g + f * tg;
        T.b = T.b + f * tb;
        P.o_post = T.o + f * T.o;
        T.o = P.o_post;
        P.spawn = true;
        c.ao += L.n_ao;
        c.sh += L.shadows ? L.n : 0;
    }
    int cls = classify_ray(in.type, T.term);
    P.dest = assign_destination(S, in.part, in.type, cls, in.org, in.dir);
    if (P.dest == GXY_TERMINATED) {
        c.term++;
        add_pixel(J.fb, J.cam.width, x, y, T.r, T.g, T.b, T.o);
    } else if (P.dest == GXY_DROP_ON_FLOOR) {
        c.drop++;
    } else if (P.dest == GXY_KEEP_HERE) {
        c.keep++;
    } else {
        c.hand++;
    }
}

// Trace then finish one primary ray segment.
__device__ __forceinline__ void primary_ray(const DevScene &S, const DevTF *tfs, const DevJob &J, const TraceIn &in,
                                            int x, int y, PrimOut &P, RayStats &st, LocalCounters &c) {
    c.seg++;
    P.T = trace_core<true, false>(S, tfs, in, st);
    primary_finish(S, J, in, x, y, P, c);
}

// Warp-collective: write the continuation, AO and shadow rays of the lanes'
// primary results (act = this lane has a result).
__device__ __forceinline__ void emit_primary(const DevScene &S, const DevJob &J, int job, bool act, const TraceIn &in,
                                             int x, int y, const PrimOut &P, const FrameArgs &A, LocalCounters &c) {
    const DevLights &L = J.L;
    const TraceOut &T = P.T;
    // continuing primary -> primary queue
    unsigned cont = (act && (P.dest >= 0 || P.dest == GXY_KEEP_HERE)) ? 1u : 0u;
    unsigned idx = warp_reserve(cont, A.qout_count + Q_PRIM, A.qcap[Q_PRIM], c.ovf);
    if (cont && idx != 0xffffffffu) {
        int np_ = P.dest >= 0 ? P.dest : in.part;
        put_ray(A.qout[Q_PRIM], idx, in.org, T.t, in.dir, in.tmax, T.r, T.g, T.b, T.o, x, y,
                make_meta(in.type, np_, job));
        c.enq++;
    }
    // AO rays (TraceRays.ispc:661-730); payload uses o before diffuse
    unsigned nao = (act && P.spawn) ? (unsigned)L.n_ao : 0u;
    idx = warp_reserve(nao, A.qout_count + Q_AO, A.qcap[Q_AO], c.ovf);
    if (nao && idx != 0xffffffffu) {
        V3 b0, b1;
        ao_basis(T.n, b0, b1);
        V3 o = v3(in.org.x + T.t * in.dir.x, in.org.y + T.t * in.dir.y, in.org.z + T.t * in.dir.z);
        o = v3(o.x + S.epsilon * T.n.x, o.y + S.epsilon * T.n.y, o.z + S.epsilon * T.n.z);
        ShadeIn sh;
        sh.n = T.n; sh.x = x; sh.y = y;
        for (int j = 0; j < L.n_ao; j++) {
            Spawned s = ao_ray(S, L, sh, j, P.ar, P.ag, P.ab, b0, b1, o);
            put_ray(A.qout[Q_AO], idx + j, s.o, 0.0f, s.d, s.tmax, s.r, s.g, s.b, 0.0f, x, y,
                    make_meta(GXY_RAY_AO, in.part, job));
        }
        c.enq += nao;
    }
    // shadow rays (TraceRays.ispc:813-854); payload uses o after diffuse
    unsigned nsh = (act && P.spawn && L.shadows) ? (unsigned)L.n : 0u;
    idx = warp_reserve(nsh, A.qout_count + Q_SHADOW, A.qcap[Q_SHADOW], c.ovf);
    if (nsh && idx != 0xffffffffu) {
        float Kd = -L.Kd / L.n;
        for (int k = 0; k < L.n; k++) {
            V3 sp = v3(in.org.x + T.t * in.dir.x + S.epsilon * T.n.x, in.org.y + T.t * in.dir.y + S.epsilon * T.n.y,
                       in.org.z + T.t * in.dir.z + S.epsilon * T.n.z);
            V3 lv;
            if (L.type[k]) lv = nrm(v3(L.l[k].x, L.l[k].y, L.l[k].z) - sp);
            else lv = neg(v3(L.l[k].x, L.l[k].y, L.l[k].z));
            lv = nrm(lv);
            float dd = dot(T.n, lv);
            if (dd < 0) dd = 0;
            float dff = (1.0f - P.o_post) * Kd * dd;
            put_ray(A.qout[Q_SHADOW], idx + k, sp, 0.0f, lv, INFINITY, dff * T.sc.x, dff * T.sc.y, dff * T.sc.z,
                    0.0f, x, y, make_meta(GXY_RAY_SHADOW, in.part, job));
        }
        c.enq += nsh;
    }
}

// Trace one shadow/AO ray: a ray that ends on a surface adds its payload, a
// ray leaving its brick continues in the neighbour, the rest are dropped.
__device__ __forceinline__ int secondary_ray(const DevScene &S, const DevTF *tfs, const DevJob &J, const TraceIn &in,
                                             int x, int y, TraceOut &T, RayStats &st, LocalCounters &c) {
    c.seg++;
    T = trace_core<true, true>(S, tfs, in, st);
    int dest;
    if (T.cull) {
        dest = GXY_DROP_ON_FLOOR;
    } else {
        int cls = classify_ray(in.type, T.term);
        dest = assign_destination(S, in.part, in.type, cls, in.org, in.dir);
    }
    if (dest == GXY_TERMINATED) {
        c.term++;
        add_pixel(J.fb, J.cam.width, x, y, T.r, T.g, T.b, T.o);
    } else if (dest == GXY_DROP_ON_FLOOR) {
        c.drop++;
    } else {
        c.hand++;
    }
    return dest;
}

// Warp-collective: hand shadow/AO rays to their neighbour brick's queue.
__device__ __forceinline__ void emit_secondary(bool act, int dest, int q, int job, const TraceIn &in, int x, int y,
                                               const TraceOut &T, const FrameArgs &A, LocalCounters &c,
                                               float carry = 0.0f) {
    unsigned cs = (act && dest >= 0 && q == Q_SHADOW) ? 1u : 0u;
    unsigned ca = (act && dest >= 0 && q == Q_AO) ? 1u : 0u;
    unsigned is = warp_reserve(cs, A.qout_count + Q_SHADOW, A.qcap[Q_SHADOW], c.ovf);
    unsigned ia = warp_reserve(ca, A.qout_count + Q_AO, A.qcap[Q_AO], c.ovf);
    if (cs && is != 0xffffffffu)
        put_ray(A.qout[Q_SHADOW], is, in.org, T.t, in.dir, in.tmax, T.r, T.g, T.b, T.o, x, y,
                make_meta(in.type, dest, job), __float_as_int(carry));
    if (ca && ia != 0xffffffffu)
        put_ray(A.qout[Q_AO], ia, in.org, T.t, in.dir, in.tmax, T.r, T.g, T.b, T.o, x, y, make_meta(in.type, dest, job),
                __float_as_int(carry));
    c.enq += cs + ca;
}

// Job of a global camera-pixel index (binary search over the jobs' first pixels).
__device__ __forceinline__ int find_job(const long long *pix0, int n, long long i) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pix0[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Camera-ray generation over items [0, n_items) of a grid-stride loop.
// BATCH: pixels of all jobs (job by binary search); USCENE: every job uses
// the scene Sp (kernel parameter, TFs in shared memory), otherwise each
// job's scene is read from its device copy and TFs from global memory.
template <bool BATCH, bool USCENE>
__device__ __forceinline__ void camera_pass(const DevScene &Sp, const DevTF *tfs_uniform, const FrameArgs &A,
                                            const long long *pix0_sh, int64_t n_items, int64_t start, int64_t stride,
                                            RayStats &st, LocalCounters &c) {
    for (int64_t base = start; base < n_items; base += stride) {
        int64_t i = base + threadIdx.x;
        bool valid = i < n_items;
        TraceIn in;
        uint64_t pending = 0;
        int x = 0, y = 0, job = 0;
        const DevJob *J = &A.job0;
        if (valid) {
            if (BATCH) {
                job = find_job(pix0_sh, A.n_jobs, i);
                J = A.jobs + job;
            }
            const DevScene &S = USCENE ? Sp : *J->scene;
            int w = J->cam.width;
            int64_t li = i - (BATCH ? J->pix0 : 0);
            x = (int)(li % w);
            y = (int)(li / w) + (BATCH ? 0 : A.band_y0);
            pending = camera_ray(S, J->cam, x, y, in.org, in.dir);
            in.t = 0.0f;
            in.tmax = FLT_MAX;
            in.r = in.g = in.b = in.o = 0.0f;
            in.type = GXY_RAY_PRIMARY;
        }
        while (__any_sync(0xffffffffu, pending != 0)) {
            bool act = pending != 0;
            PrimOut P;
            const DevScene &S = USCENE ? Sp : *J->scene;
            if (act) {
                int p = __ffsll((long long)pending) - 1;
                pending &= pending - 1;
                in.part = p;
                c.prim++;
                primary_ray(S, USCENE ? tfs_uniform : S.tfs, *J, in, x, y, P, st, c);
            }
            emit_primary(S, *J, job, act, in, x, y, P, A, c);
        }
    }
}

// Queue pass over items [0, n_prim + n_sec): primaries first, then shadow
// rays, then AO rays.
template <bool BATCH, bool USCENE>
__device__ __forceinline__ void queue_pass(const DevScene &Sp, const DevTF *tfs_uniform, const FrameArgs &A,
                                           const unsigned n[NQ], int64_t start, int64_t stride, RayStats &st,
                                           LocalCounters &c) {
    const int64_t np = n[Q_PRIM], ns = n[Q_SHADOW];
    const int64_t n_items = np + ns + (int64_t)n[Q_AO];
    for (int64_t base = start; base < n_items; base += stride) {
        int64_t i = base + threadIdx.x;
        bool valid = i < n_items;
        TraceIn in;
        int x = 0, y = 0, job = 0;
        int q = i < np ? Q_PRIM : (i < np + ns ? Q_SHADOW : Q_AO);
        if (valid) load_ray(A.qin[q], q == Q_PRIM ? i : (q == Q_SHADOW ? i - np : i - np - ns), in, x, y, job);
        const DevJob &J = BATCH ? A.jobs[valid ? job : 0] : A.job0;
        const DevScene &S = USCENE ? Sp : *J.scene;
        const DevTF *tfs = USCENE ? tfs_uniform : S.tfs;
        bool actp = valid && q == Q_PRIM, acts = valid && q != Q_PRIM;
        PrimOut P;
        TraceOut T;
        int dest = GXY_DROP_ON_FLOOR;
        bool to_march = false;
        SecQuery sq;
        if (actp) primary_ray(S, tfs, J, in, x, y, P, st, c);
        if (acts) {
            if (A.split) {
                c.seg++;
                sq = sec_query(S, in, st);
                if (sq.cull) c.drop++;
                else to_march = true;
                acts = false;
            } else {
                dest = secondary_ray(S, tfs, J, in, x, y, T, st, c);
            }
        }
        if (__any_sync(0xffffffffu, actp)) emit_primary(S, J, job, actp, in, x, y, P, A, c);
        if (__any_sync(0xffffffffu, acts)) emit_secondary(acts, dest, q, job, in, x, y, T, A, c);
        if (A.split && __any_sync(0xffffffffu, to_march)) {
            unsigned idx = warp_reserve(to_march ? 1u : 0u, A.qmarch_count, A.qmarch_cap, c.ovf);
            if (to_march && idx != 0xffffffffu) {
                int meta = make_meta(in.type | (sq.surface ? 8 : 0), in.part, job);
                DRay *p = A.qmarch + idx;
                p->o = make_float4(in.org.x, in.org.y, in.org.z, in.t);
                p->d = make_float4(in.dir.x, in.dir.y, in.dir.z, in.tmax);
                p->c = make_float4(in.r, in.g, in.b, in.o);
                p->m = make_int4(x, y, meta, __float_as_int(sq.t_term));
            }
        }
    }
}

// Host-driven generations (one launch per kind, counts from the host); the
// single-frame path and the per-launch profile use these.
// The transfer functions of the scene's volumes in dynamic shared memory
// (tf_smem bytes at launch): a geometry-only scene holds none, so its
// traversal keeps the whole L1.
extern __shared__ DevTF dyn_tfs[];
static size_t tf_smem(const DevScene &S) { return sizeof(DevTF) * (size_t)S.n_vol; }

template <int KIND, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_primary(DevScene S, FrameArgs A) {
    DevTF *tfs = dyn_tfs;
    load_tfs(S, tfs);
    RayStats st;
    LocalCounters c;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x, stride = (int64_t)gridDim.x * blockDim.x;
    if (KIND == K_CAMERA) {
        camera_pass<false, true>(S, tfs, A, nullptr, (int64_t)A.job0.cam.width * A.band_rows, start, stride, st,
                                 c);
    } else {
        unsigned n[NQ] = {frame_nin(A, Q_PRIM), 0u, 0u};
        queue_pass<false, true>(S, tfs, A, n, start, stride, st, c);
    }
    flush_counters(A.ctr, c, st);
}

template <int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_secondary(DevScene S, FrameArgs A) {
    DevTF *tfs = dyn_tfs;
    load_tfs(S, tfs);
    RayStats st;
    LocalCounters c;
    unsigned n[NQ] = {0u, frame_nin(A, Q_SHADOW), frame_nin(A, Q_AO)};
    queue_pass<false, true>(S, tfs, A, n, (int64_t)blockIdx.x * blockDim.x, (int64_t)gridDim.x * blockDim.x, st, c);
    flush_counters(A.ctr, c, st);
}

// Device-driven wavefront of a batch of jobs: camera generation, then
// generations of all queues until they are empty or max_gen is reached, in
// ONE cooperative launch with a grid barrier between generations.  Queue
// sets ping-pong (2), queue counters rotate over 3 sets so that the set a
// generation will write is zeroed two barriers after it was last read.
struct WaveArgs {
    DRay *q[2][NQ];
    unsigned *counts;                  // 3 x NQ
    int max_gen;
    int *status;                       // [0] generations run, [1] rays left after max_gen
};

template <bool USCENE>
__global__ void __launch_bounds__(kThreads) k_wavefront(DevScene Su, FrameArgs A, WaveArgs W) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ DevTF tfs[kMaxVol];
    __shared__ long long pix0[kMaxJobs];
    for (int j = threadIdx.x; j < A.n_jobs; j += blockDim.x) pix0[j] = A.jobs[j].pix0;
    if (USCENE) load_tfs(Su, tfs);
    else __syncthreads();
    RayStats st;
    LocalCounters c;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x, stride = (int64_t)gridDim.x * blockDim.x;
    for (int k = 0; k < NQ; k++) A.qout[k] = W.q[0][k];
    A.qout_count = W.counts + 0;
    camera_pass<true, USCENE>(Su, tfs, A, pix0, A.total_pix, start, stride, st, c);
    grid.sync();
    int g = 1;
    for (; g < W.max_gen; g++) {
        const unsigned *cin = W.counts + NQ * ((g - 1) % 3);
        if (blockIdx.x == 0 && threadIdx.x < NQ) W.counts[NQ * ((g + 1) % 3) + threadIdx.x] = 0;
        unsigned n[NQ];
        for (int k = 0; k < NQ; k++) {
            unsigned v = *((volatile const unsigned *)(cin + k));
            n[k] = v > A.qcap[k] ? A.qcap[k] : v;
        }
        if (n[0] + n[1] + n[2] == 0) break;
        for (int k = 0; k < NQ; k++) {
            A.qin[k] = W.q[(g - 1) & 1][k];
            A.qout[k] = W.q[g & 1][k];
        }
        A.qout_count = W.counts + NQ * (g % 3);
        queue_pass<true, USCENE>(Su, tfs, A, n, start, stride, st, c);
        grid.sync();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.status[0] = g;
        const unsigned *cin = W.counts + NQ * ((g - 1) % 3);
        W.status[1] = (g >= W.max_gen) ? (int)(cin[0] + cin[1] + cin[2]) : 0;
    }
    flush_counters(A.ctr, c, st);
}

// Per-generation batch kernel (no grid barrier, so batches on different
// streams run concurrently): generation g reads the queue counts that
// generation g-1 left in device memory (counts + 3*(g-1)) and appends to
// counts + 3*g.  KIND: K_CAMERA (all jobs' pixels), K_SECONDARY, which
// here takes the primary, shadow and AO queues in one index space, or
// K_PRIMARY (the primary queue alone, beside the split shadow/AO passes).
// Shared memory: the uniform scene's transfer functions in dynamic shared
// memory (batch_tf_smem bytes at launch; none for a geometry-only scene or
// a batch of several scenes, whose rays read their own scene's tables), the
// jobs' first pixels only in the camera generation.
template <int KIND, bool USCENE, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_batch_gen(DevScene Su, FrameArgs A, const unsigned *cin) {
    DevTF *tfs = dyn_tfs;
    __shared__ long long pix0[KIND == K_CAMERA ? kMaxJobs : 1];
    if (KIND == K_CAMERA)
        for (int j = threadIdx.x; j < A.n_jobs; j += blockDim.x) pix0[j] = A.jobs[j].pix0;
    if (USCENE) load_tfs(Su, tfs);
    else __syncthreads();
    RayStats st;
    LocalCounters c;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x, stride = (int64_t)gridDim.x * blockDim.x;
    if (KIND == K_CAMERA) {
        camera_pass<true, USCENE>(Su, tfs, A, pix0, A.total_pix, start, stride, st, c);
    } else {
        unsigned n[NQ];
        for (int k = 0; k < NQ; k++) {
            unsigned v = __ldg(cin + k);
            n[k] = v > A.qcap[k] ? A.qcap[k] : v;
            if (KIND == K_PRIMARY && k != Q_PRIM) n[k] = 0;   // primaries only
        }
        if (n[0] + n[1] + n[2] == 0) return;   // uniform over the grid: no barrier below is skipped partially
        queue_pass<true, USCENE>(Su, tfs, A, n, start, stride, st, c);
    }
    flush_counters(A.ctr, c, st);
}

// Set-up of the shadow/AO query of a record `in` in its partition: the clip
// to the partition (sec_clip: dir, ray_t0, ray_t), the slice planes (a
// plane before ray_t becomes the stop, `surface`; one before tmax sets
// `slice_ahead`), the zero-payload test and the occlusion shortcut
// (GXY_TUNE_SKIP_MODE bit 3): when every march position of this partition,
// tEntry .. ray_t, lies in clear superbricks, the march would leave the
// payload as it is, so a surface anywhere before ray_t ends the ray here
// with the payload unchanged -- the nearest surface is not needed and the
// query may stop at the first hit before `stop_below` = ray_t (-inf: no
// shortcut).
__device__ __forceinline__ void sec_query_setup(const DevScene &S, const FrameArgs &A, const TraceIn &in, V3 &dir,
                                                float &ray_t0, float &ray_t, bool &surface, bool &slice_ahead,
                                                bool &zero, float &stop_below) {
    float tEntry, tExitVolume;
    sec_clip(S, in, dir, ray_t0, ray_t, tEntry, tExitVolume);
    surface = false;
    slice_ahead = false;
    for (int m = 0; m < S.n_vol; m++) {
        const DevVolume &vv = S.vol[m];
        for (int k = 0; k < vv.n_slices; k++) {
            float4 pl = vv.slices[k];
            V3 pn = v3(pl.x, pl.y, pl.z);
            float denom = dot(dir, pn);
            if (fabsf(denom) > 0.0001f) {
                float t = (pl.w - dot(in.org, pn)) / denom;
                if (t >= ray_t0 && t <= in.tmax) slice_ahead = true;
                if (t >= ray_t0 && t <= ray_t) {
                    ray_t = t;
                    surface = true;
                }
            }
        }
    }
    zero = in.r == 0.0f && in.g == 0.0f && in.b == 0.0f && in.o == 0.0f;
    stop_below = -INFINITY;
    if ((A.skip_mode & 8) && S.vol[0].sclear && !zero) {
        const DevVolume &vv = S.vol[0];
        const VolPos g = vol_pos(vv, in.org + tEntry * dir);
        if (__ldg(vv.sclear + super_of(vv, g)) && clear_run_end(vv, in.org, dir, g, tEntry, ray_t) > ray_t)
            stop_below = ray_t;
    }
}

// Query pass of split shadow/AO tracing with per-lane refill: each lane
// runs the box clip and slice test of its ray, then steps the resumable
// BVH8 traversal a few nodes at a time; a lane whose traversal is complete
// finishes the query (cull, or append to the march queue with the stop
// distance and surface flag) and takes the next ray of the shadow+AO input,
// so warps stay full while traversals of different lengths proceed.
template <bool BATCH, int MINB, bool LINES>
__global__ void __launch_bounds__(kThreads, MINB) k_sec_query(DevScene S, FrameArgs A) {
    RayStats st;
    LocalCounters c;
    const int lane = threadIdx.x & 31;
    const unsigned ns = BATCH ? min(__ldg(A.nin_dev + Q_SHADOW), A.qcap[Q_SHADOW]) : frame_nin(A, Q_SHADOW);
    const unsigned n = ns + (BATCH ? min(__ldg(A.nin_dev + Q_AO), A.qcap[Q_AO]) : frame_nin(A, Q_AO));
    unsigned *cursor = A.qmarch_count + 2;
    // records this warp has taken from the queue and not yet handed out:
    // [wnext, wend), refilled queue_chunk records at a time (GXY_TUNE_QUEUE_CHUNK)
    unsigned wnext = 0, wend = 0;
    TravState T;
    uint2 stack_mem[64];
    LocalStack stack{stack_mem};
    unsigned src = 0;   // the lane's input record (shadow, then AO index space)
    float ray_t = 0.0f;
    float stop_below = -INFINITY;   // clear segment: any hit before this ends the ray here
    float carry_out = 0.0f;         // closest hit handed on with the march record (0: none)
    bool have = false, done = false, surface = false, slice_ahead = false, zero = false;
    for (;;) {
        bool need = !have;
        unsigned mask = __ballot_sync(0xffffffffu, need);
        unsigned base = 0, split = 32, base2 = 0;   // ranks below `split` from base, the rest from base2
        if (mask) {
            const unsigned cnt = (unsigned)__popc(mask);
            if (A.queue_chunk <= 0) {
                if (lane == 0) base = atomicAdd(cursor, cnt);
                base = __shfl_sync(0xffffffffu, base, 0);
            } else {
                const unsigned avail = wend - wnext;
                base = wnext;
                if (avail >= cnt) {
                    wnext += cnt;
                } else {
                    const unsigned take = max((unsigned)A.queue_chunk, cnt - avail);
                    unsigned nb = 0;
                    if (lane == 0) nb = atomicAdd(cursor, take);
                    nb = __shfl_sync(0xffffffffu, nb, 0);
                    split = avail;
                    base2 = nb;
                    wnext = nb + (cnt - avail);
                    wend = nb + take;
                }
            }
        }
        if (need) {
            const unsigned r = __popc(mask & ((1u << lane) - 1u));
            unsigned idx = r < split ? base + r : base2 + (r - split);
            if (idx < n) {
                TraceIn in;
                int x, y, job;
                src = idx;
                load_ray(idx < ns ? A.qin[Q_SHADOW] : A.qin[Q_AO], idx < ns ? idx : idx - ns, in, x, y, job);
                c.seg++;
                // sec_query_setup's steps, written out here: as a call, the
                // kernel's register allocation spilled (72 bytes at 80
                // registers per thread)
                V3 dir;
                float ray_t0, tEntry, tExitVolume;
                sec_clip(S, in, dir, ray_t0, ray_t, tEntry, tExitVolume);
                surface = false;
                slice_ahead = false;
                for (int m = 0; m < S.n_vol; m++) {
                    const DevVolume &vv = S.vol[m];
                    for (int k = 0; k < vv.n_slices; k++) {
                        float4 pl = vv.slices[k];
                        V3 pn = v3(pl.x, pl.y, pl.z);
                        float denom = dot(dir, pn);
                        if (fabsf(denom) > 0.0001f) {
                            float t = (pl.w - dot(in.org, pn)) / denom;
                            if (t >= ray_t0 && t <= in.tmax) slice_ahead = true;
                            if (t >= ray_t0 && t <= ray_t) {
                                ray_t = t;
                                surface = true;
                            }
                        }
                    }
                }
                zero = in.r == 0.0f && in.g == 0.0f && in.b == 0.0f && in.o == 0.0f;
                // occlusion shortcut (sec_query_setup)
                stop_below = -INFINITY;
                if ((A.skip_mode & 8) && S.vol[0].sclear && !zero) {
                    const DevVolume &vv = S.vol[0];
                    const VolPos g = vol_pos(vv, in.org + tEntry * dir);
                    if (__ldg(vv.sclear + super_of(vv, g)) && clear_run_end(vv, in.org, dir, g, tEntry, ray_t) > ray_t)
                        stop_below = ray_t;
                }
                // A ray handed on from the previous partition carries the
                // closest hit its query found over its whole extent (the
                // spare word of the record); it is this query's answer as
                // well, so there is no traversal.
                const float carried =
                    A.qmarch_hit ? __int_as_float(__ldg(reinterpret_cast<const int *>(
                                                      (idx < ns ? A.qin[Q_SHADOW] + idx : A.qin[Q_AO] + (idx - ns))) + 15))
                                 : 0.0f;
                // no traversal for a zero payload (culled whatever the query
                // finds) or a slice surface inside a clear segment (the ray
                // ends there, see the shortcut above)
                if (zero || (surface && stop_below > -INFINITY)) {
                    done = true;
                } else if (carried > 0.0f) {
                    T.found = true;
                    T.h.t = carried;
                    done = true;
                } else {
                    done = trav_init(S, T, in.org, dir, ray_t0, in.tmax);
                }
                have = true;
            }
        }
        if (!__any_sync(0xffffffffu, have)) break;
        // one copy of the step body: unrolled copies overflow the instruction cache
#pragma unroll 1
        for (int k = 0; k < max(A.trav_steps, 1) && have && !done; k++)
            done = trav_step<LINES>(S, T, stack, st.nodes, st.tris, st.sphs, st.ovf, stop_below);
        bool fin = have && done;
        bool to_march = false;
        if (fin && stop_below > -INFINITY && (surface || (T.found && T.h.t < stop_below))) {
            // ends at a surface inside its clear segment: terminate as the
            // march pass would (payload unchanged, SURFACE)
            TraceIn in;
            int x, y, job;
            load_ray(src < ns ? A.qin[Q_SHADOW] : A.qin[Q_AO], src < ns ? src : src - ns, in, x, y, job);
            const bool op = fmin_(fmin_(in.r, in.g), in.b) >= 1.0f || in.o > S.opaque_alpha;
            const int cls = classify_ray(in.type, (op ? GXY_RAY_OPAQUE : 0) | GXY_RAY_SURFACE);
            const int dest = assign_destination(S, in.part, in.type, cls, in.org, in.dir);
            const DevJob &J = BATCH ? A.jobs[job] : A.job0;
            if (dest == GXY_TERMINATED) {
                c.term++;
                add_pixel(J.fb, J.cam.width, x, y, in.r, in.g, in.b, in.o);
            } else {
                c.drop++;
            }
            fin = false;
            have = false;
        }
        if (fin) {
            bool h = !zero && T.found;
            carry_out = h ? T.h.t : 0.0f;
            if (h && T.h.t < ray_t) {
                ray_t = T.h.t;
                surface = true;
            }
            bool cull = zero || (!h && !surface && !slice_ahead && !S.has_iso);
            if (cull) c.drop++;
            else to_march = true;
        }
        if (__any_sync(0xffffffffu, to_march)) {
            unsigned idx = warp_reserve(to_march ? 1u : 0u, A.qmarch_count, A.qmarch_cap, c.ovf);
            if (to_march && idx != 0xffffffffu) {
                // the input record with the surface flag in its type bits
                // (shadow and AO types leave bit 3 free) and the stop distance
                // in the spare word; re-read here so no ray fields stay live
                // through the traversal
                const float4 *q = reinterpret_cast<const float4 *>(src < ns ? A.qin[Q_SHADOW] + src
                                                                            : A.qin[Q_AO] + (src - ns));
                int4 m = __ldg(reinterpret_cast<const int4 *>(q + 3));
                DRay *p = A.qmarch + idx;
                p->o = __ldg(q);
                p->d = __ldg(q + 1);
                p->c = __ldg(q + 2);
                p->m = make_int4(m.x, m.y, m.z | (surface ? 8 : 0), __float_as_int(ray_t));
                if (A.qmarch_hit) A.qmarch_hit[idx] = carry_out;
            }
        }
        if (fin) have = false;
    }
    flush_counters(A.ctr, c, st);
}

// Warp-per-packet form of k_sec_query (GXY_TUNE_SEC_PACKET): a warp takes 32
// consecutive shadow/AO records, each lane clips its ray and tests the
// slices as k_sec_query does, and the warp finds the 32 rays' closest hits
// with one shared BVH8 traversal (packet_closest: each node line fetched
// once per warp, every lane testing its own ray).  The occlusion shortcut,
// carried hits, the cull and the march records are k_sec_query's, so the
// frames are the same; only the node and test counters differ.
template <int MINB, bool LINES>
__global__ void __launch_bounds__(kThreads, MINB) k_sec_packet(DevScene S, FrameArgs A) {
    __shared__ uint2 wstacks[kThreads / 32][64];
    RayStats st;
    LocalCounters c;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint2 *wstack = wstacks[threadIdx.x >> 5];
    const unsigned ns = frame_nin(A, Q_SHADOW);
    const unsigned n = ns + frame_nin(A, Q_AO);
    unsigned *cursor = A.qmarch_count + 2;
    for (;;) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(cursor, 32u);
        base = __shfl_sync(FULL, base, 0);
        if (base >= n) break;
        const unsigned src = base + lane;
        const bool valid = src < n;
        TraceIn in;
        in.org = v3(0, 0, 0);
        in.dir = v3(1, 1, 1);
        in.t = 0.f;
        in.tmax = 0.f;
        in.r = in.g = in.b = in.o = 0.f;
        in.type = 0;
        in.part = 0;
        int x = 0, y = 0, job = 0;
        V3 dir = v3(1, 1, 1);
        float ray_t0 = 0.f, ray_t = 0.f, stop_below = -INFINITY, carried = 0.f;
        bool surface = false, slice_ahead = false, zero = true;
        const DRay *rec = valid ? (src < ns ? A.qin[Q_SHADOW] + src : A.qin[Q_AO] + (src - ns)) : nullptr;
        if (valid) {
            load_ray(src < ns ? A.qin[Q_SHADOW] : A.qin[Q_AO], src < ns ? src : src - ns, in, x, y, job);
            c.seg++;
            float tEntry, tExitVolume;
            sec_clip(S, in, dir, ray_t0, ray_t, tEntry, tExitVolume);
            for (int m = 0; m < S.n_vol; m++) {
                const DevVolume &vv = S.vol[m];
                for (int k = 0; k < vv.n_slices; k++) {
                    const float4 pl = vv.slices[k];
                    const V3 pn = v3(pl.x, pl.y, pl.z);
                    const float denom = dot(dir, pn);
                    if (fabsf(denom) > 0.0001f) {
                        const float t = (pl.w - dot(in.org, pn)) / denom;
                        if (t >= ray_t0 && t <= in.tmax) slice_ahead = true;
                        if (t >= ray_t0 && t <= ray_t) {
                            ray_t = t;
                            surface = true;
                        }
                    }
                }
            }
            zero = in.r == 0.0f && in.g == 0.0f && in.b == 0.0f && in.o == 0.0f;
            if ((A.skip_mode & 8) && S.vol[0].sclear && !zero) {
                const DevVolume &vv = S.vol[0];
                const VolPos g = vol_pos(vv, in.org + tEntry * dir);
                if (__ldg(vv.sclear + super_of(vv, g)) && clear_run_end(vv, in.org, dir, g, tEntry, ray_t) > ray_t)
                    stop_below = ray_t;
            }
            carried = A.qmarch_hit ? __int_as_float(__ldg(reinterpret_cast<const int *>(rec) + 15)) : 0.0f;
        }
        const bool active = valid && !zero && !(surface && stop_below > -INFINITY) && !(carried > 0.0f);
        GeoHit gh;
        bool found = packet_closest<LINES>(S, in.org, dir, ray_t0, in.tmax, active, wstack, gh, st.nodes, st.tris,
                                           st.sphs, st.ovf);
        float hit_t = gh.t;
        if (valid && carried > 0.0f) {
            found = true;
            hit_t = carried;
        }
        bool to_march = false;
        float carry_out = 0.0f;
        if (valid && stop_below > -INFINITY && (surface || (found && hit_t < stop_below))) {
            // ends at a surface inside its clear segment, payload unchanged
            const bool op = fmin_(fmin_(in.r, in.g), in.b) >= 1.0f || in.o > S.opaque_alpha;
            const int cls = classify_ray(in.type, (op ? GXY_RAY_OPAQUE : 0) | GXY_RAY_SURFACE);
            const int dest = assign_destination(S, in.part, in.type, cls, in.org, in.dir);
            if (dest == GXY_TERMINATED) {
                c.term++;
                add_pixel(A.job0.fb, A.job0.cam.width, x, y, in.r, in.g, in.b, in.o);
            } else {
                c.drop++;
            }
        } else if (valid) {
            const bool h = !zero && found;
            carry_out = h ? hit_t : 0.0f;
            if (h && hit_t < ray_t) {
                ray_t = hit_t;
                surface = true;
            }
            if (zero || (!h && !surface && !slice_ahead && !S.has_iso)) c.drop++;
            else to_march = true;
        }
        const unsigned idx = warp_reserve(to_march ? 1u : 0u, A.qmarch_count, A.qmarch_cap, c.ovf);
        if (to_march && idx != 0xffffffffu) {
            const float4 *q = reinterpret_cast<const float4 *>(rec);
            const int4 m = __ldg(reinterpret_cast<const int4 *>(q + 3));
            DRay *p = A.qmarch + idx;
            p->o = __ldg(q);
            p->d = __ldg(q + 1);
            p->c = __ldg(q + 2);
            p->m = make_int4(m.x, m.y, m.z | (surface ? 8 : 0), __float_as_int(ray_t));
            if (A.qmarch_hit) A.qmarch_hit[idx] = carry_out;
        }
    }
    flush_counters(A.ctr, c, st);
}

// Query pass of split camera-ray tracing with per-lane refill: a lane takes
// the next pixel (BATCH: of all jobs, job by binary search) from a device cursor, and for each brick
// its camera ray enters first (Camera.cpp:431-441) clips to the brick, tests
// the slices, then steps the resumable BVH8 traversal a few nodes at a time;
// a finished query writes a march record (origin, direction, stop distance,
// surface flag; hit normal and colour beside it), and the lane moves to its
// next brick or pixel.  The
// first record of pixel i goes to slot i and a pixel whose ray enters no
// brick leaves a hole record (meta -1) there, so the march pass reads the
// records in pixel order; further bricks of one pixel go after slot npix.
template <bool BATCH, int MINB, bool LINES>
__global__ void __launch_bounds__(kThreads, MINB) k_cam_query(DevScene S, FrameArgs A) {
    __shared__ DevTF tfs[1];   // split passes: one volume (split_eligible)
    __shared__ long long pix0[BATCH ? kMaxJobs : 1];
    if (BATCH)
        for (int j = threadIdx.x; j < A.n_jobs; j += blockDim.x) pix0[j] = A.jobs[j].pix0;
    load_tf0(S, tfs);
    RayStats st;
    LocalCounters c;
    const int lane = threadIdx.x & 31;
    const unsigned npix =
        BATCH ? (unsigned)A.total_pix : (unsigned)A.job0.cam.width * (unsigned)A.band_rows;
    unsigned *cursor = A.pmarch_count + 2;
    TravState T;
    uint2 stack_mem[64];
    LocalStack stack{stack_mem};
    V3 hit_n = v3(0, 0, 0), hit_c = v3(0, 0, 0);
    int x = 0, y = 0, part = 0, job = 0;
    // The camera ray lives in T between bricks and after the query: T.org is
    // its origin and T.dir its direction with exact zeros replaced by 1e-6;
    // bit a of zmask marks a component that was zero (no ray copy stays live).
    int zmask = 0;
    unsigned pix = 0;   // global pixel index (all jobs' pixels in job order)
    uint64_t pending = 0;
    float ray_t = 0.0f;
    bool have = false, done = false, surface = false, exhausted = false, first = false;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(A.pmarch_count, npix);   // slots [0, npix)
    for (;;) {
        bool need = !have && pending == 0 && !exhausted;
        unsigned mask = __ballot_sync(0xffffffffu, need);
        unsigned base = 0;
        if (mask) {
            if (lane == 0) base = atomicAdd(cursor, (unsigned)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, 0);
        }
        V3 org, dir0;
        bool fresh = false;
        if (need) {
            unsigned idx = base + __popc(mask & ((1u << lane) - 1u));
            if (idx < npix) {
                pix = idx;
                unsigned li = idx;
                if (BATCH) {
                    job = find_job(pix0, A.n_jobs, idx);
                    li = idx - (unsigned)pix0[job];
                }
                const DevCamera &cam = BATCH ? A.jobs[job].cam : A.job0.cam;
                x = (int)(li % (unsigned)cam.width);
                y = (int)(li / (unsigned)cam.width) + (BATCH ? 0 : A.band_y0);
                pending = camera_ray(S, cam, x, y, org, dir0);
                fresh = true;
                first = true;
                if (!pending) A.pmarch[idx].m = make_int4(x, y, -1, 0);
            } else {
                exhausted = true;
            }
        }
        if (!have && pending) {
            if (!fresh) {   // a further brick of the pixel: its ray from T
                org = T.org;
                dir0 = v3((zmask & 1) ? 0.f : T.dir.x, (zmask & 2) ? 0.f : T.dir.y, (zmask & 4) ? 0.f : T.dir.z);
            }
            zmask = (dir0.x == 0.f ? 1 : 0) | (dir0.y == 0.f ? 2 : 0) | (dir0.z == 0.f ? 4 : 0);
            part = __ffsll((long long)pending) - 1;
            pending &= pending - 1;
            c.prim++;
            c.seg++;
            TraceIn in;
            in.org = org;
            in.dir = dir0;
            in.t = 0.0f;
            in.tmax = FLT_MAX;
            in.part = part;
            V3 dir;
            float ray_t0, tEntry, tExitVolume;
            sec_clip(S, in, dir, ray_t0, ray_t, tEntry, tExitVolume);
            surface = false;
            hit_n = v3(0, 0, 0);
            hit_c = v3(0, 0, 0);
            cam_slices(S, tfs, org, dir, ray_t0, ray_t, surface, hit_n, hit_c);
            done = trav_init(S, T, org, dir, ray_t0, ray_t);
            have = true;
        }
        if (!__any_sync(0xffffffffu, have || pending != 0 || !exhausted)) break;
#pragma unroll 1
        for (int k = 0; k < max(A.trav_steps, 1) && have && !done; k++)
            done = trav_step<LINES>(S, T, stack, st.nodes, st.tris, st.sphs, st.ovf);
        bool fin = have && done;
        if (fin && T.found) {
            ray_t = T.h.t;
            surface = true;
            geometry_shade(S, T.h, T.org, T.dir, hit_n, hit_c);
        }
        if (__any_sync(0xffffffffu, fin)) {
            bool extra = fin && !first;
            unsigned idx = pix;
            if (__any_sync(0xffffffffu, extra)) {
                unsigned e = warp_reserve(extra ? 1u : 0u, A.pmarch_count + 3, A.pmarch_cap - npix, c.ovf);
                unsigned got = __ballot_sync(0xffffffffu, extra && e != 0xffffffffu);
                if (lane == 0 && got) atomicAdd(A.pmarch_count, (unsigned)__popc(got));
                if (extra) idx = e == 0xffffffffu ? e : npix + e;
            }
            if (fin && idx != 0xffffffffu) {
                first = false;
                DRay *r = A.pmarch + idx;
                r->o = make_float4(T.org.x, T.org.y, T.org.z, 0.0f);
                r->d = make_float4((zmask & 1) ? 0.f : T.dir.x, (zmask & 2) ? 0.f : T.dir.y,
                                   (zmask & 4) ? 0.f : T.dir.z, FLT_MAX);
                r->c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                r->m = make_int4(x, y, make_meta(GXY_RAY_PRIMARY | (surface ? 8 : 0), part, job), __float_as_int(ray_t));
                A.pmarch_hit[2 * (size_t)idx] = make_float4(hit_n.x, hit_n.y, hit_n.z, hit_c.x);
                A.pmarch_hit[2 * (size_t)idx + 1] = make_float4(hit_c.y, hit_c.z, 0.0f, 0.0f);
            }
        }
        if (fin) have = false;
    }
    flush_counters(A.ctr, c, st);
}

// Query pass of split tracing for handed-off primaries (single-frame path,
// generations after the camera's): the primary queue's rays, each carrying
// its composited colour and distance, with per-lane refill as k_cam_query --
// clip to the ray's brick, slices, resumable BVH8 traversal -- then a march
// record (stop distance, surface flag, hit normal and colour beside it) for
// k_prim_march, which composites with clear-brick skipping, shades, spawns,
// classifies and routes exactly as for camera rays.
template <bool BATCH, int MINB, bool LINES>
__global__ void __launch_bounds__(kThreads, MINB) k_prim_query(DevScene S, FrameArgs A) {
    __shared__ DevTF tfs[1];   // split passes: one volume (split_eligible)
    load_tf0(S, tfs);
    RayStats st;
    LocalCounters c;
    const int lane = threadIdx.x & 31;
    const unsigned n = BATCH ? min(__ldg(A.nin_dev + Q_PRIM), A.qcap[Q_PRIM]) : frame_nin(A, Q_PRIM);
    unsigned *cursor = A.pmarch_count + 2;
    TravState T;
    uint2 stack_mem[64];
    LocalStack stack{stack_mem};
    V3 hit_n = v3(0, 0, 0), hit_c = v3(0, 0, 0);
    unsigned src = 0;
    float ray_t = 0.0f;
    bool have = false, done = false, surface = false;
    for (;;) {
        const bool need = !have;
        const unsigned mask = __ballot_sync(0xffffffffu, need);
        unsigned base = 0;
        if (mask) {
            if (lane == 0) base = atomicAdd(cursor, (unsigned)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, 0);
        }
        if (need) {
            const unsigned idx = base + __popc(mask & ((1u << lane) - 1u));
            if (idx < n) {
                TraceIn in;
                int x, y, job;
                src = idx;
                load_ray(A.qin[Q_PRIM], idx, in, x, y, job);
                c.seg++;
                V3 dir;
                float ray_t0, tEntry, tExitVolume;
                sec_clip(S, in, dir, ray_t0, ray_t, tEntry, tExitVolume);
                surface = false;
                hit_n = v3(0, 0, 0);
                hit_c = v3(0, 0, 0);
                cam_slices(S, tfs, in.org, dir, ray_t0, ray_t, surface, hit_n, hit_c);
                done = trav_init(S, T, in.org, dir, ray_t0, ray_t);
                have = true;
            }
        }
        if (!__any_sync(0xffffffffu, have)) break;
#pragma unroll 1
        for (int k = 0; k < max(A.trav_steps, 1) && have && !done; k++)
            done = trav_step<LINES>(S, T, stack, st.nodes, st.tris, st.sphs, st.ovf);
        const bool fin = have && done;
        if (fin && T.found) {
            ray_t = T.h.t;
            surface = true;
            geometry_shade(S, T.h, T.org, T.dir, hit_n, hit_c);
        }
        if (__any_sync(0xffffffffu, fin)) {
            const unsigned idx = warp_reserve(fin ? 1u : 0u, A.pmarch_count, A.pmarch_cap, c.ovf);
            if (fin && idx != 0xffffffffu) {
                // the input record with the stop distance and the surface
                // flag; the hit beside it
                const float4 *q = reinterpret_cast<const float4 *>(A.qin[Q_PRIM] + src);
                const int4 m = __ldg(reinterpret_cast<const int4 *>(q + 3));
                DRay *r = A.pmarch + idx;
                r->o = __ldg(q);
                r->d = __ldg(q + 1);
                r->c = __ldg(q + 2);
                r->m = make_int4(m.x, m.y, m.z | (surface ? 8 : 0), __float_as_int(ray_t));
                A.pmarch_hit[2 * (size_t)idx] = make_float4(hit_n.x, hit_n.y, hit_n.z, hit_c.x);
                A.pmarch_hit[2 * (size_t)idx + 1] = make_float4(hit_c.y, hit_c.z, 0.0f, 0.0f);
            }
        }
        if (fin) have = false;
    }
    flush_counters(A.ctr, c, st);
}

// Query pass of split camera-ray tracing, warp-cooperative: a warp takes
// the next 8x4 pixel tile from a device cursor and, for each brick the
// lanes' camera rays enter first (Camera.cpp:431-441), clips and tests
// slices per lane, then finds the closest hits of the 32 coherent rays with
// one shared traversal (packet_closest).  Records as k_cam_query: pixel i's
// first record in slot i, a hole record for a pixel whose ray enters no
// brick, further bricks after slot npix.  Single frame: the tiles of the
// band of rows [band_y0, band_y0 + band_rows); BATCH: the tiles of every
// job's image, job by job (DevJob::tile0), a tile never spanning two jobs,
// so a warp's rays share one camera.
template <bool BATCH, int MINB, bool LINES>
__global__ void __launch_bounds__(kThreads, MINB) k_cam_packet(DevScene S, FrameArgs A) {
    __shared__ DevTF tfs[1];   // split passes: one volume (split_eligible)
    __shared__ uint2 wstacks[kThreads / 32][64];
    __shared__ long long tile0[BATCH ? kMaxJobs : 1];
    if (BATCH)
        for (int j = threadIdx.x; j < A.n_jobs; j += blockDim.x) tile0[j] = A.jobs[j].tile0;
    load_tf0(S, tfs);
    RayStats st;
    LocalCounters c;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint2 *wstack = wstacks[threadIdx.x >> 5];
    const unsigned npix = BATCH ? (unsigned)A.total_pix : (unsigned)A.job0.cam.width * (unsigned)A.band_rows;
    const unsigned ntiles = BATCH ? (unsigned)A.total_tiles
                                  : (unsigned)(A.job0.cam.width + 7) / 8 * (unsigned)((A.band_rows + 3) / 4);
    unsigned *cursor = A.pmarch_count + 2;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(A.pmarch_count, npix);   // slots [0, npix)
    for (;;) {
        unsigned tile = 0;
        if (lane == 0) tile = atomicAdd(cursor, 1u);
        tile = __shfl_sync(FULL, tile, 0);
        if (tile >= ntiles) break;
        int job = 0;
        if (BATCH) {
            job = find_job(tile0, A.n_jobs, tile);
            tile -= (unsigned)tile0[job];
        }
        const DevCamera &cam = BATCH ? A.jobs[job].cam : A.job0.cam;
        const int w = cam.width;
        const int y0 = BATCH ? 0 : A.band_y0, hgt = BATCH ? cam.height : A.band_rows;   // rows [y0, y0 + hgt)
        const unsigned tiles_x = (unsigned)(w + 7) / 8;
        const int x = (int)(tile % tiles_x) * 8 + (lane & 7), yb = (int)(tile / tiles_x) * 4 + (lane >> 3);
        const int y = y0 + yb;
        const bool valid = x < w && yb < hgt;
        // slot: the pixel's index within the band (BATCH: among all jobs' pixels)
        const unsigned pix = valid ? (BATCH ? (unsigned)A.jobs[job].pix0 : 0u) + (unsigned)yb * (unsigned)w + (unsigned)x
                                   : 0u;
        V3 org = v3(0, 0, 0), dir0 = v3(1, 1, 1);
        uint64_t pending = 0;
        if (valid) {
            pending = camera_ray(S, cam, x, y, org, dir0);
            if (!pending) A.pmarch[pix].m = make_int4(x, y, -1, 0);
        }
        bool first = true;
        while (__any_sync(FULL, pending != 0)) {
            const bool act = pending != 0;
            int part = 0;
            V3 dir = dir0, hit_n = v3(0, 0, 0), hit_c = v3(0, 0, 0);
            float ray_t0 = 0.f, ray_t = 0.f;
            bool surface = false;
            if (act) {
                part = __ffsll((long long)pending) - 1;
                pending &= pending - 1;
                c.prim++;
                c.seg++;
                TraceIn in;
                in.org = org;
                in.dir = dir0;
                in.t = 0.0f;
                in.tmax = FLT_MAX;
                in.part = part;
                float tEntry, tExitVolume;
                sec_clip(S, in, dir, ray_t0, ray_t, tEntry, tExitVolume);
                cam_slices(S, tfs, org, dir, ray_t0, ray_t, surface, hit_n, hit_c);
            }
            GeoHit gh;
            const bool found =
                packet_closest<LINES>(S, org, dir, ray_t0, ray_t, act, wstack, gh, st.nodes, st.tris, st.sphs, st.ovf);
            if (act && found) {
                ray_t = gh.t;
                surface = true;
                geometry_shade(S, gh, org, dir, hit_n, hit_c);
            }
            const bool extra = act && !first;
            unsigned idx = pix;
            if (__any_sync(FULL, extra)) {
                unsigned e = warp_reserve(extra ? 1u : 0u, A.pmarch_count + 3, A.pmarch_cap - npix, c.ovf);
                unsigned got = __ballot_sync(FULL, extra && e != 0xffffffffu);
                if (lane == 0 && got) atomicAdd(A.pmarch_count, (unsigned)__popc(got));
                if (extra) idx = e == 0xffffffffu ? e : npix + e;
            }
            if (act && idx != 0xffffffffu) {
                first = false;
                DRay *r = A.pmarch + idx;
                r->o = make_float4(org.x, org.y, org.z, 0.0f);
                r->d = make_float4(dir0.x, dir0.y, dir0.z, FLT_MAX);
                r->c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                r->m = make_int4(x, y, make_meta(GXY_RAY_PRIMARY | (surface ? 8 : 0), part, job), __float_as_int(ray_t));
                A.pmarch_hit[2 * (size_t)idx] = make_float4(hit_n.x, hit_n.y, hit_n.z, hit_c.x);
                A.pmarch_hit[2 * (size_t)idx + 1] = make_float4(hit_c.y, hit_c.z, 0.0f, 0.0f);
            }
        }
    }
    flush_counters(A.ctr, c, st);
}

// March pass of split primary tracing with per-lane refill: composite the
// volume up to the query pass's stop distance, then shade (ambient, AO spawn,
// diffuse, shadow spawn), classify, route and accumulate as primary_ray does.
template <bool BATCH, int MINB, int SKIP>
__global__ void __launch_bounds__(kThreads, MINB) k_prim_march(DevScene S, FrameArgs A) {
    __shared__ DevTF tfs[1];   // split passes: one volume (split_eligible)
    load_tf0(S, tfs);
    RayStats st;
    LocalCounters c;
    const int lane = threadIdx.x & 31;
    const unsigned n = min(*((volatile unsigned *)A.pmarch_count), A.pmarch_cap);
    unsigned *cursor = A.pmarch_count + 1;
    SecMarch M;
    TraceIn in;
    V3 hn = v3(0, 0, 0), hc = v3(0, 0, 0);
    int x = 0, y = 0, job = 0;
    bool have = false;
    for (;;) {
        // fetch until every idle lane holds a record or the records are used
        // up; hole records (meta -1, pixels with no brick) are passed over
        bool need = !have;
        while (__any_sync(0xffffffffu, need)) {
            unsigned mask = __ballot_sync(0xffffffffu, need);
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(cursor, (unsigned)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (need) {
                unsigned idx = base + __popc(mask & ((1u << lane) - 1u));
                need = false;
                int4 m = make_int4(0, 0, -1, 0);
                if (idx < n) m = __ldg(reinterpret_cast<const int4 *>(A.pmarch + idx) + 3);
                if (idx < n && m.z < 0) {
                    need = true;
                } else if (idx < n) {
                    load_ray(A.pmarch, idx, in, x, y, job);
                    float4 h0 = __ldg(A.pmarch_hit + 2 * (size_t)idx), h1 = __ldg(A.pmarch_hit + 2 * (size_t)idx + 1);
                    hn = v3(h0.x, h0.y, h0.z);
                    hc = v3(h0.w, h1.x, h1.y);
                    bool surface = (in.type & 8) != 0;
                    in.type &= 7;
                    sec_march_init(S, in, __int_as_float(m.w), surface, M);
                    have = true;
                    c.march++;
                }
            }
        }
        if (!__any_sync(0xffffffffu, have)) break;
        if (have && !M.done) prim_march_steps<SKIP>(S, tfs[0], M, max(A.march_steps, 1), A.skip_mode & 1, st);
        bool fin = have && M.done;
        PrimOut P;
        const DevJob &J = BATCH ? A.jobs[fin ? job : 0] : A.job0;
        if (fin) {
            TraceOut &T = P.T;
            T.t = M.tTerm;
            T.term = prim_march_term(S, M);
            T.r = M.cr; T.g = M.cg; T.b = M.cb; T.o = M.ca;
            T.surface = M.surface;
            T.n = hn;
            T.sc = hc;
            T.cull = false;
            primary_finish(S, J, in, x, y, P, c);
        }
        if (__any_sync(0xffffffffu, fin)) emit_primary(S, J, job, fin, in, x, y, P, A, c);
        if (fin) have = false;
    }
    flush_counters(A.ctr, c, st);
}

// March pass of split shadow/AO tracing with per-lane refill: a lane whose
// ray has finished takes the next record of the march queue while the other
// lanes keep marching, so warps stay full across rays of different march
// lengths.  Each record carries the query pass's stop distance and surface
// flag.  USCENE / batch as for the other frame kernels (uniform scene only).
template <bool BATCH, int MINB, int SKIP, bool CONT = false>
__global__ void __launch_bounds__(kThreads, MINB) k_sec_march(DevScene S, FrameArgs A) {
    __shared__ DevTF tfs[1];   // split passes: one volume (split_eligible)
    load_tf0(S, tfs);
    RayStats st;
    LocalCounters c;
    const int lane = threadIdx.x & 31;
    const unsigned n = min(*((volatile unsigned *)A.qmarch_count), A.qmarch_cap);
    unsigned *cursor = A.qmarch_count + 1;
    SecMarch M;
    TraceIn in;
    int x = 0, y = 0, job = 0, q = Q_SHADOW;
    float carry = 0.0f;   // the query's closest hit, handed on if the ray changes partition
    bool have = false;
    for (;;) {
        bool need = !have;
        unsigned mask = __ballot_sync(0xffffffffu, need);
        unsigned base = 0;
        if (mask) {
            if (lane == 0) base = atomicAdd(cursor, (unsigned)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, 0);
        }
        if (need) {
            unsigned idx = base + __popc(mask & ((1u << lane) - 1u));
            if (idx < n) {
                load_ray(A.qmarch, idx, in, x, y, job);
                int4 m = __ldg(reinterpret_cast<const int4 *>(A.qmarch + idx) + 3);
                carry = A.qmarch_hit ? __ldg(A.qmarch_hit + idx) : 0.0f;
                bool surface = (in.type & 8) != 0;
                in.type &= 7;
                q = in.type == GXY_RAY_SHADOW ? Q_SHADOW : Q_AO;
                sec_march_init(S, in, __int_as_float(m.w), surface, M);
                have = true;
                c.march++;
            }
        }
        if (!__any_sync(0xffffffffu, have)) break;
        if (have && !M.done) sec_march_steps<SKIP>(S, tfs[0], M, max(A.march_steps, 1), 1, st);
        bool fin = have && M.done;
        int dest = GXY_DROP_ON_FLOOR;
        TraceOut T;
        if (fin) {
            const DevJob &J = BATCH ? A.jobs[job] : A.job0;
            int term = sec_march_term(S, M);
            int cls = classify_ray(in.type, term);
            dest = assign_destination(S, in.part, in.type, cls, in.org, in.dir);
            T.t = M.tTerm;
            T.r = M.cr; T.g = M.cg; T.b = M.cb; T.o = M.ca;
            if (dest == GXY_TERMINATED) {
                c.term++;
                add_pixel(J.fb, J.cam.width, x, y, T.r, T.g, T.b, T.o);
            } else if (dest == GXY_DROP_ON_FLOOR) {
                c.drop++;
            } else {
                c.hand++;
            }
            if (CONT && dest >= 0 && A.qmarch_hit) {
                // The ray moves on to brick `dest`.  It carries its query's
                // closest hit over its whole extent (carry, 0: none), which
                // is the next query's answer too, so the next generation's
                // query needs no traversal: its set-up and decisions run
                // here, and the lane marches on in the new brick.
                TraceIn nx = in;
                nx.t = M.tTerm;
                nx.r = M.cr; nx.g = M.cg; nx.b = M.cb; nx.o = M.ca;
                nx.part = dest;
                c.seg++;
                V3 ndir;
                float nt0, nt, nstop;
                bool nsurf, nahead, nzero;
                sec_query_setup(S, A, nx, ndir, nt0, nt, nsurf, nahead, nzero, nstop);
                const bool found = !nzero && !(nsurf && nstop > -INFINITY) && carry > 0.0f;
                dest = GXY_DROP_ON_FLOOR;   // nothing is written to the next generation's queues
                if (nstop > -INFINITY && (nsurf || (found && carry < nstop))) {
                    // ends at a surface inside its clear segment (payload unchanged)
                    const bool op = fmin_(fmin_(nx.r, nx.g), nx.b) >= 1.0f || nx.o > S.opaque_alpha;
                    const int ncls = classify_ray(nx.type, (op ? GXY_RAY_OPAQUE : 0) | GXY_RAY_SURFACE);
                    if (assign_destination(S, nx.part, nx.type, ncls, nx.org, nx.dir) == GXY_TERMINATED) {
                        c.term++;
                        add_pixel(J.fb, J.cam.width, x, y, nx.r, nx.g, nx.b, nx.o);
                    } else {
                        c.drop++;
                    }
                } else {
                    if (found && carry < nt) {
                        nt = carry;
                        nsurf = true;
                    }
                    if (nzero || (!found && !nsurf && !nahead && !S.has_iso)) {
                        c.drop++;
                    } else {
                        c.march++;
                        in = nx;
                        sec_march_init(S, in, nt, nsurf, M);
                        fin = false;
                    }
                }
            }
        }
        if (__any_sync(0xffffffffu, fin && dest >= 0)) emit_secondary(fin, dest, q, job, in, x, y, T, A, c, carry);
        if (fin) have = false;
    }
    flush_counters(A.ctr, c, st);
}

// -------------------------------------------------------- RayList kernels
struct RLDev {
    float *f[20];
    int32_t *i[5];
    int n;
};
enum { F_OX, F_OY, F_OZ, F_DX, F_DY, F_DZ, F_NX, F_NY, F_NZ, F_SAMPLE, F_R, F_G, F_B, F_O, F_SR, F_SG, F_SB, F_SO, F_T,
       F_TMAX };
enum { I_X, I_Y, I_TYPE, I_TERM, I_CLS };

__global__ void k_rl_trace(DevScene S, int part, RLDev R, DevCounters *ctr) {
    __shared__ DevTF tfs[kMaxVol];
    load_tfs(S, tfs);
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    RayStats st;
    if (i < R.n) {
        TraceIn in;
        in.org = v3(R.f[F_OX][i], R.f[F_OY][i], R.f[F_OZ][i]);
        in.dir = v3(R.f[F_DX][i], R.f[F_DY][i], R.f[F_DZ][i]);
        in.t = R.f[F_T][i];
        in.tmax = R.f[F_TMAX][i];
        in.r = R.f[F_R][i]; in.g = R.f[F_G][i]; in.b = R.f[F_B][i]; in.o = R.f[F_O][i];
        in.type = R.i[I_TYPE][i];
        in.part = part;
        TraceOut T = trace_core<false, false>(S, tfs, in, st);
        R.f[F_R][i] = T.r; R.f[F_G][i] = T.g; R.f[F_B][i] = T.b; R.f[F_O][i] = T.o;
        R.i[I_TERM][i] = T.term;
        R.f[F_T][i] = T.t;
        if (T.surface) {
            R.f[F_SR][i] = T.sc.x; R.f[F_SG][i] = T.sc.y; R.f[F_SB][i] = T.sc.z; R.f[F_SO][i] = 1.0f;
            R.f[F_NX][i] = T.n.x; R.f[F_NY][i] = T.n.y; R.f[F_NZ][i] = T.n.z;
        }
        if (st.ovf) atomicExch(&ctr->overflow, 1);
    }
}

// counts of secondaries per ray: [0,n) AO, [n,2n) shadow
__global__ void k_rl_counts(RLDev R, int n_ao, int n_sh, int *cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R.n) return;
    bool hit = R.i[I_TYPE][i] == GXY_RAY_PRIMARY && (R.i[I_TERM][i] & GXY_RAY_SURFACE);
    cnt[i] = hit ? n_ao : 0;
    cnt[R.n + i] = hit ? n_sh : 0;
}

__device__ __forceinline__ void rl_put(RLDev &O, int k, V3 o, V3 d, float r, float g, float b, float tmax, int x, int y,
                                       int type) {
    O.f[F_OX][k] = o.x; O.f[F_OY][k] = o.y; O.f[F_OZ][k] = o.z;
    O.f[F_DX][k] = d.x; O.f[F_DY][k] = d.y; O.f[F_DZ][k] = d.z;
    O.f[F_R][k] = r; O.f[F_G][k] = g; O.f[F_B][k] = b; O.f[F_O][k] = 0.0f;
    O.f[F_T][k] = 0.0f; O.f[F_TMAX][k] = tmax;
    O.i[I_X][k] = x; O.i[I_Y][k] = y; O.i[I_TYPE][k] = type; O.i[I_TERM][k] = 0;
}

// Ambient, AO spawn, diffuse, shadow spawn in the order of TraceRays::Trace
// with GXY_REVERSE_LIGHTING (TraceRays.cpp:124-131).  off: exclusive scans
// of the per-ray counts ([0,n) AO, [n,2n) shadow, shadow block after AO).
__global__ void k_rl_shade(DevScene S, DevLights L, RLDev R, RLDev O, const int *off, int ao_total) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R.n) return;
    if (!(R.i[I_TYPE][i] == GXY_RAY_PRIMARY && (R.i[I_TERM][i] & GXY_RAY_SURFACE))) return;
    float o = R.f[F_O][i];
    V3 n = v3(R.f[F_NX][i], R.f[F_NY][i], R.f[F_NZ][i]);
    V3 sc = v3(R.f[F_SR][i], R.f[F_SG][i], R.f[F_SB][i]);
    V3 org = v3(R.f[F_OX][i], R.f[F_OY][i], R.f[F_OZ][i]);
    V3 dir = v3(R.f[F_DX][i], R.f[F_DY][i], R.f[F_DZ][i]);
    float t = R.f[F_T][i];
    int x = R.i[I_X][i], y = R.i[I_Y][i];
    // ambient
    float s = L.Ka * (1.0f - o);
    R.f[F_R][i] += s * sc.x;
    R.f[F_G][i] += s * sc.y;
    R.f[F_B][i] += s * sc.z;
    // AO
    if (L.n_ao) {
        float Ka = -L.Ka / L.n_ao;
        float as = Ka * (1.0f - o);
        float ar = as * sc.x, ag = as * sc.y, ab = as * sc.z;
        V3 b0, b1;
        ao_basis(n, b0, b1);
        V3 p = v3(org.x + t * dir.x, org.y + t * dir.y, org.z + t * dir.z);
        p = v3(p.x + S.epsilon * n.x, p.y + S.epsilon * n.y, p.z + S.epsilon * n.z);
        ShadeIn h;
        h.n = n; h.x = x; h.y = y;
        int base = off[i];
        for (int j = 0; j < L.n_ao; j++) {
            Spawned sp = ao_ray(S, L, h, j, ar, ag, ab, b0, b1, p);
            rl_put(O, base + j, sp.o, sp.d, sp.r, sp.g, sp.b, sp.tmax, x, y, GXY_RAY_AO);
        }
    }
    // diffuse
    float Kd = L.Kd / L.n;
    float tr = 0, tg = 0, tb = 0;
    for (int k = 0; k < L.n; k++) {
        V3 lv;
        if (L.type[k]) {
            V3 sp = v3(org.x + t * dir.x, org.y + t * dir.y, org.z + t * dir.z);
            lv = nrm(v3(L.l[k].x, L.l[k].y, L.l[k].z) - sp);
        } else {
            lv = neg(v3(L.l[k].x, L.l[k].y, L.l[k].z));
        }
        float dd = dot(n, lv);
        if (dd > 0) {
            float dff = (1.0f - o) * dd;
            tr += dff * sc.x; tg += dff * sc.y; tb += dff * sc.z;
        }
    }
    float f = Kd * (1 - o);
    R.f[F_R][i] = R.f[F_R][i] + f * tr;
    R.f[F_G][i] = R.f[F_G][i] + f * tg;
    R.f[F_B][i] = R.f[F_B][i] + f * tb;
    float o2 = o + f * o;
    R.f[F_O][i] = o2;
    // shadows
    if (L.shadows) {
        float Kds = -L.Kd / L.n;
        int base = ao_total + off[R.n + i];
        for (int k = 0; k < L.n; k++) {
            V3 sp = v3(org.x + t * dir.x + S.epsilon * n.x, org.y + t * dir.y + S.epsilon * n.y,
                       org.z + t * dir.z + S.epsilon * n.z);
            V3 lv;
            if (L.type[k]) lv = nrm(v3(L.l[k].x, L.l[k].y, L.l[k].z) - sp);
            else lv = neg(v3(L.l[k].x, L.l[k].y, L.l[k].z));
            lv = nrm(lv);
            float dd = dot(n, lv);
            if (dd < 0) dd = 0;
            float dff = (1.0f - o2) * Kds * dd;
            rl_put(O, base + k, sp, lv, dff * sc.x, dff * sc.y, dff * sc.z, INFINITY, x, y, GXY_RAY_SHADOW);
        }
    }
}

__global__ void k_rl_classify(RLDev R) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R.n) return;
    R.i[I_CLS][i] = classify_ray(R.i[I_TYPE][i], R.i[I_TERM][i]);
}

__global__ void k_rl_assign(DevScene S, int part, RLDev R) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R.n) return;
    V3 o = v3(R.f[F_OX][i], R.f[F_OY][i], R.f[F_OZ][i]);
    V3 d = v3(R.f[F_DX][i], R.f[F_DY][i], R.f[F_DZ][i]);
    R.i[I_CLS][i] = assign_destination(S, part, R.i[I_TYPE][i], R.i[I_CLS][i], o, d);
}

__global__ void k_rl_accumulate(RLDev R, float *fb, int w, int h) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R.n) return;
    if (R.i[I_CLS][i] != GXY_TERMINATED) return;
    int x = R.i[I_X][i], y = R.i[I_Y][i];
    if (x < 0 || y < 0 || x >= w || y >= h) return;
    float4 *p = reinterpret_cast<float4 *>(fb) + ((size_t)y * w + x);
    atomicAdd(p, make_float4(R.f[F_R][i], R.f[F_G][i], R.f[F_B][i], R.f[F_O][i]));
}

// camera rays of one partition: flag pass, then ordered scatter
__global__ void k_rl_camera_flags(DevScene S, DevCamera C, int part, int *flag) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)C.width * C.height) return;
    V3 o, d;
    uint64_t m = camera_ray(S, C, (int)(i % C.width), (int)(i / C.width), o, d);
    flag[i] = (m >> part) & 1ull;
}
__global__ void k_rl_camera_write(DevScene S, DevCamera C, int part, const int *flag, const int *pos, RLDev O) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)C.width * C.height || !flag[i]) return;
    V3 o, d;
    int x = (int)(i % C.width), y = (int)(i / C.width);
    camera_ray(S, C, x, y, o, d);
    int k = pos[i];
    O.f[F_OX][k] = o.x; O.f[F_OY][k] = o.y; O.f[F_OZ][k] = o.z;
    O.f[F_DX][k] = d.x; O.f[F_DY][k] = d.y; O.f[F_DZ][k] = d.z;
    O.f[F_R][k] = 0; O.f[F_G][k] = 0; O.f[F_B][k] = 0; O.f[F_O][k] = 0;
    O.f[F_T][k] = 0; O.f[F_TMAX][k] = FLT_MAX;
    O.i[I_X][k] = x; O.i[I_Y][k] = y; O.i[I_TYPE][k] = GXY_RAY_PRIMARY; O.i[I_TERM][k] = 0;
}

// ============================================================ frame loop
// Run-time tuning knobs (gxy_gpu_set_tuning): resident blocks per SM the
// kernels are compiled for (register budget 2 -> 128, 3 -> 80 registers per
// thread) and the grid-stride grid size in blocks per SM.
static int g_tune_minb = 3;
static int g_tune_grid_per_sm = 16;
static int g_tune_split = 1;   // split shadow/AO tracing into query + refill-march passes
static int g_tune_split_prim = 1;   // split camera rays into query + refill-march passes
static int g_tune_sah = 0;          // BVH binary tree by binned SAH (else radix-tree splits)
bool sah_builder() { return g_tune_sah != 0; }
int sah_cluster_size() { return g_tune_sah == 1 ? 256 : g_tune_sah; }
static int g_tune_leaf = 1;         // primitives per BVH8 leaf (at most)
static int g_tune_trav_steps = 8;   // node visits per refill round of the query passes
static int g_tune_march_steps = 16; // samples per refill round of the march passes
static int g_tune_skip_mode = 9;    // clear-brick skipping per pass (GXY_TUNE_SKIP_MODE bits)
static int g_tune_carry_hits = 1;   // hand the closest hit on with shadow/AO rays that change partition
static int g_tune_cam_packet = 1;   // single-frame camera query: warp-cooperative (1) or per-lane refill (0)
static int g_tune_queue_chunk = 0;  // shadow/AO query: records per block taken from the queue at once (0: as needed)
static int g_tune_split_handoff = 1; // handed-off primaries of volume scenes: query + skipping march (1) or one pass (0)
static int g_tune_sec_packet = 0;    // shadow/AO query of a frame: per-lane refill (0) or warp per 32-ray packet (1)
static int g_tune_runahead = 16;     // frame generations launched per host read of the queue counts, at most
static int g_tune_query_blocks = 3;  // shadow/AO query at 2 (128 registers), 3 (80) or 4 (64) blocks per SM (blocks_per_sm 3)
static int g_tune_pmarch_blocks = 2; // camera-ray march at 2 (128 registers) or 3 (80) blocks per SM (blocks_per_sm 3)
static int g_tune_pquery_blocks = 2; // frame camera and handed-off primary queries at 2 (128 registers) or 4 (64)
static int g_tune_continue = 1;      // shadow/AO rays that change brick march on in the same lane (carried hits on)
int leaf_max() { return g_tune_leaf; }
static int g_tune_collapse = 1;     // BVH8 collapse: surface-area cost programme (1) or largest child first (0)
bool collapse_cost() { return g_tune_collapse != 0; }

// The split path applies to volume-rendered scenes with one volume and no
// isovalues (the march pass keeps one sample value per lane).
static bool split_eligible(const DevScene &S) {
    return g_tune_split && S.integrate && !S.has_iso && S.n_vol == 1;
}

static unsigned grid_for(int64_t n) {
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_device);
    int64_t want = (n + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)sms * g_tune_grid_per_sm;   // grid-stride grid cap
    if (want > cap) want = cap;
    return (unsigned)(want < 1 ? 1 : want);
}

// The refill march keeps every resident warp busy until its queue is empty:
// one wave of resident blocks.
static unsigned march_grid(int minb) {
    int sms = 152, per = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_device);
    if (minb == 3) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sec_march<false, 3, 0>, kThreads, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sec_march<false, 2, 0>, kThreads, 0);
    return (unsigned)(sms * (per < 1 ? 1 : per));
}

// The march passes with or without clear-brick skipping (march_steps'
// SKIP levels): the camera-ray march skips per position whenever the scene
// has the flags; the shadow/AO march takes the lean superbrick jumps with
// GXY_TUNE_SKIP_MODE bit 1 and per-position skipping with bit 2.
// Grid of a refill kernel (it loops over its queue until the queue is
// empty): one wave of the blocks that fit on the SMs at its own register
// budget.
template <class K>
static unsigned one_wave(K kernel) {
    int sms = 152, per = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kThreads, 0);
    return (unsigned)(sms * (per < 1 ? 1 : per));
}
template <bool BATCH, int MINB>
static void launch_prim_march(cudaStream_t st, const DevScene &S, const FrameArgs &A) {
    if (S.vol[0].clear)
        k_prim_march<BATCH, MINB, 2><<<one_wave(k_prim_march<BATCH, MINB, 2>), kThreads, 0, st>>>(S, A);
    else
        k_prim_march<BATCH, MINB, 0><<<one_wave(k_prim_march<BATCH, MINB, 0>), kThreads, 0, st>>>(S, A);
}
template <bool BATCH, int MINB, bool CONT = false>
static void launch_sec_march(unsigned grid, cudaStream_t st, const DevScene &S, const FrameArgs &A) {
    if (S.vol[0].clear && (A.skip_mode & 4)) k_sec_march<BATCH, MINB, 2, CONT><<<grid, kThreads, 0, st>>>(S, A);
    else if (S.vol[0].clear && (A.skip_mode & 2)) k_sec_march<BATCH, MINB, 1, CONT><<<grid, kThreads, 0, st>>>(S, A);
    else k_sec_march<BATCH, MINB, 0, CONT><<<grid, kThreads, 0, st>>>(S, A);
}

// The shadow/AO march and the batches' camera query run at 4 resident
// blocks per SM when the tuning asks for 3 (64 registers: more warps to
// cover node-fetch and voxel-gather latency; measured faster than 80
// registers).  The frame path's queries and camera-ray march have their own
// knobs, measured on the mixed 2048^2 frame: the shadow/AO query spills at
// 64 registers and is faster at 3 blocks of 80 (GXY_TUNE_QUERY_BLOCKS;
// 4.77 -> 4.54 ms per frame), the camera and handed-off primary queries at
// 2 blocks of 128 (GXY_TUNE_PQUERY_BLOCKS; 1.39 -> 1.33 and 0.78 -> 0.63
// ms), and the camera-ray march at 2 blocks of 128 (GXY_TUNE_PMARCH_BLOCKS;
// 1.40 -> 1.36 ms).
static unsigned query_grid() {
    int sms = 152, per = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sec_query<false, 4, false>, kThreads, 0);
    return (unsigned)(sms * (per < 1 ? 1 : per));
}

// Queue memory of the frame path.  Every buffer grows to the exact worst
// case of what the next launch can write, computed from counts the host
// knows, so no ray is ever dropped for want of room: Galaxy never loses a
// ray either -- it splits an over-large list and enqueues every part
// (Renderer.cpp:674-690).  Where the worst case does not fit the HBM budget
// (or GXY_TUNE_QUEUE_LIMIT), the frame is split into bands of image rows,
// each a complete wavefront, as Galaxy splits lists.
static int g_tune_queue_limit = 0;   // records per queue buffer; 0 = none

// Grow *buf (capacity *cap records of `rec` bytes, plus `side` bytes per
// record in *aux when aux is given) to at least n records.  A buffer only
// grows; headroom of 1/8 keeps repeated frames from regrowing it.  If the
// larger buffer cannot be had, the old capacity is taken back when possible
// and GXY_ERR_OOM is returned.
static int grow(void **buf, void **aux, size_t *cap, size_t n, size_t rec, size_t side) {
    if (*cap >= n) return GXY_OK;
    if (g_tune_queue_limit && n > (size_t)g_tune_queue_limit)
        return set_error(GXY_ERR_OOM, "queue of " + std::to_string(n) + " records exceeds GXY_TUNE_QUEUE_LIMIT");
    const size_t old = *cap;
    auto release = [&]() {
        arena().free(*buf);
        *buf = nullptr;
        if (aux) {
            arena().free(*aux);
            *aux = nullptr;
        }
        *cap = 0;
    };
    auto take = [&](size_t want) -> bool {
        if (!want) return false;
        if (arena().alloc(buf, want * rec) != GXY_OK) return false;
        if (aux && side && arena().alloc(aux, want * side) != GXY_OK) {
            arena().free(*buf);
            *buf = nullptr;
            return false;
        }
        *cap = want;
        return true;
    };
    release();
    size_t want = n + n / 8 + 1024;
    if (g_tune_queue_limit && want > (size_t)g_tune_queue_limit) want = (size_t)g_tune_queue_limit;
    if (want > 0xffffffffull) want = n;
    if (n > 0xffffffffull) return set_error(GXY_ERR_INVALID, "queue too large");
    if (take(want) || take(n)) return GXY_OK;
    cudaGetLastError();
    take(old);
    return set_error(GXY_ERR_OOM, "no room for a queue of " + std::to_string(n) + " records");
}

static int grow_set(Scene *sc, int set, const size_t need[3]) {
    for (int k = 0; k < 3; k++) {
        int rc = grow((void **)&sc->q[set][k], nullptr, &sc->qcap[set][k], need[k] ? need[k] : 1, sizeof(DRay), 0);
        if (rc) return rc;
    }
    return GXY_OK;
}

// Room for a band of P pixels emitting E camera rays (per partition,
// Camera.cpp:431-441).  Its camera generation writes at most E continuing
// primaries, nl*E shadow and na*E AO rays (queue set 0) and, split, P slots
// plus one record per further partition (march records); the first hand-off
// generation at most E, 2*nl*E and 2*na*E (set 1) and (nl+na)*E march
// records.  Set 0 and the camera march records are allocated here; set 1
// and the march records only have to fit the budget (and the queue limit),
// since they grow to the counts actually queued.
static int fit_band(Scene *sc, size_t P, size_t E, int nl, int na, bool split_prim, bool split) {
    const size_t set0[3] = {E, E * (size_t)nl, E * (size_t)na};
    const size_t set1[3] = {E, 2 * E * (size_t)nl, 2 * E * (size_t)na};
    const size_t pm = P + (E > P ? E - P : 0) + 32, qm = split ? E * (size_t)(nl + na) + 32 : 0;
    if (g_tune_queue_limit) {
        const size_t lim = (size_t)g_tune_queue_limit;
        for (int k = 0; k < 3; k++)
            if (set0[k] > lim || set1[k] > lim)
                return set_error(GXY_ERR_OOM, "band exceeds GXY_TUNE_QUEUE_LIMIT");
        if ((split_prim && pm > lim) || qm > lim) return set_error(GXY_ERR_OOM, "band exceeds GXY_TUNE_QUEUE_LIMIT");
    }
    size_t extra = 0;   // bytes beyond what is allocated now
    for (int k = 0; k < 3; k++) {
        if (set0[k] > sc->qcap[0][k]) extra += (set0[k] - sc->qcap[0][k]) * sizeof(DRay);
        if (set1[k] > sc->qcap[1][k]) extra += (set1[k] - sc->qcap[1][k]) * sizeof(DRay);
    }
    if (split_prim && pm > sc->pmarch_cap) extra += (pm - sc->pmarch_cap) * (sizeof(DRay) + 2 * sizeof(float4));
    if (qm > sc->qmarch_cap) extra += (qm - sc->qmarch_cap) * (sizeof(DRay) + sizeof(float));
    if (!arena().would_fit(extra)) return set_error(GXY_ERR_OOM, "band's queues exceed the HBM budget");
    int rc = grow_set(sc, 0, set0);
    if (rc == GXY_OK && split_prim)
        rc = grow((void **)&sc->pmarch, (void **)&sc->pmarch_hit, &sc->pmarch_cap, pm, sizeof(DRay),
                  2 * sizeof(float4));
    return rc;
}

// Per image row: camera rays emitted beyond one per pixel (a ray whose entry
// point lies on a face shared by bricks is emitted by each, Camera.cpp:440-441).
__global__ void k_row_extra(DevScene S, DevCamera C, unsigned *rowx) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)C.width * C.height) return;
    V3 o, d;
    const int x = (int)(i % C.width), y = (int)(i / C.width);
    const int k = __popcll(camera_ray(S, C, x, y, o, d));
    if (k > 1) atomicAdd(rowx + y, (unsigned)(k - 1));
}

static void add_counters(DevCounters &a, const DevCounters &b) {
    const unsigned long long *pb = &b.primary;
    unsigned long long *pa = &a.primary;
    for (int k = 0; k < 15; k++) pa[k] += pb[k];
    a.overflow |= b.overflow;
}

// One frame: generation 0 from the camera, then generations of the primary
// queue and the shadow+AO queues until every queue is empty.  Each
// generation counts its output into a ring slot in device memory.  The host
// reads the counts after the camera generation and then once per block of
// up to GXY_TUNE_RUNAHEAD generations: it grows the queues the block writes
// to the block's worst case beforehand, and the block's later generations
// take their input counts from the ring (the launch grids are sized to the
// bounds).  Each launch adds into its own counter slot, and when profiling
// is on a pair of events brackets each launch, so profiling adds no syncs.
// When the camera generation's queues do not fit, the image is rendered in
// bands of rows, each band a complete wavefront into the same framebuffer.
static int render(Scene *sc, const gxy_camera &cam, const gxy_lighting &lt, float *fb, cudaStream_t st) {
    if (cam.width <= 0 || cam.height <= 0) return set_error(GXY_ERR_INVALID, "bad image size");
    DevScene &S = sc->S;
    FrameArgs A;
    memset(&A, 0, sizeof A);
    A.job0.cam = setup_camera(cam);
    int rc = setup_lights(lt, A.job0.L);
    if (rc) return rc;
    if (A.job0.L.n == 0) return set_error(GXY_ERR_INVALID, "lighting needs at least one light");
    const int W = cam.width, H = cam.height;
    const int nl = A.job0.L.shadows ? A.job0.L.n : 0, na = A.job0.L.n_ao;
    // a primary spawns shadow/AO rays only at a surface: geometry, an
    // isosurface or a slice plane
    bool spawns = S.nodes != nullptr || S.has_iso;
    for (int m = 0; m < S.n_vol; m++) spawns = spawns || S.vol[m].n_slices > 0;
    const int snl = spawns ? nl : 0, sna = spawns ? na : 0;
    const bool split = split_eligible(S), split_prim = split && g_tune_split_prim;
    const int maxl = Scene::kMaxLaunch;
    // a pair of events per launch, and the frame's start (the last)
    if (sc->profile && (int)sc->events.size() < 2 * maxl + 1) {
        for (int k = (int)sc->events.size(); k < 2 * maxl + 1; k++) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            sc->events.push_back(e);
        }
    }
    if (!sc->side) {
        CK(cudaStreamCreateWithFlags(&sc->side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&sc->fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&sc->join, cudaEventDisableTiming));
    }
    // camera rays per row: one per pixel, plus the rays a pixel emits into a
    // further partition (counted on the device when there are several)
    std::vector<unsigned> rowx(H, 0u);
    if (S.np > 1) {
        if (sc->rowx_cap < (size_t)H) {
            arena().free(sc->rowx);
            sc->rowx = nullptr;
            sc->rowx_cap = 0;
            if ((rc = arena().alloc((void **)&sc->rowx, (size_t)H * sizeof(unsigned)))) return rc;
            sc->rowx_cap = H;
        }
        CK(cudaMemsetAsync(sc->rowx, 0, (size_t)H * sizeof(unsigned), st));
        const int64_t npix = (int64_t)W * H;
        k_row_extra<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(S, A.job0.cam, sc->rowx);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(rowx.data(), sc->rowx, (size_t)H * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    // bands: the whole image if its camera generation fits, else halve
    auto band_max = [&](int rows, size_t &P, size_t &E) {
        P = (size_t)W * rows;
        E = 0;
        for (int y0 = 0; y0 < H; y0 += rows) {
            size_t e = 0;
            for (int y = y0; y < std::min(H, y0 + rows); y++) e += (size_t)W + rowx[y];
            E = std::max(E, e);
        }
    };
    int rows = H;
    for (;;) {
        size_t P, E;
        band_max(rows, P, E);
        rc = fit_band(sc, P, E, nl, na, split_prim, split);
        if (rc == GXY_OK) break;
        if (rows == 1) return set_error(GXY_ERR_OOM, "not even one image row's camera rays fit: " + last_error());
        rows = (rows + 1) / 2;
    }
    A.job0.fb = fb;
    A.job0.scene = sc->d_scene;
    A.job0.pix0 = 0;
    A.n_jobs = 1;
    A.trav_steps = g_tune_trav_steps;
    A.queue_chunk = g_tune_queue_chunk / (kThreads / 32);
    A.march_steps = g_tune_march_steps;
    A.skip_mode = g_tune_skip_mode;
    A.qmarch_count = sc->qcount + 12;   // [0] records, [1] march cursor, [2] query cursor
    A.pmarch_count = sc->qcount + 8;    // [0] records, [1] march cursor, [2] camera query cursor, [3] extra slots
    // rays_in of a launch whose input count stayed in device memory is
    // filled in from the count ring when the host reads it (slot >= 0)
    struct LaunchRec { int gen, kind; unsigned rays_in; int slot; };
    std::vector<LaunchRec> recs;
    int nl_launch = 0;
    const bool lines = S.n_seg > 0;
    sc->last = DevCounters{};
    sc->gens.clear();
    if (sc->profile) CK(cudaEventRecord(sc->events[2 * maxl], st));
    int64_t gens_total = 0;
    auto launch = [&](int kind, int gen, unsigned rays_in, int64_t items, cudaStream_t st) -> int {
        if (nl_launch >= maxl) return set_error(GXY_ERR_TIMEOUT, "too many launches in one frame");
        A.ctr = sc->ctr + nl_launch;
        unsigned g = grid_for(items);
        if (sc->profile) CK(cudaEventRecord(sc->events[2 * nl_launch], st));
        if (kind == K_SECONDARY && A.split) CK(cudaMemsetAsync(A.qmarch_count, 0, 3 * sizeof(unsigned), st));
        if ((kind == K_CAMERA && A.split_prim) || kind == K_PQUERY)
            CK(cudaMemsetAsync(A.pmarch_count, 0, 4 * sizeof(unsigned), st));
        if (g_tune_minb == 3) {
            const bool pq2 = g_tune_pquery_blocks == 2;
            if (kind == K_CAMERA && A.split_prim && g_tune_cam_packet && pq2 && lines)
                k_cam_packet<false, 2, true><<<one_wave(k_cam_packet<false, 2, true>), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA && A.split_prim && g_tune_cam_packet && pq2)
                k_cam_packet<false, 2, false><<<one_wave(k_cam_packet<false, 2, false>), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA && A.split_prim && g_tune_cam_packet && lines)
                k_cam_packet<false, 4, true><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA && A.split_prim && g_tune_cam_packet)
                k_cam_packet<false, 4, false><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA && A.split_prim && lines) k_cam_query<false, 4, true><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA && A.split_prim) k_cam_query<false, 4, false><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA) k_primary<K_CAMERA, 3><<<g, kThreads, tf_smem(S), st>>>(S, A);
            else if (kind == K_PRIMARY) k_primary<K_PRIMARY, 3><<<g, kThreads, tf_smem(S), st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && g_tune_sec_packet && lines)
                k_sec_packet<4, true><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && g_tune_sec_packet)
                k_sec_packet<4, false><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && g_tune_query_blocks == 2 && lines)
                k_sec_query<false, 2, true><<<one_wave(k_sec_query<false, 2, true>), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && g_tune_query_blocks == 2)
                k_sec_query<false, 2, false><<<one_wave(k_sec_query<false, 2, false>), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && g_tune_query_blocks == 3 && lines)
                k_sec_query<false, 3, true><<<one_wave(k_sec_query<false, 3, true>), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && g_tune_query_blocks == 3)
                k_sec_query<false, 3, false><<<one_wave(k_sec_query<false, 3, false>), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && lines) k_sec_query<false, 4, true><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split) k_sec_query<false, 4, false><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY) k_secondary<3><<<g, kThreads, tf_smem(S), st>>>(S, A);
            else if (kind == K_PMARCH && g_tune_pmarch_blocks == 2) launch_prim_march<false, 2>(st, S, A);
            else if (kind == K_PMARCH) launch_prim_march<false, 3>(st, S, A);
            else if (kind == K_PQUERY && pq2 && lines)
                k_prim_query<false, 2, true><<<one_wave(k_prim_query<false, 2, true>), kThreads, 0, st>>>(S, A);
            else if (kind == K_PQUERY && pq2)
                k_prim_query<false, 2, false><<<one_wave(k_prim_query<false, 2, false>), kThreads, 0, st>>>(S, A);
            else if (kind == K_PQUERY && lines) k_prim_query<false, 4, true><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (kind == K_PQUERY) k_prim_query<false, 4, false><<<query_grid(), kThreads, 0, st>>>(S, A);
            else if (g_tune_continue && A.qmarch_hit) launch_sec_march<false, 4, true>(query_grid(), st, S, A);
            else launch_sec_march<false, 4>(query_grid(), st, S, A);
        } else {
            if (kind == K_CAMERA && A.split_prim && g_tune_cam_packet && lines)
                k_cam_packet<false, 2, true><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA && A.split_prim && g_tune_cam_packet)
                k_cam_packet<false, 2, false><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA && A.split_prim && lines) k_cam_query<false, 2, true><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA && A.split_prim) k_cam_query<false, 2, false><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_CAMERA) k_primary<K_CAMERA, 2><<<g, kThreads, tf_smem(S), st>>>(S, A);
            else if (kind == K_PRIMARY) k_primary<K_PRIMARY, 2><<<g, kThreads, tf_smem(S), st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && g_tune_sec_packet && lines)
                k_sec_packet<2, true><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && g_tune_sec_packet)
                k_sec_packet<2, false><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split && lines) k_sec_query<false, 2, true><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY && A.split) k_sec_query<false, 2, false><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_SECONDARY) k_secondary<2><<<g, kThreads, tf_smem(S), st>>>(S, A);
            else if (kind == K_PMARCH) launch_prim_march<false, 2>(st, S, A);
            else if (kind == K_PQUERY && lines) k_prim_query<false, 2, true><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else if (kind == K_PQUERY) k_prim_query<false, 2, false><<<march_grid(2), kThreads, 0, st>>>(S, A);
            else launch_sec_march<false, 2>(march_grid(2), st, S, A);
        }
        CK(cudaGetLastError());
        if (sc->profile) CK(cudaEventRecord(sc->events[2 * nl_launch + 1], st));
        recs.push_back({gen, kind, rays_in, -1});
        nl_launch++;
        return GXY_OK;
    };
    // per-generation queue counts (generation g counts into slot g % kRing)
    unsigned *ring = sc->qcount + 16;
    auto slot = [&](int g) { return ring + 3 * (g % Scene::kRing); };
    unsigned hring[3 * Scene::kRing];
    auto read_ring = [&]() -> int {
        CK(cudaMemcpyAsync(hring, ring, sizeof hring, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (LaunchRec &r : recs) {
            if (r.slot < 0) continue;
            const unsigned *c = hring + 3 * r.slot;
            r.rays_in = (r.kind == K_PRIMARY || r.kind == K_PQUERY) ? c[Q_PRIM] : c[Q_SHADOW] + c[Q_AO];
            r.slot = -1;
        }
        return GXY_OK;
    };
    // counter slots and per-launch statistics of the launches so far
    auto collect = [&]() -> int {
        if (!nl_launch) return GXY_OK;
        for (const LaunchRec &r : recs)
            if (r.slot >= 0) {
                if (int rc2 = read_ring()) return rc2;
                break;
            }
        std::vector<DevCounters> slots(nl_launch);
        CK(cudaMemcpyAsync(slots.data(), sc->ctr, nl_launch * sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int k = 0; k < nl_launch; k++) add_counters(sc->last, slots[k]);
        if (sc->profile) {
            for (int k = 0; k < nl_launch; k++) {
                gxy_generation_stats g{};
                float ms = 0, t0 = 0;
                CK(cudaEventElapsedTime(&ms, sc->events[2 * k], sc->events[2 * k + 1]));
                CK(cudaEventElapsedTime(&t0, sc->events[2 * maxl], sc->events[2 * k]));
                g.ms = ms;
                g.start_ms = t0;
                g.generation = recs[k].gen;
                g.kind = recs[k].kind;
                g.rays_in = recs[k].kind == K_CAMERA ? 0
                            : (recs[k].kind == K_MARCH || recs[k].kind == K_PMARCH) ? (int64_t)slots[k].marched
                                                                                      : recs[k].rays_in;
                const DevCounters &c = slots[k];
                g.enqueued = (int64_t)c.enqueued;
                g.segments = (int64_t)c.segments;
                g.samples = (int64_t)c.samples;
                g.samples_skipped = (int64_t)c.skipped;
                g.nodes = (int64_t)c.nodes;
                g.tri_tests = (int64_t)c.tri_tests;
                g.sph_tests = (int64_t)c.sph_tests;
                g.terminated = (int64_t)c.terminated;
                sc->gens.push_back(g);
            }
        }
        recs.clear();
        nl_launch = 0;
        return GXY_OK;
    };
    for (int y0 = 0; y0 < H; y0 += rows) {
        A.band_y0 = y0;
        A.band_rows = std::min(rows, H - y0);
        A.total_pix = (long long)W * A.band_rows;
        A.split = split ? 1 : 0;
        A.split_prim = split_prim ? 1 : 0;
        A.qmarch = sc->qmarch;
        A.qmarch_hit = g_tune_carry_hits ? sc->qmarch_hit : nullptr;
        A.qmarch_cap = (unsigned)sc->qmarch_cap;
        A.pmarch = sc->pmarch;
        A.pmarch_hit = sc->pmarch_hit;
        A.pmarch_cap = (unsigned)sc->pmarch_cap;
        // counter slots: a band ends its launches' records before the next
        if (nl_launch > maxl - 64 && (rc = collect())) return rc;
        CK(cudaMemsetAsync(sc->ctr + nl_launch, 0, (maxl - nl_launch) * sizeof(DevCounters), st));
        CK(cudaMemsetAsync(sc->qcount, 0, (16 + 3 * Scene::kRing) * sizeof(unsigned), st));
        // generation g appends to the queue set g & 1 and counts into ring
        // slot g % kRing; the camera generation is g = 0
        for (int k = 0; k < 3; k++) {
            A.qout[k] = sc->q[0][k];
            A.qcap[k] = (unsigned)sc->qcap[0][k];
        }
        A.qout_count = slot(0);
        A.nin_dev = nullptr;
        if ((rc = launch(K_CAMERA, 0, 0, A.total_pix, st))) return rc;
        if (A.split_prim && (rc = launch(K_PMARCH, 0, 0, 1 << 30, st))) return rc;
        A.split_prim = 0;   // later generations trace handed-off primaries in one pass
        if ((rc = read_ring())) return rc;
        int gen = 1, cur = 0;   // cur: the queue set the last generation wrote
        unsigned n[3];
        for (int k = 0; k < 3; k++) n[k] = hring[k];
        for (;;) {
            for (int k = 0; k < 3; k++)
                if (n[k] > sc->qcap[cur][k]) n[k] = (unsigned)sc->qcap[cur][k];   // overflow already flagged
            if (n[0] + n[1] + n[2] == 0) break;
            const int nxt = cur ^ 1;
            // worst case of the j-th output from here: a primary continues
            // at most once per generation and spawns nl shadow and na AO
            // rays; a shadow/AO ray moves on at most once
            auto need = [&](int j, size_t out[3]) {
                out[Q_PRIM] = n[Q_PRIM];
                out[Q_SHADOW] = (size_t)n[Q_SHADOW] + (size_t)j * snl * n[Q_PRIM];
                out[Q_AO] = (size_t)n[Q_AO] + (size_t)j * sna * n[Q_PRIM];
            };
            auto fits = [&](int set, int j) {
                size_t w[3];
                need(j, w);
                for (int k = 0; k < 3; k++)
                    if (w[k] > sc->qcap[set][k]) return false;
                return true;
            };
            const size_t sa = (size_t)n[Q_SHADOW] + n[Q_AO], fan = (size_t)(snl + sna) * n[Q_PRIM];
            // A block runs to the generation count of the scene's previous
            // frame (at most GXY_TUNE_RUNAHEAD generations), so a repeated
            // view launches no generation without rays; a frame that outlasts
            // it goes on one generation per read.  The block writes its odd
            // outputs (1, 3, ...) to set nxt and its even ones to set cur.
            // Set cur holds the rays the block starts from, so it cannot
            // grow: the block ends before an even output that would not fit
            // there.  Set nxt and the march queue then grow to the block's
            // worst case; if they cannot, the block is one generation.
            const int kcap = sc->bounces > gen ? (int)std::min<int64_t>(g_tune_runahead, sc->bounces - gen) : 1;
            int K = 1;
            while (K < kcap && (((K + 1) & 1) || fits(cur, K + 1))) K++;
            size_t w[3];
            need((K & 1) ? K : K - 1, w);
            int grc = grow_set(sc, nxt, w);
            if (grc && K > 1) {
                cudaGetLastError();
                K = 1;
                need(1, w);
                grc = grow_set(sc, nxt, w);
            }
            const bool split_handoff = split_prim && g_tune_split_handoff && n[Q_PRIM];
            if (grc == GXY_OK && A.split) {
                grc = grow((void **)&sc->qmarch, (void **)&sc->qmarch_hit, &sc->qmarch_cap, sa + (K - 1) * fan + 32,
                           sizeof(DRay), sizeof(float));
                if (grc && K > 1) {
                    cudaGetLastError();
                    K = 1;
                    grc = grow((void **)&sc->qmarch, (void **)&sc->qmarch_hit, &sc->qmarch_cap, sa + 32, sizeof(DRay),
                               sizeof(float));
                }
            }
            if (grc == GXY_OK && split_handoff)
                grc = grow((void **)&sc->pmarch, (void **)&sc->pmarch_hit, &sc->pmarch_cap, (size_t)n[Q_PRIM] + 32,
                           sizeof(DRay), 2 * sizeof(float4));
            // a queue that cannot grow keeps its room; a generation that then
            // runs out of it reports GXY_ERR_OVERFLOW
            if (grc) {
                cudaGetLastError();
                K = 1;
            }
            A.pmarch = sc->pmarch;
            A.pmarch_hit = sc->pmarch_hit;
            A.pmarch_cap = (unsigned)sc->pmarch_cap;
            A.qmarch = sc->qmarch;
            A.qmarch_hit = g_tune_carry_hits ? sc->qmarch_hit : nullptr;
            A.qmarch_cap = (unsigned)sc->qmarch_cap;
            for (int j = 0; j < K; j++) {
                const int g = gen + j, in = (j & 1) ? nxt : cur, out = in ^ 1;
                // upper bounds of this generation's inputs (exact for j = 0)
                const unsigned np = n[Q_PRIM];
                const size_t nsa = sa + (size_t)j * fan;
                CK(cudaMemsetAsync(slot(g), 0, 3 * sizeof(unsigned), st));
                for (int k = 0; k < 3; k++) {
                    A.qin[k] = sc->q[in][k];
                    A.nin[k] = j ? (unsigned)sc->qcap[in][k] : n[k];
                    A.qout[k] = sc->q[out][k];
                    A.qcap[k] = (unsigned)sc->qcap[out][k];
                }
                A.nin_dev = j ? slot(g - 1) : nullptr;
                A.qout_count = slot(g);
                // Continuing primaries and shadow/AO rays of one generation are
                // independent (both only append to the next generation's queues), so
                // the primaries, whose launch is bound by its longest march, run on
                // the side stream beside the shadow/AO passes.
                const bool sec = nsa != 0;
                const bool overlap = np && sec;
                if (nl_launch + 4 > maxl && (rc = collect())) return rc;
                const int first = nl_launch;
                if (overlap) {
                    CK(cudaEventRecord(sc->fork, st));
                    CK(cudaStreamWaitEvent(sc->side, sc->fork, 0));
                }
                if (np && split_handoff) {
                    if ((rc = launch(K_PQUERY, g, np, np, overlap ? sc->side : st))) return rc;
                    if ((rc = launch(K_PMARCH, g, 0, 1 << 30, overlap ? sc->side : st))) return rc;
                } else if (np && (rc = launch(K_PRIMARY, g, np, np, overlap ? sc->side : st))) {
                    return rc;
                }
                if (overlap) CK(cudaEventRecord(sc->join, sc->side));
                if (sec && (rc = launch(K_SECONDARY, g, (unsigned)std::min<size_t>(nsa, 0xffffffffu), (int64_t)nsa, st)))
                    return rc;
                if (sec && A.split && (rc = launch(K_MARCH, g, 0, 1 << 30, st))) return rc;
                if (overlap) CK(cudaStreamWaitEvent(st, sc->join, 0));
                if (j)
                    for (int k = first; k < nl_launch; k++)
                        if (recs[k].kind != K_PMARCH && recs[k].kind != K_MARCH) recs[k].slot = (g - 1) % Scene::kRing;
            }
            // one read of the counts per block
            if ((rc = read_ring())) return rc;
            int done = K;   // generations of the block that had input
            for (int j = 0; j < K; j++) {
                const unsigned *c = hring + 3 * ((gen + j) % Scene::kRing);
                if (c[0] + c[1] + c[2] == 0) {
                    done = j + 1;
                    break;
                }
            }
            const unsigned *c = hring + 3 * ((gen + done - 1) % Scene::kRing);
            for (int k = 0; k < 3; k++) n[k] = c[k];
            cur = (done & 1) ? nxt : cur;
            gen += done;
        }
        gens_total = std::max<int64_t>(gens_total, gen);
    }
    if ((rc = collect())) return rc;
    sc->bounces = gens_total;
    sc->bands = (H + rows - 1) / rows;
    if (sc->last.overflow) return set_error(GXY_ERR_OVERFLOW, "a ray queue or traversal stack overflowed");
    return GXY_OK;
}

// ------------------------------------------------- RayList host plumbing
struct DevRayList {
    RLDev d{};
    std::vector<void *> bufs;
    ~DevRayList() {
        for (void *p : bufs) arena().free(p);
    }
    int alloc(int n) {
        d.n = n;
        size_t cnt = n > 0 ? (size_t)n : 1;
        for (int k = 0; k < 20; k++) {
            int rc = arena().alloc((void **)&d.f[k], cnt * sizeof(float));
            if (rc) return rc;
            bufs.push_back(d.f[k]);
        }
        for (int k = 0; k < 5; k++) {
            int rc = arena().alloc((void **)&d.i[k], cnt * sizeof(int32_t));
            if (rc) return rc;
            bufs.push_back(d.i[k]);
        }
        return GXY_OK;
    }
};
static float *const *host_f(const gxy_raylist &r, float **tmp) {
    float *f[20] = {r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.nx, r.ny, r.nz, r.sample,
                    r.r, r.g, r.b, r.o, r.sr, r.sg, r.sb, r.so, r.t, r.tMax};
    for (int k = 0; k < 20; k++) tmp[k] = f[k];
    return tmp;
}
static int32_t *const *host_i(const gxy_raylist &r, int32_t **tmp) {
    int32_t *v[5] = {r.x, r.y, r.type, r.term, r.classification};
    for (int k = 0; k < 5; k++) tmp[k] = v[k];
    return tmp;
}
static int rl_upload(const gxy_raylist &h, DevRayList &d, int n) {
    float *hf[20];
    int32_t *hi[5];
    host_f(h, hf);
    host_i(h, hi);
    for (int k = 0; k < 20; k++) {
        if (hf[k]) CK(cudaMemcpy(d.d.f[k], hf[k], n * sizeof(float), cudaMemcpyHostToDevice));
        else CK(cudaMemset(d.d.f[k], 0, n * sizeof(float)));
    }
    for (int k = 0; k < 5; k++) {
        if (hi[k]) CK(cudaMemcpy(d.d.i[k], hi[k], n * sizeof(int32_t), cudaMemcpyHostToDevice));
        else CK(cudaMemset(d.d.i[k], 0, n * sizeof(int32_t)));
    }
    return GXY_OK;
}
static int rl_download(const DevRayList &d, gxy_raylist &h, int n) {
    float *hf[20];
    int32_t *hi[5];
    host_f(h, hf);
    host_i(h, hi);
    for (int k = 0; k < 20; k++)
        if (hf[k] && n) CK(cudaMemcpy(hf[k], d.d.f[k], n * sizeof(float), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 5; k++)
        if (hi[k] && n) CK(cudaMemcpy(hi[k], d.d.i[k], n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return GXY_OK;
}

}  // namespace gxy

using namespace gxy;

// ================================================================== C ABI
#define GUARD_BEGIN try {
#define GUARD_END                                                       \
    }                                                                   \
    catch (const std::exception &e) {                                   \
        return set_error(GXY_ERR_INVALID, std::string("exception: ") + e.what()); \
    }                                                                   \
    catch (...) {                                                       \
        return set_error(GXY_ERR_INVALID, "unknown exception");         \
    }

extern "C" {

int gxy_gpu_init(int device, size_t hbm_budget_bytes) {
    GUARD_BEGIN
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return set_error(GXY_ERR_INVALID, "no such device");
    CK(cudaSetDevice(device));
    g_device = device;
    arena().set_budget(hbm_budget_bytes);
    g_init = true;
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_shutdown(void) {
    GUARD_BEGIN
    if (g_init) cudaDeviceSynchronize();
    g_init = false;
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_last_error(char *buf, int buflen) {
    if (!buf || buflen <= 0) return GXY_ERR_INVALID;
    snprintf(buf, (size_t)buflen, "%s", last_error().c_str());
    return GXY_OK;
}

int gxy_gpu_hbm_in_use(size_t *bytes) {
    if (!bytes) return GXY_ERR_INVALID;
    *bytes = arena().in_use();
    return GXY_OK;
}

int gxy_gpu_scene_commit(const gxy_scene_desc *desc, gxy_scene *out) {
    GUARD_BEGIN
    if (!g_init) return set_error(GXY_ERR_NOT_INIT, "gxy_gpu_init not called");
    if (!desc || !out) return set_error(GXY_ERR_INVALID, "null argument");
    std::unique_ptr<Scene> sc(new Scene());
    int rc = commit(desc, sc.get());
    if (rc) return rc;
    *out = reinterpret_cast<gxy_scene>(sc.release());
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_scene_release(gxy_scene scene) {
    GUARD_BEGIN
    if (!scene) return set_error(GXY_ERR_INVALID, "null scene");
    cudaDeviceSynchronize();
    delete reinterpret_cast<Scene *>(scene);
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_scene_set_tf(gxy_scene scene, int vis_kind, int index, const gxy_tf *tf, void *stream) {
    GUARD_BEGIN
    if (!scene || !tf) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    std::lock_guard<std::mutex> lk(sc->mu);
    return scene_set_tf(sc, vis_kind, index, *tf, (cudaStream_t)stream);
    GUARD_END
}

int gxy_gpu_scene_view(gxy_scene scene, gxy_scene *out) {
    GUARD_BEGIN
    if (!scene || !out) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *base = reinterpret_cast<Scene *>(scene);
    std::unique_ptr<Scene> v(new Scene());
    {
        std::lock_guard<std::mutex> lk(base->mu);
        int rc = scene_view(base, v.get());
        if (rc) return rc;
    }
    *out = reinterpret_cast<gxy_scene>(v.release());
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_scene_partition_info(gxy_scene scene, int partition, gxy_partition_info *out) {
    if (!scene || !out) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    if (partition < 0 || partition >= sc->S.np) return set_error(GXY_ERR_INVALID, "bad partition");
    const DevPartition &P = sc->S.part[partition];
    for (int a = 0; a < 3; a++) {
        out->global_box[a] = sc->S.glo[a];
        out->global_box[3 + a] = sc->S.ghi[a];
        out->local_box[a] = P.lo[a];
        out->local_box[3 + a] = P.hi[a];
    }
    for (int k = 0; k < 6; k++) out->neighbors[k] = P.nb[k];
    out->n_partitions = sc->S.np;
    return GXY_OK;
}

int gxy_scene_partition_layout(const gxy_scene_desc *desc, int partition, gxy_partition_info *out) {
    GUARD_BEGIN
    if (!desc || !out) return set_error(GXY_ERR_INVALID, "null argument");
    int rc = check_partition_extents(*desc);
    if (rc) return rc;
    int np = desc_partition_count(*desc);
    if (np > kMaxPart || partition < 0 || partition >= np) return set_error(GXY_ERR_INVALID, "bad partition");
    // geometry box as the commit computes it
    std::vector<float> g = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    bool any = false;
    for (int s = 0; s < desc->n_triangle_sets; s++) {
        const gxy_triangles_vis &t = desc->triangles[s];
        for (int64_t i = 0; i < t.n_vertices; i++)
            for (int a = 0; a < 3; a++) {
                g[a] = fminf(g[a], t.vertices[3 * i + a]);
                g[3 + a] = fmaxf(g[3 + a], t.vertices[3 * i + a]);
                any = true;
            }
    }
    for (int s = 0; s < desc->n_particle_sets; s++) {
        const gxy_particles_vis &q = desc->particles[s];
        for (int64_t i = 0; i < q.n; i++) {
            float r = sphere_radius(q, i);
            for (int a = 0; a < 3; a++) {
                g[a] = fminf(g[a], q.centers[3 * i + a] - r);
                g[3 + a] = fmaxf(g[3 + a], q.centers[3 * i + a] + r);
                any = true;
            }
        }
    }
    if (desc->n_pathline_sets < 0 || desc->n_pathline_sets > 4) return set_error(GXY_ERR_INVALID, "bad path-line set count");
    for (int s = 0; s < desc->n_pathline_sets; s++) {
        const gxy_pathlines_vis &q = desc->pathlines[s];
        for (int64_t i = 0; i < q.n_vertices; i++) {
            float r = pathline_radius(q, i);
            for (int a = 0; a < 3; a++) {
                g[a] = fminf(g[a], q.vertices[3 * i + a] - r);
                g[3 + a] = fmaxf(g[3 + a], q.vertices[3 * i + a] + r);
                any = true;
            }
        }
    }
    if (desc->has_box) g.assign(desc->box, desc->box + 6);
    else if (!any) g = {-1, -1, -1, 1, 1, 1};
    DevScene S;
    memset(&S, 0, sizeof S);
    make_partitions(*desc, g, S);
    const DevPartition &P = S.part[partition];
    for (int a = 0; a < 3; a++) {
        out->global_box[a] = S.glo[a];
        out->global_box[3 + a] = S.ghi[a];
        out->local_box[a] = P.lo[a];
        out->local_box[3 + a] = P.hi[a];
    }
    for (int k = 0; k < 6; k++) out->neighbors[k] = P.nb[k];
    out->n_partitions = S.np;
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_scene_bvh_info(gxy_scene scene, int64_t *n_nodes, int64_t *n_prim_refs, double *build_ms) {
    if (!scene) return set_error(GXY_ERR_INVALID, "null scene");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    if (n_nodes) *n_nodes = sc->bvh.n_nodes;
    if (n_prim_refs) *n_prim_refs = sc->bvh.n_slots;
    if (build_ms) *build_ms = sc->bvh.build_ms;
    return GXY_OK;
}

int gxy_resolve_lights(const gxy_lighting *in, const gxy_camera *camera, gxy_lighting *out) {
    if (!in || !camera || !out) return set_error(GXY_ERR_INVALID, "null argument");
    // Rendering::resolve_lights (Rendering.cpp:157-216)
    F3h vp = h3(camera->eye[0], camera->eye[1], camera->eye[2]);
    F3h vu = gnorm(h3(camera->up[0], camera->up[1], camera->up[2]));
    F3h vd = gnorm(h3(camera->dir[0], camera->dir[1], camera->dir[2]));
    F3h right = gnorm(hcross(vd, vu));
    F3h up = hcross(vd, right);
    gxy_lighting r = *in;
    for (int i = 0; i < in->n_lights && i < GXY_MAX_LIGHTS; i++) {
        if (in->types[i] == GXY_LIGHT_CAMERA) {
            const float *l = in->lights[i];
            F3h p = hadd(hadd(hadd(vp, hmul(l[0], right)), hmul(l[1], up)), hmul(l[2], vd));
            r.lights[i][0] = p.x; r.lights[i][1] = p.y; r.lights[i][2] = p.z;
            r.types[i] = GXY_LIGHT_POINT;
        }
    }
    *out = r;
    return GXY_OK;
}

int gxy_gpu_render(gxy_scene scene, const gxy_camera *camera, const gxy_lighting *lighting, float *fb_rgba,
                   void *stream) {
    GUARD_BEGIN
    if (!scene || !camera || !lighting || !fb_rgba) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    std::lock_guard<std::mutex> lk(sc->mu);
    return render(sc, *camera, *lighting, fb_rgba, (cudaStream_t)stream);
    GUARD_END
}

int gxy_gpu_render_host(gxy_scene scene, const gxy_camera *camera, const gxy_lighting *lighting,
                        float *host_fb_rgba, void *stream) {
    GUARD_BEGIN
    if (!scene || !camera || !lighting || !host_fb_rgba) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    std::lock_guard<std::mutex> lk(sc->mu);
    cudaStream_t st = (cudaStream_t)stream;
    size_t elems = (size_t)camera->width * camera->height * 4;
    if (sc->fbtmp_elems < elems) {
        arena().free(sc->fbtmp);
        sc->fbtmp = nullptr;
        sc->fbtmp_elems = 0;
        int rc = arena().alloc((void **)&sc->fbtmp, elems * sizeof(float));
        if (rc) return rc;
        sc->fbtmp_elems = elems;
    }
    CK(cudaMemsetAsync(sc->fbtmp, 0, elems * sizeof(float), st));
    int rc = render(sc, *camera, *lighting, sc->fbtmp, st);
    if (rc) return rc;
    CK(cudaMemcpyAsync(host_fb_rgba, sc->fbtmp, elems * sizeof(float), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_query_counters(gxy_scene scene, gxy_counters *out) {
    if (!scene || !out) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    const DevCounters &c = sc->last;
    memset(out, 0, sizeof *out);
    out->primary_rays = (int64_t)c.primary;
    out->shadow_rays = (int64_t)c.shadow;
    out->ao_rays = (int64_t)c.ao;
    out->secondary_rays = (int64_t)(c.shadow + c.ao);
    out->segments = (int64_t)c.segments;
    out->handoffs = (int64_t)c.handoffs;
    out->terminated = (int64_t)c.terminated;
    out->dropped = (int64_t)c.dropped;
    out->kept = (int64_t)c.kept;
    out->bounces = sc->bounces;
    out->samples = (int64_t)c.samples;
    out->nodes = (int64_t)c.nodes;
    out->prim_tests = (int64_t)(c.tri_tests + c.sph_tests);
    out->overflow = c.overflow;
    out->samples_skipped = (int64_t)c.skipped;
    out->bands = sc->bands;
    return GXY_OK;
}

// extra counters for the roofline: triangle and sphere tests, queue records written
int gxy_gpu_query_counters_ex(gxy_scene scene, int64_t *tri_tests, int64_t *sph_tests, int64_t *enqueued) {
    if (!scene) return set_error(GXY_ERR_INVALID, "null scene");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    if (tri_tests) *tri_tests = (int64_t)sc->last.tri_tests;
    if (sph_tests) *sph_tests = (int64_t)sc->last.sph_tests;
    if (enqueued) *enqueued = (int64_t)sc->last.enqueued;
    return GXY_OK;
}

int gxy_gpu_set_tuning(int knob, int value) {
    if (knob == GXY_TUNE_BLOCKS_PER_SM) {
        if (value != 2 && value != 3) return set_error(GXY_ERR_INVALID, "blocks per SM must be 2 or 3");
        g_tune_minb = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_GRID_PER_SM) {
        if (value < 1 || value > 64) return set_error(GXY_ERR_INVALID, "grid blocks per SM must be 1..64");
        g_tune_grid_per_sm = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_SPLIT_SECONDARY) {
        g_tune_split = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_SPLIT_PRIMARY) {
        g_tune_split_prim = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_BVH_SAH) {
        if (value < 0 || value > (1 << 20)) return set_error(GXY_ERR_INVALID, "bad SAH cluster size");
        g_tune_sah = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_LEAF_MAX) {
        if (value < 1 || value > 4) return set_error(GXY_ERR_INVALID, "leaf size must be 1-4");
        g_tune_leaf = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_CAMERA_PACKET) {
        g_tune_cam_packet = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_TRAV_STEPS) {
        if (value < 1 || value > 64) return set_error(GXY_ERR_INVALID, "traversal steps must be 1-64");
        g_tune_trav_steps = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_MARCH_STEPS) {
        if (value < 1 || value > 256) return set_error(GXY_ERR_INVALID, "march steps must be 1-256");
        g_tune_march_steps = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_SKIP_CLEAR) {
        g_tune_skip_clear = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_CARRY_HITS) {
        g_tune_carry_hits = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_SKIP_MODE) {
        if (value < 0 || value > 15) return set_error(GXY_ERR_INVALID, "skip mode must be 0-15");
        g_tune_skip_mode = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_BVH_COLLAPSE) {
        g_tune_collapse = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_SEC_PACKET) {
        g_tune_sec_packet = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_RUNAHEAD) {
        if (value < 1 || value > 16) return set_error(GXY_ERR_INVALID, "run-ahead must be 1-16 generations");
        g_tune_runahead = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_SPLIT_HANDOFF) {
        g_tune_split_handoff = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_QUERY_BLOCKS) {
        if (value < 2 || value > 4) return set_error(GXY_ERR_INVALID, "query blocks per SM must be 2, 3 or 4");
        g_tune_query_blocks = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_CONTINUE) {
        g_tune_continue = value ? 1 : 0;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_PQUERY_BLOCKS) {
        if (value != 2 && value != 4) return set_error(GXY_ERR_INVALID, "primary query blocks per SM must be 2 or 4");
        g_tune_pquery_blocks = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_PMARCH_BLOCKS) {
        if (value != 2 && value != 3) return set_error(GXY_ERR_INVALID, "march blocks per SM must be 2 or 3");
        g_tune_pmarch_blocks = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_QUEUE_CHUNK) {
        if (value != 0 && (value < 256 || value > 65536))
            return set_error(GXY_ERR_INVALID, "queue chunk must be 0 or 256-65536 records");
        g_tune_queue_chunk = value;
        return GXY_OK;
    }
    if (knob == GXY_TUNE_QUEUE_LIMIT) {
        if (value < 0) return set_error(GXY_ERR_INVALID, "queue limit must be >= 0");
        g_tune_queue_limit = value;
        return GXY_OK;
    }
    return set_error(GXY_ERR_INVALID, "unknown tuning knob");
}

int gxy_gpu_get_tuning(int knob, int *value) {
    if (!value) return set_error(GXY_ERR_INVALID, "null argument");
    if (knob == GXY_TUNE_BLOCKS_PER_SM) *value = g_tune_minb;
    else if (knob == GXY_TUNE_GRID_PER_SM) *value = g_tune_grid_per_sm;
    else if (knob == GXY_TUNE_SPLIT_SECONDARY) *value = g_tune_split;
    else if (knob == GXY_TUNE_SPLIT_PRIMARY) *value = g_tune_split_prim;
    else if (knob == GXY_TUNE_BVH_SAH) *value = g_tune_sah;
    else if (knob == GXY_TUNE_LEAF_MAX) *value = g_tune_leaf;
    else if (knob == GXY_TUNE_TRAV_STEPS) *value = g_tune_trav_steps;
    else if (knob == GXY_TUNE_CAMERA_PACKET) *value = g_tune_cam_packet;
    else if (knob == GXY_TUNE_MARCH_STEPS) *value = g_tune_march_steps;
    else if (knob == GXY_TUNE_SKIP_CLEAR) *value = g_tune_skip_clear;
    else if (knob == GXY_TUNE_SKIP_MODE) *value = g_tune_skip_mode;
    else if (knob == GXY_TUNE_CARRY_HITS) *value = g_tune_carry_hits;
    else if (knob == GXY_TUNE_QUEUE_LIMIT) *value = g_tune_queue_limit;
    else if (knob == GXY_TUNE_QUEUE_CHUNK) *value = g_tune_queue_chunk;
    else if (knob == GXY_TUNE_SPLIT_HANDOFF) *value = g_tune_split_handoff;
    else if (knob == GXY_TUNE_SEC_PACKET) *value = g_tune_sec_packet;
    else if (knob == GXY_TUNE_BVH_COLLAPSE) *value = g_tune_collapse;
    else if (knob == GXY_TUNE_RUNAHEAD) *value = g_tune_runahead;
    else if (knob == GXY_TUNE_QUERY_BLOCKS) *value = g_tune_query_blocks;
    else if (knob == GXY_TUNE_PMARCH_BLOCKS) *value = g_tune_pmarch_blocks;
    else if (knob == GXY_TUNE_PQUERY_BLOCKS) *value = g_tune_pquery_blocks;
    else if (knob == GXY_TUNE_CONTINUE) *value = g_tune_continue;
    else return set_error(GXY_ERR_INVALID, "unknown tuning knob");
    return GXY_OK;
}

int gxy_tf_clear_below(const gxy_tf *tf, float *threshold) {
    if (!tf || !threshold) return set_error(GXY_ERR_INVALID, "null argument");
    DevTF t;
    tf_to_dev(*tf, t);
    *threshold = tf_clear_below(t);
    return GXY_OK;
}

int gxy_gpu_set_profiling(gxy_scene scene, int on) {
    if (!scene) return set_error(GXY_ERR_INVALID, "null scene");
    reinterpret_cast<Scene *>(scene)->profile = on ? 1 : 0;
    return GXY_OK;
}

int gxy_gpu_query_generations(gxy_scene scene, gxy_generation_stats *out, int max, int32_t *n) {
    if (!scene || !n || (max > 0 && !out)) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    int k = (int)sc->gens.size();
    *n = k;
    for (int i = 0; i < k && i < max; i++) out[i] = sc->gens[i];
    return GXY_OK;
}

int gxy_gpu_generate_initial_rays(gxy_scene scene, int partition, const gxy_camera *camera, gxy_raylist *out,
                                  int32_t *n_out) {
    GUARD_BEGIN
    if (!scene || !camera || !out || !n_out) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    if (partition < 0 || partition >= sc->S.np) return set_error(GXY_ERR_INVALID, "bad partition");
    DevCamera C = setup_camera(*camera);
    int64_t n = (int64_t)camera->width * camera->height;
    if (n <= 0 || n > 0x7fffffff) return set_error(GXY_ERR_INVALID, "bad image size");
    ScratchList tmp(arena());
    int *flag, *pos;
    int rc;
    if ((rc = tmp.alloc((void **)&flag, n * sizeof(int)))) return rc;
    if ((rc = tmp.alloc((void **)&pos, n * sizeof(int)))) return rc;
    unsigned g = (unsigned)((n + 255) / 256);
    k_rl_camera_flags<<<g, 256>>>(sc->S, C, partition, flag);
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, flag, pos, (int)n);
    void *tv;
    if ((rc = tmp.alloc(&tv, tb))) return rc;
    CK(cub::DeviceScan::ExclusiveSum(tv, tb, flag, pos, (int)n));
    int last_pos = 0, last_flag = 0;
    CK(cudaMemcpy(&last_pos, pos + n - 1, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&last_flag, flag + n - 1, sizeof(int), cudaMemcpyDeviceToHost));
    int total = last_pos + last_flag;
    *n_out = total;
    if (total > out->n) return set_error(GXY_ERR_OVERFLOW, "output RayList too small");
    DevRayList O;
    if ((rc = O.alloc(total))) return rc;
    for (int k = 0; k < 20; k++) CK(cudaMemset(O.d.f[k], 0, (total ? total : 1) * sizeof(float)));
    for (int k = 0; k < 5; k++) CK(cudaMemset(O.d.i[k], 0, (total ? total : 1) * sizeof(int32_t)));
    k_rl_camera_write<<<g, 256>>>(sc->S, C, partition, flag, pos, O.d);
    CK(cudaGetLastError());
    return rl_download(O, *out, total);
    GUARD_END
}

int gxy_gpu_trace_raylist(gxy_scene scene, int partition, const gxy_lighting *lighting, gxy_raylist *in,
                          gxy_raylist *out, int32_t *n_out) {
    GUARD_BEGIN
    if (!scene || !lighting || !in || !n_out) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    if (partition < 0 || partition >= sc->S.np) return set_error(GXY_ERR_INVALID, "bad partition");
    DevLights L;
    int rc = setup_lights(*lighting, L);
    if (rc) return rc;
    int n = in->n;
    if (n < 0) return set_error(GXY_ERR_INVALID, "negative ray count");
    *n_out = 0;
    if (n == 0) return GXY_OK;
    DevRayList R;
    if ((rc = R.alloc(n))) return rc;
    if ((rc = rl_upload(*in, R, n))) return rc;
    CK(cudaMemset(sc->ctr, 0, sizeof(DevCounters)));
    unsigned g = (unsigned)((n + 255) / 256);
    k_rl_trace<<<g, 256>>>(sc->S, partition, R.d, sc->ctr);
    CK(cudaGetLastError());
    ScratchList tmp(arena());
    int *cnt, *off;
    if ((rc = tmp.alloc((void **)&cnt, 2 * (size_t)n * sizeof(int)))) return rc;
    if ((rc = tmp.alloc((void **)&off, 2 * (size_t)n * sizeof(int)))) return rc;
    int n_sh = L.shadows ? L.n : 0;
    k_rl_counts<<<g, 256>>>(R.d, L.n_ao, n_sh, cnt);
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt, off, n);
    void *tv;
    if ((rc = tmp.alloc(&tv, tb))) return rc;
    CK(cub::DeviceScan::ExclusiveSum(tv, tb, cnt, off, n));
    CK(cub::DeviceScan::ExclusiveSum(tv, tb, cnt + n, off + n, n));
    int la[4];
    CK(cudaMemcpy(&la[0], off + n - 1, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&la[1], cnt + n - 1, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&la[2], off + 2 * n - 1, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&la[3], cnt + 2 * n - 1, sizeof(int), cudaMemcpyDeviceToHost));
    int ao_total = la[0] + la[1], sh_total = la[2] + la[3];
    int total = ao_total + sh_total;
    DevRayList O;
    if ((rc = O.alloc(total))) return rc;
    for (int k = 0; k < 20; k++) CK(cudaMemset(O.d.f[k], 0, (total ? total : 1) * sizeof(float)));
    for (int k = 0; k < 5; k++) CK(cudaMemset(O.d.i[k], 0, (total ? total : 1) * sizeof(int32_t)));
    k_rl_shade<<<g, 256>>>(sc->S, L, R.d, O.d, off, ao_total);
    CK(cudaGetLastError());
    if ((rc = rl_download(R, *in, n))) return rc;
    DevCounters c;
    CK(cudaMemcpy(&c, sc->ctr, sizeof c, cudaMemcpyDeviceToHost));
    if (c.overflow) return set_error(GXY_ERR_OVERFLOW, "BVH traversal stack overflowed");
    *n_out = total;
    if (total) {
        if (!out || total > out->n) return set_error(GXY_ERR_OVERFLOW, "secondary RayList too small");
        if ((rc = rl_download(O, *out, total))) return rc;
    }
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_classify(gxy_raylist *rays) {
    GUARD_BEGIN
    if (!rays || rays->n < 0) return set_error(GXY_ERR_INVALID, "bad RayList");
    int n = rays->n;
    if (!n) return GXY_OK;
    DevRayList R;
    int rc;
    if ((rc = R.alloc(n))) return rc;
    if ((rc = rl_upload(*rays, R, n))) return rc;
    k_rl_classify<<<(n + 255) / 256, 256>>>(R.d);
    CK(cudaGetLastError());
    CK(cudaMemcpy(rays->classification, R.d.i[I_CLS], n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_assign_destinations(gxy_scene scene, int partition, gxy_raylist *rays) {
    GUARD_BEGIN
    if (!scene || !rays || rays->n < 0) return set_error(GXY_ERR_INVALID, "bad argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    if (partition < 0 || partition >= sc->S.np) return set_error(GXY_ERR_INVALID, "bad partition");
    int n = rays->n;
    if (!n) return GXY_OK;
    DevRayList R;
    int rc;
    if ((rc = R.alloc(n))) return rc;
    if ((rc = rl_upload(*rays, R, n))) return rc;
    k_rl_assign<<<(n + 255) / 256, 256>>>(sc->S, partition, R.d);
    CK(cudaGetLastError());
    CK(cudaMemcpy(rays->classification, R.d.i[I_CLS], n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_accumulate_terminated(const gxy_raylist *rays, float *fb_rgba, int width, int height) {
    GUARD_BEGIN
    if (!rays || !fb_rgba || width <= 0 || height <= 0 || rays->n < 0)
        return set_error(GXY_ERR_INVALID, "bad argument");
    int n = rays->n;
    if (!n) return GXY_OK;
    DevRayList R;
    int rc;
    if ((rc = R.alloc(n))) return rc;
    if ((rc = rl_upload(*rays, R, n))) return rc;
    ScratchList tmp(arena());
    float *fb;
    size_t bytes = (size_t)width * height * 4 * sizeof(float);
    if ((rc = tmp.alloc((void **)&fb, bytes))) return rc;
    CK(cudaMemcpy(fb, fb_rgba, bytes, cudaMemcpyHostToDevice));
    k_rl_accumulate<<<(n + 255) / 256, 256>>>(R.d, fb, width, height);
    CK(cudaGetLastError());
    CK(cudaMemcpy(fb_rgba, fb, bytes, cudaMemcpyDeviceToHost));
    return GXY_OK;
    GUARD_END
}

}  // extern "C"

// ================================================================ batches
namespace gxy {

struct Batch {
    int64_t max_pixels = 0;
    int max_jobs = 0, max_shadow = 0, max_ao = 0;
    DRay *q[2][NQ] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    size_t qcap[NQ] = {0, 0, 0};
    unsigned *counts = nullptr;        // kMaxGen x NQ (cooperative mode uses the first 3 x NQ)
    unsigned *mcounts = nullptr;       // kBatchGens x 4: march records, march cursor (split path); then 4 for
                                       // the camera march and kBatchGens x 4 for handed-off primaries
    DRay *qmarch = nullptr;
    float *qmarch_hit = nullptr;       // per march record: the query's closest hit (carried hits)
    size_t qmarch_cap = 0;
    DRay *pmarch = nullptr;            // split camera rays (uniform-scene batches)
    float4 *pmarch_hit = nullptr;
    size_t pmarch_cap = 0;
    DevJob *d_jobs = nullptr;
    DevJob *h_jobs = nullptr;          // pinned
    DevCounters *ctr = nullptr;
    int *d_status = nullptr, *h_status = nullptr;   // pinned host copy of [gens, left]
    DevCounters *h_ctr = nullptr;                   // pinned
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;       // continuing primaries beside the shadow/AO passes
    cudaEvent_t fork[16] = {}, join[16] = {};   // per generation
    cudaEvent_t done = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int grid = 0;
    bool pending = false;
    int cooperative = 0;
    int last_rc = GXY_OK;
    // the last submission, kept for continuations: a submission that leaves
    // rays after its kBatchGens generations is continued from its queues
    FrameArgs lastA{};
    WaveArgs lastW{};
    DevScene lastS{};
    bool last_uniform = true;
    int last_jobs = 0;
    int swap = 0;                      // queue sets exchanged by an odd number of continuations
    int continuations = 0;
    std::vector<void *> dev;
    ~Batch() {
        if (stream) cudaStreamSynchronize(stream);
        for (void *p : dev) arena().free(p);
        if (h_jobs) cudaFreeHost(h_jobs);
        if (h_status) cudaFreeHost(h_status);
        if (h_ctr) cudaFreeHost(h_ctr);
        if (gexec) cudaGraphExecDestroy(gexec);
        if (done) cudaEventDestroy(done);
        for (int k = 0; k < 16; k++) {
            if (fork[k]) cudaEventDestroy(fork[k]);
            if (join[k]) cudaEventDestroy(join[k]);
        }
        if (side) cudaStreamSynchronize(side);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }
    int dalloc(void **p, size_t bytes) {
        int rc = arena().alloc(p, bytes ? bytes : 16);
        if (rc == GXY_OK) dev.push_back(*p);
        return rc;
    }
};

constexpr int kBatchGens = 10;   // generations per submission in per-generation mode

static size_t batch_tf_smem(bool uniform, const DevScene &Su) { return uniform ? tf_smem(Su) : 0; }

static int gen_grid(bool uniform, size_t smem) {
    int sms = 152, per = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_device);
    if (g_tune_minb == 3) {
        if (uniform) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_gen<K_SECONDARY, true, 3>, kThreads, smem);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_gen<K_SECONDARY, false, 3>, kThreads, smem);
    } else {
        if (uniform) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_gen<K_SECONDARY, true, 2>, kThreads, smem);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_gen<K_SECONDARY, false, 2>, kThreads, smem);
    }
    if (per < 1) per = 1;
    return sms * per;
}

static int batch_grid(bool uniform) {
    int sms = 152, per = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_device);
    if (uniform) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_wavefront<true>, kThreads, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_wavefront<false>, kThreads, 0);
    if (per < 1) per = 1;
    return sms * per;
}

// Shadow/AO march of a uniform split batch at 4 blocks per SM; rays that
// move to the next brick with a carried closest hit march on in the same
// lane (GXY_TUNE_CONTINUE), as in the frame path.
static void launch_batch_sec_march(cudaStream_t st, const DevScene &Su, const FrameArgs &a) {
    if (g_tune_continue && a.qmarch_hit) launch_sec_march<true, 4, true>(query_grid(), st, Su, a);
    else launch_sec_march<true, 4>(query_grid(), st, Su, a);
}

// Enqueue one submission on the batch stream (captured into a graph or not).
// cont: a continuation of the last submission -- no camera generation; the
// queue counts the last generation left (copied aside into d_status[2..4])
// become generation 0's, and the queue sets are exchanged so that
// generation 1 reads the set the last generation wrote.  Counters add up.
static int batch_enqueue(Batch *b, const DevScene &Su, bool uniform, const FrameArgs &A, const WaveArgs &W0,
                         int n_jobs, int cooperative, bool cont = false) {
    cudaStream_t st = b->stream;
    WaveArgs W = W0;
    if (b->swap)
        for (int k = 0; k < NQ; k++) std::swap(W.q[0][k], W.q[1][k]);
    if (!cont) CK(cudaMemcpyAsync(b->d_jobs, b->h_jobs, n_jobs * sizeof(DevJob), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(b->counts, 0, (kBatchGens + 1) * NQ * sizeof(unsigned), st));
    CK(cudaMemsetAsync(b->mcounts, 0, (2 * kBatchGens + 1) * 4 * sizeof(unsigned), st));
    if (!cont) CK(cudaMemsetAsync(b->ctr, 0, sizeof(DevCounters), st));
    if (cont)
        CK(cudaMemcpyAsync(b->counts, b->d_status + 2, NQ * sizeof(unsigned), cudaMemcpyDeviceToDevice, st));
    const int g_first = cont ? 1 : 0;
    if (!cooperative && uniform && split_eligible(Su) && g_tune_split_prim) {
        // Split passes as in a single frame: camera query + primary march,
        // then per generation the continuing primaries (side stream) beside
        // the shadow/AO query and march; counts are read on the device.
        const size_t tsm = batch_tf_smem(true, Su);
        const int grid = gen_grid(true, tsm);
        const bool lines = Su.n_seg > 0;
        for (int g = g_first; g < kBatchGens; g++) {
            FrameArgs a = A;
            for (int k = 0; k < NQ; k++) {
                a.qin[k] = W.q[(g + 1) & 1][k];
                a.qout[k] = W.q[g & 1][k];
            }
            a.qout_count = b->counts + NQ * g;
            const unsigned *cin = g ? b->counts + NQ * (g - 1) : nullptr;
            a.nin_dev = cin;
            a.split = 1;
            a.qmarch = b->qmarch;
            a.qmarch_hit = g_tune_carry_hits ? b->qmarch_hit : nullptr;
            a.qmarch_count = b->mcounts + 4 * g;
            a.qmarch_cap = (unsigned)b->qmarch_cap;
            a.split_prim = 1;
            a.pmarch = b->pmarch;
            a.pmarch_hit = b->pmarch_hit;
            a.pmarch_count = b->mcounts + 4 * kBatchGens;
            a.pmarch_cap = (unsigned)b->pmarch_cap;
            const bool mb3 = g_tune_minb == 3;
            if (g == 0) {
                if (mb3 && g_tune_cam_packet) {
                    // warp-cooperative camera query over every job's 8x4 tiles
                    if (g_tune_pquery_blocks == 2 && lines)
                        k_cam_packet<true, 2, true><<<one_wave(k_cam_packet<true, 2, true>), kThreads, 0, st>>>(Su, a);
                    else if (g_tune_pquery_blocks == 2)
                        k_cam_packet<true, 2, false><<<one_wave(k_cam_packet<true, 2, false>), kThreads, 0, st>>>(Su, a);
                    else if (lines) k_cam_packet<true, 4, true><<<query_grid(), kThreads, 0, st>>>(Su, a);
                    else k_cam_packet<true, 4, false><<<query_grid(), kThreads, 0, st>>>(Su, a);
                    if (g_tune_pmarch_blocks == 2) launch_prim_march<true, 2>(st, Su, a);
                    else launch_prim_march<true, 3>(st, Su, a);
                } else if (mb3) {
                    if (g_tune_pquery_blocks == 2 && lines)
                        k_cam_query<true, 2, true><<<one_wave(k_cam_query<true, 2, true>), kThreads, 0, st>>>(Su, a);
                    else if (g_tune_pquery_blocks == 2)
                        k_cam_query<true, 2, false><<<one_wave(k_cam_query<true, 2, false>), kThreads, 0, st>>>(Su, a);
                    else if (lines) k_cam_query<true, 4, true><<<query_grid(), kThreads, 0, st>>>(Su, a);
                    else k_cam_query<true, 4, false><<<query_grid(), kThreads, 0, st>>>(Su, a);
                    if (g_tune_pmarch_blocks == 2) launch_prim_march<true, 2>(st, Su, a);
                    else launch_prim_march<true, 3>(st, Su, a);
                } else {
                    if (lines) k_cam_query<true, 2, true><<<march_grid(2), kThreads, 0, st>>>(Su, a);
                    else k_cam_query<true, 2, false><<<march_grid(2), kThreads, 0, st>>>(Su, a);
                    launch_prim_march<true, 2>(st, Su, a);
                }
            } else {
                CK(cudaEventRecord(b->fork[g], st));
                CK(cudaStreamWaitEvent(b->side, b->fork[g], 0));
                if (g_tune_split_handoff) {
                    // handed-off primaries as the frame path traces them: a
                    // query to the partition exit into this generation's
                    // march records, then the skipping camera-ray march
                    FrameArgs ap = a;
                    ap.pmarch_count = b->mcounts + 4 * (kBatchGens + g);
                    const bool pq2 = !mb3 || g_tune_pquery_blocks == 2;
                    if (pq2 && lines)
                        k_prim_query<true, 2, true><<<one_wave(k_prim_query<true, 2, true>), kThreads, 0, b->side>>>(Su, ap);
                    else if (pq2)
                        k_prim_query<true, 2, false><<<one_wave(k_prim_query<true, 2, false>), kThreads, 0, b->side>>>(Su, ap);
                    else if (lines)
                        k_prim_query<true, 4, true><<<query_grid(), kThreads, 0, b->side>>>(Su, ap);
                    else
                        k_prim_query<true, 4, false><<<query_grid(), kThreads, 0, b->side>>>(Su, ap);
                    if (!mb3 || g_tune_pmarch_blocks == 2) launch_prim_march<true, 2>(b->side, Su, ap);
                    else launch_prim_march<true, 3>(b->side, Su, ap);
                } else if (mb3) {
                    k_batch_gen<K_PRIMARY, true, 3><<<grid, kThreads, tsm, b->side>>>(Su, a, cin);
                } else {
                    k_batch_gen<K_PRIMARY, true, 2><<<grid, kThreads, tsm, b->side>>>(Su, a, cin);
                }
                CK(cudaEventRecord(b->join[g], b->side));
                if (mb3 && g_tune_query_blocks == 2) {
                    if (lines) k_sec_query<true, 2, true><<<one_wave(k_sec_query<true, 2, true>), kThreads, 0, st>>>(Su, a);
                    else k_sec_query<true, 2, false><<<one_wave(k_sec_query<true, 2, false>), kThreads, 0, st>>>(Su, a);
                    launch_batch_sec_march(st, Su, a);
                } else if (mb3 && g_tune_query_blocks == 3) {
                    if (lines) k_sec_query<true, 3, true><<<one_wave(k_sec_query<true, 3, true>), kThreads, 0, st>>>(Su, a);
                    else k_sec_query<true, 3, false><<<one_wave(k_sec_query<true, 3, false>), kThreads, 0, st>>>(Su, a);
                    launch_batch_sec_march(st, Su, a);
                } else if (mb3) {
                    if (lines) k_sec_query<true, 4, true><<<query_grid(), kThreads, 0, st>>>(Su, a);
                    else k_sec_query<true, 4, false><<<query_grid(), kThreads, 0, st>>>(Su, a);
                    launch_batch_sec_march(st, Su, a);
                } else {
                    if (lines) k_sec_query<true, 2, true><<<march_grid(2), kThreads, 0, st>>>(Su, a);
                    else k_sec_query<true, 2, false><<<march_grid(2), kThreads, 0, st>>>(Su, a);
                    launch_sec_march<true, 2>(march_grid(2), st, Su, a);
                }
                CK(cudaStreamWaitEvent(st, b->join[g], 0));
            }
            CK(cudaGetLastError());
        }
        CK(cudaMemsetAsync(b->d_status, 0, 4 * sizeof(int), st));
        CK(cudaMemcpyAsync(b->d_status + 2, b->counts + NQ * (kBatchGens - 1), NQ * sizeof(unsigned),
                           cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(b->h_status, b->d_status, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(b->h_ctr, b->ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
        return GXY_OK;
    }
    if (!cooperative) {
        const bool split = uniform && split_eligible(Su);
        // generation g reads counts[g-1], writes counts[g] and queue set g&1
        const size_t tsm = batch_tf_smem(uniform, Su);
        int grid = gen_grid(uniform, tsm);
        for (int g = g_first; g < kBatchGens; g++) {
            FrameArgs a = A;
            for (int k = 0; k < NQ; k++) {
                a.qin[k] = W.q[(g + 1) & 1][k];
                a.qout[k] = W.q[g & 1][k];
            }
            a.qout_count = b->counts + NQ * g;
            a.split = (split && g > 0) ? 1 : 0;
            a.qmarch = b->qmarch;
            a.qmarch_count = b->mcounts + 4 * g;
            a.qmarch_cap = (unsigned)b->qmarch_cap;
            const unsigned *cin = g ? b->counts + NQ * (g - 1) : nullptr;
#define GXY_GEN_LAUNCH(MB)                                                                          \
    do {                                                                                            \
        if (g == 0) {                                                                               \
            if (uniform) k_batch_gen<K_CAMERA, true, MB><<<grid, kThreads, tsm, st>>>(Su, a, cin);  \
            else k_batch_gen<K_CAMERA, false, MB><<<grid, kThreads, tsm, st>>>(Su, a, cin);         \
        } else {                                                                                    \
            if (uniform) k_batch_gen<K_SECONDARY, true, MB><<<grid, kThreads, tsm, st>>>(Su, a, cin); \
            else k_batch_gen<K_SECONDARY, false, MB><<<grid, kThreads, tsm, st>>>(Su, a, cin);        \
        }                                                                                           \
    } while (0)
            if (g_tune_minb == 3) GXY_GEN_LAUNCH(3);
            else GXY_GEN_LAUNCH(2);
#undef GXY_GEN_LAUNCH
            if (a.split) {
                if (g_tune_minb == 3) launch_sec_march<true, 4>(query_grid(), st, Su, a);
                else launch_sec_march<true, 2>(march_grid(2), st, Su, a);
            }
            CK(cudaGetLastError());
        }
        // status: generations run, rays left after the last one
        CK(cudaMemsetAsync(b->d_status, 0, 4 * sizeof(int), st));
        CK(cudaMemcpyAsync(b->d_status + 2, b->counts + NQ * (kBatchGens - 1), NQ * sizeof(unsigned),
                           cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(b->h_status, b->d_status, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(b->h_ctr, b->ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
        return GXY_OK;
    }
    FrameArgs a = A;
    WaveArgs w = W;
    DevScene s = Su;
    void *args[] = {&s, &a, &w};
    int grid = batch_grid(uniform);
    if (uniform)
        CK(cudaLaunchCooperativeKernel((const void *)k_wavefront<true>, dim3(grid), dim3(kThreads), args, 0, st));
    else
        CK(cudaLaunchCooperativeKernel((const void *)k_wavefront<false>, dim3(grid), dim3(kThreads), args, 0, st));
    CK(cudaMemcpyAsync(b->h_status, b->d_status, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(b->h_ctr, b->ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
    return GXY_OK;
}

}  // namespace gxy

extern "C" {

int gxy_gpu_batch_create(int64_t max_pixels, int max_jobs, int max_shadow, int max_ao, gxy_batch *out) {
    GUARD_BEGIN
    if (!g_init) return set_error(GXY_ERR_NOT_INIT, "gxy_gpu_init not called");
    if (!out || max_pixels <= 0 || max_jobs <= 0 || max_jobs > kMaxJobs || max_shadow < 0 ||
        max_shadow > GXY_MAX_LIGHTS || max_ao < 0 || max_ao > 64)
        return set_error(GXY_ERR_INVALID, "bad batch limits");
    std::unique_ptr<Batch> b(new Batch());
    b->max_pixels = max_pixels;
    b->max_jobs = max_jobs;
    b->max_shadow = max_shadow;
    b->max_ao = max_ao;
    size_t slack = (size_t)max_pixels / 8 + 4096;
    size_t need[NQ] = {(size_t)max_pixels + slack, (size_t)max_pixels * max_shadow + slack,
                       (size_t)max_pixels * max_ao + slack};
    size_t bytes = 0;
    for (int k = 0; k < NQ; k++) bytes += 2 * need[k] * sizeof(DRay);
    bytes += (need[1] + need[2]) * (sizeof(DRay) + sizeof(float)) + need[0] * (sizeof(DRay) + 2 * sizeof(float4));   // march queues
    if (!arena().would_fit(bytes + 16 * 1024 * 1024))
        return set_error(GXY_ERR_ADMISSION, "batch queues (" + std::to_string(bytes) + " bytes) exceed the HBM budget");
    for (int k = 0; k < NQ; k++) {
        for (int s = 0; s < 2; s++) {
            int rc = b->dalloc((void **)&b->q[s][k], need[k] * sizeof(DRay));
            if (rc) return rc == GXY_ERR_OOM ? set_error(GXY_ERR_ADMISSION, last_error()) : rc;
        }
        if (need[k] > 0xffffffffull) return set_error(GXY_ERR_INVALID, "batch too large");
        b->qcap[k] = need[k];
    }
    int rc;
    if ((rc = b->dalloc((void **)&b->counts, (kBatchGens + 1) * NQ * sizeof(unsigned)))) return rc;
    if ((rc = b->dalloc((void **)&b->mcounts, (2 * kBatchGens + 1) * 4 * sizeof(unsigned)))) return rc;
    b->qmarch_cap = need[1] + need[2];
    if ((rc = b->dalloc((void **)&b->qmarch, b->qmarch_cap * sizeof(DRay)))) return rc;
    if ((rc = b->dalloc((void **)&b->qmarch_hit, b->qmarch_cap * sizeof(float)))) return rc;
    b->pmarch_cap = need[0];
    if ((rc = b->dalloc((void **)&b->pmarch, b->pmarch_cap * sizeof(DRay)))) return rc;
    if ((rc = b->dalloc((void **)&b->pmarch_hit, 2 * b->pmarch_cap * sizeof(float4)))) return rc;
    if ((rc = b->dalloc((void **)&b->d_jobs, max_jobs * sizeof(DevJob)))) return rc;
    if ((rc = b->dalloc((void **)&b->ctr, sizeof(DevCounters)))) return rc;
    if ((rc = b->dalloc((void **)&b->d_status, 8 * sizeof(int)))) return rc;
    CK(cudaMallocHost((void **)&b->h_jobs, max_jobs * sizeof(DevJob)));
    CK(cudaMallocHost((void **)&b->h_status, 8 * sizeof(int)));
    CK(cudaMallocHost((void **)&b->h_ctr, sizeof(DevCounters)));
    CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    for (int k = 0; k < 16; k++) {
        CK(cudaEventCreateWithFlags(&b->fork[k], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
    }
    *out = reinterpret_cast<gxy_batch>(b.release());
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_batch_release(gxy_batch batch) {
    GUARD_BEGIN
    if (!batch) return set_error(GXY_ERR_INVALID, "null batch");
    delete reinterpret_cast<Batch *>(batch);
    return GXY_OK;
    GUARD_END
}

int gxy_gpu_batch_stream(gxy_batch batch, void **stream) {
    if (!batch || !stream) return set_error(GXY_ERR_INVALID, "null argument");
    *stream = reinterpret_cast<Batch *>(batch)->stream;
    return GXY_OK;
}

int gxy_gpu_batch_submit(gxy_batch batch, const gxy_job *jobs, int n_jobs, int flags) {
    const int use_graph = flags & GXY_BATCH_GRAPH;
    const int cooperative = flags & GXY_BATCH_COOPERATIVE;
    GUARD_BEGIN
    if (!batch || !jobs || n_jobs <= 0) return set_error(GXY_ERR_INVALID, "bad argument");
    Batch *b = reinterpret_cast<Batch *>(batch);
    if (b->pending) {
        cudaError_t q = cudaEventQuery(b->done);
        if (q == cudaErrorNotReady) return set_error(GXY_ERR_INVALID, "previous submission still running");
    }
    if (n_jobs > b->max_jobs) return set_error(GXY_ERR_INVALID, "too many jobs for this batch");
    long long pix = 0, tiles = 0;
    Scene *first = reinterpret_cast<Scene *>(jobs[0].scene);
    bool uniform = true;
    for (int j = 0; j < n_jobs; j++) {
        const gxy_job &J = jobs[j];
        if (!J.scene || !J.fb_rgba || J.camera.width <= 0 || J.camera.height <= 0)
            return set_error(GXY_ERR_INVALID, "bad job " + std::to_string(j));
        Scene *sc = reinterpret_cast<Scene *>(J.scene);
        if (sc != first) uniform = false;
        DevJob &D = b->h_jobs[j];
        D.cam = setup_camera(J.camera);
        int rc = setup_lights(J.lighting, D.L);
        if (rc) return rc;
        if (D.L.n == 0) return set_error(GXY_ERR_INVALID, "lighting needs at least one light");
        if ((D.L.shadows ? D.L.n : 0) > b->max_shadow || D.L.n_ao > b->max_ao)
            return set_error(GXY_ERR_ADMISSION, "job needs more secondary rays per pixel than the batch holds");
        D.fb = J.fb_rgba;
        D.scene = sc->d_scene;
        D.pix0 = pix;
        D.tile0 = tiles;
        pix += (long long)J.camera.width * J.camera.height;
        tiles += (long long)((J.camera.width + 7) / 8) * ((J.camera.height + 3) / 4);
    }
    if (pix > b->max_pixels) return set_error(GXY_ERR_ADMISSION, "batch pixel budget exceeded");
    FrameArgs A;
    memset(&A, 0, sizeof A);
    A.jobs = b->d_jobs;
    A.n_jobs = n_jobs;
    A.trav_steps = g_tune_trav_steps;
    A.queue_chunk = g_tune_queue_chunk / (kThreads / 32);
    A.march_steps = g_tune_march_steps;
    A.skip_mode = g_tune_skip_mode;
    A.total_pix = pix;
    A.total_tiles = tiles;
    A.job0 = b->h_jobs[0];
    for (int k = 0; k < NQ; k++) A.qcap[k] = (unsigned)b->qcap[k];
    A.ctr = b->ctr;
    WaveArgs W;
    for (int s = 0; s < 2; s++)
        for (int k = 0; k < NQ; k++) W.q[s][k] = b->q[s][k];
    W.counts = b->counts;
    W.max_gen = 64;
    W.status = b->d_status;
    const DevScene &Su = first->S;
    b->swap = 0;
    b->continuations = 0;
    b->lastA = A;
    b->lastW = W;
    b->lastS = Su;
    b->last_uniform = uniform;
    b->last_jobs = n_jobs;
    if (use_graph) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int rc = batch_enqueue(b, Su, uniform, A, W, n_jobs, cooperative);
        cudaGraph_t gg = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &gg);
        if (rc) return rc;
        if (e != cudaSuccess) return set_error(GXY_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
        g = gg;
        bool updated = false;
        if (b->gexec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(b->gexec, g, &info) == cudaSuccess) updated = true;
            else {
                cudaGetLastError();
                cudaGraphExecDestroy(b->gexec);
                b->gexec = nullptr;
            }
        }
        if (!updated) CK(cudaGraphInstantiate(&b->gexec, g, 0));
        cudaGraphDestroy(g);
        CK(cudaGraphLaunch(b->gexec, b->stream));
    } else {
        int rc = batch_enqueue(b, Su, uniform, A, W, n_jobs, cooperative);
        if (rc) return rc;
    }
    b->cooperative = cooperative;
    CK(cudaEventRecord(b->done, b->stream));
    b->pending = true;
    b->last_rc = GXY_OK;
    return GXY_OK;
    GUARD_END
}

// A finished submission: its status, or -- when rays are left after its
// generations and nothing overflowed -- a continuation from its queues
// (*continued, the batch stays pending).  Up to kMaxContinuations.
constexpr int kMaxContinuations = 64;
static int batch_finish(Batch *b, bool *continued) {
    *continued = false;
    int left = b->cooperative ? b->h_status[1] : (b->h_status[2] + b->h_status[3] + b->h_status[4]);
    if (left > 0 && !b->cooperative && !b->h_ctr->overflow && b->continuations < kMaxContinuations) {
        b->swap ^= 1;
        b->continuations++;
        int rc = batch_enqueue(b, b->lastS, b->last_uniform, b->lastA, b->lastW, b->last_jobs, 0, true);
        if (rc == GXY_OK && cudaEventRecord(b->done, b->stream) != cudaSuccess)
            rc = set_error(GXY_ERR_CUDA, "event record failed");
        if (rc) {
            b->pending = false;
            return b->last_rc = rc;
        }
        *continued = true;
        return GXY_OK;
    }
    b->pending = false;
    if (left > 0) return b->last_rc = set_error(GXY_ERR_OVERFLOW, "rays left after the generation limit");
    if (b->h_ctr->overflow) return b->last_rc = set_error(GXY_ERR_OVERFLOW, "a batch queue overflowed");
    return b->last_rc = GXY_OK;
}

int gxy_gpu_batch_poll(gxy_batch batch, int *done) {
    GUARD_BEGIN
    if (!batch || !done) return set_error(GXY_ERR_INVALID, "null argument");
    Batch *b = reinterpret_cast<Batch *>(batch);
    if (!b->pending) {
        *done = 1;
        return b->last_rc;
    }
    cudaError_t e = cudaEventQuery(b->done);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return GXY_OK;
    }
    if (e != cudaSuccess) return set_error(GXY_ERR_CUDA, cudaGetErrorString(e));
    bool cont = false;
    int rc = batch_finish(b, &cont);
    *done = cont ? 0 : 1;
    return rc;
    GUARD_END
}

int gxy_gpu_batch_wait(gxy_batch batch, int timeout_ms) {
    GUARD_BEGIN
    if (!batch) return set_error(GXY_ERR_INVALID, "null batch");
    Batch *b = reinterpret_cast<Batch *>(batch);
    if (!b->pending) return b->last_rc;
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaEventQuery(b->done);
        if (e == cudaSuccess) {
            bool cont = false;
            int rc = batch_finish(b, &cont);
            if (!cont) return rc;
            continue;
        }
        if (e != cudaErrorNotReady) return set_error(GXY_ERR_CUDA, cudaGetErrorString(e));
        double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_ms >= 0 && ms > timeout_ms) return set_error(GXY_ERR_TIMEOUT, "batch did not finish in time");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    GUARD_END
}

int gxy_gpu_batch_counters(gxy_batch batch, gxy_counters *out) {
    if (!batch || !out) return set_error(GXY_ERR_INVALID, "null argument");
    Batch *b = reinterpret_cast<Batch *>(batch);
    const DevCounters &c = *b->h_ctr;
    memset(out, 0, sizeof *out);
    out->primary_rays = (int64_t)c.primary;
    out->shadow_rays = (int64_t)c.shadow;
    out->ao_rays = (int64_t)c.ao;
    out->secondary_rays = (int64_t)(c.shadow + c.ao);
    out->segments = (int64_t)c.segments;
    out->handoffs = (int64_t)c.handoffs;
    out->terminated = (int64_t)c.terminated;
    out->dropped = (int64_t)c.dropped;
    out->kept = (int64_t)c.kept;
    out->bounces = b->cooperative ? b->h_status[0] : kBatchGens + (int64_t)b->continuations * (kBatchGens - 1);
    out->bands = 1;
    out->samples = (int64_t)c.samples;
    out->nodes = (int64_t)c.nodes;
    out->prim_tests = (int64_t)(c.tri_tests + c.sph_tests);
    out->overflow = c.overflow;
    out->samples_skipped = (int64_t)c.skipped;
    return GXY_OK;
}

}  // extern "C"

// ===================================================== allocation-free entry
// gxy_gpu_generate_initial_rays_noalloc: the camera-ray pass of
// gxy_gpu_generate_initial_rays for callers that may not allocate device
// memory, writing into a RayList the caller already holds in GPU-addressable
// memory.  Its scratch -- one flag and one output offset per pixel plus the
// scan's temporary storage -- is the fixed array below, part of this
// library's device image: every GPU that loads the library holds it until the
// process exits, and every call on that GPU shares it.  All of a call's work
// goes to the calling thread's per-thread default stream, which the call
// synchronises before it returns.
namespace gxy {

constexpr int64_t kNoAllocMaxPixels = int64_t(1) << 20;   // 1024 x 1024 camera pixels
constexpr size_t kNoAllocPosOffset = (size_t)kNoAllocMaxPixels * sizeof(int);
constexpr size_t kNoAllocScanOffset = 2 * (size_t)kNoAllocMaxPixels * sizeof(int);
constexpr size_t kNoAllocScanBytes = size_t(256) << 10;   // CUB scan temporary storage
constexpr size_t kNoAllocScratchBytes = kNoAllocScanOffset + kNoAllocScanBytes;   // 8.25 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_addr[kNoAllocMaxDevices];

// Device address of g_noalloc_scratch on the current device.  In host code
// the symbol names a host-side stand-in, not device memory, so the address is
// looked up with cudaGetSymbolAddress, once per device with that device
// current, on the first call there (which also loads this library's device
// code on that device, the array included, under lazy module loading).  A
// cached address is re-validated on every call: after a cudaDeviceReset the
// module is loaded afresh and the old address no longer names device memory
// of this device, so it is looked up again.
static int noalloc_scratch(unsigned char **out) {
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error(GXY_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_addr[dev]) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, g_noalloc_addr[dev]) != cudaSuccess || a.type != cudaMemoryTypeDevice ||
            a.device != dev) {
            cudaGetLastError();
            g_noalloc_addr[dev] = nullptr;
        }
    }
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        if (!p) return set_error(GXY_ERR_CUDA, "cudaGetSymbolAddress gave a null scratch address");
        g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_noalloc_addr[dev];
    return GXY_OK;
}

// True if a kernel on device `dev` may write through `p`: memory of that
// device, managed memory, or pinned host memory mapped at the same address.
static bool gpu_addressable(const void *p, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeDevice) return a.device == dev;
    if (a.type == cudaMemoryTypeManaged) return true;
    if (a.type == cudaMemoryTypeHost) return a.devicePointer == p;
    return false;
}

// True if the `bytes` bytes from `p` are GPU-addressable from device `dev`:
// both ends pass gpu_addressable and, for device and managed memory, the
// range lies inside the one allocation that holds `p` (cuMemGetAddressRange,
// taken through the runtime's driver entry points, so no driver library is
// linked).
static bool gpu_range_ok(const void *p, size_t bytes, int dev) {
    if (!gpu_addressable(p, dev)) return false;
    if (bytes == 0) return true;
    const char *last = static_cast<const char *>(p) + (bytes - 1);
    if (!gpu_addressable(last, dev)) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeHost) return true;
    typedef int (*range_fn)(unsigned long long *, size_t *, unsigned long long);
    static range_fn fn = nullptr;
    static bool looked = false;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!looked) {
            void *f = nullptr;
            cudaDriverEntryPointQueryResult q;
            if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 3020, cudaEnableDefault, &q) ==
                    cudaSuccess &&
                q == cudaDriverEntryPointSuccess)
                fn = reinterpret_cast<range_fn>(f);
            else
                cudaGetLastError();
            looked = true;
        }
    }
    if (!fn) return true;   // both ends checked above
    unsigned long long base = 0;
    size_t size = 0;
    if (fn(&base, &size, (unsigned long long)(uintptr_t)p) != 0) return false;
    const unsigned long long lo = (unsigned long long)(uintptr_t)p;
    return lo >= base && lo - base + bytes <= size;
}

// Zero the 25 arrays of the first n records (fields the camera pass leaves
// unset read as zero, as in gxy_gpu_generate_initial_rays); a kernel rather
// than cudaMemset, so it serves every GPU-addressable memory kind alike.
__global__ void k_rl_zero(RLDev O, int n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < 20; k++) O.f[k][i] = 0.0f;
    for (int k = 0; k < 5; k++) O.i[k][i] = 0;
}

}  // namespace gxy

extern "C" int gxy_gpu_generate_initial_rays_noalloc(gxy_scene scene, int partition, const gxy_camera *camera,
                                                     gxy_raylist *out, int32_t *n_out) {
    GUARD_BEGIN
    if (!scene || !camera || !out || !n_out) return set_error(GXY_ERR_INVALID, "null argument");
    Scene *sc = reinterpret_cast<Scene *>(scene);
    if (partition < 0 || partition >= sc->S.np) return set_error(GXY_ERR_INVALID, "bad partition");
    if (camera->width <= 0 || camera->height <= 0) return set_error(GXY_ERR_INVALID, "bad image size");
    int64_t n = (int64_t)camera->width * camera->height;
    if (n > kNoAllocMaxPixels)
        return set_error(GXY_ERR_INVALID, "image of " + std::to_string(n) +
                                              " pixels exceeds the 1048576-pixel limit of the allocation-free "
                                              "camera-ray entry point");
    if (out->n < 0) return set_error(GXY_ERR_INVALID, "negative RayList capacity");
    int dev = -1;
    CK(cudaGetDevice(&dev));
    float *of[20];
    int32_t *oi[5];
    host_f(*out, of);
    host_i(*out, oi);
    // every array must hold out->n records in memory the GPU can write
    const size_t cap = (size_t)out->n;
    for (int k = 0; k < 20; k++)
        if (!of[k] || !gpu_range_ok(of[k], cap * sizeof(float), dev))
            return set_error(GXY_ERR_INVALID, "output RayList float array " + std::to_string(k) +
                                                  " is not memory the GPU can address for its capacity");
    for (int k = 0; k < 5; k++)
        if (!oi[k] || !gpu_range_ok(oi[k], cap * sizeof(int32_t), dev))
            return set_error(GXY_ERR_INVALID, "output RayList int array " + std::to_string(k) +
                                                  " is not memory the GPU can address for its capacity");
    unsigned char *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    int *flag = reinterpret_cast<int *>(scratch);
    int *pos = reinterpret_cast<int *>(scratch + kNoAllocPosOffset);
    void *scan_tmp = scratch + kNoAllocScanOffset;
    size_t scan_bytes = 0;
    CK(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, flag, pos, (int)n, cudaStreamPerThread));
    if (scan_bytes > kNoAllocScanBytes)
        return set_error(GXY_ERR_OVERFLOW, "scan temporary storage does not fit the fixed scratch");
    // The flag pass writes flag[0, n), the scan writes pos[0, n) and sets up
    // its own temporary storage, so nothing left by an earlier call is read.
    const cudaStream_t st = cudaStreamPerThread;
    DevCamera C = setup_camera(*camera);
    unsigned g = (unsigned)((n + 255) / 256);
    k_rl_camera_flags<<<g, 256, 0, st>>>(sc->S, C, partition, flag);
    CK(cudaGetLastError());
    CK(cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, flag, pos, (int)n, st));
    int last[2] = {0, 0};
    CK(cudaMemcpyAsync(&last[0], pos + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&last[1], flag + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int total = last[0] + last[1];
    *n_out = total;
    if (total > out->n) return set_error(GXY_ERR_OVERFLOW, "output RayList too small");
    if (total) {
        RLDev O{};
        for (int k = 0; k < 20; k++) O.f[k] = of[k];
        for (int k = 0; k < 5; k++) O.i[k] = oi[k];
        O.n = total;
        k_rl_zero<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(O, total);
        CK(cudaGetLastError());
        k_rl_camera_write<<<g, 256, 0, st>>>(sc->S, C, partition, flag, pos, O);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(st));
    return GXY_OK;
    GUARD_END
}

// gxy_dev.cuh -- device-side data layout and per-ray algorithms of the
// GB300 ray path: scene tables, the 128-byte BVH8 node, the 64-byte queue
// record, primitive tests, BVH8 traversal, the volume march and the
// shading/spawn arithmetic.
//
// Arithmetic contract: translation units that include this header are built
// with -fmad=false, so every expression below rounds exactly as written
// (the same IEEE single-precision operations, in the same order, as the
// semantics stated for Galaxy's TraceRays.ispc).  The only fused operations
// are the explicit __fmaf_rn calls of the BVH box test, which decides only
// which primitives are tested, never a result.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gxy_gpu.h"

namespace gxy {

// ----------------------------------------------------------------- layout
constexpr int kMaxVol = GXY_MAX_VOLUMES;
constexpr int kMaxPart = GXY_MAX_PARTITIONS;
constexpr uint32_t kSphereBit = 0x80000000u;
constexpr uint32_t kLineBit = 0x40000000u;     // with kSphereBit: a path-line segment

struct DevTF {                       // one resampled transfer function, 4 KB
    float colors[GXY_TF_SIZE * 3];
    float opac[GXY_TF_SIZE];
    float r0, r1, k, pad;            // k = 255 / (r1 - r0)
};

// Voxels are stored in bricks of 4x4x4 cells with a one-voxel apron: brick
// (bx, by, bz) holds voxels 4b .. 4b+4 on each axis (5^3 floats, padded to
// 128 = one 512-byte block), so the 8 corners of any cell lie in one brick,
// within 124 contiguous bytes (at most two 128-byte lines).
constexpr int kBrick = 4, kBrickSide = 5, kBrickFloats = 128;
struct DevVolume {
    const float *data;               // bricked
    int nx, ny, nz;
    int nbx, nby;                    // bricks along x and y
    float ox, oy, oz, dx, dy, dz;
    float ux, uy, uz;                // clamp bounds: float just below n-1
    float ix, iy, iz;                // 1 / delta
    int tf;                          // index into DevScene::tfs
    int n_slices;
    float4 slices[GXY_MAX_SLICES];
    int n_iso;
    float iso[GXY_MAX_ISOVALUES];
    int volume_render;
    // Per brick, 1 when every trilinear sample inside it lies below the
    // transfer function's zero-opacity threshold (tf_clear_below), so an
    // interval between two such samples composites nothing.
    const unsigned char *clear;
    // Per superbrick of kSuper^3 bricks (32^3 cells): 1 when every brick
    // within one brick of it is clear, so a position whose computed cell is
    // within a brick (4 voxels) of the superbrick lies in a clear brick.
    const unsigned char *sclear;
    int nsx, nsy, nsz;
};
constexpr int kSuper = 8;            // bricks per superbrick side
constexpr int kSuperCells = kSuper * kBrick;

struct DevPartition {
    float lo[3], hi[3];
    int nb[6];
};

struct DevTriSet {                   // triangles [prim_base, prim_base+n)
    int64_t prim_base, n;
    const int32_t *indices;          // 3 per triangle (set-local vertex ids)
    const float *vertices;           // 3 per vertex
    const float *normals;            // 3 per vertex or null
    const float *data;               // per vertex or null
    int tf;
};

struct DevSphSet {                   // spheres [prim_base, prim_base+n)
    int64_t prim_base, n;
    const float *centers;
    const float *data;
    int tf;
    float eps;
};

struct DevLineSet {                  // path-line segments [prim_base, prim_base+n)
    int64_t prim_base, n;
    const int32_t *indices;          // first vertex of each segment
    const float *vertices;           // 3 per vertex
    const float *radius;             // per vertex, MAP_RADIUS of the data
    float radius0, radius1, value0, value1;
    int tf;
};

// 128-byte wide node: one L2 line.  Child i's box is
// origin + q * 2^(e-127) per axis, with q the 16-bit lower/upper bounds.
struct __align__(128) BVH8Node {
    float ox, oy, oz;
    uint32_t child_base;             // first internal child node
    uint32_t prim_base;              // first leaf primitive slot
    uint8_t ex, ey, ez, imask;       // exponents; bit i: child i is internal
    uint8_t meta[8];                 // internal: rank; leaf: (count-1)<<5 | offset; 0xff: empty
    uint16_t qlo[3][8];
    uint16_t qhi[3][8];
};
static_assert(sizeof(BVH8Node) == 128, "BVH8 node must fill one 128-byte line");

// Leaf primitive slot: 3 float4.  Triangle: (v0, id) (v1, -) (v2, -).
// Sphere: (center, id | kSphereBit) (radius, eps, -, -) (-).
// Path-line segment: (A, id | kSphereBit | kLineBit) (B, radius0) (-).
// Ids are the primitive's index (triangles, then spheres, then segments)
// plus these bits, so they order like the index (fewer than 2^30 primitives).
struct DevScene {
    int n_vol;
    DevVolume vol[kMaxVol];
    int np;
    float glo[3], ghi[3];
    DevPartition part[kMaxPart];
    int integrate;                   // some volume is rendered or has isovalues
    int has_iso;                     // some volume has isovalues
    float step, march_eps, epsilon, opaque_alpha, rate;
    int rate_pow2;                   // rate is a power of two: x / rate == x * inv_rate exactly
    float inv_rate;
    // geometry
    const BVH8Node *nodes;
    const float4 *slots;
    int64_t n_tri, n_sph, n_seg;
    int n_tri_sets, n_sph_sets, n_line_sets;
    DevTriSet tri_sets[4];
    DevSphSet sph_sets[4];
    DevLineSet line_sets[4];
    const DevTF *tfs;
    const float4 *ao;                // 256 x (cos 2pi u, sin 2pi u, sqrt(1-v), sqrt(v))
};

// 64-byte queue record.
struct __align__(16) DRay {
    float4 o;                        // origin, t
    float4 d;                        // direction, tMax
    float4 c;                        // r g b o
    int4 m;                          // x, y, meta (type | part<<4 | job<<12), spare
};
__host__ __device__ inline int ray_type(int meta) { return meta & 0xf; }
__host__ __device__ inline int ray_part(int meta) { return (meta >> 4) & 0xff; }
__host__ __device__ inline int ray_job(int meta) { return (meta >> 12) & 0xfffff; }
__host__ __device__ inline int make_meta(int type, int part, int job) { return type | (part << 4) | (job << 12); }

// Per-frame constants: camera and lighting of one render job.
struct DevCamera {
    float3 eye, center, vr, vu, vdir;
    float off_x, off_y, scaling;
    int ortho;
    int width, height;
};
struct DevLights {
    int n;
    float3 l[GXY_MAX_LIGHTS];
    int type[GXY_MAX_LIGHTS];
    float Ka, Kd;
    int n_ao;
    float ao_radius;
    int shadows;
};

struct DevCounters {
    unsigned long long primary, shadow, ao, segments, handoffs, terminated, dropped, kept, samples, nodes, tri_tests,
        sph_tests, enqueued, marched, skipped;
    int overflow;        // a queue or a traversal stack ran out of room
    int pad;
};

// ------------------------------------------------------------ vector math
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 nrm(V3 a) {   // v * (1/sqrt(v.v)); zero stays zero
    float l2 = dot(a, a);
    if (l2 == 0.0f) return a;
    float inv = 1.0f / sqrtf(l2);
    return inv * a;
}
__device__ __forceinline__ float fmin_(float a, float b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ float fmax_(float a, float b) { return (a < b) ? b : a; }   // std::max

// ------------------------------------------------------ transfer function
// Piecewise-linear lookup over 256 entries (NaN -> 0, clamp outside range,
// index f = (v - r0) * (255 / (r1 - r0))).
__device__ __forceinline__ float tf_opacity(const DevTF &tf, float v) {
    if (isnan(v)) return 0.0f;
    if (v <= tf.r0) return tf.opac[0];
    if (v >= tf.r1) return tf.opac[255];
    float f = (v - tf.r0) * tf.k;
    int i = (int)floorf(f);
    i = i > 254 ? 254 : (i < 0 ? 0 : i);
    float rem = f - (float)i;
    return (1.0f - rem) * tf.opac[i] + rem * tf.opac[i + 1];
}
__device__ __forceinline__ V3 tf_color(const DevTF &tf, float v) {
    if (isnan(v)) return v3(0, 0, 0);
    const float *c = tf.colors;
    if (v <= tf.r0) return v3(c[0], c[1], c[2]);
    if (v >= tf.r1) return v3(c[765], c[766], c[767]);
    float f = (v - tf.r0) * tf.k;
    int i = (int)floorf(f);
    i = i > 254 ? 254 : (i < 0 ? 0 : i);
    float rem = f - (float)i;
    float a = 1.0f - rem;
    return v3(a * c[3 * i] + rem * c[3 * i + 3], a * c[3 * i + 1] + rem * c[3 * i + 4],
              a * c[3 * i + 2] + rem * c[3 * i + 5]);
}

// Opacity and colour of one value with a single index computation (the
// same arithmetic as tf_opacity and tf_color).  Returns the opacity; the
// colour is only evaluated when want_color and the opacity is positive.
__device__ __forceinline__ float tf_lookup(const DevTF &tf, float v, bool want_color, V3 &col) {
    if (isnan(v)) {
        col = v3(0, 0, 0);
        return 0.0f;
    }
    const float *c = tf.colors;
    float op;
    if (v <= tf.r0) {
        op = tf.opac[0];
        if (want_color && op > 0.0f) col = v3(c[0], c[1], c[2]);
        return op;
    }
    if (v >= tf.r1) {
        op = tf.opac[255];
        if (want_color && op > 0.0f) col = v3(c[765], c[766], c[767]);
        return op;
    }
    float f = (v - tf.r0) * tf.k;
    int i = (int)floorf(f);
    i = i > 254 ? 254 : (i < 0 ? 0 : i);
    float rem = f - (float)i;
    float a = 1.0f - rem;
    op = a * tf.opac[i] + rem * tf.opac[i + 1];
    if (want_color && op > 0.0f)
        col = v3(a * c[3 * i] + rem * c[3 * i + 3], a * c[3 * i + 1] + rem * c[3 * i + 4],
                 a * c[3 * i + 2] + rem * c[3 * i + 5]);
    return op;
}

// ---------------------------------------------------------------- volume
// Trilinear sample of the dataset grid at world point p, clamped to the grid;
// grid coordinate (p - origin) * (1 / delta).
// Corner (ix, iy, iz) of cell (ix, iy, iz) in the bricked layout; the other
// corners are at +1 (x), +kBrickSide (y) and +kBrickSide^2 (z).
__device__ __forceinline__ const float *cell_base(const DevVolume &v, int ix, int iy, int iz) {
    const int bx = ix >> 2, by = iy >> 2, bz = iz >> 2;
    const size_t brick = ((size_t)bz * v.nby + by) * v.nbx + bx;
    return v.data + brick * kBrickFloats + ((iz & 3) * kBrickSide + (iy & 3)) * kBrickSide + (ix & 3);
}

__device__ __forceinline__ float vol_sample(const DevVolume &v, V3 p) {
    float gx = (p.x - v.ox) * v.ix;
    float gy = (p.y - v.oy) * v.iy;
    float gz = (p.z - v.oz) * v.iz;
    if (!(gx >= 0.0f)) gx = 0.0f;
    if (!(gy >= 0.0f)) gy = 0.0f;
    if (!(gz >= 0.0f)) gz = 0.0f;
    if (gx > v.ux) gx = v.ux;
    if (gy > v.uy) gy = v.uy;
    if (gz > v.uz) gz = v.uz;
    int ix = (int)gx, iy = (int)gy, iz = (int)gz;
    float fx = gx - (float)ix, fy = gy - (float)iy, fz = gz - (float)iz;
    const float *b = cell_base(v, ix, iy, iz);
    constexpr int SY = kBrickSide, SZ = kBrickSide * kBrickSide;
    float v000 = __ldg(b), v100 = __ldg(b + 1), v010 = __ldg(b + SY), v110 = __ldg(b + SY + 1);
    float v001 = __ldg(b + SZ), v101 = __ldg(b + SZ + 1), v011 = __ldg(b + SZ + SY), v111 = __ldg(b + SZ + SY + 1);
    float ax = 1.0f - fx;
    float v00 = ax * v000 + fx * v100;
    float v10 = ax * v010 + fx * v110;
    float v01 = ax * v001 + fx * v101;
    float v11 = ax * v011 + fx * v111;
    float ay = 1.0f - fy;
    float v0 = ay * v00 + fy * v10;
    float v1 = ay * v01 + fy * v11;
    return (1.0f - fz) * v0 + fz * v1;
}

// Same sample, with the 8 corner values of the last cell kept in registers:
// consecutive half-voxel steps usually stay in one cell.
struct CellCache {
    int ix, iy, iz;
    float c[8];
};

// Clamped grid coordinate of a world point and its cell, as vol_sample
// computes them.
struct VolPos {
    float gx, gy, gz;
    int ix, iy, iz;
};
__device__ __forceinline__ VolPos vol_pos(const DevVolume &v, V3 p) {
    VolPos g;
    g.gx = (p.x - v.ox) * v.ix;
    g.gy = (p.y - v.oy) * v.iy;
    g.gz = (p.z - v.oz) * v.iz;
    if (!(g.gx >= 0.0f)) g.gx = 0.0f;
    if (!(g.gy >= 0.0f)) g.gy = 0.0f;
    if (!(g.gz >= 0.0f)) g.gz = 0.0f;
    if (g.gx > v.ux) g.gx = v.ux;
    if (g.gy > v.uy) g.gy = v.uy;
    if (g.gz > v.uz) g.gz = v.uz;
    g.ix = (int)g.gx; g.iy = (int)g.gy; g.iz = (int)g.gz;
    return g;
}

// Linear index of the brick holding the cell of g.
__device__ __forceinline__ int brick_of(const DevVolume &v, const VolPos &g) {
    return ((g.iz >> 2) * v.nby + (g.iy >> 2)) * v.nbx + (g.ix >> 2);
}

// Linear index of the superbrick holding the cell of g.
__device__ __forceinline__ int super_of(const DevVolume &v, const VolPos &g) {
    return ((g.iz >> 5) * v.nsy + (g.iy >> 5)) * v.nsx + (g.ix >> 5);
}

__device__ __forceinline__ float vol_sample_at(const DevVolume &v, const VolPos &g, CellCache &cc) {
    if (g.ix != cc.ix || g.iy != cc.iy || g.iz != cc.iz) {
        const float *b = cell_base(v, g.ix, g.iy, g.iz);
        constexpr int SY = kBrickSide, SZ = kBrickSide * kBrickSide;
        cc.c[0] = __ldg(b); cc.c[1] = __ldg(b + 1); cc.c[2] = __ldg(b + SY); cc.c[3] = __ldg(b + SY + 1);
        cc.c[4] = __ldg(b + SZ); cc.c[5] = __ldg(b + SZ + 1); cc.c[6] = __ldg(b + SZ + SY);
        cc.c[7] = __ldg(b + SZ + SY + 1);
        cc.ix = g.ix; cc.iy = g.iy; cc.iz = g.iz;
    }
    float fx = g.gx - (float)g.ix, fy = g.gy - (float)g.iy, fz = g.gz - (float)g.iz;
    float ax = 1.0f - fx;
    float v00 = ax * cc.c[0] + fx * cc.c[1];
    float v10 = ax * cc.c[2] + fx * cc.c[3];
    float v01 = ax * cc.c[4] + fx * cc.c[5];
    float v11 = ax * cc.c[6] + fx * cc.c[7];
    float ay = 1.0f - fy;
    float v0 = ay * v00 + fy * v10;
    float v1 = ay * v01 + fy * v11;
    return (1.0f - fz) * v0 + fz * v1;
}

__device__ __forceinline__ float vol_sample_cached(const DevVolume &v, V3 p, CellCache &cc) {
    return vol_sample_at(v, vol_pos(v, p), cc);
}

// Central-difference gradient, one grid spacing either side.
__device__ __forceinline__ V3 vol_gradient(const DevVolume &v, V3 p) {
    V3 g;
    g.x = (vol_sample(v, v3(p.x + v.dx, p.y, p.z)) - vol_sample(v, v3(p.x - v.dx, p.y, p.z))) / (2.0f * v.dx);
    g.y = (vol_sample(v, v3(p.x, p.y + v.dy, p.z)) - vol_sample(v, v3(p.x, p.y - v.dy, p.z))) / (2.0f * v.dy);
    g.z = (vol_sample(v, v3(p.x, p.y, p.z + v.dz)) - vol_sample(v, v3(p.x, p.y, p.z - v.dz))) / (2.0f * v.dz);
    return g;
}

// -------------------------------------------------------------- primitives
// Moller-Trumbore; caller checks t against (t0, tfar).
__device__ __forceinline__ bool tri_test(V3 org, V3 dir, V3 v0, V3 v1, V3 v2, float &t, float &u, float &v) {
    V3 e1 = v1 - v0, e2 = v2 - v0;
    V3 pv = cross(dir, e2);
    float det = dot(e1, pv);
    if (det == 0.0f) return false;
    float inv = 1.0f / det;
    V3 tv = org - v0;
    u = dot(tv, pv) * inv;
    if (u < 0.0f || u > 1.0f) return false;
    V3 qv = cross(tv, e1);
    v = dot(dir, qv) * inv;
    if (v < 0.0f || u + v > 1.0f) return false;
    t = dot(e2, qv) * inv;
    return true;
}

// Data-driven sphere: t_in if in (t0, tfar), else t_out if in (t0+eps, tfar).
__device__ __forceinline__ bool sph_test(V3 org, V3 dir, V3 c, float r, float eps, float t0, float tfar, float &t) {
    float approx = dot(c - org, dir);
    V3 close = org + approx * dir;
    V3 A = c - close;
    float a = dot(dir, dir);
    float b = 2.0f * dot(dir, A);
    float cc = dot(A, A) - r * r;
    float rad = b * b - 4.0f * a * cc;
    if (rad < 0.0f) return false;
    float srad = sqrtf(rad);
    float r2a = 1.0f / (2.0f * a);
    float tin = (b - srad) * r2a + approx;
    float tout = (b + srad) * r2a + approx;
    if (tin > t0 && tin < tfar) { t = tin; return true; }
    if (tout > t0 + eps && tout < tfar) { t = tout; return true; }
    return false;
}

// Path-line segment as DataDrivenPathLines_intersect_kernel intersects it
// (DataDrivenPathLines.ispc:100-203): a cylinder A-B of radius r clipped at
// its caps, joined with spheres of radius r at A and B, each with the
// numerical fix of moving the ray origin to an approximate distance first;
// rcp/rcpf are taken as exact reciprocals.  Accepted distance: t_in if in
// (t0, tfar), else t_out if in (t0, tfar).
__device__ __forceinline__ void line_sphere(V3 org, V3 dir, V3 c, float r, float &t_in, float &t_out) {
    const float approx = dot(c - org, dir);
    const V3 close = org + approx * dir;
    const V3 A = c - close;
    const float a = dot(dir, dir);
    const float b = -2.f * dot(dir, A);
    const float cc = dot(A, A) - r * r;
    const float rad = b * b - 4.f * a * cc;
    if (rad < 0.f) return;
    const float srad = sqrtf(rad);
    const float r2a = 1.0f / (2.f * a);
    t_in = fmin_(t_in, approx + (-b - srad) * r2a);
    t_out = fmax_(t_out, approx + (-b + srad) * r2a);
}
__device__ __forceinline__ void line_cylinder(V3 org, V3 dir, V3 A0, V3 B0, float r, float &t_in, float &t_out) {
    const V3 center = 0.5f * (A0 + B0);
    const float approx = dot(center - org, dir);
    const V3 close = org + approx * dir;
    const V3 A = A0 - close, B = B0 - close;
    const V3 AB = B - A;
    const V3 AOxAB = cross(AB, A);
    const V3 VxAB = cross(dir, AB);
    const float ab2 = dot(AB, AB);
    const float a = dot(VxAB, VxAB);
    if (a == 0.f) return;
    const float b = 2.f * dot(VxAB, AOxAB);
    const float c = dot(AOxAB, AOxAB) - ((r * r) * ab2);
    const float rad = b * b - 4.f * a * c;
    if (rad < 0.f) return;
    const float srad = sqrtf(rad);
    const float dVAB = dot(dir, AB);
    if (dVAB == 0.f) return;
    const float rVAB = 1.0f / dVAB;
    const float tA = dot(AB, A) * rVAB, tB = dot(AB, B) * rVAB;
    const float r2a = 1.0f / (2.f * a);
    const float c_in = approx + fmax_((-b - srad) * r2a, fmin_(tA, tB));
    const float c_out = approx + fmin_((-b + srad) * r2a, fmax_(tA, tB));
    if (c_in < c_out) {
        t_in = c_in;
        t_out = c_out;
    }
}
static __device__ __forceinline__ bool line_test(V3 org, V3 dir, V3 A, V3 B, float r, float t0, float tfar, float &t) {
    float t_in = INFINITY, t_out = -INFINITY;
    line_cylinder(org, dir, A, B, r, t_in, t_out);
    line_sphere(org, dir, A, r, t_in, t_out);
    line_sphere(org, dir, B, r, t_in, t_out);
    if (!(t_in < t_out)) return false;
    if (t_in > t0 && t_in < tfar) { t = t_in; return true; }
    if (t_out > t0 && t_out < tfar) { t = t_out; return true; }
    return false;
}

// --------------------------------------------------------- BVH8 traversal
struct GeoHit {
    float t, u, v;
    uint32_t prim;   // global primitive id (with kSphereBit for spheres)
};

// Packed pairs of floats (element 0 in the low word) for the f32x2
// arithmetic of sm_100-family GPUs: one instruction does two element-wise
// round-to-nearest operations.
__device__ __forceinline__ uint64_t f2pack(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }
__device__ __forceinline__ uint64_t f2dup(float a) { return f2pack(__float_as_uint(a), __float_as_uint(a)); }
__device__ __forceinline__ float f2get(uint64_t v, int h) {
    return __uint_as_float(h ? (uint32_t)(v >> 32) : (uint32_t)v);
}
__device__ __forceinline__ uint64_t f2add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// Both 16-bit fields of w as exact floats, packed: each field placed in the
// mantissa of 2^23 (bits 0x4B000000 | q) minus 2^23 -- full-rate byte
// permutes and one packed add instead of integer-to-float conversions.
__device__ __forceinline__ uint64_t q16x2(uint32_t w) {
    return f2add(f2pack(__byte_perm(w, 0x4B000000u, 0x7610), __byte_perm(w, 0x4B000000u, 0x7632)),
                 0xCB000000CB000000ull);   // - 2^23 in both halves
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Slab test of the 8 quantised child boxes of one BVH8 node (first two
// 16-byte words n0, n1 and the 96 bytes of planes q) for a ray with origin
// org and reciprocal direction (idx, idy, idz) over [t0, tmax].  A plane at
// quantised position k lies at origin + k * 2^e, so its distance is
// k * (2^e * id) + (origin - org) * id, one fused multiply-add.  The two
// children of a slot pair share each 32-bit plane word, so a pair is decoded
// and tested with packed f32x2 operations (the same round-to-nearest FMA per
// child).  Outputs: key[i] = entry distance (low 3 bits replaced by the slot)
// of a hit inner child, else 0xffffffff; leafhits = mask of hit leaf slots.
__device__ __forceinline__ void node_children(float4 n0, float4 n1, const uint4 *q, V3 org, float idx, float idy,
                                              float idz, float t0, float tmax, uint32_t key[8], int &n_inner,
                                              uint32_t &leafhits) {
    const uint32_t *W = &q[0].x;   // lo x, y, z planes: words 0-11; hi planes: words 12-23
    const bool sx = idx < 0.0f, sy = idy < 0.0f, sz = idz < 0.0f;
    const uint32_t e4 = __float_as_uint(n1.y);
    const uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
    const float scx = __uint_as_float((e4 & 0xffu) << 23);
    const float scy = __uint_as_float(((e4 >> 8) & 0xffu) << 23);
    const float scz = __uint_as_float(((e4 >> 16) & 0xffu) << 23);
    const uint32_t imask = e4 >> 24;
    const uint64_t Ax = f2dup(scx * idx), Bx = f2dup((n0.x - org.x) * idx);
    const uint64_t Ay = f2dup(scy * idy), By = f2dup((n0.y - org.y) * idy);
    const uint64_t Az = f2dup(scz * idz), Bz = f2dup((n0.z - org.z) * idz);
    uint32_t hitm = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t lx = W[k], ly = W[4 + k], lz = W[8 + k], hx = W[12 + k], hy = W[16 + k], hz = W[20 + k];
        const uint64_t txa = f2fma(q16x2(sx ? hx : lx), Ax, Bx), txb = f2fma(q16x2(sx ? lx : hx), Ax, Bx);
        const uint64_t tya = f2fma(q16x2(sy ? hy : ly), Ay, By), tyb = f2fma(q16x2(sy ? ly : hy), Ay, By);
        const uint64_t tza = f2fma(q16x2(sz ? hz : lz), Az, Bz), tzb = f2fma(q16x2(sz ? lz : hz), Az, Bz);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int i = 2 * k + h;
            float tn = fmaxf(max3f(f2get(txa, h), f2get(tya, h), f2get(tza, h)), t0);
            float tf = fminf(min3f(f2get(txb, h), f2get(tyb, h), f2get(tzb, h)), tmax);
            if (tn <= tf * 1.00000048f + 1e-30f) hitm |= 1u << i;
            key[i] = (__float_as_uint(tn) & ~7u) | (uint32_t)i;
        }
    }
    // Empty slots carry meta 0xff; every filled slot's meta byte is below
    // 0x80 (inner: rank < 8; leaf: (count - 1) << 5 | offset < 128), so the
    // bytes' high bits are the empty mask: gather bits 7, 15, 23, 31 to
    // bits 21-24 with one multiply (the partial products do not overlap).
    const uint32_t elo = ((((meta_lo >> 7) & 0x01010101u) * 0x00204081u) >> 21) & 0xfu;
    const uint32_t ehi = ((((meta_hi >> 7) & 0x01010101u) * 0x00204081u) >> 21) & 0xfu;
    hitm &= ~(elo | (ehi << 4));
    const uint32_t inner = hitm & imask;
    leafhits = hitm & ~imask;
    n_inner = __popc(inner);
#pragma unroll
    for (int i = 0; i < 8; i++)
        if (!((inner >> i) & 1u)) key[i] = 0xffffffffu;
}

// 32-bit compare-exchange for the sorting network below.
__device__ __forceinline__ void cas(uint32_t &a, uint32_t &b) {
    uint32_t lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

// Closest hit in (t0, tfar) with ties broken by the smaller primitive id.
// ANY: return at the first accepted hit.  Per wide node: the 8 child boxes
// are tested from the quantised planes with one fused multiply-add per slab;
// leaf children are intersected at once; hit internal children are ordered
// near to far by a 19-comparator sorting network over 32-bit keys (entry
// distance with the child slot in the low 3 bits -- non-negative floats
// order like their bit patterns), the nearest is visited next and the rest
// go on a stack of (node, entry distance) pairs.  Everything stays in
// registers except the stack.
template <bool ANY>
__device__ __noinline__ bool bvh_closest(const DevScene &S, V3 org, V3 dir, float t0, float tfar, GeoHit &h,
                                         unsigned &nodes, unsigned &tris, unsigned &sphs, int &ovf) {
    if (!S.nodes) return false;
    const float idx = 1.0f / dir.x, idy = 1.0f / dir.y, idz = 1.0f / dir.z;
    h.t = tfar;
    h.prim = 0xffffffffu;
    bool found = false;
    uint2 stack[64];
    int sp = 0;
    uint32_t cur = 0;
    float cur_tn = t0;
    for (;;) {
        if (cur_tn <= h.t) {
            const float4 *np = reinterpret_cast<const float4 *>(S.nodes + cur);
            float4 n0 = __ldg(np), n1 = __ldg(np + 1);
            uint32_t child_base = __float_as_uint(n0.w);
            uint32_t prim_base = __float_as_uint(n1.x);
            uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
            uint4 q[6];
#pragma unroll
            for (int k = 0; k < 6; k++) q[k] = __ldg(reinterpret_cast<const uint4 *>(np + 2 + k));
            nodes++;
            uint32_t key[8];
            uint32_t leafhits;
            int n_inner;
            node_children(n0, n1, q, org, idx, idy, idz, t0, h.t, key, n_inner, leafhits);
            while (leafhits) {
                int i = __ffs(leafhits) - 1;
                leafhits &= leafhits - 1;
                uint32_t mb = (i < 4 ? meta_lo >> (8 * i) : meta_hi >> (8 * (i - 4))) & 0xffu;
                uint32_t s = prim_base + (mb & 31u);
                uint32_t cnt = (mb >> 5) + 1;
                for (uint32_t k = 0; k < cnt; k++, s++) {
                    const float4 *rp = S.slots + 3 * (size_t)s;
                    float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
                    uint32_t id = __float_as_uint(r0.w);
                    float t, u = 0.0f, v = 0.0f;
                    bool ok;
                    if (id & kLineBit) {
                        tris++;   // path-line segments count as primitive tests with triangles
                        ok = line_test(org, dir, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), r1.w, t0, tfar, t);
                    } else if (id & kSphereBit) {
                        sphs++;
                        ok = sph_test(org, dir, v3(r0.x, r0.y, r0.z), r1.x, r1.y, t0, tfar, t);
                    } else {
                        tris++;
                        float4 r2 = __ldg(rp + 2);
                        ok = tri_test(org, dir, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), v3(r2.x, r2.y, r2.z), t, u,
                                      v) &&
                             t > t0 && t < tfar;
                    }
                    if (ok && (t < h.t || (t == h.t && id < h.prim))) {
                        h.t = t; h.u = u; h.v = v; h.prim = id;
                        found = true;
                        if (ANY) return true;
                    }
                }
            }
            if (n_inner) {
                // sorting network for 8 keys (Batcher, 19 comparators)
                cas(key[0], key[1]); cas(key[2], key[3]); cas(key[4], key[5]); cas(key[6], key[7]);
                cas(key[0], key[2]); cas(key[1], key[3]); cas(key[4], key[6]); cas(key[5], key[7]);
                cas(key[1], key[2]); cas(key[5], key[6]); cas(key[0], key[4]); cas(key[3], key[7]);
                cas(key[1], key[5]); cas(key[2], key[6]);
                cas(key[1], key[4]); cas(key[3], key[6]);
                cas(key[2], key[4]); cas(key[3], key[5]);
                cas(key[3], key[4]);
#pragma unroll
                for (int j = 7; j >= 1; j--) {
                    if (j < n_inner) {
                        uint32_t slot = key[j] & 7u;
                        const uint32_t mb = slot;   // inner children sit in the first slots, in rank order
                        if (sp < 64) stack[sp++] = make_uint2(child_base + mb, key[j] & ~7u);
                        else ovf = 1;   // reported as GXY_ERR_OVERFLOW by the host
                    }
                }
                uint32_t slot = key[0] & 7u;
                const uint32_t mb = slot;   // inner children sit in the first slots, in rank order
                cur = child_base + mb;
                cur_tn = __uint_as_float(key[0] & ~7u);
                continue;
            }
        }
        if (sp == 0) break;
        uint2 e = stack[--sp];
        cur = e.x;
        cur_tn = __uint_as_float(e.y);
    }
    return found;
}

// ------------------------------------------------------------------------
// Resumable form of bvh_closest<false> (same node order, same tests, same
// tie rule): trav_step visits one wide node per call, so a persistent lane
// can interleave traversal steps of successive rays.
struct TravState {                   // scalars only, so it lives in registers
    V3 org, dir;
    float idx, idy, idz;
    float t0, tfar, cur_tn;
    uint32_t cur;
    int sp;
    GeoHit h;
    bool found;
};

__device__ __forceinline__ bool trav_init(const DevScene &S, TravState &T, V3 org, V3 dir, float t0, float tfar) {
    T.org = org;
    T.dir = dir;
    T.idx = 1.0f / dir.x;
    T.idy = 1.0f / dir.y;
    T.idz = 1.0f / dir.z;
    T.t0 = t0;
    T.tfar = tfar;
    T.h.t = tfar;
    T.h.prim = 0xffffffffu;
    T.found = false;
    T.sp = 0;
    T.cur = 0;
    T.cur_tn = t0;
    return S.nodes == nullptr;   // done at once without geometry
}

// One node visit; returns true when the traversal is complete.
// Traversal stack of (node, entry distance) pairs, 64 entries deep, in the
// lane's local memory.  (A variant with the first 16 entries in shared
// memory measured slower: the shared allocation takes L1 capacity that the
// node fetches use.)
struct LocalStack {
    uint2 *p;
    __device__ __forceinline__ uint2 get(int i) const { return p[i]; }
    __device__ __forceinline__ void set(int i, uint2 v) { p[i] = v; }
};
// LINES: the scene has path-line segments (their test is compiled in only
// then, so the register budget of the common case is unchanged).
// stop_below: the query may end at the first accepted hit nearer than this
// (the caller needs no more than "some hit before stop_below" then).
template <bool LINES, class STACK>
__device__ __forceinline__ bool trav_step(const DevScene &S, TravState &T, STACK &stack, unsigned &nodes,
                                          unsigned &tris, unsigned &sphs, int &ovf, float stop_below = -INFINITY) {
    while (!(T.cur_tn <= T.h.t)) {
        if (T.sp == 0) return true;
        uint2 e = stack.get(--T.sp);
        T.cur = e.x;
        T.cur_tn = __uint_as_float(e.y);
    }
    const V3 org = T.org, dir = T.dir;
    const float idx = T.idx, idy = T.idy, idz = T.idz, t0 = T.t0, tfar = T.tfar;
    const float4 *np = reinterpret_cast<const float4 *>(S.nodes + T.cur);
    float4 n0 = __ldg(np), n1 = __ldg(np + 1);
    uint32_t child_base = __float_as_uint(n0.w);
    uint32_t prim_base = __float_as_uint(n1.x);
    uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
    uint4 q[6];
#pragma unroll
    for (int k = 0; k < 6; k++) q[k] = __ldg(reinterpret_cast<const uint4 *>(np + 2 + k));
    nodes++;
    uint32_t key[8];
    uint32_t leafhits;
    int n_inner;
    node_children(n0, n1, q, org, idx, idy, idz, t0, T.h.t, key, n_inner, leafhits);
    while (leafhits) {
        int i = __ffs(leafhits) - 1;
        leafhits &= leafhits - 1;
        uint32_t mb = (i < 4 ? meta_lo >> (8 * i) : meta_hi >> (8 * (i - 4))) & 0xffu;
        uint32_t s = prim_base + (mb & 31u);
        uint32_t cnt = (mb >> 5) + 1;
        for (uint32_t k = 0; k < cnt; k++, s++) {
            const float4 *rp = S.slots + 3 * (size_t)s;
            float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
            uint32_t id = __float_as_uint(r0.w);
            float t, u = 0.0f, v = 0.0f;
            bool ok;
            if (LINES && (id & kLineBit)) {
                tris++;   // path-line segments count as primitive tests with triangles
                ok = line_test(org, dir, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), r1.w, t0, tfar, t);
            } else if (id & kSphereBit) {
                sphs++;
                ok = sph_test(org, dir, v3(r0.x, r0.y, r0.z), r1.x, r1.y, t0, tfar, t);
            } else {
                tris++;
                float4 r2 = __ldg(rp + 2);
                ok = tri_test(org, dir, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), v3(r2.x, r2.y, r2.z), t, u, v) &&
                     t > t0 && t < tfar;
            }
            if (ok && (t < T.h.t || (t == T.h.t && id < T.h.prim))) {
                T.h.t = t; T.h.u = u; T.h.v = v; T.h.prim = id;
                T.found = true;
            }
        }
    }
    if (T.found && T.h.t < stop_below) return true;
    if (n_inner) {
        cas(key[0], key[1]); cas(key[2], key[3]); cas(key[4], key[5]); cas(key[6], key[7]);
        cas(key[0], key[2]); cas(key[1], key[3]); cas(key[4], key[6]); cas(key[5], key[7]);
        cas(key[1], key[2]); cas(key[5], key[6]); cas(key[0], key[4]); cas(key[3], key[7]);
        cas(key[1], key[5]); cas(key[2], key[6]);
        cas(key[1], key[4]); cas(key[3], key[6]);
        cas(key[2], key[4]); cas(key[3], key[5]);
        cas(key[3], key[4]);
#pragma unroll
        for (int j = 7; j >= 1; j--) {
            if (j < n_inner) {
                uint32_t slot = key[j] & 7u;
                const uint32_t mb = slot;   // inner children sit in the first slots, in rank order
                if (T.sp < 64) stack.set(T.sp++, make_uint2(child_base + mb, key[j] & ~7u));
                else ovf = 1;
            }
        }
        uint32_t slot = key[0] & 7u;
        const uint32_t mb = slot;   // inner children sit in the first slots, in rank order
        T.cur = child_base + mb;
        T.cur_tn = __uint_as_float(key[0] & ~7u);
        return false;
    }
    if (T.sp == 0) return true;
    uint2 e = stack.get(--T.sp);
    T.cur = e.x;
    T.cur_tn = __uint_as_float(e.y);
    return false;
}


// ------------------------------------------------------------------------
// Warp-cooperative closest hit for the 32 rays of a warp (one per lane;
// active = false gives the lane an empty interval), for coherent rays such
// as camera rays of an 8x4 pixel tile.  The warp walks one node stack in
// shared memory (wstack: 64 entries of this warp): every lane tests its own
// ray against the 8 children of the same node, so each node line is fetched
// once for the warp; a child any lane enters is visited, nearest first by
// the smallest entry distance over the lanes; a stacked node is skipped once
// that distance lies beyond every lane's current hit.  Each lane tests the
// primitives of the leaves its own ray enters, with the same tests and tie
// rule as bvh_closest, so it finds the same closest hit.  All 32 lanes call
// it together.  nodes counts node lines fetched (once per warp).
template <bool LINES>
__device__ __forceinline__ bool packet_closest(const DevScene &S, V3 org, V3 dir, float t0, float tfar, bool active,
                                               uint2 *wstack, GeoHit &h, unsigned &nodes, unsigned &tris,
                                               unsigned &sphs, int &ovf) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    if (!active) {   // an interval no box test passes
        org = v3(0.f, 0.f, 0.f);
        dir = v3(1.f, 1.f, 1.f);
        t0 = 0.f;
        tfar = -1.f;
    }
    const float idx = 1.0f / dir.x, idy = 1.0f / dir.y, idz = 1.0f / dir.z;
    h.t = tfar;
    h.u = h.v = 0.f;
    h.prim = 0xffffffffu;
    bool found = false;
    if (!S.nodes) return false;
    int sp = 0;
    uint32_t cur = 0;
    for (;;) {
        const float4 *np = reinterpret_cast<const float4 *>(S.nodes + cur);
        float4 n0 = __ldg(np), n1 = __ldg(np + 1);
        uint4 q[6];
#pragma unroll
        for (int k = 0; k < 6; k++) q[k] = __ldg(reinterpret_cast<const uint4 *>(np + 2 + k));
        if (lane == 0) nodes++;
        const uint32_t child_base = __float_as_uint(n0.w), prim_base = __float_as_uint(n1.x);
        const uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
        uint32_t key[8];
        uint32_t leafhits;
        int n_inner;
        node_children(n0, n1, q, org, idx, idy, idz, t0, h.t, key, n_inner, leafhits);
        while (leafhits) {
            int i = __ffs(leafhits) - 1;
            leafhits &= leafhits - 1;
            uint32_t mb = (i < 4 ? meta_lo >> (8 * i) : meta_hi >> (8 * (i - 4))) & 0xffu;
            uint32_t s = prim_base + (mb & 31u);
            uint32_t cnt = (mb >> 5) + 1;
            for (uint32_t k = 0; k < cnt; k++, s++) {
                const float4 *rp = S.slots + 3 * (size_t)s;
                float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
                uint32_t id = __float_as_uint(r0.w);
                float t, u = 0.0f, v = 0.0f;
                bool ok;
                if (LINES && (id & kLineBit)) {
                    tris++;
                    ok = line_test(org, dir, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), r1.w, t0, tfar, t);
                } else if (id & kSphereBit) {
                    sphs++;
                    ok = sph_test(org, dir, v3(r0.x, r0.y, r0.z), r1.x, r1.y, t0, tfar, t);
                } else {
                    tris++;
                    float4 r2 = __ldg(rp + 2);
                    ok = tri_test(org, dir, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), v3(r2.x, r2.y, r2.z), t, u, v) &&
                         t > t0 && t < tfar;
                }
                if (ok && (t < h.t || (t == h.t && id < h.prim))) {
                    h.t = t; h.u = u; h.v = v; h.prim = id;
                    found = true;
                }
            }
        }
        // children entered by any lane, keyed by the nearest entry over the
        // lanes; lane j < 8 holds slot j's key and its rank among the 8 (the
        // keys of entered children are distinct -- the slot is in the low
        // bits -- and 0xffffffff marks the others, which rank last)
        uint32_t m[8];
#pragma unroll
        for (int i = 0; i < 8; i++) m[i] = __reduce_min_sync(FULL, key[i]);
        uint32_t mine = m[0];
#pragma unroll
        for (int i = 1; i < 8; i++)
            if (lane == i) mine = m[i];
        const bool entered = lane < 8 && mine != 0xffffffffu;
        const int cnt = __popc(__ballot_sync(FULL, entered));
        if (cnt) {
            int rank = 0;
#pragma unroll
            for (int i = 0; i < 8; i++) rank += m[i] < mine ? 1 : 0;
            // far-to-near onto the stack: rank cnt-1 deepest ... rank 1 on
            // top; inner children sit in the first slots, in rank order, so
            // slot j's node is child_base + j
            if (sp + cnt - 1 > 64) {
                ovf = 1;
            } else {
                if (entered && rank >= 1) wstack[sp + (cnt - 1 - rank)] = make_uint2(child_base + (mine & 7u), mine & ~7u);
                sp += cnt - 1;
            }
            __syncwarp();
            cur = child_base + (__reduce_min_sync(FULL, entered ? mine : 0xffffffffu) & 7u);
            continue;
        }
        // pop the nearest stacked node some lane may still need
        const unsigned far = __reduce_max_sync(FULL, __float_as_uint(fmaxf(h.t, 0.0f)));
        bool got = false;
        while (sp > 0) {
            uint2 e = wstack[--sp];
            if (e.y <= far) {
                cur = e.x;
                got = true;
                break;
            }
        }
        __syncwarp();
        if (!got) break;
    }
    return found;
}

}  // namespace gxy

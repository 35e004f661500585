// gxy_oracle.cpp -- CPU restatement of Galaxy's ray-processing path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: a scalar C++
// restatement of the reference algorithm, used by tests/, by the smoke check
// and by bench.py's CPU-baseline leg.  Nothing in the product library links
// or calls it.  It shares no code with galaxy_gb300/csrc; the only common
// piece is the C struct layout of include/gxy_gpu.h (the interface).
//
// Parity status: pinned perceptually against Galaxy's own gold images
// (tests/golden/golds, rendered by gxywriter at 512x512 from the radial
// volumes) -- see tests/test_oracle_golds.py.  At ray/hit/sample level the
// reference's arithmetic lives in OSPRay 1.8.5 / Embree 3.6.1, which are not
// in the Galaxy tree; the definitions used for those call sites are stated
// below (TF lookup, trilinear sampling, gradient, normalize+face-forward,
// triangle and sphere tests) and are applied identically by the GPU path.
//
// Every function cites the Galaxy source it restates (paths inside the
// Galaxy tree).  GXY_REVERSE_LIGHTING is ON (CMakeLists.txt:66 default).
//
// Arithmetic rules: compile with -ffp-contract=off (no fused multiply-add),
// IEEE division and sqrt, evaluation order as written.

#include "../include/gxy_gpu.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <thread>
#include <vector>

namespace gxo {

// ------------------------------------------------------------------ vectors
template <class T> struct V3 {
    T x, y, z;
};
template <class T> static inline V3<T> mk(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> static inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> static inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> static inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> static inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> static inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> static inline V3<T> neg(V3<T> a) { return {-a.x, -a.y, -a.z}; }
// normalize: v * (1/sqrt(v.v)); zero vectors are returned unchanged.
template <class T> static inline V3<T> normalize(V3<T> a) {
    T l2 = dot(a, a);
    if (l2 == T(0)) return a;
    T inv = T(1) / std::sqrt(l2);
    return inv * a;
}
typedef V3<float> F3;
typedef V3<double> D3;
template <class T> static inline V3<T> tov(F3 a) { return {(T)a.x, (T)a.y, (T)a.z}; }

// Galaxy's own normalize (src/data/dtypes.h:164): d = len; d = 1.0/d (double); v *= d.
static inline F3 gxy_normalize(F3 a) {
    float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    if (l != 0.0f) {
        float d = (float)(1.0 / (double)l);
        a.x *= d; a.y *= d; a.z *= d;
    }
    return a;
}

// ------------------------------------------------------------- AO tables
// UV.ih:21-58 holds 256 randomU (base-2 radical inverse) and 256 randomV
// (base-3 radical inverse) values printed with 6 significant digits.  They are
// regenerated here: the radical inverse is accumulated in float32 and the
// value is rounded through "%.6g" (checked entry by entry against the tables
// in tests/golden/ao_tables.json).
static float radical_inverse_f32(int i, int base) {
    float inv = 1.0f / (float)base, f = inv, r = 0.0f;
    while (i > 0) {
        r = r + f * (float)(i % base);
        f = f * inv;
        i /= base;
    }
    return r;
}
struct AOTables {
    float u[256], v[256];
    float cos2pu[256], sin2pu[256], sq1mv[256], sqv[256];
    AOTables() {
        char buf[64];
        for (int i = 0; i < 256; i++) {
            snprintf(buf, sizeof buf, "%.6g", (double)radical_inverse_f32(i, 2));
            u[i] = strtof(buf, nullptr);
            snprintf(buf, sizeof buf, "%.6g", (double)radical_inverse_f32(i, 3));
            v[i] = strtof(buf, nullptr);
            float a = 6.28318530717958647692f * u[i];
            cos2pu[i] = cosf(a);
            sin2pu[i] = sinf(a);
            sq1mv[i] = sqrtf(1.0f - v[i]);
            sqv[i] = sqrtf(v[i]);
        }
    }
};
static const AOTables &ao_tables() {
    static AOTables t;
    return t;
}

// ------------------------------------------------------ transfer function
// OSPRay 1.8.5 piecewise_linear lookup at the call sites TraceRays.ispc:238,
// 303,522,529 (OSPRay is not vendored; definition stated here): NaN -> 0;
// clamp to the first/last entry outside valueRange; otherwise map to
// [0,255] as (v - r0) * (255 / (r1 - r0)), floor, and interpolate with the
// next entry.
template <class T> static V3<T> tf_color(const gxy_tf &tf, T v) {
    if (std::isnan(v)) return {T(0), T(0), T(0)};
    const float *c = tf.colors;
    if (v <= T(tf.range[0])) return {T(c[0]), T(c[1]), T(c[2])};
    if (v >= T(tf.range[1])) return {T(c[765]), T(c[766]), T(c[767])};
    T k = T(255) / (T(tf.range[1]) - T(tf.range[0]));
    T f = (v - T(tf.range[0])) * k;
    int i = (int)std::floor(f);
    if (i > 254) i = 254;
    if (i < 0) i = 0;
    T rem = f - T(i);
    T a = T(1) - rem;
    return {a * T(c[3 * i]) + rem * T(c[3 * i + 3]), a * T(c[3 * i + 1]) + rem * T(c[3 * i + 4]),
            a * T(c[3 * i + 2]) + rem * T(c[3 * i + 5])};
}
template <class T> static T tf_opacity(const gxy_tf &tf, T v) {
    if (std::isnan(v)) return T(0);
    const float *o = tf.opacities;
    if (v <= T(tf.range[0])) return T(o[0]);
    if (v >= T(tf.range[1])) return T(o[255]);
    T k = T(255) / (T(tf.range[1]) - T(tf.range[0]));
    T f = (v - T(tf.range[0])) * k;
    int i = (int)std::floor(f);
    if (i > 254) i = 254;
    if (i < 0) i = 0;
    T rem = f - T(i);
    return (T(1) - rem) * T(o[i]) + rem * T(o[i + 1]);
}

// ---------------------------------------------------------------- volume
// OSPRay shared_structured_volume sample at TraceRays.ispc:234,322 (created at
// OsprayVolume.cpp:25-52).  Definition: grid coordinate g = (p - origin) * (1/delta)
// over the whole dataset grid, clamped to [0, counts-1) (upper bound the float
// just below counts-1), lower corner = (int)g, trilinear interpolation in the
// order x, then y, then z with lerp(a,b,f) = (1-f)*a + f*b -- the same scheme as
// Galaxy's own CPU sampler Volume::Sample (Volume.cpp:546-590).  Sampling the
// dataset grid rather than a ghosted brick copy gives the same values for
// every point inside a brick's box, because the brick's 1-voxel ghost shell
// holds exactly the dataset voxels the stencil reaches.
struct Vol {
    const gxy_volume_vis *vis;
    const float *data;
    int nx, ny, nz;
    float ox, oy, oz, dx, dy, dz;
    float ux, uy, uz;  // clamp upper bounds
    float ix, iy, iz;  // 1/delta
};
template <class T> static T vol_sample(const Vol &v, V3<T> p) {
    T gx, gy, gz;
    if (sizeof(T) == sizeof(float)) {
        gx = (p.x - T(v.ox)) * T(v.ix);
        gy = (p.y - T(v.oy)) * T(v.iy);
        gz = (p.z - T(v.oz)) * T(v.iz);
    } else {
        gx = (p.x - T(v.ox)) / T(v.dx);
        gy = (p.y - T(v.oy)) / T(v.dy);
        gz = (p.z - T(v.oz)) / T(v.dz);
    }
    if (!(gx >= T(0))) gx = T(0);
    if (!(gy >= T(0))) gy = T(0);
    if (!(gz >= T(0))) gz = T(0);
    if (gx > T(v.ux)) gx = T(v.ux);
    if (gy > T(v.uy)) gy = T(v.uy);
    if (gz > T(v.uz)) gz = T(v.uz);
    int ix = (int)gx, iy = (int)gy, iz = (int)gz;
    T fx = gx - T(ix), fy = gy - T(iy), fz = gz - T(iz);
    size_t sx = 1, sy = (size_t)v.nx, sz = (size_t)v.nx * (size_t)v.ny;
    const float *b = v.data + (size_t)iz * sz + (size_t)iy * sy + (size_t)ix;
    T v000 = b[0], v100 = b[sx], v010 = b[sy], v110 = b[sy + sx];
    T v001 = b[sz], v101 = b[sz + sx], v011 = b[sz + sy], v111 = b[sz + sy + sx];
    T ax = T(1) - fx;
    T v00 = ax * v000 + fx * v100;
    T v10 = ax * v010 + fx * v110;
    T v01 = ax * v001 + fx * v101;
    T v11 = ax * v011 + fx * v111;
    T ay = T(1) - fy;
    T v0 = ay * v00 + fy * v10;
    T v1 = ay * v01 + fy * v11;
    return (T(1) - fz) * v0 + fz * v1;
}
// OSPRay computeGradient at TraceRays.ispc:299.  Definition: central
// differences one grid spacing either side, divided by twice the spacing.
static F3 vol_gradient(const Vol &v, F3 p) {
    F3 g;
    g.x = (vol_sample<float>(v, mk(p.x + v.dx, p.y, p.z)) - vol_sample<float>(v, mk(p.x - v.dx, p.y, p.z))) /
          (2.0f * v.dx);
    g.y = (vol_sample<float>(v, mk(p.x, p.y + v.dy, p.z)) - vol_sample<float>(v, mk(p.x, p.y - v.dy, p.z))) /
          (2.0f * v.dy);
    g.z = (vol_sample<float>(v, mk(p.x, p.y, p.z + v.dz)) - vol_sample<float>(v, mk(p.x, p.y, p.z - v.dz))) /
          (2.0f * v.dz);
    return g;
}

// ------------------------------------------------------------------ boxes
struct Box {
    F3 lo, hi;
};
// Box::intersect (src/data/Box.cpp:107-150).
static bool box_intersect(const Box &b, F3 org, F3 dir, float &tmin, float &tmax) {
    tmin = (b.lo.x - org.x) / dir.x;
    tmax = (b.hi.x - org.x) / dir.x;
    if (tmin > tmax) std::swap(tmin, tmax);
    if (tmax < 0) return false;
    float tymin = (b.lo.y - org.y) / dir.y;
    float tymax = (b.hi.y - org.y) / dir.y;
    if (tymin > tymax) std::swap(tymin, tymax);
    if (tymax < 0) return false;
    if ((tmin > tymax) || (tymin > tmax)) return false;
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = (b.lo.z - org.z) / dir.z;
    float tzmax = (b.hi.z - org.z) / dir.z;
    if (tzmin > tzmax) std::swap(tzmin, tzmax);
    if (tzmax < 0) return false;
    if ((tmin > tzmax) || (tzmin > tmax)) return false;
    if (tzmin > tmin) tmin = tzmin;
    if (tzmax < tmax) tmax = tzmax;
    if (tmin < 0) tmin = 0;
    return true;
}
// Box::exit_face (src/data/Box.cpp:84-97).
static int box_exit_face(const Box &b, F3 o, F3 d) {
    float tx = (d.x > 0.0001f) ? ((b.hi.x - o.x) / d.x) : (d.x < -0.0001f) ? ((b.lo.x - o.x) / d.x) : FLT_MAX;
    float ty = (d.y > 0.0001f) ? ((b.hi.y - o.y) / d.y) : (d.y < -0.0001f) ? ((b.lo.y - o.y) / d.y) : FLT_MAX;
    float tz = (d.z > 0.0001f) ? ((b.hi.z - o.z) / d.z) : (d.z < -0.0001f) ? ((b.lo.z - o.z) / d.z) : FLT_MAX;
    if (tx < 0) tx = FLT_MAX;
    if (ty < 0) ty = FLT_MAX;
    if (tz < 0) tz = FLT_MAX;
    if (tx < ty && tx < tz) return (d.x < 0) ? 0 : 1;
    else if (ty < tz) return (d.y < 0) ? 2 : 3;
    else return (d.z < 0) ? 4 : 5;
}
// MyIntersectBox (TraceRays.ispc:90-106) with rcp(d) = 1/d.
static void my_intersect_box(F3 org, F3 dir, const Box &b, float &t0, float &t1) {
    F3 r = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    F3 mins = mk((b.lo.x - org.x) * r.x, (b.lo.y - org.y) * r.y, (b.lo.z - org.z) * r.z);
    F3 maxs = mk((b.hi.x - org.x) * r.x, (b.hi.y - org.y) * r.y, (b.hi.z - org.z) * r.z);
    t0 = std::max(std::min(mins.x, maxs.x), std::max(std::min(mins.y, maxs.y), std::min(mins.z, maxs.z)));
    t1 = std::min(std::max(mins.x, maxs.x), std::min(std::max(mins.y, maxs.y), std::max(mins.z, maxs.z)));
}

// ------------------------------------------------------------- geometry
// Primitive ids: all triangles of set 0, set 1, ..., then all spheres of
// particle set 0, 1, ..., then all path-line segments of set 0, 1, ...
// Closest hit = smallest t in (t0, tfar), ties broken by the smaller
// primitive id.
struct Geo {
    struct TriSet { const gxy_triangles_vis *v; int64_t base; };
    struct SphSet { const gxy_particles_vis *v; int64_t base; float eps; };
    struct LineSet { const gxy_pathlines_vis *v; int64_t base; std::vector<float> rad; };
    std::vector<TriSet> tsets;
    std::vector<SphSet> ssets;
    std::vector<LineSet> lsets;
    int64_t n_tri = 0, n_sph = 0, n_seg = 0;
    // flat per-primitive arrays
    std::vector<F3> tv0, tv1, tv2;
    std::vector<float> srad;
    std::vector<F3> scen;
    std::vector<F3> la, lb;      // segment end points
    std::vector<float> lr;       // segment capsule radius (radius0 of its set)
    // binary BVH
    struct Node { float lo[3], hi[3]; int32_t left, right, first, count; };
    std::vector<Node> nodes;
    std::vector<int64_t> order;
};

static float sphere_radius(const gxy_particles_vis &p, int64_t i) {
    // DataDrivenSpheres.ispc:104-116
    if (p.value0 != p.value1 && p.data) {
        float d = (p.data[i] - p.value0) / (p.value1 - p.value0);
        if (d > 1) return p.radius1;
        else if (d < 0) return p.radius0;
        else return p.radius0 + d * (p.radius1 - p.radius0);
    }
    return p.radius0;
}
// MAP_RADIUS (DataDrivenPathLines.cpp:11-19): per-vertex path-line radius;
// without data every vertex has radius0.
static float pathline_radius(const gxy_pathlines_vis &q, int64_t i) {
    if (q.value0 == q.value1 || !q.data) return q.radius0;
    float R = (q.data[i] - q.value0) / (q.value1 - q.value0);
    return (R <= 0.0f) ? q.radius0 : (R >= 1.0f) ? q.radius1 : q.radius0 + R * (q.radius1 - q.radius0);
}
// DataDrivenSpheresGeometry_set (DataDrivenSpheres.ispc:211-220).
static float sphere_epsilon(float r0) {
    float e = logf(r0);
    if (e < 0.f) e = -1.f / e;
    if (e > r0 / 100.0f) e = r0 / 100.0f;
    return e;
}

static void prim_bounds(const Geo &g, int64_t p, float lo[3], float hi[3]) {
    if (p < g.n_tri) {
        F3 a = g.tv0[p], b = g.tv1[p], c = g.tv2[p];
        lo[0] = std::min({a.x, b.x, c.x}); hi[0] = std::max({a.x, b.x, c.x});
        lo[1] = std::min({a.y, b.y, c.y}); hi[1] = std::max({a.y, b.y, c.y});
        lo[2] = std::min({a.z, b.z, c.z}); hi[2] = std::max({a.z, b.z, c.z});
    } else if (p < g.n_tri + g.n_sph) {
        int64_t s = p - g.n_tri;
        F3 c = g.scen[s];
        float r = g.srad[s];
        lo[0] = c.x - r; lo[1] = c.y - r; lo[2] = c.z - r;
        hi[0] = c.x + r; hi[1] = c.y + r; hi[2] = c.z + r;
    } else {
        // DataDrivenPathLines_bounds (DataDrivenPathLines.ispc:37-68)
        int64_t s = p - g.n_tri - g.n_sph;
        F3 a = g.la[s], b = g.lb[s];
        float r = g.lr[s];
        lo[0] = std::min(a.x, b.x) - r; lo[1] = std::min(a.y, b.y) - r; lo[2] = std::min(a.z, b.z) - r;
        hi[0] = std::max(a.x, b.x) + r; hi[1] = std::max(a.y, b.y) + r; hi[2] = std::max(a.z, b.z) + r;
    }
}

static void build_bvh(Geo &g) {
    int64_t n = g.n_tri + g.n_sph + g.n_seg;
    g.order.resize(n);
    for (int64_t i = 0; i < n; i++) g.order[i] = i;
    g.nodes.clear();
    if (n == 0) return;
    std::vector<float> cen(3 * n), blo(3 * n), bhi(3 * n);
    for (int64_t i = 0; i < n; i++) {
        prim_bounds(g, i, &blo[3 * i], &bhi[3 * i]);
        for (int k = 0; k < 3; k++) cen[3 * i + k] = 0.5f * (blo[3 * i + k] + bhi[3 * i + k]);
    }
    struct Item { int32_t node; int64_t first, count; };
    std::vector<Item> st;
    g.nodes.push_back(Geo::Node{});
    st.push_back({0, 0, n});
    while (!st.empty()) {
        Item it = st.back();
        st.pop_back();
        Geo::Node nd{};
        float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int k = 0; k < 3; k++) { nd.lo[k] = FLT_MAX; nd.hi[k] = -FLT_MAX; }
        for (int64_t i = it.first; i < it.first + it.count; i++) {
            int64_t p = g.order[i];
            for (int k = 0; k < 3; k++) {
                nd.lo[k] = std::min(nd.lo[k], blo[3 * p + k]);
                nd.hi[k] = std::max(nd.hi[k], bhi[3 * p + k]);
                clo[k] = std::min(clo[k], cen[3 * p + k]);
                chi[k] = std::max(chi[k], cen[3 * p + k]);
            }
        }
        // pad the box so the slab test can never reject a primitive the
        // primitive test would accept
        for (int k = 0; k < 3; k++) {
            float pad = 1e-5f * (std::fabs(nd.lo[k]) + std::fabs(nd.hi[k])) + 1e-7f;
            nd.lo[k] -= pad;
            nd.hi[k] += pad;
        }
        if (it.count <= 4) {
            nd.left = nd.right = -1;
            nd.first = (int32_t)it.first;
            nd.count = (int32_t)it.count;
            g.nodes[it.node] = nd;
            continue;
        }
        int axis = 0;
        float ext = chi[0] - clo[0];
        for (int k = 1; k < 3; k++)
            if (chi[k] - clo[k] > ext) { ext = chi[k] - clo[k]; axis = k; }
        int64_t mid = it.first + it.count / 2;
        std::nth_element(g.order.begin() + it.first, g.order.begin() + mid, g.order.begin() + it.first + it.count,
                         [&](int64_t a, int64_t b) {
                             float ca = cen[3 * a + axis], cb = cen[3 * b + axis];
                             return ca < cb || (ca == cb && a < b);
                         });
        int32_t l = (int32_t)g.nodes.size();
        g.nodes.push_back(Geo::Node{});
        g.nodes.push_back(Geo::Node{});
        nd.left = l;
        nd.right = l + 1;
        nd.first = nd.count = 0;
        g.nodes[it.node] = nd;
        st.push_back({l, it.first, mid - it.first});
        st.push_back({l + 1, mid, it.first + it.count - mid});
    }
}

struct GeoHit {
    float t;
    int64_t prim;
    float u, v;
};

// Moller-Trumbore with t in (t0, tbest), definition of the Embree triangle
// test behind traceRay (TraceRays.ispc:117; DataDrivenTriangleMesh.cpp:132-139).
static inline bool tri_test(F3 org, F3 dir, F3 v0, F3 v1, F3 v2, float &t, float &u, float &v) {
    F3 e1 = v1 - v0, e2 = v2 - v0;
    F3 pv = cross(dir, e2);
    float det = dot(e1, pv);
    if (det == 0.0f) return false;
    float inv = 1.0f / det;
    F3 tv = org - v0;
    u = dot(tv, pv) * inv;
    if (u < 0.0f || u > 1.0f) return false;
    F3 qv = cross(tv, e1);
    v = dot(dir, qv) * inv;
    if (v < 0.0f || u + v > 1.0f) return false;
    t = dot(e2, qv) * inv;
    return true;
}

// DataDrivenSpheres_intersect_kernel (DataDrivenSpheres.ispc:118-141): returns
// the accepted distance (t_in if in (t0,tfar), else t_out if in (t0+eps,tfar)).
static inline bool sph_test(F3 org, F3 dir, F3 c, float r, float eps, float t0, float tfar, float &t) {
    float approx = dot(c - org, dir);
    F3 close = org + approx * dir;
    F3 A = c - close;
    float a = dot(dir, dir);
    float b = 2.f * dot(dir, A);
    float cc = dot(A, A) - r * r;
    float rad = b * b - 4.f * a * cc;
    if (rad < 0.f) return false;
    float srad = sqrtf(rad);
    float r2a = 1.0f / (2.f * a);
    float tin = (b - srad) * r2a + approx;
    float tout = (b + srad) * r2a + approx;
    if (tin > t0 && tin < tfar) { t = tin; return true; }
    if (tout > t0 + eps && tout < tfar) { t = tout; return true; }
    return false;
}

// DataDrivenPathLines_intersect_kernel (DataDrivenPathLines.ispc:100-203):
// cylinder A-B of radius r clipped at its caps, joined with spheres of radius
// r at A and B, each after moving the origin to an approximate distance;
// rcp/rcpf taken as exact reciprocals.  Accepted distance: t_in if in
// (t0, tfar), else t_out if in (t0, tfar).
static inline void line_sphere(F3 org, F3 dir, F3 c, float r, float &t_in, float &t_out) {
    const float approx = dot(c - org, dir);
    const F3 close = org + approx * dir;
    const F3 A = c - close;
    const float a = dot(dir, dir);
    const float b = -2.f * dot(dir, A);
    const float cc = dot(A, A) - r * r;
    const float rad = b * b - 4.f * a * cc;
    if (rad < 0.f) return;
    const float srad = std::sqrt(rad);
    const float r2a = 1.0f / (2.f * a);
    t_in = std::min(t_in, approx + (-b - srad) * r2a);
    t_out = std::max(t_out, approx + (-b + srad) * r2a);
}
static inline void line_cylinder(F3 org, F3 dir, F3 A0, F3 B0, float r, float &t_in, float &t_out) {
    const F3 center = 0.5f * (A0 + B0);
    const float approx = dot(center - org, dir);
    const F3 close = org + approx * dir;
    const F3 A = A0 - close, B = B0 - close;
    const F3 AB = B - A;
    const F3 AOxAB = cross(AB, A);
    const F3 VxAB = cross(dir, AB);
    const float ab2 = dot(AB, AB);
    const float a = dot(VxAB, VxAB);
    if (a == 0.f) return;
    const float b = 2.f * dot(VxAB, AOxAB);
    const float c = dot(AOxAB, AOxAB) - ((r * r) * ab2);
    const float rad = b * b - 4.f * a * c;
    if (rad < 0.f) return;
    const float srad = std::sqrt(rad);
    const float dVAB = dot(dir, AB);
    if (dVAB == 0.f) return;
    const float rVAB = 1.0f / dVAB;
    const float tA = dot(AB, A) * rVAB, tB = dot(AB, B) * rVAB;
    const float r2a = 1.0f / (2.f * a);
    const float c_in = approx + std::max((-b - srad) * r2a, std::min(tA, tB));
    const float c_out = approx + std::min((-b + srad) * r2a, std::max(tA, tB));
    if (c_in < c_out) {
        t_in = c_in;
        t_out = c_out;
    }
}
static inline bool line_test(F3 org, F3 dir, F3 A, F3 B, float r, float t0, float tfar, float &t) {
    float t_in = INFINITY, t_out = -INFINITY;
    line_cylinder(org, dir, A, B, r, t_in, t_out);
    line_sphere(org, dir, A, r, t_in, t_out);
    line_sphere(org, dir, B, r, t_in, t_out);
    if (!(t_in < t_out)) return false;
    if (t_in > t0 && t_in < tfar) { t = t_in; return true; }
    if (t_out > t0 && t_out < tfar) { t = t_out; return true; }
    return false;
}

static bool geo_closest(const Geo &g, F3 org, F3 dir, float t0, float tfar, GeoHit &h, bool any_hit = false) {
    if (g.nodes.empty()) return false;
    F3 inv = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    h.t = tfar;
    h.prim = INT64_MAX;
    bool found = false;
    int32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Geo::Node &nd = g.nodes[stack[--sp]];
        // slab test against [t0, h.t]
        float tx0 = (nd.lo[0] - org.x) * inv.x, tx1 = (nd.hi[0] - org.x) * inv.x;
        float ty0 = (nd.lo[1] - org.y) * inv.y, ty1 = (nd.hi[1] - org.y) * inv.y;
        float tz0 = (nd.lo[2] - org.z) * inv.z, tz1 = (nd.hi[2] - org.z) * inv.z;
        float tn = std::max(std::max(std::min(tx0, tx1), std::min(ty0, ty1)), std::max(std::min(tz0, tz1), t0));
        float tf = std::min(std::min(std::max(tx0, tx1), std::max(ty0, ty1)), std::min(std::max(tz0, tz1), h.t));
        if (tn > tf * 1.0000002f + 1e-30f) continue;
        if (nd.left < 0) {
            for (int32_t i = nd.first; i < nd.first + nd.count; i++) {
                int64_t p = g.order[i];
                float t, u = 0, v = 0;
                bool hit;
                if (p < g.n_tri) {
                    hit = tri_test(org, dir, g.tv0[p], g.tv1[p], g.tv2[p], t, u, v) && t > t0 && t < tfar;
                } else if (p >= g.n_tri + g.n_sph) {
                    int64_t s = p - g.n_tri - g.n_sph;
                    hit = line_test(org, dir, g.la[s], g.lb[s], g.lr[s], t0, tfar, t);
                } else {
                    int64_t s = p - g.n_tri;
                    float eps = 0;
                    for (auto &ss : g.ssets)
                        if (s >= ss.base - g.n_tri) eps = ss.eps;
                    hit = sph_test(org, dir, g.scen[s], g.srad[s], eps, t0, tfar, t);
                }
                if (hit && (t < h.t || (t == h.t && p < h.prim))) {
                    h.t = t; h.prim = p; h.u = u; h.v = v;
                    found = true;
                    if (any_hit) return true;
                }
            }
        } else {
            if (sp + 2 > 128) { fprintf(stderr, "oracle: bvh stack overflow\n"); abort(); }
            stack[sp++] = nd.right;
            stack[sp++] = nd.left;
        }
    }
    return found;
}

// --------------------------------------------------------------- scene
struct Scene {
    gxy_scene_desc desc;
    std::vector<gxy_volume_vis> vols_desc;
    std::vector<gxy_triangles_vis> tris_desc;
    std::vector<gxy_particles_vis> parts_desc;
    std::vector<gxy_pathlines_vis> lines_desc;
    std::vector<float> extents;    // partition document, 6 per brick
    std::vector<Vol> vols;
    Geo geo;
    Box gbox;
    std::vector<Box> lbox;
    std::vector<int> neighbors;  // 6 per partition
    int np = 1;
    bool integrate = false;
    float step = -1, epsilon = 0;  // march step and epsilon (TraceRays.ispc:342-361)
};

// Volume::partition (Volume.cpp:133-172) on the first volume's grid, or a
// uniform split of the geometry box; neighbours as Volume.cpp:371-376.
static void setup_partitions(Scene &s) {
    const gxy_scene_desc &d = s.desc;
    if (d.n_partition_extents > 0) {
        // Geometry::get_partitioning (Geometry.cpp:279-350)
        const int n = d.n_partition_extents;
        const float *E = s.extents.data();
        s.np = n;
        s.lbox.resize(n);
        s.neighbors.assign(6 * n, -1);
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
        s.gbox.lo = mk(g[0], g[2], g[4]);
        s.gbox.hi = mk(g[1], g[3], g[5]);
        for (int p = 0; p < n; p++) {
            const float *l = E + 6 * p;
            s.lbox[p].lo = mk(l[0], l[2], l[4]);
            s.lbox[p].hi = mk(l[1], l[3], l[5]);
            int *nb = &s.neighbors[6 * p];
            for (int i = 0; i < n; i++) {
                const float *e = E + 6 * i;
#define LAST(a) (e[2 * (a) + 1] == l[2 * (a)])
#define NEXT(a) (e[2 * (a)] == l[2 * (a) + 1])
#define EQ(a) (e[2 * (a)] == l[2 * (a)])
                if (LAST(0) && EQ(1) && EQ(2)) nb[0] = i;
                if (NEXT(0) && EQ(1) && EQ(2)) nb[1] = i;
                if (EQ(0) && LAST(1) && EQ(2)) nb[2] = i;
                if (EQ(0) && NEXT(1) && EQ(2)) nb[3] = i;
                if (EQ(0) && EQ(1) && LAST(2)) nb[4] = i;
                if (EQ(0) && EQ(1) && NEXT(2)) nb[5] = i;
#undef LAST
#undef NEXT
#undef EQ
            }
        }
        return;
    }
    int PX = std::max(1, d.partitions[0]), PY = std::max(1, d.partitions[1]), PZ = std::max(1, d.partitions[2]);
    s.np = PX * PY * PZ;
    s.lbox.resize(s.np);
    s.neighbors.resize(6 * s.np);
    if (d.n_volumes > 0) {
        const gxy_volume_vis &v = d.volumes[0];
        int ni = v.counts[0] - 2, nj = v.counts[1] - 2, nk = v.counts[2] - 2;
        int di = ni / PX, dj = nj / PY, dk = nk / PZ;
        // global box: origin + delta, counts - 2 (Volume.cpp:379-381; Box::set Box.cpp:68-80)
        s.gbox.lo = mk(v.origin[0] + v.deltas[0], v.origin[1] + v.deltas[1], v.origin[2] + v.deltas[2]);
        s.gbox.hi = mk(s.gbox.lo.x + (ni - 1) * v.deltas[0], s.gbox.lo.y + (nj - 1) * v.deltas[1],
                       s.gbox.lo.z + (nk - 1) * v.deltas[2]);
        for (int k = 0; k < PZ; k++)
            for (int j = 0; j < PY; j++)
                for (int i = 0; i < PX; i++) {
                    int p = i + j * PX + k * PX * PY;
                    int offx = 1 + i * di, offy = 1 + j * dj, offz = 1 + k * dk;
                    int cx = 1 + ((i == PX - 1) ? ni - offx : di);
                    int cy = 1 + ((j == PY - 1) ? nj - offy : dj);
                    int cz = 1 + ((k == PZ - 1) ? nk - offz : dk);
                    Box b;
                    b.lo = mk(v.origin[0] + (offx * v.deltas[0]), v.origin[1] + (offy * v.deltas[1]),
                              v.origin[2] + (offz * v.deltas[2]));
                    b.hi = mk(b.lo.x + (cx - 1) * v.deltas[0], b.lo.y + (cy - 1) * v.deltas[1],
                              b.lo.z + (cz - 1) * v.deltas[2]);
                    s.lbox[p] = b;
                }
    } else {
        Box g;
        if (d.has_box) {
            g.lo = mk(d.box[0], d.box[1], d.box[2]);
            g.hi = mk(d.box[3], d.box[4], d.box[5]);
        } else {
            float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            int64_t n = s.geo.n_tri + s.geo.n_sph;
            for (int64_t p = 0; p < n; p++) {
                float a[3], b[3];
                prim_bounds(s.geo, p, a, b);
                for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], a[k]); hi[k] = std::max(hi[k], b[k]); }
            }
            // path lines: vertices grown by their radius (DataDrivenPathLines.cpp:79-86)
            for (auto &ls : s.geo.lsets) {
                const gxy_pathlines_vis &q = *ls.v;
                for (int64_t i = 0; i < q.n_vertices; i++)
                    for (int k = 0; k < 3; k++) {
                        lo[k] = std::min(lo[k], q.vertices[3 * i + k] - ls.rad[i]);
                        hi[k] = std::max(hi[k], q.vertices[3 * i + k] + ls.rad[i]);
                    }
                n += q.n_vertices;
            }
            if (n == 0) { for (int k = 0; k < 3; k++) { lo[k] = -1; hi[k] = 1; } }
            g.lo = mk(lo[0], lo[1], lo[2]);
            g.hi = mk(hi[0], hi[1], hi[2]);
        }
        s.gbox = g;
        float ex = (g.hi.x - g.lo.x) / PX, ey = (g.hi.y - g.lo.y) / PY, ez = (g.hi.z - g.lo.z) / PZ;
        for (int k = 0; k < PZ; k++)
            for (int j = 0; j < PY; j++)
                for (int i = 0; i < PX; i++) {
                    int p = i + j * PX + k * PX * PY;
                    Box b;
                    b.lo = mk(g.lo.x + i * ex, g.lo.y + j * ey, g.lo.z + k * ez);
                    b.hi = mk(i == PX - 1 ? g.hi.x : g.lo.x + (i + 1) * ex, j == PY - 1 ? g.hi.y : g.lo.y + (j + 1) * ey,
                              k == PZ - 1 ? g.hi.z : g.lo.z + (k + 1) * ez);
                    s.lbox[p] = b;
                }
    }
    for (int k = 0; k < PZ; k++)
        for (int j = 0; j < PY; j++)
            for (int i = 0; i < PX; i++) {
                int p = i + j * PX + k * PX * PY;
                int *nb = &s.neighbors[6 * p];
                nb[0] = (i > 0) ? p - 1 : -1;
                nb[1] = (i < PX - 1) ? p + 1 : -1;
                nb[2] = (j > 0) ? p - PX : -1;
                nb[3] = (j < PY - 1) ? p + PX : -1;
                nb[4] = (k > 0) ? p - PX * PY : -1;
                nb[5] = (k < PZ - 1) ? p + PX * PY : -1;
            }
}

static Scene *scene_create(const gxy_scene_desc *d) {
    Scene *s = new Scene();
    s->desc = *d;
    s->vols_desc.assign(d->volumes, d->volumes + d->n_volumes);
    s->tris_desc.assign(d->triangles, d->triangles + d->n_triangle_sets);
    s->parts_desc.assign(d->particles, d->particles + d->n_particle_sets);
    if (d->n_pathline_sets > 0) s->lines_desc.assign(d->pathlines, d->pathlines + d->n_pathline_sets);
    if (d->n_partition_extents > 0)
        s->extents.assign(d->partition_extents, d->partition_extents + 6 * d->n_partition_extents);
    s->desc.partition_extents = s->extents.data();
    s->desc.volumes = s->vols_desc.data();
    s->desc.triangles = s->tris_desc.data();
    s->desc.particles = s->parts_desc.data();
    s->desc.pathlines = s->lines_desc.data();
    if (!(s->desc.sampling_rate > 0)) s->desc.sampling_rate = 1.0f;
    if (!(s->desc.opaque_alpha > 0)) s->desc.opaque_alpha = 0.999f;
    for (auto &v : s->vols_desc) {
        Vol vol;
        vol.vis = &v;
        vol.data = v.samples;
        vol.nx = v.counts[0]; vol.ny = v.counts[1]; vol.nz = v.counts[2];
        vol.ox = v.origin[0]; vol.oy = v.origin[1]; vol.oz = v.origin[2];
        vol.dx = v.deltas[0]; vol.dy = v.deltas[1]; vol.dz = v.deltas[2];
        vol.ux = nextafterf((float)(vol.nx - 1), 0.0f);
        vol.uy = nextafterf((float)(vol.ny - 1), 0.0f);
        vol.uz = nextafterf((float)(vol.nz - 1), 0.0f);
        vol.ix = 1.0f / vol.dx;
        vol.iy = 1.0f / vol.dy;
        vol.iz = 1.0f / vol.dz;
        s->vols.push_back(vol);
        if (v.volume_render || v.n_isovalues > 0) s->integrate = true;
        // samplingStep = smallest spacing; step = samplingStep / samplingRate
        float sstep = std::min(v.deltas[0], std::min(v.deltas[1], v.deltas[2]));
        float st = sstep / s->desc.sampling_rate;
        if (s->step < 0 || s->step > st) {
            s->step = st;
            s->epsilon = s->desc.epsilon * st;
        }
    }
    Geo &g = s->geo;
    for (auto &t : s->tris_desc) {
        g.tsets.push_back({&t, g.n_tri});
        for (int64_t i = 0; i < t.n_triangles; i++) {
            const int32_t *ix = t.indices + 3 * i;
            g.tv0.push_back(mk(t.vertices[3 * ix[0]], t.vertices[3 * ix[0] + 1], t.vertices[3 * ix[0] + 2]));
            g.tv1.push_back(mk(t.vertices[3 * ix[1]], t.vertices[3 * ix[1] + 1], t.vertices[3 * ix[1] + 2]));
            g.tv2.push_back(mk(t.vertices[3 * ix[2]], t.vertices[3 * ix[2] + 1], t.vertices[3 * ix[2] + 2]));
        }
        g.n_tri += t.n_triangles;
    }
    for (auto &p : s->parts_desc) {
        g.ssets.push_back({&p, g.n_tri + g.n_sph, sphere_epsilon(p.radius0)});
        for (int64_t i = 0; i < p.n; i++) {
            g.scen.push_back(mk(p.centers[3 * i], p.centers[3 * i + 1], p.centers[3 * i + 2]));
            g.srad.push_back(sphere_radius(p, i));
        }
        g.n_sph += p.n;
    }
    for (auto &q : s->lines_desc) {
        Geo::LineSet ls{&q, g.n_tri + g.n_sph + g.n_seg, {}};
        for (int64_t i = 0; i < q.n_vertices; i++) ls.rad.push_back(pathline_radius(q, i));
        for (int64_t i = 0; i < q.n_segments; i++) {
            const float *a = q.vertices + 3 * (int64_t)q.indices[i], *b = a + 3;
            g.la.push_back(mk(a[0], a[1], a[2]));
            g.lb.push_back(mk(b[0], b[1], b[2]));
            g.lr.push_back(q.radius0);
        }
        g.n_seg += q.n_segments;
        g.lsets.push_back(std::move(ls));
    }
    build_bvh(g);
    setup_partitions(*s);
    return s;
}

// ------------------------------------------------------------- ray list
struct Rays {
    std::vector<float> ox, oy, oz, dx, dy, dz, nx, ny, nz, sample, r, g, b, o, sr, sg, sb, so, t, tMax;
    std::vector<int32_t> x, y, type, term, cls;
    int n = 0;
    void resize(int m) {
        n = m;
        for (auto *v : {&ox, &oy, &oz, &dx, &dy, &dz, &nx, &ny, &nz, &sample, &r, &g, &b, &o, &sr, &sg, &sb, &so, &t, &tMax})
            v->assign(m, 0.0f);
        for (auto *v : {&x, &y, &type, &term, &cls}) v->assign(m, 0);
    }
    void copy_from(const Rays &s, int i, int j) {
        ox[j] = s.ox[i]; oy[j] = s.oy[i]; oz[j] = s.oz[i]; dx[j] = s.dx[i]; dy[j] = s.dy[i]; dz[j] = s.dz[i];
        nx[j] = s.nx[i]; ny[j] = s.ny[i]; nz[j] = s.nz[i]; sample[j] = s.sample[i];
        r[j] = s.r[i]; g[j] = s.g[i]; b[j] = s.b[i]; o[j] = s.o[i];
        sr[j] = s.sr[i]; sg[j] = s.sg[i]; sb[j] = s.sb[i]; so[j] = s.so[i]; t[j] = s.t[i]; tMax[j] = s.tMax[i];
        x[j] = s.x[i]; y[j] = s.y[i]; type[j] = s.type[i]; term[j] = s.term[i]; cls[j] = s.cls[i];
    }
};

static void rays_from_c(const gxy_raylist &c, Rays &r) {
    r.resize(c.n);
    size_t fb = sizeof(float) * c.n, ib = sizeof(int32_t) * c.n;
#define CPF(F) if (c.F) memcpy(r.F.data(), c.F, fb);
#define CPI(F) if (c.F) memcpy(r.F.data(), c.F, ib);
    CPF(ox) CPF(oy) CPF(oz) CPF(dx) CPF(dy) CPF(dz) CPF(nx) CPF(ny) CPF(nz) CPF(sample)
    CPF(r) CPF(g) CPF(b) CPF(o) CPF(sr) CPF(sg) CPF(sb) CPF(so) CPF(t) CPF(tMax)
    CPI(x) CPI(y) CPI(type) CPI(term)
    if (c.classification) memcpy(r.cls.data(), c.classification, ib);
#undef CPF
#undef CPI
}
static void rays_to_c(const Rays &r, gxy_raylist &c, int n) {
    size_t fb = sizeof(float) * n, ib = sizeof(int32_t) * n;
#define CPF(F) if (c.F) memcpy(c.F, r.F.data(), fb);
#define CPI(F) if (c.F) memcpy(c.F, r.F.data(), ib);
    CPF(ox) CPF(oy) CPF(oz) CPF(dx) CPF(dy) CPF(dz) CPF(nx) CPF(ny) CPF(nz) CPF(sample)
    CPF(r) CPF(g) CPF(b) CPF(o) CPF(sr) CPF(sg) CPF(sb) CPF(so) CPF(t) CPF(tMax)
    CPI(x) CPI(y) CPI(type) CPI(term)
    if (c.classification) memcpy(c.classification, r.cls.data(), ib);
#undef CPF
#undef CPI
}

// --------------------------------------------------------------- tracing
struct Hit {
    float t = 0;
    F3 normal{0, 0, 0};
    F3 color{0, 0, 0};
    float opacity = 0;
    float sample = 0;
};

struct Stats {
    int64_t samples = 0, prim = 0, shadow = 0, ao = 0, segments = 0, terminated = 0, handoffs = 0;
};

// Per-ray body of TraceRays_TraceRays (TraceRays.ispc:366-620).  VT is the
// value type of volume sampling and compositing: float for the reference
// arithmetic, double for the FP64 re-evaluation (sample positions and loop
// control stay float, so both runs visit the same t sequence).
template <class VT>
static void trace_one(const Scene &S, int part, Rays &R, int i, Stats *st, double *out64 = nullptr) {
    const Box &box = S.lbox[part];
    bool shade = R.type[i] == GXY_RAY_PRIMARY;
    F3 org = mk(R.ox[i], R.oy[i], R.oz[i]);
    F3 dir = mk(R.dx[i], R.dy[i], R.dz[i]);
    if (dir.x == 0.f) dir.x = 1e-6f;
    if (dir.y == 0.f) dir.y = 1e-6f;
    if (dir.z == 0.f) dir.z = 1e-6f;
    float ray_t0 = R.t[i];
    float ray_t = R.tMax[i];
    float tTimeout = ray_t;
    V3<VT> col = mk<VT>(R.r[i], R.g[i], R.b[i]);
    VT cola = R.o[i];
    float tEntry, tExitVolume;
    my_intersect_box(org, dir, box, tEntry, tExitVolume);
    if (tEntry < ray_t0) tEntry = ray_t0;
    else if (tEntry > ray_t0) ray_t0 = tEntry;
    ray_t = std::min(ray_t, tExitVolume);
    Hit hit;
    bool surface_hit = false;
    // LookForSliceHit (TraceRays.ispc:143-250)
    {
        int vid = -1;
        for (int m = 0; m < (int)S.vols.size(); m++) {
            const gxy_volume_vis &vv = *S.vols[m].vis;
            for (int k = 0; k < vv.n_slices; k++) {
                F3 pn = mk(vv.slices[k][0], vv.slices[k][1], vv.slices[k][2]);
                float dd = vv.slices[k][3];
                float denom = dot(dir, pn);
                if (std::fabs(denom) > 0.0001f) {
                    float t = (dd - dot(org, pn)) / denom;
                    if (t >= ray_t0 && t <= ray_t) {
                        hit.normal = denom > 0 ? neg(pn) : pn;
                        hit.opacity = 1.0f;
                        hit.t = t;
                        vid = m;
                        ray_t = t;
                        surface_hit = true;
                    }
                }
            }
        }
        if (surface_hit && shade) {
            F3 p = org + hit.t * dir;
            hit.sample = vol_sample<float>(S.vols[vid], p);
            hit.color = tf_color<float>(S.vols[vid].vis->tf, hit.sample);
            hit.opacity = 1.0f;
        }
    }
    // LookForGeometryHit (TraceRays.ispc:108-141)
    {
        GeoHit gh;
        if (geo_closest(S.geo, org, dir, ray_t0, ray_t, gh)) {
            ray_t = gh.t;
            surface_hit = true;
            if (shade) {
                const Geo &g = S.geo;
                F3 Ng, Ns;
                F3 colr = mk(1.f, 1.f, 1.f);
                int64_t p = gh.prim;
                if (p < g.n_tri) {
                    const Geo::TriSet *ts = &g.tsets[0];
                    for (auto &q : g.tsets)
                        if (p >= q.base) ts = &q;
                    int64_t lp = p - ts->base;
                    const gxy_triangles_vis &tv = *ts->v;
                    F3 e1 = g.tv1[p] - g.tv0[p], e2 = g.tv2[p] - g.tv0[p];
                    Ng = cross(e1, e2);
                    Ns = Ng;
                    const int32_t *ix = tv.indices + 3 * lp;
                    float bx = 1.0f - gh.u - gh.v, by = gh.u, bz = gh.v;
                    if (tv.normals) {
                        F3 na = mk(tv.normals[3 * ix[0]], tv.normals[3 * ix[0] + 1], tv.normals[3 * ix[0] + 2]);
                        F3 nb = mk(tv.normals[3 * ix[1]], tv.normals[3 * ix[1] + 1], tv.normals[3 * ix[1] + 2]);
                        F3 nc = mk(tv.normals[3 * ix[2]], tv.normals[3 * ix[2] + 1], tv.normals[3 * ix[2] + 2]);
                        Ns = (bx * na + by * nb) + bz * nc;  // DataDrivenTriangleMesh.ispc:46-53
                    }
                    if (tv.data) {  // DataDrivenTriangleMesh.ispc:106-117
                        float dv = bx * tv.data[ix[0]] + by * tv.data[ix[1]] + bz * tv.data[ix[2]];
                        colr = tf_color<float>(tv.tf, dv);
                    }
                } else if (p >= g.n_tri + g.n_sph) {
                    // DataDrivenPathLines.ispc:186-196 (u, Ng) and 213-268 (colour)
                    const Geo::LineSet *ls = &g.lsets[0];
                    for (auto &q : g.lsets)
                        if (p >= q.base) ls = &q;
                    const gxy_pathlines_vis &lv = *ls->v;
                    const int32_t idx = lv.indices[p - ls->base];
                    const float *va = lv.vertices + 3 * (int64_t)idx;
                    F3 A = mk(va[0], va[1], va[2]), B = mk(va[3], va[4], va[5]);
                    F3 P = org + gh.t * dir;
                    const float ab2 = dot(B - A, B - A);
                    float u = ab2 == 0.f ? 0.f : dot(P - A, B - A) * (1.0f / ab2);  // zero length: end sphere
                    u = std::min(std::max(u, 0.f), 1.f);
                    F3 PonAxis = A + u * (B - A);
                    Ng = normalize(P - PonAxis);
                    Ns = Ng;
                    float radius = ((1.f - u) * ls->rad[idx]) + (u * ls->rad[idx + 1]);
                    const float r0 = lv.radius0, r1 = lv.radius1, v0 = lv.value0, v1 = lv.value1;
                    float dataval;
                    if (r0 == r1) dataval = v0;
                    else if (r0 < r1 && radius < r0) dataval = v0;
                    else if (r0 < r1 && radius > r1) dataval = v1;
                    else if (r0 > r1 && radius < r1) dataval = v1;
                    else if (r0 > r1 && radius > r0) dataval = v0;
                    else dataval = v0 + ((radius - r0) / (r1 - r0)) * (v1 - v0);
                    colr = tf_color<float>(lv.tf, dataval);
                } else {
                    int64_t s = p - g.n_tri;
                    const Geo::SphSet *ss = &g.ssets[0];
                    for (auto &q : g.ssets)
                        if (p >= q.base) ss = &q;
                    int64_t lp = p - ss->base;
                    Ng = (org + gh.t * dir) - g.scen[s];  // DataDrivenSpheres.ispc:152
                    Ns = Ng;
                    if (ss->v->data) colr = tf_color<float>(ss->v->tf, ss->v->data[lp]);  // :56-62
                }
                // postIntersect DG_NORMALIZE | DG_FACEFORWARD (OSPRay; definition)
                Ng = normalize(Ng);
                Ns = normalize(Ns);
                if (dot(dir, Ng) >= 0.f) Ng = neg(Ng);
                if (dot(Ng, Ns) < 0.f) Ns = neg(Ns);
                hit.color = colr;
                hit.opacity = 1.0f;
                hit.normal = Ns;
                hit.t = gh.t;
            }
        }
    }
    float tTermination = ray_t;
    if (S.integrate) {
        // march (TraceRays.ispc:446-570)
        const float step = S.step, epsilon = S.epsilon;
        const float oa = S.desc.opaque_alpha;
        const VT rate = (VT)S.desc.sampling_rate;
        float tLast, tThis;
        VT sLast[GXY_MAX_VOLUMES], sThis[GXY_MAX_VOLUMES];
        int nv = (int)S.vols.size();
        bool hit_iso = false;
        tLast = tEntry + epsilon;
        bool opaque = (std::min(std::min(col.x, col.y), col.z) >= VT(1) || cola > VT(oa));
        for (tThis = tEntry; tThis <= tTermination && !opaque && !hit_iso;
             tThis = (tThis == tEntry) ? (tEntry + epsilon)
                     : (((tThis + step) > tTermination) && (tThis < tTermination)) ? tTermination
                                                                                   : tThis + step) {
            V3<VT> coord = tov<VT>(org) + VT(tThis) * tov<VT>(dir);
            V3<VT> cf = coord;
            for (int m = 0; m < nv; m++) sThis[m] = vol_sample<VT>(S.vols[m], cf);
            if (st) st->samples++;
            if (tThis > tEntry && tLast >= epsilon) {
                // LookForIsoHit (TraceRays.ispc:252-310)
                bool h = false;
                int vid = -1;
                for (int m = 0; m < nv; m++) {
                    const gxy_volume_vis &vv = *S.vols[m].vis;
                    VT sl = sLast[m], sti = sThis[m];
                    for (int k = 0; k < vv.n_isovalues; k++) {
                        VT iso = vv.isovalues[k];
                        if (((iso >= sl) && (iso < sti)) || ((iso <= sl) && (iso > sti))) {
                            h = true;
                            vid = m;
                            hit.t = (float)(VT(tLast) + ((iso - sl) / (sti - sl)) * (VT(tThis) - VT(tLast)));
                            hit.sample = (float)iso;
                        }
                    }
                }
                if (h) {
                    F3 hp = org + hit.t * dir;
                    if (shade) {
                        F3 n = normalize(vol_gradient(S.vols[vid], hp));
                        if (dot(dir, n) > 0) n = neg(n);
                        hit.normal = n;
                        hit.color = tf_color<float>(S.vols[vid].vis->tf, hit.sample);
                        hit.opacity = 1.0f;
                    }
                    tTermination = hit.t;
                    tThis = hit.t;
                    surface_hit = true;
                    hit_iso = true;
                    V3<VT> c2 = tov<VT>(org) + VT(tThis) * tov<VT>(dir);
                    for (int m = 0; m < nv; m++) sThis[m] = vol_sample<VT>(S.vols[m], c2);
                }
                for (int m = 0; m < nv; m++) {
                    const gxy_volume_vis &vv = *S.vols[m].vis;
                    if (vv.volume_render) {
                        VT sv = (sLast[m] + sThis[m]) / VT(2);
                        VT so = tf_opacity<VT>(vv.tf, sv);
                        if (so > VT(0)) {
                            VT wo = so / rate;
                            if (wo > VT(1)) wo = VT(1);
                            if (wo < VT(0)) wo = VT(0);
                            if (shade) {
                                V3<VT> sc = tf_color<VT>(vv.tf, sv);
                                VT f = VT(1) - cola;
                                col.x = col.x + f * (wo * sc.x);
                                col.y = col.y + f * (wo * sc.y);
                                col.z = col.z + f * (wo * sc.z);
                                cola = cola + f * wo;
                            } else {
                                VT w = ((VT(tThis) - VT(tLast)) / VT(step)) * wo;
                                VT f = VT(1) - w;
                                col.x = col.x * f;
                                col.y = col.y * f;
                                col.z = col.z * f;
                                cola = cola * f;
                            }
                        }
                    }
                    sLast[m] = sThis[m];
                }
            }
            for (int m = 0; m < nv; m++) sLast[m] = sThis[m];
            opaque = (std::min(std::min(col.x, col.y), col.z) >= VT(1) || cola > VT(oa));
            if (opaque) tTermination = tThis;
            tLast = tThis;
        }
        ray_t = tTermination;
    }
    if (out64) {
        out64[0] = (double)col.x; out64[1] = (double)col.y; out64[2] = (double)col.z; out64[3] = (double)cola;
    }
    R.r[i] = (float)col.x;
    R.g[i] = (float)col.y;
    R.b[i] = (float)col.z;
    R.o[i] = (float)cola;
    float oa = S.desc.opaque_alpha;
    bool op = std::min(std::min(R.r[i], R.g[i]), R.b[i]) >= 1.0f || R.o[i] > oa;
    R.term[i] = op ? GXY_RAY_OPAQUE : 0;
    R.t[i] = ray_t;
    if (surface_hit) {
        R.term[i] |= GXY_RAY_SURFACE;
        if (hit.opacity > 0.999f) R.term[i] |= GXY_RAY_OPAQUE;
        R.sr[i] = hit.color.x;
        R.sg[i] = hit.color.y;
        R.sb[i] = hit.color.z;
        R.so[i] = 1.0f;
        R.nx[i] = hit.normal.x;
        R.ny[i] = hit.normal.y;
        R.nz[i] = hit.normal.z;
    } else if (tTermination == tExitVolume) {
        R.term[i] |= GXY_RAY_BOUNDARY;
    } else if (tTermination == tTimeout) {
        R.term[i] |= GXY_RAY_TIMEOUT;
    }
}

// TraceRays::Trace (TraceRays.cpp:68-146) with GXY_REVERSE_LIGHTING.
// Worker threads of the RayList entry points (oracle_set_threads); the
// per-ray trace has no shared state, so rays are split into chunks.
static int g_threads = 1;
template <class F> static void parallel_rays(int n, F f) {
    const int nt = std::max(1, std::min(g_threads, n / 256 + 1));
    if (nt == 1) {
        for (int i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++)
        th.emplace_back([&]() {
            for (;;) {
                const int a = next.fetch_add(1024);
                if (a >= n) break;
                const int b = std::min(n, a + 1024);
                for (int i = a; i < b; i++) f(i);
            }
        });
    for (auto &t : th) t.join();
}

static void trace_list(const Scene &S, int part, const gxy_lighting &L, Rays &in, Rays &out, Stats *st) {
    if (st) {
        for (int i = 0; i < in.n; i++) trace_one<float>(S, part, in, i, st);
    } else {
        parallel_rays(in.n, [&](int i) { trace_one<float>(S, part, in, i, nullptr); });
    }
    const float eps = S.desc.epsilon;
    int n = in.n;
    std::vector<int> ao_off(n), sh_off(n, -1);
    int nout = 0;
    for (int i = 0; i < n; i++) {
        ao_off[i] = nout;
        if (in.type[i] == GXY_RAY_PRIMARY && (in.term[i] & GXY_RAY_SURFACE)) nout += L.n_ao;
    }
    int ao_knt = nout;
    if (L.shadows) {
        for (int i = 0; i < n; i++) {
            if (in.type[i] == GXY_RAY_PRIMARY && (in.term[i] & GXY_RAY_SURFACE)) {
                sh_off[i] = nout;
                nout += L.n_lights;
            } else sh_off[i] = -1;
        }
    }
    int sh_knt = nout - ao_knt;
    out.resize(nout);
    // TraceRays_ambientLighting (TraceRays.ispc:735-761)
    for (int i = 0; i < n; i++)
        if (in.type[i] == GXY_RAY_PRIMARY && (in.term[i] & GXY_RAY_SURFACE)) {
            float s = L.Ka * (1.0f - in.o[i]);
            in.r[i] += s * in.sr[i];
            in.g[i] += s * in.sg[i];
            in.b[i] += s * in.sb[i];
        }
    // TraceRays_generateAORays (TraceRays.ispc:625-733)
    if (ao_knt) {
        const AOTables &T = ao_tables();
        float Ka = -L.Ka / L.n_ao;
        for (int i = 0; i < n; i++) {
            if (!(in.type[i] == GXY_RAY_PRIMARY && (in.term[i] & GXY_RAY_SURFACE))) continue;
            F3 nrm = mk(in.nx[i], in.ny[i], in.nz[i]);
            float as = Ka * (1.0f - in.o[i]);
            float ar = as * in.sr[i], ag = as * in.sg[i], ab = as * in.sb[i];
            F3 b0 = mk(1.f, 0.f, 0.f);
            if (std::fabs(dot(b0, nrm)) > 0.95f) b0 = mk(0.f, 1.f, 0.f);
            F3 b1 = normalize(cross(b0, nrm));
            b0 = normalize(cross(b1, nrm));
            float ox = in.ox[i] + in.t[i] * in.dx[i];
            float oy = in.oy[i] + in.t[i] * in.dy[i];
            float oz = in.oz[i] + in.t[i] * in.dz[i];
            ox = ox + eps * nrm.x;
            oy = oy + eps * nrm.y;
            oz = oz + eps * nrm.z;
            for (int j = 0; j < L.n_ao; j++) {
                int off = ao_off[i] + j;
                int r = ((in.x[i] * 9949 + in.y[i] * 9613 + j * 9151) >> 8) & 0xff;
                float x = T.cos2pu[r] * T.sq1mv[r];
                float y = T.sin2pu[r] * T.sq1mv[r];
                float z = T.sqv[r] + eps;
                F3 rd = (x * b0 + y * b1) + z * nrm;
                out.ox[off] = ox; out.oy[off] = oy; out.oz[off] = oz;
                out.dx[off] = rd.x; out.dy[off] = rd.y; out.dz[off] = rd.z;
                out.r[off] = ar; out.g[off] = ag; out.b[off] = ab; out.o[off] = 0.0f;
                out.t[off] = 0.0f; out.tMax[off] = L.ao_radius;
                out.x[off] = in.x[i]; out.y[off] = in.y[i];
                out.type[off] = GXY_RAY_AO; out.term[off] = 0;
            }
        }
    }
    // TraceRays_diffuseLighting (TraceRays.ispc:859-923)
    {
        float Kd = L.Kd / L.n_lights;
        for (int i = 0; i < n; i++) {
            if (!(in.type[i] == GXY_RAY_PRIMARY && (in.term[i] & GXY_RAY_SURFACE))) continue;
            F3 nrm = mk(in.nx[i], in.ny[i], in.nz[i]);
            float tr = 0, tg = 0, tb = 0;
            for (int k = 0; k < L.n_lights; k++) {
                F3 lv;
                if (L.types[k]) {
                    float t = in.t[i];
                    F3 sp = mk(in.ox[i] + t * in.dx[i], in.oy[i] + t * in.dy[i], in.oz[i] + t * in.dz[i]);
                    lv = normalize(mk(L.lights[k][0], L.lights[k][1], L.lights[k][2]) - sp);
                } else {
                    lv = neg(mk(L.lights[k][0], L.lights[k][1], L.lights[k][2]));
                }
                float d = dot(nrm, lv);
                if (d > 0) {
                    float dff = (1.0f - in.o[i]) * d;
                    tr += dff * in.sr[i];
                    tg += dff * in.sg[i];
                    tb += dff * in.sb[i];
                }
            }
            float f = Kd * (1 - in.o[i]);
            in.r[i] = in.r[i] + f * tr;
            in.g[i] = in.g[i] + f * tg;
            in.b[i] = in.b[i] + f * tb;
            in.o[i] = in.o[i] + f * in.o[i];
        }
    }
    // TraceRays_generateShadowRays (TraceRays.ispc:763-857)
    if (sh_knt) {
        float Kd = -L.Kd / L.n_lights;
        for (int i = 0; i < n; i++) {
            int off = sh_off[i];
            if (off == -1) continue;
            F3 nrm = mk(in.nx[i], in.ny[i], in.nz[i]);
            for (int k = 0; k < L.n_lights; k++) {
                F3 sp = mk(in.ox[i] + in.t[i] * in.dx[i] + eps * in.nx[i],
                           in.oy[i] + in.t[i] * in.dy[i] + eps * in.ny[i],
                           in.oz[i] + in.t[i] * in.dz[i] + eps * in.nz[i]);
                F3 lv;
                if (L.types[k]) lv = normalize(mk(L.lights[k][0], L.lights[k][1], L.lights[k][2]) - sp);
                else lv = neg(mk(L.lights[k][0], L.lights[k][1], L.lights[k][2]));
                lv = normalize(lv);
                float d = dot(nrm, lv);
                if (d < 0) d = 0;
                float dff = (1.0f - in.o[i]) * Kd * d;
                out.ox[off] = sp.x; out.oy[off] = sp.y; out.oz[off] = sp.z;
                out.dx[off] = lv.x; out.dy[off] = lv.y; out.dz[off] = lv.z;
                out.r[off] = dff * in.sr[i]; out.g[off] = dff * in.sg[i]; out.b[off] = dff * in.sb[i];
                out.o[off] = 0.0f; out.t[off] = 0.0f; out.tMax[off] = INFINITY;
                out.x[off] = in.x[i]; out.y[off] = in.y[i];
                out.type[off] = GXY_RAY_SHADOW; out.term[off] = 0;
                off++;
            }
        }
    }
    if (st) { st->ao += ao_knt; st->shadow += sh_knt; st->segments += n; }
}

// Renderer::Classify (Renderer.cpp:304-421), reverse lighting.
static void classify(Rays &R) {
    for (int i = 0; i < R.n; i++) {
        int typ = R.type[i], term = R.term[i];
        if (typ == GXY_RAY_PRIMARY) {
            if (term & GXY_RAY_BOUNDARY) R.cls[i] = GXY_RAY_BOUNDARY;
            else if ((term & GXY_RAY_OPAQUE) | (term & GXY_RAY_TIMEOUT)) R.cls[i] = GXY_TERMINATED;
            else R.cls[i] = GXY_KEEP_HERE;
        } else if (typ == GXY_RAY_SHADOW) {
            if ((term & GXY_RAY_OPAQUE) | (term & GXY_RAY_SURFACE)) R.cls[i] = GXY_TERMINATED;
            else if (term & GXY_RAY_BOUNDARY) R.cls[i] = GXY_RAY_BOUNDARY;
            else R.cls[i] = GXY_DROP_ON_FLOOR;
        } else if (typ == GXY_RAY_AO) {
            if ((term & GXY_RAY_OPAQUE) | (term & GXY_RAY_SURFACE)) R.cls[i] = GXY_TERMINATED;
            else if (term & GXY_RAY_BOUNDARY) R.cls[i] = GXY_RAY_BOUNDARY;
            else if (term & GXY_RAY_TIMEOUT) R.cls[i] = GXY_DROP_ON_FLOOR;
            else R.cls[i] = GXY_DROP_ON_FLOOR;
        }
    }
}

// Renderer::AssignDestinations (Renderer.cpp:423-454).  Classification value
// RAY_BOUNDARY (4) marks "to the exit face".
static void assign_destinations(const Scene &S, int part, Rays &R) {
    const Box &b = S.lbox[part];
    for (int i = 0; i < R.n; i++) {
        if (R.cls[i] == GXY_RAY_BOUNDARY) {
            int f = box_exit_face(b, mk(R.ox[i], R.oy[i], R.oz[i]), mk(R.dx[i], R.dy[i], R.dz[i]));
            int nb = S.neighbors[6 * part + f];
            if (nb >= 0) R.cls[i] = nb;
            else {
                int t = R.type[i];
                R.cls[i] = (t == GXY_RAY_SHADOW || t == GXY_RAY_AO) ? GXY_DROP_ON_FLOOR : GXY_TERMINATED;
            }
        }
    }
}

// HandleTerminatedRays + AddLocalPixels (Renderer.cpp:456-502, Rendering.cpp:125-153).
static int64_t accumulate(const Rays &R, float *fb, int w, int h) {
    int64_t k = 0;
    for (int i = 0; i < R.n; i++) {
        if (R.cls[i] != GXY_TERMINATED) continue;
        int x = R.x[i], y = R.y[i];
        if (x < 0 || y < 0 || x >= w || y >= h) continue;
        float *p = fb + 4 * ((size_t)y * w + x);
        p[0] += R.r[i]; p[1] += R.g[i]; p[2] += R.b[i]; p[3] += R.o[i];
        k++;
    }
    return k;
}

// Camera::generate_initial_rays + SpawnRays (Camera.cpp:379-493, 528-829) for
// the pixel rows [y0, y1) and one partition.
static void camera_rays(const Scene &S, int part, const gxy_camera &c, int y0, int y1, Rays &R) {
    int width = c.width, height = c.height;
    F3 veye = mk(c.eye[0], c.eye[1], c.eye[2]);
    F3 vu = mk(c.up[0], c.up[1], c.up[2]);
    F3 vdir = mk(c.dir[0], c.dir[1], c.dir[2]);
    F3 center;
    bool ortho = c.aov == 0.0f;
    if (ortho) {
        center = veye + vdir;
        vdir = gxy_normalize(vdir);
    } else {
        float d = (float)(1.0 / tan(2 * 3.1415926 * (c.aov / 2.0) / 360.0));
        vdir = gxy_normalize(vdir);
        center = veye + d * vdir;
    }
    F3 vr = gxy_normalize(cross(vdir, vu));
    vu = gxy_normalize(cross(vr, vdir));
    float pixel_scaling = (float)((((width < height) ? width : height) - 1.0) / 2.0);
    float off_x = (float)((width - 1) / 2.0);
    float off_y = (float)((height - 1) / 2.0);
    float scaling = (float)(1.0 / pixel_scaling);
    const Box &gb = S.gbox;
    const Box &lb = S.lbox[part];
    std::vector<int> xs, ys;
    std::vector<F3> os, ds;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < width; x++) {
            float fx = ((float)x - off_x) * scaling;
            float fy = ((float)y - off_y) * scaling;
            F3 xy = mk(center.x + fx * vr.x + fy * vu.x, center.y + fx * vr.y + fy * vu.y,
                       center.z + fx * vr.z + fy * vu.z);
            F3 vorg, vray;
            if (ortho) { vorg = xy - vdir; vray = vdir; }
            else { vorg = veye; vray = gxy_normalize(xy - veye); }
            float gmin = 0, gmax = 0, lmin = 0, lmax = 0;
            bool hit = box_intersect(gb, vorg, vray, gmin, gmax);
            if (hit) hit = box_intersect(lb, vorg, vray, lmin, lmax);
            float d = std::fabs(lmin) - std::fabs(gmin);
            if (hit && (lmax >= 0) && (d < 0.000001f) && (d > -0.000001f)) {
                xs.push_back(x); ys.push_back(y); os.push_back(vorg); ds.push_back(vray);
            }
        }
    int cnt = (int)xs.size();
    R.resize(cnt);
    for (int k = 0; k < cnt; k++) {
        R.x[k] = xs[k]; R.y[k] = ys[k];
        R.ox[k] = os[k].x; R.oy[k] = os[k].y; R.oz[k] = os[k].z;
        R.dx[k] = ds[k].x; R.dy[k] = ds[k].y; R.dz[k] = ds[k].z;
        R.t[k] = 0; R.tMax[k] = FLT_MAX;
        R.type[k] = GXY_RAY_PRIMARY;
    }
}

// One frame over pixel rows [y0, y1): the ray-list loop of
// processRays_task::work (Renderer.cpp:511-651) with local enqueue of
// secondaries (Renderer.cpp:674-690) and neighbour hand-off.
static void render_rows(const Scene &S, const gxy_camera &cam, const gxy_lighting &L, float *fb, int y0, int y1,
                        Stats *st, int64_t *n_primary) {
    std::deque<std::pair<int, Rays>> q;
    for (int p = 0; p < S.np; p++) {
        Rays R;
        camera_rays(S, p, cam, y0, y1, R);
        if (n_primary) *n_primary += R.n;
        if (R.n) q.emplace_back(p, std::move(R));
    }
    while (!q.empty()) {
        int part = q.front().first;
        Rays R = std::move(q.front().second);
        q.pop_front();
        while (R.n) {
            Rays out;
            trace_list(S, part, L, R, out, st);
            if (out.n) q.emplace_back(part, std::move(out));
            classify(R);
            assign_destinations(S, part, R);
            int64_t k = accumulate(R, fb, cam.width, cam.height);
            if (st) st->terminated += k;
            std::vector<int> cnt(S.np, 0);
            int keep = 0;
            for (int i = 0; i < R.n; i++) {
                if (R.cls[i] >= 0) cnt[R.cls[i]]++;
                else if (R.cls[i] == GXY_KEEP_HERE) keep++;
            }
            for (int p = 0; p < S.np; p++) {
                if (!cnt[p]) continue;
                Rays to;
                to.resize(cnt[p]);
                int j = 0;
                for (int i = 0; i < R.n; i++)
                    if (R.cls[i] == p) to.copy_from(R, i, j++);
                if (st) st->handoffs += cnt[p];
                q.emplace_back(p, std::move(to));
            }
            Rays kept;
            kept.resize(keep);
            int j = 0;
            for (int i = 0; i < R.n; i++)
                if (R.cls[i] == GXY_KEEP_HERE) kept.copy_from(R, i, j++);
            R = std::move(kept);
        }
    }
}

}  // namespace gxo

using namespace gxo;

// ================================================================ C API
extern "C" {

void *oracle_scene_create(const gxy_scene_desc *d) { return d ? (void *)scene_create(d) : nullptr; }
void oracle_scene_destroy(void *s) { delete (Scene *)s; }

int oracle_partition_info(void *sp, int part, gxy_partition_info *out) {
    Scene *s = (Scene *)sp;
    if (!s || !out || part < 0 || part >= s->np) return -1;
    const Box &g = s->gbox, &l = s->lbox[part];
    float gb[6] = {g.lo.x, g.lo.y, g.lo.z, g.hi.x, g.hi.y, g.hi.z};
    float lb[6] = {l.lo.x, l.lo.y, l.lo.z, l.hi.x, l.hi.y, l.hi.z};
    memcpy(out->global_box, gb, sizeof gb);
    memcpy(out->local_box, lb, sizeof lb);
    for (int k = 0; k < 6; k++) out->neighbors[k] = s->neighbors[6 * part + k];
    out->n_partitions = s->np;
    return 0;
}

int oracle_generate_initial_rays(void *sp, int part, const gxy_camera *cam, gxy_raylist *out, int32_t *n_out) {
    Scene *s = (Scene *)sp;
    Rays R;
    camera_rays(*s, part, *cam, 0, cam->height, R);
    if (R.n > out->n) return -4;
    rays_to_c(R, *out, R.n);
    *n_out = R.n;
    return 0;
}

int oracle_trace_raylist(void *sp, int part, const gxy_lighting *L, gxy_raylist *in, gxy_raylist *out,
                         int32_t *n_out) {
    Scene *s = (Scene *)sp;
    Rays R, O;
    rays_from_c(*in, R);
    trace_list(*s, part, *L, R, O, nullptr);
    rays_to_c(R, *in, R.n);
    *n_out = O.n;
    if (O.n > out->n) return -4;
    rays_to_c(O, *out, O.n);
    return 0;
}

// Trace only (TraceRays_TraceRays) with the FP64 value path; writes the
// composited rgba of every ray into rgba64 (4 per ray).
int oracle_trace_f64(void *sp, int part, gxy_raylist *in, double *rgba64) {
    Scene *s = (Scene *)sp;
    Rays R;
    rays_from_c(*in, R);
    parallel_rays(R.n, [&](int i) { trace_one<double>(*s, part, R, i, nullptr, rgba64 + 4 * i); });
    return 0;
}

// Threads used by oracle_trace_raylist and oracle_trace_f64 (default 1).
void oracle_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

int oracle_classify(gxy_raylist *rl) {
    Rays R;
    rays_from_c(*rl, R);
    classify(R);
    memcpy(rl->classification, R.cls.data(), sizeof(int32_t) * R.n);
    return 0;
}

int oracle_assign_destinations(void *sp, int part, gxy_raylist *rl) {
    Rays R;
    rays_from_c(*rl, R);
    assign_destinations(*(Scene *)sp, part, R);
    memcpy(rl->classification, R.cls.data(), sizeof(int32_t) * R.n);
    return 0;
}

int oracle_accumulate(gxy_raylist *rl, float *fb, int w, int h) {
    Rays R;
    rays_from_c(*rl, R);
    accumulate(R, fb, w, h);
    return 0;
}

// Render rows [row0,row1) (row1 <= 0 means all rows) with nthreads threads
// over row blocks; counters[0..5] = primary, shadow, ao, segments, samples,
// terminated.
int oracle_render(void *sp, const gxy_camera *cam, const gxy_lighting *L, float *fb, int nthreads, int row0, int row1,
                  int64_t *counters) {
    Scene *s = (Scene *)sp;
    if (row1 <= 0 || row1 > cam->height) row1 = cam->height;
    if (row0 < 0) row0 = 0;
    if (nthreads < 1) nthreads = 1;
    std::vector<Stats> st(nthreads);
    std::vector<int64_t> prim(nthreads, 0);
    std::atomic<int> next{row0};
    const int chunk = 4;
    auto work = [&](int tid) {
        for (;;) {
            int a = next.fetch_add(chunk);
            if (a >= row1) break;
            int b = std::min(row1, a + chunk);
            render_rows(*s, *cam, *L, fb, a, b, &st[tid], &prim[tid]);
        }
    };
    if (nthreads == 1) work(0);
    else {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; t++) th.emplace_back(work, t);
        for (auto &t : th) t.join();
    }
    if (counters) {
        int64_t c[6] = {0, 0, 0, 0, 0, 0};
        for (int t = 0; t < nthreads; t++) {
            c[0] += prim[t]; c[1] += st[t].shadow; c[2] += st[t].ao; c[3] += st[t].segments;
            c[4] += st[t].samples; c[5] += st[t].terminated;
        }
        memcpy(counters, c, sizeof c);
    }
    return 0;
}

// MappedVis::local_commit (MappedVis.cpp:277-338): resample colormap
// (x,r,g,b) and opacitymap (x,a) control points to 256 entries; valueRange is
// the data range if given, else the colormap's x span.
int oracle_tf_resample(const float *cmap, int ncm, const float *omap, int nom, int has_range, float rmin, float rmax,
                       gxy_tf *out) {
    if (ncm < 2 || nom < 2) return -1;
    int i0 = 0, i1 = 1;
    float xmin = cmap[0], xmax = cmap[4 * (ncm - 1)];
    for (int i = 0; i < 256; i++) {
        float x = xmin + (i / (255.0)) * (xmax - xmin);
        if (x > xmax) x = xmax;
        while (i1 < ncm - 1 && cmap[4 * i1] < x) i0++, i1++;
        float d = (x - cmap[4 * i0]) / (cmap[4 * i1] - cmap[4 * i0]);
        out->colors[3 * i + 0] = cmap[4 * i0 + 1] + d * (cmap[4 * i1 + 1] - cmap[4 * i0 + 1]);
        out->colors[3 * i + 1] = cmap[4 * i0 + 2] + d * (cmap[4 * i1 + 2] - cmap[4 * i0 + 2]);
        out->colors[3 * i + 2] = cmap[4 * i0 + 3] + d * (cmap[4 * i1 + 3] - cmap[4 * i0 + 3]);
    }
    i0 = 0; i1 = 1;
    xmin = omap[0]; xmax = omap[2 * (nom - 1)];
    for (int i = 0; i < 256; i++) {
        float x = xmin + (i / (255.0)) * (xmax - xmin);
        if (x > xmax) x = xmax;
        while (i1 < nom - 1 && omap[2 * i1] < x) i0++, i1++;
        float d = (x - omap[2 * i0]) / (omap[2 * i1] - omap[2 * i0]);
        out->opacities[i] = omap[2 * i0 + 1] + d * (omap[2 * i1 + 1] - omap[2 * i0 + 1]);
    }
    if (has_range) { out->range[0] = rmin; out->range[1] = rmax; }
    else { out->range[0] = cmap[0]; out->range[1] = cmap[4 * (ncm - 1)]; }
    return 0;
}

// The transfer function's opacity of one value, in single precision (the
// lookup the march composites with).
float oracle_tf_opacity(const gxy_tf *tf, float v) { return tf_opacity<float>(*tf, v); }

int oracle_ao_tables(float *u, float *v) {
    const AOTables &t = ao_tables();
    memcpy(u, t.u, sizeof t.u);
    memcpy(v, t.v, sizeof t.v);
    return 0;
}

// ColorImageWriter::Write (ImageWriter.cpp:30-48): (unsigned char)(255*v)
// without clamping, alpha 0xff, rows flipped.  The float->uchar conversion of
// an out-of-range value is undefined in C++; it is defined here as C
// truncation to int32 followed by the low 8 bits.
int oracle_quantize(const float *fb, int w, int h, uint8_t *rgba8) {
    for (int y = 0; y < h; y++) {
        uint8_t *b = rgba8 + (size_t)((h - 1) - y) * w * 4;
        const float *p = fb + (size_t)y * w * 4;
        for (int x = 0; x < w; x++) {
            for (int c = 0; c < 3; c++) {
                float v = 255.0f * p[4 * x + c];
                if (!(v > -2147483648.0f)) v = -2147483648.0f;
                if (v > 2147483520.0f) v = 2147483520.0f;
                *b++ = (uint8_t)(((uint32_t)(int32_t)v) & 0xffu);
            }
            *b++ = 0xff;
        }
    }
    return 0;
}

}  // extern "C"

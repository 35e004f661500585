// trace.cuh -- the per-ray body of Galaxy's tracer on the GPU.
//
// trace_core follows TraceRays_TraceRays (src/renderer/TraceRays.ispc:366-620)
// statement by statement: zero direction components -> 1e-6, slab clip
// against the partition box (MyIntersectBox, :90-106), slice planes
// (LookForSliceHit, :143-250), closest geometry hit through the BVH8
// (LookForGeometryHit, :108-141), the front-to-back march with isosurface
// search and compositing (:446-570) and the termination flags (:574-617).
// shade_* follow TraceRays_ambientLighting / generateAORays /
// diffuseLighting / generateShadowRays (:625-923) in the reverse-lighting
// order of TraceRays::Trace (TraceRays.cpp:124-131).
#pragma once

#include "gxy_dev.cuh"

namespace gxy {

struct TraceIn {
    V3 org, dir;        // as stored in the ray list (dir not yet adjusted)
    float t, tmax;
    float r, g, b, o;
    int type, part;
};

struct TraceOut {
    float t;
    int term;
    float r, g, b, o;
    V3 n;               // surface normal (valid when term & SURFACE)
    V3 sc;              // surface colour
    bool surface;
    bool cull;          // frame path: the ray's framebuffer contribution is provably zero
};

struct RayStats {
    unsigned samples = 0, nodes = 0, tris = 0, sphs = 0;
    unsigned skipped = 0;            // march positions whose sample was never read (clear bricks)
    int ovf = 0;
};

// Surface attributes of a geometry hit: normal (normalised, face-forwarded)
// and colour, as OSPRay postIntersect with DG_NG|DG_NS|DG_NORMALIZE|
// DG_FACEFORWARD|DG_COLOR over the DataDrivenTriangleMesh /
// DataDrivenSpheres / DataDrivenPathLines post-intersect functions.
__device__ __forceinline__ void geometry_shade_body(const DevScene &S, const GeoHit &gh, V3 org, V3 dir, V3 &n_out,
                                                    V3 &c_out) {
    V3 Ng, Ns;
    V3 col = v3(1.f, 1.f, 1.f);
    if (gh.prim & kLineBit) {
        // DataDrivenPathLines.ispc:186-196 (u and Ng of the hit) and 213-268
        int64_t p = gh.prim & ~(kSphereBit | kLineBit);
        int k = 0;
        while (k + 1 < S.n_line_sets && p >= S.line_sets[k + 1].prim_base) k++;
        const DevLineSet &L = S.line_sets[k];
        const int idx = __ldg(L.indices + (p - L.prim_base));
        const float *V = L.vertices;
        V3 A = v3(__ldg(V + 3 * idx), __ldg(V + 3 * idx + 1), __ldg(V + 3 * idx + 2));
        V3 B = v3(__ldg(V + 3 * idx + 3), __ldg(V + 3 * idx + 4), __ldg(V + 3 * idx + 5));
        V3 P = org + gh.t * dir;
        const float ab2 = dot(B - A, B - A);
        float u = ab2 == 0.f ? 0.f : dot(P - A, B - A) * (1.0f / ab2);   // zero-length segment: its end sphere
        u = fmin_(fmax_(u, 0.f), 1.f);
        V3 PonAxis = A + u * (B - A);
        Ng = nrm(P - PonAxis);
        Ns = Ng;
        float radius = ((1.f - u) * __ldg(L.radius + idx)) + (u * __ldg(L.radius + idx + 1));
        const float r0 = L.radius0, r1 = L.radius1, v0 = L.value0, v1 = L.value1;
        float dataval;
        if (r0 == r1) dataval = v0;
        else if (r0 < r1 && radius < r0) dataval = v0;
        else if (r0 < r1 && radius > r1) dataval = v1;
        else if (r0 > r1 && radius < r1) dataval = v1;
        else if (r0 > r1 && radius > r0) dataval = v0;
        else dataval = v0 + ((radius - r0) / (r1 - r0)) * (v1 - v0);
        col = tf_color(S.tfs[L.tf], dataval);
    } else if (!(gh.prim & kSphereBit)) {
        int64_t p = gh.prim;
        int k = 0;
        while (k + 1 < S.n_tri_sets && p >= S.tri_sets[k + 1].prim_base) k++;
        const DevTriSet &T = S.tri_sets[k];
        int64_t lp = p - T.prim_base;
        const int32_t *ix = T.indices + 3 * lp;
        int i0 = __ldg(ix), i1 = __ldg(ix + 1), i2 = __ldg(ix + 2);
        const float *V = T.vertices;
        V3 a = v3(__ldg(V + 3 * i0), __ldg(V + 3 * i0 + 1), __ldg(V + 3 * i0 + 2));
        V3 b = v3(__ldg(V + 3 * i1), __ldg(V + 3 * i1 + 1), __ldg(V + 3 * i1 + 2));
        V3 c = v3(__ldg(V + 3 * i2), __ldg(V + 3 * i2 + 1), __ldg(V + 3 * i2 + 2));
        Ng = cross(b - a, c - a);
        Ns = Ng;
        float bx = 1.0f - gh.u - gh.v, by = gh.u, bz = gh.v;
        if (T.normals) {
            const float *N = T.normals;
            V3 na = v3(__ldg(N + 3 * i0), __ldg(N + 3 * i0 + 1), __ldg(N + 3 * i0 + 2));
            V3 nb = v3(__ldg(N + 3 * i1), __ldg(N + 3 * i1 + 1), __ldg(N + 3 * i1 + 2));
            V3 nc = v3(__ldg(N + 3 * i2), __ldg(N + 3 * i2 + 1), __ldg(N + 3 * i2 + 2));
            Ns = (bx * na + by * nb) + bz * nc;
        }
        if (T.data) {
            float dv = bx * __ldg(T.data + i0) + by * __ldg(T.data + i1) + bz * __ldg(T.data + i2);
            col = tf_color(S.tfs[T.tf], dv);
        }
    } else {
        int64_t p = gh.prim & ~kSphereBit;
        int k = 0;
        while (k + 1 < S.n_sph_sets && p >= S.sph_sets[k + 1].prim_base) k++;
        const DevSphSet &P = S.sph_sets[k];
        int64_t lp = p - P.prim_base;
        V3 c = v3(__ldg(P.centers + 3 * lp), __ldg(P.centers + 3 * lp + 1), __ldg(P.centers + 3 * lp + 2));
        Ng = (org + gh.t * dir) - c;
        Ns = Ng;
        if (P.data) col = tf_color(S.tfs[P.tf], __ldg(P.data + lp));
    }
    Ng = nrm(Ng);
    Ns = nrm(Ns);
    if (dot(dir, Ng) >= 0.f) Ng = neg(Ng);
    if (dot(Ng, Ns) < 0.f) Ns = neg(Ns);
    n_out = Ns;
    c_out = col;
}
// One out-of-line copy: inlined into the refill query loops it raised spills.
__device__ __noinline__ void geometry_shade(const DevScene &S, const GeoHit &gh, V3 org, V3 dir, V3 &n_out,
                                            V3 &c_out) {
    geometry_shade_body(S, gh, org, dir, n_out, c_out);
}

// tfs: the volumes' transfer functions (shared-memory copies), indexed by volume.
//
// FRAME = false: the exact per-brick semantics (RayList drop-in).
// FRAME = true (whole-frame path), for shadow and AO rays only -- their only
// effect is a framebuffer contribution if they end on a surface, or nothing
// if they are dropped (reverse lighting):
//   * without volume integration, the first geometry hit in the brick
//     decides (any-hit traversal);
//   * with volume integration, one closest-hit query covers the ray's whole
//     remaining extent (t0, tMax); the in-brick hit is that hit if it lies
//     before the brick exit.  If there is no geometry hit, no slice plane and
//     no isosurface anywhere ahead, every brick the ray would cross finds no
//     surface and the ray is eventually dropped -- it is culled before the
//     march.  A ray whose payload is exactly zero adds nothing wherever it
//     ends and is culled before its query.  Culling never changes a pixel.
// SECONDARY: the caller guarantees a shadow/AO ray (no shading code).
template <bool FRAME, bool SECONDARY>
__device__ __forceinline__ TraceOut trace_core(const DevScene &S, const DevTF *tfs, const TraceIn &R, RayStats &st) {
    const DevPartition &P = S.part[R.part];
    const bool shade = !SECONDARY && R.type == GXY_RAY_PRIMARY;
    V3 org = R.org, dir = R.dir;
    if (dir.x == 0.f) dir.x = 1e-6f;
    if (dir.y == 0.f) dir.y = 1e-6f;
    if (dir.z == 0.f) dir.z = 1e-6f;
    float ray_t0 = R.t, ray_t = R.tmax;
    const float tTimeout = ray_t;
    float cr = R.r, cg = R.g, cb = R.b, ca = R.o;
    float tEntry, tExitVolume;
    {
        float rx = 1.0f / dir.x, ry = 1.0f / dir.y, rz = 1.0f / dir.z;
        float mnx = (P.lo[0] - org.x) * rx, mxx = (P.hi[0] - org.x) * rx;
        float mny = (P.lo[1] - org.y) * ry, mxy = (P.hi[1] - org.y) * ry;
        float mnz = (P.lo[2] - org.z) * rz, mxz = (P.hi[2] - org.z) * rz;
        tEntry = fmax_(fmin_(mnx, mxx), fmax_(fmin_(mny, mxy), fmin_(mnz, mxz)));
        tExitVolume = fmin_(fmax_(mnx, mxx), fmin_(fmax_(mny, mxy), fmax_(mnz, mxz)));
    }
    if (tEntry < ray_t0) tEntry = ray_t0;
    else if (tEntry > ray_t0) ray_t0 = tEntry;
    ray_t = fmin_(ray_t, tExitVolume);

    bool surface_hit = false;
    bool slice_ahead = false;   // FRAME secondaries: a slice plane in [t0, tMax]
    float hit_t = 0.f, hit_opacity = 0.f, hit_sample = 0.f;
    V3 hit_n = v3(0, 0, 0), hit_c = v3(0, 0, 0);
    TraceOut out;
    out.cull = false;
    // slice planes
    {
        int vid = -1;
        for (int m = 0; m < S.n_vol; m++) {
            const DevVolume &vv = S.vol[m];
            for (int k = 0; k < vv.n_slices; k++) {
                float4 pl = vv.slices[k];
                V3 pn = v3(pl.x, pl.y, pl.z);
                float denom = dot(dir, pn);
                if (fabsf(denom) > 0.0001f) {
                    float t = (pl.w - dot(org, pn)) / denom;
                    if (FRAME && !shade && t >= ray_t0 && t <= R.tmax) slice_ahead = true;
                    if (t >= ray_t0 && t <= ray_t) {
                        hit_n = denom > 0 ? neg(pn) : pn;
                        hit_opacity = 1.0f;
                        hit_t = t;
                        vid = m;
                        ray_t = t;
                        surface_hit = true;
                    }
                }
            }
        }
        if (surface_hit && shade) {
            V3 p = org + hit_t * dir;
            hit_sample = vol_sample(S.vol[vid], p);
            hit_c = tf_color(tfs[vid], hit_sample);
            hit_opacity = 1.0f;
        }
    }
    // geometry
    if (FRAME && !shade && !S.integrate) {
        GeoHit gh;
        if (!surface_hit &&
            bvh_closest<true>(S, org, dir, ray_t0, ray_t, gh, st.nodes, st.tris, st.sphs, st.ovf)) {
            ray_t = gh.t;
            surface_hit = true;
        }
    } else if (FRAME && !shade) {
        bool zero = R.r == 0.0f && R.g == 0.0f && R.b == 0.0f && R.o == 0.0f;
        if (zero) {   // culled whatever the query finds: skip the query
            out.cull = true;
            return out;
        }
        GeoHit gh;
        bool h = bvh_closest<false>(S, org, dir, ray_t0, R.tmax, gh, st.nodes, st.tris, st.sphs, st.ovf);
        if (h && gh.t < ray_t) {
            ray_t = gh.t;
            surface_hit = true;
        }
        if (!h && !surface_hit && !slice_ahead && !S.has_iso) {
            out.cull = true;
            return out;
        }
    } else if (S.nodes) {
        GeoHit gh;
        bool h = bvh_closest<false>(S, org, dir, ray_t0, ray_t, gh, st.nodes, st.tris, st.sphs, st.ovf);
        if (h) {
            ray_t = gh.t;
            surface_hit = true;
            if (shade) {
                geometry_shade(S, gh, org, dir, hit_n, hit_c);
                hit_opacity = 1.0f;
                hit_t = gh.t;
            }
        }
    }
    float tTermination = ray_t;
    if (S.integrate) {
        const float step = S.step, epsilon = S.march_eps, oa = S.opaque_alpha, rate = S.rate;
        const int nv = S.n_vol;
        float sLast[kMaxVol], sThis[kMaxVol];
        CellCache cc;
        cc.ix = -1; cc.iy = -1; cc.iz = -1;
        bool hit_iso = false;
        float tLast = tEntry + epsilon;
        bool opaque = (fmin_(fmin_(cr, cg), cb) >= 1.0f || ca > oa);
        float tThis = tEntry;
        while (tThis <= tTermination && !opaque && !hit_iso) {
            V3 coord = org + tThis * dir;
            if (nv == 1) sThis[0] = vol_sample_cached(S.vol[0], coord, cc);
            else
                for (int m = 0; m < nv; m++) sThis[m] = vol_sample(S.vol[m], coord);
            st.samples++;
            if (tThis > tEntry && tLast >= epsilon) {
                bool h = false;
                int vid = -1;
                for (int m = 0; m < nv; m++) {
                    const DevVolume &vv = S.vol[m];
                    float sl = sLast[m], sti = sThis[m];
                    for (int k = 0; k < vv.n_iso; k++) {
                        float iso = vv.iso[k];
                        if (((iso >= sl) && (iso < sti)) || ((iso <= sl) && (iso > sti))) {
                            h = true;
                            vid = m;
                            hit_t = tLast + ((iso - sl) / (sti - sl)) * (tThis - tLast);
                            hit_sample = iso;
                        }
                    }
                }
                if (h) {
                    if (shade) {
                        V3 hp = org + hit_t * dir;
                        V3 n = nrm(vol_gradient(S.vol[vid], hp));
                        if (dot(dir, n) > 0) n = neg(n);
                        hit_n = n;
                        hit_c = tf_color(tfs[vid], hit_sample);
                        hit_opacity = 1.0f;
                    }
                    tTermination = hit_t;
                    tThis = hit_t;
                    surface_hit = true;
                    hit_iso = true;
                    V3 c2 = org + tThis * dir;
                    for (int m = 0; m < nv; m++) sThis[m] = vol_sample(S.vol[m], c2);
                }
                for (int m = 0; m < nv; m++) {
                    const DevVolume &vv = S.vol[m];
                    if (vv.volume_render) {
                        float sv = (sLast[m] + sThis[m]) / 2.0f;
                        V3 sc;
                        float so = tf_lookup(tfs[m], sv, shade, sc);
                        if (so > 0.0f) {
                            float wo = S.rate_pow2 ? so * S.inv_rate : so / rate;
                            if (wo > 1.0f) wo = 1.0f;
                            if (wo < 0.0f) wo = 0.0f;
                            if (shade) {
                                float f = 1.0f - ca;
                                cr = cr + f * (wo * sc.x);
                                cg = cg + f * (wo * sc.y);
                                cb = cb + f * (wo * sc.z);
                                ca = ca + f * wo;
                            } else {
                                float w = ((tThis - tLast) / step) * wo;
                                float f = 1.0f - w;
                                cr = cr * f;
                                cg = cg * f;
                                cb = cb * f;
                                ca = ca * f;
                            }
                        }
                    }
                    sLast[m] = sThis[m];
                }
            }
            for (int m = 0; m < nv; m++) sLast[m] = sThis[m];
            opaque = (fmin_(fmin_(cr, cg), cb) >= 1.0f || ca > oa);
            if (opaque) tTermination = tThis;
            tLast = tThis;
            tThis = (tThis == tEntry) ? (tEntry + epsilon)
                    : (((tThis + step) > tTermination) && (tThis < tTermination)) ? tTermination
                                                                                   : tThis + step;
        }
        ray_t = tTermination;
    }
    out.r = cr; out.g = cg; out.b = cb; out.o = ca;
    bool op = fmin_(fmin_(cr, cg), cb) >= 1.0f || ca > S.opaque_alpha;
    int term = op ? GXY_RAY_OPAQUE : 0;
    out.t = ray_t;
    out.surface = surface_hit;
    if (surface_hit) {
        term |= GXY_RAY_SURFACE;
        if (hit_opacity > 0.999f) term |= GXY_RAY_OPAQUE;
        out.n = hit_n;
        out.sc = hit_c;
    } else if (tTermination == tExitVolume) {
        term |= GXY_RAY_BOUNDARY;
    } else if (tTermination == tTimeout) {
        term |= GXY_RAY_TIMEOUT;
    }
    out.term = term;
    return out;
}

// Box::exit_face (src/data/Box.cpp:84-97).
__device__ __forceinline__ int exit_face(const DevPartition &b, V3 o, V3 d) {
    const float FM = 3.402823466e+38f;
    float tx = (d.x > 0.0001f) ? ((b.hi[0] - o.x) / d.x) : (d.x < -0.0001f) ? ((b.lo[0] - o.x) / d.x) : FM;
    float ty = (d.y > 0.0001f) ? ((b.hi[1] - o.y) / d.y) : (d.y < -0.0001f) ? ((b.lo[1] - o.y) / d.y) : FM;
    float tz = (d.z > 0.0001f) ? ((b.hi[2] - o.z) / d.z) : (d.z < -0.0001f) ? ((b.lo[2] - o.z) / d.z) : FM;
    if (tx < 0) tx = FM;
    if (ty < 0) ty = FM;
    if (tz < 0) tz = FM;
    if (tx < ty && tx < tz) return (d.x < 0) ? 0 : 1;
    else if (ty < tz) return (d.y < 0) ? 2 : 3;
    else return (d.z < 0) ? 4 : 5;
}

// Renderer::Classify (Renderer.cpp:304-421), reverse lighting; RAY_BOUNDARY
// (4) marks "to the exit face" until destinations are assigned.
__device__ __forceinline__ int classify_ray(int type, int term) {
    if (type == GXY_RAY_PRIMARY) {
        if (term & GXY_RAY_BOUNDARY) return GXY_RAY_BOUNDARY;
        if ((term & GXY_RAY_OPAQUE) | (term & GXY_RAY_TIMEOUT)) return GXY_TERMINATED;
        return GXY_KEEP_HERE;
    }
    if (type == GXY_RAY_SHADOW || type == GXY_RAY_AO) {
        if ((term & GXY_RAY_OPAQUE) | (term & GXY_RAY_SURFACE)) return GXY_TERMINATED;
        if (term & GXY_RAY_BOUNDARY) return GXY_RAY_BOUNDARY;
        return GXY_DROP_ON_FLOOR;
    }
    return GXY_DROP_ON_FLOOR;
}

// Renderer::AssignDestinations (Renderer.cpp:423-454) for one ray.
__device__ __forceinline__ int assign_destination(const DevScene &S, int part, int type, int cls, V3 o, V3 d) {
    if (cls != GXY_RAY_BOUNDARY) return cls;
    int f = exit_face(S.part[part], o, d);
    int nb = S.part[part].nb[f];
    if (nb >= 0) return nb;
    return (type == GXY_RAY_SHADOW || type == GXY_RAY_AO) ? GXY_DROP_ON_FLOOR : GXY_TERMINATED;
}

// One secondary ray produced by shading.
struct Spawned {
    V3 o, d;
    float r, g, b, tmax;
    int type;
};

// Surface point + normal of a primary surface hit, the inputs of the
// lighting functions.
struct ShadeIn {
    V3 org, dir;      // stored (unadjusted) ray
    float t;
    V3 n, sc;
    int x, y;
};

// AO ray j (TraceRays.ispc:661-730) with payload ambient_{r,g,b}.
__device__ __forceinline__ Spawned ao_ray(const DevScene &S, const DevLights &L, const ShadeIn &h, int j, float ar,
                                          float ag, float ab, V3 b0, V3 b1, V3 o) {
    int r = ((h.x * 9949 + h.y * 9613 + j * 9151) >> 8) & 0xff;
    float4 tab = __ldg(S.ao + r);
    float x = tab.x * tab.z;
    float y = tab.y * tab.z;
    float z = tab.w + S.epsilon;
    V3 rd = (x * b0 + y * b1) + z * h.n;
    Spawned s;
    s.o = o;
    s.d = rd;
    s.r = ar; s.g = ag; s.b = ab;
    s.tmax = L.ao_radius;
    s.type = GXY_RAY_AO;
    return s;
}

__device__ __forceinline__ void ao_basis(V3 n, V3 &b0, V3 &b1) {
    b0 = v3(1.f, 0.f, 0.f);
    if (fabsf(dot(b0, n)) > 0.95f) b0 = v3(0.f, 1.f, 0.f);
    b1 = nrm(cross(b0, n));
    b0 = nrm(cross(b1, n));
}

}  // namespace gxy

namespace gxy {

// ------------------------------------------------------------------------
// Split tracing of shadow/AO rays in volume scenes (whole-frame path):
//   sec_query  -- box clip, slice planes and the full-extent geometry query
//                 of trace_core<true, true>; returns whether the ray is culled
//                 and otherwise the distance the march stops at
//                 (tTermination) and whether a surface ends the ray;
//   SecMarch   -- the march of trace_core (one volume, no isovalues) as a
//                 resumable state, so a lane whose ray is done can take the
//                 next ray while the others keep marching.
// The arithmetic is that of trace_core statement for statement.

struct SecQuery {
    float t_term;
    bool surface;
    bool cull;
};

__device__ __forceinline__ void sec_clip(const DevScene &S, const TraceIn &R, V3 &dir, float &ray_t0, float &ray_t,
                                         float &tEntry, float &tExitVolume) {
    const DevPartition &P = S.part[R.part];
    dir = R.dir;
    if (dir.x == 0.f) dir.x = 1e-6f;
    if (dir.y == 0.f) dir.y = 1e-6f;
    if (dir.z == 0.f) dir.z = 1e-6f;
    ray_t0 = R.t;
    ray_t = R.tmax;
    V3 org = R.org;
    float rx = 1.0f / dir.x, ry = 1.0f / dir.y, rz = 1.0f / dir.z;
    float mnx = (P.lo[0] - org.x) * rx, mxx = (P.hi[0] - org.x) * rx;
    float mny = (P.lo[1] - org.y) * ry, mxy = (P.hi[1] - org.y) * ry;
    float mnz = (P.lo[2] - org.z) * rz, mxz = (P.hi[2] - org.z) * rz;
    tEntry = fmax_(fmin_(mnx, mxx), fmax_(fmin_(mny, mxy), fmin_(mnz, mxz)));
    tExitVolume = fmin_(fmax_(mnx, mxx), fmin_(fmax_(mny, mxy), fmax_(mnz, mxz)));
    if (tEntry < ray_t0) tEntry = ray_t0;
    else if (tEntry > ray_t0) ray_t0 = tEntry;
    ray_t = fmin_(ray_t, tExitVolume);
}

__device__ __forceinline__ SecQuery sec_query(const DevScene &S, const TraceIn &R, RayStats &st) {
    SecQuery q;
    V3 dir;
    float ray_t0, ray_t, tEntry, tExitVolume;
    sec_clip(S, R, dir, ray_t0, ray_t, tEntry, tExitVolume);
    const V3 org = R.org;
    bool surface_hit = false, slice_ahead = false;
    for (int m = 0; m < S.n_vol; m++) {
        const DevVolume &vv = S.vol[m];
        for (int k = 0; k < vv.n_slices; k++) {
            float4 pl = vv.slices[k];
            V3 pn = v3(pl.x, pl.y, pl.z);
            float denom = dot(dir, pn);
            if (fabsf(denom) > 0.0001f) {
                float t = (pl.w - dot(org, pn)) / denom;
                if (t >= ray_t0 && t <= R.tmax) slice_ahead = true;
                if (t >= ray_t0 && t <= ray_t) {
                    ray_t = t;
                    surface_hit = true;
                }
            }
        }
    }
    // a zero payload is culled whatever the query finds: skip the query
    bool zero = R.r == 0.0f && R.g == 0.0f && R.b == 0.0f && R.o == 0.0f;
    GeoHit gh;
    bool h = !zero && bvh_closest<false>(S, org, dir, ray_t0, R.tmax, gh, st.nodes, st.tris, st.sphs, st.ovf);
    if (h && gh.t < ray_t) {
        ray_t = gh.t;
        surface_hit = true;
    }
    q.cull = zero || (!h && !surface_hit && !slice_ahead && !S.has_iso);
    q.t_term = ray_t;
    q.surface = surface_hit;
    return q;
}

struct SecMarch {
    V3 org, dir;
    float tEntry, tExitVolume, tTimeout, tTerm, tThis, tLast, sLast;
    float cr, cg, cb, ca;
    bool surface, opaque, done;
    bool bclear;                     // the brick `bid` is clear
    bool prev_clear;                 // the previous position lay in a clear brick
    bool lazy;                       // sLast not read yet (its interval composited nothing)
    int bid;
    int sbid;                        // superbrick whose clear run was last looked up
    float tRun;                      // positions t < tRun lie in a run of clear superbricks
    CellCache cc;
};

// Sample position of march distance t; one expression at every use (device
// code is built without multiply-add contraction), so a sample read late
// (SecMarch::lazy) equals the one its own step would have read.
__device__ __forceinline__ V3 march_point(const SecMarch &M, float t) { return M.org + t * M.dir; }

__device__ __forceinline__ void sec_march_init(const DevScene &S, const TraceIn &R, float t_term, bool surface,
                                               SecMarch &M) {
    float ray_t0, ray_t;
    sec_clip(S, R, M.dir, ray_t0, ray_t, M.tEntry, M.tExitVolume);
    M.org = R.org;
    M.tTimeout = R.tmax;
    M.tTerm = t_term;
    M.surface = surface;
    M.cr = R.r; M.cg = R.g; M.cb = R.b; M.ca = R.o;
    M.tLast = M.tEntry + S.march_eps;
    M.opaque = (fmin_(fmin_(M.cr, M.cg), M.cb) >= 1.0f || M.ca > S.opaque_alpha);
    M.tThis = M.tEntry;
    M.sLast = 0.0f;
    M.cc.ix = -1; M.cc.iy = -1; M.cc.iz = -1;
    M.bid = -1;
    M.sbid = -1;
    M.tRun = -INFINITY;
    M.bclear = false;
    M.prev_clear = false;
    M.lazy = false;
    M.done = !(M.tThis <= M.tTerm && !M.opaque);
}

// Up to `steps` iterations of the march loop (TraceRays.ispc:470-556), as a
// resumable state.  PRIMARY composites front to back with the primary-ray
// weight `color += (1 - color.a) * clamp(alpha/rate) * [rgb, 1]`; otherwise
// the shadow/AO attenuation `color *= 1 - (dt/step) * clamp(alpha/rate)`.
//
// Empty-space skipping with unchanged results: an interval between two
// positions that both lie in clear bricks has zero opacity (tf_clear_below),
// so its compositing is a no-op and neither sample is needed for it.  The
// step then reads no voxels; the position still counts as a sample and the
// distance sequence (tThis, tLast, tTerm) advances exactly as Galaxy's.  A
// sample skipped this way is read later, from the same position, only if
// the next interval does composite.
// Distances t >= t0 along the ray over which every sample position lies in
// the brick of g, as vol_pos computes positions: the ray's span inside the
// brick's box shrunk by m = 1/64 voxel per side.  Per axis, to first order,
// the computed grid coordinate of org + t*dir differs from the exact one by
// at most u (|inv| (3|t d| + 2|o| + |vo|) + |g|), and the exact coordinate at
// a computed slab distance (B - g0) * rcp(d * inv) from the slab B by at most
// u (2 |inv| (|o| + |vo|) + 4 |inv| |t d|), u = 2^-24.  Their sum stays below
// u K with K = 7 |inv| (T |d| + |o| + |vo|) + 2 (hi + 1) (T the largest |t|,
// hi the box's upper grid coordinate, which also covers the rounding of the
// shrunk bounds); K < 2^17 keeps it under m / 2.  False when that bound
// fails on some axis or the span is empty.  A zero direction component
// leaves its coordinate exactly constant (o + t*0 == o).
__device__ __forceinline__ bool brick_axis(float o, float d, float vo, float inv, int b, float t0, float &lo_t,
                                           float &hi_t) {
    constexpr float m = 1.0f / 64.0f;
    if (d == 0.0f) {
        lo_t = -INFINITY;
        hi_t = INFINITY;
        return true;
    }
    const float lo = (float)(kBrick * b) + m, hi = (float)(kBrick * b + kBrick) - m;
    const float g0 = (o - vo) * inv, dg = d * inv;
    if (dg == 0.0f) return false;
    const float r = __frcp_rn(dg);
    const float ta = (lo - g0) * r, tb = (hi - g0) * r;
    lo_t = fminf(ta, tb);
    hi_t = fmaxf(ta, tb);
    const float T = fmaxf(fabsf(t0), fabsf(hi_t));
    return 7.0f * fabsf(inv) * (T * fabsf(d) + fabsf(o) + fabsf(vo)) + 2.0f * (hi + 1.0f) < 131072.0f;
}

__device__ __forceinline__ bool brick_span(const DevVolume &v, V3 org, V3 dir, const VolPos &g, float t0,
                                           float &t_in, float &t_out) {
    float lx, hx, ly, hy, lz, hz;
    if (!brick_axis(org.x, dir.x, v.ox, v.ix, g.ix >> 2, t0, lx, hx)) return false;
    if (!brick_axis(org.y, dir.y, v.oy, v.iy, g.iy >> 2, t0, ly, hy)) return false;
    if (!brick_axis(org.z, dir.z, v.oz, v.iz, g.iz >> 2, t0, lz, hz)) return false;
    t_in = fmaxf(fmaxf(lx, ly), lz);
    t_out = fminf(fminf(hx, hy), hz);
    return t_in <= t_out;
}

// End of the run of clear superbricks that holds the cell of g at distance
// t0: the distance at which the ray enters a superbrick that is not clear,
// +inf when it enters none before tEnd.  A 3-D DDA over the superbrick grid
// along G(t) = (org - origin) * inv + t * dir * inv; a position the march
// computes at t < the result lies, up to rounding far below a voxel (K <
// 2^20 per axis: under 1/16 voxel), in or next to a visited superbrick, so
// in a brick their dilated flags cover.  Positions outside the grid clamp
// to its edge cells, so an axis that leaves the grid stays on its edge
// superbrick.  At most 64 superbricks per call.
// One axis of the DDA: the distance of the next superbrick boundary and
// the distance between boundaries; false when the rounding bound fails.
__device__ __forceinline__ bool dda_axis(float o, float d, float vo, float inv, int c, float T, int &sgn, float &tn,
                                         float &dt) {
    if (!(fabsf(inv) * (T * fabsf(d) + fabsf(o) + fabsf(vo)) < 1048576.0f)) return false;
    // (one rounded reciprocal instead of two divisions: the superbricks'
    // one-brick dilation dwarfs the extra rounding)
    const float g0 = (o - vo) * inv, dg = d * inv, r = __frcp_rn(dg);
    if (dg > 0.0f) {
        sgn = 1;
        tn = ((float)((c + 1) * kSuperCells) - g0) * r;
        dt = (float)kSuperCells * r;
    } else if (dg < 0.0f) {
        sgn = -1;
        tn = ((float)(c * kSuperCells) - g0) * r;
        dt = -(float)kSuperCells * r;
    } else {
        sgn = 0;
        tn = INFINITY;
        dt = 0.0f;
    }
    return true;
}

// Step one axis of the DDA; an axis that leaves the grid stays on its edge
// superbrick (positions outside the grid clamp to its edge cells).
__device__ __forceinline__ void dda_step(int &c, int sgn, int n, float &tn, float dt) {
    c += sgn;
    tn += dt;
    if (c < 0 || c >= n) {
        c = c < 0 ? 0 : n - 1;
        tn = INFINITY;
    }
}

__device__ __forceinline__ float clear_run_end(const DevVolume &v, V3 org, V3 dir, const VolPos &g, float t0,
                                               float tEnd) {
    const float T = fmaxf(fabsf(t0), fabsf(tEnd));
    int cx = g.ix >> 5, cy = g.iy >> 5, cz = g.iz >> 5, sx, sy, sz;
    float tx, ty, tz, dx, dy, dz;
    if (!dda_axis(org.x, dir.x, v.ox, v.ix, cx, T, sx, tx, dx) || !dda_axis(org.y, dir.y, v.oy, v.iy, cy, T, sy, ty, dy) ||
        !dda_axis(org.z, dir.z, v.oz, v.iz, cz, T, sz, tz, dz))
        return t0;
    float t = fminf(fminf(tx, ty), tz);
    for (int k = 0; k < 64; k++) {
        if (!(t <= tEnd)) return INFINITY;
        if (t == tx) dda_step(cx, sx, v.nsx, tx, dx);
        else if (t == ty) dda_step(cy, sy, v.nsy, ty, dy);
        else dda_step(cz, sz, v.nsz, tz, dz);
        if (!__ldg(v.sclear + (cz * v.nsy + cy) * v.nsx + cx)) return t;
        t = fminf(fminf(tx, ty), tz);
    }
    return t;
}

// Positions one fast run may pass over (a brick holds at most about
// 4 sqrt(3) * sampling_rate of them; the cap only bounds the loop), and one
// pass of a superbrick run.
constexpr int kMaxRun = 64;
constexpr int kMaxCount = 4096;

// Composite the interval ending at tThis whose sample value is sv.
template <bool PRIMARY>
__device__ __forceinline__ void march_composite(const DevScene &S, const DevTF &tf, SecMarch &M, float sv,
                                                float tThis) {
    V3 sc;
    float so = tf_lookup(tf, sv, PRIMARY, sc);
    if (so > 0.0f) {
        float wo = S.rate_pow2 ? so * S.inv_rate : so / S.rate;
        if (wo > 1.0f) wo = 1.0f;
        if (wo < 0.0f) wo = 0.0f;
        if (PRIMARY) {
            float f = 1.0f - M.ca;
            M.cr = M.cr + f * (wo * sc.x);
            M.cg = M.cg + f * (wo * sc.y);
            M.cb = M.cb + f * (wo * sc.z);
            M.ca = M.ca + f * wo;
        } else {
            float w = ((tThis - M.tLast) / S.step) * wo;
            float f = 1.0f - w;
            M.cr = M.cr * f;
            M.cg = M.cg * f;
            M.cb = M.cb * f;
            M.ca = M.ca * f;
        }
        // only a composited interval changes the colour, so only here can
        // the ray become opaque (it was not before)
        M.opaque = (fmin_(fmin_(M.cr, M.cg), M.cb) >= 1.0f || M.ca > S.opaque_alpha);
        if (M.opaque) M.tTerm = tThis;
    }
}

// Next march distance after tThis (TraceRays.ispc:548-553).
__device__ __forceinline__ float march_next(float t, float tEntry, float epsilon, float step, float tTerm) {
    return (t == tEntry) ? (tEntry + epsilon) : (((t + step) > tTerm) && (t < tTerm)) ? tTerm : t + step;
}

// Pass over the positions t of the distance sequence with t < tr and
// t <= tTerm, exactly as repeated march_next would, counting them (at most
// cap); t becomes the first position not passed over, tl the last one
// passed over.  Inside one binade [2^(e-1), 2^e) of positive floats, with
// t away from tEntry, fl(t + step) = t + D ulps for a fixed D: the floats of
// the binade are the integers of their bit patterns, t is on that grid, and
// the rounding of t + step to it does not depend on t except on an exact
// tie (step / ulp = n + 1/2, left to single steps).  So a chunk of positions
// is an arithmetic progression in the bit pattern, taken while every
// position stays below tr and every successor stays at or below tTerm (no
// clamp) and at least one ulp below the binade's end (t + step then rounds
// inside the binade).  Other positions take single march_next steps.
__device__ __forceinline__ int advance_clear(float &t, float &tl, float tr, float tTerm, float tEntry, float epsilon,
                                             float step, int cap) {
    int k = 0;
    while (k < cap && t < tr && t <= tTerm) {
        const int tb = __float_as_int(t);
        const int E = (tb >> 23) & 0xff;
        if (t > 0.0f && t != tEntry && E >= 24 && E < 254) {
            const int bend = (tb & 0x7f800000) + 0x00800000;
            const float tn = t + step;
            const int D = __float_as_int(tn) - tb;
            const float r = step * __int_as_float((277 - E) << 23);   // step / ulp(t), exact
            if (D >= 1 && __float_as_int(tn) < bend && r - floorf(r) != 0.5f) {
                const int A = min(__float_as_int(tTerm), bend - 1) - tb;
                const int B = tr < INFINITY ? __float_as_int(tr) - tb : 0x7fffffff;
                int m = min(A / D, (B - 1) / D + 1);
                m = min(m, cap - k);
                if (m >= 1) {
                    tl = __int_as_float(tb + (m - 1) * D);
                    t = __int_as_float(tb + m * D);
                    k += m;
                    continue;
                }
            }
        }
        tl = t;
        t = march_next(t, tEntry, epsilon, step, tTerm);
        k++;
    }
    return k;
}

// Lean skipping: if the position at tp (already marched, or the first
// position tEntry) lies in a clear superbrick, pass over the following
// positions of the clear superbrick run ahead (their predecessors are all
// clear), then read the sample of the last one passed over, so the plain
// march resumes with a valid sLast.
__device__ __forceinline__ void lean_run(const DevVolume &vv, SecMarch &M, float tp, float epsilon, float step,
                                         RayStats &st) {
    const VolPos g = vol_pos(vv, march_point(M, tp));
    if (!__ldg(vv.sclear + super_of(vv, g))) return;
    const float tr = clear_run_end(vv, M.org, M.dir, g, tp, M.tTerm);
    float t = M.tThis, tl = M.tLast;
    const int k = advance_clear(t, tl, tr, M.tTerm, M.tEntry, epsilon, step, kMaxCount);
    if (k) {
        M.tThis = t;
        M.tLast = tl;
        M.done = !(t <= M.tTerm);
        st.samples += k;
        st.skipped += k;
        if (!M.done) {
            M.sLast = vol_sample_at(vv, vol_pos(vv, march_point(M, tl)), M.cc);
            st.skipped--;
        }
    }
}

// SKIP 0: every position sampled.  SKIP 1 (lean): as 0, plus, at the
// first position and after each refill round, a jump over the run of clear
// superbricks ahead (lean_run); no extra march state.  SKIP 2: per-position
// clear-brick skipping with lazy samples, superbrick runs and (runs) brick
// runs.  The scene must carry the clear flags for 1 and 2.
template <bool PRIMARY, int SKIP>
__device__ __forceinline__ void march_steps(const DevScene &S, const DevTF &tf, SecMarch &M, int steps, int runs,
                                            RayStats &st) {
    const DevVolume &vv = S.vol[0];
    const float step = S.step, epsilon = S.march_eps;
    if constexpr (SKIP < 2) {
        if (SKIP == 1 && M.tThis == M.tEntry) lean_run(vv, M, M.tEntry, epsilon, step, st);
        for (int it = 0; it < steps && !M.done; it++) {
            float tThis = M.tThis;
            float sThis = vol_sample_at(vv, vol_pos(vv, march_point(M, tThis)), M.cc);
            st.samples++;
            if (tThis > M.tEntry && M.tLast >= epsilon && vv.volume_render)
                march_composite<PRIMARY>(S, tf, M, (M.sLast + sThis) / 2.0f, tThis);
            M.sLast = sThis;
            M.tLast = tThis;
            M.tThis = march_next(tThis, M.tEntry, epsilon, step, M.tTerm);
            M.done = !(M.tThis <= M.tTerm && !M.opaque);
        }
        if (SKIP == 1 && !M.done) lean_run(vv, M, M.tLast, epsilon, step, st);
    } else {
        for (int it = 0; it < steps && !M.done; it++) {
            if (M.tThis < M.tRun) {
                // inside a run of clear superbricks whose previous position is
                // clear too: only the distance sequence advances
                float t = M.tThis, tl = M.tLast;
                const float tTerm = M.tTerm;
                const int k = advance_clear(t, tl, M.tRun, tTerm, M.tEntry, epsilon, step, kMaxCount);
                M.tThis = t;
                M.tLast = tl;
                M.lazy = true;
                M.prev_clear = true;
                M.done = !(t <= tTerm);
                st.samples += k;
                st.skipped += k;
                continue;
            }
            float tThis = M.tThis;
            VolPos g = vol_pos(vv, march_point(M, tThis));
            int bid = brick_of(vv, g);
            if (bid != M.bid) {
                M.bid = bid;
                M.bclear = __ldg(vv.clear + bid) != 0;
            }
            st.samples++;
            if (tThis > M.tEntry && M.tLast >= epsilon && vv.volume_render && !(M.bclear && M.prev_clear)) {
                if (M.lazy) {
                    M.sLast = vol_sample_at(vv, vol_pos(vv, march_point(M, M.tLast)), M.cc);
                    st.skipped--;
                }
                float sThis = vol_sample_at(vv, g, M.cc);
                march_composite<PRIMARY>(S, tf, M, (M.sLast + sThis) / 2.0f, tThis);
                M.sLast = sThis;
                M.lazy = false;
            } else {
                M.lazy = true;
                st.skipped++;
            }
            M.prev_clear = M.bclear;
            M.tLast = tThis;
            M.tThis = march_next(tThis, M.tEntry, epsilon, step, M.tTerm);
            M.done = !(M.tThis <= M.tTerm && !M.opaque);
            // A clear brick in a superbrick not looked up yet: find the run of
            // clear superbricks ahead (the next iterations count through it).
            if (M.bclear && !M.done) {
                const int sb = super_of(vv, g);
                if (sb != M.sbid) {
                    M.sbid = sb;
                    if (__ldg(vv.sclear + sb)) {
                        M.tRun = clear_run_end(vv, M.org, M.dir, g, tThis, M.tTerm);
                        if (M.tThis < M.tRun) continue;
                    }
                }
            }
            // Fast run through the rest of a clear brick: the positions that
            // provably stay in it (brick_span) have clear intervals on both
            // sides, so only the distance sequence advances.  The colour, and
            // with it `opaque` (false here), does not change.
            float t_in, t_out;
            if (runs && !M.done && M.bclear && brick_span(vv, M.org, M.dir, g, tThis, t_in, t_out) &&
                M.tThis >= t_in) {
                float t = M.tThis, tl = M.tLast;
                const float tTerm = M.tTerm;
                // positions t <= t_out: below the next float up from t_out
                const int k = advance_clear(t, tl, nextafterf(t_out, INFINITY), tTerm, M.tEntry, epsilon, step, kMaxRun);
                if (k) {
                    M.tThis = t;
                    M.tLast = tl;
                    M.lazy = true;
                    M.done = !(t <= tTerm);
                    st.samples += k;
                    st.skipped += k;
                }
            }
        }
    }
}

template <int SKIP>
__device__ __forceinline__ void sec_march_steps(const DevScene &S, const DevTF &tf, SecMarch &M, int steps,
                                                int runs, RayStats &st) {
    march_steps<false, SKIP>(S, tf, M, steps, runs, st);
}

// Termination flags of a finished march (TraceRays.ispc:574-617, shadow/AO).
__device__ __forceinline__ int sec_march_term(const DevScene &S, const SecMarch &M) {
    bool op = fmin_(fmin_(M.cr, M.cg), M.cb) >= 1.0f || M.ca > S.opaque_alpha;
    int term = op ? GXY_RAY_OPAQUE : 0;
    if (M.surface) term |= GXY_RAY_SURFACE;
    else if (M.tTerm == M.tExitVolume) term |= GXY_RAY_BOUNDARY;
    else if (M.tTerm == M.tTimeout) term |= GXY_RAY_TIMEOUT;
    return term;
}

}  // namespace gxy

namespace gxy {

// ------------------------------------------------------------------------
// Split tracing of primary rays in volume scenes (whole-frame path): the
// camera queries (k_cam_packet, k_cam_query in render.cu) clip the ray to
// its brick (sec_clip), take the nearest slice plane with its surface colour
// (cam_slices) and then the in-brick closest geometry hit with its normal and
// colour -- trace_core<true,false> up to the march; prim_march_steps then
// composites the volume up to that distance as a resumable state.
__device__ __forceinline__ void cam_slices(const DevScene &S, const DevTF *tfs, V3 org, V3 dir, float ray_t0,
                                           float &ray_t, bool &surface, V3 &hit_n, V3 &hit_c) {
    float hit_t = 0.f;
    int vid = -1;
    for (int m = 0; m < S.n_vol; m++) {
        const DevVolume &vv = S.vol[m];
        for (int k = 0; k < vv.n_slices; k++) {
            float4 pl = vv.slices[k];
            V3 pn = v3(pl.x, pl.y, pl.z);
            float denom = dot(dir, pn);
            if (fabsf(denom) > 0.0001f) {
                float t = (pl.w - dot(org, pn)) / denom;
                if (t >= ray_t0 && t <= ray_t) {
                    hit_n = denom > 0 ? neg(pn) : pn;
                    hit_t = t;
                    vid = m;
                    ray_t = t;
                    surface = true;
                }
            }
        }
    }
    if (surface) hit_c = tf_color(tfs[vid], vol_sample(S.vol[vid], org + hit_t * dir));
}

// Compositing march of a primary ray (TraceRays.ispc:470-556 with the
// primary-ray weight).
template <int SKIP>
__device__ __forceinline__ void prim_march_steps(const DevScene &S, const DevTF &tf, SecMarch &M, int steps,
                                                 int runs, RayStats &st) {
    march_steps<true, SKIP>(S, tf, M, steps, runs, st);
}

// Termination flags of a finished primary march: a surface found with
// shading has opacity 1 (TraceRays.ispc:195,240,304; postIntersect colour w=1).
__device__ __forceinline__ int prim_march_term(const DevScene &S, const SecMarch &M) {
    bool op = fmin_(fmin_(M.cr, M.cg), M.cb) >= 1.0f || M.ca > S.opaque_alpha;
    int term = op ? GXY_RAY_OPAQUE : 0;
    if (M.surface) term |= GXY_RAY_SURFACE | GXY_RAY_OPAQUE;
    else if (M.tTerm == M.tExitVolume) term |= GXY_RAY_BOUNDARY;
    else if (M.tTerm == M.tTimeout) term |= GXY_RAY_TIMEOUT;
    return term;
}

}  // namespace gxy

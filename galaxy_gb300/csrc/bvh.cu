// bvh.cu -- GPU construction of the 8-wide BVH over triangles and spheres.
//
// Replaces the Embree BVH that ospCommit(model) builds in Galaxy
// (Visualization::SetOsprayObjects, src/renderer/Visualization.cpp:207-285).
//
// Steps, all on the device:
//  1. primitive bounds and centroid bounds;
//  2. 63-bit Morton codes (21 bits per axis) and a radix sort of (code, id);
//  3. Karras' binary radix tree (LBVH) over the sorted codes;
//  4. bottom-up refit of the binary nodes' boxes;
//  5. top-down collapse to 8-wide nodes, one kernel per level: each wide node
//     starts from a binary node's two children and repeatedly opens the child
//     with the largest surface area (the surface-area-heuristic greedy
//     choice) until it has 8 children; subtrees of at most kLeafMax
//     primitives (leaf_max(): 1-4, so 8 leaves fit the 5-bit primitive
//     offset of a meta byte) become leaves.  Child boxes are quantised to 16 bits
//     against a power-of-two grid so a node fills one 128-byte line.
#include <cub/cub.cuh>

#include <cfloat>
#include <cstring>
#include <algorithm>
#include <chrono>
#include <vector>

#include "gxy_dev.cuh"
#include "gxy_host.h"

namespace gxy {

__device__ __forceinline__ void prim_box(const DevScene &S, uint32_t p, float3 &lo, float3 &hi) {
    if (p < S.n_tri) {
        int s = 0;
        while (s + 1 < S.n_tri_sets && p >= S.tri_sets[s + 1].prim_base) s++;
        const DevTriSet &T = S.tri_sets[s];
        int64_t lp = p - T.prim_base;
        const int32_t *ix = T.indices + 3 * lp;
        float3 a = make_float3(T.vertices[3 * ix[0]], T.vertices[3 * ix[0] + 1], T.vertices[3 * ix[0] + 2]);
        float3 b = make_float3(T.vertices[3 * ix[1]], T.vertices[3 * ix[1] + 1], T.vertices[3 * ix[1] + 2]);
        float3 c = make_float3(T.vertices[3 * ix[2]], T.vertices[3 * ix[2] + 1], T.vertices[3 * ix[2] + 2]);
        lo = make_float3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
        hi = make_float3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
    } else if ((int64_t)p < S.n_tri + S.n_sph) {
        int s = 0;
        while (s + 1 < S.n_sph_sets && (int64_t)p >= S.sph_sets[s + 1].prim_base) s++;
        const DevSphSet &P = S.sph_sets[s];
        int64_t lp = (int64_t)p - P.prim_base;
        lo = hi = make_float3(P.centers[3 * lp], P.centers[3 * lp + 1], P.centers[3 * lp + 2]);   // radius added by caller
    } else {
        // DataDrivenPathLines_bounds (DataDrivenPathLines.ispc:37-68): segment box grown by radius0
        int s = 0;
        while (s + 1 < S.n_line_sets && (int64_t)p >= S.line_sets[s + 1].prim_base) s++;
        const DevLineSet &L = S.line_sets[s];
        const int idx = L.indices[(int64_t)p - L.prim_base];
        const float *a = L.vertices + 3 * idx, *b = a + 3;
        const float r = L.radius0;
        lo = make_float3(fminf(a[0], b[0]) - r, fminf(a[1], b[1]) - r, fminf(a[2], b[2]) - r);
        hi = make_float3(fmaxf(a[0], b[0]) + r, fmaxf(a[1], b[1]) + r, fmaxf(a[2], b[2]) + r);
    }
}

struct BuildBuffers {
    float4 *plo = nullptr, *phi = nullptr;           // primitive boxes (by prim id)
    unsigned long long *keys = nullptr, *keys2 = nullptr;
    uint32_t *ids = nullptr, *ids2 = nullptr;
    int *left = nullptr, *right = nullptr, *parent = nullptr, *first = nullptr, *last = nullptr;
    int *flags = nullptr;
    float4 *nlo = nullptr, *nhi = nullptr;           // binary internal node boxes
    int2 *qa = nullptr, *qb = nullptr;               // work queues (binary ref, wide index)
    unsigned int *ctr = nullptr;                     // [0] nodes [1] slots [2] queue out
    unsigned int *cbounds = nullptr;                 // centroid bounds as ordered uints
};

__device__ __forceinline__ unsigned int f2o(float f) {   // order-preserving float -> uint
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(unsigned int u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Primitive boxes.  Spheres use the radius array prepared by the commit
// (sph_radius, by sphere index).
__global__ void k_prim_bounds(DevScene S, const float *sph_radius, int64_t n, float4 *plo, float4 *phi,
                              unsigned int *cb) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float3 lo = make_float3(FLT_MAX, FLT_MAX, FLT_MAX), hi = make_float3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    float3 c = make_float3(0, 0, 0);
    bool valid = p < n;
    if (valid) {
        prim_box(S, (uint32_t)p, lo, hi);
        if (p >= S.n_tri && p < S.n_tri + S.n_sph) {
            float r = sph_radius[p - S.n_tri];
            lo = make_float3(lo.x - r, lo.y - r, lo.z - r);
            hi = make_float3(hi.x + r, hi.y + r, hi.z + r);
        }
        plo[p] = make_float4(lo.x, lo.y, lo.z, 0.0f);
        phi[p] = make_float4(hi.x, hi.y, hi.z, 0.0f);
        c = make_float3(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z));
    }
    // block reduction of centroid bounds
    __shared__ float s[6][32];
    float v[6] = {valid ? c.x : FLT_MAX, valid ? c.y : FLT_MAX, valid ? c.z : FLT_MAX,
                  valid ? c.x : -FLT_MAX, valid ? c.y : -FLT_MAX, valid ? c.z : -FLT_MAX};
    for (int k = 0; k < 6; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            float w = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k] = k < 3 ? fminf(v[k], w) : fmaxf(v[k], w);
        }
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 6; k++) s[k][warp] = v[k];
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        for (int k = 0; k < 6; k++) {
            float w = lane < nw ? s[k][lane] : (k < 3 ? FLT_MAX : -FLT_MAX);
            for (int o = 16; o > 0; o >>= 1) {
                float x = __shfl_xor_sync(0xffffffffu, w, o);
                w = k < 3 ? fminf(w, x) : fmaxf(w, x);
            }
            if (lane == 0) {
                if (k < 3) atomicMin(&cb[k], f2o(w));
                else atomicMax(&cb[k], f2o(w));
            }
        }
    }
}

__device__ __forceinline__ unsigned long long spread21(unsigned long long x) {
    x &= 0x1fffffull;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(int64_t n, const float4 *plo, const float4 *phi, const unsigned int *cb,
                         unsigned long long *keys, uint32_t *ids) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    float lo[3] = {o2f(cb[0]), o2f(cb[1]), o2f(cb[2])};
    float hi[3] = {o2f(cb[3]), o2f(cb[4]), o2f(cb[5])};
    float4 a = plo[p], b = phi[p];
    float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    unsigned long long q[3];
    for (int k = 0; k < 3; k++) {
        float e = hi[k] - lo[k];
        float f = e > 0.0f ? (c[k] - lo[k]) / e : 0.5f;
        f = fminf(fmaxf(f, 0.0f), 1.0f);
        q[k] = (unsigned long long)fminf(f * 2097152.0f, 2097151.0f);
    }
    keys[p] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    ids[p] = (uint32_t)p;
}

__device__ __forceinline__ int delta(const unsigned long long *k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll(a ^ b);
}

// Karras 2012: internal node i of the binary radix tree.  Children are
// encoded as >= 0 internal index or ~leaf for leaves.
__global__ void k_karras(int n, const unsigned long long *k, int *left, int *right, int *parent, int *first, int *last,
                         int *leaf_parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(k, n, i, i - d);
    int lmax = 2;
    while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(k, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int g = i + s * d + (d < 0 ? -1 : 0);
    int lo = i < j ? i : j, hi = i < j ? j : i;
    int lc = (lo == g) ? ~g : g;
    int rc = (hi == g + 1) ? ~(g + 1) : g + 1;
    left[i] = lc;
    right[i] = rc;
    first[i] = lo;
    last[i] = hi;
    if (lc >= 0) parent[lc] = i; else leaf_parent[~lc] = i;
    if (rc >= 0) parent[rc] = i; else leaf_parent[~rc] = i;
}

__global__ void k_refit(int n, const uint32_t *ids, const float4 *plo, const float4 *phi, const int *left,
                        const int *right, const int *parent, const int *leaf_parent, int *flags, float4 *nlo,
                        float4 *nhi) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = leaf_parent[i];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&flags[node], 1) == 0) return;   // first arrival: sibling not ready
        __threadfence();
        int c[2] = {left[node], right[node]};
        float4 lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0), hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0);
        for (int k = 0; k < 2; k++) {
            float4 a, b;
            if (c[k] >= 0) { a = __ldcg(&nlo[c[k]]); b = __ldcg(&nhi[c[k]]); }
            else { uint32_t p = ids[~c[k]]; a = plo[p]; b = phi[p]; }
            lo = make_float4(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z), 0);
            hi = make_float4(fmaxf(hi.x, b.x), fmaxf(hi.y, b.y), fmaxf(hi.z, b.z), 0);
        }
        __stcg(&nlo[node], lo);
        __stcg(&nhi[node], hi);
        node = node == 0 ? -1 : parent[node];
    }
}

// ---------------------------------------------------------------------
// Binned-SAH refinement of the top of the radix tree.  The radix tree is cut
// into clusters -- maximal subtrees of at most C primitives -- and the tree
// above them is rebuilt top down by binned SAH over the clusters' boxes
// (k_sah_level, on the device), so the levels that every ray visits get
// surface-area splits while the bottom keeps the Morton structure.
__global__ void k_clusters(int n, int C, const int *parent, const int *leaf_parent, const int *first, const int *last,
                           int *refs, unsigned int *count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n - 1) {   // internal node i
        int size = last[i] - first[i] + 1;
        if (size <= C) {
            int p = i == 0 ? -1 : parent[i];
            if (p < 0 || last[p] - first[p] + 1 > C) refs[atomicAdd(count, 1u)] = i;
        }
    }
    if (i < n) {       // leaf i (a single primitive) under a node larger than C
        int p = leaf_parent[i];
        if (last[p] - first[p] + 1 > C) refs[atomicAdd(count, 1u)] = ~i;
    }
}

__global__ void k_cluster_info(int m, const int *refs, const uint32_t *ids, const float4 *plo, const float4 *phi,
                               const int *first, const int *last, const float4 *nlo, const float4 *nhi,
                               float4 *clo, float4 *chi) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    int r = refs[k];
    float4 a, b;
    int cnt;
    if (r >= 0) { a = nlo[r]; b = nhi[r]; cnt = last[r] - first[r] + 1; }
    else { uint32_t p = ids[~r]; a = plo[p]; b = phi[p]; cnt = 1; }
    a.w = __int_as_float(cnt);
    clo[k] = a;
    chi[k] = b;
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    float x = hi.x - lo.x, y = hi.y - lo.y, z = hi.z - lo.z;
    return x * y + y * z + z * x;
}

__device__ __forceinline__ uint8_t quant_exp(float extent) {
    float s = extent / 65535.0f;
    if (!(s > 0.0f)) return 1;
    uint32_t b = __float_as_uint(s);
    uint32_t e = (b >> 23) & 0xffu;
    if (b & 0x7fffffu) e++;
    if (e < 1) e = 1;
    if (e > 254) e = 254;
    return (uint8_t)e;
}

// Leaf primitive slot record (3 float4), see BVH8Node in gxy_dev.cuh.
__device__ void write_slot(const DevScene &S, const float *sph_radius, uint32_t p, float4 *slots, uint32_t s) {
    float4 *r = slots + 3 * (size_t)s;
    if (p < S.n_tri) {
        int k = 0;
        while (k + 1 < S.n_tri_sets && (int64_t)p >= S.tri_sets[k + 1].prim_base) k++;
        const DevTriSet &T = S.tri_sets[k];
        const int32_t *ix = T.indices + 3 * ((int64_t)p - T.prim_base);
        const float *V = T.vertices;
        r[0] = make_float4(V[3 * ix[0]], V[3 * ix[0] + 1], V[3 * ix[0] + 2], __uint_as_float(p));
        r[1] = make_float4(V[3 * ix[1]], V[3 * ix[1] + 1], V[3 * ix[1] + 2], 0.0f);
        r[2] = make_float4(V[3 * ix[2]], V[3 * ix[2] + 1], V[3 * ix[2] + 2], 0.0f);
    } else if ((int64_t)p < S.n_tri + S.n_sph) {
        int k = 0;
        while (k + 1 < S.n_sph_sets && (int64_t)p >= S.sph_sets[k + 1].prim_base) k++;
        const DevSphSet &P = S.sph_sets[k];
        int64_t lp = (int64_t)p - P.prim_base;
        r[0] = make_float4(P.centers[3 * lp], P.centers[3 * lp + 1], P.centers[3 * lp + 2],
                           __uint_as_float(p | kSphereBit));
        r[1] = make_float4(sph_radius[(int64_t)p - S.n_tri], P.eps, 0.0f, 0.0f);
        r[2] = make_float4(0, 0, 0, 0);
    } else {
        int k = 0;
        while (k + 1 < S.n_line_sets && (int64_t)p >= S.line_sets[k + 1].prim_base) k++;
        const DevLineSet &L = S.line_sets[k];
        const int idx = L.indices[(int64_t)p - L.prim_base];
        const float *a = L.vertices + 3 * idx, *b = a + 3;
        r[0] = make_float4(a[0], a[1], a[2], __uint_as_float(p | kSphereBit | kLineBit));
        r[1] = make_float4(b[0], b[1], b[2], L.radius0);
        r[2] = make_float4(0, 0, 0, 0);
    }
}

// Cost-optimal collapse (GXY_TUNE_BVH_COLLAPSE 1, single-primitive leaves):
// choose which binary nodes become wide nodes so that the summed surface
// area of the wide nodes -- proportional to the expected number of node
// visits of a ray -- is smallest while no wide node has more than 8
// children, by a dynamic programme over the binary tree, bottom up as the
// refit runs.  For binary node n and j = 1..8 child slots of its parent:
//   D(n, j) = min over k of C(left, k) + C(right, j - k)   (n spread over j slots)
//   C(n, 1) = area(n) + D(n, 8)                            (n one slot: a wide node)
//   C(n, j) = min(C(n, j - 1), D(n, j))                    (at most j slots)
// with C = 0 for a primitive.  Per node: cost[8] = C(n, 1..8); choice[j-1]
// = the slot count j' that attains C(n, j) (1: one slot), choice[8 + j-1] =
// the split k of D(n, j).  The collapse then expands D(root, 8).
__global__ void k_collapse_cost(int n, int root, const int *left, const int *right, const int *parent,
                                const int *leaf_parent, int *flags, const float4 *nlo, const float4 *nhi,
                                float *cost, uint8_t *choice) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = leaf_parent[i];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&flags[node], 1) == 0) return;   // first arrival: sibling not ready
        __threadfence();
        float cl[8], cr[8];
        const int l = left[node], r = right[node];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            cl[j] = l >= 0 ? __ldcg(cost + 8 * (size_t)l + j) : 0.0f;
            cr[j] = r >= 0 ? __ldcg(cost + 8 * (size_t)r + j) : 0.0f;
        }
        float d[9];
        uint8_t dk[9];
        d[1] = FLT_MAX;
        dk[1] = 0;
        for (int j = 2; j <= 8; j++) {
            float best = FLT_MAX;
            int bk = 1;
            for (int k = 1; k < j; k++) {
                const float v = cl[k - 1] + cr[j - k - 1];
                if (v < best) {
                    best = v;
                    bk = k;
                }
            }
            d[j] = best;
            dk[j] = (uint8_t)bk;
        }
        float c[9];
        uint8_t cj[9];
        c[1] = half_area(nlo[node], nhi[node]) + d[8];
        cj[1] = 1;
        for (int j = 2; j <= 8; j++) {
            c[j] = c[j - 1];
            cj[j] = cj[j - 1];
            if (d[j] < c[j]) {
                c[j] = d[j];
                cj[j] = (uint8_t)j;
            }
        }
#pragma unroll
        for (int j = 1; j <= 8; j++) {
            __stcg(cost + 8 * (size_t)node + (j - 1), c[j]);
            choice[16 * (size_t)node + (j - 1)] = cj[j];
            choice[16 * (size_t)node + 8 + (j - 1)] = dk[j];
        }
        node = node == root ? -1 : parent[node];
    }
}

// One level of the collapse.  Work item: (binary ref, wide node index).
__global__ void k_collapse(DevScene S, const float *sph_radius, int n, const int2 *qin, int nq, int2 *qout,
                           unsigned int *ctr, const int *left, const int *right, const int *first, const int *last,
                           const uint32_t *ids, const float4 *plo, const float4 *phi, const float4 *nlo,
                           const float4 *nhi, BVH8Node *nodes, float4 *slots, int max_nodes, int max_slots,
                           int kLeafMax, const uint8_t *choice) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nq) return;
    int2 item = qin[w];
    int ref = item.x;
    int widx = item.y;
    int ch[8];
    int nc = 0;
    auto size_of = [&](int r) { return r >= 0 ? last[r] - first[r] + 1 : 1; };
    auto box_of = [&](int r, float4 &lo, float4 &hi) {
        if (r >= 0) { lo = nlo[r]; hi = nhi[r]; }
        else { uint32_t p = ids[~r]; lo = plo[p]; hi = phi[p]; }
    };
    if (ref >= 0 && size_of(ref) > kLeafMax && choice) {
        // cost-optimal children: expand D(ref, 8) by the stored choices
        int2 stk[24];   // (binary ref, slots << 1 | spread-over-slots)
        int sp = 0;
        stk[sp++] = make_int2(ref, (8 << 1) | 1);
        while (sp > 0 && nc < 8) {
            const int2 e = stk[--sp];
            const int m = e.x, j = e.y >> 1;
            if (e.y & 1) {   // D(m, j): left gets k slots, right j - k
                const int k = choice[16 * (size_t)m + 8 + (j - 1)];
                if (sp + 2 > 24) break;
                stk[sp++] = make_int2(right[m], (j - k) << 1);
                stk[sp++] = make_int2(left[m], k << 1);
            } else if (m < 0) {
                ch[nc++] = m;                                       // a primitive
            } else {
                const int jj = choice[16 * (size_t)m + (j - 1)];
                if (jj == 1) ch[nc++] = m;                          // a wide node of its own
                else stk[sp++] = make_int2(m, (jj << 1) | 1);
            }
        }
    } else if (ref >= 0 && size_of(ref) > kLeafMax) {
        ch[nc++] = left[ref];
        ch[nc++] = right[ref];
        while (nc < 8) {
            int best = -1;
            float ba = -1.0f;
            for (int k = 0; k < nc; k++) {
                if (ch[k] >= 0 && size_of(ch[k]) > kLeafMax) {
                    float4 lo, hi;
                    box_of(ch[k], lo, hi);
                    float a = half_area(lo, hi);
                    if (a > ba) { ba = a; best = k; }
                }
            }
            if (best < 0) break;
            int r = ch[best];
            ch[best] = left[r];
            ch[nc++] = right[r];
        }
    } else {
        ch[nc++] = ref;   // whole (small) tree as one leaf: only for a small root
    }
    // inner children first (stable), so an inner child's rank among the
    // node's inner children is its slot: the traversal finds it at
    // child_base + slot without reading the meta byte
    {
        int tmp[8], m = 0;
        for (int k = 0; k < nc; k++)
            if (ch[k] >= 0 && size_of(ch[k]) > kLeafMax) tmp[m++] = ch[k];
        for (int k = 0; k < nc; k++)
            if (!(ch[k] >= 0 && size_of(ch[k]) > kLeafMax)) tmp[m++] = ch[k];
        for (int k = 0; k < nc; k++) ch[k] = tmp[k];
    }
    int n_int = 0, n_prims = 0;
    for (int k = 0; k < nc; k++) {
        if (ch[k] >= 0 && size_of(ch[k]) > kLeafMax) n_int++;
        else n_prims += size_of(ch[k]);
    }
    unsigned int cbase = n_int ? atomicAdd(&ctr[0], (unsigned)n_int) : 0u;
    unsigned int pbase = n_prims ? atomicAdd(&ctr[1], (unsigned)n_prims) : 0u;
    if ((int)(cbase + n_int) > max_nodes || (int)(pbase + n_prims) > max_slots) {
        atomicExch(&ctr[3], 1u);
        return;
    }
    float4 lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0), hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0);
    float4 clo[8], chi[8];
    for (int k = 0; k < nc; k++) {
        box_of(ch[k], clo[k], chi[k]);
        lo = make_float4(fminf(lo.x, clo[k].x), fminf(lo.y, clo[k].y), fminf(lo.z, clo[k].z), 0);
        hi = make_float4(fmaxf(hi.x, chi[k].x), fmaxf(hi.y, chi[k].y), fmaxf(hi.z, chi[k].z), 0);
    }
    BVH8Node nd;
    nd.ox = lo.x; nd.oy = lo.y; nd.oz = lo.z;
    nd.child_base = cbase;
    nd.prim_base = pbase;
    nd.ex = quant_exp(hi.x - lo.x);
    nd.ey = quant_exp(hi.y - lo.y);
    nd.ez = quant_exp(hi.z - lo.z);
    float sc[3] = {__uint_as_float((uint32_t)nd.ex << 23), __uint_as_float((uint32_t)nd.ey << 23),
                   __uint_as_float((uint32_t)nd.ez << 23)};
    float org[3] = {lo.x, lo.y, lo.z};
    nd.imask = 0;
    int irank = 0, poff = 0;
    for (int k = 0; k < 8; k++) {
        nd.meta[k] = 0xff;
        for (int a = 0; a < 3; a++) { nd.qlo[a][k] = 0; nd.qhi[a][k] = 0; }
    }
    for (int k = 0; k < nc; k++) {
        float cl[3] = {clo[k].x, clo[k].y, clo[k].z}, chh[3] = {chi[k].x, chi[k].y, chi[k].z};
        for (int a = 0; a < 3; a++) {
            float ql = floorf((cl[a] - org[a]) / sc[a]) - 1.0f;
            float qh = ceilf((chh[a] - org[a]) / sc[a]) + 1.0f;
            nd.qlo[a][k] = (uint16_t)fminf(fmaxf(ql, 0.0f), 65535.0f);
            nd.qhi[a][k] = (uint16_t)fminf(fmaxf(qh, 0.0f), 65535.0f);
        }
        int r = ch[k];
        if (r >= 0 && size_of(r) > kLeafMax) {
            nd.imask |= (uint8_t)(1u << k);
            nd.meta[k] = (uint8_t)irank;
            unsigned int qi = atomicAdd(&ctr[2], 1u);
            qout[qi] = make_int2(r, (int)(cbase + irank));
            irank++;
        } else {
            int f = r >= 0 ? first[r] : ~r;
            int cnt = size_of(r);
            // (cnt <= 4 and poff < 32 keep a filled slot's byte below 0x80;
            // the traversal reads bit 7 of the meta bytes as "empty slot")
            nd.meta[k] = (uint8_t)(((cnt - 1) << 5) | poff);
            for (int j = 0; j < cnt; j++) write_slot(S, sph_radius, ids[f + j], slots, pbase + poff + j);
            poff += cnt;
        }
    }
    nodes[widx] = nd;
}

static inline unsigned blocks_for(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// Build the BVH8 for the geometry described by S (S.nodes/S.slots are set
// on success).  sph_radius: per-sphere radius (device).
// Binned-SAH build over the clusters on the device (box lo/hi, primitive
// count in lo.w): top down, one level of split tasks per launch, one block
// per task.  Per task: the box and the centroid bounds of its clusters; 32
// centroid bins on each axis; cost area(L)*prims(L) + area(R)*prims(R) at
// every bin boundary, the cheapest kept (the first of equals, axes x, y, z);
// a stable partition at that boundary (by position when every centroid
// coincides).  A segment of one cluster becomes a child ref (refs[k]); a
// longer one a new top node (binary node base + id) and a task of the next
// level.  A top node's size is stated as at least 5 primitives so that the
// collapse, which decides leaves by size (at most 4 primitives per leaf),
// always opens it.
struct SahTask {
    int node, begin, end;
};
constexpr int kSahBins = 32;

__device__ __forceinline__ float sah_area(float lx, float ly, float lz, float hx, float hy, float hz) {
    float x = hx - lx, y = hy - ly, z = hz - lz;
    return x * y + y * z + z * x;
}
__device__ __forceinline__ float sah_cen(const float4 &lo, const float4 &hi, int a) {
    const float l = a == 0 ? lo.x : a == 1 ? lo.y : lo.z, h = a == 0 ? hi.x : a == 1 ? hi.y : hi.z;
    return 0.5f * (l + h);
}
__device__ __forceinline__ int sah_bin(float c, float cmin, float ext) {
    return min(kSahBins - 1, (int)((c - cmin) / ext * kSahBins));
}

__global__ void __launch_bounds__(256) k_sah_level(const float4 *clo, const float4 *chi, const int *refs,
                                                   const int *idx_in, int *idx_out, const SahTask *tin,
                                                   const unsigned *n_in, SahTask *tout, unsigned *n_out,
                                                   unsigned *node_ctr, int base, int *left, int *right, int *first,
                                                   int *last, float4 *nlo, float4 *nhi) {
    __shared__ unsigned s_lo[3], s_hi[3], s_cmin[3], s_cmax[3];
    __shared__ int s_count;
    __shared__ unsigned s_blo[3][kSahBins][3], s_bhi[3][kSahBins][3];
    __shared__ int s_bn[3][kSahBins], s_bc[3][kSahBins];
    __shared__ int s_axis, s_bin, s_nleft, s_warp[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned ntask = *n_in;
    for (unsigned t = blockIdx.x; t < ntask; t += gridDim.x) {
        const SahTask T = tin[t];
        // 1. node box, centroid bounds, primitive count
        if (tid < 3) {
            s_lo[tid] = s_cmin[tid] = 0xffffffffu;
            s_hi[tid] = s_cmax[tid] = 0u;
        }
        if (tid == 0) s_count = 0;
        for (int i = tid; i < 3 * kSahBins * 3; i += blockDim.x) {
            (&s_blo[0][0][0])[i] = 0xffffffffu;
            (&s_bhi[0][0][0])[i] = 0u;
        }
        for (int i = tid; i < 3 * kSahBins; i += blockDim.x) {
            (&s_bn[0][0])[i] = 0;
            (&s_bc[0][0])[i] = 0;
        }
        __syncthreads();
        for (int i0 = T.begin; i0 < T.end; i0 += blockDim.x) {
            const int i = i0 + tid;
            const bool ok = i < T.end;
            float4 lo = make_float4(0, 0, 0, 0), hi = lo;
            if (ok) {
                const int k = idx_in[i];
                lo = clo[k];
                hi = chi[k];
            }
            const float l3[3] = {lo.x, lo.y, lo.z}, h3[3] = {hi.x, hi.y, hi.z};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float c = 0.5f * (l3[a] + h3[a]);
                const unsigned vl = __reduce_min_sync(0xffffffffu, ok ? f2o(l3[a]) : 0xffffffffu);
                const unsigned vh = __reduce_max_sync(0xffffffffu, ok ? f2o(h3[a]) : 0u);
                const unsigned cl = __reduce_min_sync(0xffffffffu, ok ? f2o(c) : 0xffffffffu);
                const unsigned ch = __reduce_max_sync(0xffffffffu, ok ? f2o(c) : 0u);
                if (lane == 0) {
                    atomicMin(&s_lo[a], vl);
                    atomicMax(&s_hi[a], vh);
                    atomicMin(&s_cmin[a], cl);
                    atomicMax(&s_cmax[a], ch);
                }
            }
            const int cnt = __reduce_add_sync(0xffffffffu, ok ? __float_as_int(lo.w) : 0);
            if (lane == 0) atomicAdd(&s_count, cnt);
        }
        __syncthreads();
        float cmin[3], ext[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            cmin[a] = o2f(s_cmin[a]);
            ext[a] = o2f(s_cmax[a]) - cmin[a];
        }
        // 2. bins on every axis with a centroid extent
        for (int i = T.begin + tid; i < T.end; i += blockDim.x) {
            const int k = idx_in[i];
            const float4 lo = clo[k], hi = chi[k];
            const float l3[3] = {lo.x, lo.y, lo.z}, h3[3] = {hi.x, hi.y, hi.z};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (!(ext[a] > 0.f)) continue;
                const int b = sah_bin(sah_cen(lo, hi, a), cmin[a], ext[a]);
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    atomicMin(&s_blo[a][b][q], f2o(l3[q]));
                    atomicMax(&s_bhi[a][b][q], f2o(h3[q]));
                }
                atomicAdd(&s_bn[a][b], __float_as_int(lo.w));
                atomicAdd(&s_bc[a][b], 1);
            }
        }
        __syncthreads();
        // 3. the cheapest bin boundary (as the sweep from both ends)
        if (tid == 0) {
            float best = FLT_MAX;
            int best_axis = -1, best_bin = 0, best_left = 0;
            for (int a = 0; a < 3; a++) {
                if (!(ext[a] > 0.f)) continue;
                float lcost[kSahBins];
                int litems[kSahBins];
                float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                int ln = 0, lc = 0;
                for (int b = 0; b < kSahBins; b++) {
                    for (int q = 0; q < 3; q++) {
                        if (s_bc[a][b]) {
                            llo[q] = fminf(llo[q], o2f(s_blo[a][b][q]));
                            lhi[q] = fmaxf(lhi[q], o2f(s_bhi[a][b][q]));
                        }
                    }
                    ln += s_bn[a][b];
                    lc += s_bc[a][b];
                    litems[b] = lc;
                    lcost[b] = lc ? sah_area(llo[0], llo[1], llo[2], lhi[0], lhi[1], lhi[2]) * ln : 0.f;
                }
                float rlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                int rn = 0;
                for (int b = kSahBins - 1; b >= 1; b--) {
                    for (int q = 0; q < 3; q++) {
                        if (s_bc[a][b]) {
                            rlo[q] = fminf(rlo[q], o2f(s_blo[a][b][q]));
                            rhi[q] = fmaxf(rhi[q], o2f(s_bhi[a][b][q]));
                        }
                    }
                    rn += s_bn[a][b];
                    const int left_items = litems[b - 1];
                    if (left_items == 0 || left_items == T.end - T.begin) continue;
                    const float cost = lcost[b - 1] + sah_area(rlo[0], rlo[1], rlo[2], rhi[0], rhi[1], rhi[2]) * rn;
                    if (cost < best) {
                        best = cost;
                        best_axis = a;
                        best_bin = b - 1;
                        best_left = left_items;
                    }
                }
            }
            s_axis = best_axis;
            s_bin = best_bin;
            s_nleft = best_axis < 0 ? (T.end - T.begin) / 2 : best_left;
        }
        __syncthreads();
        const int axis = s_axis, bbin = s_bin, nleft = s_nleft;
        // 4. stable partition into idx_out (order kept on each side)
        int lbase = 0, rbase = 0;
        for (int i0 = T.begin; i0 < T.end; i0 += blockDim.x) {
            const int i = i0 + tid;
            const bool ok = i < T.end;
            int k = 0;
            bool is_left = false;
            if (ok) {
                k = idx_in[i];
                is_left = axis < 0 ? (i - T.begin) < nleft
                                   : sah_bin(sah_cen(clo[k], chi[k], axis), cmin[axis], ext[axis]) <= bbin;
            }
            const unsigned bl = __ballot_sync(0xffffffffu, ok && is_left);
            const unsigned br = __ballot_sync(0xffffffffu, ok && !is_left);
            if (lane == 0) s_warp[warp] = (int)(__popc(bl) | (__popc(br) << 16));
            __syncthreads();
            int lo_l = 0, lo_r = 0, tot_l = 0, tot_r = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
                const int v = s_warp[w];
                if (w < warp) {
                    lo_l += v & 0xffff;
                    lo_r += v >> 16;
                }
                tot_l += v & 0xffff;
                tot_r += v >> 16;
            }
            const unsigned lt = (1u << lane) - 1u;
            if (ok) {
                const int pos = is_left ? T.begin + lbase + lo_l + __popc(bl & lt)
                                        : T.begin + nleft + rbase + lo_r + __popc(br & lt);
                idx_out[pos] = k;
            }
            lbase += tot_l;
            rbase += tot_r;
            __syncthreads();
        }
        // 5. the node and its children
        if (tid == 0) {
            const int node = base + T.node;
            nlo[node] = make_float4(o2f(s_lo[0]), o2f(s_lo[1]), o2f(s_lo[2]), 0.f);
            nhi[node] = make_float4(o2f(s_hi[0]), o2f(s_hi[1]), o2f(s_hi[2]), 0.f);
            first[node] = 0;
            last[node] = max(s_count, 5) - 1;   // stated size >= 5: never a leaf
            const int rb[2] = {T.begin, T.begin + nleft}, re[2] = {T.begin + nleft, T.end};
            int child[2];
            for (int c = 0; c < 2; c++) {
                if (re[c] - rb[c] == 1) {
                    child[c] = refs[idx_out[rb[c]]];
                } else {
                    const int id = (int)atomicAdd(node_ctr, 1u);
                    tout[atomicAdd(n_out, 1u)] = SahTask{id, rb[c], re[c]};
                    child[c] = base + id;
                }
            }
            left[node] = child[0];
            right[node] = child[1];
        }
        __syncthreads();
    }
}

// Parents of the binned-SAH top tree's children (top nodes base .. base +
// ntop - 1), so that bottom-up passes climb from the clusters into it.
__global__ void k_top_parents(int ntop, int base, const int *left, const int *right, int *parent,
                              int *leaf_parent) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntop) return;
    const int node = base + t;
    const int c[2] = {left[node], right[node]};
    for (int k = 0; k < 2; k++) {
        if (c[k] >= 0) parent[c[k]] = node;
        else leaf_parent[~c[k]] = node;
    }
}

__global__ void k_iota(int m, int *idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) idx[i] = i;
}

int build_bvh8(DevScene &S, const float *sph_radius, DeviceArena &arena, cudaStream_t st, BVHInfo &info) {
    auto t_start = std::chrono::steady_clock::now();
    int64_t n64 = S.n_tri + S.n_sph + S.n_seg;
    info = BVHInfo{};
    if (n64 == 0) {
        S.nodes = nullptr;
        S.slots = nullptr;
        return GXY_OK;
    }
    // leaf-slot ids carry kind bits 30 and 31
    if (n64 >= ((int64_t)1 << 30)) return set_error(GXY_ERR_INVALID, "more than 2^30 primitives for the BVH");
    int n = (int)n64;
    BuildBuffers B;
    ScratchList scratch(arena);
    int rc = GXY_OK;
#define ALLOC(p, cnt)                                                                        \
    do {                                                                                     \
        rc = scratch.alloc((void **)&(p), sizeof(*(p)) * (size_t)(cnt));                    \
        if (rc) return rc;                                                                   \
    } while (0)
    ALLOC(B.plo, n); ALLOC(B.phi, n);
    ALLOC(B.keys, n); ALLOC(B.keys2, n); ALLOC(B.ids, n); ALLOC(B.ids2, n);
    int ni = n > 1 ? n - 1 : 1;
    const int C = sah_builder() ? sah_cluster_size() : 0;   // top-level SAH over clusters of <= C primitives
    const int ncap = (C > 1 && n > C) ? 2 * ni : ni;       // room for the top tree's nodes after the radix tree's
    ALLOC(B.left, ncap); ALLOC(B.right, ncap); ALLOC(B.parent, ncap); ALLOC(B.first, ncap); ALLOC(B.last, ncap);
    ALLOC(B.flags, ncap); ALLOC(B.nlo, ncap); ALLOC(B.nhi, ncap);
    int *leaf_parent;
    ALLOC(leaf_parent, n);
    ALLOC(B.ctr, 8);
    ALLOC(B.cbounds, 8);
    // worst-case wide nodes: every wide node has >= 2 children
    int max_nodes = n + 1;
    int max_slots = n;
    ALLOC(B.qa, max_nodes); ALLOC(B.qb, max_nodes);
    unsigned int hb[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0, 0, 0, 0, 0};
    CK(cudaMemcpyAsync(B.cbounds, hb, sizeof hb, cudaMemcpyHostToDevice, st));
    k_prim_bounds<<<blocks_for(n, 256), 256, 0, st>>>(S, sph_radius, n, B.plo, B.phi, B.cbounds);
    k_morton<<<blocks_for(n, 256), 256, 0, st>>>(n, B.plo, B.phi, B.cbounds, B.keys, B.ids);
    CK(cudaGetLastError());
    size_t tmp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, B.keys, B.keys2, B.ids, B.ids2, n, 0, 63, st);
    unsigned char *tmp;
    ALLOC(tmp, tmp_bytes);
    CK(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, B.keys, B.keys2, B.ids, B.ids2, n, 0, 63, st));
    int root_ref = n > 1 ? 0 : ~0;
    if (n > 1) {
        CK(cudaMemsetAsync(B.flags, 0, sizeof(int) * ni, st));
        k_karras<<<blocks_for(n - 1, 256), 256, 0, st>>>(n, B.keys2, B.left, B.right, B.parent, B.first, B.last,
                                                         leaf_parent);
        k_refit<<<blocks_for(n, 256), 256, 0, st>>>(n, B.ids2, B.plo, B.phi, B.left, B.right, B.parent, leaf_parent,
                                                    B.flags, B.nlo, B.nhi);
        CK(cudaGetLastError());
    }
    if (C > 1 && n > C) {
        int *refs;
        float4 *clo, *chi;
        ALLOC(refs, n); ALLOC(clo, n); ALLOC(chi, n);
        CK(cudaMemsetAsync(B.ctr + 6, 0, sizeof(unsigned int), st));
        k_clusters<<<blocks_for(n, 256), 256, 0, st>>>(n, C, B.parent, leaf_parent, B.first, B.last, refs, B.ctr + 6);
        unsigned int m = 0;
        CK(cudaMemcpyAsync(&m, B.ctr + 6, sizeof m, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (m >= 2 && m <= (unsigned)n) {
            k_cluster_info<<<blocks_for(m, 256), 256, 0, st>>>((int)m, refs, B.ids2, B.plo, B.phi, B.first, B.last,
                                                               B.nlo, B.nhi, clo, chi);
            CK(cudaGetLastError());
            // the top tree on the device, level by level; the host reads the
            // number of open tasks once per 16 levels
            int *idxa, *idxb;
            SahTask *ta, *tb;
            unsigned *tctr;   // [0], [1] task counts (ping-pong), [2] top nodes
            ALLOC(idxa, m); ALLOC(idxb, m); ALLOC(ta, m); ALLOC(tb, m); ALLOC(tctr, 4);
            k_iota<<<blocks_for(m, 256), 256, 0, st>>>((int)m, idxa);
            const SahTask root_task{0, 0, (int)m};
            const unsigned c0[4] = {1u, 0u, 1u, 0u};
            CK(cudaMemcpyAsync(ta, &root_task, sizeof root_task, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(tctr, c0, sizeof c0, cudaMemcpyHostToDevice, st));
            const int base = ni;
            int cur = 0;
            for (int lvl = 0;; lvl += 16) {
                for (int k = 0; k < 16; k++) {
                    CK(cudaMemsetAsync(tctr + (cur ^ 1), 0, sizeof(unsigned), st));
                    k_sah_level<<<1024, 256, 0, st>>>(clo, chi, refs, cur ? idxb : idxa, cur ? idxa : idxb,
                                                      cur ? tb : ta, tctr + cur, cur ? ta : tb, tctr + (cur ^ 1),
                                                      tctr + 2, base, B.left, B.right, B.first, B.last, B.nlo,
                                                      B.nhi);
                    cur ^= 1;
                }
                CK(cudaGetLastError());
                unsigned open = 0;
                CK(cudaMemcpyAsync(&open, tctr + cur, sizeof open, cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                if (!open) break;
                if (lvl > (int)m) return set_error(GXY_ERR_INVALID, "SAH top build did not converge");
            }
            root_ref = base;
            info.sah_levels = (int)m;   // clusters under the SAH top tree
            // the top tree's m - 1 nodes as parents of their children
            k_top_parents<<<blocks_for(m - 1, 256), 256, 0, st>>>((int)m - 1, base, B.left, B.right, B.parent,
                                                                  leaf_parent);
            CK(cudaGetLastError());
        }
    }
    uint8_t *choice = nullptr;   // cost-optimal collapse: per binary node, the programme's choices
    if (collapse_cost() && leaf_max() == 1 && root_ref >= 0 && n > 1) {
        float *cost;
        ALLOC(cost, 8 * (size_t)ncap);
        ALLOC(choice, 16 * (size_t)ncap);
        CK(cudaMemsetAsync(B.flags, 0, sizeof(int) * ncap, st));
        k_collapse_cost<<<blocks_for(n, 256), 256, 0, st>>>(n, root_ref, B.left, B.right, B.parent, leaf_parent,
                                                            B.flags, B.nlo, B.nhi, cost, choice);
        CK(cudaGetLastError());
    }
    BVH8Node *nodes;
    float4 *slots;
    rc = arena.alloc((void **)&nodes, sizeof(BVH8Node) * (size_t)max_nodes);
    if (rc) return rc;
    rc = arena.alloc((void **)&slots, sizeof(float4) * 3 * (size_t)max_slots);
    if (rc) { arena.free(nodes); return rc; }
    // root: wide node 0 from the binary root (radix-tree root 0, the SAH top
    // tree's root, or the single leaf)
    int2 root = make_int2(root_ref, 0);
    unsigned int c0[8] = {1, 0, 0, 0, 0, 0, 0, 0};
    CK(cudaMemcpyAsync(B.ctr, c0, sizeof c0, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B.qa, &root, sizeof root, cudaMemcpyHostToDevice, st));
    int nq = 1;
    int levels = 0;
    while (nq > 0) {
        CK(cudaMemsetAsync(B.ctr + 2, 0, sizeof(unsigned int), st));
        k_collapse<<<blocks_for(nq, 128), 128, 0, st>>>(S, sph_radius, n, B.qa, nq, B.qb, B.ctr, B.left, B.right,
                                                        B.first, B.last, B.ids2, B.plo, B.phi, B.nlo, B.nhi, nodes,
                                                        slots, max_nodes, max_slots, leaf_max(), choice);
        CK(cudaGetLastError());
        unsigned int hc[4];
        CK(cudaMemcpyAsync(hc, B.ctr, sizeof hc, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hc[3]) {
            arena.free(nodes);
            arena.free(slots);
            return set_error(GXY_ERR_OVERFLOW, "BVH8 collapse exceeded its node budget");
        }
        nq = (int)hc[2];
        std::swap(B.qa, B.qb);
        levels++;
        info.n_nodes = hc[0];
        info.n_slots = hc[1];
        if (levels > 200) return set_error(GXY_ERR_INVALID, "BVH8 collapse did not converge");
    }
    S.nodes = nodes;
    S.slots = slots;
    info.levels = levels;
    info.nodes_ptr = nodes;
    info.slots_ptr = slots;
    info.build_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    return GXY_OK;
#undef ALLOC
}

}  // namespace gxy

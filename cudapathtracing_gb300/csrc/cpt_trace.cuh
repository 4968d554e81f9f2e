// cpt_trace.cuh — closest-hit traversal of the BVH2 layout and primitive intersection in
// FP32 (traverseIterative BVH.cuh:282-332, Hittable::hit Hittable.cuh:487-503).
//
// The traversal returns the closest hit like the reference but orders children near-first
// and prunes boxes beyond the closest hit so far (the reference tests every box the ray
// line crosses).  Leaves are tested as soon as their box is hit, with [0.001, closest], as
// in the reference; only exact ties may resolve to a different primitive.
#pragma once

#include "cpt_device.cuh"

namespace cpt {

struct Hit {
    float t, u, v;
    int leaf;   // sorted leaf index, -1 on a miss
};

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// Möller–Trumbore exactly as Triangle::hit (Hittable.cuh:85-111): eps 1e-8 on the
// determinant, inclusive u, v, u+v and t bounds.
__device__ __forceinline__ bool hit_triangle(float3 o, float3 d, float3 p0, float3 e1, float3 e2, float tmin,
                                             float tmax, float& t, float& u, float& v)
{
    float3 h = cross3(d, e2);
    float a = dot3(e1, h);
    if (fabsf(a) < 1e-8f) return false;
    float f = 1.0f / a;
    float3 s = o - p0;
    u = f * dot3(s, h);
    if (u < 0.0f || u > 1.0f) return false;
    float3 q = cross3(s, e1);
    v = f * dot3(d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    t = f * dot3(e2, q);
    return !(t < tmin || t > tmax);
}

// Sphere::hit (Hittable.cuh:27-44).
__device__ __forceinline__ bool hit_sphere(float3 o, float3 d, float3 c, float r, float tmin, float tmax, float& t)
{
    float3 oc = o - c;
    float a = dot3(d, d);
    float b = dot3(d, oc);
    float cc = dot3(oc, oc) - r * r;
    float disc = b * b - a * cc;
    if (disc < 0.0f) return false;
    float sq = sqrtf(disc);
    t = (-b - sq) / a;
    if (t < tmin || t > tmax) t = (-b + sq) / a;
    return !(t < tmin || t > tmax);
}

// Light::hit (Hittable.cuh:367-398): one-sided rectangle, only when visible.
__device__ __forceinline__ bool hit_light(const DevLight& L, float3 o, float3 d, float tmin, float tmax, float& t)
{
    if (!L.visible) return false;
    float denom = dot3(d, L.normal);
    if (fabsf(denom) < 1e-6f || denom > 0.0f) return false;
    t = dot3(L.center - o, L.normal) / denom;
    if (t < tmin || t > tmax) return false;
    float3 hp = o + t * d;
    float3 diff = hp - L.center;
    float u = dot3(diff, L.eu), v = dot3(diff, L.ev);
    return fabsf(u) <= L.w / 2.0f && fabsf(v) <= L.h / 2.0f;
}

__device__ __forceinline__ bool hit_leaf(const SceneView& s, int k, float3 o, float3 d, float tmax, float& t, float& u,
                                         float& v)
{
    const float4* r = s.leaf_rec + 3 * (size_t)k;
    float4 r0 = ldg4(r), r1 = ldg4(r + 1);
    int kind = __float_as_int(r1.w);
    if (kind == CPT_KIND_TRI) {
        float4 r2 = ldg4(r + 2);
        return hit_triangle(o, d, f3(r0.x, r0.y, r0.z), f3(r1.x, r1.y, r1.z), f3(r2.x, r2.y, r2.z), 0.001f, tmax, t, u,
                            v);
    }
    u = v = 0.f;
    if (kind == CPT_KIND_SPHERE) return hit_sphere(o, d, f3(r0.x, r0.y, r0.z), r1.x, 0.001f, tmax, t);
    return hit_light(s.lights[__float_as_int(r1.x)], o, d, 0.001f, tmax, t);
}

// Occlusion test of leaf k for a shadow ray aimed at light `skip`: any primitive hit in
// [0.001, tmax] occludes, except that light itself.
__device__ __forceinline__ bool occludes_leaf(const SceneView& s, int k, float3 o, float3 d, float tmax, int skip)
{
    const float4* r = s.leaf_rec + 3 * (size_t)k;
    float4 r0 = ldg4(r), r1 = ldg4(r + 1);
    int kind = __float_as_int(r1.w);
    float t, u, v;
    if (kind == CPT_KIND_TRI) {
        float4 r2 = ldg4(r + 2);
        return hit_triangle(o, d, f3(r0.x, r0.y, r0.z), f3(r1.x, r1.y, r1.z), f3(r2.x, r2.y, r2.z), 0.001f, tmax, t, u,
                            v);
    }
    if (kind == CPT_KIND_SPHERE) return hit_sphere(o, d, f3(r0.x, r0.y, r0.z), r1.x, 0.001f, tmax, t);
    int li = __float_as_int(r1.x);
    return li != skip && hit_light(s.lights[li], o, d, 0.001f, tmax, t);
}

// One leaf reached by a traversal.  Closest-hit queries (ANY false) keep the nearest hit in
// [0.001, best]; occlusion queries (ANY true) return true at the first occluder.
template <bool ANY>
__device__ __forceinline__ bool visit_leaf(const SceneView& s, int leaf, float3 o, float3 d, float& best, Hit& hit,
                                           int skip)
{
    if (ANY) {
        if (!occludes_leaf(s, leaf, o, d, best, skip)) return false;
        hit.leaf = leaf;
        return true;
    }
    float t, u, v;
    if (hit_leaf(s, leaf, o, d, best, t, u, v)) {
        best = t; hit.t = t; hit.u = u; hit.v = v; hit.leaf = leaf;
    }
    return false;
}

// Inverse direction for slab tests.  A zero component (an axis-parallel ray, e.g. a cosine
// sample with r1 = 1 from a floor) would make 1/d infinite and turn slab distances into NaN,
// which the min/max chain then drops: boxes are wrongly accepted or rejected.  Components
// below 1e-20 in magnitude are replaced by +-1e-20 (the limit of a nearly parallel ray); the
// primitive tests keep the exact direction.
__device__ __forceinline__ float3 safe_inverse(float3 d)
{
    const float e = 1e-20f;
    float x = fabsf(d.x) < e ? copysignf(e, d.x) : d.x;
    float y = fabsf(d.y) < e ? copysignf(e, d.y) : d.y;
    float z = fabsf(d.z) < e ? copysignf(e, d.z) : d.z;
    return f3(1.0f / x, 1.0f / y, 1.0f / z);
}

__device__ __forceinline__ uint32_t word_of(const float4& f, int w)
{
    return __float_as_uint(w == 0 ? f.x : (w == 1 ? f.y : (w == 2 ? f.z : f.w)));
}

// Closest hit through the compressed 8-wide BVH (layout in wide.cu).  A visit decodes the 8
// 8-bit quantised child boxes and tests them; hit children are recorded in a byte mask at bit
// positions slot ^ (7 ^ octant), which orders them roughly front to back for this ray (the slots
// were assigned by direction at build time).  Leaf children are tested at once, nearest bit
// first (the reference tests leaves as it reaches them); the traversal continues with the first
// internal child and keeps the rest as one node-group entry (node, remaining hit bits) on the
// stack, as in compressed wide BVH traversal (Ylitie et al. 2017); a popped group yields its next
// child from the node's child list.  Boxes are tested against the closest hit so far, so far
// subtrees are culled.  With ANY the walk is an occlusion query (visit_leaf) that stops at the
// first occluder.  The walk advances one node per step() so that a warp can refill finished lanes
// (dynamic fetching); Stack64 keeps group entries (in shared and local memory, or local only).
template <bool ANY, typename Stack64>
struct WideWalk {
    float3 o, d, idir;
    float tmin, best;
    uint32_t first, node;
    int sp, skip;
    Hit hit;
    Stack64 stack;

    __device__ __forceinline__ void start(float3 o_, float3 d_, float tmin_, float tmax_, int skip_)
    {
        o = o_;
        d = d_;
        idir = safe_inverse(d_);
        first = 7u ^ ((d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u));
        tmin = tmin_;
        best = tmax_;
        node = 0;
        sp = 0;
        skip = skip_;
        hit.leaf = -1;
        hit.t = tmax_;
        hit.u = hit.v = 0.f;
    }

    // Visits one node; returns true when the traversal has finished.
    __device__ __forceinline__ bool step(const SceneView& s, int* err)
    {
        const float4* np = s.wide + CPT_WIDE_F4 * (size_t)node;
        const float4 f0 = ldg4(np), f1 = ldg4(np + 1), f2 = ldg4(np + 2);
        const float4 qx = ldg4(np + 3), qy = ldg4(np + 4), qz = ldg4(np + 5);
        const uint32_t e = __float_as_uint(f0.w);
        const float ax = __uint_as_float((e & 0xFFu) << 23) * idir.x;
        const float ay = __uint_as_float(((e >> 8) & 0xFFu) << 23) * idir.y;
        const float az = __uint_as_float(((e >> 16) & 0xFFu) << 23) * idir.z;
        const float bx = (f0.x - o.x) * idir.x, by = (f0.y - o.y) * idir.y, bz = (f0.z - o.z) * idir.z;
        uint32_t ihits = 0, lhits = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int ref = (int)(i < 4 ? word_of(f1, i & 3) : word_of(f2, i & 3));
            if (ref == CPT_WIDE_EMPTY) continue;
            const int lo = i >> 2, sh = (i & 3) * 8;
            const float lx = (float)((word_of(qx, lo) >> sh) & 0xFFu), hx = (float)((word_of(qx, 2 + lo) >> sh) & 0xFFu);
            const float ly = (float)((word_of(qy, lo) >> sh) & 0xFFu), hy = (float)((word_of(qy, 2 + lo) >> sh) & 0xFFu);
            const float lz = (float)((word_of(qz, lo) >> sh) & 0xFFu), hz = (float)((word_of(qz, 2 + lo) >> sh) & 0xFFu);
            const float x0 = fmaf(lx, ax, bx), x1 = fmaf(hx, ax, bx);
            const float y0 = fmaf(ly, ay, by), y1 = fmaf(hy, ay, by);
            const float z0 = fmaf(lz, az, bz), z1 = fmaf(hz, az, bz);
            const float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
            const float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), best));
            if (tn <= tf) {
                const uint32_t bit = 1u << ((uint32_t)i ^ first);
                if (ref >= 0) ihits |= bit;
                else lhits |= bit;
            }
        }
        while (lhits) {
            const uint32_t slot = (uint32_t)(__ffs(lhits) - 1) ^ first;
            lhits &= lhits - 1;
            const int leaf = ~(int)(slot < 4 ? word_of(f1, slot & 3) : word_of(f2, slot & 3));
            if (visit_leaf<ANY>(s, leaf, o, d, best, hit, skip)) return true;
        }
        // Continue with the first hit internal child; the others stay on the stack as one group
        // (this node, remaining hit bits) and are read back from the node when popped.
        if (ihits) {
            const uint32_t slot = (uint32_t)(__ffs(ihits) - 1) ^ first;
            const uint32_t rest = ihits & (ihits - 1);
            const uint32_t cur = node;
            node = slot < 4 ? word_of(f1, slot & 3) : word_of(f2, slot & 3);
            if (rest) {
                if (sp >= CPT_WSTACK) {
                    if (err) atomicOr(err, CPT_DEVERR_STACK);
                    return true;
                }
                stack.put(sp++, (uint64_t)cur | ((uint64_t)rest << 32));
            }
            return false;
        }
        if (sp == 0) return true;
        const uint64_t g = stack.get(--sp);
        const uint32_t gnode = (uint32_t)g;
        const uint32_t hits = (uint32_t)(g >> 32);
        const uint32_t slot = (uint32_t)(__ffs(hits) - 1) ^ first;
        const uint32_t rest = hits & (hits - 1);
        if (rest) stack.put(sp++, (uint64_t)gnode | ((uint64_t)rest << 32));
        node = (uint32_t)__ldg(reinterpret_cast<const int*>(s.wide + CPT_WIDE_F4 * (size_t)gnode + 1) + slot);
        return false;
    }
};

// Group-entry stacks of the wide traversal: the whole stack in local memory, or the bottom SHORT
// entries in the block's dynamic shared memory (wide_short_stack_bytes) and the rest in local
// memory; thread t owns the column t, t + T, ... of 64-bit words.
struct LocalStack64 {
    uint64_t s[CPT_WSTACK];
    __device__ __forceinline__ void init() {}
    __device__ __forceinline__ void put(int i, uint64_t v) { s[i] = v; }
    __device__ __forceinline__ uint64_t get(int i) const { return s[i]; }
};

template <int SHORT>
struct ShortStack64 {
    uint64_t* col;
    int stride;
    uint64_t spill[CPT_WSTACK - SHORT];
    __device__ __forceinline__ void init()
    {
        extern __shared__ int cpt_short_stack_smem[];
        const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
        col = reinterpret_cast<uint64_t*>(cpt_short_stack_smem) + t;
        stride = blockDim.x * blockDim.y * blockDim.z;
    }
    __device__ __forceinline__ void put(int i, uint64_t v)
    {
        if (i < SHORT) col[i * stride] = v;
        else spill[i - SHORT] = v;
    }
    __device__ __forceinline__ uint64_t get(int i) const { return i < SHORT ? col[i * stride] : spill[i - SHORT]; }
};

template <bool ANY>
__device__ __forceinline__ bool trace_closest_wide(const SceneView& s, float3 o, float3 d, float tmin, float tmax,
                                                   Hit& hit, int* err, int skip)
{
    WideWalk<ANY, LocalStack64> w;
    w.stack.init();
    w.start(o, d, tmin, tmax, skip);
    while (!w.step(s, err)) {}
    hit = w.hit;
    return hit.leaf >= 0;
}

// Slab distances of both children of BVH2 node `node` (t = box * idir - o * idir per axis) and
// their references, from the full 64-byte node or the compressed 32-byte one (s.node_q).
struct Bvh2Slabs {
    float ax0, ax1, ay0, ay1, az0, az1, bx0, bx1, by0, by1, bz0, bz1;
    int ca, cb;
};

__device__ __forceinline__ float u8f(uint32_t w, int k) { return (float)((w >> (8 * k)) & 0xFFu); }

__device__ __forceinline__ void bvh2_slabs(const SceneView& s, int node, float3 o, float3 idir, float3 ood,
                                           Bvh2Slabs& r)
{
    if (s.node_q) {
        const float4* np = s.nodes + 2 * (size_t)node;
        const float4 q0 = ldg4(np), q1 = ldg4(np + 1);
        const uint32_t e = __float_as_uint(q0.w);
        const float sx = __uint_as_float((e & 0xFFu) << 23) * idir.x;
        const float sy = __uint_as_float(((e >> 8) & 0xFFu) << 23) * idir.y;
        const float sz = __uint_as_float(((e >> 16) & 0xFFu) << 23) * idir.z;
        const float bx = (q0.x - o.x) * idir.x, by = (q0.y - o.y) * idir.y, bz = (q0.z - o.z) * idir.z;
        const uint32_t w0 = __float_as_uint(q1.x), w1 = __float_as_uint(q1.y), w2 = __float_as_uint(q1.z);
        const int split = __float_as_int(q1.w);
        r.ax0 = fmaf(u8f(w0, 0), sx, bx); r.ax1 = fmaf(u8f(w0, 3), sx, bx);
        r.ay0 = fmaf(u8f(w0, 1), sy, by); r.ay1 = fmaf(u8f(w1, 0), sy, by);
        r.az0 = fmaf(u8f(w0, 2), sz, bz); r.az1 = fmaf(u8f(w1, 1), sz, bz);
        r.bx0 = fmaf(u8f(w1, 2), sx, bx); r.bx1 = fmaf(u8f(w2, 1), sx, bx);
        r.by0 = fmaf(u8f(w1, 3), sy, by); r.by1 = fmaf(u8f(w2, 2), sy, by);
        r.bz0 = fmaf(u8f(w2, 0), sz, bz); r.bz1 = fmaf(u8f(w2, 3), sz, bz);
        r.ca = ((e >> 24) & 1u) ? ~split : split;
        r.cb = ((e >> 25) & 1u) ? ~(split + 1) : split + 1;
        return;
    }
    const float4* np = s.nodes + 4 * (size_t)node;
    const float4 n0 = ldg4(np), n1 = ldg4(np + 1), n2 = ldg4(np + 2), n3 = ldg4(np + 3);
    r.ax0 = fmaf(n0.x, idir.x, -ood.x); r.ax1 = fmaf(n0.y, idir.x, -ood.x);
    r.ay0 = fmaf(n0.z, idir.y, -ood.y); r.ay1 = fmaf(n0.w, idir.y, -ood.y);
    r.az0 = fmaf(n2.x, idir.z, -ood.z); r.az1 = fmaf(n2.y, idir.z, -ood.z);
    r.bx0 = fmaf(n1.x, idir.x, -ood.x); r.bx1 = fmaf(n1.y, idir.x, -ood.x);
    r.by0 = fmaf(n1.z, idir.y, -ood.y); r.by1 = fmaf(n1.w, idir.y, -ood.y);
    r.bz0 = fmaf(n2.z, idir.z, -ood.z); r.bz1 = fmaf(n2.w, idir.z, -ood.z);
    r.ca = __float_as_int(n3.x);
    r.cb = __float_as_int(n3.y);
}

// Binary-node traversal (Aila–Laine node layout): near child first, far child pushed.  The
// stack (ShortStack: shared memory, then local memory) holds at most one entry per level.  ANY as in
// trace_closest_wide.
template <bool ANY, typename Stack>
__device__ __forceinline__ bool trace_closest_bvh2(const SceneView& s, float3 o, float3 d, float tmin, float tmax,
                                                   Hit& hit, int* err, int skip)
{
    const float3 idir = safe_inverse(d);
    const float3 ood = f3(o.x * idir.x, o.y * idir.y, o.z * idir.z);
    Stack stack;
    stack.init();
    int sp = 0;
    int node = 0;
    float best = tmax;
    for (;;) {
        Bvh2Slabs r;
        bvh2_slabs(s, node, o, idir, ood, r);
        float an = fmaxf(fmaxf(fminf(r.ax0, r.ax1), fminf(r.ay0, r.ay1)), fmaxf(fminf(r.az0, r.az1), tmin));
        float af = fminf(fminf(fmaxf(r.ax0, r.ax1), fmaxf(r.ay0, r.ay1)), fminf(fmaxf(r.az0, r.az1), best));
        float bn = fmaxf(fmaxf(fminf(r.bx0, r.bx1), fminf(r.by0, r.by1)), fmaxf(fminf(r.bz0, r.bz1), tmin));
        float bf = fminf(fminf(fmaxf(r.bx0, r.bx1), fmaxf(r.by0, r.by1)), fminf(fmaxf(r.bz0, r.bz1), best));
        int ca = r.ca, cb = r.cb;
        bool ha = an <= af, hb = bn <= bf;
        if (ha && ca < 0 && visit_leaf<ANY>(s, ~ca, o, d, best, hit, skip)) return true;
        if (hb && cb < 0 && visit_leaf<ANY>(s, ~cb, o, d, best, hit, skip)) return true;
        bool ta = ha && ca >= 0, tb = hb && cb >= 0;
        if (ta && tb) {
            bool anear = an <= bn;
            if (sp >= CPT_STACK) {
                if (err) atomicOr(err, CPT_DEVERR_STACK);
                break;
            }
            stack.put(sp++, anear ? cb : ca);
            node = anear ? ca : cb;
        } else if (ta) {
            node = ca;
        } else if (tb) {
            node = cb;
        } else {
            if (sp == 0) break;
            node = stack.get(--sp);
        }
    }
    return hit.leaf >= 0;
}

// ---------------------------------------------------------------- step-wise BVH2 traversal
// One ray's traversal state, advanced one node per call, so that a warp can refill lanes whose
// ray finished with new rays instead of waiting for its slowest lane (dynamic ray fetching,
// Aila & Laine 2009).  The visit order and pruning are those of trace_closest_bvh2.
template <bool ANY, typename Stack>
struct Bvh2Walk {
    float3 o, d, idir, ood;
    float tmin, best;
    int node, sp, skip;
    Hit hit;
    Stack stack;   // init() once per kernel, before the first start()

    __device__ __forceinline__ void start(float3 o_, float3 d_, float tmin_, float tmax_, int skip_)
    {
        o = o_;
        d = d_;
        idir = safe_inverse(d_);
        ood = f3(o.x * idir.x, o.y * idir.y, o.z * idir.z);
        tmin = tmin_;
        best = tmax_;
        node = 0;
        sp = 0;
        skip = skip_;
        hit.leaf = -1;
        hit.t = tmax_;
        hit.u = hit.v = 0.f;
    }

    // Visits one node; returns true when the traversal has finished.
    __device__ __forceinline__ bool step(const SceneView& s, int* err)
    {
        Bvh2Slabs r;
        bvh2_slabs(s, node, o, idir, ood, r);
        float an = fmaxf(fmaxf(fminf(r.ax0, r.ax1), fminf(r.ay0, r.ay1)), fmaxf(fminf(r.az0, r.az1), tmin));
        float af = fminf(fminf(fmaxf(r.ax0, r.ax1), fmaxf(r.ay0, r.ay1)), fminf(fmaxf(r.az0, r.az1), best));
        float bn = fmaxf(fmaxf(fminf(r.bx0, r.bx1), fminf(r.by0, r.by1)), fmaxf(fminf(r.bz0, r.bz1), tmin));
        float bf = fminf(fminf(fmaxf(r.bx0, r.bx1), fmaxf(r.by0, r.by1)), fminf(fmaxf(r.bz0, r.bz1), best));
        int ca = r.ca, cb = r.cb;
        bool ha = an <= af, hb = bn <= bf;
        if (ha && ca < 0 && visit_leaf<ANY>(s, ~ca, o, d, best, hit, skip)) return true;
        if (hb && cb < 0 && visit_leaf<ANY>(s, ~cb, o, d, best, hit, skip)) return true;
        bool ta = ha && ca >= 0, tb = hb && cb >= 0;
        if (ta && tb) {
            bool anear = an <= bn;
            if (sp >= CPT_STACK) {
                if (err) atomicOr(err, CPT_DEVERR_STACK);
                return true;
            }
            stack.put(sp++, anear ? cb : ca);
            node = anear ? ca : cb;
        } else if (ta) {
            node = ca;
        } else if (tb) {
            node = cb;
        } else {
            if (sp == 0) return true;
            node = stack.get(--sp);
        }
        return false;
    }
};

__device__ __forceinline__ uint32_t lane_mask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Traces work items [0, n) through the BVH2 with dynamic fetching: every loop trip each busy lane
// advances its ray by one node, and once CPT_REFILL lanes (or all) are idle they take the next
// items from *fetch (one atomic per warp).  load(i, o, d, tmin, tmax, skip, scene) supplies item
// i's ray (skip: the light an occlusion query aims at; scene: which of views(scene) it traverses,
// for batches that mix scenes), store(i, hit) takes its result (for ANY, hit.leaf >= 0 means
// occluded).  All 32 lanes of every warp must call this together.  Returns the number of rays
// traced by the lane.
constexpr int CPT_REFILL = 8;

template <typename Walk, typename Views, typename Load, typename Store>
__device__ __forceinline__ uint32_t trace_items_walk(const Views& views, int n, int* fetch, int* err, Load load,
                                                     Store store)
{
    const int lane = threadIdx.x & 31;
    Walk w;
    w.stack.init();
    int item = -1, scene = 0;
    bool exhausted = false;
    uint32_t rays = 0;
    for (;;) {
        const bool idle = item < 0;
        const uint32_t m = __ballot_sync(0xffffffffu, idle);
        // refill once at least CPT_REFILL lanes are idle (one atomic and one divergent ray load per
        // batch instead of per finished ray): 1 -> 8 lanes is +10 % on the 1080p render (16: same)
        if (__popc(m) >= CPT_REFILL && !exhausted) {
            int base = 0;
            if (lane == 0) base = atomicAdd(fetch, __popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + __popc(m) >= n) exhausted = true;
            if (idle) {
                const int r = base + __popc(m & lane_mask_lt());
                if (r < n) {
                    float3 o, d;
                    float tmn, tmx;
                    int skip = -1;
                    load(r, o, d, tmn, tmx, skip, scene);
                    w.start(o, d, tmn, tmx, skip);
                    item = r;
                    rays++;
                }
            }
        }
        if (__all_sync(0xffffffffu, item < 0)) break;
        if (item >= 0 && w.step(views(scene), err)) {
            store(item, w.hit, scene);
            item = -1;
        }
    }
    return rays;
}

template <bool ANY, typename Stack, typename Views, typename Load, typename Store>
__device__ __forceinline__ uint32_t trace_items_bvh2_views(const Views& views, int n, int* fetch, int* err, Load load,
                                                           Store store)
{
    return trace_items_walk<Bvh2Walk<ANY, Stack>>(views, n, fetch, err, load, store);
}

// Dynamic fetching over the 8-wide BVH (the same refill policy).
template <bool ANY, typename Stack64, typename Views, typename Load, typename Store>
__device__ __forceinline__ uint32_t trace_items_wide_views(const Views& views, int n, int* fetch, int* err, Load load,
                                                           Store store)
{
    return trace_items_walk<WideWalk<ANY, Stack64>>(views, n, fetch, err, load, store);
}

// The same over one scene.
template <bool ANY, typename Stack = ShortStack, typename Load, typename Store>
__device__ __forceinline__ uint32_t trace_items_bvh2(const SceneView& s, int n, int* fetch, int* err, Load load,
                                                     Store store)
{
    return trace_items_bvh2_views<ANY, Stack>(
        [&](int) -> const SceneView& { return s; }, n, fetch, err,
        [&](int i, float3& o, float3& d, float& tmn, float& tmx, int& skip, int&) { load(i, o, d, tmn, tmx, skip); },
        [&](int i, const Hit& h, int) { store(i, h); });
}

// Closest hit over [tmin (boxes), tmax]; false on a miss.  WIDE selects the traversal layout at
// compile time (each kernel is instantiated for the layout the scene was built with), so a
// kernel carries the registers and code of one traversal only.  *err gets CPT_DEVERR_STACK if a
// fixed stack would overflow.  With ANY the query is an occlusion test (see occluded).  Stack is
// where the binary traversal keeps its stack (ShortStack needs short_stack_bytes at launch).
template <bool WIDE, bool ANY = false, typename Stack = ShortStack>
__device__ __forceinline__ bool trace_closest(const SceneView& s, float3 o, float3 d, float tmin, float tmax, Hit& hit,
                                              int* err, int skip = -1)
{
    hit.leaf = -1;
    hit.t = tmax;
    hit.u = hit.v = 0.f;
    if (s.n_prims <= 0) return false;
    if (s.n_internal == 0) {
        float best = tmax;
        visit_leaf<ANY>(s, 0, o, d, best, hit, skip);
        return hit.leaf >= 0;
    }
    if (WIDE) return trace_closest_wide<ANY>(s, o, d, tmin, tmax, hit, err, skip);
    return trace_closest_bvh2<ANY, Stack>(s, o, d, tmin, tmax, hit, err, skip);
}

// Visibility of light `light` along a shadow ray whose hit on that light is at t_light (from
// hit_light with the same origin and direction).  The reference's test is "the closest hit is
// that light" (Render.cu:178-181); except for exact ties in t it equals "nothing but that light is
// hit in [0.001, t_light]", which this occlusion query answers and which stops at the first
// occluder instead of searching for the closest one.
template <bool WIDE, typename Stack = ShortStack>
__device__ __forceinline__ bool occluded(const SceneView& s, float3 o, float3 d, float t_light, int light, int* err)
{
    Hit h;
    return trace_closest<WIDE, true, Stack>(s, o, d, 0.001f, t_light, h, err, light);
}

}  // namespace cpt

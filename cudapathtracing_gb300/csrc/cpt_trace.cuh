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

__device__ __forceinline__ void cas(float& ka, uint32_t& va, float& kb, uint32_t& vb)
{
    if (kb < ka) {
        float tk = ka; ka = kb; kb = tk;
        uint32_t tv = va; va = vb; vb = tv;
    }
}

// Closest hit through the compressed 8-wide BVH (layout in wide.cu).  Each visit decodes the 8
// quantised child boxes, tests leaf children at once (as the reference tests leaves when it
// reaches them), sorts the hit internal children by entry distance with a 19-comparator Batcher
// network held in registers, continues with the nearest and pushes the others far-to-near with
// their entry distance; popped entries farther than the closest hit are skipped.
__device__ __forceinline__ bool trace_closest_wide(const SceneView& s, float3 o, float3 d, float tmin, float tmax,
                                                   Hit& hit, int* err)
{
    const float3 idir = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float best = tmax;
    uint64_t stack[CPT_WSTACK];
    int sp = 0;
    uint32_t node = 0;
    for (;;) {
        const float4* np = s.wide + 5 * (size_t)node;
        const float4 h0 = ldg4(np), h1 = ldg4(np + 1), q0 = ldg4(np + 2), q1 = ldg4(np + 3), q2 = ldg4(np + 4);
        const uint32_t e = __float_as_uint(h0.w);
        const float ax = __uint_as_float((e & 0xFFu) << 23) * idir.x;
        const float ay = __uint_as_float(((e >> 8) & 0xFFu) << 23) * idir.y;
        const float az = __uint_as_float(((e >> 16) & 0xFFu) << 23) * idir.z;
        const float bx = (h0.x - o.x) * idir.x, by = (h0.y - o.y) * idir.y, bz = (h0.z - o.z) * idir.z;
        const uint32_t cb = __float_as_uint(h1.x), lb = __float_as_uint(h1.y);
        float key[8];
        uint32_t val[8];
        uint32_t leafmask = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int w = i >> 2, sh = (i & 3) * 8;
            const uint32_t m = ((w ? __float_as_uint(h1.w) : __float_as_uint(h1.z)) >> sh) & 0xFFu;
            key[i] = INFINITY;
            val[i] = 0;
            if (m == 0xFFu) continue;
            const float lx = (float)(((w ? __float_as_uint(q0.y) : __float_as_uint(q0.x)) >> sh) & 0xFFu);
            const float hx = (float)(((w ? __float_as_uint(q0.w) : __float_as_uint(q0.z)) >> sh) & 0xFFu);
            const float ly = (float)(((w ? __float_as_uint(q1.y) : __float_as_uint(q1.x)) >> sh) & 0xFFu);
            const float hy = (float)(((w ? __float_as_uint(q1.w) : __float_as_uint(q1.z)) >> sh) & 0xFFu);
            const float lz = (float)(((w ? __float_as_uint(q2.y) : __float_as_uint(q2.x)) >> sh) & 0xFFu);
            const float hz = (float)(((w ? __float_as_uint(q2.w) : __float_as_uint(q2.z)) >> sh) & 0xFFu);
            const float x0 = fmaf(lx, ax, bx), x1 = fmaf(hx, ax, bx);
            const float y0 = fmaf(ly, ay, by), y1 = fmaf(hy, ay, by);
            const float z0 = fmaf(lz, az, bz), z1 = fmaf(hz, az, bz);
            const float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
            const float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), best));
            if (tn <= tf) {
                if (m & 0x80u) {
                    key[i] = tn;
                    val[i] = cb + (m & 0x7Fu);
                } else {
                    leafmask |= 1u << i;
                }
            }
        }
        // Leaf children in slot order, one copy of the primitive tests.
        while (leafmask) {
            const int i = __ffs(leafmask) - 1;
            leafmask &= leafmask - 1;
            const uint32_t m = ((i >> 2 ? __float_as_uint(h1.w) : __float_as_uint(h1.z)) >> ((i & 3) * 8)) & 0xFFu;
            const int leaf = (int)(lb + m);
            float t, u, v;
            if (hit_leaf(s, leaf, o, d, best, t, u, v)) {
                best = t; hit.t = t; hit.u = u; hit.v = v; hit.leaf = leaf;
            }
        }
        cas(key[0], val[0], key[1], val[1]); cas(key[2], val[2], key[3], val[3]);
        cas(key[4], val[4], key[5], val[5]); cas(key[6], val[6], key[7], val[7]);
        cas(key[0], val[0], key[2], val[2]); cas(key[1], val[1], key[3], val[3]);
        cas(key[4], val[4], key[6], val[6]); cas(key[5], val[5], key[7], val[7]);
        cas(key[1], val[1], key[2], val[2]); cas(key[5], val[5], key[6], val[6]);
        cas(key[0], val[0], key[4], val[4]); cas(key[1], val[1], key[5], val[5]);
        cas(key[2], val[2], key[6], val[6]); cas(key[3], val[3], key[7], val[7]);
        cas(key[2], val[2], key[4], val[4]); cas(key[3], val[3], key[5], val[5]);
        cas(key[1], val[1], key[2], val[2]); cas(key[3], val[3], key[4], val[4]);
        cas(key[5], val[5], key[6], val[6]);
        bool have_next = false;
#pragma unroll
        for (int i = 7; i >= 1; --i) {
            if (key[i] < INFINITY && key[i] <= best) {
                if (sp >= CPT_WSTACK) {
                    if (err) atomicOr(err, CPT_DEVERR_STACK);
                    return hit.leaf >= 0;
                }
                stack[sp++] = ((uint64_t)__float_as_uint(key[i]) << 32) | val[i];
            }
        }
        if (key[0] < INFINITY && key[0] <= best) {
            node = val[0];
            have_next = true;
        }
        while (!have_next && sp > 0) {
            uint64_t top = stack[--sp];
            if (__uint_as_float((uint32_t)(top >> 32)) <= best) {
                node = (uint32_t)top;
                have_next = true;
            }
        }
        if (!have_next) break;
    }
    return hit.leaf >= 0;
}

// Binary-node traversal (Aila–Laine node layout): near child first, far child pushed.  The
// stack cannot overflow for Karras trees over 64-bit keys (at most 65 levels).
__device__ __forceinline__ bool trace_closest_bvh2(const SceneView& s, float3 o, float3 d, float tmin, float tmax,
                                                   Hit& hit, int* err)
{
    const float3 idir = f3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    const float3 ood = f3(o.x * idir.x, o.y * idir.y, o.z * idir.z);
    int stack[CPT_STACK];
    int sp = 0;
    int node = 0;
    float best = tmax;
    for (;;) {
        const float4* np = s.nodes + 4 * (size_t)node;
        float4 n0 = ldg4(np), n1 = ldg4(np + 1), n2 = ldg4(np + 2), n3 = ldg4(np + 3);
        // child A
        float ax0 = fmaf(n0.x, idir.x, -ood.x), ax1 = fmaf(n0.y, idir.x, -ood.x);
        float ay0 = fmaf(n0.z, idir.y, -ood.y), ay1 = fmaf(n0.w, idir.y, -ood.y);
        float az0 = fmaf(n2.x, idir.z, -ood.z), az1 = fmaf(n2.y, idir.z, -ood.z);
        float an = fmaxf(fmaxf(fminf(ax0, ax1), fminf(ay0, ay1)), fmaxf(fminf(az0, az1), tmin));
        float af = fminf(fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1)), fminf(fmaxf(az0, az1), best));
        // child B
        float bx0 = fmaf(n1.x, idir.x, -ood.x), bx1 = fmaf(n1.y, idir.x, -ood.x);
        float by0 = fmaf(n1.z, idir.y, -ood.y), by1 = fmaf(n1.w, idir.y, -ood.y);
        float bz0 = fmaf(n2.z, idir.z, -ood.z), bz1 = fmaf(n2.w, idir.z, -ood.z);
        float bn = fmaxf(fmaxf(fminf(bx0, bx1), fminf(by0, by1)), fmaxf(fminf(bz0, bz1), tmin));
        float bf = fminf(fminf(fmaxf(bx0, bx1), fmaxf(by0, by1)), fminf(fmaxf(bz0, bz1), best));
        int ca = __float_as_int(n3.x), cb = __float_as_int(n3.y);
        bool ha = an <= af, hb = bn <= bf;
        float t, u, v;
        if (ha && ca < 0 && hit_leaf(s, ~ca, o, d, best, t, u, v)) {
            best = t; hit.t = t; hit.u = u; hit.v = v; hit.leaf = ~ca;
        }
        if (hb && cb < 0 && hit_leaf(s, ~cb, o, d, best, t, u, v)) {
            best = t; hit.t = t; hit.u = u; hit.v = v; hit.leaf = ~cb;
        }
        bool ta = ha && ca >= 0, tb = hb && cb >= 0;
        if (ta && tb) {
            bool anear = an <= bn;
            if (sp >= CPT_STACK) {
                if (err) atomicOr(err, CPT_DEVERR_STACK);
                break;
            }
            stack[sp++] = anear ? cb : ca;
            node = anear ? ca : cb;
        } else if (ta) {
            node = ca;
        } else if (tb) {
            node = cb;
        } else {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    return hit.leaf >= 0;
}

// Closest hit over [tmin (boxes), tmax]; false on a miss.  WIDE selects the traversal layout at
// compile time (each kernel is instantiated for the layout the scene was built with), so a
// kernel carries the registers and code of one traversal only.  *err gets CPT_DEVERR_STACK if a
// fixed stack would overflow.
template <bool WIDE>
__device__ __forceinline__ bool trace_closest(const SceneView& s, float3 o, float3 d, float tmin, float tmax, Hit& hit,
                                              int* err)
{
    hit.leaf = -1;
    hit.t = tmax;
    hit.u = hit.v = 0.f;
    if (s.n_prims <= 0) return false;
    if (s.n_internal == 0) {
        float t, u, v;
        if (hit_leaf(s, 0, o, d, tmax, t, u, v)) {
            hit.t = t; hit.u = u; hit.v = v; hit.leaf = 0;
            return true;
        }
        return false;
    }
    if (WIDE) return trace_closest_wide(s, o, d, tmin, tmax, hit, err);
    return trace_closest_bvh2(s, o, d, tmin, tmax, hit, err);
}

}  // namespace cpt

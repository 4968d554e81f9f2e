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

// Closest hit over [tmin (boxes), tmax].  Returns false on a miss.  *err gets
// CPT_DEVERR_STACK if the fixed stack would overflow (cannot happen for Karras trees over
// 64-bit keys, whose depth is at most 65).
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

}  // namespace cpt

// cpt_shade.cuh — FP32 surface records and BSDFs (HitRecord.cuh, Material.cuh).
//
// The formulas are the reference's; two are rewritten in mathematically identical but
// FP32-stable forms:
//   D   (DistributionGGX, Material.cuh:250-265): tan^2(theta) (cos^2 phi/ax^2 + sin^2 phi/ay^2)
//        = (x^2/ax^2 + y^2/ay^2) / z^2 in the local frame (no 0/0 at the pole);
//   Lambda (Material.cuh:266-277): alpha^2 tan^2(acos c) = (ax^2 x^2 + ay^2 y^2) / c^2 with
//        c = max(z, 0) (no acos/tan near 0 and pi/2).
#pragma once

#include "cpt_device.cuh"
#include "cpt_trace.cuh"

namespace cpt {

enum { M_NONE = 0, M_LIGHT = 1, M_OPAQUE = 2, M_SPEC = 3, M_ROUGH = 4, M_VOLUME = 5, M_LAMBERT = 6 };

struct Surf {            // HitRecord (HitRecord.cuh:5-30)
    float3 pos, color, normal, wm;
    float t;
    float ax, ay, eta, sigma_t, albedo;
    int type;
    int prim;            // primitive index (reference order)
    bool front;
};

__device__ __forceinline__ void set_face_normal(Surf& sf, float3 d, float3 outward)   // HitRecord.cuh:32-36
{
    sf.front = dot3(d, outward) < 0.0f;
    sf.normal = sf.front ? outward : -outward;
}

// Luminance of a radiance sample (Rec. 709 weights).
__device__ __forceinline__ float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// G-buffer channel 7 of the config estimator: the variance of the pixel mean's luminance, from the
// sum of the samples' radiance and the sum of their squared luminances (spp samples).  With one
// sample the squared luminance stands in for it.  Both integrators add the same samples in the same
// order (groups in group order), so they write the same value.
__device__ __forceinline__ float mean_variance(float3 sum, float sum_y2, int spp)
{
    if (spp <= 1) return sum_y2;
    const float ys = luminance(sum);
    const float v = (sum_y2 - ys * ys / (float)spp) / ((float)(spp - 1) * (float)spp);
    return fmaxf(v, 0.f);
}

// Nearest texel of an 8-bit RGB image at (u, v) (HitRecord::sampleTexture, HitRecord.cuh:38-49;
// the same rule in Camera::getSkyBox, Camera.cuh:56-61): x = clamp(int(u * w), 0, w - 1), y likewise,
// texels / 255.  The float-to-int conversion saturates, so far-out coordinates clamp too.
__device__ __forceinline__ float3 texel(const DevImage& im, float u, float v)
{
    const int x = min(max(__float2int_rz(u * (float)im.w), 0), im.w - 1);
    const int y = min(max(__float2int_rz(v * (float)im.h), 0), im.h - 1);
    const uint8_t* p = im.rgb + 3 * ((size_t)y * im.w + x);
    const float k = 1.0f / 255.0f;
    return f3((float)__ldg(p) * k, (float)__ldg(p + 1) * k, (float)__ldg(p + 2) * k);
}

// Radiance of a ray that leaves the scene (Camera::getSkyBox, Camera.cuh:50-63): the background
// colour, or the equirectangular sky image at u = atan2(-z, x) / 2pi + 0.5, v = 0.5 - asin(y) / pi
// of the unit direction.
__device__ __forceinline__ float3 sky_radiance(const SceneView& s, float3 d)
{
    if (!s.sky.rgb) return s.cam.background;
    const float3 n = unit3(d);
    const float u = atan2f(-n.z, n.x) * (0.5f / CPT_PI_F) + 0.5f;
    const float v = 0.5f - asinf(fminf(fmaxf(n.y, -1.0f), 1.0f)) * (1.0f / CPT_PI_F);
    return texel(s.sky, u, v);
}

// Surface record of a hit.  reference_materials maps Lambertian to Opaque and uses
// eta = 1.51 (the reference has neither a Lambertian nor a per-material IOR).
__device__ __forceinline__ void make_surface(const SceneView& s, float3 o, float3 d, const Hit& h,
                                             bool reference_materials, Surf& sf)
{
    const float4* r = s.leaf_rec + 3 * (size_t)h.leaf;
    float4 r0 = ldg4(r), r1 = ldg4(r + 1);
    int kind = __float_as_int(r1.w);
    sf.t = h.t;
    sf.prim = __float_as_int(r0.w);
    sf.pos = o + h.t * d;
    sf.wm = f3(0.f, 0.f, 0.f);
    if (kind == CPT_KIND_LIGHT) {
        const DevLight& L = s.lights[__float_as_int(r1.x)];
        sf.color = L.color;
        sf.type = M_LIGHT;
        sf.ax = sf.ay = 1.f;
        sf.eta = 1.51f;
        sf.sigma_t = sf.albedo = 0.f;
        set_face_normal(sf, d, L.normal);
        return;
    }
    uint32_t mi;
    float3 outward;
    float tu = 0.f, tv = 0.f;   // interpolated texture coordinates (triangles)
    if (kind == CPT_KIND_SPHERE) {
        mi = s.sphere_mat[sf.prim - s.n_lights];
        outward = (sf.pos - f3(r0.x, r0.y, r0.z)) / r1.x;
    } else {
        uint32_t ti = (uint32_t)(sf.prim - s.n_lights - s.n_spheres);
        mi = s.tri_mat[ti];
        float4 r2 = ldg4(r + 2);
        float3 e1 = f3(r1.x, r1.y, r1.z), e2 = f3(r2.x, r2.y, r2.z);
        bool smooth = false;
        float3 n0, n1, n2;
        if (s.tri_n) {
            const float* tn = s.tri_n + 9 * (size_t)ti;
            n0 = f3(tn[0], tn[1], tn[2]);
            n1 = f3(tn[3], tn[4], tn[5]);
            n2 = f3(tn[6], tn[7], tn[8]);
            const float E = 1e-8f;   // the reference's "normals provided" test (Hittable.cuh:123-125)
            smooth = !(n0.x < E && n0.y < E && n0.z < E && n1.x < E && n1.y < E && n1.z < E && n2.x < E && n2.y < E &&
                       n2.z < E);
        }
        if (smooth) {
            float w = 1.0f - h.u - h.v;
            outward = unit3(w * n0 + h.u * n1 + h.v * n2);
        } else {
            outward = unit3(cross3(e1, e2));
        }
        if (s.tri_uv) {   // Hittable.cuh:123-125
            const float* uv = s.tri_uv + 6 * (size_t)ti;
            const float w = 1.0f - h.u - h.v;
            tu = w * uv[0] + h.u * uv[2] + h.v * uv[4];
            tv = w * uv[1] + h.u * uv[3] + h.v * uv[5];
        }
    }
    const DevMaterial& m = s.mats[mi];
    sf.color = (kind == CPT_KIND_TRI && m.tex >= 0) ? texel(s.tex[m.tex], tu, tv) : m.color;
    sf.ax = m.ax;
    sf.ay = m.ay;
    sf.type = m.type;
    sf.eta = m.eta;
    sf.sigma_t = m.sigma_t;
    sf.albedo = m.albedo;
    if (reference_materials) {
        if (sf.type == M_LAMBERT || sf.type < M_LIGHT || sf.type > M_VOLUME) sf.type = M_OPAQUE;
        sf.eta = 1.51f;
    }
    set_face_normal(sf, d, outward);
}

// ------------------------------------------------------------------ BSDF (Material.cuh)
__device__ __forceinline__ float3 world_to_local(float3 N, float3 W)   // Material.cuh:238-248
{
    float3 up = f3(0.f, 0.f, 1.f);
    if (fabsf(N.z) > 0.99999f) up = f3(1.f, 0.f, 0.f);
    float3 x = unit3(cross3(up, N));
    float3 y = cross3(N, x);
    return f3(dot3(W, x), dot3(W, y), dot3(W, N));
}

__device__ __forceinline__ float ggx_D(float ax, float ay, float3 N, float3 H)   // Material.cuh:250-265
{
    float3 w = world_to_local(N, H);
    float cos2 = w.z * w.z;
    float e = (w.x * w.x / (ax * ax) + w.y * w.y / (ay * ay)) / cos2;
    float cos4 = cos2 * cos2;
    return 1.0f / (CPT_PI_F * ax * ay * cos4 * (1.0f + e) * (1.0f + e));
}

__device__ __forceinline__ float ggx_lambda(float ax, float ay, float3 N, float3 R)   // Material.cuh:266-277
{
    float3 w = world_to_local(N, R);
    float c = fmaxf(w.z, 0.0f);
    float a2t2 = (ax * ax * w.x * w.x + ay * ay * w.y * w.y) / (c * c);
    return (sqrtf(1.0f + a2t2) - 1.0f) / 2.0f;
}

__device__ __forceinline__ float smith_G2(float ax, float ay, float3 N, float3 V, float3 L)
{
    return 1.0f / (1.0f + ggx_lambda(ax, ay, N, V) + ggx_lambda(ax, ay, N, L));
}
__device__ __forceinline__ float smith_G1(float ax, float ay, float3 N, float3 W) { return 1.0f / (1.0f + ggx_lambda(ax, ay, N, W)); }

__device__ __forceinline__ float fresnel_conductor(float3 N, float3 V, float3 L, float n, float k)   // Material.cuh:287-295
{
    float ci = fmaxf(dot3(N, V), 0.f);
    float ct = fmaxf(dot3(N, L), 0.f);
    // r_parl = (eta ci - ct) / (eta ci + ct), r_perp = (ci - eta ct) / (ci + eta ct), eta = n + ik
    float ax_ = ci * n - ct, ay_ = ci * k, bx = ci * n + ct, by = ci * k;
    float den = bx * bx + by * by;
    float px = (ax_ * bx + ay_ * by) / den, py = (ay_ * bx - ax_ * by) / den;
    float cx = ci - ct * n, cy = -ct * k, dx = ci + ct * n, dy = ct * k;
    float den2 = dx * dx + dy * dy;
    float qx = (cx * dx + cy * dy) / den2, qy = (cy * dx - cx * dy) / den2;
    return (px * px + py * py + qx * qx + qy * qy) / 2.0f;
}

__device__ __forceinline__ float fresnel_dielectric(float3 N, float3 V, float eta)   // Material.cuh:305-318
{
    float ci = fabsf(dot3(N, V));
    float si = sqrtf(fmaxf(0.f, 1.0f - ci * ci));
    float st = si / eta;
    if (st >= 1.0f) return 1.0f;
    float ct = sqrtf(fmaxf(0.f, 1.0f - st * st));
    float rpar = (eta * ci - ct) / (eta * ci + ct);
    float rper = (ci - eta * ct) / (ci + eta * ct);
    return (rpar * rpar + rper * rper) * 0.5f;
}

// Material::fr (Material.cuh:24-93), plus Lambertian albedo/pi.
__device__ __forceinline__ float3 bsdf_eval(const Surf& sf, float3 ray_d, float3 dir)
{
    if (sf.type == M_LAMBERT) return sf.color / CPT_PI_F;
    float3 V = unit3(-ray_d);
    float3 L = unit3(dir);
    float3 H = unit3(V + L);
    const float3 n = sf.normal;
    bool reflect = dot3(V, n) * dot3(L, n) > 0.0f;
    if (sf.type == M_SPEC) {
        float rr = sf.front ? sf.eta : (1.0f / sf.eta);
        float ct = fabsf(dot3(n, L));
        float F = fresnel_dielectric(n, V, rr);
        return (reflect ? F : 1.0f - F) * sf.color / ct;
    } else if (!reflect) {
        // Only the rough dielectric transmits.  For the conductor this branch is reached only by
        // a grazing direction whose cosine changes sign when it is renormalised in FP32 (the
        // caller saw it above the surface); it has no transmission lobe (and no sampled
        // microfacet normal), so it contributes nothing.
        if (sf.type != M_ROUGH) return f3(0.f, 0.f, 0.f);
        float rr = sf.front ? sf.eta : (1.0f / sf.eta);
        float D = ggx_D(sf.ax, sf.ay, n, sf.wm);
        if (dot3(sf.wm, V) < 0.f) V = -V;
        if (dot3(sf.wm, L) < 0.f) L = -L;
        float G = smith_G2(sf.ax, sf.ay, n, V, L);
        float F = fresnel_dielectric(sf.wm, V, rr);
        float ci = fabsf(dot3(n, V)), ct = fabsf(dot3(n, L));
        float mb = fabsf(dot3(L, sf.wm)) + fabsf(dot3(V, sf.wm)) / rr;
        float den = mb * mb;
        float spec = (1.0f - F) * D * G * fabsf(dot3(sf.wm, L) * dot3(sf.wm, V) / (ci * ct * den));
        return spec * sf.color;
    } else {
        float nn = 2.63f, kk = 9.08f;
        if (sf.type == M_ROUGH) { nn = 1.58f; kk = 0.001f; }
        float D = ggx_D(sf.ax, sf.ay, n, H);
        float G = smith_G2(sf.ax, sf.ay, n, V, L);
        float F = fresnel_conductor(n, V, L, nn, kk);
        float NdotL = fmaxf(dot3(n, L), 0.f), NdotV = fmaxf(dot3(n, V), 0.f);
        float den = 4.0f * NdotV * NdotL + 0.001f;
        return (D * G * F) / den * sf.color;
    }
}

// brdf (Material.cuh:201-235): VNDF reflection sampling of the anisotropic GGX.
__device__ __forceinline__ void sample_ggx_reflect(const Surf& sf, float3 ray_d, float3& dir, float& pdf, float r1,
                                                   float r2)
{
    float3 w = sf.normal;
    float3 a = (fabsf(w.z) > 0.99999f) ? f3(1.f, 0.f, 0.f) : f3(0.f, 0.f, 1.f);
    float3 u = unit3(cross3(a, w));
    float3 v = cross3(w, u);
    float3 urd = -unit3(ray_d);
    float3 Wo = f3(dot3(urd, u), dot3(urd, v), dot3(urd, w));
    float3 Wh = unit3(f3(sf.ax * Wo.x, sf.ay * Wo.y, Wo.z));
    float3 T1 = (Wh.z < 0.99999f) ? unit3(cross3(f3(0.f, 0.f, 1.f), Wh)) : unit3(cross3(f3(1.f, 0.f, 0.f), Wh));
    float3 T2 = cross3(Wh, T1);
    float r = sqrtf(r1);
    float sn, cs;
    sincosf(2.0f * CPT_PI_F * r2, &sn, &cs);
    float px = r * cs, py = r * sn;
    float h = sqrtf(1.0f - px * px);
    float lx = (1.0f + Wh.z) / 2.0f;
    py = (1.0f - lx) * h + lx * py;
    float pz = sqrtf(fmaxf(0.f, 1.0f - (px * px + py * py)));
    float3 nh = px * T1 + py * T2 + pz * Wh;
    float3 Wm = unit3(f3(sf.ax * nh.x, sf.ay * nh.y, fmaxf(1e-6f, nh.z)));
    float3 Wi = -Wo + 2.0f * dot3(Wo, Wm) * Wm;
    dir = unit3(Wi.x * u + Wi.y * v + Wi.z * w);
    if (dot3(dir, sf.normal) < 0.f) {
        pdf = -1.f;
        return;
    }
    float3 H = unit3(dir + urd);
    pdf = smith_G1(sf.ax, sf.ay, sf.normal, urd) / Wo.z * ggx_D(sf.ax, sf.ay, sf.normal, H) / 4.0f;
}

// Material::sampleLight (Material.cuh:95-193) + cosine-weighted Lambertian (the reference's
// commented sampler, Material.cuh:177-188).  Writes sf.wm for the rough dielectric.
__device__ __forceinline__ void bsdf_sample(Surf& sf, float3 ray_d, float3& dir, float& pdf, float r1, float r2, float r3)
{
    const float3 n = sf.normal;
    if (sf.type == M_SPEC) {
        float rr = sf.front ? sf.eta : (1.0f / sf.eta);
        float3 urd = unit3(ray_d);
        float R = fresnel_dielectric(n, -urd, rr);
        if (r3 < R) {
            dir = urd - 2.0f * dot3(urd, n) * n;
            pdf = R;
        } else {
            float3 vperp = (1.0f / rr) * (urd + dot3(-urd, n) * n);
            float3 vpar = -sqrtf(fabsf(1.0f - len2(vperp))) * n;
            dir = unit3(vperp + vpar);
            pdf = 1.0f - R;
        }
    } else if (sf.type == M_ROUGH) {
        float3 w = n;
        float3 a = (fabsf(w.x) > 0.9f) ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
        float3 u = unit3(cross3(w, a));
        float3 v = cross3(w, u);
        float3 urd = -unit3(ray_d);
        float3 Wo = f3(dot3(urd, u), dot3(urd, v), dot3(urd, w));
        float3 Wh = unit3(f3(sf.ax * Wo.x, sf.ay * Wo.y, Wo.z));
        float3 T1 = (Wh.z < 0.99999f) ? unit3(cross3(f3(0.f, 0.f, 1.f), Wh)) : f3(1.f, 0.f, 0.f);
        float3 T2 = cross3(Wh, T1);
        float r = sqrtf(r1);
        float sn, cs;
        sincosf(2.0f * CPT_PI_F * r2, &sn, &cs);
        float px = r * cs, py = r * sn;
        float h = sqrtf(1.0f - px * px);
        float lx = (1.0f + Wh.z) / 2.0f;
        py = (1.0f - lx) * h + lx * py;
        float pz = sqrtf(fmaxf(0.f, 1.0f - (px * px + py * py)));
        float3 nh = px * T1 + py * T2 + pz * Wh;
        float3 Wm = unit3(f3(sf.ax * nh.x, sf.ay * nh.y, fmaxf(1e-6f, nh.z)));
        float3 sn3 = unit3(Wm.x * u + Wm.y * v + Wm.z * w);
        sf.wm = sn3;
        float rr = sf.front ? sf.eta : (1.0f / sf.eta);
        float R = fresnel_dielectric(sn3, -urd, rr);
        if (r3 < R) {
            sample_ggx_reflect(sf, ray_d, dir, pdf, r1, r2);
            pdf *= R;
        } else {
            float3 vperp = (1.0f / rr) * (urd + dot3(-urd, sn3) * sn3);
            float3 vpar = -sqrtf(fabsf(1.0f - len2(vperp))) * sn3;
            float3 rd = unit3(vperp + vpar);
            float3 Wi = f3(dot3(rd, u), dot3(rd, v), dot3(rd, w));
            dir = rd;
            if (dot3(dir, n) > 0.f) {
                pdf = -1.f;
                return;
            }
            float mb = dot3(-Wi, Wm) + dot3(Wo, Wm) / rr;
            float den = mb * mb;
            float dwm = fabsf(dot3(Wi, Wm)) / den;
            pdf = smith_G1(sf.ax, sf.ay, n, urd) / Wo.z * ggx_D(sf.ax, sf.ay, n, sn3) * dot3(Wo, Wm) * dwm * (1.0f - R);
        }
    } else if (sf.type == M_OPAQUE) {
        sample_ggx_reflect(sf, ray_d, dir, pdf, r1, r2);
    } else if (sf.type == M_LAMBERT) {
        float sinT = sqrtf(1.0f - r1), cosT = sqrtf(r1);
        float3 w = n;
        float3 a = (fabsf(w.x) > 0.9f) ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
        float3 u = unit3(cross3(w, a));
        float3 v = cross3(w, u);
        float sn, cs;
        sincosf(2.0f * CPT_PI_F * r2, &sn, &cs);
        dir = cs * sinT * u + sn * sinT * v + cosT * w;
        pdf = cosT / CPT_PI_F;
    } else {
        pdf = -1.f;
    }
}

}  // namespace cpt

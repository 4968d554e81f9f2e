// render.cu — the megakernel integrator: one thread per pixel, samples in sequence with one
// PCG32 stream per pixel (render, Render.cu:16-261, STATIC mode), in FP32.
//
//   estimator REFERENCE: the reference's estimator (RR 0.7 from the first bounce, NEE only at
//     Opaque with pdf 1/(width*width), emission ignored after the first NEE, the sigma_maj = 25
//     volume), with the same order of random draws so that paths match the FP64 oracle.
//   estimator CONFIG: the config estimator (depth limit, RR from rr_depth on, Lambertian,
//     per-material IOR, homogeneous media with sigma_t and albedo), with one PCG32 sub-stream
//     per sample and group-wise sample sums (Pcg32::init_sample, sample_group).
#include <cuda_runtime.h>

#include <type_traits>

#include "cpt_internal.h"
#include "cpt_shade.cuh"

namespace cpt {

namespace {

// Traversal stack of the megakernel: local memory.  (A shared-memory short stack made this
// 122-register kernel slower on GB300; the wavefront's trace kernels use one.)
using MkStack = LocalStack;
constexpr size_t mk_stack_smem(int threads) { return std::is_same<MkStack, ShortStack>::value ? short_stack_bytes(threads) : 0; }

__device__ __forceinline__ float3 camera_dir(const DevCamera& c, int i, int j, float rx, float ry)   // Camera.cuh:37-43
{
    float3 p = c.pixel_center + (rx - 0.5f + (float)i) * c.delta_h + (ry - 0.5f + (float)j) * c.delta_v;
    return p - c.look_from;
}

struct PixelResult {
    float3 rgb;
    float3 gn;
    float gdepth;
    float3 galb;
    float gvar;   // variance of the pixel mean's luminance (config estimator), 0 otherwise
    uint32_t rays;
};

__device__ __forceinline__ int prim_of(const SceneView& s, const Hit& h)
{
    return h.leaf >= 0 ? __float_as_int(ldg4(s.leaf_rec + 3 * (size_t)h.leaf).w) : -1;
}

template <bool WIDE>
__device__ PixelResult pixel_reference(const SceneView& s, int i, int j, const RenderArgs& a)
{
    PixelResult out;
    out.rays = 0;
    out.gvar = 0.f;
    const DevCamera& cam = s.cam;
    Pcg32 rng;
    rng.init(a.seed, (uint64_t)j * cam.width + i);
    float3 pix = f3(0.f, 0.f, 0.f);
    for (int sample = 0; sample < a.spp; ++sample) {
        float rx = rng.uniform();
        float ry = rng.uniform();
        float3 o = cam.look_from;
        float3 d = camera_dir(cam, i, j, rx, ry);
        float3 thr = f3(1.f, 1.f, 1.f), rad = f3(0.f, 0.f, 0.f);
        out.gn = f3(0.f, 0.f, 0.f);
        out.gdepth = CPT_INF_F;
        out.galb = f3(0.f, 0.f, 0.f);
        bool has_sample_light = false;
        for (int guard = 0;; ++guard) {
            if (guard >= a.iter_limit) {
                atomicOr(a.err, CPT_DEVERR_ITER);
                break;
            }
            Hit h;
            bool hit = trace_closest<WIDE, false, MkStack>(s, o, d, 0.001f, CPT_INF_F, h, a.err);
            out.rays++;
            Surf sf;
            if (hit) make_surface(s, o, d, h, true, sf);
            if (hit && sf.type == M_VOLUME) {   // Render.cu:64-135
                const float sig = 25.0f;
                o = sf.pos;
                Hit vh;
                bool vhit = trace_closest<WIDE, false, MkStack>(s, o, d, 0.001f, CPT_INF_F, vh, a.err);
                out.rays++;
                if (!vhit) continue;
                float dmax = vh.t;
                float t = -logf(rng.one_minus_uniform_from(rng.next())) / sig;
                float3 pos = sf.pos + t * d;
                o = pos;
                for (int vguard = 0; t < dmax; ++vguard) {
                    if (vguard >= a.iter_limit) {
                        atomicOr(a.err, CPT_DEVERR_ITER);
                        break;
                    }
                    if (rng.uniform() > 0.8f) break;
                    thr = thr * (expf(-t * sig) / 0.8f);
                    float z = 1.0f - 2.0f * rng.uniform();
                    float r = sqrtf(1.0f - z * z);
                    float phi = 2.0f * CPT_PI_F * rng.uniform();
                    float sn, cs;
                    sincosf(phi, &sn, &cs);
                    float3 nd = unit3(f3(r * cs, r * sn, z));
                    o = pos;
                    d = nd;
                    pos = sf.pos + t * nd;
                    vhit = trace_closest<WIDE, false, MkStack>(s, o, d, 0.001f, CPT_INF_F, vh, a.err);
                    out.rays++;
                    if (vhit) dmax = vh.t;
                    t = -logf(rng.one_minus_uniform_from(rng.next())) / sig;
                    if (t > dmax || !vhit) break;
                }
                continue;
            }
            if (!hit) {
                rad = rad + thr * sky_radiance(s, d);
                break;
            }
            if (sf.type == M_LIGHT) {
                if (!has_sample_light) rad = rad + thr * sf.color;
                break;
            }
            out.gn = sf.normal;   // depth stays 0 in STATIC mode: the last surface wins (Render.cu:152-159)
            out.gdepth = sqrtf(len2(cam.look_from - sf.pos));
            out.galb = sf.color;
            for (int k = 0; k < s.n_lights; ++k) {   // Render.cu:163-187
                if (sf.type != M_OPAQUE) break;
                const DevLight& L = s.lights[k];
                float lw = L.w, lh = L.w;   // the reference uses the width twice (Render.cu:170-171)
                float pdf_l = 1.0f / (lw * lh);
                float ub = rng.uniform();   // second draw first: the order of the compiled reference
                float ua = rng.uniform();
                float3 lp = L.center + ((ua - 0.5f) * lw) * L.eu + ((ub - 0.5f) * lh) * L.ev;
                float3 dir = unit3(lp - sf.pos);
                Hit lh2;
                trace_closest<WIDE, false, MkStack>(s, sf.pos, dir, 0.001f, CPT_INF_F, lh2, a.err);
                out.rays++;
                int obst = prim_of(s, lh2);
                if (dot3(dir, sf.normal) > 0.f && dot3(-dir, L.normal) > 0.f && obst == k) {
                    float3 fr = bsdf_eval(sf, d, dir);
                    float3 cl = L.color * fr * dot3(dir, sf.normal) * dot3(-dir, L.normal) / len2(lp - sf.pos) / pdf_l;
                    rad = rad + thr * cl;
                }
                has_sample_light = true;
            }
            const float P = 0.7f;   // Render.cu:199-204
            if (rng.uniform() > P) break;
            float r1 = rng.uniform(), r2 = rng.uniform(), r3 = rng.uniform();
            float3 dir;
            float pdf;
            bsdf_sample(sf, d, dir, pdf, r1, r2, r3);
            if (!(pdf > 0.f)) break;   // also ends the path on a NaN pdf (0/0 at a grazing direction)
            float3 fr = bsdf_eval(sf, d, dir);
            thr = thr * (fr * fabsf(dot3(dir, sf.normal)) / pdf / P);
            o = sf.pos;
            d = dir;
        }
        pix = pix + rad;
    }
    out.rgb = pix / (float)a.spp;
    return out;
}

template <bool WIDE>
__device__ PixelResult pixel_config(const SceneView& s, int i, int j, const RenderArgs& a)
{
    PixelResult out;
    out.rays = 0;
    out.gn = f3(0.f, 0.f, 0.f);
    out.gdepth = CPT_INF_F;
    out.galb = f3(0.f, 0.f, 0.f);
    const DevCamera& cam = s.cam;
    const uint64_t stream = (uint64_t)j * cam.width + i;
    const int group = sample_group(a.spp);
    float3 pix = f3(0.f, 0.f, 0.f), gsum = f3(0.f, 0.f, 0.f);
    float pix_y2 = 0.f, gsum_y2 = 0.f;   // sums of the samples' squared luminances
    for (int sample = 0; sample < a.spp; ++sample) {
        Pcg32 rng;
        rng.init_sample(a.seed, stream, (uint32_t)sample);
        float rx = rng.uniform();
        float ry = rng.uniform();
        float3 o = cam.look_from;
        float3 d = camera_dir(cam, i, j, rx, ry);
        float3 thr = f3(1.f, 1.f, 1.f), rad = f3(0.f, 0.f, 0.f);
        bool count_emission = true, in_medium = false;
        float m_sigma = 0.f, m_albedo = 0.f;
        int depth = 0;
        for (int guard = 0;; ++guard) {
            if (guard >= a.iter_limit) {
                atomicOr(a.err, CPT_DEVERR_ITER);
                break;
            }
            Hit h;
            bool hit = trace_closest<WIDE, false, MkStack>(s, o, d, 0.001f, CPT_INF_F, h, a.err);
            out.rays++;
            if (in_medium) {
                float t_hit = hit ? h.t : CPT_INF_F;
                float t = -logf(rng.uniform()) / m_sigma;
                if (t < t_hit) {
                    float3 pos = o + t * d;
                    thr = thr * m_albedo;
                    depth++;
                    if (a.max_depth > 0 && depth >= a.max_depth) break;
                    float P = 1.0f;
                    if (depth >= a.rr_depth) {
                        P = a.rr_prob;
                        if (rng.uniform() > P) break;
                    }
                    thr = thr * (1.0f / P);
                    float z = 1.0f - 2.0f * rng.uniform();
                    float r = sqrtf(fmaxf(0.f, 1.0f - z * z));
                    float phi = 2.0f * CPT_PI_F * rng.uniform();
                    float sn, cs;
                    sincosf(phi, &sn, &cs);
                    o = pos;
                    d = f3(r * cs, r * sn, z);
                    count_emission = true;
                    continue;
                }
            }
            if (!hit) {
                rad = rad + thr * sky_radiance(s, d);
                break;
            }
            Surf sf;
            make_surface(s, o, d, h, false, sf);
            if (sf.type == M_VOLUME) {
                in_medium = sf.front;
                m_sigma = sf.sigma_t;
                m_albedo = sf.albedo;
                o = sf.pos;
                continue;
            }
            if (sf.type == M_LIGHT) {
                if (count_emission) rad = rad + thr * sf.color;
                break;
            }
            if (depth == 0 && sample < group && out.gdepth >= CPT_INF_F) {   // first surface hit of group 0
                out.gn = sf.normal;
                out.gdepth = sqrtf(len2(cam.look_from - sf.pos));
                out.galb = sf.color;
            }
            bool diffuse_like = (sf.type == M_OPAQUE || sf.type == M_LAMBERT);
            if (diffuse_like) {
                for (int k = 0; k < s.n_lights; ++k) {
                    const DevLight& L = s.lights[k];
                    float area = L.w * L.h;
                    float ua = rng.uniform();
                    float ub = rng.uniform();
                    float3 lp = L.center + ((ua - 0.5f) * L.w) * L.eu + ((ub - 0.5f) * L.h) * L.ev;
                    float3 dir = unit3(lp - sf.pos);
                    float cs_ = dot3(dir, sf.normal), cl_ = dot3(-dir, L.normal);
                    if (!(cs_ > 0.f && cl_ > 0.f)) continue;   // cannot contribute: no shadow ray
                    float tl;
                    if (!hit_light(L, sf.pos, dir, 0.001f, CPT_INF_F, tl)) continue;   // cannot see the light
                    out.rays++;
                    if (!occluded<WIDE, MkStack>(s, sf.pos, dir, tl, k, a.err)) {
                        float3 fr = bsdf_eval(sf, d, dir);
                        float g = cs_ * cl_ / len2(lp - sf.pos) * area;
                        rad = rad + thr * (L.color * fr * g);
                    }
                }
            }
            count_emission = !diffuse_like || s.n_lights == 0;
            depth++;
            if (a.max_depth > 0 && depth >= a.max_depth) break;
            float P = 1.0f;
            if (depth >= a.rr_depth) {
                P = a.rr_prob;
                if (rng.uniform() > P) break;
            }
            float r1 = rng.uniform(), r2 = rng.uniform(), r3 = rng.uniform();
            float3 dir;
            float pdf;
            bsdf_sample(sf, d, dir, pdf, r1, r2, r3);
            if (!(pdf > 0.f)) break;   // also ends the path on a NaN pdf (0/0 at a grazing direction)
            float3 fr = bsdf_eval(sf, d, dir);
            thr = thr * (fr * fabsf(dot3(dir, sf.normal)) / pdf / P);
            o = sf.pos;
            d = dir;
        }
        gsum = gsum + rad;
        const float y = luminance(rad);
        gsum_y2 += y * y;
        if ((sample + 1) % group == 0 || sample + 1 == a.spp) {
            pix = pix + gsum;
            gsum = f3(0.f, 0.f, 0.f);
            pix_y2 += gsum_y2;
            gsum_y2 = 0.f;
        }
    }
    out.rgb = pix / (float)a.spp;
    out.gvar = mean_variance(pix, pix_y2, a.spp);
    return out;
}

__device__ __forceinline__ uint8_t to_u8(float x)   // Render.cu:256-258
{
    float c = sqrtf(x);
    c = c > 1.0f ? 1.0f : (c < 0.0f ? 0.0f : c);
    return (uint8_t)(254.99f * c);
}

// At most 72 registers (121 uncapped: 4 blocks of 128 per SM): the spilled values cost less than
// the occupancy they buy (1080p spheres, default block: 649 -> 823 Mrays/s; 64: 813, 80: 783, 96: 729).
template <int EST, bool WIDE>
__global__ void __maxnreg__(72) k_render(SceneView s, RenderArgs a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = a.row_begin + blockIdx.y * blockDim.y + threadIdx.y;
    bool active = i < s.cam.width && j < a.row_end;
    uint32_t rays = 0;
    if (active) {
        PixelResult r = EST == 0 ? pixel_reference<WIDE>(s, i, j, a) : pixel_config<WIDE>(s, i, j, a);
        size_t off = (size_t)j * s.cam.width + i;
        if (a.flags & CPT_RENDER_ACCUMULATE) {
            a.rgb[3 * off] += r.rgb.x;
            a.rgb[3 * off + 1] += r.rgb.y;
            a.rgb[3 * off + 2] += r.rgb.z;
        } else {
            a.rgb[3 * off] = r.rgb.x;
            a.rgb[3 * off + 1] = r.rgb.y;
            a.rgb[3 * off + 2] = r.rgb.z;
        }
        if (a.rgba8) {
            uchar4 c = make_uchar4(to_u8(r.rgb.x), to_u8(r.rgb.y), to_u8(r.rgb.z), 255);
            reinterpret_cast<uchar4*>(a.rgba8)[off] = c;
        }
        if (a.gbuf) {
            float4* g = reinterpret_cast<float4*>(a.gbuf) + 2 * off;
            g[0] = make_float4(r.gn.x, r.gn.y, r.gn.z, r.gdepth);
            g[1] = make_float4(r.galb.x, r.galb.y, r.galb.z, r.gvar);
        }
        rays = r.rays;
    }
    unsigned long long rc = rays;
#pragma unroll
    for (int o = 16; o; o >>= 1) rc += __shfl_xor_sync(0xffffffffu, rc, o);
    if ((threadIdx.x + threadIdx.y * blockDim.x) % 32 == 0 && a.ray_counter) atomicAdd(a.ray_counter, rc);
}

}  // namespace

cpt_status launch_render_megakernel(const SceneView& view, const RenderArgs& args, cudaStream_t stream, int bx, int by)
{
    if (bx * by % 32 != 0) return fail(CPT_ERR_INVALID_ARGUMENT, "render block size must be a multiple of 32 threads");
    int rows = args.row_end - args.row_begin;
    if (rows <= 0) return CPT_OK;
    dim3 block(bx, by);
    dim3 grid((view.cam.width + bx - 1) / bx, (rows + by - 1) / by);
    const bool wide = view.wide != nullptr;
    if (bx * by > 512) return fail(CPT_ERR_INVALID_ARGUMENT, "render block: at most 512 threads");
    const size_t smem = mk_stack_smem(bx * by);
    if (args.estimator == CPT_ESTIMATOR_REFERENCE) {
        if (wide) k_render<0, true><<<grid, block, smem, stream>>>(view, args);
        else k_render<0, false><<<grid, block, smem, stream>>>(view, args);
    } else {
        if (wide) k_render<1, true><<<grid, block, smem, stream>>>(view, args);
        else k_render<1, false><<<grid, block, smem, stream>>>(view, args);
    }
    CPT_CUDA(cudaGetLastError());
    add_launches(1);
    return CPT_OK;
}

}  // namespace cpt

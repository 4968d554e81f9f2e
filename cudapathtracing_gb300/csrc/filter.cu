// filter.cu — the reference's non-learned denoiser, in FP32 on device-resident images:
//
//   cpt_filter_bilateral  separable joint-bilateral filter (gaussianSeparate, Render.cu:356-398),
//                         horizontal pass then vertical pass as the REAL_TIME loop runs it
//                         (main.cu:99-103): weights exp(-i^2/2sg^2 - |c_n - c|^2/2sr^2
//                         - |n_n - n|^2/2sn^2 - (d_n - d)^2/2sd^2) over a (2R+1)-tap window with
//                         clamped borders, normalised by their sum.
//   cpt_filter_temporal   reprojection + exponential blend with the previous frame
//                         (addPrevious, Render.cu:400-420, Camera::getPrePositionInImg,
//                         Camera.cuh:103-132).
//
// Images are W*H float3 (row j = 0 at the bottom, as rendered); the G-buffer is the renderer's
// 2 float4 per pixel, (normal, depth) then (albedo, 0), depth 999999 (INF) on a miss.
//
// The reference reads the world position of the first hit from a separate buffer; this build
// reconstructs it as look_from + depth * unit(direction through the pixel centre), which differs
// from the sample's jittered hit point by less than a pixel footprint.  The reference indexes
// the previous frame at int(x * W) for x in [0, 1], which reaches W at x = 1; here the index is
// clamped to the image.
#include <cuda_runtime.h>

#include <cmath>

#include "cpt_internal.h"

namespace cpt {

namespace {

struct BilateralConsts {
    float kg, kr, kn, kd;   // 1 / (2 sigma^2) of the four terms
    int radius;
};

// One separable pass over `src`: the centre value and the neighbours come from the same image
// (in the reference the centre is read from pic, which holds the same values as the pass input).
template <bool HORIZONTAL>
__global__ void __launch_bounds__(256) k_bilateral_pass(const float* __restrict__ src, const float4* __restrict__ gbuf,
                                                        float* __restrict__ out, int W, int H, BilateralConsts k)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t off = (size_t)y * W + x;
    const float4 g = __ldg(gbuf + 2 * off);
    const float3 c = f3(__ldg(src + 3 * off), __ldg(src + 3 * off + 1), __ldg(src + 3 * off + 2));
    float3 acc = f3(0.f, 0.f, 0.f);
    float wsum = 0.f;
    for (int i = -k.radius; i <= k.radius; ++i) {
        int nx = x, ny = y;
        if (HORIZONTAL) nx = min(max(x + i, 0), W - 1);
        else ny = min(max(y + i, 0), H - 1);
        const size_t n = (size_t)ny * W + nx;
        const float3 p = f3(__ldg(src + 3 * n), __ldg(src + 3 * n + 1), __ldg(src + 3 * n + 2));
        const float4 gp = __ldg(gbuf + 2 * n);
        const float3 dc = p - c;
        const float3 dn = f3(g.x - gp.x, g.y - gp.y, g.z - gp.z);
        const float dd = g.w - gp.w;
        const float e = -(float)(i * i) * k.kg - dot3(dc, dc) * k.kr - dot3(dn, dn) * k.kn - dd * dd * k.kd;
        const float w = expf(e);
        wsum += w;
        acc = acc + w * p;
    }
    const float3 r = acc / wsum;
    out[3 * off] = r.x;
    out[3 * off + 1] = r.y;
    out[3 * off + 2] = r.z;
}

// The previous camera's frame (getPrePositionInImg) and the current camera's pixel rays.
struct Reproj {
    float3 from, right, up, fwd;   // previous camera
    float sx, sy;                  // focal / viewport width, focal / viewport height
    float3 cur_from, cur_pc, cur_dh, cur_dv;
};

__global__ void __launch_bounds__(256) k_temporal(float* __restrict__ rgb, const float* __restrict__ prev,
                                                  const float4* __restrict__ gbuf, int W, int H, Reproj r, float alpha)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t off = (size_t)y * W + x;
    const float depth = __ldg(gbuf + 2 * off).w;
    size_t src = off;
    if (depth < CPT_INF_F) {
        const float3 dir = unit3(r.cur_pc + (float)x * r.cur_dh + (float)y * r.cur_dv - r.cur_from);
        const float3 pos = r.cur_from + depth * dir;
        const float3 v = unit3(pos - r.from);
        const float px = dot3(v, r.right), py = dot3(v, r.up), pz = dot3(v, r.fwd);
        const float u = 0.5f + (px / pz) * r.sx;
        const float w = 0.5f + (py / pz) * r.sy;
        if (u >= 0.f && w >= 0.f && u <= 1.f && w <= 1.f) {
            const int i = min((int)(u * (float)W), W - 1);
            const int j = min((int)(w * (float)H), H - 1);
            src = (size_t)j * W + i;
        }
    }
    for (int c = 0; c < 3; ++c) rgb[3 * off + c] = rgb[3 * off + c] * alpha + __ldg(prev + 3 * src + c) * (1.0f - alpha);
}

struct V3 {
    double x, y, z;
};
inline V3 v3(const double* a) { return {a[0], a[1], a[2]}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 unit(V3 a)
{
    double l = std::sqrt(dot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}
inline float3 tof(V3 a) { return make_float3((float)a.x, (float)a.y, (float)a.z); }

inline int image_height(const cpt_camera& c)
{
    double hh = c.width / c.aspect_ratio;   // Camera.cu:8-9
    return hh < 1 ? 1 : (int)hh;
}

}  // namespace

cpt_status filter_bilateral(const float* rgb, const float* gbuf, float* out, int W, int H, const cpt_filter_params& p,
                            cudaStream_t stream)
{
    if (W <= 0 || H <= 0) return CPT_OK;
    if (p.radius < 0 || p.radius > 256 || !(p.sigma_g > 0) || !(p.sigma_r > 0) || !(p.sigma_n > 0) || !(p.sigma_d > 0))
        return fail(CPT_ERR_INVALID_ARGUMENT, "bilateral filter: sigmas must be positive, radius in [0, 256]");
    if (!rgb || !gbuf || !out) return fail(CPT_ERR_INVALID_ARGUMENT, "bilateral filter: null buffer");
    if (((uintptr_t)gbuf & 15u)) return fail(CPT_ERR_INVALID_ARGUMENT, "bilateral filter: G-buffer must be 16-byte aligned");
    BilateralConsts k;
    k.kg = 1.0f / (2.0f * p.sigma_g * p.sigma_g);
    k.kr = 1.0f / (2.0f * p.sigma_r * p.sigma_r);
    k.kn = 1.0f / (2.0f * p.sigma_n * p.sigma_n);
    k.kd = 1.0f / (2.0f * p.sigma_d * p.sigma_d);
    k.radius = p.radius;
    float* tmp = nullptr;
    CPT_CUDA(cudaMallocAsync((void**)&tmp, (size_t)W * H * 3 * sizeof(float), stream));
    dim3 block(32, 8), grid((W + 31) / 32, (H + 7) / 8);
    k_bilateral_pass<true><<<grid, block, 0, stream>>>(rgb, (const float4*)gbuf, tmp, W, H, k);
    k_bilateral_pass<false><<<grid, block, 0, stream>>>(tmp, (const float4*)gbuf, out, W, H, k);
    add_launches(2);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(tmp, stream);
    if (e != cudaSuccess) return cuda_fail(e, "bilateral filter launch");
    return CPT_OK;
}

cpt_status filter_temporal(float* rgb, const float* prev, const float* gbuf, const cpt_camera& cam,
                           const cpt_camera& prev_cam, float alpha, cudaStream_t stream)
{
    const int W = cam.width, H = image_height(cam);
    if (W <= 0) return CPT_OK;
    if (!rgb || !prev || !gbuf) return fail(CPT_ERR_INVALID_ARGUMENT, "temporal filter: null buffer");
    if (((uintptr_t)gbuf & 15u)) return fail(CPT_ERR_INVALID_ARGUMENT, "temporal filter: G-buffer must be 16-byte aligned");
    if (prev_cam.width != cam.width || image_height(prev_cam) != H)
        return fail(CPT_ERR_INVALID_ARGUMENT, "temporal filter: cameras differ in image size");
    if (!(alpha >= 0.f && alpha <= 1.f)) return fail(CPT_ERR_INVALID_ARGUMENT, "temporal filter: alpha in [0, 1]");
    // previous camera frame, in double (Camera.cuh:109-123)
    const V3 from = v3(prev_cam.look_from), at = v3(prev_cam.look_at), vup = {0.0, 1.0, 0.0};
    const V3 fwd = unit(at - from);
    const V3 right = unit(cross(fwd, vup));
    const V3 up = cross(right, fwd);
    const double focal = std::sqrt(dot(from - at, from - at));
    const double h = std::tan(prev_cam.vfov_deg * 3.14159265358979323846 / 180.0 / 2.0);
    const double vh = 2.0 * h * focal;
    const double vw = (double)W / H * vh;
    Reproj r;
    r.from = tof(from);
    r.right = tof(right);
    r.up = tof(up);
    r.fwd = tof(fwd);
    r.sx = (float)(focal / vw);
    r.sy = (float)(focal / vh);
    const DevCamera dc = camera_of(cam);
    r.cur_from = dc.look_from;
    r.cur_pc = dc.pixel_center;
    r.cur_dh = dc.delta_h;
    r.cur_dv = dc.delta_v;
    dim3 block(32, 8), grid((W + 31) / 32, (H + 7) / 8);
    k_temporal<<<grid, block, 0, stream>>>(rgb, prev, (const float4*)gbuf, W, H, r, alpha);
    add_launches(1);
    CPT_CUDA(cudaGetLastError());
    return CPT_OK;
}

}  // namespace cpt

// kpcn.cu — kernel-predicting denoiser (KPCN, Bako et al. 2017) with a 5-level U-Net
// (32-64-96-128-160 channels, two 3x3 convolutions per level, 2x2 average pooling, nearest 2x
// upsampling with skip concatenation) predicting a 5x5 filter per pixel that is applied to the
// noisy radiance.  Training and inference run on this file's kernels only:
//
//   convolutions   implicit GEMM on the BF16 tensor cores (mma.sync m16n8k16, FP32 accumulate):
//                  forward (+bias, ReLU), input gradient (the same kernel on the output gradient
//                  with the taps flipped), weight gradient (pixel-split GEMM with a fixed-order
//                  reduction of the partial sums, so gradients are deterministic)
//   pooling / upsampling / concatenation   channel-sliced NHWC views, no copies
//   kernel apply   softmax over 25 logits, weighted 5x5 gather of the noisy radiance, and its
//                  gradient
//   loss           L1 between sqrt(x + 1e-3) of the output and of the target (the display
//                  transform the RMSE is measured in), mean over pixels
//   optimiser      Adam on FP32 master weights; BF16 weight copies are refreshed each step
//
// Activations are NHWC BF16 with an explicit channel stride and offset (a view), so a skip
// connection is written by its producer straight into its slice of the decoder's concatenation
// buffer.  Gradients of activations are FP32.  Images are padded to multiples of 16 (four
// poolings); the feature kernel writes zeros in the padding and the kernel apply clamps its
// gather to the real image.
//
// Input features (11 channels, padded to 32 with zeros): log(1 + radiance) (3), albedo (3),
// octahedral normal (2), depth / (1 + depth) (1, 1 on a miss), the 3x3 variance of
// log(1 + luminance) around the pixel (1), and log(1 + the standard deviation of the pixel mean's
// luminance) from the renderer's own samples (G-buffer channel 7) (1).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cpt_internal.h"

namespace cpt {
namespace kpcn {

constexpr int KSIZE = 5;           // predicted filter: 5 x 5
constexpr int KTAPS = KSIZE * KSIZE;
constexpr int IN_CH = 32;          // input features padded from 11 to 32 channels
constexpr int OUT_CH = 32;         // logits padded from 25 to 32 channels
constexpr int NUM_FEATURES = 11;   // written by k_features; the rest of IN_CH is zero
static_assert(NUM_FEATURES <= IN_CH && IN_CH % 32 == 0, "feature padding");

struct View {                      // NHWC tensor slice: element (p, c) at ptr[p * cs + co + c]
    void* ptr;
    int cs, co, C;
};

struct ConvSpec {
    int cin, cout;
    bool relu;
};

// Encoder c0a..c4b, decoder d3a..d0b, output.  Decoder inputs are [upsampled | skip].
constexpr int NCONV = 19;
constexpr ConvSpec SPECS[NCONV] = {
    {IN_CH, 32, true}, {32, 32, true},       // level 0
    {32, 64, true},    {64, 64, true},       // level 1
    {64, 96, true},    {96, 96, true},       // level 2
    {96, 128, true},   {128, 128, true},     // level 3
    {128, 160, true},  {160, 160, true},     // level 4
    {288, 128, true},  {128, 128, true},     // d3: [up(160) | skip(128)]
    {224, 96, true},   {96, 96, true},       // d2: [up(128) | skip(96)]
    {160, 64, true},   {64, 64, true},       // d1: [up(96) | skip(64)]
    {96, 32, true},    {32, 32, true},       // d0: [up(64) | skip(32)]
    {32, OUT_CH, false},                     // logits
};

// ------------------------------------------------------------------ tensor-core MMA
__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return __ldg(reinterpret_cast<const unsigned int*>(p)); }

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

struct Geo {
    int N, H, W;   // padded image size; pixels p = (n * H + y) * W + x
};

// 3x3 convolution, stride 1, zero padding, as an implicit GEMM: rows = pixels, columns = output
// channels, K = 9 taps x input channels.  One warp computes 16 pixels x (8 * NT) channels,
// loading its A (activations) and B (weights, [tap][cout][cin]) fragments directly from global
// memory (L1/L2 serve the re-reads).  out32 (optional) receives FP32 values (stored, or added
// when accumulate); out16 (optional) receives BF16 values after bias and ReLU.
template <int NT>
__global__ void __launch_bounds__(128) k_conv3x3(Geo g, View in, const __nv_bfloat16* __restrict__ w,
                                                 const float* __restrict__ bias, int cout, bool relu, View out16,
                                                 View out32, bool accumulate)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gq = lane >> 2, tq = lane & 3;
    const long P = (long)g.N * g.H * g.W;
    const long tile = (long)blockIdx.x * 4 + warp;
    const long p0 = tile * 16 + gq, p1 = p0 + 8;
    if (tile * 16 >= P) return;
    const int n_base = blockIdx.y * 8 * NT;
    // pixel coordinates of the two rows this lane loads
    const int x0 = (int)(p0 % g.W), y0 = (int)((p0 / g.W) % g.H);
    const int x1 = (int)(p1 % g.W), y1 = (int)((p1 / g.W) % g.H);
    const __nv_bfloat16* inp = reinterpret_cast<const __nv_bfloat16*>(in.ptr);
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int cin = in.C;
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        const bool v0 = p0 < P && (unsigned)(y0 + dy) < (unsigned)g.H && (unsigned)(x0 + dx) < (unsigned)g.W;
        const bool v1 = p1 < P && (unsigned)(y1 + dy) < (unsigned)g.H && (unsigned)(x1 + dx) < (unsigned)g.W;
        const long q0 = p0 + (long)dy * g.W + dx, q1 = p1 + (long)dy * g.W + dx;
        const __nv_bfloat16* r0 = inp + q0 * in.cs + in.co;
        const __nv_bfloat16* r1 = inp + q1 * in.cs + in.co;
        const __nv_bfloat16* wt = w + (size_t)tap * cout * cin;
        for (int k = 0; k < cin; k += 16) {
            const uint32_t a0 = v0 ? ld32(r0 + k + 2 * tq) : 0u;
            const uint32_t a1 = v1 ? ld32(r1 + k + 2 * tq) : 0u;
            const uint32_t a2 = v0 ? ld32(r0 + k + 8 + 2 * tq) : 0u;
            const uint32_t a3 = v1 ? ld32(r1 + k + 8 + 2 * tq) : 0u;
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                const __nv_bfloat16* wr = wt + (size_t)(n_base + 8 * j + gq) * cin + k;
                mma_bf16(acc[j], a0, a1, a2, a3, ld32(wr + 2 * tq), ld32(wr + 8 + 2 * tq));
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int c = n_base + 8 * j + 2 * tq;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const long p = h ? p1 : p0;
            if (p >= P) continue;
            float v0 = acc[j][2 * h], v1 = acc[j][2 * h + 1];
            if (bias) {
                v0 += bias[c];
                v1 += bias[c + 1];
            }
            if (out32.ptr) {
                float* o = reinterpret_cast<float*>(out32.ptr) + p * out32.cs + out32.co + c;
                if (accumulate) {
                    o[0] += v0;
                    o[1] += v1;
                } else {
                    o[0] = v0;
                    o[1] = v1;
                }
            }
            if (out16.ptr) {
                if (relu) {
                    v0 = fmaxf(v0, 0.f);
                    v1 = fmaxf(v1, 0.f);
                }
                __nv_bfloat16* o = reinterpret_cast<__nv_bfloat16*>(out16.ptr) + p * out16.cs + out16.co + c;
                *reinterpret_cast<unsigned int*>(o) = pack_bf16(__float2bfloat16_rn(v0), __float2bfloat16_rn(v1));
            }
        }
    }
}

}  // namespace kpcn
}  // namespace cpt

#include "kpcn_tc.cuh"

namespace cpt {
namespace kpcn {

// Weight gradient of a 3x3 convolution: dW[tap][ci][co] = sum_p X[p + off(tap), ci] dZ[p, co].
// Block (128 threads) = one tap, a 32 x 32 (ci, co) tile, and one chunk of pixels; the chunk is
// staged in shared memory 64 pixels at a time and multiplied on the tensor cores (warp w owns
// ci rows 16 (w / 2) and co columns 16 (w % 2)).  Partial sums go to part[chunk][tap][ci][co]
// and are added in chunk order by k_wgrad_reduce.  The centre-tap blocks of the first ci tile
// also sum their dZ columns into bpart[chunk][co] (the bias gradient's partial sums).
constexpr int WG_PIX = 64;
constexpr int WG_CHUNKS = 256;  // pixel chunks (blocks along z) per weight gradient
__global__ void __launch_bounds__(128) k_wgrad(Geo g, View x, View dz, int cin, int cout, long chunk_pixels,
                                               float* __restrict__ part, float* __restrict__ bpart)
{
    __shared__ __nv_bfloat16 xs[WG_PIX][32 + 8];
    __shared__ __nv_bfloat16 zs[WG_PIX][32 + 8];
    const int tap = blockIdx.y % 9;
    const int co_t = blockIdx.y / 9;
    const int ci_t = blockIdx.x;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const long P = (long)g.N * g.H * g.W;
    const long pbeg = (long)blockIdx.z * chunk_pixels, pend = min(P, pbeg + chunk_pixels);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gq = lane >> 2, tq = lane & 3;
    const int mrow = (warp >> 1) * 16, ncol = (warp & 1) * 16;
    const __nv_bfloat16* xp = reinterpret_cast<const __nv_bfloat16*>(x.ptr);
    const __nv_bfloat16* zp = reinterpret_cast<const __nv_bfloat16*>(dz.ptr);
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    const bool bias_block = tap == 4 && ci_t == 0;
    float bsum = 0.f;
    for (long pb = pbeg; pb < pend; pb += WG_PIX) {
        // stage: 64 pixels x 32 channels of X (shifted by the tap) and of dZ; 2 channels per load
        for (int e = threadIdx.x; e < WG_PIX * 16; e += 128) {
            const int r = e >> 4, c2 = (e & 15) * 2;
            const long p = pb + r;
            uint32_t xv = 0u, zv = 0u;
            if (p < pend) {
                const int px = (int)(p % g.W), py = (int)((p / g.W) % g.H);
                const int ci = ci_t * 32 + c2, co = co_t * 32 + c2;
                if ((unsigned)(py + dy) < (unsigned)g.H && (unsigned)(px + dx) < (unsigned)g.W && ci < cin)
                    xv = ld32(xp + (p + (long)dy * g.W + dx) * x.cs + x.co + ci);
                if (co < cout) zv = ld32(zp + p * dz.cs + dz.co + co);
            }
            *reinterpret_cast<uint32_t*>(&xs[r][c2]) = xv;
            *reinterpret_cast<uint32_t*>(&zs[r][c2]) = zv;
        }
        __syncthreads();
        if (bias_block && threadIdx.x < 32)
            for (int r = 0; r < WG_PIX; ++r) bsum += __bfloat162float(zs[r][threadIdx.x]);
#pragma unroll
        for (int kk = 0; kk < WG_PIX; kk += 16) {
            // A = X^T (rows ci, K = pixels); B = dZ (K = pixels, columns co)
            const int m0 = mrow + gq, k0 = kk + 2 * tq;
            const uint32_t a0 = pack_bf16(xs[k0][m0], xs[k0 + 1][m0]);
            const uint32_t a1 = pack_bf16(xs[k0][m0 + 8], xs[k0 + 1][m0 + 8]);
            const uint32_t a2 = pack_bf16(xs[k0 + 8][m0], xs[k0 + 9][m0]);
            const uint32_t a3 = pack_bf16(xs[k0 + 8][m0 + 8], xs[k0 + 9][m0 + 8]);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int n0 = ncol + 8 * j + gq;
                const uint32_t b0 = pack_bf16(zs[k0][n0], zs[k0 + 1][n0]);
                const uint32_t b1 = pack_bf16(zs[k0 + 8][n0], zs[k0 + 9][n0]);
                mma_bf16(acc[j], a0, a1, a2, a3, b0, b1);
            }
        }
        __syncthreads();
    }
    if (bias_block && threadIdx.x < 32 && co_t * 32 + (int)threadIdx.x < cout)
        bpart[(size_t)blockIdx.z * cout + co_t * 32 + threadIdx.x] = bsum;
    float* out = part + ((size_t)blockIdx.z * 9 + tap) * cin * cout;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int co = co_t * 32 + ncol + 8 * j + 2 * tq;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int ci = ci_t * 32 + mrow + gq + 8 * h;
            if (ci < cin && co < cout) {
                out[(size_t)ci * cout + co] = acc[j][2 * h];
                out[(size_t)ci * cout + co + 1] = acc[j][2 * h + 1];
            }
        }
    }
}

// grad[i] = sum over chunks of part[chunk][i] in a fixed order: a block of 256 threads covers 32
// consecutive i; its 8 warps sum chunks w, w + 8, ... and the 8 partial sums are added in order.
__global__ void k_wgrad_reduce(const float* __restrict__ part, int chunks, size_t n, float* __restrict__ grad)
{
    __shared__ float red[8][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (size_t i0 = (size_t)blockIdx.x * 32; i0 < n; i0 += (size_t)gridDim.x * 32) {
        const size_t i = i0 + lane;
        float s = 0.f;
        if (i < n)
            for (int c = w; c < chunks; c += 8) s += part[(size_t)c * n + i];
        red[w][lane] = s;
        __syncthreads();
        if (w == 0 && i < n) {
            float t = 0.f;
#pragma unroll
            for (int k = 0; k < 8; ++k) t += red[k][lane];
            grad[i] = t;
        }
        __syncthreads();
    }
}

// dZ = dA * (A > 0) (ReLU backward) as BF16; without relu the gradient is converted only
// dZ (BF16) = FP32 gradient, zeroed where the ReLU's output was not positive; 8 channels per item
// (16- and 32-byte accesses; channel counts, strides and offsets are multiples of 8).
__global__ void k_relu_back(View g32, View act, long P, int C, bool relu, View dz)
{
    const int C8 = C / 8;
    const long n = P * C8;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const long p = i / C8;
        const int c = (int)(i - p * C8) * 8;
        const float4* gp = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(g32.ptr) + p * g32.cs + g32.co + c);
        const float4 u = gp[0], w = gp[1];
        float v[8] = {u.x, u.y, u.z, u.w, w.x, w.y, w.z, w.w};
        if (relu) {
            const uint4 a = *reinterpret_cast<const uint4*>(reinterpret_cast<const __nv_bfloat16*>(act.ptr) + p * act.cs + act.co + c);
            const __nv_bfloat162* ah = reinterpret_cast<const __nv_bfloat162*>(&a);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(ah[j]);
                if (f.x <= 0.f) v[2 * j] = 0.f;
                if (f.y <= 0.f) v[2 * j + 1] = 0.f;
            }
        }
        uint4 o;
        __nv_bfloat162* oh = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
        for (int j = 0; j < 4; ++j) oh[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(dz.ptr) + p * dz.cs + dz.co + c) = o;
    }
}

// 2x2 average pooling (fine geometry g) and its gradient (added into the fine gradient view)
// 2x2 average pooling and nearest 2x upsampling over NHWC views, one coarse pixel x 8 channels
// (BF16, 16-byte accesses) or x 4 channels (FP32 gradients, 16-byte accesses) per work item; channel
// counts, strides and offsets of the views are multiples of 8 (BF16) / 4 (FP32).
__device__ __forceinline__ void coarse_pixel(long q, int Wc, int Hc, int& x, int& y, long& b)
{
    x = (int)(q % Wc);
    const long r = q / Wc;
    y = (int)(r % Hc);
    b = r / Hc;
}

__global__ void k_pool(Geo g, View in, View out)
{
    const int Ho = g.H / 2, Wo = g.W / 2, C8 = in.C / 8;
    const long n = (long)g.N * Ho * Wo * C8;
    const __nv_bfloat16* ip = reinterpret_cast<const __nv_bfloat16*>(in.ptr);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C8) * 8;
        const long q = i / C8;
        int x, y;
        long b;
        coarse_pixel(q, Wo, Ho, x, y, b);
        const long p00 = (b * g.H + 2 * y) * g.W + 2 * x;
        const long src[4] = {p00, p00 + 1, p00 + g.W, p00 + g.W + 1};
        float s[8] = {};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint4 v = *reinterpret_cast<const uint4*>(ip + src[k] * in.cs + in.co + c);
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(h[j]);
                s[2 * j] += f.x;
                s[2 * j + 1] += f.y;
            }
        }
        uint4 o;
        __nv_bfloat162* oh = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
        for (int j = 0; j < 4; ++j) oh[j] = __floats2bfloat162_rn(0.25f * s[2 * j], 0.25f * s[2 * j + 1]);
        *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out.ptr) + q * out.cs + out.co + c) = o;
    }
}

// gin (fine, FP32) += gradient of the average pool: a quarter of the coarse gradient on each of the
// four fine pixels
__global__ void k_pool_back(Geo g, View gout, View gin)
{
    const int Ho = g.H / 2, Wo = g.W / 2, C4 = gin.C / 4;
    const long n = (long)g.N * Ho * Wo * C4;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C4) * 4;
        const long q = i / C4;
        int x, y;
        long b;
        coarse_pixel(q, Wo, Ho, x, y, b);
        const float4 gq = *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(gout.ptr) + q * gout.cs + gout.co + c);
        const long p00 = (b * g.H + 2 * y) * g.W + 2 * x;
        const long dst[4] = {p00, p00 + 1, p00 + g.W, p00 + g.W + 1};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float4* d = reinterpret_cast<float4*>(reinterpret_cast<float*>(gin.ptr) + dst[k] * gin.cs + gin.co + c);
            float4 v = *d;
            v.x += 0.25f * gq.x;
            v.y += 0.25f * gq.y;
            v.z += 0.25f * gq.z;
            v.w += 0.25f * gq.w;
            *d = v;
        }
    }
}

// nearest 2x upsampling from the coarse geometry gc into the fine view, and its gradient
__global__ void k_upsample(Geo gc, View in, View out)
{
    const int C8 = in.C / 8, Wf = gc.W * 2;
    const long n = (long)gc.N * gc.H * gc.W * C8;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C8) * 8;
        const long q = i / C8;
        int x, y;
        long b;
        coarse_pixel(q, gc.W, gc.H, x, y, b);
        const uint4 v = *reinterpret_cast<const uint4*>(reinterpret_cast<const __nv_bfloat16*>(in.ptr) + q * in.cs + in.co + c);
        const long p00 = (b * gc.H * 2 + 2 * y) * Wf + 2 * x;
        const long dst[4] = {p00, p00 + 1, p00 + Wf, p00 + Wf + 1};
#pragma unroll
        for (int k = 0; k < 4; ++k)
            *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out.ptr) + dst[k] * out.cs + out.co + c) = v;
    }
}

__global__ void k_upsample_back(Geo gc, View gout, View gin)
{
    const int C4 = gin.C / 4, Wf = gc.W * 2;
    const long n = (long)gc.N * gc.H * gc.W * C4;
    const float* gp = reinterpret_cast<const float*>(gout.ptr);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C4) * 4;
        const long q = i / C4;
        int x, y;
        long b;
        coarse_pixel(q, gc.W, gc.H, x, y, b);
        const long p00 = (b * gc.H * 2 + 2 * y) * Wf + 2 * x;
        const long src[4] = {p00, p00 + 1, p00 + Wf, p00 + Wf + 1};
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 v = *reinterpret_cast<const float4*>(gp + src[k] * gout.cs + gout.co + c);
            s.x += v.x;
            s.y += v.y;
            s.z += v.z;
            s.w += v.w;
        }
        *reinterpret_cast<float4*>(reinterpret_cast<float*>(gin.ptr) + q * gin.cs + gin.co + c) = s;
    }
}

// ------------------------------------------------------------------ features and kernel apply
__device__ __forceinline__ float log_lum(float3 c) { return log1pf(fmaxf(0.f, 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z)); }

// Images: rgb [N][Hr][Wr][3] f32, gbuf [N][Hr][Wr][8] f32 (renderer layout) -> features
// [N][H][W][IN_CH] bf16 and radiance [N][H][W][3] f32 on the padded geometry g.
__global__ void k_features(Geo g, int Hr, int Wr, const float* __restrict__ rgb, const float* __restrict__ gbuf,
                           bool gbuf_aligned, __nv_bfloat16* __restrict__ feat, float* __restrict__ rad)
{
    const long P = (long)g.N * g.H * g.W;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
        const int x = (int)(p % g.W), y = (int)((p / g.W) % g.H), b = (int)(p / ((long)g.W * g.H));
        float f[IN_CH];
#pragma unroll
        for (int c = 0; c < IN_CH; ++c) f[c] = 0.f;
        float3 r = f3(0.f, 0.f, 0.f);
        if (x < Wr && y < Hr) {
            const size_t o = ((size_t)b * Hr + y) * Wr + x;
            r = f3(fmaxf(rgb[3 * o], 0.f), fmaxf(rgb[3 * o + 1], 0.f), fmaxf(rgb[3 * o + 2], 0.f));
            float4 g0, g1;
            if (gbuf_aligned) {
                g0 = __ldg(reinterpret_cast<const float4*>(gbuf + 8 * o));
                g1 = __ldg(reinterpret_cast<const float4*>(gbuf + 8 * o) + 1);
            } else {
                const float* gb = gbuf + 8 * o;
                g0 = make_float4(gb[0], gb[1], gb[2], gb[3]);
                g1 = make_float4(gb[4], gb[5], gb[6], gb[7]);
            }
            f[0] = log1pf(r.x);
            f[1] = log1pf(r.y);
            f[2] = log1pf(r.z);
            f[3] = g1.x;
            f[4] = g1.y;
            f[5] = g1.z;
            float nx = g0.x, ny = g0.y, nz = g0.z;
            const float l1 = fabsf(nx) + fabsf(ny) + fabsf(nz);
            if (l1 > 0.f) {
                nx /= l1;
                ny /= l1;
                if (nz < 0.f) {
                    const float ox = (1.f - fabsf(ny)) * (nx >= 0.f ? 1.f : -1.f);
                    const float oy = (1.f - fabsf(nx)) * (ny >= 0.f ? 1.f : -1.f);
                    nx = ox;
                    ny = oy;
                }
            }
            f[6] = nx;
            f[7] = ny;
            const float d = g0.w;
            f[8] = d >= CPT_INF_F ? 1.f : d / (1.f + d);
            // 3x3 variance, two-pass (no cancellation of m2 - m^2 in FP32)
            float l9[9], m = 0.f;
            for (int k = 0; k < 9; ++k) {
                const int xx = min(max(x + k % 3 - 1, 0), Wr - 1), yy = min(max(y + k / 3 - 1, 0), Hr - 1);
                const size_t q = ((size_t)b * Hr + yy) * Wr + xx;
                l9[k] = log_lum(f3(rgb[3 * q], rgb[3 * q + 1], rgb[3 * q + 2]));
                m += l9[k];
            }
            m /= 9.f;
            float var = 0.f;
            for (int k = 0; k < 9; ++k) var += (l9[k] - m) * (l9[k] - m);
            f[9] = var / 9.f;
            // standard deviation of the pixel mean (G-buffer channel 7: variance of its luminance)
            f[10] = log1pf(sqrtf(fmaxf(g1.w, 0.f)));
        }
        uint4* fo = reinterpret_cast<uint4*>(feat + p * IN_CH);
#pragma unroll
        for (int c = 0; c < IN_CH; c += 8)
            fo[c / 8] = make_uint4(pack_bf16(__float2bfloat16_rn(f[c]), __float2bfloat16_rn(f[c + 1])),
                                   pack_bf16(__float2bfloat16_rn(f[c + 2]), __float2bfloat16_rn(f[c + 3])),
                                   pack_bf16(__float2bfloat16_rn(f[c + 4]), __float2bfloat16_rn(f[c + 5])),
                                   pack_bf16(__float2bfloat16_rn(f[c + 6]), __float2bfloat16_rn(f[c + 7])));
        rad[3 * p] = r.x;
        rad[3 * p + 1] = r.y;
        rad[3 * p + 2] = r.z;
    }
}

// out = sum_k softmax(logits)_k * rad[neighbour k] (5x5, clamped to the real image Hr x Wr)
__global__ void k_apply(Geo g, int Hr, int Wr, const float* __restrict__ logits, const float* __restrict__ rad,
                        float* __restrict__ wts, float* __restrict__ out)
{
    const long P = (long)g.N * g.H * g.W;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
        const int x = (int)(p % g.W), y = (int)((p / g.W) % g.H), b = (int)(p / ((long)g.W * g.H));
        float lg[28];
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(logits + p * OUT_CH) + i);
            lg[4 * i] = v.x;
            lg[4 * i + 1] = v.y;
            lg[4 * i + 2] = v.z;
            lg[4 * i + 3] = v.w;
        }
        float mx = lg[0];
#pragma unroll
        for (int k = 1; k < KTAPS; ++k) mx = fmaxf(mx, lg[k]);
        float e[KTAPS], s = 0.f;
#pragma unroll
        for (int k = 0; k < KTAPS; ++k) {
            e[k] = expf(lg[k] - mx);
            s += e[k];
        }
        const float inv = 1.f / s;
        float3 acc = f3(0.f, 0.f, 0.f);
        const int xc = min(x, Wr - 1), yc = min(y, Hr - 1);
#pragma unroll
        for (int k = 0; k < KTAPS; ++k) {
            const float wk = e[k] * inv;
            if (wts) wts[p * KTAPS + k] = wk;
            const int xx = min(max(xc + k % KSIZE - KSIZE / 2, 0), Wr - 1);
            const int yy = min(max(yc + k / KSIZE - KSIZE / 2, 0), Hr - 1);
            const long q = ((long)b * g.H + yy) * g.W + xx;
            acc = acc + wk * f3(rad[3 * q], rad[3 * q + 1], rad[3 * q + 2]);
        }
        out[3 * p] = acc.x;
        out[3 * p + 1] = acc.y;
        out[3 * p + 2] = acc.z;
    }
}

// dlogit_k = w_k (dw_k - sum_j w_j dw_j), dw_k = <dout, rad[neighbour k]>; written as BF16 dZ of
// the output convolution (channels 25..31 zero)
__global__ void k_apply_back(Geo g, int Hr, int Wr, const float* __restrict__ wts, const float* __restrict__ rad,
                             const float* __restrict__ dout, __nv_bfloat16* __restrict__ dlogits)
{
    const long P = (long)g.N * g.H * g.W;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
        const int x = (int)(p % g.W), y = (int)((p / g.W) % g.H), b = (int)(p / ((long)g.W * g.H));
        const float3 go = f3(dout[3 * p], dout[3 * p + 1], dout[3 * p + 2]);
        const int xc = min(x, Wr - 1), yc = min(y, Hr - 1);
        float dw[KTAPS], dot = 0.f;
        for (int k = 0; k < KTAPS; ++k) {
            const int xx = min(max(xc + k % KSIZE - KSIZE / 2, 0), Wr - 1);
            const int yy = min(max(yc + k / KSIZE - KSIZE / 2, 0), Hr - 1);
            const long q = ((long)b * g.H + yy) * g.W + xx;
            dw[k] = dot3(go, f3(rad[3 * q], rad[3 * q + 1], rad[3 * q + 2]));
            dot += wts[p * KTAPS + k] * dw[k];
        }
        __nv_bfloat16* o = dlogits + p * OUT_CH;
        for (int k = 0; k < OUT_CH; ++k) {
            const float v = k < KTAPS ? wts[p * KTAPS + k] * (dw[k] - dot) : 0.f;
            o[k] = __float2bfloat16_rn(v);
        }
    }
}

// L1 of sqrt(x + LOSS_EPS) over the real pixels (the display transform of the evaluation, without
// its clamp); dout = d(mean loss)/d(out); per-block partial sums
constexpr float LOSS_EPS = 1e-3f;
__global__ void k_loss(Geo g, int Hr, int Wr, const float* __restrict__ out, const float* __restrict__ target,
                       float* __restrict__ dout, float* __restrict__ partial, float scale)
{
    __shared__ float red[256];
    const long P = (long)g.N * g.H * g.W;
    float s = 0.f;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
        const int x = (int)(p % g.W), y = (int)((p / g.W) % g.H), b = (int)(p / ((long)g.W * g.H));
        const bool real = x < Wr && y < Hr;
        for (int c = 0; c < 3; ++c) {
            float gr = 0.f;
            if (real) {
                const float o = out[3 * p + c];
                const float t = target[(((size_t)b * Hr + y) * Wr + x) * 3 + c];
                const float lo = sqrtf(fmaxf(o, 0.f) + LOSS_EPS), lt = sqrtf(fmaxf(t, 0.f) + LOSS_EPS);
                const float d = lo - lt;
                s += fabsf(d);
                gr = o > 0.f ? scale * (d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f)) * 0.5f / lo : 0.f;
            }
            dout[3 * p + c] = gr;
        }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// BF16 weight copies of every convolution: forward [tap][cout][cin]; input-gradient
// [tap][cin][cout] with the tap flipped (tap' = 8 - tap).  Master layout [tap][cin][cout].
__global__ void k_weight_copies(const float* __restrict__ w, int cin, int cout, __nv_bfloat16* __restrict__ wf,
                                __nv_bfloat16* __restrict__ wd)
{
    const size_t n = (size_t)9 * cin * cout;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int co = (int)(i % cout);
        const int ci = (int)((i / cout) % cin);
        const int tap = (int)(i / ((size_t)cout * cin));
        const __nv_bfloat16 v = __float2bfloat16_rn(w[i]);
        wf[((size_t)tap * cout + co) * cin + ci] = v;
        wd[((size_t)(8 - tap) * cin + ci) * cout + co] = v;
    }
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// copy of the real image out of the padded output
__global__ void k_crop(Geo g, int Hr, int Wr, const float* __restrict__ src, float* __restrict__ dst)
{
    const long n = (long)g.N * Hr * Wr;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int x = (int)(i % Wr), y = (int)((i / Wr) % Hr), b = (int)(i / ((long)Wr * Hr));
        const long p = ((long)b * g.H + y) * g.W + x;
        dst[3 * i] = src[3 * p];
        dst[3 * i + 1] = src[3 * p + 1];
        dst[3 * i + 2] = src[3 * p + 2];
    }
}

inline int grid_for(long n, int t = 256) { return (int)std::max<long>(1, std::min<long>((n + t - 1) / t, 152L * 16)); }

// ------------------------------------------------------------------ host side
inline View vw(void* p, int cs, int co, int C) { return View{p, cs, co, C}; }
inline View none() { return View{nullptr, 0, 0, 0}; }

struct Net {
    int device = 0;
    // parameters: per convolution W [9][cin][cout] then b [cout], all in one FP32 array
    size_t woff[NCONV], boff[NCONV], w16off[NCONV];
    size_t n_params = 0, n_w16 = 0;
    float *w = nullptr, *gw = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wf16 = nullptr, *wd16 = nullptr;
    long step = 0;
    bool copies_fresh = false;
    bool logits_stored = false;   // the last forward pass wrote n.logits (not the fused apply)
    // convolution engine: 0 = mma.sync kernel, 1 = tcgen05 kernel with cp.async copies, 2 = TMA-fed
    // warp-specialised persistent tcgen05 kernels (row tiles where the width allows, else im2col
    // tiles; k_conv3x3_tc where a TMA alignment rule fails)
    int backend = 2;
    int sm_count = 152;
    int ws_per_sm = 4;        // CTAs of k_conv3x3_ws per SM allowed by its registers and threads
    int ws_smem_max = 0;      // largest dynamic shared memory of one k_conv3x3_ws / _rows CTA
    int rows_apply_per_sm = 2;   // CTAs per SM of the row-tile kernel with the fused apply epilogue
    int* err = nullptr;
    // activations / gradients for the current geometry
    int N = 0, H = 0, W = 0;
    Geo geo[5];
    long P[5];
    char* arena = nullptr;
    size_t arena_bytes = 0;
    __nv_bfloat16 *X0, *A0a, *cat0, *p1, *A1a, *cat1, *p2, *A2a, *cat2, *p3, *A3a, *cat3, *p4, *A4a, *A4b;
    __nv_bfloat16 *D3a, *D3b, *D2a, *D2b, *D1a, *D1b, *D0a, *D0b, *dz[5];
    float *logits, *rad, *wts, *out, *dout, *loss_part;
    float *G_D0b, *G_D0a, *G_cat0, *G_D1b, *G_D1a, *G_cat1, *G_D2b, *G_D2a, *G_cat2, *G_D3b, *G_D3a, *G_cat3;
    float *G_A4b, *G_A4a, *G_p4, *G_A3a, *G_p3, *G_A2a, *G_p2, *G_A1a, *G_p1, *G_A0a;
    float* wpart = nullptr;
    float* bpart = nullptr;   // bias-gradient partial sums per pixel chunk

    ~Net()
    {
        cudaFree(arena);
        cudaFree(w);
        cudaFree(gw);
        cudaFree(m);
        cudaFree(v);
        cudaFree(wf16);
        cudaFree(wd16);
        cudaFree(err);
    }
};

cpt_status net_init(Net& n, uint64_t seed)
{
    size_t off = 0, o16 = 0;
    for (int i = 0; i < NCONV; ++i) {
        n.woff[i] = off;
        off += (size_t)9 * SPECS[i].cin * SPECS[i].cout;
        n.boff[i] = off;
        off += SPECS[i].cout;
        n.w16off[i] = o16;
        o16 += (size_t)9 * SPECS[i].cin * SPECS[i].cout;
    }
    n.n_params = off;
    n.n_w16 = o16;
    // He-normal weights from PCG32 (Box-Muller), zero biases; the logits layer starts small so
    // the first predicted kernels are close to a uniform 5x5 box
    std::vector<float> h(off, 0.f);
    uint64_t st = 0, inc = (seed << 1u) | 1u;
    auto next = [&]() {
        uint64_t old = st;
        st = old * CPT_PCG_MULT + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u), rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((0u - rot) & 31u));
    };
    next();
    st += 0x853c49e6748fea9bULL;
    next();
    for (int i = 0; i < NCONV; ++i) {
        const double stdv = std::sqrt(2.0 / (9.0 * SPECS[i].cin)) * (i == NCONV - 1 ? 0.1 : 1.0);
        const size_t cnt = (size_t)9 * SPECS[i].cin * SPECS[i].cout;
        for (size_t k = 0; k < cnt; ++k) {
            const double u1 = ((double)next() + 1.0) / 4294967296.0, u2 = (double)next() / 4294967296.0;
            h[n.woff[i] + k] = (float)(stdv * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    CPT_CUDA(cudaMalloc((void**)&n.w, off * sizeof(float)));
    CPT_CUDA(cudaMalloc((void**)&n.gw, off * sizeof(float)));
    CPT_CUDA(cudaMalloc((void**)&n.m, off * sizeof(float)));
    CPT_CUDA(cudaMalloc((void**)&n.v, off * sizeof(float)));
    CPT_CUDA(cudaMalloc((void**)&n.wf16, o16 * sizeof(__nv_bfloat16)));
    CPT_CUDA(cudaMalloc((void**)&n.wd16, o16 * sizeof(__nv_bfloat16)));
    CPT_CUDA(cudaMemcpy(n.w, h.data(), off * sizeof(float), cudaMemcpyHostToDevice));
    CPT_CUDA(cudaDeviceGetAttribute(&n.sm_count, cudaDevAttrMultiProcessorCount, n.device));
    CPT_CUDA(cudaMalloc((void**)&n.err, sizeof(int)));
    CPT_CUDA(cudaMemset(n.err, 0, sizeof(int)));
    CPT_CUDA(cudaFuncSetAttribute(k_conv3x3_tc<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_MAX));
    CPT_CUDA(cudaFuncSetAttribute(k_conv3x3_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_MAX));
    {
        int optin = 0;
        CPT_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, n.device));
        cudaFuncAttributes fa;
        CPT_CUDA(cudaFuncGetAttributes(&fa, k_conv3x3_ws<64>));
        cudaFuncAttributes fr;
        CPT_CUDA(cudaFuncGetAttributes(&fr, k_conv3x3_rows<64, false>));
        n.ws_smem_max = optin - (int)std::max(fa.sharedSizeBytes, fr.sharedSizeBytes);
        cudaFuncAttributes fapply;
        CPT_CUDA(cudaFuncGetAttributes(&fapply, k_conv3x3_rows<32, true>));
        n.ws_smem_max = std::min(n.ws_smem_max, optin - (int)fapply.sharedSizeBytes);
        CPT_CUDA(cudaFuncSetAttribute(k_conv3x3_rows<32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      n.ws_smem_max));
        CPT_CUDA(cudaFuncSetAttribute(k_conv3x3_rows<64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      n.ws_smem_max));
        CPT_CUDA(cudaFuncSetAttribute(k_conv3x3_rows<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      n.ws_smem_max));
        n.rows_apply_per_sm = std::max(1, std::min(2048 / 192, 65536 / (192 * std::max(1, (fapply.numRegs + 7) / 8 * 8))));
        CPT_CUDA(cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, WT_SMEM));
        CPT_CUDA(cudaFuncSetAttribute(k_conv3x3_ws<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, n.ws_smem_max));
        CPT_CUDA(cudaFuncSetAttribute(k_conv3x3_ws<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, n.ws_smem_max));
        // registers and threads: 65536 / (192 threads x registers rounded to 8 per thread)
        const int regs = std::max(1, (std::max(fa.numRegs, fr.numRegs) + 7) / 8 * 8);
        n.ws_per_sm = std::max(1, std::min(2048 / 192, 65536 / (192 * regs)));
    }
    CPT_CUDA(cudaMemset(n.gw, 0, off * sizeof(float)));
    CPT_CUDA(cudaMemset(n.m, 0, off * sizeof(float)));
    CPT_CUDA(cudaMemset(n.v, 0, off * sizeof(float)));
    n.copies_fresh = false;
    return CPT_OK;
}

cpt_status refresh_copies(Net& n, cudaStream_t s)
{
    if (n.copies_fresh) return CPT_OK;
    for (int i = 0; i < NCONV; ++i) {
        const size_t cnt = (size_t)9 * SPECS[i].cin * SPECS[i].cout;
        k_weight_copies<<<grid_for((long)cnt), 256, 0, s>>>(n.w + n.woff[i], SPECS[i].cin, SPECS[i].cout,
                                                            n.wf16 + n.w16off[i], n.wd16 + n.w16off[i]);
    }
    add_launches(NCONV);
    CPT_CUDA(cudaGetLastError());
    n.copies_fresh = true;
    return CPT_OK;
}

// (Re)allocates the activation arena for N images of H x W (multiples of 16).
cpt_status ensure_geometry(Net& n, int N, int H, int W)
{
    if (n.arena && n.N == N && n.H == H && n.W == W) return CPT_OK;
    cudaFree(n.arena);
    n.arena = nullptr;
    n.N = N;
    n.H = H;
    n.W = W;
    for (int l = 0; l < 5; ++l) {
        n.geo[l] = Geo{N, H >> l, W >> l};
        n.P[l] = (long)N * (H >> l) * (W >> l);
    }
    const long* P = n.P;
    struct Req {
        void** dst;
        size_t bytes;
    };
    std::vector<Req> reqs;
    auto b16 = [&](__nv_bfloat16** d, long px, int c) { reqs.push_back({(void**)d, (size_t)px * c * 2}); };
    auto f32 = [&](float** d, long cnt) { reqs.push_back({(void**)d, (size_t)cnt * 4}); };
    b16(&n.X0, P[0], IN_CH); b16(&n.A0a, P[0], 32); b16(&n.cat0, P[0], 96);
    b16(&n.p1, P[1], 32); b16(&n.A1a, P[1], 64); b16(&n.cat1, P[1], 160);
    b16(&n.p2, P[2], 64); b16(&n.A2a, P[2], 96); b16(&n.cat2, P[2], 224);
    b16(&n.p3, P[3], 96); b16(&n.A3a, P[3], 128); b16(&n.cat3, P[3], 288);
    b16(&n.p4, P[4], 128); b16(&n.A4a, P[4], 160); b16(&n.A4b, P[4], 160);
    b16(&n.D3a, P[3], 128); b16(&n.D3b, P[3], 128); b16(&n.D2a, P[2], 96); b16(&n.D2b, P[2], 96);
    b16(&n.D1a, P[1], 64); b16(&n.D1b, P[1], 64); b16(&n.D0a, P[0], 32); b16(&n.D0b, P[0], 32);
    const int dzc[5] = {32, 64, 96, 128, 160};
    for (int l = 0; l < 5; ++l) b16(&n.dz[l], P[l], dzc[l]);
    f32(&n.logits, P[0] * OUT_CH); f32(&n.rad, P[0] * 3); f32(&n.wts, P[0] * KTAPS); f32(&n.out, P[0] * 3);
    f32(&n.dout, P[0] * 3); f32(&n.loss_part, 152 * 16);
    f32(&n.G_D0b, P[0] * 32); f32(&n.G_D0a, P[0] * 32); f32(&n.G_cat0, P[0] * 96);
    f32(&n.G_D1b, P[1] * 64); f32(&n.G_D1a, P[1] * 64); f32(&n.G_cat1, P[1] * 160);
    f32(&n.G_D2b, P[2] * 96); f32(&n.G_D2a, P[2] * 96); f32(&n.G_cat2, P[2] * 224);
    f32(&n.G_D3b, P[3] * 128); f32(&n.G_D3a, P[3] * 128); f32(&n.G_cat3, P[3] * 288);
    f32(&n.G_A4b, P[4] * 160); f32(&n.G_A4a, P[4] * 160); f32(&n.G_p4, P[4] * 128);
    f32(&n.G_A3a, P[3] * 128); f32(&n.G_p3, P[3] * 96); f32(&n.G_A2a, P[2] * 96); f32(&n.G_p2, P[2] * 64);
    f32(&n.G_A1a, P[1] * 64); f32(&n.G_p1, P[1] * 32); f32(&n.G_A0a, P[0] * 32);
    // weight-gradient partial sums: at most WG_CHUNKS pixel chunks per layer
    size_t maxw = 0;
    for (int i = 0; i < NCONV; ++i) maxw = std::max(maxw, (size_t)9 * SPECS[i].cin * SPECS[i].cout);
    f32(&n.wpart, (long)(WG_CHUNKS * maxw));
    f32(&n.bpart, (long)WG_CHUNKS * 512);
    size_t total = 0;
    for (auto& r : reqs) total += align_up(r.bytes, 256);
    CPT_CUDA(cudaMalloc((void**)&n.arena, total));
    n.arena_bytes = total;
    char* p = n.arena;
    for (auto& r : reqs) {
        *r.dst = p;
        p += align_up(r.bytes, 256);
    }
    return CPT_OK;
}

// Driver entry points of the tensor-map encoders (resolved once through the runtime, so the
// library does not link libcuda directly); null when the driver does not provide them.
struct TmaEncoders {
    PFN_cuTensorMapEncodeIm2col_v12000 im2col = nullptr;
    PFN_cuTensorMapEncodeTiled_v12000 tiled = nullptr;
};

const TmaEncoders& tma_encoders()
{
    static const TmaEncoders enc = [] {
        TmaEncoders e;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeIm2col", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            e.im2col = reinterpret_cast<PFN_cuTensorMapEncodeIm2col_v12000>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            e.tiled = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        cudaGetLastError();
        return e;
    }();
    return enc;
}

// Tensor maps of k_conv3x3_ws: the input view as a {C, W, H, N} im2col tensor (window corners
// -1 .. -1: base pixel = output pixel - 1, tap offsets 0..2, zero fill outside the image), 128
// pixels x kc channels per load, and the weights [9 * cout][cin] as a tiled tensor with
// kc x n_tile boxes; swizzle 128 B (kc 64) or 64 B (kc 32), matching smem_desc_sw.  False when a
// TMA alignment rule does not hold (16-byte base addresses and strides) or the encoders are
// missing, and the caller uses the cp.async kernel instead.
bool tma_maps(const Geo& g, const View& in, const __nv_bfloat16* w, int cout, int kc, int nt, CUtensorMap& ta,
              CUtensorMap& tb)
{
    const TmaEncoders& e = tma_encoders();
    if (!e.im2col || !e.tiled) return false;
    const char* a = reinterpret_cast<const char*>(in.ptr) + (size_t)in.co * 2;
    if ((reinterpret_cast<uintptr_t>(a) & 15) || (in.cs * 2) % 16 || (reinterpret_cast<uintptr_t>(w) & 15) ||
        (in.C * 2) % 16 || in.C % kc || nt % 16 || nt > 256)
        return false;
    const CUtensorMapSwizzle sw = kc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
    const cuuint64_t rs = (cuuint64_t)in.cs * 2;
    const cuuint64_t adim[4] = {(cuuint64_t)in.C, (cuuint64_t)g.W, (cuuint64_t)g.H, (cuuint64_t)g.N};
    const cuuint64_t astr[3] = {rs, rs * g.W, rs * g.W * g.H};
    const int lo[2] = {-1, -1}, hi[2] = {-1, -1};
    const cuuint32_t one[4] = {1, 1, 1, 1};
    if (e.im2col(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<char*>(a), adim, astr, lo, hi, (cuuint32_t)kc,
                 (cuuint32_t)TC_M, one, CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const cuuint64_t bdim[2] = {(cuuint64_t)in.C, (cuuint64_t)9 * cout};
    const cuuint64_t bstr[1] = {(cuuint64_t)in.C * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kc, (cuuint32_t)nt};
    return e.tiled(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(w), bdim, bstr, box, one,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of k_conv3x3_rows: the input view as a tiled {C, W, H, N} tensor with kc x 130 x 3
// x 1 boxes (a row tile with its halo; pixels outside the image read as zeros) and the weights
// [9 * cout][cin] with kc x n_tile boxes, both with the kc * 2-byte swizzle.
bool row_maps(const Geo& g, const View& in, const __nv_bfloat16* w, int cout, int kc, int nt, bool pitched,
              CUtensorMap& ta, CUtensorMap& tb)
{
    const TmaEncoders& e = tma_encoders();
    if (!e.tiled || !e.im2col) return false;
    const char* a = reinterpret_cast<const char*>(in.ptr) + (size_t)in.co * 2;
    if ((reinterpret_cast<uintptr_t>(a) & 15) || (in.cs * 2) % 16 || (reinterpret_cast<uintptr_t>(w) & 15) ||
        in.C % kc || nt % 16 || nt > 256 || (!pitched && g.W % TC_M))
        return false;
    const CUtensorMapSwizzle sw = kc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
    const cuuint64_t rs = (cuuint64_t)in.cs * 2;
    const cuuint64_t adim[4] = {(cuuint64_t)in.C, (cuuint64_t)g.W, (cuuint64_t)g.H, (cuuint64_t)g.N};
    const cuuint64_t astr[3] = {rs, rs * g.W, rs * g.W * g.H};
    const cuuint32_t abox[4] = {(cuuint32_t)kc, (cuuint32_t)ROW_PIX, 3, 1};
    const cuuint32_t one[4] = {1, 1, 1, 1};
    // pitched: base positions x in [-1, W - 1] (W + 1 per row: lower corner -1, upper corner 0),
    // y in [-1, H - 2]; corners listed W first, like the dimensions
    const int lo[2] = {-1, -1}, hi[2] = {0, -1};
    const CUresult ra =
        pitched ? e.im2col(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<char*>(a), adim, astr, lo, hi,
                           (cuuint32_t)kc, (cuuint32_t)ROW_PIX, one, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE)
                : e.tiled(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<char*>(a), adim, astr, abox, one,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (ra != CUDA_SUCCESS) return false;
    const cuuint64_t bdim[2] = {(cuuint64_t)in.C, (cuuint64_t)9 * cout};
    const cuuint64_t bstr[1] = {(cuuint64_t)in.C * 2};
    const cuuint32_t bbox[2] = {(cuuint32_t)kc, (cuuint32_t)nt};
    return e.tiled(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(w), bdim, bstr, bbox, one,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// tcgen05 convolution: cout split into grid.y tiles of at most 256 channels (multiples of 16).
// With ap (the logits layer at inference, cout == 32) the row-tile kernel applies the predicted
// kernels in its epilogue instead of storing the logits; returns whether it did.
bool conv_tc(Net& n, const __nv_bfloat16* w, const float* bias, int cout, bool relu, const Geo& g, View in, View out16,
             View out32, cudaStream_t s, const ApplyArgs* ap = nullptr)
{
    const long P = (long)g.N * g.H * g.W;
    const int tiles = (cout + 255) / 256;
    const int nt = cout / tiles;
    int ncols = 32;
    while (ncols < nt) ncols <<= 1;
    const int kc = in.C % 64 == 0 ? 64 : 32;
    CUtensorMap ta, tb;
    // row tiles: halo-reusing activation boxes (tiled when W % 128 == 0, else im2col over the W + 1
    // pitch), weights resident when they fit next to two stages, else streamed with each stage
    RowPlan rp;
    rp.pitched = g.W % TC_M != 0;
    rp.a_seg = rp.pitched ? (ROW_PIX * kc * 2 + 1023) / 1024 * 1024 : ROW_PIX * kc * 2;
    rp.a_region = (3 * rp.a_seg + 1023) / 1024 * 1024;
    const int b_all = row_b_bytes(in.C, nt, kc), b_stage = 9 * nt * kc * 2;
    rp.resident = b_all + 2 * rp.a_region + 1024 <= n.ws_smem_max;
    rp.stage = rp.a_region + (rp.resident ? 0 : b_stage);
    const int b_bytes = rp.resident ? b_all : 0;
    if (n.backend == 2 && b_bytes + 2 * rp.stage + 1024 <= n.ws_smem_max &&
        row_maps(g, in, w, cout, kc, nt, rp.pitched, ta, tb)) {
        const int max_ctas = 512 / (2 * ncols);
        const int per_sm = std::max(1, std::min({max_ctas, n.ws_per_sm, TC_SM_SMEM / (b_bytes + 2 * rp.stage + 3072)}));
        const int share = std::min(TC_SM_SMEM / per_sm - 2048, n.ws_smem_max) - 1024;
        const int nst = std::max(2, std::min(TC_WS_STAGES, (share - b_bytes) / rp.stage));
        const int smem = std::max(b_bytes + nst * rp.stage + 1024, TC_SM_SMEM / (max_ctas + 1) + 1024);
        const long q = (long)g.N * g.H * (rp.pitched ? g.W + 1 : g.W);
        const long m_tiles = (q + TC_M - 1) / TC_M;
        dim3 grid((unsigned)std::min<long>(m_tiles, (long)per_sm * n.sm_count), (unsigned)tiles);
        if (ap && cout == 32 && bias && kc == 32) {
            // the apply epilogue needs more registers: its own CTAs-per-SM limit
            const int ps = std::max(1, std::min(per_sm, n.rows_apply_per_sm));
            dim3 ga((unsigned)std::min<long>(m_tiles, (long)ps * n.sm_count), 1u);
            k_conv3x3_rows<32, true><<<ga, 192, smem, s>>>(ta, tb, g, in.C, bias, cout, nt, ncols, nst, rp, *ap, relu,
                                                          out16, out32, n.err);
            return true;
        }
        const ApplyArgs none_ap{nullptr, nullptr, 0, 0};
        if (kc == 64)
            k_conv3x3_rows<64, false><<<grid, 192, smem, s>>>(ta, tb, g, in.C, bias, cout, nt, ncols, nst, rp, none_ap,
                                                              relu, out16, out32, n.err);
        else
            k_conv3x3_rows<32, false><<<grid, 192, smem, s>>>(ta, tb, g, in.C, bias, cout, nt, ncols, nst, rp, none_ap,
                                                              relu, out16, out32, n.err);
        return false;
    }
    if (n.backend == 2 && tma_maps(g, in, w, cout, kc, nt, ta, tb)) {
        // warp-specialised persistent kernel fed by TMA, two accumulators per CTA: per_sm CTAs per
        // SM (tensor memory: 2 * ncols columns each), each with as many stages as its share of the
        // SM's shared memory holds (2 .. TC_WS_STAGES)
        const int max_ctas = 512 / (2 * ncols);
        const int stage = tc_stage_bytes(kc, nt);
        const int per_sm = std::max(1, std::min({max_ctas, n.ws_per_sm, TC_SM_SMEM / (2 * stage + 3072)}));
        const int share = std::min(TC_SM_SMEM / per_sm - 2048, n.ws_smem_max) - 1024;
        const int nst = std::max(2, std::min(TC_WS_STAGES, share / stage));
        // at most max_ctas CTAs of this launch fit on an SM, whatever the occupancy calculator says
        const int smem = std::max(nst * stage + 1024, TC_SM_SMEM / (max_ctas + 1) + 1024);
        const long m_tiles = (P + TC_M - 1) / TC_M;
        dim3 grid((unsigned)std::min<long>(m_tiles, (long)per_sm * n.sm_count), (unsigned)tiles);
        if (kc == 64)
            k_conv3x3_ws<64><<<grid, 192, smem, s>>>(ta, tb, g, in.C, bias, cout, nt, ncols, nst, relu, out16, out32,
                                                     n.err);
        else
            k_conv3x3_ws<32><<<grid, 192, smem, s>>>(ta, tb, g, in.C, bias, cout, nt, ncols, nst, relu, out16, out32,
                                                     n.err);
        return false;
    }
    // shared memory large enough that at most 512 / ncols CTAs fit on an SM (tensor memory)
    const int max_ctas = 512 / ncols;
    const int smem = std::max(tc_smem_bytes(kc, nt), TC_SM_SMEM / (max_ctas + 1) + 1024);
    dim3 grid((unsigned)((P + TC_M - 1) / TC_M), (unsigned)tiles);
    if (kc == 64)
        k_conv3x3_tc<64><<<grid, 128, smem, s>>>(g, in, w, bias, cout, nt, ncols, relu, out16, out32, n.err);
    else
        k_conv3x3_tc<32><<<grid, 128, smem, s>>>(g, in, w, bias, cout, nt, ncols, relu, out16, out32, n.err);
    return false;
}

// Forward convolution of layer i; with ap, returns true when the kernel apply was fused into it
// (conv_tc), false when the caller still has to run k_apply.
bool conv(Net& n, int i, const Geo& g, View in, View out16, View out32, cudaStream_t s, const ApplyArgs* ap = nullptr)
{
    const ConvSpec& c = SPECS[i];
    in.C = c.cin;
    if (n.backend >= 1) return conv_tc(n, n.wf16 + n.w16off[i], n.w + n.boff[i], c.cout, c.relu, g, in, out16, out32, s, ap);
    const long P = (long)g.N * g.H * g.W;
    dim3 grid((unsigned)(((P + 15) / 16 + 3) / 4), (unsigned)(c.cout / 32));
    k_conv3x3<4><<<grid, 128, 0, s>>>(g, in, n.wf16 + n.w16off[i], n.w + n.boff[i], c.cout, c.relu, out16, out32,
                                      false);
    return false;
}

// input gradient: G (FP32, stored or added) = conv(dZ, flipped weights)
void dgrad(Net& n, int i, const Geo& g, View dz, View gin, cudaStream_t s)
{
    const ConvSpec& c = SPECS[i];
    dz.C = c.cout;
    if (n.backend >= 1) {
        conv_tc(n, n.wd16 + n.w16off[i], nullptr, c.cin, false, g, dz, none(), gin, s);
        return;
    }
    const long P = (long)g.N * g.H * g.W;
    dim3 grid((unsigned)(((P + 15) / 16 + 3) / 4), (unsigned)(c.cin / 32));
    k_conv3x3<4><<<grid, 128, 0, s>>>(g, dz, n.wd16 + n.w16off[i], nullptr, c.cin, false, none(), gin, false);
}

// Tensor maps of k_wgrad_tc: X as an im2col {cin, W, H, N} tensor (64 channels x 64 pixels per
// load, window corners -1 .. -1) and dZ as a 2D {cout, P} tensor (64 x 64 boxes), 128-byte swizzle.
bool wgrad_maps(const Geo& g, const View& x, const View& dz, CUtensorMap& tx, CUtensorMap& tz)
{
    const TmaEncoders& e = tma_encoders();
    if (!e.im2col || !e.tiled) return false;
    const char* xa = reinterpret_cast<const char*>(x.ptr) + (size_t)x.co * 2;
    const char* za = reinterpret_cast<const char*>(dz.ptr) + (size_t)dz.co * 2;
    if ((reinterpret_cast<uintptr_t>(xa) & 15) || (reinterpret_cast<uintptr_t>(za) & 15) || (x.cs * 2) % 16 ||
        (dz.cs * 2) % 16 || x.C % 32 || dz.C % 32)
        return false;
    const cuuint64_t rs = (cuuint64_t)x.cs * 2;
    const cuuint64_t xdim[4] = {(cuuint64_t)x.C, (cuuint64_t)g.W, (cuuint64_t)g.H, (cuuint64_t)g.N};
    const cuuint64_t xstr[3] = {rs, rs * g.W, rs * g.W * g.H};
    const int lo[2] = {-1, -1}, hi[2] = {-1, -1};
    const cuuint32_t one[4] = {1, 1, 1, 1};
    if (e.im2col(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<char*>(xa), xdim, xstr, lo, hi, 64,
                 (cuuint32_t)WT_PIX, one, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const cuuint64_t zdim[2] = {(cuuint64_t)dz.C, (cuuint64_t)g.N * g.H * g.W};
    const cuuint64_t zstr[1] = {(cuuint64_t)dz.cs * 2};
    const cuuint32_t zbox[2] = {64, (cuuint32_t)WT_PIX};
    return e.tiled(&tz, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<char*>(za), zdim, zstr, zbox, one,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

void wgrad(Net& n, int i, const Geo& g, View x, View dz, cudaStream_t s)
{
    const ConvSpec& c = SPECS[i];
    const long P = (long)g.N * g.H * g.W;
    x.C = c.cin;
    dz.C = c.cout;
    CUtensorMap tx, tz;
    if (n.backend == 2 && wgrad_maps(g, x, dz, tx, tz)) {
        // tcgen05: grid = pixel chunks x (3 tap rows x 64-channel ci slices x 128-channel co slices),
        // at most one wave of two CTAs per SM (no partial second wave), at least two tiles per chunk
        const int ns = (c.cin + 63) / 64, ms = (c.cout + 127) / 128;
        const long tiles = (P + WT_PIX - 1) / WT_PIX;
        long chunks = std::max(1L, std::min<long>({2L * n.sm_count / (3 * ns * ms), (long)WG_CHUNKS,
                                                   std::max(1L, tiles / 2)}));
        const int tpc = (int)((tiles + chunks - 1) / chunks);
        chunks = (tiles + tpc - 1) / tpc;
        dim3 grid((unsigned)chunks, (unsigned)(3 * ns * ms));
        k_wgrad_tc<<<grid, 192, WT_SMEM, s>>>(tx, tz, g, c.cin, c.cout, ns, tpc, n.wpart, n.err);
        // bias partial sums over their own (finer) pixel chunks, 8 channels per thread
        const long bcp = std::max<long>(256, (P + WG_CHUNKS - 1) / WG_CHUNKS);
        const int bchunks = (int)((P + bcp - 1) / bcp);
        k_bgrad<<<(unsigned)bchunks, 256, 0, s>>>(dz, P, c.cout, bcp, n.bpart);
        const size_t cnt = (size_t)9 * c.cin * c.cout;
        k_wgrad_reduce<<<grid_for((long)cnt, 32), 256, 0, s>>>(n.wpart, (int)chunks, cnt, n.gw + n.woff[i]);
        k_wgrad_reduce<<<grid_for((long)c.cout, 32), 256, 0, s>>>(n.bpart, bchunks, (size_t)c.cout, n.gw + n.boff[i]);
        return;
    }
    // chunk = ceil(P / WG_CHUNKS) rounded up to WG_PIX, so there are at most WG_CHUNKS chunks
    const long cp = std::max<long>(WG_PIX, ((P + WG_CHUNKS - 1) / WG_CHUNKS + WG_PIX - 1) / WG_PIX * WG_PIX);
    const int chunks = (int)((P + cp - 1) / cp);
    dim3 grid((unsigned)((c.cin + 31) / 32), (unsigned)(9 * ((c.cout + 31) / 32)), (unsigned)chunks);
    k_wgrad<<<grid, 128, 0, s>>>(g, x, dz, c.cin, c.cout, cp, n.wpart, n.bpart);
    const size_t cnt = (size_t)9 * c.cin * c.cout;
    k_wgrad_reduce<<<grid_for((long)cnt, 32), 256, 0, s>>>(n.wpart, chunks, cnt, n.gw + n.woff[i]);
    k_wgrad_reduce<<<grid_for((long)c.cout, 32), 256, 0, s>>>(n.bpart, chunks, (size_t)c.cout, n.gw + n.boff[i]);
}

void relu_back(const Geo& g, View g32, View act, int C, bool relu, View dz, cudaStream_t s)
{
    const long P = (long)g.N * g.H * g.W;
    k_relu_back<<<grid_for(P * C), 256, 0, s>>>(g32, act, P, C, relu, dz);
}

void forward(Net& n, int Hr, int Wr, bool train, cudaStream_t s)
{
    const Geo* G = n.geo;
    conv(n, 0, G[0], vw(n.X0, IN_CH, 0, IN_CH), vw(n.A0a, 32, 0, 32), none(), s);
    conv(n, 1, G[0], vw(n.A0a, 32, 0, 32), vw(n.cat0, 96, 64, 32), none(), s);
    k_pool<<<grid_for(n.P[1] * 32), 256, 0, s>>>(G[0], vw(n.cat0, 96, 64, 32), vw(n.p1, 32, 0, 32));
    conv(n, 2, G[1], vw(n.p1, 32, 0, 32), vw(n.A1a, 64, 0, 64), none(), s);
    conv(n, 3, G[1], vw(n.A1a, 64, 0, 64), vw(n.cat1, 160, 96, 64), none(), s);
    k_pool<<<grid_for(n.P[2] * 64), 256, 0, s>>>(G[1], vw(n.cat1, 160, 96, 64), vw(n.p2, 64, 0, 64));
    conv(n, 4, G[2], vw(n.p2, 64, 0, 64), vw(n.A2a, 96, 0, 96), none(), s);
    conv(n, 5, G[2], vw(n.A2a, 96, 0, 96), vw(n.cat2, 224, 128, 96), none(), s);
    k_pool<<<grid_for(n.P[3] * 96), 256, 0, s>>>(G[2], vw(n.cat2, 224, 128, 96), vw(n.p3, 96, 0, 96));
    conv(n, 6, G[3], vw(n.p3, 96, 0, 96), vw(n.A3a, 128, 0, 128), none(), s);
    conv(n, 7, G[3], vw(n.A3a, 128, 0, 128), vw(n.cat3, 288, 160, 128), none(), s);
    k_pool<<<grid_for(n.P[4] * 128), 256, 0, s>>>(G[3], vw(n.cat3, 288, 160, 128), vw(n.p4, 128, 0, 128));
    conv(n, 8, G[4], vw(n.p4, 128, 0, 128), vw(n.A4a, 160, 0, 160), none(), s);
    conv(n, 9, G[4], vw(n.A4a, 160, 0, 160), vw(n.A4b, 160, 0, 160), none(), s);
    k_upsample<<<grid_for(n.P[3] * 160), 256, 0, s>>>(G[4], vw(n.A4b, 160, 0, 160), vw(n.cat3, 288, 0, 160));
    conv(n, 10, G[3], vw(n.cat3, 288, 0, 288), vw(n.D3a, 128, 0, 128), none(), s);
    conv(n, 11, G[3], vw(n.D3a, 128, 0, 128), vw(n.D3b, 128, 0, 128), none(), s);
    k_upsample<<<grid_for(n.P[2] * 128), 256, 0, s>>>(G[3], vw(n.D3b, 128, 0, 128), vw(n.cat2, 224, 0, 128));
    conv(n, 12, G[2], vw(n.cat2, 224, 0, 224), vw(n.D2a, 96, 0, 96), none(), s);
    conv(n, 13, G[2], vw(n.D2a, 96, 0, 96), vw(n.D2b, 96, 0, 96), none(), s);
    k_upsample<<<grid_for(n.P[1] * 96), 256, 0, s>>>(G[2], vw(n.D2b, 96, 0, 96), vw(n.cat1, 160, 0, 96));
    conv(n, 14, G[1], vw(n.cat1, 160, 0, 160), vw(n.D1a, 64, 0, 64), none(), s);
    conv(n, 15, G[1], vw(n.D1a, 64, 0, 64), vw(n.D1b, 64, 0, 64), none(), s);
    k_upsample<<<grid_for(n.P[0] * 64), 256, 0, s>>>(G[1], vw(n.D1b, 64, 0, 64), vw(n.cat0, 96, 0, 64));
    conv(n, 16, G[0], vw(n.cat0, 96, 0, 96), vw(n.D0a, 32, 0, 32), none(), s);
    conv(n, 17, G[0], vw(n.D0a, 32, 0, 32), vw(n.D0b, 32, 0, 32), none(), s);
    // at inference the row-tile kernel applies the predicted kernels in its epilogue (no logits
    // stored); training keeps the logits and the softmax weights for the backward pass
    const ApplyArgs ap{n.rad, n.out, Hr, Wr};
    const bool fused = conv(n, 18, G[0], vw(n.D0b, 32, 0, 32), none(), vw(n.logits, OUT_CH, 0, OUT_CH), s,
                            train ? nullptr : &ap);
    if (!fused) k_apply<<<grid_for(n.P[0]), 256, 0, s>>>(G[0], Hr, Wr, n.logits, n.rad, train ? n.wts : nullptr, n.out);
    n.logits_stored = !fused;
    add_launches(19 + 4 + 4 + (fused ? 0 : 1));
}

void backward(Net& n, int Hr, int Wr, cudaStream_t s)
{
    const Geo* G = n.geo;
    k_apply_back<<<grid_for(n.P[0]), 256, 0, s>>>(G[0], Hr, Wr, n.wts, n.rad, n.dout, n.dz[0]);
    // output conv (no ReLU): dZ = dlogits
    wgrad(n, 18, G[0], vw(n.D0b, 32, 0, 32), vw(n.dz[0], OUT_CH, 0, OUT_CH), s);
    dgrad(n, 18, G[0], vw(n.dz[0], OUT_CH, 0, OUT_CH), vw(n.G_D0b, 32, 0, 32), s);
    // decoder level 0
    relu_back(G[0], vw(n.G_D0b, 32, 0, 32), vw(n.D0b, 32, 0, 32), 32, true, vw(n.dz[0], 32, 0, 32), s);
    wgrad(n, 17, G[0], vw(n.D0a, 32, 0, 32), vw(n.dz[0], 32, 0, 32), s);
    dgrad(n, 17, G[0], vw(n.dz[0], 32, 0, 32), vw(n.G_D0a, 32, 0, 32), s);
    relu_back(G[0], vw(n.G_D0a, 32, 0, 32), vw(n.D0a, 32, 0, 32), 32, true, vw(n.dz[0], 32, 0, 32), s);
    wgrad(n, 16, G[0], vw(n.cat0, 96, 0, 96), vw(n.dz[0], 32, 0, 32), s);
    dgrad(n, 16, G[0], vw(n.dz[0], 32, 0, 32), vw(n.G_cat0, 96, 0, 96), s);
    k_upsample_back<<<grid_for(n.P[1] * 64), 256, 0, s>>>(G[1], vw(n.G_cat0, 96, 0, 64), vw(n.G_D1b, 64, 0, 64));
    // decoder level 1
    relu_back(G[1], vw(n.G_D1b, 64, 0, 64), vw(n.D1b, 64, 0, 64), 64, true, vw(n.dz[1], 64, 0, 64), s);
    wgrad(n, 15, G[1], vw(n.D1a, 64, 0, 64), vw(n.dz[1], 64, 0, 64), s);
    dgrad(n, 15, G[1], vw(n.dz[1], 64, 0, 64), vw(n.G_D1a, 64, 0, 64), s);
    relu_back(G[1], vw(n.G_D1a, 64, 0, 64), vw(n.D1a, 64, 0, 64), 64, true, vw(n.dz[1], 64, 0, 64), s);
    wgrad(n, 14, G[1], vw(n.cat1, 160, 0, 160), vw(n.dz[1], 64, 0, 64), s);
    dgrad(n, 14, G[1], vw(n.dz[1], 64, 0, 64), vw(n.G_cat1, 160, 0, 160), s);
    k_upsample_back<<<grid_for(n.P[2] * 96), 256, 0, s>>>(G[2], vw(n.G_cat1, 160, 0, 96), vw(n.G_D2b, 96, 0, 96));
    // decoder level 2
    relu_back(G[2], vw(n.G_D2b, 96, 0, 96), vw(n.D2b, 96, 0, 96), 96, true, vw(n.dz[2], 96, 0, 96), s);
    wgrad(n, 13, G[2], vw(n.D2a, 96, 0, 96), vw(n.dz[2], 96, 0, 96), s);
    dgrad(n, 13, G[2], vw(n.dz[2], 96, 0, 96), vw(n.G_D2a, 96, 0, 96), s);
    relu_back(G[2], vw(n.G_D2a, 96, 0, 96), vw(n.D2a, 96, 0, 96), 96, true, vw(n.dz[2], 96, 0, 96), s);
    wgrad(n, 12, G[2], vw(n.cat2, 224, 0, 224), vw(n.dz[2], 96, 0, 96), s);
    dgrad(n, 12, G[2], vw(n.dz[2], 96, 0, 96), vw(n.G_cat2, 224, 0, 224), s);
    k_upsample_back<<<grid_for(n.P[3] * 128), 256, 0, s>>>(G[3], vw(n.G_cat2, 224, 0, 128),
                                                            vw(n.G_D3b, 128, 0, 128));
    // decoder level 3
    relu_back(G[3], vw(n.G_D3b, 128, 0, 128), vw(n.D3b, 128, 0, 128), 128, true, vw(n.dz[3], 128, 0, 128), s);
    wgrad(n, 11, G[3], vw(n.D3a, 128, 0, 128), vw(n.dz[3], 128, 0, 128), s);
    dgrad(n, 11, G[3], vw(n.dz[3], 128, 0, 128), vw(n.G_D3a, 128, 0, 128), s);
    relu_back(G[3], vw(n.G_D3a, 128, 0, 128), vw(n.D3a, 128, 0, 128), 128, true, vw(n.dz[3], 128, 0, 128), s);
    wgrad(n, 10, G[3], vw(n.cat3, 288, 0, 288), vw(n.dz[3], 128, 0, 128), s);
    dgrad(n, 10, G[3], vw(n.dz[3], 128, 0, 128), vw(n.G_cat3, 288, 0, 288), s);
    k_upsample_back<<<grid_for(n.P[4] * 160), 256, 0, s>>>(G[4], vw(n.G_cat3, 288, 0, 160),
                                                            vw(n.G_A4b, 160, 0, 160));
    // encoder level 4
    relu_back(G[4], vw(n.G_A4b, 160, 0, 160), vw(n.A4b, 160, 0, 160), 160, true, vw(n.dz[4], 160, 0, 160), s);
    wgrad(n, 9, G[4], vw(n.A4a, 160, 0, 160), vw(n.dz[4], 160, 0, 160), s);
    dgrad(n, 9, G[4], vw(n.dz[4], 160, 0, 160), vw(n.G_A4a, 160, 0, 160), s);
    relu_back(G[4], vw(n.G_A4a, 160, 0, 160), vw(n.A4a, 160, 0, 160), 160, true, vw(n.dz[4], 160, 0, 160), s);
    wgrad(n, 8, G[4], vw(n.p4, 128, 0, 128), vw(n.dz[4], 160, 0, 160), s);
    dgrad(n, 8, G[4], vw(n.dz[4], 160, 0, 160), vw(n.G_p4, 128, 0, 128), s);
    k_pool_back<<<grid_for(n.P[3] * 128), 256, 0, s>>>(G[3], vw(n.G_p4, 128, 0, 128), vw(n.G_cat3, 288, 160, 128));
    // encoder level 3
    relu_back(G[3], vw(n.G_cat3, 288, 160, 128), vw(n.cat3, 288, 160, 128), 128, true, vw(n.dz[3], 128, 0, 128), s);
    wgrad(n, 7, G[3], vw(n.A3a, 128, 0, 128), vw(n.dz[3], 128, 0, 128), s);
    dgrad(n, 7, G[3], vw(n.dz[3], 128, 0, 128), vw(n.G_A3a, 128, 0, 128), s);
    relu_back(G[3], vw(n.G_A3a, 128, 0, 128), vw(n.A3a, 128, 0, 128), 128, true, vw(n.dz[3], 128, 0, 128), s);
    wgrad(n, 6, G[3], vw(n.p3, 96, 0, 96), vw(n.dz[3], 128, 0, 128), s);
    dgrad(n, 6, G[3], vw(n.dz[3], 128, 0, 128), vw(n.G_p3, 96, 0, 96), s);
    k_pool_back<<<grid_for(n.P[2] * 96), 256, 0, s>>>(G[2], vw(n.G_p3, 96, 0, 96), vw(n.G_cat2, 224, 128, 96));
    // encoder level 2
    relu_back(G[2], vw(n.G_cat2, 224, 128, 96), vw(n.cat2, 224, 128, 96), 96, true, vw(n.dz[2], 96, 0, 96), s);
    wgrad(n, 5, G[2], vw(n.A2a, 96, 0, 96), vw(n.dz[2], 96, 0, 96), s);
    dgrad(n, 5, G[2], vw(n.dz[2], 96, 0, 96), vw(n.G_A2a, 96, 0, 96), s);
    relu_back(G[2], vw(n.G_A2a, 96, 0, 96), vw(n.A2a, 96, 0, 96), 96, true, vw(n.dz[2], 96, 0, 96), s);
    wgrad(n, 4, G[2], vw(n.p2, 64, 0, 64), vw(n.dz[2], 96, 0, 96), s);
    dgrad(n, 4, G[2], vw(n.dz[2], 96, 0, 96), vw(n.G_p2, 64, 0, 64), s);
    k_pool_back<<<grid_for(n.P[1] * 64), 256, 0, s>>>(G[1], vw(n.G_p2, 64, 0, 64), vw(n.G_cat1, 160, 96, 64));
    // encoder level 1
    relu_back(G[1], vw(n.G_cat1, 160, 96, 64), vw(n.cat1, 160, 96, 64), 64, true, vw(n.dz[1], 64, 0, 64), s);
    wgrad(n, 3, G[1], vw(n.A1a, 64, 0, 64), vw(n.dz[1], 64, 0, 64), s);
    dgrad(n, 3, G[1], vw(n.dz[1], 64, 0, 64), vw(n.G_A1a, 64, 0, 64), s);
    relu_back(G[1], vw(n.G_A1a, 64, 0, 64), vw(n.A1a, 64, 0, 64), 64, true, vw(n.dz[1], 64, 0, 64), s);
    wgrad(n, 2, G[1], vw(n.p1, 32, 0, 32), vw(n.dz[1], 64, 0, 64), s);
    dgrad(n, 2, G[1], vw(n.dz[1], 64, 0, 64), vw(n.G_p1, 32, 0, 32), s);
    k_pool_back<<<grid_for(n.P[0] * 32), 256, 0, s>>>(G[0], vw(n.G_p1, 32, 0, 32), vw(n.G_cat0, 96, 64, 32));
    // encoder level 0
    relu_back(G[0], vw(n.G_cat0, 96, 64, 32), vw(n.cat0, 96, 64, 32), 32, true, vw(n.dz[0], 32, 0, 32), s);
    wgrad(n, 1, G[0], vw(n.A0a, 32, 0, 32), vw(n.dz[0], 32, 0, 32), s);
    dgrad(n, 1, G[0], vw(n.dz[0], 32, 0, 32), vw(n.G_A0a, 32, 0, 32), s);
    relu_back(G[0], vw(n.G_A0a, 32, 0, 32), vw(n.A0a, 32, 0, 32), 32, true, vw(n.dz[0], 32, 0, 32), s);
    wgrad(n, 0, G[0], vw(n.X0, IN_CH, 0, IN_CH), vw(n.dz[0], 32, 0, 32), s);
    add_launches(1 + 19 * 3 + 18 + 4 + 4 + 18);
}

cpt_status prepare(Net& n, int N, int Hr, int Wr, const float* rgb, const float* gbuf, cudaStream_t s)
{
    const int H = (Hr + 15) / 16 * 16, W = (Wr + 15) / 16 * 16;
    cpt_status st = ensure_geometry(n, N, H, W);
    if (st != CPT_OK) return st;
    st = refresh_copies(n, s);
    if (st != CPT_OK) return st;
    const bool aligned = (reinterpret_cast<uintptr_t>(gbuf) & 15) == 0;   // G-buffer rows as float4 pairs
    k_features<<<grid_for(n.P[0]), 256, 0, s>>>(n.geo[0], Hr, Wr, rgb, gbuf, aligned, n.X0, n.rad);
    add_launches(1);
    return CPT_OK;
}

}  // namespace kpcn
}  // namespace cpt

// ------------------------------------------------------------------ C ABI
using namespace cpt;

struct cpt_denoiser {
    kpcn::Net net;
};

static bool check_dims(int32_t n, int32_t h, int32_t w) { return n > 0 && h > 0 && w > 0 && (long)n * h * w < (1L << 31); }

CPT_EXPORT cpt_status cpt_denoiser_create(int device, uint64_t seed, cpt_denoiser** out)
{
    if (!out) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_create: out is NULL");
    *out = nullptr;
    CPT_CUDA(cudaSetDevice(device));
    cpt_denoiser* d = new cpt_denoiser;
    d->net.device = device;
    cpt_status st = kpcn::net_init(d->net, seed);
    if (st != CPT_OK) {
        delete d;
        return st;
    }
    *out = d;
    return CPT_OK;
}

// Convolution engine: 0 = mma.sync kernel, 1 = tcgen05 kernel with cp.async copies, 2 = TMA-fed
// warp-specialised persistent tcgen05 kernels (the default).
CPT_EXPORT cpt_status cpt_denoiser_set_backend(cpt_denoiser* d, int32_t backend)
{
    if (!d || backend < 0 || backend > 2) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_set_backend: 0, 1 or 2");
    d->net.backend = backend;
    return CPT_OK;
}

// Device error word of the last passes (CPT_DEVERR_ITER: a tensor-core barrier wait timed out);
// reading clears it.
CPT_EXPORT cpt_status cpt_denoiser_check(cpt_denoiser* d)
{
    if (!d) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_check: null");
    int e = 0;
    CPT_CUDA(cudaSetDevice(d->net.device));
    CPT_CUDA(cudaMemcpy(&e, d->net.err, sizeof e, cudaMemcpyDeviceToHost));
    CPT_CUDA(cudaMemset(d->net.err, 0, sizeof e));
    if (e) return fail(CPT_ERR_TIMEOUT, "denoiser: a tensor-core barrier wait timed out");
    return CPT_OK;
}

namespace {
// Self-test of the bounded barrier wait that every tensor-core kernel uses: a barrier that
// nothing arrives on (no copy or MMA is issued, so nothing is in flight when the wait gives up).
// mbar_wait returns false after its cycle budget (about 1 s) and sets the error word, which
// cpt_denoiser_check reports as CPT_ERR_TIMEOUT; the context stays usable.
__global__ void k_wait_selftest(int* err)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        cpt::kpcn::mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        cpt::kpcn::mbar_wait(&bar, 0u, err);
    }
}
}  // namespace

CPT_EXPORT cpt_status cpt_denoiser_wait_selftest(cpt_denoiser* d)
{
    if (!d) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_wait_selftest: null");
    CPT_CUDA(cudaSetDevice(d->net.device));
    k_wait_selftest<<<1, 32>>>(d->net.err);
    add_launches(1);
    CPT_CUDA(cudaGetLastError());
    CPT_CUDA(cudaDeviceSynchronize());
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_denoiser_destroy(cpt_denoiser* d)
{
    delete d;
    return CPT_OK;
}

CPT_EXPORT uint64_t cpt_denoiser_num_params(const cpt_denoiser* d) { return d ? d->net.n_params : 0; }

CPT_EXPORT cpt_status cpt_denoiser_get_params(cpt_denoiser* d, float* host)
{
    if (!d || !host) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_get_params: null argument");
    CPT_CUDA(cudaSetDevice(d->net.device));
    CPT_CUDA(cudaMemcpy(host, d->net.w, d->net.n_params * sizeof(float), cudaMemcpyDeviceToHost));
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_denoiser_set_params(cpt_denoiser* d, const float* host)
{
    if (!d || !host) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_set_params: null argument");
    CPT_CUDA(cudaSetDevice(d->net.device));
    CPT_CUDA(cudaMemcpy(d->net.w, host, d->net.n_params * sizeof(float), cudaMemcpyHostToDevice));
    CPT_CUDA(cudaMemset(d->net.m, 0, d->net.n_params * sizeof(float)));
    CPT_CUDA(cudaMemset(d->net.v, 0, d->net.n_params * sizeof(float)));
    d->net.step = 0;
    d->net.copies_fresh = false;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_denoiser_get_grads(cpt_denoiser* d, float* host)
{
    if (!d || !host) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_get_grads: null argument");
    CPT_CUDA(cudaSetDevice(d->net.device));
    CPT_CUDA(cudaMemcpy(host, d->net.gw, d->net.n_params * sizeof(float), cudaMemcpyDeviceToHost));
    return CPT_OK;
}

// Copies one internal tensor of the last forward/backward pass (for tests): activations as BF16
// values widened to float, gradients as float.  *count receives the number of elements.
CPT_EXPORT cpt_status cpt_denoiser_export(cpt_denoiser* d, const char* name, float* host, uint64_t capacity,
                                          uint64_t* count)
{
    if (!d || !name || !count) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_export: null argument");
    kpcn::Net& n = d->net;
    if (!n.arena) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_export: nothing computed yet");
    const long* P = n.P;
    struct T {
        const char* name;
        const void* ptr;
        long elems;
        bool b16;
    } table[] = {
        {"X0", n.X0, P[0] * kpcn::IN_CH, true}, {"A0a", n.A0a, P[0] * 32, true}, {"cat0", n.cat0, P[0] * 96, true},
        {"p1", n.p1, P[1] * 32, true}, {"A1a", n.A1a, P[1] * 64, true}, {"cat1", n.cat1, P[1] * 160, true},
        {"p2", n.p2, P[2] * 64, true}, {"A2a", n.A2a, P[2] * 96, true}, {"cat2", n.cat2, P[2] * 224, true},
        {"p3", n.p3, P[3] * 96, true}, {"A3a", n.A3a, P[3] * 128, true}, {"cat3", n.cat3, P[3] * 288, true},
        {"p4", n.p4, P[4] * 128, true}, {"A4a", n.A4a, P[4] * 160, true}, {"A4b", n.A4b, P[4] * 160, true},
        {"D3a", n.D3a, P[3] * 128, true}, {"D3b", n.D3b, P[3] * 128, true}, {"D2a", n.D2a, P[2] * 96, true},
        {"D2b", n.D2b, P[2] * 96, true}, {"D1a", n.D1a, P[1] * 64, true}, {"D1b", n.D1b, P[1] * 64, true},
        {"D0a", n.D0a, P[0] * 32, true}, {"D0b", n.D0b, P[0] * 32, true},
        {"logits", n.logits, P[0] * kpcn::OUT_CH, false}, {"out", n.out, P[0] * 3, false},
        {"G_D0b", n.G_D0b, P[0] * 32, false}, {"G_D0a", n.G_D0a, P[0] * 32, false},
        {"G_cat0", n.G_cat0, P[0] * 96, false}, {"G_D1b", n.G_D1b, P[1] * 64, false},
        {"G_cat1", n.G_cat1, P[1] * 160, false}, {"G_D2b", n.G_D2b, P[2] * 96, false},
        {"G_cat2", n.G_cat2, P[2] * 224, false}, {"G_D3b", n.G_D3b, P[3] * 128, false},
        {"G_cat3", n.G_cat3, P[3] * 288, false}, {"G_A4b", n.G_A4b, P[4] * 160, false},
        {"G_p4", n.G_p4, P[4] * 128, false}, {"G_p3", n.G_p3, P[3] * 96, false}, {"G_p2", n.G_p2, P[2] * 64, false},
        {"G_p1", n.G_p1, P[1] * 32, false}, {"G_A0a", n.G_A0a, P[0] * 32, false},
    };
    for (const T& t : table) {
        if (std::strcmp(t.name, name) != 0) continue;
        if (t.ptr == n.logits && !n.logits_stored)
            return fail(CPT_ERR_UNSUPPORTED, "cpt_denoiser_export: the last pass did not store \"logits\" (cpt_denoise "
                                             "applies the predicted kernels inside the last convolution)");
        *count = (uint64_t)t.elems;
        if (!host || capacity < (uint64_t)t.elems) return CPT_OK;
        CPT_CUDA(cudaSetDevice(n.device));
        CPT_CUDA(cudaDeviceSynchronize());
        if (t.b16) {
            std::vector<uint16_t> raw(t.elems);
            CPT_CUDA(cudaMemcpy(raw.data(), t.ptr, t.elems * 2, cudaMemcpyDeviceToHost));
            for (long i = 0; i < t.elems; ++i) {
                uint32_t u = (uint32_t)raw[i] << 16;
                std::memcpy(&host[i], &u, 4);
            }
        } else {
            CPT_CUDA(cudaMemcpy(host, t.ptr, t.elems * 4, cudaMemcpyDeviceToHost));
        }
        return CPT_OK;
    }
    return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_export: unknown tensor");
}

CPT_EXPORT cpt_status cpt_denoiser_train_step(cpt_denoiser* d, int32_t n, int32_t h, int32_t w, const float* rgb,
                                              const float* gbuf, const float* target, float lr, int32_t update,
                                              float* loss, void* stream_)
{
    if (!d || !rgb || !gbuf || !target) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_train_step: null argument");
    if (!check_dims(n, h, w) || h % 16 || w % 16)
        return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoiser_train_step: crops must be multiples of 16");
    cudaStream_t s = (cudaStream_t)stream_;
    kpcn::Net& net = d->net;
    CPT_CUDA(cudaSetDevice(net.device));
    cpt_status st = kpcn::prepare(net, n, h, w, rgb, gbuf, s);
    if (st != CPT_OK) return st;
    kpcn::forward(net, h, w, true, s);
    const int lb = kpcn::grid_for(net.P[0]);
    const float scale = 1.0f / (float)((double)n * h * w * 3.0);
    kpcn::k_loss<<<lb, 256, 0, s>>>(net.geo[0], h, w, net.out, target, net.dout, net.loss_part, scale);
    kpcn::backward(net, h, w, s);
    if (update) {
        net.step += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)net.step), c2 = 1.f - std::pow(b2, (float)net.step);
        kpcn::k_adam<<<kpcn::grid_for((long)net.n_params), 256, 0, s>>>(net.w, net.gw, net.m, net.v, net.n_params, lr,
                                                                        b1, b2, 1e-8f, c1, c2);
        net.copies_fresh = false;
        add_launches(1);
    }
    add_launches(1);
    CPT_CUDA(cudaGetLastError());
    if (loss) {
        std::vector<float> part(lb);
        CPT_CUDA(cudaMemcpyAsync(part.data(), net.loss_part, lb * sizeof(float), cudaMemcpyDeviceToHost, s));
        CPT_CUDA(cudaStreamSynchronize(s));
        double sum = 0.0;
        for (float x : part) sum += x;
        *loss = (float)(sum * scale);
    }
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_denoise(cpt_denoiser* d, int32_t n, int32_t h, int32_t w, const float* rgb,
                                  const float* gbuf, float* out, void* stream_)
{
    if (!d || !rgb || !gbuf || !out) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoise: null argument");
    if (!check_dims(n, h, w)) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_denoise: bad image size");
    cudaStream_t s = (cudaStream_t)stream_;
    kpcn::Net& net = d->net;
    CPT_CUDA(cudaSetDevice(net.device));
    cpt_status st = kpcn::prepare(net, n, h, w, rgb, gbuf, s);
    if (st != CPT_OK) return st;
    kpcn::forward(net, h, w, false, s);
    kpcn::k_crop<<<kpcn::grid_for((long)n * h * w), 256, 0, s>>>(net.geo[0], h, w, net.out, out);
    add_launches(1);
    CPT_CUDA(cudaGetLastError());
    return CPT_OK;
}

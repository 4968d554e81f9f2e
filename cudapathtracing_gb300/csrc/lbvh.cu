// lbvh.cu — LBVH construction on the GPU (Device::buildBVH, Device.cuh:169-195).
//
//   k_prep        centroid (FP64) + Morton code + leaf box per primitive
//                 (generateMortonCodes Device.cuh:134-142, morton3D BVH.cuh:23-41,
//                  Hittable ctors Hittable.cuh:456-462)
//   radix sort    stable LSD over the 30-bit codes, three 10-bit digits, per-tile ranking with
//                 __match_any_sync (replaces thrust::sort_by_key Device.cuh:187-189: keys are
//                 code<<32|index, so a stable sort of codes with ascending indices is the
//                 same permutation)
//   k_emit        Karras 2012 range/split per internal node (generateHierarchy BVH.cuh:174-241)
//   refit         atomic-free: an internal node covers the contiguous sorted leaves
//                 [first, last], so its box is a range union, answered from a 4-ary pyramid
//                 of unions of the leaf boxes (replaces the serial constructAABB BVH.cuh:243-280;
//                 min/max is exact, so the boxes equal the pairwise unions)
//
// All boxes are FP32 rounded outwards from the reference's FP64 boxes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "cpt_internal.h"
#include "cpt_quant.cuh"

namespace cpt {

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;   // 4096 keys per tile
constexpr int RS_BITS = 10;
constexpr int RS_BINS = 1 << RS_BITS;            // 1024 digits
constexpr uint32_t RS_MASK = RS_BINS - 1;
constexpr int RS_PASSES = 3;                     // bits 0-9, 10-19, 20-29: the whole 30-bit code
constexpr int RS_DPT = RS_BINS / RS_THREADS;     // digits per thread in the per-tile scans
static_assert(RS_BITS * RS_PASSES >= 30 && RS_BINS % RS_THREADS == 0, "radix digits");

__device__ __forceinline__ uint32_t expand_bits(uint32_t v)   // BVH.cuh:12-19
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// morton3D (BVH.cuh:23-41) in double with explicitly rounded operations (no contraction).
__device__ __forceinline__ uint32_t morton_axis(double c, double mn, double mx)
{
    double nrm = __ddiv_rn(__dsub_rn(c, mn), __dsub_rn(mx, mn));
    double x = __dmul_rn(nrm, 1024.0);
    x = x > 0.0 ? x : 0.0;        // mMax(x, 0.0): NaN -> 0
    x = x < 1023.0 ? x : 1023.0;  // mMin(x, 1023.0)
    return (uint32_t)x;
}

__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }   // mMin
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }   // mMax

template <typename VT>
__device__ __forceinline__ void load_tri(const VT* __restrict__ v, uint32_t t, double p[9])
{
#pragma unroll
    for (int k = 0; k < 9; ++k) p[k] = (double)v[9ull * t + k];
}

// Constants of the fast Morton paths for one axis: the reference's bounds, the scale
// k = 1024 / (max - min) in FP64, and min and k as FP32 (hi) and as unevaluated FP32 pairs
// (hi + lo, within 2^-48 relative of the FP64 values).
struct MortonAxis {
    double mn, mx, k64;
    float mn32, k32;      // RN32(min), RN32(k)
    float mn_lo, k_lo;    // RN32(min - mn32), RN32(k - k32)
};

// floor(x) for 0 <= x < 2^23 on the integer units, without conversion or directed-rounding
// instructions: f = x with its fractional mantissa bits cleared, and the integer from the
// significand shifted by the exponent.
__device__ __forceinline__ int floor_small(float x, float& f)
{
    const uint32_t b = __float_as_uint(x);
    const int e = (int)(b >> 23) - 127;
    if (e < 0) {
        f = 0.0f;
        return 0;
    }
    const uint32_t sh = 23u - (uint32_t)e;
    f = __uint_as_float(b & ~((1u << sh) - 1u));
    return (int)(((b & 0x7FFFFFu) | 0x800000u) >> sh);
}

// Morton cell of a triangle-centroid coordinate, equal to the reference's exactly rounded FP64
// sequence morton_axis(RN((p0 + p1 + p2) / 3), min, max) (BVH.cuh:23-33 on the centroid of
// Hittable.cuh:459-461), computed without its two FP64 divisions where that is provably safe:
//   1. FP32: x = (s * (1/3) - min) * k with s = p0 + p1 + p2.  Its distance to the reference's
//      x is below tol = 2^-20 (k (|p0| + |p1| + |p2| + |min|) + 2 |x|), four times the worst-case
//      sum of the rounding errors (two additions, the multiplications and the rounded 1/3 and
//      k, each at most 2^-24 relative).  The cell is floor(x) when x is farther than tol from
//      every cell boundary (the integers 1 .. 1023; below 1 the cell is 0, at or above 1023 it
//      is 1023).
//   2. Otherwise the same in unevaluated pairs of FP32 numbers (TwoSum and FMA-based TwoProd,
//      about 44 significant bits), with tol = 2^-40 (...): still on the FP32 units, whereas one
//      lane on an FP64 path costs its whole warp the part's low FP64 issue rate.
//   3. Otherwise the reference's own sequence with IEEE divisions, in FP64.
// Non-finite intermediates (a degenerate axis) always take step 3.
__device__ __forceinline__ int cell_of(float x, float tol)
{
    if (!(tol < 0.25f) || !(fabsf(x) < 1e30f)) return -1;   // also rejects NaN and infinities
    if (x < 1.0f - tol) return 0;
    if (x > 1023.0f + tol) return 1023;
    float f;
    const int c = floor_small(x, f);   // here 1 - tol <= x <= 1023 + tol
    return (x - f > tol && f + 1.0f - x > tol) ? c : -1;
}

// Step 3.  Out of line, with the widening inside, so that the compiler cannot evaluate any of it
// speculatively beside the FP32 steps.
template <typename VT>
__device__ __noinline__ uint32_t morton_tri_axis_fp64(VT a_, VT b_, VT c_, MortonAxis m)
{
    const double a = (double)a_, b = (double)b_, c = (double)c_;
    return morton_axis(__ddiv_rn(__dadd_rn(__dadd_rn(a, b), c), 3.0), m.mn, m.mx);
}

// Error-free transformations on FP32 (Knuth's TwoSum; the product's error from one FMA).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e)
{
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

constexpr float THIRD_HI = 0x1.555556p-2f;    // RN32(1/3)
constexpr float THIRD_LO = -0x1.555556p-27f;  // RN32(1/3 - THIRD_HI); the rest is below 2^-50

// Step 2 (and 3 where it cannot decide).  Out of line: it runs for a fraction of a percent of the
// coordinates.
__device__ __noinline__ uint32_t morton_tri_axis_ff(float a, float b, float c, MortonAxis m)
{
    // s = a + b + c as hi + lo
    float s1, e1, s2, e2;
    two_sum(a, b, s1, e1);
    two_sum(s1, c, s2, e2);
    const float slo = __fadd_rn(e1, e2);
    // y = s / 3
    float y, ye;
    two_prod(s2, THIRD_HI, y, ye);
    ye = __fadd_rn(ye, __fadd_rn(__fmul_rn(s2, THIRD_LO), __fmul_rn(slo, THIRD_HI)));
    // z = y - min
    float z, ze;
    two_sum(y, -m.mn32, z, ze);
    ze = __fadd_rn(ze, __fsub_rn(ye, m.mn_lo));
    // x = z * k
    float x, xe;
    two_prod(z, m.k32, x, xe);
    xe = __fadd_rn(xe, __fadd_rn(__fmul_rn(z, m.k_lo), __fmul_rn(ze, m.k32)));
    const float mag = fabsf(a) + fabsf(b) + fabsf(c) + fabsf(m.mn32);
    const float tol = 0x1p-40f * (m.k32 * mag + 2.0f * fabsf(x));
    if (isfinite(x) && isfinite(xe) && isfinite(tol) && tol < 0.25f) {
        const float xs = __fadd_rn(x, xe);
        if (xs < 1.0f - tol) return 0u;
        if (xs > 1023.0f + tol) return 1023u;
        float f;
        const int cell = floor_small(fminf(fmaxf(x, 0.0f), 1024.0f), f);
        // signed distances of x + xe above floor(x) and below floor(x) + 1 (x - f and f + 1 - x are
        // exact); xe can move the sum across either integer
        const float below = __fadd_rn(__fsub_rn(x, f), xe), above = __fsub_rn(__fsub_rn(__fadd_rn(f, 1.0f), x), xe);
        if (below > tol && above > tol) return (uint32_t)min(cell, 1023);
        if (below < -tol && cell >= 1) return (uint32_t)min(cell - 1, 1023);
        if (above < -tol) return (uint32_t)min(cell + 1, 1023);
    }
    return morton_tri_axis_fp64<float>(a, b, c, m);
}

template <typename VT>
__device__ __forceinline__ uint32_t morton_tri_axis(VT a, VT b, VT c, const MortonAxis& m)
{
    const float a32 = (float)a, b32 = (float)b, c32 = (float)c;
    const float x32 = ((a32 + b32 + c32) * (1.0f / 3.0f) - m.mn32) * m.k32;
    const float mag = fabsf(a32) + fabsf(b32) + fabsf(c32) + fabsf(m.mn32);
    const float tol32 = 0x1p-20f * (m.k32 * mag + 2.0f * fabsf(x32));
    const int cell = cell_of(x32, tol32);
    if (cell >= 0) return (uint32_t)cell;
    return morton_tri_axis_ff(a32, b32, c32, m);
}

// Triangle centroid and padded box (Hittable.cuh:459-461, AABB.cuh:30-40), boxes rounded
// outwards to FP32.
__device__ __forceinline__ void tri_center_box(const double p[9], double c[3], float4& bmin, float4& bmax)
{
    double mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        c[a] = __ddiv_rn(__dadd_rn(__dadd_rn(p[a], p[3 + a]), p[6 + a]), 3.0);
        mn[a] = __dsub_rn(dmin(dmin(p[a], p[3 + a]), p[6 + a]), 0.0001);
        mx[a] = __dadd_rn(dmax(dmax(p[a], p[3 + a]), p[6 + a]), 0.0001);
    }
    bmin = make_float4(__double2float_rd(mn[0]), __double2float_rd(mn[1]), __double2float_rd(mn[2]), 0.f);
    bmax = make_float4(__double2float_ru(mx[0]), __double2float_ru(mx[1]), __double2float_ru(mx[2]), 0.f);
}

// Conversions between FP32 and FP64 by bit manipulation on the integer units: on this part the
// FP64 pipe also executes the hardware conversions, and it is the scarce resource of k_prep.
// widen: exact float -> double.  narrow_rd / narrow_ru: double -> float rounded down / up.  Values
// outside the normal range of the narrower type take the hardware conversion, out of line (an
// inline conversion is evaluated for every value and then discarded by a select).
__device__ __noinline__ double widen_hw(float f) { return (double)f; }
__device__ __noinline__ float narrow_hw_rd(double d) { return __double2float_rd(d); }
__device__ __noinline__ float narrow_hw_ru(double d) { return __double2float_ru(d); }

__device__ __forceinline__ double widen(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xFFu;
    if (e == 0u || e == 0xFFu) return widen_hw(f);   // zero, subnormal, infinity, NaN
    const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(b << 29));
}

template <bool UP>
__device__ __forceinline__ float narrow(double d)
{
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if (e < 897u || e > 1150u) return UP ? narrow_hw_ru(d) : narrow_hw_rd(d);
    uint32_t fb = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const bool inexact = (lo & 0x1FFFFFFFu) != 0u;
    const bool negative = (hi >> 31) != 0u;
    // truncation rounds the magnitude down; moving away from zero is one step up in the bits
    if (inexact && (UP ? !negative : negative)) fb += 1u;
    return __uint_as_float(fb);
}

// The reference's padding in FP64: RD32(RN64(x - 1e-4)) (UP false) or RU32(RN64(x + 1e-4)).
template <bool UP>
__device__ __noinline__ float pad_fp64(float x)
{
    return UP ? narrow<true>(__dadd_rn(widen(x), 0.0001)) : narrow<false>(__dsub_rn(widen(x), 0.0001));
}

// The same value from FP32 operations.  c = RN64(1e-4) is split as PAD_HI + PAD_LO (PAD_HI =
// RN32(c), PAD_LO = RN32(c - PAD_HI) = 2.53e-12, within 2^-62 of the exact remainder).  TwoSum
// gives x -+ PAD_HI = s + e exactly, so the exact q = x -+ c is s + r with r = e -+ PAD_LO.  For
// |s| >= 2^-10, |r| is below half the spacing of the floats next to s, so the directed rounding of
// q is s or its neighbour, by the sign of r.  It equals the rounding of RN64(q) unless RN64 moves
// q onto or across s, which needs |r| <= 2^-53 |q|.  The result is therefore certain when |r| >
// 2^-50 |s| (double rounding) + 2^-23 |r| (rounding of r) + 2^-62 (PAD_LO); otherwise, and for
// |s| outside [2^-10, 2^100) or a non-finite x, the FP64 sequence runs.  tests/test_pad_fp32.py
// restates this in numpy float32 and compares it bit for bit with the FP64 sequence on sweeps of
// float32 bit patterns; coordinates of magnitude 0.01 .. 4000 never take the fallback.
constexpr float PAD_HI = 0x1.a36e2ep-14f;
constexpr float PAD_LO = 0x1.638866p-39f;

template <bool UP>
__device__ __forceinline__ float pad_fp32(float x)
{
    const float h = UP ? PAD_HI : -PAD_HI;
    const float s = __fadd_rn(x, h);
    const float bb = __fsub_rn(s, x);
    const float e = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(h, bb));
    const float r = UP ? __fadd_rn(e, PAD_LO) : __fsub_rn(e, PAD_LO);
    const float as = fabsf(s);
    const float tol = 0x1p-50f * as + 0x1p-23f * fabsf(r) + 0x1p-62f;
    if (!(as >= 0x1p-10f && as < 0x1p100f) || !(fabsf(r) > tol)) return pad_fp64<UP>(x);
    const uint32_t sb = __float_as_uint(s);
    const bool away = UP ? r > 0.f : r < 0.f;   // the neighbour of s in the rounding direction
    const bool neg = (sb >> 31) != 0u;
    return away ? __uint_as_float((UP != neg) ? sb + 1u : sb - 1u) : s;
}

// Padded triangle box (AABB::pad, AABB.cuh:30-40) rounded outwards to FP32.  For FP32 vertices
// the minimum and maximum are exact in FP32; the padding is the reference's FP64 operation,
// evaluated by pad_fp32.
__device__ __forceinline__ void tri_box(const float p[9], float4& bmin, float4& bmax)
{
    float mn[3], mx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        mn[a] = fminf(fminf(p[a], p[3 + a]), p[6 + a]);
        mx[a] = fmaxf(fmaxf(p[a], p[3 + a]), p[6 + a]);
    }
    bmin = make_float4(pad_fp32<false>(mn[0]), pad_fp32<false>(mn[1]), pad_fp32<false>(mn[2]), 0.f);
    bmax = make_float4(pad_fp32<true>(mx[0]), pad_fp32<true>(mx[1]), pad_fp32<true>(mx[2]), 0.f);
}

template <typename VT>
__global__ void k_prep(uint32_t n_extra, const double* __restrict__ extra_c, const float4* __restrict__ extra_box,
                       uint32_t n_tri, const VT* __restrict__ tri_v, MortonAxis ax, MortonAxis ay, MortonAxis az,
                       uint32_t* __restrict__ code, uint32_t* __restrict__ idx, float4* __restrict__ box)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n = n_extra + n_tri;
    if (i >= n) return;
    float4 bmin, bmax;
    uint32_t xx, yy, zz;
    if (i < n_extra) {
        bmin = extra_box[2ull * i];
        bmax = extra_box[2ull * i + 1];
        xx = morton_axis(extra_c[3ull * i], ax.mn, ax.mx);
        yy = morton_axis(extra_c[3ull * i + 1], ay.mn, ay.mx);
        zz = morton_axis(extra_c[3ull * i + 2], az.mn, az.mx);
    } else if (sizeof(VT) == sizeof(float)) {
        const float* v = reinterpret_cast<const float*>(tri_v) + 9ull * (i - n_extra);
        float p[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) p[k] = __ldg(v + k);
        tri_box(p, bmin, bmax);
        xx = morton_tri_axis(p[0], p[3], p[6], ax);
        yy = morton_tri_axis(p[1], p[4], p[7], ay);
        zz = morton_tri_axis(p[2], p[5], p[8], az);
    } else {
        double p[9], c[3];
        load_tri(tri_v, i - n_extra, p);
        tri_center_box(p, c, bmin, bmax);
        xx = morton_axis(c[0], ax.mn, ax.mx);
        yy = morton_axis(c[1], ay.mn, ay.mx);
        zz = morton_axis(c[2], az.mn, az.mx);
    }
    code[i] = expand_bits(xx) * 4 + expand_bits(yy) * 2 + expand_bits(zz);
    idx[i] = i;
    box[2ull * i] = bmin;
    box[2ull * i + 1] = bmax;
}

template <typename VT>
__global__ void k_prim_boxes(uint32_t n_extra, const float4* __restrict__ extra_box, uint32_t n_tri,
                             const VT* __restrict__ tri_v, const uint32_t* __restrict__ order,
                             float4* __restrict__ leaf_box, uint32_t n)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t i = order[k];
    float4 bmin, bmax;
    if (i < n_extra) {
        bmin = extra_box[2ull * i];
        bmax = extra_box[2ull * i + 1];
    } else if (sizeof(VT) == sizeof(float)) {
        const float* v = reinterpret_cast<const float*>(tri_v) + 9ull * (i - n_extra);
        float p[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) p[q] = __ldg(v + q);
        tri_box(p, bmin, bmax);
    } else {
        double p[9], c[3];
        load_tri(tri_v, i - n_extra, p);
        tri_center_box(p, c, bmin, bmax);
    }
    leaf_box[2ull * k] = bmin;
    leaf_box[2ull * k + 1] = bmax;
}

// ---------------------------------------------------------------- radix sort
// Digit totals of all passes (they do not depend on the order): totals[pass][digit].
__global__ void k_digit_totals(const uint32_t* __restrict__ code, uint32_t n, uint32_t* __restrict__ totals)
{
    __shared__ uint32_t h[RS_PASSES][RS_BINS];
    for (int t = threadIdx.x; t < RS_PASSES * RS_BINS; t += blockDim.x) (&h[0][0])[t] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t c = code[i];
#pragma unroll
        for (int p = 0; p < RS_PASSES; ++p) atomicAdd(&h[p][(c >> (RS_BITS * p)) & RS_MASK], 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < RS_PASSES * RS_BINS; t += blockDim.x) {
        uint32_t v = (&h[0][0])[t];
        if (v) atomicAdd(&totals[t], v);
    }
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Per-tile digit counts, digit-major: counts[d * num_tiles + tile].  Each warp aggregates
// equal digits with __match_any_sync; the group leader adds to the warp's private row.
__global__ void __launch_bounds__(RS_THREADS) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                           uint32_t* __restrict__ counts, uint32_t num_tiles)
{
    __shared__ uint32_t wh[RS_WARPS][RS_BINS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int t = threadIdx.x; t < RS_WARPS * RS_BINS; t += RS_THREADS) (&wh[0][0])[t] = 0;
    __syncthreads();
    const uint32_t tile = blockIdx.x;
    const uint32_t base = tile * RS_TILE + w * 32 * RS_ITEMS;
#pragma unroll 4
    for (int it = 0; it < RS_ITEMS; ++it) {
        uint32_t e = base + it * 32 + lane;
        uint32_t d = e < n ? (keys[e] >> shift) & RS_MASK : (uint32_t)RS_BINS;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (d < (uint32_t)RS_BINS && lane == __ffs(peers) - 1) wh[w][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) {
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < RS_WARPS; ++k) s += wh[k][d];
        counts[(size_t)d * num_tiles + tile] = s;
    }
}

// Exclusive scan of counts into global offsets.  Block d scans row d and adds the number
// of keys with a smaller digit (from the pass's totals).
__global__ void __launch_bounds__(256) k_radix_scan(uint32_t* __restrict__ counts, uint32_t num_tiles,
                                                    const uint32_t* __restrict__ totals)
{
    __shared__ uint32_t s_part[8];
    __shared__ uint32_t s_carry;
    const int d = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t b = 0;
    for (int t = threadIdx.x; t < d; t += 256) b += totals[t];
#pragma unroll
    for (int o = 16; o; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
    if (lane == 0) s_part[w] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int k = 0; k < 8; ++k) s += s_part[k];
        s_carry = s;
    }
    __syncthreads();
    uint32_t* row = counts + (size_t)d * num_tiles;
    for (uint32_t start = 0; start < num_tiles; start += 256) {
        uint32_t i = start + threadIdx.x;
        uint32_t v = i < num_tiles ? row[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        __syncthreads();
        if (lane == 31) s_part[w] = x;
        __syncthreads();
        uint32_t wpre = 0;
        for (int k = 0; k < w; ++k) wpre += s_part[k];
        uint32_t carry = s_carry;
        if (i < num_tiles) row[i] = carry + wpre + x - v;
        __syncthreads();
        if (threadIdx.x == 255) s_carry = carry + wpre + x;
        __syncthreads();
    }
}

// Shared memory of the scatter kernel (73,760 bytes, dynamic: three blocks per SM).
struct ScatterSmem {
    uint32_t wh[RS_WARPS][RS_BINS];   // per-warp digit counts, then per-warp exclusive offsets
    uint32_t start[RS_BINS];          // tile-local start of each digit
    uint32_t gofs[RS_BINS];           // global start of each digit's run of this tile
    uint32_t keys[RS_TILE];
    uint32_t vals[RS_TILE];
    uint32_t wsum[RS_WARPS];
};

// Stable scatter: rank each key within its tile (warp-ordered, lane-ordered), stage the tile
// in shared memory in sorted order, then write runs to their global offsets.
__global__ void __launch_bounds__(RS_THREADS, 3) k_radix_scatter(const uint32_t* __restrict__ keys_in,
                                                              const uint32_t* __restrict__ vals_in,
                                                              uint32_t* __restrict__ keys_out,
                                                              uint32_t* __restrict__ vals_out, uint32_t n, int shift,
                                                              const uint32_t* __restrict__ offsets, uint32_t num_tiles)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ScatterSmem& S = *reinterpret_cast<ScatterSmem*>(smem_raw);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int t = threadIdx.x; t < RS_WARPS * RS_BINS; t += RS_THREADS) (&S.wh[0][0])[t] = 0;
    __syncthreads();
    const uint32_t tile = blockIdx.x;
    const uint32_t base = tile * RS_TILE + w * 32 * RS_ITEMS;
    const uint32_t lt = lanemask_lt();
    uint32_t k[RS_ITEMS], v[RS_ITEMS], rank[RS_ITEMS];
#pragma unroll
    for (int it = 0; it < RS_ITEMS; ++it) {
        uint32_t e = base + it * 32 + lane;
        bool valid = e < n;
        k[it] = valid ? keys_in[e] : 0u;
        v[it] = valid ? vals_in[e] : 0u;
        uint32_t d = valid ? (k[it] >> shift) & RS_MASK : (uint32_t)RS_BINS;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        int leader = __ffs(peers) - 1;
        uint32_t old = (lane == leader && valid) ? S.wh[w][d] : 0u;
        old = __shfl_sync(0xffffffffu, old, leader);
        if (lane == leader && valid) S.wh[w][d] = old + __popc(peers);
        rank[it] = old + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();
    // Digits RS_DPT * t .. RS_DPT * t + RS_DPT - 1 belong to thread t: exclusive prefix over warps
    // (in place), the tile's count of each, and their exclusive prefix within the thread.
    uint32_t local[RS_DPT];
    uint32_t tsum = 0;
#pragma unroll
    for (int j = 0; j < RS_DPT; ++j) {
        const int d = RS_DPT * threadIdx.x + j;
        uint32_t run = 0;
#pragma unroll
        for (int q = 0; q < RS_WARPS; ++q) {
            uint32_t c = S.wh[q][d];
            S.wh[q][d] = run;
            run += c;
        }
        local[j] = tsum;
        tsum += run;
        S.gofs[d] = offsets[(size_t)d * num_tiles + tile];
    }
    // Block exclusive scan of the threads' sums -> S.start.
    uint32_t x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) S.wsum[w] = x;
    __syncthreads();
    uint32_t wpre = 0;
    for (int q = 0; q < w; ++q) wpre += S.wsum[q];
#pragma unroll
    for (int j = 0; j < RS_DPT; ++j) S.start[RS_DPT * threadIdx.x + j] = wpre + x - tsum + local[j];
    __syncthreads();
#pragma unroll
    for (int it = 0; it < RS_ITEMS; ++it) {
        uint32_t e = base + it * 32 + lane;
        if (e < n) {
            uint32_t d = (k[it] >> shift) & RS_MASK;
            uint32_t pos = S.start[d] + S.wh[w][d] + rank[it];
            S.keys[pos] = k[it];
            S.vals[pos] = v[it];
        }
    }
    __syncthreads();
    uint32_t tile_n = min((uint32_t)RS_TILE, n - tile * RS_TILE);
    for (uint32_t p = threadIdx.x; p < tile_n; p += RS_THREADS) {
        uint32_t kk = S.keys[p];
        uint32_t d = (kk >> shift) & RS_MASK;
        uint32_t g = S.gofs[d] + (p - S.start[d]);
        keys_out[g] = kk;
        vals_out[g] = S.vals[p];
    }
}

// ---------------------------------------------------------------- Karras emission
// The reference's keys are code << 32 | primitive (Device.cuh:187-189), so the length of the common
// prefix of keys i and j (delta, BVH.cuh:120-128) is clz(code_i ^ code_j) when the codes differ and
// 32 + clz(prim_i ^ prim_j) when they are equal: the primitive word is read only then.
__device__ __forceinline__ int prefix_len(uint32_t ci, uint32_t oi, const uint32_t* __restrict__ code,
                                          const uint32_t* __restrict__ order, int j)
{
    const uint32_t cj = code[j];
    if (cj != ci) return __clz(ci ^ cj);
    const uint32_t oj = order[j];
    return oi == oj ? 64 : 32 + __clz(oi ^ oj);
}

__device__ __forceinline__ int delta_k(const uint32_t* code, const uint32_t* order, int n, uint32_t ci, uint32_t oi,
                                       int j)   // BVH.cuh:120-128
{
    if (j < 0 || j >= n) return -1;
    return prefix_len(ci, oi, code, order, j);
}

__global__ void k_emit(const uint32_t* __restrict__ code, const uint32_t* __restrict__ order, int n,
                       int2* __restrict__ child, int2* __restrict__ range)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n - 1) return;
    // determineRange (BVH.cuh:130-172)
    const uint32_t ci = code[idx], oi = order[idx];
    int dn = delta_k(code, order, n, ci, oi, idx + 1);
    int dp = delta_k(code, order, n, ci, oi, idx - 1);
    int d = (dn > dp) ? 1 : -1;
    int dmin_ = delta_k(code, order, n, ci, oi, idx - d);
    int lmax = 2;
    while (delta_k(code, order, n, ci, oi, idx + lmax * d) > dmin_) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta_k(code, order, n, ci, oi, idx + (l + t) * d) > dmin_) l += t;
    int j = idx + l * d;
    int first = min(idx, j), last = max(idx, j);
    // findSplit (BVH.cuh:81-118): equal keys split in the middle, otherwise binary search for the
    // last position that shares more than the range's common prefix with the first key
    const uint32_t cf = code[first], of = order[first];
    const int common = prefix_len(cf, of, code, order, last);
    int split;
    if (common == 64) {
        split = (first + last) >> 1;
    } else {
        split = first;
        int step = last - first;
        do {
            step = (step + 1) >> 1;
            int ns = split + step;
            if (ns < last) {
                if (prefix_len(cf, of, code, order, ns) > common) split = ns;
            }
        } while (step > 1);
    }
    int a = (split == first) ? ~split : split;
    int b = (split + 1 == last) ? ~(split + 1) : split + 1;
    child[idx] = make_int2(a, b);
    if (range) range[idx] = make_int2(first, last);
}

// ---------------------------------------------------------------- range-union refit
// The box pyramid: level 0 is the sorted leaf boxes (n of them); level l + 1 holds
// ceil(size(l) / 4) boxes, box j the union of boxes 4j .. 4j + 3 of level l; the levels above
// the leaves are stored back to back (two float4 per box) down to a level of one box.
__device__ __forceinline__ void box_union(float4& mn, float4& mx, float4 a, float4 b)
{
    mn.x = fminf(mn.x, a.x); mn.y = fminf(mn.y, a.y); mn.z = fminf(mn.z, a.z);
    mx.x = fmaxf(mx.x, b.x); mx.y = fmaxf(mx.y, b.y); mx.z = fmaxf(mx.z, b.z);
}

__device__ __forceinline__ void empty_box(float4& mn, float4& mx)
{
    mn = make_float4(INFINITY, INFINITY, INFINITY, 0.f);
    mx = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
}

__device__ __forceinline__ void shfl_union(float4& mn, float4& mx, int o)
{
    mn.x = fminf(mn.x, __shfl_xor_sync(0xffffffffu, mn.x, o));
    mn.y = fminf(mn.y, __shfl_xor_sync(0xffffffffu, mn.y, o));
    mn.z = fminf(mn.z, __shfl_xor_sync(0xffffffffu, mn.z, o));
    mx.x = fmaxf(mx.x, __shfl_xor_sync(0xffffffffu, mx.x, o));
    mx.y = fmaxf(mx.y, __shfl_xor_sync(0xffffffffu, mx.y, o));
    mx.z = fmaxf(mx.z, __shfl_xor_sync(0xffffffffu, mx.z, o));
}

__device__ __forceinline__ void store_box(float4* __restrict__ a, uint32_t j, float4 mn, float4 mx)
{
    a[2ull * j] = mn;
    a[2ull * j + 1] = mx;
}

constexpr int PYR_THREADS = 256;   // one block reduces 256 boxes: up to four levels per launch

// Writes the next `depth` (1 to 4) pyramid levels above a level of n boxes.  Thread t of block b
// holds box 256 b + t of that level (an empty box past n); `out` is the first level to write.
// Every thread of the block must call it (it shuffles and synchronises); depth is uniform.
__device__ __forceinline__ void pyramid_up(float4 mn, float4 mx, uint32_t n, float4* __restrict__ out, int depth)
{
    __shared__ float4 s_mn[PYR_THREADS / 16], s_mx[PYR_THREADS / 16];
    const uint32_t t = threadIdx.x, i = blockIdx.x * PYR_THREADS + t;
    shfl_union(mn, mx, 1);
    shfl_union(mn, mx, 2);
    const uint32_t n1 = (n + 3) / 4;
    if ((t & 3u) == 0 && (i >> 2) < n1) store_box(out, i >> 2, mn, mx);
    if (depth == 1) return;
    float4* out2 = out + 2ull * n1;
    shfl_union(mn, mx, 4);
    shfl_union(mn, mx, 8);
    const uint32_t n2 = (n1 + 3) / 4;
    if ((t & 15u) == 0 && (i >> 4) < n2) store_box(out2, i >> 4, mn, mx);
    if (depth == 2) return;
    if ((t & 15u) == 0) {
        s_mn[t >> 4] = mn;
        s_mx[t >> 4] = mx;
    }
    __syncthreads();
    if (t >= 32) return;
    // warp 0: lane L < 16 holds group L of 16 boxes
    if (t < PYR_THREADS / 16) {
        mn = s_mn[t];
        mx = s_mx[t];
    } else {
        empty_box(mn, mx);
    }
    float4* out3 = out2 + 2ull * n2;
    const uint32_t n3 = (n2 + 3) / 4;
    shfl_union(mn, mx, 1);
    shfl_union(mn, mx, 2);
    const uint32_t j3 = blockIdx.x * (PYR_THREADS / 64) + (t >> 2);
    if ((t & 3u) == 0 && t < PYR_THREADS / 16 && j3 < n3) store_box(out3, j3, mn, mx);
    if (depth == 3) return;
    float4* out4 = out3 + 2ull * n3;
    const uint32_t n4 = (n3 + 3) / 4;
    shfl_union(mn, mx, 4);
    shfl_union(mn, mx, 8);
    if (t == 0 && blockIdx.x < n4) store_box(out4, blockIdx.x, mn, mx);
}

// Pyramid levels above level `in` (n boxes), `depth` of them, starting at `out`.
__global__ void __launch_bounds__(PYR_THREADS) k_pyramid(const float4* __restrict__ in, uint32_t n,
                                                         float4* __restrict__ out, int depth)
{
    const uint32_t i = blockIdx.x * PYR_THREADS + threadIdx.x;
    float4 mn, mx;
    empty_box(mn, mx);
    if (i < n) {
        mn = in[2ull * i];
        mx = in[2ull * i + 1];
    }
    pyramid_up(mn, mx, n, out, depth);
}

// Sorted leaf boxes, (optionally) the reference's 64-bit keys, and (when `levels` is set) the
// first `depth` pyramid levels above them.
__global__ void __launch_bounds__(PYR_THREADS) k_leaves(const uint32_t* __restrict__ code,
                                                        const uint32_t* __restrict__ order, uint32_t n,
                                                        const float4* __restrict__ box_unsorted,
                                                        float4* __restrict__ leaf_box, uint64_t* __restrict__ keys,
                                                        float4* __restrict__ levels, int depth)
{
    const uint32_t k = blockIdx.x * PYR_THREADS + threadIdx.x;
    float4 mn, mx;
    empty_box(mn, mx);
    if (k < n) {
        const uint32_t p = order[k];
        mn = box_unsorted[2ull * p];
        mx = box_unsorted[2ull * p + 1];
        leaf_box[2ull * k] = mn;
        leaf_box[2ull * k + 1] = mx;
        if (keys) keys[k] = ((uint64_t)code[k] << 32) | p;
    }
    if (levels) pyramid_up(mn, mx, n, levels, depth);
}

// Union of leaf boxes [lo, hi) (exclusive hi) from the pyramid: at each level the partial groups
// at both ends (at most three boxes each), then up one level with the aligned middle; the last
// level visited holds at most six boxes of the range.  All loads of a level are independent, so
// a thread has up to six in flight at once.
__device__ __forceinline__ void range_union(const float4* __restrict__ leaves, const float4* __restrict__ levels,
                                            uint32_t n, int count, uint32_t lo, uint32_t hi, float4& mn, float4& mx)
{
    empty_box(mn, mx);
    const float4* a = leaves;
    const float4* next = levels;
    uint32_t na = n;
    for (int l = 0;; ++l) {
        const uint32_t lo_up = (lo + 3u) & ~3u, hi_dn = hi & ~3u;
        if (l == count || lo_up >= hi_dn) {
#pragma unroll
            for (uint32_t j = 0; j < 6; ++j)
                if (lo + j < hi) box_union(mn, mx, a[2ull * (lo + j)], a[2ull * (lo + j) + 1]);
            return;
        }
#pragma unroll
        for (uint32_t j = 0; j < 3; ++j) {
            if (lo + j < lo_up) box_union(mn, mx, a[2ull * (lo + j)], a[2ull * (lo + j) + 1]);
            if (hi_dn + j < hi) box_union(mn, mx, a[2ull * (hi_dn + j)], a[2ull * (hi_dn + j) + 1]);
        }
        lo = lo_up >> 2;
        hi = hi_dn >> 2;
        na = (na + 3) / 4;
        a = next;
        next += 2ull * na;
    }
}

// Node i's box = union of its sorted leaf range (min and max are exact, so the result equals the
// pairwise unions of the reference's bottom-up refit).
__global__ void k_node_boxes(const float4* __restrict__ leaves, const float4* __restrict__ levels, uint32_t n,
                             int count, const int2* __restrict__ range, float4* __restrict__ node_box)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int2 r = range[i];
    float4 mn, mx;
    range_union(leaves, levels, n, count, (uint32_t)r.x, (uint32_t)r.y + 1u, mn, mx);
    node_box[2ull * i] = mn;
    node_box[2ull * i + 1] = mx;
}

// ---------------------------------------------------------------- traversal layout
// BVH2 node i: (A.lo.x, A.hi.x, A.lo.y, A.hi.y), (B.lo.x, B.hi.x, B.lo.y, B.hi.y),
// (A.lo.z, A.hi.z, B.lo.z, B.hi.z), (childA, childB, 0, 0) — 64 bytes, four 16-byte loads.
__global__ void k_bvh2_nodes(const int2* __restrict__ child, const float4* __restrict__ node_box,
                             const float4* __restrict__ leaf_box, uint32_t n_internal, float4* __restrict__ nodes)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_internal) return;
    int2 c = child[i];
    const float4* ba = c.x < 0 ? leaf_box + 2ull * (uint32_t)(~c.x) : node_box + 2ull * (uint32_t)c.x;
    const float4* bb = c.y < 0 ? leaf_box + 2ull * (uint32_t)(~c.y) : node_box + 2ull * (uint32_t)c.y;
    float4 amn = ba[0], amx = ba[1], bmn = bb[0], bmx = bb[1];
    nodes[4ull * i + 0] = make_float4(amn.x, amx.x, amn.y, amx.y);
    nodes[4ull * i + 1] = make_float4(bmn.x, bmx.x, bmn.y, bmx.y);
    nodes[4ull * i + 2] = make_float4(amn.z, amx.z, bmn.z, bmx.z);
    nodes[4ull * i + 3] = make_float4(__int_as_float(c.x), __int_as_float(c.y), 0.f, 0.f);
}

// Compressed BVH2 node i (32 bytes, one memory sector per visit instead of two): both child boxes
// quantised outwards to 8 bits on a grid anchored at the node box's minimum (cpt_quant.cuh), and
// the split index of the Karras tree, whose children are always split and split + 1 (each a leaf
// or an internal node, as two flags say):
//   float4 q0: origin xyz; w = ex | ey << 8 | ez << 16 | leaf(A) << 24 | leaf(B) << 25
//   uint4  q1: x = A.lo.x | A.lo.y << 8 | A.lo.z << 16 | A.hi.x << 24
//              y = A.hi.y | A.hi.z << 8 | B.lo.x << 16 | B.lo.y << 24
//              z = B.lo.z | B.hi.x << 8 | B.hi.y << 16 | B.hi.z << 24
//              w = split
__global__ void k_bvh2_qnodes(const int2* __restrict__ child, const float4* __restrict__ node_box,
                              const float4* __restrict__ leaf_box, uint32_t n_internal, float4* __restrict__ nodes)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_internal) return;
    int2 c = child[i];
    const float4* ba = c.x < 0 ? leaf_box + 2ull * (uint32_t)(~c.x) : node_box + 2ull * (uint32_t)c.x;
    const float4* bb = c.y < 0 ? leaf_box + 2ull * (uint32_t)(~c.y) : node_box + 2ull * (uint32_t)c.y;
    const float4 amn = ba[0], amx = ba[1], bmn = bb[0], bmx = bb[1];
    const float ox = fminf(amn.x, bmn.x), oy = fminf(amn.y, bmn.y), oz = fminf(amn.z, bmn.z);
    const uint32_t ex = grid_exponent(ox, fmaxf(amx.x, bmx.x)), ey = grid_exponent(oy, fmaxf(amx.y, bmx.y)),
                   ez = grid_exponent(oz, fmaxf(amx.z, bmx.z));
    const float sx = inv_grid(ex), sy = inv_grid(ey), sz = inv_grid(ez);
    const uint32_t split = (uint32_t)(c.x < 0 ? ~c.x : c.x);
    const uint32_t flags = (c.x < 0 ? 1u : 0u) | (c.y < 0 ? 2u : 0u);
    const uint32_t w0 = q_lo(amn.x, ox, sx) | q_lo(amn.y, oy, sy) << 8 | q_lo(amn.z, oz, sz) << 16 | q_hi(amx.x, ox, sx) << 24;
    const uint32_t w1 = q_hi(amx.y, oy, sy) | q_hi(amx.z, oz, sz) << 8 | q_lo(bmn.x, ox, sx) << 16 | q_lo(bmn.y, oy, sy) << 24;
    const uint32_t w2 = q_lo(bmn.z, oz, sz) | q_hi(bmx.x, ox, sx) << 8 | q_hi(bmx.y, oy, sy) << 16 | q_hi(bmx.z, oz, sz) << 24;
    nodes[2ull * i] = make_float4(ox, oy, oz, __uint_as_float(ex | ey << 8 | ez << 16 | flags << 24));
    nodes[2ull * i + 1] = make_float4(__uint_as_float(w0), __uint_as_float(w1), __uint_as_float(w2), __uint_as_float(split));
}

// Triangle edge b - a of FP32 vertices, rounded once from the FP64 difference.  When both are
// normal and their exponents differ by at most 28, the difference of the two 24-bit significands
// spans at most 53 bits, so the FP64 subtraction is exact and one FP32 subtraction rounds the same
// exact value; so it is when either is zero.  Otherwise the FP64 sequence runs, out of line.
__device__ __noinline__ float edge64(float b, float a) { return (float)((double)b - (double)a); }

__device__ __forceinline__ float edge32(float b, float a)
{
    const int eb = (int)((__float_as_uint(b) >> 23) & 0xFFu), ea = (int)((__float_as_uint(a) >> 23) & 0xFFu);
    const bool normal = eb != 0 && eb != 0xFF && ea != 0 && ea != 0xFF;
    const bool zero = (__float_as_uint(b) << 1) == 0u || (__float_as_uint(a) << 1) == 0u;
    const bool finite = eb != 0xFF && ea != 0xFF;
    return ((normal && abs(eb - ea) <= 28) || (zero && finite)) ? __fsub_rn(b, a) : edge64(b, a);
}

// Leaf record k (48 bytes) for primitive order[k]:
//   triangle: (p0, id), (p1 - p0, TRI), (p2 - p0, 0)   edges formed in double, rounded once
//   sphere:   (centre, id), (radius, 0, 0, SPHERE), 0
//   light:    (0, 0, 0, id), (light index, 0, 0, LIGHT), 0
template <typename VT>
__global__ void k_leaf_records(const uint32_t* __restrict__ order, uint32_t n, uint32_t n_lights, uint32_t n_spheres,
                               const VT* __restrict__ tri_v, const float4* __restrict__ spheres,
                               float4* __restrict__ rec)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t p = order[k];
    float4 r0, r1, r2 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p < n_lights) {
        r0 = make_float4(0.f, 0.f, 0.f, __int_as_float((int)p));
        r1 = make_float4(__int_as_float((int)p), 0.f, 0.f, __int_as_float(CPT_KIND_LIGHT));
    } else if (p < n_lights + n_spheres) {
        float4 s = spheres[p - n_lights];
        r0 = make_float4(s.x, s.y, s.z, __int_as_float((int)p));
        r1 = make_float4(s.w, 0.f, 0.f, __int_as_float(CPT_KIND_SPHERE));
    } else if (sizeof(VT) == sizeof(float)) {
        const float* v = reinterpret_cast<const float*>(tri_v) + 9ull * (p - n_lights - n_spheres);
        float q[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) q[k] = __ldg(v + k);
        r0 = make_float4(q[0], q[1], q[2], __int_as_float((int)p));
        r1 = make_float4(edge32(q[3], q[0]), edge32(q[4], q[1]), edge32(q[5], q[2]), __int_as_float(CPT_KIND_TRI));
        r2 = make_float4(edge32(q[6], q[0]), edge32(q[7], q[1]), edge32(q[8], q[2]), 0.f);
    } else {
        double q[9];
        load_tri(tri_v, p - n_lights - n_spheres, q);
        r0 = make_float4((float)q[0], (float)q[1], (float)q[2], __int_as_float((int)p));
        r1 = make_float4((float)(q[3] - q[0]), (float)(q[4] - q[1]), (float)(q[5] - q[2]), __int_as_float(CPT_KIND_TRI));
        r2 = make_float4((float)(q[6] - q[0]), (float)(q[7] - q[1]), (float)(q[8] - q[2]), 0.f);
    }
    rec[3ull * k] = r0;
    rec[3ull * k + 1] = r1;
    rec[3ull * k + 2] = r2;
}

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

struct ScratchLayout {
    size_t code0, code1, val1, counts, totals, box_unsorted, levels, total;
    uint32_t num_tiles;
    int level_count;   // pyramid levels above the leaves (0 for a single leaf)
};

ScratchLayout layout_for(uint32_t n)
{
    ScratchLayout L;
    std::memset(&L, 0, sizeof L);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.num_tiles = (n + RS_TILE - 1) / RS_TILE;
    L.code0 = take((size_t)n * 4);
    // The sort's second key/value buffers and its tile counts are dead once the sort has ended;
    // the box pyramid, built after it, takes their place.
    const size_t n4 = align_up((size_t)n * 4, 256);
    const size_t counts = align_up((size_t)RS_BINS * std::max(1u, L.num_tiles) * 4, 256);
    const size_t sort_bytes = 2 * n4 + counts + (size_t)RS_PASSES * RS_BINS * 4;
    size_t lv_boxes = 0;
    for (uint32_t m = n; m > 1;) {
        m = (m + 3) / 4;
        lv_boxes += m;
        L.level_count++;
    }
    const size_t shared = take(std::max(sort_bytes, lv_boxes * 32));
    L.code1 = shared;
    L.val1 = shared + n4;
    L.counts = shared + 2 * n4;
    L.totals = shared + 2 * n4 + counts;
    L.levels = shared;
    L.box_unsorted = take((size_t)n * 32);
    L.total = off;
    return L;
}

// The pyramid above the sorted leaf boxes, from level `from` (1: the leaves' first level is
// already in the scratch), then the node boxes.
cpt_status refit_from_leaves(uint32_t n, const ScratchLayout& SL, char* base, const int2* range, float4* node_box,
                             const float4* leaf_box, cudaStream_t stream, int from = 0)
{
    if (n < 2) return CPT_OK;
    float4* levels = (float4*)(base + SL.levels);
    // walk to level `from`
    const float4* in = leaf_box;
    float4* out = levels;
    uint32_t m = n;
    for (int l = 0; l < from; ++l) {
        const uint32_t up = (m + 3) / 4;
        in = out;
        out += 2ull * up;
        m = up;
    }
    int launches = 1;
    for (int l = from; l < SL.level_count; l += 4) {
        const int depth = std::min(4, SL.level_count - l);
        k_pyramid<<<blocks_for(m, PYR_THREADS), PYR_THREADS, 0, stream>>>(in, m, out, depth);
        launches++;
        for (int d = 0; d < depth; ++d) {
            const uint32_t up = (m + 3) / 4;
            in = out;
            out += 2ull * up;
            m = up;
        }
    }
    k_node_boxes<<<blocks_for(n - 1, 256), 256, 0, stream>>>(leaf_box, levels, n, SL.level_count, range, node_box);
    add_launches(launches);
    CPT_CUDA(cudaGetLastError());
    return CPT_OK;
}

}  // namespace

size_t lbvh_scratch_bytes(uint32_t n) { return layout_for(std::max(n, 1u)).total; }

cpt_status lbvh_build(uint32_t n_extra, const double* extra_centroid, const float4* extra_box, uint32_t n_tri,
                      const float* tri_f32, const double* tri_f64, const double smin_in[3], const double smax_in[3],
                      const LbvhBuffers& out, void* scratch, size_t scratch_bytes, cudaStream_t stream,
                      LbvhTimings* timings)
{
    uint64_t n64 = (uint64_t)n_extra + n_tri;
    if (n64 == 0) return CPT_OK;
    if (n64 > 0x7fffffffull) return fail(CPT_ERR_INVALID_ARGUMENT, "lbvh_build: too many primitives");
    uint32_t n = (uint32_t)n64;
    if (n_tri && !tri_f32 && !tri_f64) return fail(CPT_ERR_INVALID_ARGUMENT, "lbvh_build: no triangle vertices");
    if (n_extra && (!extra_centroid || !extra_box)) return fail(CPT_ERR_INVALID_ARGUMENT, "lbvh_build: extra prims");
    if (!out.order || !out.leaf_box || (n > 1 && (!out.child || !out.node_box || !out.range)))
        return fail(CPT_ERR_INVALID_ARGUMENT, "lbvh_build: missing output buffer");
    ScratchLayout SL = layout_for(n);
    if (!scratch || scratch_bytes < SL.total || ((uintptr_t)scratch & 255u))
        return fail(CPT_ERR_INVALID_ARGUMENT, "lbvh_build: scratch too small or not 256-byte aligned");
    char* base = (char*)scratch;
    // Keys and values ping-pong between (code0, val0 = out.order) and (code1, val1); k_prep fills
    // the pair that makes the last pass end in out.order.
    uint32_t* code0 = (uint32_t*)(base + SL.code0);
    uint32_t* code1 = (uint32_t*)(base + SL.code1);
    uint32_t* val0 = out.order;
    uint32_t* val1 = (uint32_t*)(base + SL.val1);
    constexpr bool odd = (RS_PASSES & 1) != 0;
    uint32_t* kin = odd ? code1 : code0;
    uint32_t* vin = odd ? val1 : val0;
    uint32_t* kout = odd ? code0 : code1;
    uint32_t* vout = odd ? val0 : val1;
    uint32_t* counts = (uint32_t*)(base + SL.counts);
    uint32_t* totals = (uint32_t*)(base + SL.totals);
    float4* box_unsorted = (float4*)(base + SL.box_unsorted);

    // Device::buildBVH: expand the mesh bounds by 1, fall back to [-20,20]^3 (Device.cuh:174-181).
    double3 smin = make_double3(smin_in[0] - 1.0, smin_in[1] - 1.0, smin_in[2] - 1.0);
    double3 smax = make_double3(smax_in[0] + 1.0, smax_in[1] + 1.0, smax_in[2] + 1.0);
    if (smin.x > smax.x) {
        smin = make_double3(-20.0, -20.0, -20.0);
        smax = make_double3(20.0, 20.0, 20.0);
    }

    cudaEvent_t ev[5];
    if (timings)
        for (auto& e : ev) CPT_CUDA(cudaEventCreate(&e));
    if (timings) CPT_CUDA(cudaEventRecord(ev[0], stream));
    auto axis = [](double mn, double mx) {
        MortonAxis m;
        m.mn = mn;
        m.mx = mx;
        m.k64 = 1024.0 / (mx - mn);
        m.mn32 = (float)mn;
        m.k32 = (float)m.k64;
        m.mn_lo = (float)(mn - (double)m.mn32);
        m.k_lo = (float)(m.k64 - (double)m.k32);
        return m;
    };
    const MortonAxis ax = axis(smin.x, smax.x), ay = axis(smin.y, smax.y), az = axis(smin.z, smax.z);
    if (tri_f64)
        k_prep<double><<<blocks_for(n, 256), 256, 0, stream>>>(n_extra, extra_centroid, extra_box, n_tri, tri_f64, ax,
                                                               ay, az, kin, vin, box_unsorted);
    else
        k_prep<float><<<blocks_for(n, 256), 256, 0, stream>>>(n_extra, extra_centroid, extra_box, n_tri, tri_f32, ax,
                                                              ay, az, kin, vin, box_unsorted);
    CPT_CUDA(cudaGetLastError());
    add_launches(1);
    if (timings) CPT_CUDA(cudaEventRecord(ev[1], stream));

    // Radix sort: RS_PASSES passes of RS_BITS bits, ending in code0/val0 (= out.order).
    CPT_CUDA(cudaMemsetAsync(totals, 0, RS_PASSES * RS_BINS * 4, stream));
    k_digit_totals<<<std::min(blocks_for(n, 256), 1024u), 256, 0, stream>>>(kin, n, totals);
    CPT_CUDA(cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(ScatterSmem)));
    CPT_CUDA(cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  cudaSharedmemCarveoutMaxShared));
    CPT_CUDA(cudaFuncSetAttribute(k_radix_hist, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  cudaSharedmemCarveoutMaxShared));
    for (int p = 0; p < RS_PASSES; ++p) {
        k_radix_hist<<<SL.num_tiles, RS_THREADS, 0, stream>>>(kin, n, RS_BITS * p, counts, SL.num_tiles);
        k_radix_scan<<<RS_BINS, 256, 0, stream>>>(counts, SL.num_tiles, totals + p * RS_BINS);
        k_radix_scatter<<<SL.num_tiles, RS_THREADS, sizeof(ScatterSmem), stream>>>(kin, vin, kout, vout, n, RS_BITS * p,
                                                                                  counts, SL.num_tiles);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    CPT_CUDA(cudaGetLastError());
    add_launches(1 + 3 * RS_PASSES);
    if (timings) CPT_CUDA(cudaEventRecord(ev[2], stream));

    // Emission + sorted leaf boxes.
    if (n > 1) k_emit<<<blocks_for(n - 1, 256), 256, 0, stream>>>(kin, vin, (int)n, out.child, out.range);
    const int depth = std::min(4, SL.level_count);
    float4* levels = depth > 0 ? (float4*)(base + SL.levels) : nullptr;
    k_leaves<<<blocks_for(n, PYR_THREADS), PYR_THREADS, 0, stream>>>(kin, vin, n, box_unsorted, out.leaf_box,
                                                                    out.keys, levels, depth);
    CPT_CUDA(cudaGetLastError());
    add_launches((n > 1 ? 1 : 0) + 1);
    if (timings) CPT_CUDA(cudaEventRecord(ev[3], stream));

    cpt_status st = refit_from_leaves(n, SL, base, out.range, out.node_box, out.leaf_box, stream, depth);
    if (st != CPT_OK) return st;
    if (timings) {
        CPT_CUDA(cudaEventRecord(ev[4], stream));
        CPT_CUDA(cudaEventSynchronize(ev[4]));
        CPT_CUDA(cudaEventElapsedTime(&timings->ms_prep, ev[0], ev[1]));
        CPT_CUDA(cudaEventElapsedTime(&timings->ms_sort, ev[1], ev[2]));
        CPT_CUDA(cudaEventElapsedTime(&timings->ms_emit, ev[2], ev[3]));
        CPT_CUDA(cudaEventElapsedTime(&timings->ms_refit, ev[3], ev[4]));
        for (auto& e : ev) cudaEventDestroy(e);
    }
    return CPT_OK;
}

cpt_status lbvh_leaf_boxes(uint32_t n_extra, const float4* extra_box, uint32_t n_tri, const float* tri_f32,
                           const double* tri_f64, const uint32_t* order, float4* leaf_box, uint32_t n,
                           cudaStream_t stream)
{
    if (n == 0) return CPT_OK;
    if (tri_f64)
        k_prim_boxes<double><<<blocks_for(n, 256), 256, 0, stream>>>(n_extra, extra_box, n_tri, tri_f64, order, leaf_box, n);
    else
        k_prim_boxes<float><<<blocks_for(n, 256), 256, 0, stream>>>(n_extra, extra_box, n_tri, tri_f32, order, leaf_box, n);
    CPT_CUDA(cudaGetLastError());
    add_launches(1);
    return CPT_OK;
}

cpt_status lbvh_refit(uint32_t n, const LbvhBuffers& out, void* scratch, size_t scratch_bytes, cudaStream_t stream)
{
    ScratchLayout SL = layout_for(std::max(n, 1u));
    if (!scratch || scratch_bytes < SL.total) return fail(CPT_ERR_INVALID_ARGUMENT, "lbvh_refit: scratch too small");
    return refit_from_leaves(n, SL, (char*)scratch, out.range, out.node_box, out.leaf_box, stream);
}

cpt_status build_trace_layout(uint32_t n, uint32_t n_lights, uint32_t n_spheres, const int2* child,
                              const float4* node_box, const float4* leaf_box, const uint32_t* order,
                              const float* tri_f32, const double* tri_f64, const float4* spheres, float4* nodes,
                              float4* leaf_rec, cudaStream_t stream, bool compressed)
{
    if (n == 0) return CPT_OK;
    if (n > 1 && nodes && compressed)
        k_bvh2_qnodes<<<blocks_for(n - 1, 256), 256, 0, stream>>>(child, node_box, leaf_box, n - 1, nodes);
    else if (n > 1 && nodes)
        k_bvh2_nodes<<<blocks_for(n - 1, 256), 256, 0, stream>>>(child, node_box, leaf_box, n - 1, nodes);
    if (tri_f64)
        k_leaf_records<double><<<blocks_for(n, 256), 256, 0, stream>>>(order, n, n_lights, n_spheres, tri_f64, spheres,
                                                                       leaf_rec);
    else
        k_leaf_records<float><<<blocks_for(n, 256), 256, 0, stream>>>(order, n, n_lights, n_spheres, tri_f32, spheres,
                                                                      leaf_rec);
    CPT_CUDA(cudaGetLastError());
    add_launches((n > 1 && nodes ? 1 : 0) + 1);
    return CPT_OK;
}

}  // namespace cpt

// ---------------------------------------------------------------- C ABI (low level)
CPT_EXPORT size_t cpt_lbvh_scratch_bytes(uint32_t num_prims) { return cpt::lbvh_scratch_bytes(num_prims); }

CPT_EXPORT cpt_status cpt_lbvh_build_device(uint32_t num_extra, const double* extra_centroids, const float* extra_boxes,
                                            uint32_t num_tri, const float* tri_vertices, const double scene_min[3],
                                            const double scene_max[3], uint64_t* out_keys, uint32_t* out_order,
                                            int32_t* out_children, int32_t* out_node_range, float* out_node_boxes,
                                            float* out_leaf_boxes, void* scratch, size_t scratch_bytes, void* stream)
{
    if (!scene_min || !scene_max) return cpt::fail(CPT_ERR_INVALID_ARGUMENT, "cpt_lbvh_build_device: bounds");
    cpt::LbvhBuffers b;
    b.keys = out_keys;
    b.order = out_order;
    b.child = (int2*)out_children;
    b.range = (int2*)out_node_range;
    b.node_box = (float4*)out_node_boxes;
    b.leaf_box = (float4*)out_leaf_boxes;
    return cpt::lbvh_build(num_extra, extra_centroids, (const float4*)extra_boxes, num_tri, tri_vertices, nullptr,
                           scene_min, scene_max, b, scratch, scratch_bytes, (cudaStream_t)stream, nullptr);
}

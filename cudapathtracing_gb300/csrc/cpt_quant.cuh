// cpt_quant.cuh — power-of-two grids for quantised child boxes (the 8-wide BVH and the compressed
// binary nodes).  A node's children are stored as 8-bit offsets on a grid anchored at the node
// box's minimum with 255 steps of 2^(e-127) across each axis; quantisation rounds outwards, so
// every stored box contains the child's FP32 box.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cpt {

// Biased exponent e such that 255 * 2^(e-127) >= extent (extent >= 0).
__device__ __forceinline__ uint32_t grid_exponent(float lo, float hi)
{
    float ext = __fsub_ru(hi, lo);
    float x = __fdiv_ru(ext, 255.0f);
    int e = 0;
    if (x > 0.0f) frexpf(x, &e);   // x = m * 2^e with m in [0.5, 1): 2^e > x
    e = max(-126, min(127, e));
    return (uint32_t)(e + 127);
}

__device__ __forceinline__ uint32_t q_lo(float v, float p, float inv_scale)
{
    float t = floorf(__fmul_rd(__fsub_rd(v, p), inv_scale));
    return (uint32_t)fminf(fmaxf(t, 0.0f), 255.0f);
}

__device__ __forceinline__ uint32_t q_hi(float v, float p, float inv_scale)
{
    float t = ceilf(__fmul_ru(__fsub_ru(v, p), inv_scale));
    return (uint32_t)fminf(fmaxf(t, 0.0f), 255.0f);
}

__device__ __forceinline__ float inv_grid(uint32_t e) { return __int_as_float((int)((254u - e) << 23)); }

}  // namespace cpt

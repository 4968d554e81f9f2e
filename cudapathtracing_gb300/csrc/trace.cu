// trace.cu — batched closest-hit queries (traverseIterative, BVH.cuh:282-332, called by the
// reference for camera, bounce, shadow and volume rays): one thread per ray.
#include <cuda_runtime.h>

#include "cpt_internal.h"
#include "cpt_trace.cuh"

namespace cpt {

namespace {

template <bool WIDE>
__global__ void k_trace(SceneView s, const float4* __restrict__ rays, uint64_t n, float4* __restrict__ hits, int* err)
{
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
    Hit h;
    bool hit = trace_closest<WIDE>(s, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), a.w, b.w, h, err);
    int prim = hit ? __float_as_int(ldg4(s.leaf_rec + 3 * (size_t)h.leaf).w) : -1;
    hits[i] = make_float4(hit ? h.t : -1.0f, __int_as_float(prim), h.u, h.v);
}

// Persistent BVH2 variant: warps fetch rays dynamically (trace_items_bvh2), so lanes whose ray
// finished take new rays instead of idling until the warp's slowest ray is done.
__global__ void __launch_bounds__(128) k_trace_dyn(SceneView s, const float4* __restrict__ rays, int n,
                                                   float4* __restrict__ hits, int* err, int* fetch)
{
    trace_items_bvh2<false>(
        s, n, fetch, err,
        [&](int i, float3& o, float3& d, float& tmn, float& tmx, int&) {
            float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
            o = f3(a.x, a.y, a.z);
            d = f3(b.x, b.y, b.z);
            tmn = a.w;
            tmx = b.w;
        },
        [&](int i, const Hit& h) {
            int prim = h.leaf >= 0 ? __float_as_int(ldg4(s.leaf_rec + 3 * (size_t)h.leaf).w) : -1;
            hits[i] = make_float4(h.leaf >= 0 ? h.t : -1.0f, __int_as_float(prim), h.u, h.v);
        });
}

// The same over the 8-wide BVH, with the group-entry stack's bottom entries in shared memory.
__global__ void __launch_bounds__(128) k_trace_dyn_wide(SceneView s, const float4* __restrict__ rays, int n,
                                                        float4* __restrict__ hits, int* err, int* fetch)
{
    trace_items_wide_views<false, ShortStack64<CPT_WIDE_SHORT_STACK>>(
        [&](int) -> const SceneView& { return s; }, n, fetch, err,
        [&](int i, float3& o, float3& d, float& tmn, float& tmx, int&, int&) {
            float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
            o = f3(a.x, a.y, a.z);
            d = f3(b.x, b.y, b.z);
            tmn = a.w;
            tmx = b.w;
        },
        [&](int i, const Hit& h, int) {
            int prim = h.leaf >= 0 ? __float_as_int(ldg4(s.leaf_rec + 3 * (size_t)h.leaf).w) : -1;
            hits[i] = make_float4(h.leaf >= 0 ? h.t : -1.0f, __int_as_float(prim), h.u, h.v);
        });
}

}  // namespace

cpt_status launch_trace(const SceneView& view, const cpt_ray* rays, uint64_t n, cpt_hit* hits, int* d_err,
                        cudaStream_t stream)
{
    if (n == 0) return CPT_OK;
    if (((uintptr_t)rays & 15u) || ((uintptr_t)hits & 15u))
        return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_trace_closest: rays and hits must be 16-byte aligned");
    const unsigned T = 128;
    const size_t smem = short_stack_bytes(T);
    uint64_t blocks = (n + T - 1) / T;
    if (blocks > 0x7fffffffull) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_trace_closest: too many rays");
    if (!view.wide && view.n_internal > 0 && n < 0x7fffffffull) {
        int dev = 0, sms = 0, per_sm = 0;
        CPT_CUDA(cudaGetDevice(&dev));
        CPT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_dyn, T, smem));
        int* fetch = d_err + 1;   // the scene's work counter
        CPT_CUDA(cudaMemsetAsync(fetch, 0, sizeof(int), stream));
        k_trace_dyn<<<std::max(1, per_sm) * sms, T, smem, stream>>>(view, (const float4*)rays, (int)n, (float4*)hits,
                                                                    d_err, fetch);
    } else if (view.wide && view.n_internal > 0 && n < 0x7fffffffull) {
        const size_t wsmem = wide_short_stack_bytes(T);
        int dev = 0, sms = 0, per_sm = 0;
        CPT_CUDA(cudaGetDevice(&dev));
        CPT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_dyn_wide, T, wsmem));
        int* fetch = d_err + 1;
        CPT_CUDA(cudaMemsetAsync(fetch, 0, sizeof(int), stream));
        k_trace_dyn_wide<<<std::max(1, per_sm) * sms, T, wsmem, stream>>>(view, (const float4*)rays, (int)n,
                                                                          (float4*)hits, d_err, fetch);
    } else if (view.wide)
        k_trace<true><<<(unsigned)blocks, T, smem, stream>>>(view, (const float4*)rays, n, (float4*)hits, d_err);
    else
        k_trace<false><<<(unsigned)blocks, T, smem, stream>>>(view, (const float4*)rays, n, (float4*)hits, d_err);
    CPT_CUDA(cudaGetLastError());
    add_launches(1);
    return CPT_OK;
}

}  // namespace cpt

// lbvh_static.cu — cpt_lbvh_build_device_static: the device-pointer LBVH build with its
// scratch memory in a fixed array compiled into this library, for callers that cannot
// allocate device memory themselves.
//
// Who needs it: a host that has already divided all of its device memory among its own pools
// (an engine or render server that reserves HBM at start-up and hands out nothing afterwards),
// and code running where an allocation is not allowed to happen — a real-time frame loop with a
// fixed memory budget, or a callback where cudaMalloc's implicit device synchronisation would
// stall the work in flight.  Such a caller can still pass its inputs and outputs; only the
// scratch (sort buffers, tile histograms, box hierarchy) must come from somewhere else.
//
// The scratch is g_lbvh_scratch below: 3 MiB of device memory that every GPU which loads this
// library keeps until the process exits.  It holds the scratch of builds of up to
// CPT_LBVH_STATIC_MAX_PRIMS (65,536) primitives; larger builds are rejected.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>

#include "cpt_internal.h"

namespace {

constexpr size_t kStaticScratchBytes = 3u << 20;

// File-scope device array.  In host code this name is only a stand-in for the symbol, not a
// device address; its address is obtained per context with cudaGetSymbolAddress.
__device__ __align__(256) unsigned char g_lbvh_scratch[kStaticScratchBytes];

// The device address of g_lbvh_scratch belongs to the CUDA context it was looked up in: after
// cudaDeviceReset, or from another context on the same device, the array lives elsewhere.  The
// cache is therefore keyed on the context's process-unique ID (cuCtxGetId: an ID is never
// reused, so an entry of a destroyed context can never match a later one).
constexpr int kCacheSlots = 64;
struct ScratchAddr {
    unsigned long long ctx_id;
    void* addr;
};
std::mutex g_mu;
ScratchAddr g_cache[kCacheSlots] = {};
int g_cache_next = 0;

// Driver entry points resolved through the runtime (the library does not link libcuda).
struct CtxQueries {
    PFN_cuCtxGetCurrent_v4000 current = nullptr;
    PFN_cuCtxGetId_v12000 id = nullptr;
};

const CtxQueries& ctx_queries()
{
    static const CtxQueries q = [] {
        CtxQueries r;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult res;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &res) == cudaSuccess &&
            res == cudaDriverEntryPointSuccess)
            r.current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &res) == cudaSuccess &&
            res == cudaDriverEntryPointSuccess)
            r.id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
        cudaGetLastError();
        return r;
    }();
    return q;
}

// Address of g_lbvh_scratch in the calling thread's current context (the device selected with
// cudaSetDevice).  The first call in a context looks the address up with cudaGetSymbolAddress,
// which also creates the device's primary context if none is current yet; make that first call
// before any stream capture begins.  Later calls in the same context reuse the cached address.
cpt_status static_scratch(void** out)
{
    const CtxQueries& q = ctx_queries();
    if (!q.current || !q.id) return cpt::fail(CPT_ERR_UNSUPPORTED, "driver lacks cuCtxGetCurrent / cuCtxGetId");
    CUcontext c = nullptr;
    if (q.current(&c) != CUDA_SUCCESS) return cpt::fail(CPT_ERR_CUDA, "cuCtxGetCurrent failed");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!c) {
        // No context is current on this thread yet: the runtime's first device call makes the
        // primary context current.
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_lbvh_scratch);
        if (e != cudaSuccess) return cpt::cuda_fail(e, "cudaGetSymbolAddress(g_lbvh_scratch)");
        if (q.current(&c) != CUDA_SUCCESS || !c) return cpt::fail(CPT_ERR_CUDA, "no current CUDA context");
    }
    unsigned long long id = 0;
    if (q.id(c, &id) != CUDA_SUCCESS) return cpt::fail(CPT_ERR_CUDA, "cuCtxGetId failed");
    for (const ScratchAddr& a : g_cache) {
        if (a.addr && a.ctx_id == id) {
            *out = a.addr;
            return CPT_OK;
        }
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_lbvh_scratch);
    if (e != cudaSuccess) return cpt::cuda_fail(e, "cudaGetSymbolAddress(g_lbvh_scratch)");
    g_cache[g_cache_next] = {id, p};
    g_cache_next = (g_cache_next + 1) % kCacheSlots;
    *out = p;
    return CPT_OK;
}

}  // namespace

CPT_EXPORT cpt_status cpt_lbvh_build_device_static(uint32_t num_extra, const double* extra_centroids,
                                                   const float* extra_boxes, uint32_t num_tri, const float* tri_vertices,
                                                   const double scene_min[3], const double scene_max[3],
                                                   uint64_t* out_keys, uint32_t* out_order, int32_t* out_children,
                                                   int32_t* out_node_range, float* out_node_boxes,
                                                   float* out_leaf_boxes, void* stream)
{
    uint64_t n = (uint64_t)num_extra + num_tri;
    if (n > CPT_LBVH_STATIC_MAX_PRIMS)
        return cpt::fail(CPT_ERR_INVALID_ARGUMENT,
                         "cpt_lbvh_build_device_static: at most 65536 primitives (its fixed scratch is 3 MiB); "
                         "use cpt_lbvh_build_device with caller-provided scratch for larger builds");
    if (!scene_min || !scene_max) return cpt::fail(CPT_ERR_INVALID_ARGUMENT, "cpt_lbvh_build_device_static: bounds");
    if (cpt::lbvh_scratch_bytes((uint32_t)n) > kStaticScratchBytes)
        return cpt::fail(CPT_ERR_INVALID_ARGUMENT, "cpt_lbvh_build_device_static: scratch does not fit");
    void* scratch = nullptr;
    cpt_status st = static_scratch(&scratch);
    if (st != CPT_OK) return st;
    cpt::LbvhBuffers b;
    b.keys = out_keys;
    b.order = out_order;
    b.child = (int2*)out_children;
    b.range = (int2*)out_node_range;
    b.node_box = (float4*)out_node_boxes;
    b.leaf_box = (float4*)out_leaf_boxes;
    // The build clears the digit totals it accumulates into; every other scratch word is written
    // before it is read, so the previous call's contents do no harm.
    return cpt::lbvh_build(num_extra, extra_centroids, (const float4*)extra_boxes, num_tri, tri_vertices, nullptr,
                           scene_min, scene_max, b, scratch, kStaticScratchBytes, (cudaStream_t)stream, nullptr);
}

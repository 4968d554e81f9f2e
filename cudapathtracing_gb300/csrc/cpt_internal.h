// cpt_internal.h — host-side internals of libcpt.so shared between translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "cpt.h"
#include "cpt_device.cuh"

#define CPT_EXPORT extern "C" __attribute__((visibility("default")))

namespace cpt {

// Thread-local text of the last failure (cpt_last_error_string).
void set_error(const std::string& msg);
cpt_status fail(cpt_status st, const std::string& msg);
cpt_status cuda_fail(cudaError_t e, const char* what);

#define CPT_CUDA(call)                                             \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return ::cpt::cuda_fail(_e, #call); \
    } while (0)

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Count of kernels this library has launched since it was loaded (cpt_launch_count).
void add_launches(uint64_t k);

// ---- LBVH build on caller-provided device buffers (lbvh.cu)
struct LbvhBuffers {
    uint64_t* keys;       // N, optional
    uint32_t* order;      // N
    int2* child;          // N-1: (child A, child B), leaf k encoded as ~k
    int2* range;          // N-1: (first, last), optional
    float4* node_box;     // 2*(N-1): min (w = 0), max
    float4* leaf_box;     // 2*N, sorted leaf order
};

struct LbvhTimings {
    float ms_prep, ms_sort, ms_emit, ms_refit;
};

size_t lbvh_scratch_bytes(uint32_t n);

// Builds keys/order/topology/boxes.  Primitive i < n_extra takes its centroid (double) and
// box from the extra arrays; primitive n_extra + t is triangle t of tri_f32 or tri_f64.
cpt_status lbvh_build(uint32_t n_extra, const double* extra_centroid, const float4* extra_box, uint32_t n_tri,
                      const float* tri_f32, const double* tri_f64, const double smin[3], const double smax[3],
                      const LbvhBuffers& out, void* scratch, size_t scratch_bytes, cudaStream_t stream,
                      LbvhTimings* timings);

// Range-union refit only (topology and ranges kept, boxes recomputed from new leaf boxes).
cpt_status lbvh_refit(uint32_t n, const LbvhBuffers& out, void* scratch, size_t scratch_bytes, cudaStream_t stream);

// Leaf boxes in sorted order for a refit: prim boxes recomputed from the vertices.
cpt_status lbvh_leaf_boxes(uint32_t n_extra, const float4* extra_box, uint32_t n_tri, const float* tri_f32,
                           const double* tri_f64, const uint32_t* order, float4* leaf_box, uint32_t n,
                           cudaStream_t stream);

// ---- traversal layout (lbvh.cu)
// BVH2 nodes (4 float4 per internal node, or 2 when compressed: 8-bit quantised child boxes) and
// leaf records (3 float4 per leaf).
cpt_status build_trace_layout(uint32_t n, uint32_t n_lights, uint32_t n_spheres, const int2* child,
                              const float4* node_box, const float4* leaf_box, const uint32_t* order,
                              const float* tri_f32, const double* tri_f64, const float4* spheres, float4* nodes,
                              float4* leaf_rec, cudaStream_t stream, bool compressed = false);

// ---- trace / render launchers (trace.cu, render.cu)
cpt_status launch_trace(const SceneView& view, const cpt_ray* rays, uint64_t n, cpt_hit* hits, int* d_err,
                        cudaStream_t stream);

struct RenderArgs {
    int spp, estimator, max_depth, rr_depth;
    float rr_prob;
    uint64_t seed;
    int row_begin, row_end;
    int flags;
    float* rgb;
    uint8_t* rgba8;
    float* gbuf;
    unsigned long long* ray_counter;
    int* err;
    int iter_limit;   // loop trips per sample before the error word is set (CPT_ITER_LIMIT by default)
};

// Default bounds of the device loops: trips per sample of a path loop, and wavefront graph
// replays per render (cpt_context_set_loop_limits lowers them).
constexpr int CPT_ITER_LIMIT = 1 << 16;
constexpr int CPT_MAX_REPLAYS = 1 << 20;

cpt_status launch_render_megakernel(const SceneView& view, const RenderArgs& args, cudaStream_t stream, int block_x,
                                    int block_y);

// Wavefront integrator launch shape (the autotuner's knobs) and graph-capture resources.
struct WavefrontTuning {
    int slots;                   // path slots (the wavefront size)
    int grid_trace, block_trace; // persistent grids (grid_trace_wide: the 8-wide trace kernels)
    int grid_trace_wide;
    int grid_shade, block_shade;
    int short_stack;             // traversal stack entries kept in shared memory (8, 16, 24, 32)
    bool use_graph;
    bool material_sort;          // shade slots binned by the material their ray hit
    int max_replays;             // iteration chunks replayed before the render gives up (CPT_ERR_TIMEOUT)
    cudaStream_t capture_stream; // non-default stream used only to capture the iteration graph
    cudaStream_t side_stream;    // second capture stream: shadow rays traced beside extension rays
    cudaEvent_t fork, join;      // capture-time dependencies between the two streams
};

cpt_status launch_render_wavefront(const SceneView& view, const RenderArgs& args, cudaStream_t stream,
                                   const WavefrontTuning& tune);
// Several renders (jobs) in one wavefront; every job's args share ray_counter and err with args[0],
// and every view has the same traversal layout.
cpt_status launch_render_wavefront_batch(const SceneView* views, const RenderArgs* args, int n_jobs,
                                         cudaStream_t stream, const WavefrontTuning& tune);

// The reference's joint-bilateral and temporal filters (filter.cu); device buffers.
DevCamera camera_of(const cpt_camera& c);
cpt_status filter_bilateral(const float* rgb, const float* gbuf, float* out, int W, int H, const cpt_filter_params& p,
                            cudaStream_t stream);
cpt_status filter_temporal(float* rgb, const float* prev, const float* gbuf, const cpt_camera& cam,
                           const cpt_camera& prev_cam, float alpha, cudaStream_t stream);

}  // namespace cpt

// wide.cu — collapses the binary LBVH into a compressed 8-wide BVH for traversal.
//
// Each wide node stands for one binary node b: starting from b's two children, the child with
// the largest surface area that is an internal binary node is replaced by its two children until
// there are 8 children or only leaves remain.  Children are then placed in slots by direction:
// slot s (bits: negative x, y, z) holds the child whose centroid offset from the node's centre
// points most along (+-1, +-1, +-1)_s (greedy assignment), so that a ray of octant o meets the
// children roughly in the order of slots s ^ (7 ^ o) — the ordering scheme of compressed wide
// BVHs (Ylitie, Karras, Laine 2017), which needs no sort during traversal.
//
// Node layout (128 bytes, eight 16-byte loads):
//   float4 f0   origin p.xyz (node box minimum); w = ex | ey << 8 | ez << 16 | imask << 24
//               (biased grid exponents, bit s of imask: slot s is an internal child)
//   uint4  f1   x = first internal child's wide index, y = first leaf slot,
//               z/w = meta bytes of slots 0..7: 0xFF empty, 0x80 | r internal child r, r leaf r
//   f2..f7      16-bit quantised child boxes, 8 slots each: lo.x, hi.x, lo.y, hi.y, lo.z, hi.z
//
// Child boxes sit on a power-of-two grid anchored at p with 65535 steps across the node, rounded
// outwards, so every quantised box contains the child's FP32 box.  Internal children and leaf
// children are numbered in slot order; leaf records are rewritten in leaf-slot order.
#include <cuda_runtime.h>

#include <algorithm>

#include "cpt_internal.h"

namespace cpt {

namespace {

__device__ __forceinline__ float area(float4 mn, float4 mx)
{
    float dx = mx.x - mn.x, dy = mx.y - mn.y, dz = mx.z - mn.z;
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ void ref_box(int ref, const float4* node_box, const float4* leaf_box, float4& mn, float4& mx)
{
    const float4* b = ref < 0 ? leaf_box + 2 * (size_t)(~ref) : node_box + 2 * (size_t)ref;
    mn = b[0];
    mx = b[1];
}

// Biased exponent e such that 65535 * 2^(e-127) >= extent (extent >= 0).
__device__ __forceinline__ uint32_t grid_exponent(float lo, float hi)
{
    float ext = __fsub_ru(hi, lo);
    float x = __fdiv_ru(ext, 65535.0f);
    int e = 0;
    if (x > 0.0f) frexpf(x, &e);   // x = m * 2^e with m in [0.5, 1): 2^e > x
    e = max(-126, min(127, e));
    return (uint32_t)(e + 127);
}

__device__ __forceinline__ uint32_t q_lo(float v, float p, float inv_scale)
{
    float t = floorf(__fmul_rd(__fsub_rd(v, p), inv_scale));
    return (uint32_t)fminf(fmaxf(t, 0.0f), 65535.0f);
}

__device__ __forceinline__ uint32_t q_hi(float v, float p, float inv_scale)
{
    float t = ceilf(__fmul_ru(__fsub_ru(v, p), inv_scale));
    return (uint32_t)fminf(fmaxf(t, 0.0f), 65535.0f);
}

__device__ __forceinline__ float inv_grid(uint32_t e) { return __int_as_float((int)((254u - e) << 23)); }

__global__ void k_collapse_level(const int2* __restrict__ child, const float4* __restrict__ node_box,
                                 const float4* __restrict__ leaf_box, const int2* __restrict__ tasks_in,
                                 const int* __restrict__ n_in, int2* __restrict__ tasks_out, int* __restrict__ n_out,
                                 int* __restrict__ counters, float4* __restrict__ wide, uint32_t* __restrict__ leaf_perm)
{
    const int n = *n_in;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int2 task = tasks_in[t];
        int b = task.x, wi = task.y;
        int refs[8];
        int2 c = child[b];
        refs[0] = c.x;
        refs[1] = c.y;
        int nr = 2;
        while (nr < 8) {
            int best = -1;
            float best_a = -1.0f;
            for (int k = 0; k < nr; ++k) {
                if (refs[k] < 0) continue;
                float4 mn, mx;
                ref_box(refs[k], node_box, leaf_box, mn, mx);
                float a = area(mn, mx);
                if (a > best_a) {
                    best_a = a;
                    best = k;
                }
            }
            if (best < 0) break;
            int2 cc = child[refs[best]];
            refs[best] = cc.x;
            refs[nr++] = cc.y;
        }
        float4 nmn, nmx;
        ref_box(b, node_box, leaf_box, nmn, nmx);
        const float cx = 0.5f * (nmn.x + nmx.x), cy = 0.5f * (nmn.y + nmx.y), cz = 0.5f * (nmn.z + nmx.z);
        // greedy slot assignment by direction
        int slot_of[8];
        float dx[8], dy[8], dz[8];
        for (int k = 0; k < nr; ++k) {
            float4 mn, mx;
            ref_box(refs[k], node_box, leaf_box, mn, mx);
            dx[k] = 0.5f * (mn.x + mx.x) - cx;
            dy[k] = 0.5f * (mn.y + mx.y) - cy;
            dz[k] = 0.5f * (mn.z + mx.z) - cz;
            slot_of[k] = -1;
        }
        uint32_t used = 0;
        for (int round = 0; round < nr; ++round) {
            float best = INFINITY;
            int bk = -1, bs = -1;
            for (int k = 0; k < nr; ++k) {
                if (slot_of[k] >= 0) continue;
                for (int s = 0; s < 8; ++s) {
                    if ((used >> s) & 1u) continue;
                    float cost = -((s & 1 ? -dx[k] : dx[k]) + (s & 2 ? -dy[k] : dy[k]) + (s & 4 ? -dz[k] : dz[k]));
                    if (cost < best) {
                        best = cost;
                        bk = k;
                        bs = s;
                    }
                }
            }
            slot_of[bk] = bs;
            used |= 1u << bs;
        }
        int at_slot[8];
        for (int s = 0; s < 8; ++s) at_slot[s] = 0x7fffffff;   // empty
        for (int k = 0; k < nr; ++k) at_slot[slot_of[k]] = refs[k];
        int n_int = 0, n_leaf = 0;
        for (int k = 0; k < nr; ++k) (refs[k] >= 0 ? n_int : n_leaf)++;
        int cb = n_int ? atomicAdd(&counters[0], n_int) : 0;
        int lb = n_leaf ? atomicAdd(&counters[1], n_leaf) : 0;
        uint32_t ex = grid_exponent(nmn.x, nmx.x), ey = grid_exponent(nmn.y, nmx.y), ez = grid_exponent(nmn.z, nmx.z);
        float isx = inv_grid(ex), isy = inv_grid(ey), isz = inv_grid(ez);
        uint32_t meta[2] = {0xFFFFFFFFu, 0xFFFFFFFFu};
        uint32_t q[6][4];
        for (int a = 0; a < 6; ++a)
            for (int w = 0; w < 4; ++w) q[a][w] = 0;
        uint32_t imask = 0;
        int ri = 0, rl = 0;
        for (int s = 0; s < 8; ++s) {
            int ref = at_slot[s];
            if (ref == 0x7fffffff) continue;
            float4 mn, mx;
            ref_box(ref, node_box, leaf_box, mn, mx);
            uint32_t m;
            if (ref >= 0) {
                m = 0x80u | (uint32_t)ri;
                imask |= 1u << s;
                int slot = atomicAdd(n_out, 1);
                tasks_out[slot] = make_int2(ref, cb + ri);
                ri++;
            } else {
                m = (uint32_t)rl;
                leaf_perm[lb + rl] = (uint32_t)(~ref);
                rl++;
            }
            int word = s >> 2, sh = (s & 3) * 8;
            meta[word] = (meta[word] & ~(0xFFu << sh)) | (m << sh);
            int qw = s >> 1, qs = (s & 1) * 16;
            q[0][qw] |= q_lo(mn.x, nmn.x, isx) << qs;
            q[1][qw] |= q_hi(mx.x, nmn.x, isx) << qs;
            q[2][qw] |= q_lo(mn.y, nmn.y, isy) << qs;
            q[3][qw] |= q_hi(mx.y, nmn.y, isy) << qs;
            q[4][qw] |= q_lo(mn.z, nmn.z, isz) << qs;
            q[5][qw] |= q_hi(mx.z, nmn.z, isz) << qs;
        }
        float4* dst = wide + 8 * (size_t)wi;
        dst[0] = make_float4(nmn.x, nmn.y, nmn.z, __int_as_float((int)(ex | (ey << 8) | (ez << 16) | (imask << 24))));
        dst[1] = make_float4(__int_as_float(cb), __int_as_float(lb), __int_as_float((int)meta[0]),
                             __int_as_float((int)meta[1]));
        for (int a = 0; a < 6; ++a)
            dst[2 + a] = make_float4(__int_as_float((int)q[a][0]), __int_as_float((int)q[a][1]),
                                     __int_as_float((int)q[a][2]), __int_as_float((int)q[a][3]));
    }
}

__global__ void k_collapse_init(int2* tasks, int* n_tasks, int* counters)
{
    tasks[0] = make_int2(0, 0);   // binary root -> wide node 0
    n_tasks[0] = 1;
    n_tasks[1] = 0;
    counters[0] = 1;              // wide nodes allocated (the root)
    counters[1] = 0;              // leaf slots allocated
}

__global__ void k_zero(int* p) { *p = 0; }

// Leaf records in wide-leaf-slot order: slot j holds sorted leaf leaf_perm[j].
template <typename VT>
__global__ void k_wide_leaf_records(const uint32_t* __restrict__ leaf_perm, const uint32_t* __restrict__ order,
                                    uint32_t n, uint32_t n_lights, uint32_t n_spheres, const VT* __restrict__ tri_v,
                                    const float4* __restrict__ spheres, float4* __restrict__ rec)
{
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t p = order[leaf_perm[j]];
    float4 r0, r1, r2 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p < n_lights) {
        r0 = make_float4(0.f, 0.f, 0.f, __int_as_float((int)p));
        r1 = make_float4(__int_as_float((int)p), 0.f, 0.f, __int_as_float(CPT_KIND_LIGHT));
    } else if (p < n_lights + n_spheres) {
        float4 s = spheres[p - n_lights];
        r0 = make_float4(s.x, s.y, s.z, __int_as_float((int)p));
        r1 = make_float4(s.w, 0.f, 0.f, __int_as_float(CPT_KIND_SPHERE));
    } else {
        size_t t = p - n_lights - n_spheres;
        double q[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) q[k] = (double)tri_v[9 * t + k];
        r0 = make_float4((float)q[0], (float)q[1], (float)q[2], __int_as_float((int)p));
        r1 = make_float4((float)(q[3] - q[0]), (float)(q[4] - q[1]), (float)(q[5] - q[2]), __int_as_float(CPT_KIND_TRI));
        r2 = make_float4((float)(q[6] - q[0]), (float)(q[7] - q[1]), (float)(q[8] - q[2]), 0.f);
    }
    rec[3ull * j] = r0;
    rec[3ull * j + 1] = r1;
    rec[3ull * j + 2] = r2;
}

}  // namespace

size_t wide_scratch_bytes(uint32_t n)
{
    // two task queues of up to n entries, counters, the leaf permutation
    return align_up((size_t)n * 8, 256) * 2 + 256 + align_up((size_t)n * 4, 256);
}

cpt_status build_wide(uint32_t n, uint32_t n_lights, uint32_t n_spheres, const int2* child, const float4* node_box,
                      const float4* leaf_box, const uint32_t* order, const float* tri_f32, const double* tri_f64,
                      const float4* spheres, float4* wide, float4* leaf_rec, void* scratch, size_t scratch_bytes,
                      cudaStream_t stream, uint32_t* num_wide)
{
    if (n < 2) {
        if (num_wide) *num_wide = 0;
        return CPT_OK;
    }
    if (scratch_bytes < wide_scratch_bytes(n)) return fail(CPT_ERR_INVALID_ARGUMENT, "build_wide: scratch too small");
    char* p = (char*)scratch;
    int2* tasks[2];
    tasks[0] = (int2*)p;
    p += align_up((size_t)n * 8, 256);
    tasks[1] = (int2*)p;
    p += align_up((size_t)n * 8, 256);
    int* small = (int*)p;   // [0,1] task counts, [2,3] counters
    p += 256;
    uint32_t* leaf_perm = (uint32_t*)p;
    int* n_tasks = small;
    int* counters = small + 2;
    k_collapse_init<<<1, 1, 0, stream>>>(tasks[0], n_tasks, counters);
    add_launches(1);
    // Level by level; a level whose queue is empty returns at once.  The wide tree is no deeper
    // than the binary one (at most 65 levels for 64-bit keys); check the queue every 8 levels.
    int cur = 0;
    for (int level = 0; level < 72; ++level) {
        k_zero<<<1, 1, 0, stream>>>(n_tasks + (cur ^ 1));
        k_collapse_level<<<std::max(1u, std::min((n + 255) / 256, 4096u)), 256, 0, stream>>>(
            child, node_box, leaf_box, tasks[cur], n_tasks + cur, tasks[cur ^ 1], n_tasks + (cur ^ 1), counters, wide,
            leaf_perm);
        add_launches(2);
        cur ^= 1;
        if ((level & 7) == 7) {
            int h = 0;
            CPT_CUDA(cudaMemcpyAsync(&h, n_tasks + cur, sizeof(int), cudaMemcpyDeviceToHost, stream));
            CPT_CUDA(cudaStreamSynchronize(stream));
            if (h == 0) break;
        }
    }
    int hc[2] = {0, 0};
    CPT_CUDA(cudaMemcpyAsync(hc, counters, sizeof hc, cudaMemcpyDeviceToHost, stream));
    CPT_CUDA(cudaStreamSynchronize(stream));
    if (hc[1] != (int)n) return fail(CPT_ERR_STACK_OVERFLOW, "build_wide: collapse did not reach every leaf");
    if (tri_f64)
        k_wide_leaf_records<double><<<(n + 255) / 256, 256, 0, stream>>>(leaf_perm, order, n, n_lights, n_spheres,
                                                                         tri_f64, spheres, leaf_rec);
    else
        k_wide_leaf_records<float><<<(n + 255) / 256, 256, 0, stream>>>(leaf_perm, order, n, n_lights, n_spheres,
                                                                        tri_f32, spheres, leaf_rec);
    add_launches(1);
    CPT_CUDA(cudaGetLastError());
    if (num_wide) *num_wide = (uint32_t)hc[0];
    return CPT_OK;
}

}  // namespace cpt

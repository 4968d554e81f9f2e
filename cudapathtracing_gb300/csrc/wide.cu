// wide.cu — collapses the binary LBVH into a compressed 8-wide BVH for traversal.
//
// The collapse runs level by level from the root, one launch per level with no host round trip
// in between (the level counts and bases live on the device).  Wide nodes are numbered compactly
// in that breadth-first order: level l occupies [base_l, base_l + n_l), and the internal children of a node
// are numbered consecutively (one atomic per node reserves their block in the next level), so the
// reachable nodes fill [0, num_wide) with siblings side by side and the top levels packed together
// (the hot part of the tree stays within a few megabytes).  Leaves stay in sorted Morton order in the
// leaf records.  Each wide node stands for one binary node b; starting from b's two children,
// the child with the largest surface area that is an internal binary node is replaced by its two
// children until there are 8 children or only leaves remain.  Children are then placed in slots
// by direction: slot s (bits: negative x, y, z) holds the child whose centroid offset from the
// node's centre points most along (+-1, +-1, +-1)_s (greedy assignment), so that a ray of
// octant o meets the children roughly in the order of slots s ^ (7 ^ o) — the ordering scheme of
// compressed wide BVHs (Ylitie, Karras, Laine 2017), which needs no sort during traversal.
//
// Node layout (96 bytes, six 16-byte loads):
//   float4 f0   origin p.xyz (node box minimum); w = ex | ey << 8 | ez << 16 | imask << 24
//               (biased grid exponents; bit s of imask: slot s holds an internal child)
//   int4 f1,f2  child reference of slots 0..7: >= 0 wide (= binary) node, < 0 leaf ~k,
//               CPT_WIDE_EMPTY for an unused slot
//   f3,f4,f5    8-bit quantised child boxes: (lo slots 0-3, lo 4-7, hi 0-3, hi 4-7) for x, y, z
//
// Child boxes sit on a power-of-two grid anchored at p with 255 steps across the node, rounded
// outwards, so every quantised box contains the child's FP32 box.
#include <cuda_runtime.h>

#include <algorithm>

#include "cpt_internal.h"
#include "cpt_quant.cuh"

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


// Level l: the wide nodes [base, base + n) with base = level_base[l], n = level_count[l]; wide node
// w stands for binary node tasks[w].  Internal children get the next numbers in level l + 1, which
// starts at base + n (one atomic per node reserves their consecutive block).  The candidate
// children's references, boxes and areas stay in registers (every array is indexed with
// compile-time indices only), so each box is read once: an expansion costs two dependent loads
// (the expanded node's children, then their two boxes).
constexpr int COLLAPSE_THREADS = 128;
constexpr int MAX_WIDE_LEVELS = 80;

__global__ void __launch_bounds__(COLLAPSE_THREADS, 3) k_collapse_level(const int2* __restrict__ child,
                                                                     const float4* __restrict__ node_box,
                                                                     const float4* __restrict__ leaf_box,
                                                                     int* __restrict__ tasks,
                                                                     int* __restrict__ level_count,
                                                                     int* __restrict__ level_base, int l,
                                                                     float4* __restrict__ wide)
{
    const int n = level_count[l];
    const int base = level_base[l];
    if (blockIdx.x == 0 && threadIdx.x == 0) level_base[l + 1] = base + n;
    int* n_out = level_count + l + 1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int b = tasks[base + t];   // binary node
        int refs[8];
        float4 cmn[8], cmx[8];
        float car[8];
        const int2 c = child[b];
        float4 nmn, nmx;
        ref_box(b, node_box, leaf_box, nmn, nmx);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            refs[k] = CPT_WIDE_EMPTY;
            car[k] = -1.0f;
        }
        refs[0] = c.x;
        refs[1] = c.y;
        ref_box(c.x, node_box, leaf_box, cmn[0], cmx[0]);
        ref_box(c.y, node_box, leaf_box, cmn[1], cmx[1]);
        car[0] = area(cmn[0], cmx[0]);
        car[1] = area(cmn[1], cmx[1]);
        int nr = 2;
        // Replace the internal child of largest area by its two children (the first such child in
        // candidate order on ties) until there are 8 children or only leaves remain.
#pragma unroll
        for (int step = 0; step < 6; ++step) {
            int best = -1, best_ref = 0;
            float best_a = -1.0f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k < nr && refs[k] >= 0 && car[k] > best_a) {
                    best_a = car[k];
                    best = k;
                    best_ref = refs[k];
                }
            }
            if (best < 0) break;
            const int2 cc = child[best_ref];
            float4 amn, amx, bmn, bmx;
            ref_box(cc.x, node_box, leaf_box, amn, amx);
            ref_box(cc.y, node_box, leaf_box, bmn, bmx);
            const float aa = area(amn, amx), ab = area(bmn, bmx);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k == best) {
                    refs[k] = cc.x;
                    cmn[k] = amn;
                    cmx[k] = amx;
                    car[k] = aa;
                } else if (k == nr) {
                    refs[k] = cc.y;
                    cmn[k] = bmn;
                    cmx[k] = bmx;
                    car[k] = ab;
                }
            }
            ++nr;
        }
        const float cx = 0.5f * (nmn.x + nmx.x), cy = 0.5f * (nmn.y + nmx.y), cz = 0.5f * (nmn.z + nmx.z);
        // greedy slot assignment by direction: each round takes the (child, slot) pair of least cost
        float dx[8], dy[8], dz[8];
        int slot_of[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            dx[k] = 0.5f * (cmn[k].x + cmx[k].x) - cx;
            dy[k] = 0.5f * (cmn[k].y + cmx[k].y) - cy;
            dz[k] = 0.5f * (cmn[k].z + cmx[k].z) - cz;
            slot_of[k] = -1;
        }
        uint32_t used = 0;
        for (int round = 0; round < nr; ++round) {
            float best = INFINITY;
            int bk = -1, bs = -1;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k >= nr || slot_of[k] >= 0) continue;
#pragma unroll
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
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k == bk) slot_of[k] = bs;
            used |= 1u << bs;
        }
        // Internal children take consecutive wide numbers in slot order: the child in slot s is
        // number first_child + (internal children in slots below s).
        uint32_t imask = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < nr && refs[k] >= 0) imask |= 1u << slot_of[k];
        const int n_int = __popc(imask);
        const int first_child = n_int ? atomicAdd(n_out, n_int) : 0;
        const uint32_t ex = grid_exponent(nmn.x, nmx.x), ey = grid_exponent(nmn.y, nmx.y),
                       ez = grid_exponent(nmn.z, nmx.z);
        const float isx = inv_grid(ex), isy = inv_grid(ey), isz = inv_grid(ez);
        uint32_t q[6][2];
#pragma unroll
        for (int a = 0; a < 6; ++a) q[a][0] = q[a][1] = 0;
        int at_slot[8];
#pragma unroll
        for (int s2 = 0; s2 < 8; ++s2) at_slot[s2] = CPT_WIDE_EMPTY;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k >= nr) break;
            const int s = slot_of[k];
            int ref = refs[k];
            if (ref >= 0) {
                const int num = first_child + __popc(imask & ((1u << s) - 1u));
                ref = base + n + num;   // the child's wide node number
                tasks[ref] = refs[k];
            }
#pragma unroll
            for (int s2 = 0; s2 < 8; ++s2)
                if (s2 == s) at_slot[s2] = ref;
            const uint32_t sh = (uint32_t)(s & 3) * 8u;
            const uint32_t v[6] = {q_lo(cmn[k].x, nmn.x, isx) << sh, q_hi(cmx[k].x, nmn.x, isx) << sh,
                                   q_lo(cmn[k].y, nmn.y, isy) << sh, q_hi(cmx[k].y, nmn.y, isy) << sh,
                                   q_lo(cmn[k].z, nmn.z, isz) << sh, q_hi(cmx[k].z, nmn.z, isz) << sh};
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                if (s < 4)
                    q[a][0] |= v[a];
                else
                    q[a][1] |= v[a];
            }
        }
        float4* dst = wide + CPT_WIDE_F4 * (size_t)(base + t);
        dst[0] = make_float4(nmn.x, nmn.y, nmn.z, __int_as_float((int)(ex | (ey << 8) | (ez << 16) | (imask << 24))));
        dst[1] = make_float4(__int_as_float(at_slot[0]), __int_as_float(at_slot[1]), __int_as_float(at_slot[2]),
                             __int_as_float(at_slot[3]));
        dst[2] = make_float4(__int_as_float(at_slot[4]), __int_as_float(at_slot[5]), __int_as_float(at_slot[6]),
                             __int_as_float(at_slot[7]));
#pragma unroll
        for (int a = 0; a < 3; ++a)
            dst[3 + a] = make_float4(__int_as_float((int)q[2 * a][0]), __int_as_float((int)q[2 * a][1]),
                                     __int_as_float((int)q[2 * a + 1][0]), __int_as_float((int)q[2 * a + 1][1]));
    }
}

__global__ void k_collapse_init(int* tasks, int* level_count, int* level_base)
{
    for (int i = threadIdx.x; i < MAX_WIDE_LEVELS; i += blockDim.x) {
        level_count[i] = i == 0 ? 1 : 0;   // level 0: the root
        level_base[i] = 0;
    }
    if (threadIdx.x == 0) tasks[0] = 0;   // wide node 0 stands for the binary root
}

}  // namespace

size_t wide_scratch_bytes(uint32_t n)
{
    // the binary node of every wide node (at most n - 1 of them), and the level counts and bases
    return align_up((size_t)n * 4, 256) + align_up(2 * MAX_WIDE_LEVELS * 4, 256);
}

cpt_status build_wide(uint32_t n, const int2* child, const float4* node_box, const float4* leaf_box, float4* wide,
                      void* scratch, size_t scratch_bytes, cudaStream_t stream, uint32_t* num_wide)
{
    if (n < 2) {
        if (num_wide) *num_wide = 0;
        return CPT_OK;
    }
    if (scratch_bytes < wide_scratch_bytes(n)) return fail(CPT_ERR_INVALID_ARGUMENT, "build_wide: scratch too small");
    char* p = (char*)scratch;
    int* tasks = (int*)p;
    p += align_up((size_t)n * 4, 256);
    int* level_count = (int*)p;
    int* level_base = level_count + MAX_WIDE_LEVELS;
    k_collapse_init<<<1, 128, 0, stream>>>(tasks, level_count, level_base);
    add_launches(1);
    // A grid that is resident at once; each thread takes nodes of its level in turn.  The host
    // looks at the level counts once every 16 levels (the wide tree of a few million primitives
    // has about a dozen; a level whose count is zero returns at once).
    // per device (the first 64 ordinals; others are queried on every call)
    static int resident_of[64] = {};
    int dev = 0;
    CPT_CUDA(cudaGetDevice(&dev));
    int resident = (dev >= 0 && dev < 64) ? resident_of[dev] : 0;
    if (resident == 0) {
        int sms = 0, per_sm = 0;
        CPT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_collapse_level, COLLAPSE_THREADS, 0));
        resident = std::max(1, sms * std::max(1, per_sm));
        if (dev >= 0 && dev < 64) resident_of[dev] = resident;
    }
    const unsigned grid = std::max(1u, std::min((n + COLLAPSE_THREADS - 1) / COLLAPSE_THREADS, (unsigned)resident));
    int l = 0;
    int hc[2] = {0, 0};
    for (;;) {
        const int first = l, stop = std::min(l + 16, MAX_WIDE_LEVELS - 1);
        for (; l < stop; ++l)
            k_collapse_level<<<grid, COLLAPSE_THREADS, 0, stream>>>(child, node_box, leaf_box, tasks, level_count,
                                                                    level_base, l, wide);
        add_launches(stop - first);
        CPT_CUDA(cudaGetLastError());
        // level l: its count (wide nodes still to collapse) and base (= wide nodes written)
        CPT_CUDA(cudaMemcpyAsync(&hc[0], level_count + l, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CPT_CUDA(cudaMemcpyAsync(&hc[1], level_base + l, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CPT_CUDA(cudaStreamSynchronize(stream));
        if (hc[0] == 0 || l >= MAX_WIDE_LEVELS - 1) break;
    }
    if (hc[0] != 0) return fail(CPT_ERR_STACK_OVERFLOW, "build_wide: collapse did not finish");
    if (num_wide) *num_wide = (uint32_t)hc[1];
    return CPT_OK;
}

}  // namespace cpt

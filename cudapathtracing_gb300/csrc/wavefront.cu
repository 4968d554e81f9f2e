// wavefront.cu — the wavefront integrator (config estimator).
//
// Paths live in M slots (structure of arrays).  Work items are (pixel, sample group) pairs, group
// major: each slot takes an item, runs that group's samples in sequence with the samples' own
// PCG32 sub-streams (Pcg32::init_sample), drawing the same numbers in the same order as the
// megakernel (render.cu, pixel_config), and stores the group sum; k_wf_finish adds a pixel's group
// sums in group order.  Both integrators therefore compute the same estimator, and a pixel's groups
// run in parallel, so the last iterations are not left to the slowest pixels' full sample counts.
// One iteration is four persistent kernels over compacted queues:
//
//   k_wf_trace    closest hit of every queued extension ray            (queue Q_i)
//   k_wf_shadow   occlusion query of every queued next-event shadow ray (queue S_i)
//   k_wf_resolve  slots whose last sample ended with shadow rays in flight: add the visible
//                 light contributions, store the group sum, take the next item  (queue R_i)
//   k_wf_shade    one path vertex per slot: add last iteration's visible light contributions,
//                 then medium / miss / emission / NEE (appends to S_{i+1}) / Russian roulette /
//                 BSDF sampling (appends to Q_{i+1}); a finished sample starts the next one
//
// Queues are appended with warp-aggregated atomics; counters for iteration i+1 are cleared by
// k_wf_trace of iteration i.
//
// Batches (cpt_render_batch): one wavefront renders several jobs — different scenes, image sizes,
// sample counts and depth settings.  Items are numbered job after job; each slot records the job
// of its item (Wf::job) and every kernel reads that job's scene view and parameters (WfJob) in
// place of its own.  A job's pixels draw the same streams as in a render of its own, so its image
// is the one cpt_render gives.  Kernels are instantiated with MULTI = false for single renders,
// which keep the scene and parameters in kernel arguments.
//
// Material sort (optional, Wf::bins): k_wf_trace files every traced slot into one of NBIN bins by
// the material its ray hit (miss / light / medium boundary, diffuse-like surfaces with next-event
// estimation, specular dielectrics, rough dielectrics) and k_wf_shade walks the bins in order, so
// the lanes of a warp run the same BSDF code.  A slot's result does not depend on the order in which
// slots are shaded (its random numbers come from its own sample stream), so the image is the same.  The host replays a CUDA graph of CHUNK iterations and reads
// the queue sizes after each replay to stop.
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cpt_internal.h"
#include "cpt_shade.cuh"

namespace cg = cooperative_groups;

namespace cpt {

namespace {

constexpr int CHUNK = 8;              // iterations per graph replay (even: parities repeat)
constexpr int NBIN = 4;               // shade-queue bins of the material sort
constexpr int CNT_BIN = 16;           // cnt[CNT_BIN + parity * NBIN + bin]: bin sizes
constexpr int CNT_WORDS = CNT_BIN + 2 * NBIN;

enum : uint32_t {
    F_CE = 1u << 0,        // count emission at the next surface
    F_INM = 1u << 1,       // inside a medium
    F_NEE_PREV = 1u << 2,  // pending shadow results belong to the finished sample (radp)
    F_GBUF = 1u << 3,      // G-buffer written for this pixel
};

struct WfJob;

struct Wf {
    int M, L, first_pix, npix, S, n_items;
    int* pixel;
    int* sample;            // index of the sample in flight (within the pixel)
    uint32_t* flags;
    int* depth;
    int* guard;
    int* nee;               // bit k: a shadow ray towards light k is in flight
    uint64_t* rng;
    float4* o;
    float4* d;
    float4* thr;
    float4* rad;
    float4* radp;
    float4* pix;            // sum of the item's finished samples
    float4* part;           // group sums, [group][pixel - first_pix]
    float2* med;
    float4* hit;
    int* q;                 // 2 * M
    int* rq;                // 2 * M
    int* sq;                // 2 * M * L
    float4* so;             // M * L
    float4* sd;
    float4* sc;
    int* svis;
    int* cnt;               // [0,1] Q sizes, [2,3] R sizes, [4,5] S sizes, [6] next item, [8..11] fetch
                            // counters, [CNT_BIN..] bin sizes
    int* bins;              // material sort: 2 * NBIN * M slots ([parity][bin][M]), NULL when off
    unsigned long long* rays;
    int* err;
    // batches
    const WfJob* jobs;      // device array of n_jobs, NULL for a single render
    int n_jobs;
    int* job;               // job of the slot's item
    int all_bvh2;           // every job's scene has internal nodes (dynamic fetching)
};

// One render of a batch: its scene and parameters, and its share of the items and group sums.
struct WfJob {
    SceneView view;
    RenderArgs args;
    int first_pix, npix, S;
    int item_base;          // global number of the job's first item
    long long part_base;    // offset of its group sums in Wf::part (groups x npix)
};

// Pixel range, sample group size and group-sum array of the render a slot belongs to.
struct JobGeo {
    int first_pix, npix, S;
    float4* part;
};

__device__ __forceinline__ JobGeo geo_of(const Wf& w) { return JobGeo{w.first_pix, w.npix, w.S, w.part}; }
__device__ __forceinline__ JobGeo geo_of(const Wf& w, const WfJob& J)
{
    return JobGeo{J.first_pix, J.npix, J.S, w.part + J.part_base};
}

// Job of global item `item` (jobs are in item order).
__device__ __forceinline__ int job_of_item(const Wf& w, int item)
{
    int lo = 0, hi = w.n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (w.jobs[mid].item_base <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void append(int* base, int* counter, int v)
{
    cg::coalesced_group g = cg::coalesced_threads();
    int b = 0;
    if (g.thread_rank() == 0) b = atomicAdd(counter, (int)g.size());
    b = g.shfl(b, 0);
    base[b + g.thread_rank()] = v;
}

// Appends v to bin `bin` of a binned queue (bins of M entries, sizes in counters[bin]); the lanes
// of the calling warp that pick the same bin share one atomic.
__device__ __forceinline__ void append_binned(int* bins, int* counters, int M, int bin, int v)
{
    cg::coalesced_group g = cg::coalesced_threads();
    cg::coalesced_group p = cg::labeled_partition(g, bin);
    int b = 0;
    if (p.thread_rank() == 0) b = atomicAdd(&counters[bin], (int)p.size());
    b = p.shfl(b, 0);
    bins[(size_t)bin * M + b + p.thread_rank()] = v;
}

// Shade bin of a traced ray: 0 miss, light, medium boundary (or any other cheap vertex); 1 Opaque
// or Lambertian (next-event estimation, GGX / cosine sampling); 2 specular dielectric; 3 rough
// dielectric.
__device__ __forceinline__ int shade_bin(const SceneView& s, int leaf)
{
    if (leaf < 0) return 0;
    const float4* r = s.leaf_rec + 3 * (size_t)leaf;
    const int prim = __float_as_int(__ldg(&r[0].w));
    const int kind = __float_as_int(__ldg(&r[1].w));
    if (kind == CPT_KIND_LIGHT) return 0;
    const uint32_t mi = kind == CPT_KIND_SPHERE ? __ldg(s.sphere_mat + (prim - s.n_lights))
                                                : __ldg(s.tri_mat + (prim - s.n_lights - s.n_spheres));
    switch (s.mats[mi].type) {
    case M_OPAQUE:
    case M_LAMBERT: return 1;
    case M_SPEC: return 2;
    case M_ROUGH: return 3;
    default: return 0;
    }
}

__device__ __forceinline__ void count_rays(unsigned long long* counter, uint32_t n)
{
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t tot = cg::reduce(g, n, cg::plus<uint32_t>());
    if (g.thread_rank() == 0 && tot) atomicAdd(counter, (unsigned long long)tot);
}

__device__ __forceinline__ float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 w0(float3 v) { return make_float4(v.x, v.y, v.z, 0.f); }

// A finished sample's radiance added to its item's sum: radiance in xyz, squared luminance in w
// (G-buffer channel 7, mean_variance).
__device__ __forceinline__ float4 add_sample(float4 sum, float3 r)
{
    const float y = luminance(r);
    return make_float4(sum.x + r.x, sum.y + r.y, sum.z + r.z, sum.w + y * y);
}

__device__ __forceinline__ float3 camera_dir(const DevCamera& c, int i, int j, float rx, float ry)   // Camera.cuh:37-43
{
    float3 p = c.pixel_center + (rx - 0.5f + (float)i) * c.delta_h + (ry - 0.5f + (float)j) * c.delta_v;
    return p - c.look_from;
}

__device__ __forceinline__ uint8_t to_u8(float x)
{
    float c = sqrtf(x);
    c = c > 1.0f ? 1.0f : (c < 0.0f ? 0.0f : c);
    return (uint8_t)(254.99f * c);
}

// Sample k of pixel `pixel` in slot `slot`: its generator, camera ray (two draws), fresh path state.
__device__ __forceinline__ void start_sample(const SceneView& s, const Wf& w, uint64_t seed, int slot, int pixel,
                                             int k, Pcg32& rng, uint32_t& fl)
{
    int W = s.cam.width;
    int i = pixel % W, j = pixel / W;
    rng.init_sample(seed, (uint64_t)pixel, (uint32_t)k);
    w.sample[slot] = k;
    float rx = rng.uniform();
    float ry = rng.uniform();
    w.o[slot] = w0(s.cam.look_from);
    w.d[slot] = w0(camera_dir(s.cam, i, j, rx, ry));
    w.thr[slot] = make_float4(1.f, 1.f, 1.f, 0.f);
    w.rad[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    w.depth[slot] = 0;
    w.guard[slot] = 0;
    fl = (fl & ~F_INM) | F_CE;
}

// The item in the slot is done: store its group sum (and a miss G-buffer entry when no sample of
// group 0 found a surface).
__device__ __forceinline__ void finish_item(const Wf& w, const RenderArgs& a, const JobGeo& jg, int slot, int pixel,
                                            uint32_t fl)
{
    const int g = (w.sample[slot] - 1) / jg.S;
    const size_t off = (size_t)(pixel - jg.first_pix);
    jg.part[(size_t)g * jg.npix + off] = w.pix[slot];
    if (g == 0 && a.gbuf && !(fl & F_GBUF)) {
        float4* gb = reinterpret_cast<float4*>(a.gbuf) + 2 * (size_t)pixel;
        gb[0] = make_float4(0.f, 0.f, 0.f, CPT_INF_F);
        gb[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Starts item `item` (group major within its render) in the slot with its first sample.  For a
// batch, item is global and the slot takes the item's job.
template <bool MULTI>
__device__ __forceinline__ void start_item(const SceneView& s0, const Wf& w, const RenderArgs& a0, int slot, int item)
{
    const int j = MULTI ? job_of_item(w, item) : 0;
    const SceneView& s = MULTI ? w.jobs[j].view : s0;
    const RenderArgs& a = MULTI ? w.jobs[j].args : a0;
    const JobGeo jg = MULTI ? geo_of(w, w.jobs[j]) : geo_of(w);
    if (MULTI) {
        item -= w.jobs[j].item_base;
        w.job[slot] = j;
    }
    const int g = item / jg.npix;
    const int p = jg.first_pix + (item - g * jg.npix);
    uint32_t fl = g == 0 ? 0u : F_GBUF;   // only group 0 writes the G-buffer
    Pcg32 rng;
    w.pixel[slot] = p;
    w.pix[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    w.nee[slot] = 0;
    start_sample(s, w, a.seed, slot, p, g * jg.S, rng, fl);
    w.flags[slot] = fl;
    w.rng[slot] = rng.state;
}

// Takes the next item for the slot (or leaves it idle) and queues its first ray.
template <bool MULTI>
__device__ __forceinline__ void next_item(const SceneView& s0, const Wf& w, const RenderArgs& a0, int slot, int nq)
{
    // the lanes of the warp that take an item now share one atomic on the item counter
    cg::coalesced_group g = cg::coalesced_threads();
    int first = 0;
    if (g.thread_rank() == 0) first = atomicAdd(&w.cnt[6], (int)g.size());
    const int item = g.shfl(first, 0) + (int)g.thread_rank();
    if (item >= w.n_items) {
        w.pixel[slot] = -1;
        return;
    }
    start_item<MULTI>(s0, w, a0, slot, item);
    append(w.q + (size_t)nq * w.M, &w.cnt[nq], slot);
}

template <bool MULTI>
__global__ void k_wf_init(const __grid_constant__ SceneView s, Wf w, const __grid_constant__ RenderArgs a)
{
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= w.M) return;
    if (slot == 0) {
        w.cnt[0] = w.M;
        w.cnt[1] = w.cnt[2] = w.cnt[3] = w.cnt[4] = w.cnt[5] = 0;
        w.cnt[6] = w.M;
        w.cnt[8] = w.cnt[9] = w.cnt[10] = w.cnt[11] = 0;
        for (int k = CNT_BIN; k < CNT_WORDS; ++k) w.cnt[k] = 0;
    }
    start_item<MULTI>(s, w, a, slot, slot);
    w.q[slot] = slot;   // Q_0 holds every slot in order
}

// Pixel = (sum of its group sums in group order) / spp, as the megakernel adds them (one render,
// or one job of a batch).
__global__ void k_wf_finish(JobGeo jg, RenderArgs a, int groups)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= jg.npix) return;
    float3 sum = f3(0.f, 0.f, 0.f);
    float sum_y2 = 0.f;
    for (int g = 0; g < groups; ++g) {
        const float4 part = jg.part[(size_t)g * jg.npix + p];
        sum = sum + xyz(part);
        sum_y2 += part.w;
    }
    float3 v = sum / (float)a.spp;
    size_t off = (size_t)(jg.first_pix + p);
    if (a.gbuf) a.gbuf[8 * off + 7] = mean_variance(sum, sum_y2, a.spp);
    if (a.flags & CPT_RENDER_ACCUMULATE) {
        a.rgb[3 * off] += v.x;
        a.rgb[3 * off + 1] += v.y;
        a.rgb[3 * off + 2] += v.z;
    } else {
        a.rgb[3 * off] = v.x;
        a.rgb[3 * off + 1] = v.y;
        a.rgb[3 * off + 2] = v.z;
    }
    if (a.rgba8) reinterpret_cast<uchar4*>(a.rgba8)[off] = make_uchar4(to_u8(v.x), to_u8(v.y), to_u8(v.z), 255);
}

// BVH2: at most 48 registers (5 blocks of 256 per SM): 62 % occupancy instead of 50 % for a few
// spilled values, +5.7 % on the 1080p spheres render (the shadow kernel is faster uncapped).
// 8-wide: at most 64 registers (4 blocks of 256): +4.7 % against 72; 51 registers spill (-9 %).
template <bool WIDE, int SHORT, bool SORT, bool MULTI>
__global__ void __launch_bounds__(256, WIDE ? 4 : 5) k_wf_trace(const __grid_constant__ SceneView s, Wf w, int par)
{
    const int n = w.cnt[par];
    const int nq = par ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.cnt[nq] = 0;
        w.cnt[2 + nq] = 0;
        w.cnt[4 + nq] = 0;
        w.cnt[8 + 2 * nq] = 0;   // fetch counters of the next iteration's trace and shadow kernels
        w.cnt[9 + 2 * nq] = 0;
        for (int b = 0; b < NBIN; ++b) w.cnt[CNT_BIN + nq * NBIN + b] = 0;   // its shade bins
    }
    const int* q = w.q + (size_t)par * w.M;
    int* const bins = SORT ? w.bins + (size_t)par * NBIN * w.M : nullptr;
    int* const bin_cnt = w.cnt + CNT_BIN + par * NBIN;
    const auto views = [&](int j) -> const SceneView& { return MULTI ? w.jobs[j].view : s; };
    uint32_t rays = 0;
    const auto load = [&](int i, float3& o, float3& d, float& tmn, float& tmx, int&, int& j) {
        int slot = q[i];
        o = xyz(w.o[slot]);
        d = xyz(w.d[slot]);
        tmn = 0.001f;
        tmx = CPT_INF_F;
        j = MULTI ? w.job[slot] : 0;
    };
    const auto store = [&](int i, const Hit& h, int j) {
        const int slot = q[i];
        w.hit[slot] = make_float4(h.t, __int_as_float(h.leaf), h.u, h.v);
        if (SORT) append_binned(bins, bin_cnt, w.M, shade_bin(views(j), h.leaf), slot);
    };
    if (MULTI ? w.all_bvh2 != 0 : s.n_internal > 0) {
        if (WIDE)
            rays = trace_items_wide_views<false, ShortStack64<CPT_WIDE_SHORT_STACK>>(views, n, &w.cnt[8 + 2 * par],
                                                                                     w.err, load, store);
        else
            rays = trace_items_bvh2_views<false, ShortStackN<SHORT>>(views, n, &w.cnt[8 + 2 * par], w.err, load,
                                                                    store);
    } else {
        for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
            int slot = q[idx];
            const SceneView& sv = views(MULTI ? w.job[slot] : 0);
            float4 o = w.o[slot], d = w.d[slot];
            Hit h;
            bool hit = trace_closest<WIDE>(sv, xyz(o), xyz(d), 0.001f, CPT_INF_F, h, w.err);
            w.hit[slot] = make_float4(h.t, __int_as_float(hit ? h.leaf : -1), h.u, h.v);
            if (SORT) append_binned(bins, bin_cnt, w.M, shade_bin(sv, hit ? h.leaf : -1), slot);
            rays++;
        }
    }
    count_rays(w.rays, rays);
}

template <bool WIDE, int SHORT, bool MULTI>
__global__ void __launch_bounds__(256) k_wf_shadow(const __grid_constant__ SceneView s, Wf w, int par)
{
    const int n = w.cnt[4 + par];
    const int* sq = w.sq + (size_t)par * w.M * w.L;
    const auto views = [&](int j) -> const SceneView& { return MULTI ? w.jobs[j].view : s; };
    uint32_t rays = 0;
    const auto load = [&](int i, float3& o, float3& d, float& tmn, float& tmx, int& skip, int& j) {
        int e = sq[i];
        float4 dd = w.sd[e];
        o = xyz(w.so[e]);
        d = xyz(dd);
        tmn = 0.001f;
        tmx = dd.w;
        skip = e % w.L;
        j = MULTI ? w.job[e / w.L] : 0;
    };
    const auto store = [&](int i, const Hit& h, int) { w.svis[sq[i]] = h.leaf < 0 ? 1 : 0; };
    if (MULTI ? w.all_bvh2 != 0 : s.n_internal > 0) {
        if (WIDE)
            rays = trace_items_wide_views<true, ShortStack64<CPT_WIDE_SHORT_STACK>>(views, n, &w.cnt[9 + 2 * par],
                                                                                    w.err, load, store);
        else
            rays = trace_items_bvh2_views<true, ShortStackN<SHORT>>(views, n, &w.cnt[9 + 2 * par], w.err, load,
                                                                   store);
    } else {
        for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
            int e = sq[idx];
            const SceneView& sv = views(MULTI ? w.job[e / w.L] : 0);
            float4 dd = w.sd[e];
            w.svis[e] = occluded<WIDE>(sv, xyz(w.so[e]), xyz(dd), dd.w, e % w.L, w.err) ? 0 : 1;
            rays++;
        }
    }
    count_rays(w.rays, rays);
}

// Adds the visible contributions of the shadow rays in flight, in light order.
__device__ __forceinline__ float3 add_visible(const Wf& w, int slot, int mask, float3 acc)
{
    for (int k = 0; k < w.L; ++k) {
        if (!((mask >> k) & 1)) continue;
        int e = slot * w.L + k;
        if (w.svis[e]) acc = acc + xyz(w.sc[e]);
    }
    return acc;
}

template <bool MULTI>
__global__ void __launch_bounds__(256) k_wf_resolve(const __grid_constant__ SceneView s, Wf w,
                                                    const __grid_constant__ RenderArgs a, int par)
{
    const int n = w.cnt[2 + par];
    const int nq = par ^ 1;
    const int* rq = w.rq + (size_t)par * w.M;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        int slot = rq[idx];
        float3 acc = add_visible(w, slot, w.nee[slot], xyz(w.radp[slot]));
        w.pix[slot] = add_sample(w.pix[slot], acc);
        w.nee[slot] = 0;
        if (MULTI) {
            const WfJob& J = w.jobs[w.job[slot]];
            finish_item(w, J.args, geo_of(w, J), slot, w.pixel[slot], w.flags[slot]);
        } else {
            finish_item(w, a, geo_of(w), slot, w.pixel[slot], w.flags[slot]);
        }
        next_item<MULTI>(s, w, a, slot, nq);
    }
}

// At most 64 registers (4 blocks of 256 per SM, 50 % occupancy instead of 37 % at 79 registers):
// +4.4 % on the 1080p spheres render; 48 registers: +3.7 %.
template <bool MULTI>
__global__ void __launch_bounds__(256, 4) k_wf_shade(const __grid_constant__ SceneView s0, Wf w,
                                                     const __grid_constant__ RenderArgs a0, int par)
{
    const int nq = par ^ 1;
    // the traced slots: the bins in order (material sort), else the trace queue
    const int* q = w.bins ? w.bins + (size_t)par * NBIN * w.M : w.q + (size_t)par * w.M;
    int bin_end[NBIN];
    int n = w.cnt[par];
    if (w.bins) {
        int acc = 0;
        for (int b = 0; b < NBIN; ++b) bin_end[b] = acc += w.cnt[CNT_BIN + par * NBIN + b];
        n = acc;
    }
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        int pos = idx;
        if (w.bins) {
            int b = 0;
            while (b < NBIN - 1 && idx >= bin_end[b]) ++b;
            pos = b * w.M + idx - (b ? bin_end[b - 1] : 0);
        }
        const int slot = q[pos];
        const int pixel = w.pixel[slot];
        const int job = MULTI ? w.job[slot] : 0;
        const SceneView& s = MULTI ? w.jobs[job].view : s0;
        const RenderArgs& a = MULTI ? w.jobs[job].args : a0;
        uint32_t fl = w.flags[slot];
        Pcg32 rng;
        rng.state = w.rng[slot];
        rng.inc = ((uint64_t)pixel << 1u) | 1u;
        float3 rad = xyz(w.rad[slot]);
        // 1. shadow rays from the previous vertex
        int pend = w.nee[slot];
        if (pend) {
            if (fl & F_NEE_PREV) {
                float3 accp = add_visible(w, slot, pend, xyz(w.radp[slot]));
                w.pix[slot] = add_sample(w.pix[slot], accp);
            } else {
                rad = add_visible(w, slot, pend, rad);
            }
            fl &= ~F_NEE_PREV;
        }
        // 2. the vertex (pixel_config's loop body)
        float3 o = xyz(w.o[slot]), d = xyz(w.d[slot]);
        float3 thr = xyz(w.thr[slot]);
        int depth = w.depth[slot];
        int guard = w.guard[slot] + 1;
        float4 hv = w.hit[slot];
        Hit h;
        h.t = hv.x;
        h.leaf = __float_as_int(hv.y);
        h.u = hv.z;
        h.v = hv.w;
        const bool hit = h.leaf >= 0;
        int nee = 0;
        bool cont = false;   // path continues with (o, d)
        if (guard >= a.iter_limit) {
            atomicOr(w.err, CPT_DEVERR_ITER);
        } else {
            bool done_vertex = false;
            if (fl & F_INM) {
                float2 m = w.med[slot];
                float t_hit = hit ? h.t : CPT_INF_F;
                float t = -logf(rng.uniform()) / m.x;
                if (t < t_hit) {
                    float3 pos = o + t * d;
                    thr = thr * m.y;
                    depth++;
                    done_vertex = true;
                    bool alive = !(a.max_depth > 0 && depth >= a.max_depth);
                    float P = 1.0f;
                    if (alive && depth >= a.rr_depth) {
                        P = a.rr_prob;
                        if (rng.uniform() > P) alive = false;
                    }
                    if (alive) {
                        thr = thr * (1.0f / P);
                        float z = 1.0f - 2.0f * rng.uniform();
                        float r = sqrtf(fmaxf(0.f, 1.0f - z * z));
                        float phi = 2.0f * CPT_PI_F * rng.uniform();
                        float sn, cs;
                        sincosf(phi, &sn, &cs);
                        o = pos;
                        d = f3(r * cs, r * sn, z);
                        fl |= F_CE;
                        cont = true;
                    }
                }
            }
            if (!done_vertex) {
                if (!hit) {
                    rad = rad + thr * sky_radiance(s, d);
                } else {
                    Surf sf;
                    make_surface(s, o, d, h, false, sf);
                    if (sf.type == M_VOLUME) {
                        fl = sf.front ? (fl | F_INM) : (fl & ~F_INM);
                        w.med[slot] = make_float2(sf.sigma_t, sf.albedo);
                        o = sf.pos;
                        cont = true;
                    } else if (sf.type == M_LIGHT) {
                        if (fl & F_CE) rad = rad + thr * sf.color;
                    } else {
                        if (depth == 0 && !(fl & F_GBUF)) {
                            fl |= F_GBUF;
                            if (a.gbuf) {
                                float4* g = reinterpret_cast<float4*>(a.gbuf) + 2 * (size_t)pixel;
                                g[0] = make_float4(sf.normal.x, sf.normal.y, sf.normal.z,
                                                   sqrtf(len2(s.cam.look_from - sf.pos)));
                                g[1] = make_float4(sf.color.x, sf.color.y, sf.color.z, 0.f);
                            }
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
                                if (!(cs_ > 0.f && cl_ > 0.f)) continue;
                                float tl;
                                if (!hit_light(L, sf.pos, dir, 0.001f, CPT_INF_F, tl)) continue;
                                float3 fr = bsdf_eval(sf, d, dir);
                                float g = cs_ * cl_ / len2(lp - sf.pos) * area;
                                int e = slot * w.L + k;
                                w.so[e] = w0(sf.pos);
                                w.sd[e] = make_float4(dir.x, dir.y, dir.z, tl);   // occlusion query up to the light
                                w.sc[e] = w0(thr * (L.color * fr * g));
                                nee |= 1 << k;
                            }
                        }
                        if (diffuse_like && s.n_lights > 0) fl &= ~F_CE;
                        else fl |= F_CE;
                        depth++;
                        bool alive = !(a.max_depth > 0 && depth >= a.max_depth);
                        float P = 1.0f;
                        if (alive && depth >= a.rr_depth) {
                            P = a.rr_prob;
                            if (rng.uniform() > P) alive = false;
                        }
                        if (alive) {
                            float r1 = rng.uniform(), r2 = rng.uniform(), r3 = rng.uniform();
                            float3 dir;
                            float pdf;
                            bsdf_sample(sf, d, dir, pdf, r1, r2, r3);
                            if (pdf > 0.f) {
                                float3 fr = bsdf_eval(sf, d, dir);
                                thr = thr * (fr * fabsf(dot3(dir, sf.normal)) / pdf / P);
                                o = sf.pos;
                                d = dir;
                                cont = true;
                            }
                        }
                    }
                }
            }
        }
        w.nee[slot] = nee;
        bool to_resolve = false, to_trace = false;
        if (cont) {
            w.o[slot] = w0(o);
            w.d[slot] = w0(d);
            w.thr[slot] = w0(thr);
            w.rad[slot] = w0(rad);
            w.depth[slot] = depth;
            w.guard[slot] = guard;
            to_trace = true;
        } else {
            // the sample ended
            const int k = w.sample[slot] + 1;   // next sample of the pixel
            if (nee) {
                w.radp[slot] = w0(rad);
                fl |= F_NEE_PREV;
            } else {
                w.pix[slot] = add_sample(w.pix[slot], rad);
            }
            const JobGeo jg = MULTI ? geo_of(w, w.jobs[job]) : geo_of(w);
            if (k % jg.S != 0 && k < a.spp) {   // the item's group has samples left
                start_sample(s, w, a.seed, slot, pixel, k, rng, fl);
                to_trace = true;
            } else {
                w.sample[slot] = k;
                if (nee) to_resolve = true;
                else finish_item(w, a, jg, slot, pixel, fl);
            }
        }
        w.flags[slot] = fl;
        w.rng[slot] = rng.state;
        if (nee)
            for (int k = 0; k < w.L; ++k)
                if ((nee >> k) & 1) append(w.sq + (size_t)nq * w.M * w.L, &w.cnt[4 + nq], slot * w.L + k);
        if (to_trace) append(w.q + (size_t)nq * w.M, &w.cnt[nq], slot);
        if (to_resolve) append(w.rq + (size_t)nq * w.M, &w.cnt[2 + nq], slot);
        if (!cont && !to_trace && !to_resolve) next_item<MULTI>(s0, w, a0, slot, nq);
    }
}

using WfKernel = void (*)(SceneView, Wf, int);
struct TracePair {
    WfKernel trace, shadow;
};

// The trace kernels for the scene's layout, the short-stack depth (binary layout only), the
// material sort (the binning is compiled only into the sorting variants, so that the default
// trace kernel keeps its registers) and batches.
template <bool SORT, bool MULTI>
TracePair trace_pair_of(bool wide, int short_entries)
{
    if (wide) return {k_wf_trace<true, CPT_SHORT_STACK, SORT, MULTI>, k_wf_shadow<true, CPT_SHORT_STACK, MULTI>};
    switch (short_entries) {
    case 8: return {k_wf_trace<false, 8, SORT, MULTI>, k_wf_shadow<false, 8, MULTI>};
    case 24: return {k_wf_trace<false, 24, SORT, MULTI>, k_wf_shadow<false, 24, MULTI>};
    case 32: return {k_wf_trace<false, 32, SORT, MULTI>, k_wf_shadow<false, 32, MULTI>};
    default: return {k_wf_trace<false, 16, SORT, MULTI>, k_wf_shadow<false, 16, MULTI>};
    }
}

TracePair trace_pair(bool wide, int short_entries, bool sort = false, bool multi = false)
{
    if (multi) return sort ? trace_pair_of<true, true>(wide, short_entries) : trace_pair_of<false, true>(wide, short_entries);
    return sort ? trace_pair_of<true, false>(wide, short_entries) : trace_pair_of<false, false>(wide, short_entries);
}

// CHUNK iterations: trace, shadow, resolve, shade, with the traversal of the scene's layout.
// When capturing with a side stream, the shadow kernel is forked onto it so that the two
// traversal kernels of an iteration overlap (each one's tail fills with the other's warps).
template <bool MULTI>
void enqueue_chunk(const SceneView& view, const Wf& w, const RenderArgs& args, int gt, int bt, int gs, int bs,
                   int short_entries, cudaStream_t st, const WavefrontTuning* fork)
{
    const TracePair kp = trace_pair(view.wide != nullptr, short_entries, w.bins != nullptr, MULTI);
    const size_t smem = view.wide ? wide_short_stack_bytes(bt) : short_stack_bytes(bt, short_entries);
    for (int it = 0; it < CHUNK; ++it) {
        int par = it & 1;
        cudaStream_t ss = st;
        if (fork) {
            cudaEventRecord(fork->fork, st);
            cudaStreamWaitEvent(fork->side_stream, fork->fork, 0);
            ss = fork->side_stream;
        }
        kp.trace<<<gt, bt, smem, st>>>(view, w, par);
        kp.shadow<<<gt, bt, smem, ss>>>(view, w, par);
        if (fork) {
            cudaEventRecord(fork->join, ss);
            cudaStreamWaitEvent(st, fork->join, 0);
        }
        k_wf_resolve<MULTI><<<gs, bs, 0, st>>>(view, w, args, par);
        k_wf_shade<MULTI><<<gs, bs, 0, st>>>(view, w, args, par);
    }
}

template <typename T>
cpt_status carve(char*& p, size_t& left, T** out, size_t count)
{
    size_t bytes = align_up(count * sizeof(T), 256);
    if (bytes > left) return fail(CPT_ERR_INVALID_ARGUMENT, "wavefront buffer too small");
    *out = (T*)p;
    p += bytes;
    left -= bytes;
    return CPT_OK;
}

size_t wf_bytes(int M, int L, size_t n_parts, bool sort, int n_jobs)
{
    size_t m = (size_t)M, ml = (size_t)M * std::max(L, 1);
    auto a = [](size_t b) { return align_up(b, 256); };
    return a(m * 4) * 6 + a(m * 8) + a(m * 16) * 8 + a(n_parts * 16) + a(m * 8) + a(2 * m * 4) * 2 +
           a(2 * ml * 4) + a(ml * 16) * 3 + a(ml * 4) + a(CNT_WORDS * 4) + (sort ? a(2 * NBIN * m * 4) : 0) +
           (n_jobs > 0 ? a(m * 4) + a((size_t)n_jobs * sizeof(WfJob)) : 0);
}

}  // namespace

namespace {

// A single render (jobs empty: scene and parameters in kernel arguments) or a batch (MULTI).
template <bool MULTI>
cpt_status run_wavefront(const SceneView& view, const RenderArgs& args, const std::vector<WfJob>& jobs,
                         cudaStream_t stream, const WavefrontTuning& tune)
{
    Wf w;
    std::memset(&w, 0, sizeof w);
    size_t n_items = 0, n_parts = 0;
    int L = 1;
    std::vector<WfJob> J = jobs;
    if (!MULTI) {
        const int W = view.cam.width;
        const int first = args.row_begin * W, end = args.row_end * W;
        w.first_pix = first;
        w.npix = end - first;
        if (w.npix <= 0) return CPT_OK;
        if (view.n_lights > 30) return fail(CPT_ERR_UNSUPPORTED, "wavefront integrator: at most 30 lights");
        if (args.spp <= 0) return fail(CPT_ERR_INVALID_ARGUMENT, "spp must be positive");
        w.S = sample_group(args.spp);
        n_items = n_parts = (size_t)((args.spp + w.S - 1) / w.S) * (size_t)w.npix;
        L = std::max(view.n_lights, 1);
    } else {
        for (WfJob& j : J) {
            if (j.view.n_lights > 30) return fail(CPT_ERR_UNSUPPORTED, "wavefront integrator: at most 30 lights");
            if (j.args.spp <= 0) return fail(CPT_ERR_INVALID_ARGUMENT, "spp must be positive");
            const int W = j.view.cam.width;
            j.first_pix = j.args.row_begin * W;
            j.npix = j.args.row_end * W - j.first_pix;
            j.S = sample_group(j.args.spp);
            j.item_base = (int)std::min(n_items, (size_t)INT32_MAX);
            j.part_base = (long long)n_parts;
            const size_t items = (size_t)((j.args.spp + j.S - 1) / j.S) * (size_t)std::max(j.npix, 0);
            n_items += items;
            n_parts += items;
            L = std::max(L, j.view.n_lights);
        }
        w.all_bvh2 = 1;   // every job has internal nodes (all share one layout): dynamic fetching
        for (const WfJob& j : J)
            if (j.view.n_internal <= 0) w.all_bvh2 = 0;
        if (n_items == 0) return CPT_OK;
    }
    if (n_items > (size_t)INT32_MAX / 2) return fail(CPT_ERR_UNSUPPORTED, "wavefront integrator: too many pixel groups");
    const int M = (int)std::min(n_items, (size_t)std::max(tune.slots, 1024));
    w.M = M;
    w.L = L;
    w.n_items = (int)n_items;
    w.rays = args.ray_counter;
    w.err = args.err;
    w.n_jobs = MULTI ? (int)J.size() : 0;
    size_t bytes = wf_bytes(M, L, n_parts, tune.material_sort, w.n_jobs);
    char* base = nullptr;
    CPT_CUDA(cudaMallocAsync((void**)&base, bytes, stream));
    char* p = base;
    size_t left = bytes;
    size_t ml = (size_t)M * L;
    cpt_status st = CPT_OK;
    WfJob* d_jobs = nullptr;
#define CARVE(f, n)                                   \
    if (st == CPT_OK) st = carve(p, left, &w.f, (n));
    CARVE(pixel, M) CARVE(sample, M) CARVE(flags, M) CARVE(depth, M) CARVE(guard, M) CARVE(nee, M)
    CARVE(rng, M) CARVE(o, M) CARVE(d, M) CARVE(thr, M) CARVE(rad, M) CARVE(radp, M) CARVE(pix, M) CARVE(hit, M)
    CARVE(part, n_parts)
    CARVE(so, ml) CARVE(med, M) CARVE(q, 2 * (size_t)M) CARVE(rq, 2 * (size_t)M) CARVE(sq, 2 * ml) CARVE(sd, ml)
    CARVE(sc, ml) CARVE(svis, ml) CARVE(cnt, CNT_WORDS)
    if (tune.material_sort) CARVE(bins, 2 * (size_t)NBIN * M)
    if (MULTI) CARVE(job, M)
#undef CARVE
    if (MULTI && st == CPT_OK) {
        st = carve(p, left, &d_jobs, J.size());
        if (st == CPT_OK) {
            cudaError_t e = cudaMemcpyAsync(d_jobs, J.data(), J.size() * sizeof(WfJob), cudaMemcpyHostToDevice, stream);
            if (e != cudaSuccess) st = cuda_fail(e, "batch job table");
        }
        w.jobs = d_jobs;
    }
    if (st != CPT_OK) {
        cudaFreeAsync(base, stream);
        return st;
    }
    // Q_0 = all M slots
    k_wf_init<MULTI><<<(M + 255) / 256, 256, 0, stream>>>(view, w, args);
    add_launches(1);
    const int gt = view.wide ? tune.grid_trace_wide : tune.grid_trace, gs = tune.grid_shade;
    const int bt = tune.block_trace, bs = tune.block_shade;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    bool use_graph = tune.use_graph;
    if (use_graph) {
        // Capture CHUNK iterations (4 launches each) once; replay until the queues drain.
        cudaStream_t cs = tune.capture_stream;
        CPT_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        enqueue_chunk<MULTI>(view, w, args, gt, bt, gs, bs, tune.short_stack, cs, tune.side_stream ? &tune : nullptr);
        cudaError_t ce = cudaStreamEndCapture(cs, &graph);
        if (ce != cudaSuccess) {
            cudaFreeAsync(base, stream);
            return cuda_fail(ce, "cudaStreamEndCapture");
        }
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) {
            cudaFreeAsync(base, stream);
            return cuda_fail(ce, "cudaGraphInstantiate");
        }
    }
    int host_cnt[6];
    const int max_chunks = tune.max_replays;
    bool drained = false;
    for (int chunk = 0; chunk < max_chunks; ++chunk) {
        if (use_graph) {
            CPT_CUDA(cudaGraphLaunch(exec, stream));
        } else {
            enqueue_chunk<MULTI>(view, w, args, gt, bt, gs, bs, tune.short_stack, stream, nullptr);
        }
        add_launches(4 * CHUNK);
        CPT_CUDA(cudaMemcpyAsync(host_cnt, w.cnt, sizeof host_cnt, cudaMemcpyDeviceToHost, stream));
        CPT_CUDA(cudaStreamSynchronize(stream));
        if (host_cnt[0] == 0 && host_cnt[2] == 0 && host_cnt[4] == 0) {
            drained = true;
            break;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (drained) {
        if (!MULTI) {
            const int groups = (args.spp + w.S - 1) / w.S;
            k_wf_finish<<<(w.npix + 255) / 256, 256, 0, stream>>>(JobGeo{w.first_pix, w.npix, w.S, w.part}, args,
                                                                  groups);
            add_launches(1);
        } else {
            for (const WfJob& j : J) {
                if (j.npix <= 0) continue;
                const int groups = (j.args.spp + j.S - 1) / j.S;
                k_wf_finish<<<(j.npix + 255) / 256, 256, 0, stream>>>(
                    JobGeo{j.first_pix, j.npix, j.S, w.part + j.part_base}, j.args, groups);
                add_launches(1);
            }
        }
    }
    cudaFreeAsync(base, stream);
    CPT_CUDA(cudaGetLastError());
    if (!drained) return fail(CPT_ERR_TIMEOUT, "wavefront integrator did not drain");
    return CPT_OK;
}

}  // namespace

cpt_status launch_render_wavefront(const SceneView& view, const RenderArgs& args, cudaStream_t stream,
                                   const WavefrontTuning& tune)
{
    return run_wavefront<false>(view, args, {}, stream, tune);
}

cpt_status launch_render_wavefront_batch(const SceneView* views, const RenderArgs* args, int n_jobs,
                                         cudaStream_t stream, const WavefrontTuning& tune)
{
    if (n_jobs <= 0) return CPT_OK;
    std::vector<WfJob> jobs(n_jobs);
    for (int i = 0; i < n_jobs; ++i) {
        std::memset(&jobs[i], 0, sizeof(WfJob));
        jobs[i].view = views[i];
        jobs[i].args = args[i];
    }
    return run_wavefront<true>(views[0], args[0], jobs, stream, tune);
}

}  // namespace cpt

namespace cpt {

// Persistent grid sizes: resident blocks per SM (occupancy) x SMs, for the given block sizes; the
// binary and the 8-wide trace kernels have their own register caps and shared stacks.
cpt_status wavefront_grids(int sm_count, int block_trace, int block_shade, int short_entries, int* grid_trace,
                           int* grid_trace_wide, int* grid_shade)
{
    int bw = 0, bb = 0, bs = 0;
    const TracePair wide = trace_pair(true, short_entries), bin = trace_pair(false, short_entries);
    cudaFuncAttributes fa[3];
    CPT_CUDA(cudaFuncGetAttributes(&fa[0], wide.trace));
    CPT_CUDA(cudaFuncGetAttributes(&fa[1], bin.trace));
    CPT_CUDA(cudaFuncGetAttributes(&fa[2], k_wf_shade<false>));
    if (block_trace > std::min(fa[0].maxThreadsPerBlock, fa[1].maxThreadsPerBlock) ||
        block_shade > fa[2].maxThreadsPerBlock)
        return fail(CPT_ERR_INVALID_ARGUMENT, "wavefront block size above the kernels' limit");
    CPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bw, wide.trace, block_trace,
                                                           wide_short_stack_bytes(block_trace)));
    CPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bb, bin.trace, block_trace,
                                                           short_stack_bytes(block_trace, short_entries)));
    CPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, k_wf_shade<false>, block_shade, 0));
    *grid_trace = std::max(1, bb) * sm_count;
    *grid_trace_wide = std::max(1, bw) * sm_count;
    *grid_shade = std::max(1, bs) * sm_count;
    return CPT_OK;
}

}  // namespace cpt

// kpcn_tc.cuh — the denoiser's convolutions on the 5th-generation tensor cores (tcgen05.mma,
// BF16 operands from shared memory, FP32 accumulators in tensor memory).  Four kernels:
//   k_conv3x3_tc    one output tile per CTA, operands copied by cp.async (engine 1; described
//                   below)
//   k_conv3x3_ws    warp-specialised persistent kernel fed by TMA im2col loads (engine 2)
//   k_conv3x3_rows  as k_conv3x3_ws for widths that are multiples of 128: one halo box per
//                   channel chunk read by nine row-shifted descriptors, weights resident (engine 2)
//   k_wgrad_tc      weight gradient with MN-major TMA operands (engine 2), plus k_bgrad
//
// k_conv3x3_tc: one CTA (4 warps) computes a tile of 128 consecutive pixels (the MMA's M) by N output channels
// (N = cout / tiles along grid.y, a multiple of 16, at most 256).  K = 9 taps x cin runs in chunks
// of KC = 64 (or 32) channels of one tap: the CTA's threads copy the chunk's A (128 pixel rows,
// shifted by the tap; cp.async zero-fills rows outside the image) and B (N weight rows,
// [tap][cout][cin]) into
// shared memory in the canonical K-major layout without swizzle (8-row x 16-byte core matrices;
// core matrices adjacent along K are 128 bytes apart, 8-row groups KC * 16 bytes apart); one elected
// thread issues KC / 16 tcgen05.mma (K = 16 each) per chunk and commits them to the stage's mbarrier.
// Four stages: the asynchronous copies run two chunks ahead of the MMAs, and a stage is refilled
// once the MMAs that read it (two chunks earlier) have completed, so the tensor core always has the
// next chunk queued.  The epilogue reads the accumulator rows back with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = pixels), adds the bias, applies ReLU and
// stores BF16 and/or FP32 views like k_conv3x3.
//
// Every wait is bounded: a barrier that does not complete within ~2^31 clock cycles sets
// CPT_DEVERR_ITER in *err and the CTA stops issuing work (it still frees its tensor memory).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

namespace cpt {
namespace kpcn {

constexpr int TC_M = 128;          // pixels per CTA tile (MMA M)
constexpr int TC_STAGES = 4;       // shared-memory stages (loads run TC_STAGES - 2 steps ahead)
constexpr int TC_SM_SMEM = 233472; // shared memory per SM (228 KB)

// KC channels per stage; dynamic shared memory of a launch with N = n_tile:
// TC_STAGES x (A + B) + 1 KB alignment slack
__host__ __device__ constexpr int tc_stage_bytes(int kc, int n_tile) { return (TC_M + n_tile) * kc * 2; }
__host__ __device__ constexpr int tc_smem_bytes(int kc, int n_tile) { return TC_STAGES * tc_stage_bytes(kc, n_tile) + 1024; }
constexpr int TC_SMEM_MAX = tc_smem_bytes(64, 256);   // largest launch (KC 64, N 256)

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the barrier phase with the given parity; false (and *err set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err)
{
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > (1LL << 31)) {
            if (err) atomicOr(err, CPT_DEVERR_ITER);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Shared-memory matrix descriptor: start address, leading (K) and stride (M/N) byte offsets,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 16 consecutive FP32 columns of the calling warp's 32 TMEM lanes (one lane per thread).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 16-byte asynchronous global -> shared copy; src_bytes = 0 writes zeros without reading.  The
// activation rows go through L1 (.ca): the three horizontal taps of a row read the same lines in
// consecutive chunks.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_addr(bar)) : "memory");
}

// KC channels per stage (32 or 64; in.C a multiple of KC), cout output channels in grid.y tiles of
// n_tile (a multiple of 16, <= 256); ncols = tensor-memory columns allocated (power of two >=
// n_tile).  The launch's shared memory is sized so that at most 512 / ncols CTAs share an SM, so
// tensor-memory allocations never wait on one another.
template <int KC>
__global__ void __launch_bounds__(128, 1) k_conv3x3_tc(Geo g, View in, const __nv_bfloat16* __restrict__ w,
                                                        const float* __restrict__ bias, int cout, int n_tile,
                                                        int ncols, bool relu, View out16, View out32, int* err)
{
    constexpr uint32_t lbo = 128, sbo = KC * 16;   // core matrices: +128 B along K, +KC*16 B per 8 rows
    constexpr int A_BYTES = TC_M * KC * 2;
    extern __shared__ uint8_t tc_smem_raw[];
    __shared__ uint64_t bar[TC_STAGES];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long P = (long)g.N * g.H * g.W;
    const long p_base = (long)blockIdx.x * TC_M;
    const int n_base = blockIdx.y * n_tile;
    const int cin = in.C;
    const int stage_bytes = tc_stage_bytes(KC, n_tile);
    const __nv_bfloat16* inp = reinterpret_cast<const __nv_bfloat16*>(in.ptr);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < TC_STAGES; ++k) mbar_init(&bar[k], 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = idesc_bf16(TC_M, n_tile);
    uint32_t phase[TC_STAGES];
    uint32_t uses[TC_STAGES];
    for (int k = 0; k < TC_STAGES; ++k) phase[k] = uses[k] = 0u;

    // per-thread rows of A (row-fastest: conflict-free shared stores): row tid, chunks 0..7
    const long p_row = p_base + tid;
    const int x_row = (int)(p_row % g.W), y_row = (int)((p_row / g.W) % g.H);
    const int steps_per_tap = cin / KC;
    const int total = 9 * steps_per_tap;

    auto issue_loads = [&](int step) {
        const int st = step % TC_STAGES;
        const int tap = step / steps_per_tap;
        const int c0 = (step - tap * steps_per_tap) * KC;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        const uint32_t As = smem_addr(smem + st * stage_bytes);
        const uint32_t Bs = As + A_BYTES;
        const bool row_ok = p_row < P && (unsigned)(y_row + dy) < (unsigned)g.H && (unsigned)(x_row + dx) < (unsigned)g.W;
        const __nv_bfloat16* src = row_ok ? inp + (p_row + (long)dy * g.W + dx) * in.cs + in.co + c0 : inp;
#pragma unroll
        for (int kc = 0; kc < KC / 8; ++kc)
            cp_async16(As + (tid >> 3) * sbo + kc * lbo + (tid & 7) * 16, row_ok ? src + kc * 8 : inp,
                       row_ok ? 16u : 0u);
        const __nv_bfloat16* wt = w + ((size_t)tap * cout + n_base) * cin + c0;
        for (int c = tid; c < n_tile * (KC / 8); c += 128) {
            const int n = c % n_tile, kc = c / n_tile;
            cp_async16(Bs + (n >> 3) * sbo + kc * lbo + (n & 7) * 16, wt + (size_t)n * cin + kc * 8, 16u);
        }
    };

    constexpr int AHEAD = TC_STAGES - 2;
    for (int k = 0; k < AHEAD; ++k) {
        if (k < total) issue_loads(k);
        cp_async_commit();
    }
    for (int step = 0; step < total; ++step) {
        const int kn = step + AHEAD;
        if (kn < total) {
            if (kn >= TC_STAGES) {   // the stage's previous chunk (kn - TC_STAGES) must be consumed
                const int ps = kn % TC_STAGES;
                if (!mbar_wait(&bar[ps], phase[ps], err)) abort_flag = 1;
                phase[ps] ^= 1u;
            }
            if (!abort_flag) issue_loads(kn);
        }
        cp_async_commit();
        cp_async_wait<AHEAD>();   // this step's copies have landed
        fence_async_smem();
        __syncthreads();
        if (abort_flag) break;
        const int s = step % TC_STAGES;
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_addr(smem + s * stage_bytes), b0 = a0 + A_BYTES;
#pragma unroll
            for (int j = 0; j < KC / 16; ++j)
                umma_bf16(tmem, smem_desc(a0 + j * 256, lbo, sbo), smem_desc(b0 + j * 256, lbo, sbo), idesc,
                          (step > 0 || j > 0) ? 1u : 0u);
            umma_commit(&bar[s]);
        }
        uses[s] += 1u;
    }
    cp_async_wait<0>();
    // the last commit covers every MMA issued before it
    const int sl = (total - 1) % TC_STAGES;
    bool ok = !abort_flag && mbar_wait(&bar[sl], (uses[sl] - 1u) & 1u, err);
    tc_fence_after();
    if (ok) {
        const long p = p_base + warp * 32 + lane;
        for (int c = 0; c < n_tile; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            if (p >= P) continue;
#pragma unroll
            for (int i = 0; i < 16; i += 2) {
                const int ch = n_base + c + i;
                float v0 = v[i], v1 = v[i + 1];
                if (bias) {
                    v0 += bias[ch];
                    v1 += bias[ch + 1];
                }
                if (out32.ptr) {
                    float* o = reinterpret_cast<float*>(out32.ptr) + p * out32.cs + out32.co + ch;
                    o[0] = v0;
                    o[1] = v1;
                }
                if (out16.ptr) {
                    if (relu) {
                        v0 = fmaxf(v0, 0.f);
                        v1 = fmaxf(v1, 0.f);
                    }
                    __nv_bfloat16* o = reinterpret_cast<__nv_bfloat16*>(out16.ptr) + p * out16.cs + out16.co + ch;
                    *reinterpret_cast<unsigned int*>(o) =
                        pack_bf16(__float2bfloat16_rn(v0), __float2bfloat16_rn(v1));
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// Epilogue of 16 accumulator columns of one pixel: + bias, FP32 view (stored as is) and/or BF16
// view (after ReLU), with 16-byte stores.  ch (the first channel) is a multiple of 16; the views'
// channel strides and offsets are multiples of 8.
__device__ __forceinline__ void store16(long p, int ch, float (&v)[16], const float* __restrict__ bias, bool relu,
                                        const View& out16, const View& out32)
{
    if (bias) {
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
            const float4 b = __ldg(reinterpret_cast<const float4*>(bias + ch + i));
            v[i] += b.x;
            v[i + 1] += b.y;
            v[i + 2] += b.z;
            v[i + 3] += b.w;
        }
    }
    if (out32.ptr) {
        float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(out32.ptr) + p * out32.cs + out32.co + ch);
#pragma unroll
        for (int i = 0; i < 4; ++i) o[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    }
    if (out16.ptr) {
        uint32_t h[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            float a = v[2 * i], b = v[2 * i + 1];
            if (relu) {
                a = fmaxf(a, 0.f);
                b = fmaxf(b, 0.f);
            }
            h[i] = pack_bf16(__float2bfloat16_rn(a), __float2bfloat16_rn(b));
        }
        uint4* o = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out16.ptr) + p * out16.cs + out16.co + ch);
        o[0] = make_uint4(h[0], h[1], h[2], h[3]);
        o[1] = make_uint4(h[4], h[5], h[6], h[7]);
    }
}

// ---------------------------------------------------------------- TMA-fed warp-specialised engine
// Shared-memory descriptor of a K-major operand written by TMA with a 128-byte (KC = 64) or
// 64-byte (KC = 32) swizzle: rows of KC * 2 bytes, 8-row atoms of 8 * KC * 2 bytes (the stride
// between 8-row groups), leading offset unused, layout field 2 (128 B) or 4 (64 B) in bits 61-63.
template <int KC>
__device__ __forceinline__ uint64_t smem_desc_sw(uint32_t addr)
{
    constexpr uint64_t layout = KC == 64 ? 2ull : 4ull;
    constexpr uint32_t sbo = 8 * KC * 2;
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46) |
           (layout << 61);
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// im2col load of 128 pixels x KC channels: coordinates (c, w, h, n) of the first pixel's window
// corner, tap offsets (w, h) in [0, 2]; pixels outside the image read as zeros.
__device__ __forceinline__ void tma_im2col4(uint32_t dst, const CUtensorMap* map, int c, int x, int y, int n,
                                            uint16_t ox, uint16_t oy, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.im2col.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6], {%7, %8};" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c), "r"(x), "r"(y), "r"(n), "r"(smem_addr(bar)), "h"(ox), "h"(oy)
        : "memory");
}

__device__ __forceinline__ void tma_tile4(uint32_t dst, const CUtensorMap* map, int c, int x, int y, int n, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c), "r"(x), "r"(y), "r"(n), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_tile2(uint32_t dst, const CUtensorMap* map, int c, int row, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c), "r"(row), "r"(smem_addr(bar))
        : "memory");
}

// Warp-specialised persistent convolution (192 threads).  Lane 0 of warp 0 is the producer: per
// K step it arms the stage's "full" barrier with the step's byte count and issues two TMA loads,
// an im2col load of the 128 pixel rows shifted by the tap (tma_a: the input view as a 4-D
// {C, W, H, N} tensor, window corners -1..-1, so zero padding comes from TMA's out-of-bounds
// fill) and a tile load of the N weight rows (tma_b: [9 * cout rows][cin]).  Lane 0 of warp 1
// issues the MMAs (waits "full", commits "empty" per stage and "acc full" per tile); warps 2-5
// run the epilogue of the previous tile from the other of two tensor-memory accumulators (wait
// "acc full", tcgen05.ld, stores, arrive "acc empty").  The CTA loops over pixel tiles x,
// x + gridDim.x, ...  Every wait is bounded; a timeout sets CPT_DEVERR_ITER, the roles stop, and
// the producer and MMA thread wait (bounded) for their copies and MMAs in flight before the
// tensor memory is freed.
constexpr int TC_WS_STAGES = 8;   // most shared-memory stages of k_conv3x3_ws (the launch picks nst)

template <int KC>
__global__ void __launch_bounds__(192, 1) k_conv3x3_ws(const __grid_constant__ CUtensorMap tma_a,
                                                        const __grid_constant__ CUtensorMap tma_b, Geo g, int cin,
                                                        const float* __restrict__ bias, int cout, int n_tile,
                                                        int ncols, int nst, bool relu, View out16, View out32,
                                                        int* err)
{
    constexpr int A_BYTES = TC_M * KC * 2;
    extern __shared__ uint8_t tc_smem_raw[];
    __shared__ uint64_t full[TC_WS_STAGES], empty[TC_WS_STAGES], accfull[2], accempty[2];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int ws_abort;   // set by any role whose wait timed out; the others stop
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long P = (long)g.N * g.H * g.W;
    const long m_tiles = (P + TC_M - 1) / TC_M;
    const int my_tiles = m_tiles > (long)blockIdx.x ? (int)((m_tiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    const int n_base = blockIdx.y * n_tile;
    const int stage_bytes = tc_stage_bytes(KC, n_tile);
    const int steps_per_tap = cin / KC;
    const int T = 9 * steps_per_tap;
    const long total = (long)my_tiles * T;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(2 * ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < nst; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accfull[b], 1);
            mbar_init(&accempty[b], 128);
        }
        ws_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tma_a)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tma_b)) : "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        // ---------------- producer
        if (lane == 0) {
            long gs = 0;
            for (int i = 0; i < my_tiles && !ws_abort; ++i) {
                const long p0 = ((long)blockIdx.x + (long)i * gridDim.x) * TC_M;
                const int x0 = (int)(p0 % g.W), y0 = (int)((p0 / g.W) % g.H), n0 = (int)(p0 / ((long)g.W * g.H));
                for (int k = 0; k < T; ++k, ++gs) {
                    const int st = (int)(gs % nst);
                    const long fill = gs / nst;
                    if (ws_abort) break;
                    if (fill > 0 && !mbar_wait(&empty[st], (uint32_t)((fill - 1) & 1), err)) {
                        ws_abort = 1;
                        break;
                    }
                    const int tap = k / steps_per_tap;
                    const int c0 = (k - tap * steps_per_tap) * KC;
                    const uint32_t As = smem_addr(smem + st * stage_bytes);
                    mbar_expect_tx(&full[st], (uint32_t)stage_bytes);
                    tma_im2col4(As, &tma_a, c0, x0 - 1, y0 - 1, n0, (uint16_t)(tap % 3), (uint16_t)(tap / 3), &full[st]);
                    tma_tile2(As + A_BYTES, &tma_b, c0, tap * cout + n_base, &full[st]);
                }
            }
            // copies still in flight land before the CTA leaves (every stage's last fill)
            for (int st = 0; st < nst && st < gs; ++st) {
                const long last = (gs - 1 - st) / nst;   // fills of stage st: 0..last
                mbar_wait(&full[st], (uint32_t)(last & 1), err);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(TC_M, n_tile);
            long gs = 0;
            for (; gs < total; ++gs) {
                const int st = (int)(gs % nst);
                const int i = (int)(gs / T), k = (int)(gs % T);
                const int buf = i & 1;
                if (ws_abort) break;
                if ((k == 0 && i >= 2 && !mbar_wait(&accempty[buf], (uint32_t)(((i >> 1) - 1) & 1), err)) ||
                    !mbar_wait(&full[st], (uint32_t)((gs / nst) & 1), err)) {
                    ws_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t a0 = smem_addr(smem + st * stage_bytes), b0 = a0 + A_BYTES;
                const uint32_t d = tmem + (uint32_t)(buf * ncols);
#pragma unroll
                for (int j = 0; j < KC / 16; ++j)
                    umma_bf16(d, smem_desc_sw<KC>(a0 + j * 32), smem_desc_sw<KC>(b0 + j * 32), idesc,
                              (k > 0 || j > 0) ? 1u : 0u);
                umma_commit(&empty[st]);
                if (k == T - 1) umma_commit(&accfull[buf]);
            }
            // the MMAs issued so far finish before the tensor memory is freed
            if (gs > 0) mbar_wait(&empty[(gs - 1) % nst], (uint32_t)(((gs - 1) / nst) & 1), err);
        }
    } else {
        // ---------------- epilogue (warps 2-5 own TMEM lane quarters 2, 3, 0, 1)
        const int quarter = warp & 3;
        for (int i = 0; i < my_tiles; ++i) {
            const int buf = i & 1;
            if (ws_abort) break;
            if (!mbar_wait(&accfull[buf], (uint32_t)((i >> 1) & 1), err)) {
                ws_abort = 1;
                break;
            }
            tc_fence_after();
            const long p = ((long)blockIdx.x + (long)i * gridDim.x) * TC_M + quarter * 32 + lane;
            const uint32_t base = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * ncols);
            for (int c = 0; c < n_tile; c += 16) {
                float v[16];
                tmem_ld16(base + (uint32_t)c, v);
                if (p < P) store16(p, n_base + c, v, bias, relu, out16, out32);
            }
            tc_fence_before();
            mbar_arrive(&accempty[buf]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * ncols) : "memory");
    }
}

// ---------------------------------------------------------------- row-tile engine
// A tile is 128 consecutive positions.  When W % 128 == 0 they are 128 pixels of one image row
// (x0 .. x0 + 127 of row y) and per KC-channel chunk the producer loads one TMA box of 3 rows x 130
// pixels (x0 - 1 .. x0 + 128 of rows y - 1 .. y + 1; zeros outside the image from the
// out-of-bounds fill) with the KC * 2-byte swizzle.  Other widths use positions of pitch W + 1:
// three im2col boxes of 130 positions (one per dy) whose bounding box has one extra column per row
// that reads as zeros, so position q + dx is still the left/centre/right neighbour of position q
// (across a row end it lands on the zero column); the position W of each row is a padding output
// the epilogue skips.  Either way the nine taps read the rows through descriptors whose start row
// is dy * (segment) + dx: each input pixel crosses L2 -> SM once per chunk instead of nine times.  The tensor core applies the swizzle to absolute
// shared-memory address bits (as TMA does), so a start row off the 1024-byte pattern boundary
// needs no matrix base offset (with the base-offset field set to (address >> 7) & 7 the products
// are wrong; with 0 they match the oracle bit for bit).  The weights of the CTA's output channels
// stay resident in shared memory (loaded once, 9 x cin / KC tiles of n_tile x KC) when they fit,
// else each stage also carries its chunk's nine weight tiles.  Roles and waits as in
// k_conv3x3_ws.
constexpr int ROW_PIX = TC_M + 2;   // pixels per box row (with halo)
// bytes of the activation rows of one stage (3 rows of 130 pixels x kc channels)
__host__ __device__ constexpr int row_a_tx(int kc) { return 3 * ROW_PIX * kc * 2; }
__host__ __device__ constexpr int row_b_bytes(int cin, int n_tile, int kc) { return 9 * (cin / kc) * n_tile * kc * 2; }

// Shared-memory plan of a k_conv3x3_rows launch.  pitched: the activation rows come from three
// im2col boxes (one per dy, each at a 1024-byte aligned segment a_seg apart) over positions of
// pitch W + 1 (the bounding box's extra column per row reads as zeros, so the horizontal taps stay
// row shifts whatever the width); else from one tiled box of 3 contiguous segments (W % 128 == 0).
// resident: all weights loaded once before the stages; else each stage carries its chunk's nine
// weight tiles after the activation region (a_region bytes).
struct RowPlan {
    int a_seg, a_region, stage;
    bool pitched, resident;
};

// Kernel apply fused into the logits convolution's epilogue (inference): the 32 accumulator
// columns of a pixel are its logits (25 used); softmax, then the weighted 5x5 gather of the
// noisy radiance rad [N][H][W][3] (clamped to the real Hr x Wr image) into out, as k_apply.
struct ApplyArgs {
    const float* rad;
    float* out;
    int Hr, Wr;
};

__device__ __forceinline__ void apply_pixel(long p, const Geo& g, const float (&l0)[16], const float (&l1)[16],
                                            const float* __restrict__ bias, const ApplyArgs& ap)
{
    float lg[KTAPS];
    float mx = -3.0e38f;
#pragma unroll
    for (int k = 0; k < KTAPS; ++k) {
        lg[k] = (k < 16 ? l0[k & 15] : l1[k & 15]) + __ldg(bias + k);
        mx = fmaxf(mx, lg[k]);
    }
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < KTAPS; ++k) {
        lg[k] = expf(lg[k] - mx);
        sum += lg[k];
    }
    const float inv = 1.f / sum;
    const int x = (int)(p % g.W), y = (int)((p / g.W) % g.H);
    const long b = p / ((long)g.W * g.H);
    const int xc = min(x, ap.Wr - 1), yc = min(y, ap.Hr - 1);
    float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
    for (int k = 0; k < KTAPS; ++k) {
        const float wk = lg[k] * inv;
        const int xx = min(max(xc + k % KSIZE - KSIZE / 2, 0), ap.Wr - 1);
        const int yy = min(max(yc + k / KSIZE - KSIZE / 2, 0), ap.Hr - 1);
        const float* r = ap.rad + 3 * ((b * g.H + yy) * g.W + xx);
        ax += wk * __ldg(r);
        ay += wk * __ldg(r + 1);
        az += wk * __ldg(r + 2);
    }
    ap.out[3 * p] = ax;
    ap.out[3 * p + 1] = ay;
    ap.out[3 * p + 2] = az;
}

template <int KC, bool APPLY>
__global__ void __launch_bounds__(192, 1) k_conv3x3_rows(const __grid_constant__ CUtensorMap tma_a,
                                                          const __grid_constant__ CUtensorMap tma_b, Geo g, int cin,
                                                          const float* __restrict__ bias, int cout, int n_tile,
                                                          int ncols, int nst, RowPlan rp, ApplyArgs ap, bool relu,
                                                          View out16, View out32, int* err)
{
    extern __shared__ uint8_t tc_smem_raw[];
    __shared__ uint64_t full[TC_WS_STAGES], empty[TC_WS_STAGES], accfull[2], accempty[2], bfull;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int ws_abort;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // tile positions: pixels (tiled boxes) or positions of the W + 1 pitch (im2col boxes, whose
    // position W of a row is a padding output that the epilogue skips)
    const int Wq = rp.pitched ? g.W + 1 : g.W;
    const long Q = (long)g.N * g.H * Wq;
    const long m_tiles = (Q + TC_M - 1) / TC_M;
    const int my_tiles = m_tiles > (long)blockIdx.x ? (int)((m_tiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    const int n_base = blockIdx.y * n_tile;
    const int chunks = cin / KC;
    const int b_tile = n_tile * KC * 2;                    // one weight tile: n_tile rows x KC channels
    const int b_bytes = rp.resident ? 9 * chunks * b_tile : 0;
    const uint32_t Bs = smem_addr(smem);
    const uint32_t As0 = Bs + (uint32_t)b_bytes;            // b_bytes is a multiple of 1024
    const long total = (long)my_tiles * chunks;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(2 * ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < nst; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accfull[b], 1);
            mbar_init(&accempty[b], 128);
        }
        mbar_init(&bfull, 1);
        ws_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tma_a)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tma_b)) : "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        // ---------------- producer: resident weights once, then per (tile, chunk) the activation
        // rows (one tiled box, or three im2col boxes, one per dy) and, when not resident, the
        // chunk's nine weight tiles
        if (lane == 0) {
            if (rp.resident) {
                mbar_expect_tx(&bfull, (uint32_t)b_bytes);
                for (int t = 0; t < 9; ++t)
                    for (int c = 0; c < chunks; ++c)
                        tma_tile2(Bs + (uint32_t)((t * chunks + c) * b_tile), &tma_b, c * KC, t * cout + n_base,
                                  &bfull);
            }
            const uint32_t tx = (uint32_t)(row_a_tx(KC) + (rp.resident ? 0 : 9 * b_tile));
            long gs = 0;
            for (int i = 0; i < my_tiles && !ws_abort; ++i) {
                const long p0 = ((long)blockIdx.x + (long)i * gridDim.x) * TC_M;
                const int x0 = (int)(p0 % Wq), y0 = (int)((p0 / Wq) % g.H), n0 = (int)(p0 / ((long)Wq * g.H));
                for (int c = 0; c < chunks; ++c, ++gs) {
                    const int st = (int)(gs % nst);
                    const long fill = gs / nst;
                    if (ws_abort) break;
                    if (fill > 0 && !mbar_wait(&empty[st], (uint32_t)((fill - 1) & 1), err)) {
                        ws_abort = 1;
                        break;
                    }
                    const uint32_t a = As0 + (uint32_t)(st * rp.stage);
                    mbar_expect_tx(&full[st], tx);
                    if (rp.pitched) {
                        for (int dy = 0; dy < 3; ++dy)
                            tma_im2col4(a + (uint32_t)(dy * rp.a_seg), &tma_a, c * KC, x0 - 1, y0 - 1, n0, (uint16_t)0,
                                        (uint16_t)dy, &full[st]);
                    } else {
                        tma_tile4(a, &tma_a, c * KC, x0 - 1, y0 - 1, n0, &full[st]);
                    }
                    if (!rp.resident)
                        for (int t = 0; t < 9; ++t)
                            tma_tile2(a + (uint32_t)(rp.a_region + t * b_tile), &tma_b, c * KC, t * cout + n_base,
                                      &full[st]);
                }
            }
            for (int st = 0; st < nst && st < gs; ++st) {
                const long last = (gs - 1 - st) / nst;
                mbar_wait(&full[st], (uint32_t)(last & 1), err);
            }
            if (rp.resident) mbar_wait(&bfull, 0u, err);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(TC_M, n_tile);
            long gs = 0;
            if (rp.resident && total > 0 && !mbar_wait(&bfull, 0u, err)) ws_abort = 1;
            for (; gs < total && !ws_abort; ++gs) {
                const int st = (int)(gs % nst);
                const int i = (int)(gs / chunks), c = (int)(gs % chunks);
                const int buf = i & 1;
                if ((c == 0 && i >= 2 && !mbar_wait(&accempty[buf], (uint32_t)(((i >> 1) - 1) & 1), err)) ||
                    !mbar_wait(&full[st], (uint32_t)((gs / nst) & 1), err)) {
                    ws_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t a0 = As0 + (uint32_t)(st * rp.stage);
                const uint32_t d = tmem + (uint32_t)(buf * ncols);
                for (int t = 0; t < 9; ++t) {
                    const uint32_t at = a0 + (uint32_t)((t / 3) * rp.a_seg + (t % 3) * KC * 2);
                    const uint32_t bt = rp.resident ? Bs + (uint32_t)((t * chunks + c) * b_tile)
                                                    : a0 + (uint32_t)(rp.a_region + t * b_tile);
#pragma unroll
                    for (int j = 0; j < KC / 16; ++j)
                        umma_bf16(d, smem_desc_sw<KC>(at + j * 32), smem_desc_sw<KC>(bt + j * 32), idesc,
                                  (c > 0 || t > 0 || j > 0) ? 1u : 0u);
                }
                umma_commit(&empty[st]);
                if (c == chunks - 1) umma_commit(&accfull[buf]);
            }
            if (gs > 0) mbar_wait(&empty[(gs - 1) % nst], (uint32_t)(((gs - 1) / nst) & 1), err);
        }
    } else {
        // ---------------- epilogue (warps 2-5 own TMEM lane quarters 2, 3, 0, 1)
        const int quarter = warp & 3;
        for (int i = 0; i < my_tiles; ++i) {
            const int buf = i & 1;
            if (ws_abort) break;
            if (!mbar_wait(&accfull[buf], (uint32_t)((i >> 1) & 1), err)) {
                ws_abort = 1;
                break;
            }
            tc_fence_after();
            const long q = ((long)blockIdx.x + (long)i * gridDim.x) * TC_M + quarter * 32 + lane;
            const int qx = (int)(q % Wq);
            const bool valid = q < Q && qx < g.W;
            const long p = (q / Wq) * g.W + qx;
            const uint32_t base = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * ncols);
            if (APPLY) {   // n_tile == 32: the pixel's logits
                float l0[16], l1[16];
                tmem_ld16(base, l0);
                tmem_ld16(base + 16u, l1);
                if (valid) apply_pixel(p, g, l0, l1, bias, ap);
            } else {
                for (int c = 0; c < n_tile; c += 16) {
                    float v[16];
                    tmem_ld16(base + (uint32_t)c, v);
                    if (valid) store16(p, n_base + c, v, bias, relu, out16, out32);
                }
            }
            tc_fence_before();
            mbar_arrive(&accempty[buf]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * ncols) : "memory");
    }
}

// ---------------------------------------------------------------- weight gradient on tcgen05
// dW[tap][ci][co] = sum_p X[p + off(tap), ci] dZ[p, co] as GEMMs with K = pixels.  A CTA owns one
// tap row dy (three taps), 128 output-gradient channels co (M; dZ channels beyond cout read as zeros)
// and up to 64 input channels ci (N), and a contiguous chunk of 64-pixel tiles.  Per tile the
// producer loads dZ (2D map over {cout, P}: two 64-channel boxes of 64 pixels) and, per tap, X
// through an im2col map (64 channels x 64 pixels shifted by the tap, zeros outside the image);
// both land in the 128-byte-swizzled MN-major layout (pixel rows of 128 bytes, 8-row groups
// 1024 bytes apart = SBO, 64-channel atoms 8 KB apart = LBO).  The three taps' X tiles sit in
// consecutive atoms, so one MMA with N = 3 x 64 covers all three taps (columns 64 t + ci; channels
// beyond the slice are zeros); the MMA thread accumulates over the whole chunk (4 MMAs per tile) in
// tensor memory; at the end the
// epilogue warps write the chunk's partial sums part[chunk][tap][ci][co] (lane = co: coalesced),
// which a fixed-order reduction over chunks turns into the gradient.
constexpr int WT_PIX = 64;                       // pixels (K) per tile
constexpr int WT_ATOM = WT_PIX * 128;            // one 64-channel x 64-pixel box (8 KB)
constexpr int WT_STAGE = 5 * WT_ATOM;            // dZ (2 atoms) + X for three taps
constexpr int WT_STAGES = 2;   // two CTAs per SM fit (shared and tensor memory); faster than one CTA with 4-5 stages
constexpr int WT_SMEM = WT_STAGES * WT_STAGE + 1024 + 16384;   // + alignment and slack

// MN-major operand descriptor (128-byte swizzle): LBO = stride of 64-element MN atoms, SBO = stride
// of 8-row K groups.
__device__ __forceinline__ uint64_t smem_desc_mn128(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (2ull << 61);
}

// Instruction descriptor of kind::f16 with both operands MN-major (transpose bits 15, 16).
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int m, int n) { return idesc_bf16(m, n) | (1u << 15) | (1u << 16); }

__global__ void __launch_bounds__(192, 1) k_wgrad_tc(const __grid_constant__ CUtensorMap tma_x,
                                                      const __grid_constant__ CUtensorMap tma_z, Geo g, int cin,
                                                      int cout, int n_slices, int tiles_per_chunk,
                                                      float* __restrict__ part, int* err)
{
    extern __shared__ uint8_t tc_smem_raw[];
    __shared__ uint64_t full[WT_STAGES], empty[WT_STAGES], done;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int ws_abort;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long P = (long)g.N * g.H * g.W;
    const long n_tiles = (P + WT_PIX - 1) / WT_PIX;
    const long t0 = (long)blockIdx.x * tiles_per_chunk;
    const long left = n_tiles - t0;
    const int my_tiles = left <= 0 ? 0 : (left < tiles_per_chunk ? (int)left : tiles_per_chunk);
    const int dy_row = blockIdx.y % 3;                       // taps 3 dy_row .. 3 dy_row + 2
    const int n_base = (blockIdx.y / 3 % n_slices) * 64;     // ci
    const int m_base = (blockIdx.y / (3 * n_slices)) * 128;  // co
    const int nn = cin - n_base < 64 ? cin - n_base : 64;  // 32 or 64
    const bool two_z = m_base + 64 < cout;
    const uint32_t S0 = smem_addr(smem);

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(256)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < WT_STAGES; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], 1);
        }
        mbar_init(&done, 1);
        ws_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tma_x)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tma_z)) : "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int i = 0;
            for (; i < my_tiles && !ws_abort; ++i) {
                const int st = i % WT_STAGES;
                if (i >= WT_STAGES && !mbar_wait(&empty[st], (uint32_t)(((i / WT_STAGES) - 1) & 1), err)) {
                    ws_abort = 1;
                    break;
                }
                const long p0 = (t0 + i) * WT_PIX;
                const int x0 = (int)(p0 % g.W), y0 = (int)((p0 / g.W) % g.H), n0 = (int)(p0 / ((long)g.W * g.H));
                const uint32_t a = S0 + (uint32_t)(st * WT_STAGE);
                // the second dZ atom only when it holds channels (otherwise its D rows are never read)
                mbar_expect_tx(&full[st], (uint32_t)(two_z ? WT_STAGE : WT_STAGE - WT_ATOM));
                tma_tile2(a, &tma_z, m_base, (int)p0, &full[st]);
                if (two_z) tma_tile2(a + WT_ATOM, &tma_z, m_base + 64, (int)p0, &full[st]);
                for (int t = 0; t < 3; ++t)
                    tma_im2col4(a + (uint32_t)((2 + t) * WT_ATOM), &tma_x, n_base, x0 - 1, y0 - 1, n0, (uint16_t)t,
                                (uint16_t)dy_row, &full[st]);
            }
            for (int st = 0; st < WT_STAGES && st < i; ++st)
                mbar_wait(&full[st], (uint32_t)(((i - 1 - st) / WT_STAGES) & 1), err);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16_mn(128, 192);
            int i = 0;
            for (; i < my_tiles && !ws_abort; ++i) {
                const int st = i % WT_STAGES;
                if (!mbar_wait(&full[st], (uint32_t)((i / WT_STAGES) & 1), err)) {
                    ws_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t a = S0 + (uint32_t)(st * WT_STAGE);
                // the three taps' X tiles are consecutive 64-channel atoms: one N = 192 operand
#pragma unroll
                for (int k = 0; k < WT_PIX / 16; ++k)
                    umma_bf16(tmem, smem_desc_mn128(a + k * 2048, WT_ATOM, 1024),
                              smem_desc_mn128(a + (uint32_t)(2 * WT_ATOM) + k * 2048, WT_ATOM, 1024), idesc,
                              (i > 0 || k > 0) ? 1u : 0u);
                umma_commit(&empty[st]);
            }
            if (i > 0) umma_commit(&done);   // completes when every MMA issued above has finished
            else mbar_arrive(&done);
        }
    } else {
        // ---------------- epilogue: warps 2-5 own TMEM lanes (co) 32 * (warp & 3) ..
        const int quarter = warp & 3;
        const bool ok = mbar_wait(&done, 0u, err) && !ws_abort;
        tc_fence_after();
        const int co = m_base + quarter * 32 + lane;
        for (int t = 0; t < 3 && ok; ++t) {
            float* out = part + ((size_t)blockIdx.x * 9 + dy_row * 3 + t) * cin * cout;
            for (int c = 0; c < nn; c += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(t * 64 + c), v);
                if (co < cout) {
#pragma unroll
                    for (int q = 0; q < 16; ++q) out[(size_t)(n_base + c + q) * cout + co] = v[q];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256) : "memory");
    }
}

// Bias gradient partial sums: bpart[chunk][co] = sum of dZ[p, co] over the chunk's pixels in a fixed
// order.  Thread t owns channels 8 (t % C8) .. + 7 (one 16-byte load per pixel) and pixel lane
// t / C8 of L = 256 / C8 lanes (every L-th pixel); the lanes are then added in order.
__global__ void k_bgrad(View dz, long P, int cout, long chunk_pixels, float* __restrict__ bpart)
{
    const long pbeg = (long)blockIdx.x * chunk_pixels, pend = P < pbeg + chunk_pixels ? P : pbeg + chunk_pixels;
    __shared__ float red[256][8];
    const __nv_bfloat16* zp = reinterpret_cast<const __nv_bfloat16*>(dz.ptr);
    const int C8 = cout / 8, L = 256 / C8;   // cout <= 160: C8 <= 20, L >= 12
    const int cg = threadIdx.x % C8, lane = threadIdx.x / C8;
    float acc[8] = {};
    if (lane < L)
        for (long p = pbeg + lane; p < pend; p += L) {
            const uint4 v = *reinterpret_cast<const uint4*>(zp + p * dz.cs + dz.co + cg * 8);
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(h[j]);
                acc[2 * j] += f.x;
                acc[2 * j + 1] += f.y;
            }
        }
#pragma unroll
    for (int j = 0; j < 8; ++j) red[threadIdx.x][j] = acc[j];
    __syncthreads();
    if (threadIdx.x < cout) {
        const int g8 = threadIdx.x / 8, j = threadIdx.x % 8;
        float s = 0.f;
        for (int k = 0; k < L; ++k) s += red[k * C8 + g8][j];
        bpart[(size_t)blockIdx.x * cout + threadIdx.x] = s;
    }
}

}  // namespace kpcn
}  // namespace cpt

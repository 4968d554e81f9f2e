// cpt_device.cuh — device-side types and FP32 maths shared by the LBVH, trace and render
// kernels.  Float restatements of the reference's double3 helpers (rtmath.cuh:17-112).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define CPT_INF_F 999999.0f                 // INF (rtmath.cuh:8)
#define CPT_PI_F 3.14159265358979323846f     // PI (rtmath.cuh:9)
#define CPT_STACK 64                          // Karras trees over 64-bit keys are at most 65 levels deep
#define CPT_WSTACK 72                         // 8-wide traversal: at most one node group per level
#define CPT_WIDE_F4 6                         // float4 per wide node (96 bytes)
#define CPT_WIDE_EMPTY 0x7fffffff             // child reference of an unused wide-node slot

// Primitive kinds stored in leaf records (w of the second float4).
enum { CPT_KIND_TRI = 0, CPT_KIND_SPHERE = 1, CPT_KIND_LIGHT = 2 };

// ------------------------------------------------------------------ float3 maths
__host__ __device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float3 operator*(float t, float3 v) { return f3(v.x * t, v.y * t, v.z * t); }
__host__ __device__ __forceinline__ float3 operator*(float3 v, float t) { return f3(v.x * t, v.y * t, v.z * t); }
__host__ __device__ __forceinline__ float3 operator/(float3 v, float t) { return f3(v.x / t, v.y / t, v.z / t); }
__host__ __device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float len2(float3 v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
__host__ __device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 unit3(float3 v) { return v / sqrtf(len2(v)); }

// ------------------------------------------------------------------ device scene types
struct DevMaterial {   // Material (Material.cuh:5-22) in FP32
    float3 color;
    float ax, ay;
    int type;
    float eta;
    float sigma_t, albedo;
    int tex;           // image index in SceneView::tex, -1 = plain colour
    float pad[2];
};

struct DevImage {      // 8-bit RGB texels, rows in file order (Triangle::texture, Camera::d_image)
    const uint8_t* __restrict__ rgb;
    int w, h;
};

struct DevLight {      // Light (Hittable.cuh:346-366): centre, unit normal, edge frame
    float3 center;
    float w;
    float3 normal;
    float h;
    float3 eu;
    int visible;
    float3 ev;
    int pad0;
    float3 color;
    int pad1;
};

struct DevCamera {     // Camera (Camera.cu:5-40), derived in double on the host
    float3 look_from;
    float3 pixel_center;
    float3 delta_h;
    float3 delta_v;
    float3 background;
    int width, height;
};

// Read-only view of a built scene passed to trace/render kernels by value.
struct SceneView {
    int n_prims, n_lights, n_spheres, n_tris, n_internal;
    const float4* __restrict__ nodes;      // BVH2: 4 float4 per internal node (Aila-Laine layout), or 2 (node_q)
    int node_q;                            // BVH2 nodes are compressed (quantised child boxes, 32 bytes)
    const float4* __restrict__ wide;       // BVH8: CPT_WIDE_F4 float4 per wide node, or NULL (use BVH2)
    const float4* __restrict__ leaf_rec;   // 3 float4 per leaf (sorted order, or wide slot order)
    const uint32_t* __restrict__ tri_mat;  // per triangle
    const float* __restrict__ tri_n;       // optional smooth normals, 9 per triangle
    const float4* __restrict__ spheres;    // centre xyz, radius
    const uint32_t* __restrict__ sphere_mat;
    const DevLight* __restrict__ lights;
    const DevMaterial* __restrict__ mats;
    const float* __restrict__ tri_uv;      // optional: 6 per triangle (uv0, uv1, uv2)
    const DevImage* __restrict__ tex;      // images referenced by DevMaterial::tex
    DevImage sky;                          // equirectangular sky, rgb NULL = background colour
    DevCamera cam;
};

// ------------------------------------------------------------------ PCG32
// Config estimator: sample k of a pixel draws from the pixel's PCG32 stream started k * 2^32
// draws ahead (no sample draws 2^32 numbers), so the samples of one pixel are independent and
// an integrator may run them in any order or in parallel.  Sample radiance is summed in groups
// of sample_group(spp) consecutive samples and the group sums are added in group order, which
// fixes the FP32 summation order for every integrator.
constexpr uint64_t CPT_PCG_MULT = 6364136223846793005ULL;

// The LCG step x -> a x + c applied 2^n times is x -> A x + c P; jump_mult(n) = A and
// jump_plus(n) = P (Brown 1994, "Random number generation with arbitrary strides").
constexpr uint64_t pcg_jump_mult(int n)
{
    uint64_t m = CPT_PCG_MULT;
    for (int i = 0; i < n; ++i) m *= m;
    return m;
}
constexpr uint64_t pcg_jump_plus(int n)
{
    uint64_t m = CPT_PCG_MULT, p = 1;
    for (int i = 0; i < n; ++i) {
        p *= m + 1;
        m *= m;
    }
    return p;
}
constexpr uint64_t CPT_PCG_JUMP32_MULT = pcg_jump_mult(32);
constexpr uint64_t CPT_PCG_JUMP32_PLUS = pcg_jump_plus(32);

__host__ __device__ __forceinline__ int sample_group(int spp) { return spp <= 256 ? 8 : (spp + 31) / 32; }

#ifdef __CUDACC__
// PCG32 (O'Neill 2014, pcg32_srandom_r / pcg32_random_r); uniforms are (x + 1) * 2^-32 in
// (0, 1], rounded once to FP32, the stand-in for curand_uniform_double (Render.cu:43).
struct Pcg32 {
    uint64_t state, inc;
    __device__ __forceinline__ uint32_t next()
    {
        uint64_t old = state;
        state = old * CPT_PCG_MULT + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return __funnelshift_r(xs, xs, rot);
    }
    __device__ __forceinline__ void init(uint64_t seed, uint64_t stream)
    {
        state = 0u;
        inc = (stream << 1u) | 1u;
        next();
        state += seed;
        next();
    }
    // Moves the generator k * 2^32 draws ahead in O(log k) steps.
    __device__ __forceinline__ void jump_samples(uint32_t k)
    {
        uint64_t cm = CPT_PCG_JUMP32_MULT, cp = CPT_PCG_JUMP32_PLUS * inc, am = 1, ap = 0;
        while (k) {
            if (k & 1u) {
                am *= cm;
                ap = ap * cm + cp;
            }
            cp *= cm + 1;
            cm *= cm;
            k >>= 1;
        }
        state = am * state + ap;
    }
    // Generator of sample k of the pixel with stream `stream` (config estimator).
    __device__ __forceinline__ void init_sample(uint64_t seed, uint64_t stream, uint32_t k)
    {
        init(seed, stream);
        jump_samples(k);
    }
    __device__ __forceinline__ float uniform() { return __ull2float_rn((uint64_t)next() + 1ull) * 2.3283064365386963e-10f; }
    // 1 - uniform(), computed from the integer so it is not lost to cancellation near 1.
    __device__ __forceinline__ float one_minus_uniform_from(uint32_t x) { return __uint2float_rn(~x) * 2.3283064365386963e-10f; }
};
#endif

// ------------------------------------------------------------------ traversal stack
// The binary traversal keeps the bottom SHORT entries of its stack in shared memory and the rest
// in local memory.  Every kernel that traverses the BVH2 with a short stack is launched with
// short_stack_bytes(threads per block, SHORT) of dynamic shared memory; thread t owns the column
// t, t + T, t + 2T, ... (T = threads per block), so a warp's pushes and pops hit 32 distinct banks.
// The wavefront's trace kernels are instantiated for the depths the autotuner may pick.
#define CPT_SHORT_STACK 16
inline constexpr size_t short_stack_bytes(int threads, int entries = CPT_SHORT_STACK)
{
    return (size_t)entries * threads * sizeof(int);
}

// The 8-wide traversal's short stack: 64-bit group entries.
#define CPT_WIDE_SHORT_STACK 8
inline constexpr size_t wide_short_stack_bytes(int threads, int entries = CPT_WIDE_SHORT_STACK)
{
    return (size_t)entries * threads * sizeof(uint64_t);
}

#ifdef __CUDACC__
template <int SHORT>
struct ShortStackN {
    static_assert(SHORT > 0 && SHORT < CPT_STACK, "short stack depth");
    int* col;     // this thread's column in the block's dynamic shared array
    int stride;   // threads per block
    int spill[CPT_STACK - SHORT];
    __device__ __forceinline__ void init()
    {
        extern __shared__ int cpt_short_stack_smem[];
        const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
        col = cpt_short_stack_smem + t;
        stride = blockDim.x * blockDim.y * blockDim.z;
    }
    __device__ __forceinline__ void put(int i, int v)
    {
        if (i < SHORT) col[i * stride] = v;
        else spill[i - SHORT] = v;
    }
    __device__ __forceinline__ int get(int i) const { return i < SHORT ? col[i * stride] : spill[i - SHORT]; }
};
using ShortStack = ShortStackN<CPT_SHORT_STACK>;

// The whole stack in local memory (no shared memory needed at launch).
struct LocalStack {
    int s[CPT_STACK];
    __device__ __forceinline__ void init() {}
    __device__ __forceinline__ void put(int i, int v) { s[i] = v; }
    __device__ __forceinline__ int get(int i) const { return s[i]; }
};
#endif

// ------------------------------------------------------------------ error word
// Device-side error flags set by kernels that hit a limit (stack, iteration budget).
enum { CPT_DEVERR_STACK = 1, CPT_DEVERR_ITER = 2 };

// api.cu — the C ABI of libcpt.so (include/cpt.h): contexts, scenes, LBVH build/export,
// closest-hit queries and rendering.  Scene memory is owned by the library; caller
// buffers are borrowed for the duration of a call.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "cpt_internal.h"

namespace cpt {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches(0);

void add_launches(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

void set_error(const std::string& msg) { g_last_error = msg; }

cpt_status fail(cpt_status st, const std::string& msg)
{
    set_error(msg);
    return st;
}

cpt_status cuda_fail(cudaError_t e, const char* what)
{
    cpt_status st = (e == cudaErrorMemoryAllocation) ? CPT_ERR_OUT_OF_MEMORY : CPT_ERR_CUDA;
    return fail(st, std::string(what) + ": " + cudaGetErrorString(e));
}

struct IniScene;
cpt_status ini_load(const char* path, IniScene** out);
const cpt_scene_desc* ini_desc(const IniScene* s);
void ini_free(IniScene* s);

}  // namespace cpt

using namespace cpt;

struct cpt_context {
    int device;
    int sm_count;
    int render_block_x, render_block_y;
    WavefrontTuning wf;        // grids are filled on first use
    bool wf_grids_ready;
    int bvh_width;             // traversal layout built by cpt_lbvh_build: 8 (compressed wide) or 2
    int iter_limit;            // loop trips per sample of the render loops (cpt_context_set_loop_limits)
    bool bvh2_compressed;      // BVH2 nodes of later builds: 32-byte quantised (cpt_context_set_bvh_compression)
};

namespace cpt {
cpt_status wavefront_grids(int sm_count, int block_trace, int block_shade, int short_entries, int* grid_trace,
                           int* grid_trace_wide, int* grid_shade);
size_t wide_scratch_bytes(uint32_t n);
cpt_status build_wide(uint32_t n, const int2* child, const float4* node_box, const float4* leaf_box, float4* wide,
                      void* scratch, size_t scratch_bytes, cudaStream_t stream, uint32_t* num_wide);
}

struct cpt_scene {
    cpt_context* ctx;
    uint32_t n_lights, n_spheres, n_tris, n;
    cpt_camera camera;
    DevCamera cam;
    double bmin[3], bmax[3];
    bool tri_is_f64;
    bool built;
    // inputs on the device
    float* tri_f32;
    double* tri_f64;
    float* tri_n;
    float* tri_uv;
    uint32_t* tri_mat;
    float4* spheres;
    uint32_t* sphere_mat;
    DevLight* lights;
    DevMaterial* mats;
    uint32_t n_mats;
    double* extra_c;
    float4* extra_box;
    // LBVH
    uint64_t* keys;
    uint32_t* order;
    int2* child;
    int2* range;
    float4* node_box;
    float4* leaf_box;
    void* scratch;
    size_t scratch_bytes;
    // traversal layout
    int width;          // layout of the last build: 2 or 8
    bool node_q;        // the BVH2 nodes of the last build are compressed
    float4* nodes;      // BVH2 nodes (width 2)
    float4* wide;       // compressed 8-wide nodes (width 8)
    float4* leaf_rec;
    // textures (all images' texels in one buffer) and the sky image
    uint8_t* texels;
    DevImage* tex;
    DevImage sky;
    // misc
    unsigned long long* ray_counter;
    int* err;
};

namespace {

template <typename T>
cpt_status dalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) return CPT_OK;
    CPT_CUDA(cudaMalloc((void**)p, count * sizeof(T)));
    return CPT_OK;
}

template <typename T>
void dfree(T*& p)
{
    if (p) cudaFree((void*)p);
    p = nullptr;
}

void free_scene(cpt_scene* s)
{
    dfree(s->tri_f32); dfree(s->tri_f64); dfree(s->tri_n); dfree(s->tri_mat); dfree(s->spheres);
    dfree(s->sphere_mat); dfree(s->lights); dfree(s->mats); dfree(s->extra_c); dfree(s->extra_box);
    dfree(s->keys); dfree(s->order); dfree(s->child); dfree(s->range); dfree(s->node_box); dfree(s->leaf_box);
    dfree(s->scratch); dfree(s->nodes); dfree(s->wide); dfree(s->leaf_rec); dfree(s->ray_counter); dfree(s->err);
    dfree(s->tri_uv); dfree(s->texels); dfree(s->tex);
}

// ---- reference double maths for the host-side derived quantities
struct D3 { double x, y, z; };
inline D3 d3(const double* p) { return D3{p[0], p[1], p[2]}; }
inline D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(D3 v, double t) { return D3{v.x * t, v.y * t, v.z * t}; }
inline D3 operator/(D3 v, double t) { return D3{v.x / t, v.y / t, v.z / t}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline D3 unit(D3 v) { return v / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
inline double mmin(double a, double b) { return a < b ? a : b; }
inline double mmax(double a, double b) { return a > b ? a : b; }
inline float3 tof(D3 v) { return make_float3((float)v.x, (float)v.y, (float)v.z); }
inline float rd(double x) { float f = (float)x; return (double)f > x ? std::nextafter(f, -INFINITY) : f; }
inline float ru(double x) { float f = (float)x; return (double)f < x ? std::nextafter(f, INFINITY) : f; }

// Camera ctor (Camera.cu:5-40) in double: eye, centre of pixel (0, 0) and the per-pixel steps.
struct CameraFrame {
    D3 from, pixel_center, dh, dv;
    int width, height;
};

CameraFrame camera_frame(const cpt_camera& c)
{
    CameraFrame f;
    int width = c.width;
    double hh = width / c.aspect_ratio;
    int height = hh < 1 ? 1 : (int)hh;
    D3 from = d3(c.look_from), at = d3(c.look_at), up = D3{0, 1, 0};
    double focal = std::sqrt(dot(from - at, from - at));
    double theta = c.vfov_deg * 3.14159265358979323846 / 180.0;
    double h = std::tan(theta / 2);
    double vh = 2.0 * h * focal;
    double vw = (double)width / height * vh;
    D3 w = unit(from - at);
    D3 u = unit(cross(up, w));
    D3 v = cross(w, u);
    D3 hor = u * vw, ver = v * vh;
    D3 dh = hor / width, dv = ver / height;
    D3 ul = from - hor / 2 - ver / 2 - w * focal;
    f.from = from;
    f.pixel_center = ul + dh / 2 + dv / 2;
    f.dh = dh;
    f.dv = dv;
    f.width = width;
    f.height = height;
    return f;
}

// The frame rounded to FP32 for the kernels.
DevCamera make_camera(const cpt_camera& c)
{
    const CameraFrame f = camera_frame(c);
    DevCamera k;
    k.look_from = tof(f.from);
    k.pixel_center = tof(f.pixel_center);
    k.delta_h = tof(f.dh);
    k.delta_v = tof(f.dv);
    k.background = tof(d3(c.background));
    k.width = f.width;
    k.height = f.height;
    return k;
}

// Light frame and padded box (Light ctor Hittable.cuh:359-365, Hittable(Light) :424-454).
void light_derived(const cpt_light& L, DevLight& dl, double box[6])
{
    D3 c = d3(L.center);
    D3 n = unit(d3(L.normal));
    D3 eu = std::fabs(n.x) > 0.9 ? unit(cross(D3{0, 1, 0}, n)) : unit(cross(D3{1, 0, 0}, n));
    D3 ev = unit(cross(n, eu));
    D3 N = unit(n);
    D3 T = std::fabs(N.x) > 0.9 ? unit(cross(D3{0, 1, 0}, N)) : unit(cross(D3{1, 0, 0}, N));
    D3 B = unit(cross(N, T));
    D3 k[4] = {c + T * (L.width / 2) + B * (L.height / 2), c + T * (L.width / 2) + B * (-L.height / 2),
               c + T * (-L.width / 2) + B * (L.height / 2), c + T * (-L.width / 2) + B * (-L.height / 2)};
    D3 mn = k[0], mx = k[0];
    for (int i = 1; i < 4; ++i) {
        mn = D3{mmin(mn.x, k[i].x), mmin(mn.y, k[i].y), mmin(mn.z, k[i].z)};
        mx = D3{mmax(mx.x, k[i].x), mmax(mx.y, k[i].y), mmax(mx.z, k[i].z)};
    }
    box[0] = mn.x - 0.0001; box[1] = mn.y - 0.0001; box[2] = mn.z - 0.0001;
    box[3] = mx.x + 0.0001; box[4] = mx.y + 0.0001; box[5] = mx.z + 0.0001;
    std::memset(&dl, 0, sizeof dl);
    dl.center = tof(c);
    dl.normal = tof(n);
    dl.eu = tof(eu);
    dl.ev = tof(ev);
    dl.w = (float)L.width;
    dl.h = (float)L.height;
    dl.visible = L.visible ? 1 : 0;
    dl.color = tof(d3(L.color));
}

cpt_status validate(const cpt_scene_desc* d)
{
    if (!d) return fail(CPT_ERR_INVALID_ARGUMENT, "scene description is NULL");
    if (d->num_lights && !d->lights) return fail(CPT_ERR_INVALID_ARGUMENT, "lights pointer is NULL");
    if (d->num_spheres && !d->spheres) return fail(CPT_ERR_INVALID_ARGUMENT, "spheres pointer is NULL");
    if (d->num_triangles) {
        if (!d->tri_vertices == !d->tri_vertices_f64)
            return fail(CPT_ERR_INVALID_ARGUMENT, "exactly one of tri_vertices / tri_vertices_f64 must be set");
        if (!d->tri_material) return fail(CPT_ERR_INVALID_ARGUMENT, "tri_material is NULL");
    }
    if (d->num_materials == 0 || !d->materials) return fail(CPT_ERR_INVALID_ARGUMENT, "no materials");
    if (d->num_textures && !d->textures) return fail(CPT_ERR_INVALID_ARGUMENT, "textures pointer is NULL");
    auto bad_image = [](const cpt_image& im) {
        return im.width <= 0 || im.height <= 0 || !im.rgb || (uint64_t)im.width * (uint64_t)im.height > (1ull << 30);
    };
    for (uint32_t i = 0; i < d->num_textures; ++i)
        if (bad_image(d->textures[i])) return fail(CPT_ERR_INVALID_ARGUMENT, "texture image without texels");
    if (d->sky.rgb && bad_image(d->sky)) return fail(CPT_ERR_INVALID_ARGUMENT, "sky image size");
    for (uint32_t i = 0; i < d->num_materials; ++i)
        if (d->materials[i].texture < 0 || (uint32_t)d->materials[i].texture > d->num_textures)
            return fail(CPT_ERR_INVALID_ARGUMENT, "material texture index out of range");
    for (uint32_t i = 0; i < d->num_spheres; ++i)
        if (d->spheres[i].material >= d->num_materials)
            return fail(CPT_ERR_INVALID_ARGUMENT, "sphere material index out of range");
    for (uint32_t i = 0; i < d->num_triangles; ++i)
        if (d->tri_material[i] >= d->num_materials)
            return fail(CPT_ERR_INVALID_ARGUMENT, "triangle material index out of range");
    uint64_t n = (uint64_t)d->num_lights + d->num_spheres + d->num_triangles;
    if (n > 0x7fffffffull) return fail(CPT_ERR_INVALID_ARGUMENT, "too many primitives");
    if (d->camera.width <= 0 || d->camera.aspect_ratio <= 0.0)
        return fail(CPT_ERR_INVALID_ARGUMENT, "camera width and aspect ratio must be positive");
    double hh = d->camera.width / d->camera.aspect_ratio;
    int h = hh < 1 ? 1 : (int)hh;
    if (d->camera.height != h) return fail(CPT_ERR_INVALID_ARGUMENT, "camera height must be (int)(width / aspect_ratio)");
    return CPT_OK;
}

template <typename T>
cpt_status upload(T** dst, const T* src, size_t count)
{
    cpt_status st = dalloc(dst, count);
    if (st != CPT_OK) return st;
    if (count) CPT_CUDA(cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
    return CPT_OK;
}

cpt_status h2d(void* dst, const void* src, size_t bytes)
{
    CPT_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return CPT_OK;
}

cpt_status create_scene(cpt_context* ctx, const cpt_scene_desc* d, cpt_scene** out)
{
    cpt_status st = validate(d);
    if (st != CPT_OK) return st;
    CPT_CUDA(cudaSetDevice(ctx->device));
    cpt_scene* s = new cpt_scene;
    std::memset(s, 0, sizeof *s);
    s->ctx = ctx;
    s->n_lights = d->num_lights;
    s->n_spheres = d->num_spheres;
    s->n_tris = d->num_triangles;
    s->n = s->n_lights + s->n_spheres + s->n_tris;
    s->camera = d->camera;
    s->cam = make_camera(d->camera);
    for (int a = 0; a < 3; ++a) { s->bmin[a] = d->bounds_min[a]; s->bmax[a] = d->bounds_max[a]; }
    s->tri_is_f64 = d->tri_vertices_f64 != nullptr;
    uint32_t ne = s->n_lights + s->n_spheres;
    std::vector<double> extra_c(3 * (size_t)ne);
    std::vector<float4> extra_box(2 * (size_t)ne);
    std::vector<DevLight> lights(s->n_lights);
    for (uint32_t i = 0; i < s->n_lights; ++i) {
        double b[6];
        light_derived(d->lights[i], lights[i], b);
        for (int a = 0; a < 3; ++a) extra_c[3 * i + a] = d->lights[i].center[a];
        extra_box[2 * i] = make_float4(rd(b[0]), rd(b[1]), rd(b[2]), 0.f);
        extra_box[2 * i + 1] = make_float4(ru(b[3]), ru(b[4]), ru(b[5]), 0.f);
    }
    std::vector<float4> sph(s->n_spheres);
    std::vector<uint32_t> sph_mat(s->n_spheres);
    for (uint32_t i = 0; i < s->n_spheres; ++i) {   // Hittable(Sphere): centre, unpadded box (Hittable.cuh:418-422)
        const cpt_sphere& S = d->spheres[i];
        uint32_t e = s->n_lights + i;
        double r = S.radius;
        double lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            extra_c[3 * e + a] = S.center[a];
            double p0 = S.center[a] - r, p1 = S.center[a] + r;
            lo[a] = mmin(p0, p1);
            hi[a] = mmax(p0, p1);
        }
        extra_box[2 * e] = make_float4(rd(lo[0]), rd(lo[1]), rd(lo[2]), 0.f);
        extra_box[2 * e + 1] = make_float4(ru(hi[0]), ru(hi[1]), ru(hi[2]), 0.f);
        sph[i] = make_float4((float)S.center[0], (float)S.center[1], (float)S.center[2], (float)S.radius);
        sph_mat[i] = S.material;
    }
    std::vector<DevMaterial> mats(d->num_materials);
    s->n_mats = d->num_materials;
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const cpt_material& m = d->materials[i];
        DevMaterial& dm = mats[i];
        std::memset(&dm, 0, sizeof dm);
        dm.color = make_float3((float)m.color[0], (float)m.color[1], (float)m.color[2]);
        dm.ax = (float)m.alpha_x;
        dm.ay = (float)m.alpha_y;
        dm.type = m.type;
        dm.eta = (float)m.eta;
        dm.sigma_t = (float)m.sigma_t;
        dm.albedo = (float)m.albedo;
        dm.tex = m.texture - 1;
    }
    size_t T = s->n_tris;
#define CPT_TRY(x)             \
    do {                       \
        st = (x);              \
        if (st != CPT_OK) {    \
            free_scene(s);     \
            delete s;          \
            return st;         \
        }                      \
    } while (0)
    if (s->tri_is_f64)
        CPT_TRY(upload(&s->tri_f64, d->tri_vertices_f64, 9 * T));
    else
        CPT_TRY(upload(&s->tri_f32, d->tri_vertices, 9 * T));
    if (d->tri_normals) CPT_TRY(upload(&s->tri_n, d->tri_normals, 9 * T));
    if (d->tri_uvs && T) CPT_TRY(upload(&s->tri_uv, d->tri_uvs, 6 * T));
    {   // textures then the sky, packed into one texel buffer
        std::vector<size_t> off;
        size_t total = 0;
        for (uint32_t i = 0; i < d->num_textures; ++i) {
            off.push_back(total);
            total += 3 * (size_t)d->textures[i].width * d->textures[i].height;
        }
        const size_t sky_off = total;
        if (d->sky.rgb) total += 3 * (size_t)d->sky.width * d->sky.height;
        if (total) {
            CPT_TRY(dalloc(&s->texels, total));
            for (uint32_t i = 0; i < d->num_textures; ++i)
                CPT_TRY(h2d(s->texels + off[i], d->textures[i].rgb,
                            3 * (size_t)d->textures[i].width * d->textures[i].height));
            if (d->sky.rgb)
                CPT_TRY(h2d(s->texels + sky_off, d->sky.rgb, 3 * (size_t)d->sky.width * d->sky.height));
        }
        std::vector<DevImage> imgs(d->num_textures);
        for (uint32_t i = 0; i < d->num_textures; ++i) imgs[i] = DevImage{s->texels + off[i], d->textures[i].width,
                                                                          d->textures[i].height};
        if (!imgs.empty()) CPT_TRY(upload(&s->tex, imgs.data(), imgs.size()));
        s->sky = d->sky.rgb ? DevImage{s->texels + sky_off, d->sky.width, d->sky.height} : DevImage{nullptr, 0, 0};
    }
    CPT_TRY(upload(&s->tri_mat, d->tri_material, T));
    CPT_TRY(upload(&s->spheres, sph.data(), sph.size()));
    CPT_TRY(upload(&s->sphere_mat, sph_mat.data(), sph_mat.size()));
    CPT_TRY(upload(&s->lights, lights.data(), lights.size()));
    CPT_TRY(upload(&s->mats, mats.data(), mats.size()));
    CPT_TRY(upload(&s->extra_c, extra_c.data(), extra_c.size()));
    CPT_TRY(upload(&s->extra_box, extra_box.data(), extra_box.size()));
    uint32_t n = s->n;
    uint32_t ni = n > 1 ? n - 1 : 0;
    CPT_TRY(dalloc(&s->keys, n));
    CPT_TRY(dalloc(&s->order, n));
    CPT_TRY(dalloc(&s->child, ni));
    CPT_TRY(dalloc(&s->range, ni));
    CPT_TRY(dalloc(&s->node_box, 2 * (size_t)ni));
    CPT_TRY(dalloc(&s->leaf_box, 2 * (size_t)n));
    CPT_TRY(dalloc(&s->leaf_rec, 3 * (size_t)n));
    s->scratch_bytes = lbvh_scratch_bytes(n);
    CPT_TRY(dalloc((char**)&s->scratch, s->scratch_bytes));
    CPT_TRY(dalloc(&s->ray_counter, 1));
    CPT_TRY(dalloc(&s->err, 2));   // [0] device error word, [1] work counter of batched traces
#undef CPT_TRY
    CPT_CUDA(cudaMemset(s->err, 0, 2 * sizeof(int)));
    *out = s;
    return CPT_OK;
}

SceneView view_of(const cpt_scene* s)
{
    SceneView v;
    std::memset(&v, 0, sizeof v);
    v.n_prims = (int)s->n;
    v.n_lights = (int)s->n_lights;
    v.n_spheres = (int)s->n_spheres;
    v.n_tris = (int)s->n_tris;
    v.n_internal = s->n > 1 ? (int)s->n - 1 : 0;
    v.nodes = s->nodes;
    v.node_q = s->node_q ? 1 : 0;
    v.wide = s->width == 8 ? s->wide : nullptr;
    v.leaf_rec = s->leaf_rec;
    v.tri_mat = s->tri_mat;
    v.tri_n = s->tri_n;
    v.spheres = s->spheres;
    v.sphere_mat = s->sphere_mat;
    v.lights = s->lights;
    v.mats = s->mats;
    v.tri_uv = s->tri_uv;
    v.tex = s->tex;
    v.sky = s->sky;
    v.cam = s->cam;
    return v;
}

// Traversal layout for the context's BVH width: the compressed 8-wide BVH (collapse in wide.cu,
// using the LBVH scratch for its task queues) or the BVH2 node array; leaf records in the
// matching order.  Buffers are allocated on first use.
cpt_status make_layout(cpt_scene* s, cudaStream_t stream, uint32_t* num_wide)
{
    uint32_t n = s->n;
    uint32_t ni = n > 1 ? n - 1 : 0;
    int width = s->ctx->bvh_width;
    if (width == 8 && n > 1) {
        if (!s->wide) {
            cpt_status st = dalloc(&s->wide, CPT_WIDE_F4 * (size_t)ni);
            if (st != CPT_OK) return st;
        }
        if (wide_scratch_bytes(n) > s->scratch_bytes) return fail(CPT_ERR_INVALID_ARGUMENT, "wide scratch too small");
        s->width = 8;
        // leaf records in sorted (Morton) order, shared with the binary layout
        cpt_status st = build_trace_layout(n, s->n_lights, s->n_spheres, s->child, s->node_box, s->leaf_box, s->order,
                                           s->tri_f32, s->tri_f64, s->spheres, nullptr, s->leaf_rec, stream);
        if (st != CPT_OK) return st;
        return build_wide(n, s->child, s->node_box, s->leaf_box, s->wide, s->scratch, s->scratch_bytes, stream,
                          num_wide);
    }
    if (!s->nodes && ni) {
        cpt_status st = dalloc(&s->nodes, 4 * (size_t)ni);
        if (st != CPT_OK) return st;
    }
    s->width = 2;
    s->node_q = s->ctx->bvh2_compressed;
    if (num_wide) *num_wide = 0;
    return build_trace_layout(n, s->n_lights, s->n_spheres, s->child, s->node_box, s->leaf_box, s->order, s->tri_f32,
                              s->tri_f64, s->spheres, s->nodes, s->leaf_rec, stream, s->node_q);
}

LbvhBuffers buffers_of(cpt_scene* s)
{
    LbvhBuffers b;
    b.keys = s->keys;
    b.order = s->order;
    b.child = s->child;
    b.range = s->range;
    b.node_box = s->node_box;
    b.leaf_box = s->leaf_box;
    return b;
}

// Reads and clears the device error word (synchronises the stream).
cpt_status check_device_error(cpt_scene* s, cudaStream_t stream)
{
    int e = 0;
    CPT_CUDA(cudaMemcpyAsync(&e, s->err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CPT_CUDA(cudaStreamSynchronize(stream));
    if (e) {
        CPT_CUDA(cudaMemsetAsync(s->err, 0, sizeof(int), stream));
        if (e & CPT_DEVERR_STACK) return fail(CPT_ERR_STACK_OVERFLOW, "traversal stack limit exceeded");
        return fail(CPT_ERR_TIMEOUT, "a device loop reached its iteration limit");
    }
    return CPT_OK;
}

}  // namespace

namespace cpt {
DevCamera camera_of(const cpt_camera& c) { return make_camera(c); }
}  // namespace cpt

// ---------------------------------------------------------------- exported API
CPT_EXPORT int cpt_abi_version(void) { return CPT_ABI_VERSION; }

CPT_EXPORT uint64_t cpt_launch_count(void) { return g_launches.load(); }

CPT_EXPORT const char* cpt_last_error_string(void) { return g_last_error.c_str(); }

CPT_EXPORT cpt_status cpt_context_create(int device, cpt_context** out)
{
    if (!out) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_context_create: out is NULL");
    *out = nullptr;
    int count = 0;
    CPT_CUDA(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_context_create: no such device");
    CPT_CUDA(cudaSetDevice(device));
    cpt_context* c = new cpt_context;
    c->device = device;
    CPT_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device));
    c->render_block_x = 16;
    c->render_block_y = 8;
    std::memset(&c->wf, 0, sizeof c->wf);
    c->wf.slots = 1 << 21;
    c->wf.short_stack = CPT_SHORT_STACK;
    c->wf.block_trace = 128;
    c->wf.block_shade = 128;
    c->wf.use_graph = true;
    c->wf_grids_ready = false;
    c->bvh_width = 2;   // the faster of the two layouts as measured on GB300
    c->iter_limit = CPT_ITER_LIMIT;
    c->bvh2_compressed = false;
    c->wf.max_replays = CPT_MAX_REPLAYS;
    CPT_CUDA(cudaStreamCreateWithFlags(&c->wf.capture_stream, cudaStreamNonBlocking));
    CPT_CUDA(cudaStreamCreateWithFlags(&c->wf.side_stream, cudaStreamNonBlocking));
    CPT_CUDA(cudaEventCreateWithFlags(&c->wf.fork, cudaEventDisableTiming));
    CPT_CUDA(cudaEventCreateWithFlags(&c->wf.join, cudaEventDisableTiming));
    *out = c;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_context_destroy(cpt_context* ctx)
{
    if (ctx && ctx->wf.capture_stream) cudaStreamDestroy(ctx->wf.capture_stream);
    if (ctx && ctx->wf.side_stream) cudaStreamDestroy(ctx->wf.side_stream);
    if (ctx && ctx->wf.fork) cudaEventDestroy(ctx->wf.fork);
    if (ctx && ctx->wf.join) cudaEventDestroy(ctx->wf.join);
    delete ctx;
    return CPT_OK;
}

// Internal tuning knob (the autotuner's setter): wavefront size, block sizes, graph replay.
CPT_EXPORT cpt_status cpt_context_set_wavefront(cpt_context* ctx, int slots, int block_trace, int block_shade,
                                                int use_graph)
{
    auto ok_block = [](int b, int hi) { return b >= 32 && b <= hi && b % 32 == 0; };
    if (!ctx || slots < 1024 || !ok_block(block_trace, 256) || !ok_block(block_shade, 256))
        return fail(CPT_ERR_INVALID_ARGUMENT, "wavefront: slots >= 1024, blocks multiples of 32 in [32, 256]");
    ctx->wf.slots = slots;
    ctx->wf.block_trace = block_trace;
    ctx->wf.block_shade = block_shade;
    ctx->wf.use_graph = use_graph != 0;
    ctx->wf_grids_ready = false;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_context_set_bvh_compression(cpt_context* ctx, int on)
{
    if (!ctx) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_context_set_bvh_compression: null context");
    ctx->bvh2_compressed = on != 0;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_context_set_material_sort(cpt_context* ctx, int on)
{
    if (!ctx) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_context_set_material_sort: null context");
    ctx->wf.material_sort = on != 0;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_context_set_loop_limits(cpt_context* ctx, int32_t max_trips, int32_t max_replays)
{
    if (!ctx || max_trips < 1 || max_trips > CPT_ITER_LIMIT || max_replays < 1 || max_replays > CPT_MAX_REPLAYS)
        return fail(CPT_ERR_INVALID_ARGUMENT, "loop limits: trips in [1, 65536], replays in [1, 1048576]");
    ctx->iter_limit = max_trips;
    ctx->wf.max_replays = max_replays;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_context_set_bvh_width(cpt_context* ctx, int width)
{
    if (!ctx || (width != 2 && width != 8)) return fail(CPT_ERR_INVALID_ARGUMENT, "BVH width must be 2 or 8");
    ctx->bvh_width = width;
    return CPT_OK;
}

// Internal tuning knob (the autotuner's setter): render block shape.
CPT_EXPORT cpt_status cpt_filter_bilateral(cpt_context* ctx, const float* rgb, const float* gbuf, float* out,
                                           int32_t width, int32_t height, const cpt_filter_params* params,
                                           void* stream)
{
    if (!ctx) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_filter_bilateral: null context");
    cpt_filter_params p = {8.0f, 5.0f, 0.1f, 0.2f, 16};   // Window.cu:11-14, Render.cuh:8
    if (params) p = *params;
    if (rgb == out) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_filter_bilateral: out must not alias rgb");
    CPT_CUDA(cudaSetDevice(ctx->device));
    return filter_bilateral(rgb, gbuf, out, width, height, p, (cudaStream_t)stream);
}

CPT_EXPORT cpt_status cpt_filter_temporal(cpt_context* ctx, float* rgb, const float* prev_rgb, const float* gbuf,
                                          const cpt_camera* camera, const cpt_camera* prev_camera, float alpha,
                                          void* stream)
{
    if (!ctx || !camera || !prev_camera) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_filter_temporal: null argument");
    CPT_CUDA(cudaSetDevice(ctx->device));
    return filter_temporal(rgb, prev_rgb, gbuf, *camera, *prev_camera, alpha, (cudaStream_t)stream);
}

CPT_EXPORT cpt_status cpt_context_set_short_stack(cpt_context* ctx, int entries)
{
    if (!ctx || (entries != 8 && entries != 16 && entries != 24 && entries != 32))
        return fail(CPT_ERR_INVALID_ARGUMENT, "short stack: 8, 16, 24 or 32 entries");
    ctx->wf.short_stack = entries;
    ctx->wf_grids_ready = false;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_context_set_render_block(cpt_context* ctx, int bx, int by)
{
    if (!ctx || bx <= 0 || by <= 0 || (bx * by) % 32 || bx * by > 512)   // short stacks: <= 32 KB shared
        return fail(CPT_ERR_INVALID_ARGUMENT, "render block must be a positive multiple of 32 threads, <= 512");
    ctx->render_block_x = bx;
    ctx->render_block_y = by;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_scene_create(cpt_context* ctx, const cpt_scene_desc* desc, cpt_scene** out)
{
    if (!ctx || !out) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_scene_create: null argument");
    *out = nullptr;
    return create_scene(ctx, desc, out);
}

CPT_EXPORT cpt_status cpt_scene_load_ini(cpt_context* ctx, const char* path, cpt_scene** out)
{
    if (!ctx || !out) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_scene_load_ini: null argument");
    *out = nullptr;
    IniScene* ini = nullptr;
    cpt_status st = ini_load(path, &ini);
    if (st != CPT_OK) return st;
    st = create_scene(ctx, ini_desc(ini), out);
    ini_free(ini);
    return st;
}

CPT_EXPORT cpt_status cpt_ini_load(const char* path, cpt_ini_scene** out)
{
    return ini_load(path, (IniScene**)out);
}

CPT_EXPORT cpt_status cpt_ini_describe(const cpt_ini_scene* ini, cpt_scene_desc* out)
{
    if (!ini || !out) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_ini_describe: null argument");
    *out = *ini_desc((const IniScene*)ini);
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_ini_free(cpt_ini_scene* ini)
{
    ini_free((IniScene*)ini);
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_scene_destroy(cpt_scene* s)
{
    if (!s) return CPT_OK;
    free_scene(s);
    delete s;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_scene_info(const cpt_scene* s, uint32_t* nl, uint32_t* ns, uint32_t* nt, cpt_camera* cam)
{
    if (!s) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_scene_info: scene is NULL");
    if (nl) *nl = s->n_lights;
    if (ns) *ns = s->n_spheres;
    if (nt) *nt = s->n_tris;
    if (cam) *cam = s->camera;
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_scene_update_triangles(cpt_scene* s, const float* tri, uint32_t first, uint32_t count,
                                                 void* stream)
{
    if (!s || (!tri && count)) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_scene_update_triangles: null argument");
    if ((uint64_t)first + count > s->n_tris) return fail(CPT_ERR_INVALID_ARGUMENT, "triangle range out of bounds");
    if (s->tri_is_f64) return fail(CPT_ERR_UNSUPPORTED, "scene has FP64 vertices; update with FP32 is not supported");
    if (count)
        CPT_CUDA(cudaMemcpyAsync(s->tri_f32 + 9ull * first, tri, 9ull * count * sizeof(float), cudaMemcpyHostToDevice,
                                 (cudaStream_t)stream));
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_lbvh_build(cpt_scene* s, void* stream_, cpt_bvh_stats* stats)
{
    if (!s) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_lbvh_build: scene is NULL");
    cudaStream_t stream = (cudaStream_t)stream_;
    CPT_CUDA(cudaSetDevice(s->ctx->device));
    LbvhTimings tm = {0, 0, 0, 0};
    cudaEvent_t e0, e1;
    if (stats) {
        CPT_CUDA(cudaEventCreate(&e0));
        CPT_CUDA(cudaEventCreate(&e1));
    }
    uint32_t ne = s->n_lights + s->n_spheres;
    cpt_status st = lbvh_build(ne, s->extra_c, s->extra_box, s->n_tris, s->tri_f32, s->tri_f64, s->bmin, s->bmax,
                               buffers_of(s), s->scratch, s->scratch_bytes, stream, stats ? &tm : nullptr);
    if (st != CPT_OK) return st;
    if (stats) CPT_CUDA(cudaEventRecord(e0, stream));
    uint32_t num_wide = 0;
    st = make_layout(s, stream, &num_wide);
    if (st != CPT_OK) return st;
    s->built = true;
    if (stats) {
        CPT_CUDA(cudaEventRecord(e1, stream));
        CPT_CUDA(cudaEventSynchronize(e1));
        std::memset(stats, 0, sizeof *stats);
        stats->num_prims = s->n;
        stats->num_wide_nodes = num_wide;
        stats->ms_prep = tm.ms_prep;
        stats->ms_sort = tm.ms_sort;
        stats->ms_emit = tm.ms_emit;
        stats->ms_refit = tm.ms_refit;
        CPT_CUDA(cudaEventElapsedTime(&stats->ms_collapse, e0, e1));
        stats->ms_total = tm.ms_prep + tm.ms_sort + tm.ms_emit + tm.ms_refit + stats->ms_collapse;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_lbvh_refit(cpt_scene* s, void* stream_, cpt_bvh_stats* stats)
{
    if (!s) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_lbvh_refit: scene is NULL");
    if (!s->built) return fail(CPT_ERR_NOT_BUILT, "cpt_lbvh_refit: build the LBVH first");
    cudaStream_t stream = (cudaStream_t)stream_;
    cudaEvent_t e0, e1;
    if (stats) {
        CPT_CUDA(cudaEventCreate(&e0));
        CPT_CUDA(cudaEventCreate(&e1));
        CPT_CUDA(cudaEventRecord(e0, stream));
    }
    uint32_t ne = s->n_lights + s->n_spheres;
    cpt_status st = lbvh_leaf_boxes(ne, s->extra_box, s->n_tris, s->tri_f32, s->tri_f64, s->order, s->leaf_box, s->n, stream);
    if (st != CPT_OK) return st;
    st = lbvh_refit(s->n, buffers_of(s), s->scratch, s->scratch_bytes, stream);
    if (st != CPT_OK) return st;
    st = make_layout(s, stream, nullptr);
    if (st != CPT_OK) return st;
    if (stats) {
        CPT_CUDA(cudaEventRecord(e1, stream));
        CPT_CUDA(cudaEventSynchronize(e1));
        std::memset(stats, 0, sizeof *stats);
        stats->num_prims = s->n;
        CPT_CUDA(cudaEventElapsedTime(&stats->ms_refit, e0, e1));
        stats->ms_total = stats->ms_refit;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_lbvh_export(const cpt_scene* s, uint64_t* keys, uint32_t* order, int32_t* child_a,
                                      int32_t* child_b, float* node_boxes, float* leaf_boxes)
{
    if (!s) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_lbvh_export: scene is NULL");
    if (!s->built) return fail(CPT_ERR_NOT_BUILT, "cpt_lbvh_export: build the LBVH first");
    CPT_CUDA(cudaSetDevice(s->ctx->device));
    CPT_CUDA(cudaDeviceSynchronize());
    size_t n = s->n, ni = n > 1 ? n - 1 : 0;
    if (keys) CPT_CUDA(cudaMemcpy(keys, s->keys, n * 8, cudaMemcpyDeviceToHost));
    if (order) CPT_CUDA(cudaMemcpy(order, s->order, n * 4, cudaMemcpyDeviceToHost));
    if ((child_a || child_b) && ni) {
        std::vector<int2> c(ni);
        CPT_CUDA(cudaMemcpy(c.data(), s->child, ni * sizeof(int2), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < ni; ++i) {
            if (child_a) child_a[i] = c[i].x;
            if (child_b) child_b[i] = c[i].y;
        }
    }
    auto boxes = [&](const float4* src, size_t cnt, float* dst) -> cpt_status {
        std::vector<float4> b(2 * cnt);
        if (cnt) CPT_CUDA(cudaMemcpy(b.data(), src, 2 * cnt * sizeof(float4), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < cnt; ++i) {
            float v[6] = {b[2 * i].x, b[2 * i].y, b[2 * i].z, b[2 * i + 1].x, b[2 * i + 1].y, b[2 * i + 1].z};
            std::memcpy(dst + 6 * i, v, sizeof v);
        }
        return CPT_OK;
    };
    if (node_boxes) {
        cpt_status st = boxes(s->node_box, ni, node_boxes);
        if (st != CPT_OK) return st;
    }
    if (leaf_boxes) {
        cpt_status st = boxes(s->leaf_box, n, leaf_boxes);
        if (st != CPT_OK) return st;
    }
    return CPT_OK;
}

namespace {
// mat[i] = remap[mat[i]] for i < n (material indices of a primitive range)
__global__ void k_remap_u32(uint32_t* mat, uint32_t n, const uint32_t* __restrict__ remap)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) mat[i] = remap[mat[i]];
}
}  // namespace

// getObject (Render.cu:485-496): one ray through the centre of pixel (x, y) (row 0 at the bottom,
// Camera::getSampleRay, Camera.cuh:44-48), built in double like the reference's and rounded to
// FP32; the closest primitive in the reference's numbering (a light included: every primitive's
// hit sets a material, so getObject's material test never rejects one), or -1 on a miss.
CPT_EXPORT cpt_status cpt_pick(cpt_scene* s, int32_t x, int32_t y, int32_t* prim)
{
    if (!s || !prim) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_pick: null argument");
    if (!s->built && s->n) return fail(CPT_ERR_NOT_BUILT, "cpt_pick: build the LBVH first");
    *prim = -1;
    if (x < 0 || y < 0 || x >= s->cam.width || y >= s->cam.height) return CPT_OK;
    CPT_CUDA(cudaSetDevice(s->ctx->device));
    const CameraFrame f = camera_frame(s->camera);
    const D3 px = f.pixel_center + f.dh * (double)x + f.dv * (double)y;
    const D3 dir = px - f.from;
    cpt_ray r;
    std::memset(&r, 0, sizeof r);
    r.origin[0] = (float)f.from.x;
    r.origin[1] = (float)f.from.y;
    r.origin[2] = (float)f.from.z;
    r.direction[0] = (float)dir.x;
    r.direction[1] = (float)dir.y;
    r.direction[2] = (float)dir.z;
    r.tmin = 0.001f;
    r.tmax = CPT_INF_F;
    cpt_hit h;
    cpt_status st = cpt_trace_closest(s, &r, 1, &h, 0, nullptr);
    if (st != CPT_OK) return st;
    *prim = h.prim;
    return CPT_OK;
}

// changeMaterial (Render.cu:498-522): every primitive in [first, end) keeps its colour and takes
// roughness (alpha_x, alpha_y) and the Opaque type, or SpecularDielectric when glass != 0; lights
// are left alone.  The reference edits each object's own material copy; here primitives share
// material records, so each distinct material of the range gets an edited copy appended and the
// range's indices are remapped to the copies (primitives outside the range keep the originals).
CPT_EXPORT cpt_status cpt_scene_set_material(cpt_scene* s, uint32_t first, uint32_t end, double alpha_x,
                                             double alpha_y, int32_t glass)
{
    if (!s) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_scene_set_material: null scene");
    first = std::max(first, s->n_lights);
    end = std::min(end, s->n);
    if (first >= end) return CPT_OK;
    CPT_CUDA(cudaSetDevice(s->ctx->device));
    const uint32_t sph0 = s->n_lights, tri0 = s->n_lights + s->n_spheres;
    struct Part {
        uint32_t* mat;
        uint32_t count;
    } parts[2] = {{nullptr, 0}, {nullptr, 0}};
    if (first < tri0) parts[0] = {s->sphere_mat + (first - sph0), std::min(end, tri0) - first};
    if (end > tri0) {
        const uint32_t a = std::max(first, tri0);
        parts[1] = {s->tri_mat + (a - tri0), end - a};
    }
    // distinct materials of the range
    const uint32_t n_old = s->n_mats;
    std::vector<uint32_t> remap(n_old);
    for (uint32_t i = 0; i < n_old; ++i) remap[i] = i;
    std::vector<char> used(n_old, 0);
    for (const Part& pt : parts) {
        if (!pt.count) continue;
        std::vector<uint32_t> idx(pt.count);
        CPT_CUDA(cudaMemcpy(idx.data(), pt.mat, pt.count * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint32_t m : idx)
            if (m < n_old) used[m] = 1;
    }
    std::vector<DevMaterial> mats(n_old);
    CPT_CUDA(cudaMemcpy(mats.data(), s->mats, n_old * sizeof(DevMaterial), cudaMemcpyDeviceToHost));
    for (uint32_t m = 0; m < n_old; ++m) {
        if (!used[m]) continue;
        DevMaterial e = mats[m];
        e.ax = (float)alpha_x;
        e.ay = (float)alpha_y;
        e.type = glass ? CPT_M_SPECULAR_DIELECTRIC : CPT_M_OPAQUE;
        remap[m] = (uint32_t)mats.size();
        mats.push_back(e);
    }
    DevMaterial* grown = nullptr;
    uint32_t* d_remap = nullptr;
    CPT_CUDA(cudaMalloc((void**)&grown, mats.size() * sizeof(DevMaterial)));
    cudaError_t e = cudaMalloc((void**)&d_remap, n_old * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(grown, mats.data(), mats.size() * sizeof(DevMaterial), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_remap, remap.data(), n_old * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        for (const Part& pt : parts) {
            if (!pt.count) continue;
            k_remap_u32<<<(pt.count + 255) / 256, 256>>>(pt.mat, pt.count, d_remap);
            add_launches(1);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(d_remap);
    if (e != cudaSuccess) {
        cudaFree(grown);
        return cuda_fail(e, "cpt_scene_set_material");
    }
    CPT_CUDA(cudaFree(s->mats));
    s->mats = grown;
    s->n_mats = (uint32_t)mats.size();
    return CPT_OK;
}

CPT_EXPORT cpt_status cpt_trace_closest(cpt_scene* s, const cpt_ray* rays, uint64_t n, cpt_hit* hits, int on_device,
                                        void* stream_)
{
    if (!s || (n && (!rays || !hits))) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_trace_closest: null argument");
    if (!s->built && s->n) return fail(CPT_ERR_NOT_BUILT, "cpt_trace_closest: build the LBVH first");
    if (n == 0) return CPT_OK;
    cudaStream_t stream = (cudaStream_t)stream_;
    CPT_CUDA(cudaSetDevice(s->ctx->device));
    SceneView v = view_of(s);
    if (on_device) {
        cpt_status st = launch_trace(v, rays, n, hits, s->err, stream);
        if (st != CPT_OK) return st;
        return CPT_OK;
    }
    cpt_ray* dr = nullptr;
    cpt_hit* dh = nullptr;
    CPT_CUDA(cudaMallocAsync((void**)&dr, n * sizeof(cpt_ray), stream));
    CPT_CUDA(cudaMallocAsync((void**)&dh, n * sizeof(cpt_hit), stream));
    CPT_CUDA(cudaMemcpyAsync(dr, rays, n * sizeof(cpt_ray), cudaMemcpyHostToDevice, stream));
    cpt_status st = launch_trace(v, dr, n, dh, s->err, stream);
    if (st == CPT_OK) CPT_CUDA(cudaMemcpyAsync(hits, dh, n * sizeof(cpt_hit), cudaMemcpyDeviceToHost, stream));
    cudaFreeAsync(dr, stream);
    cudaFreeAsync(dh, stream);
    if (st != CPT_OK) return st;
    return check_device_error(s, stream);
}

CPT_EXPORT cpt_status cpt_render(cpt_scene* s, const cpt_render_params* p, const cpt_render_output* out, void* stream_,
                                 cpt_render_stats* stats)
{
    if (!s || !p || !out || !out->rgb) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render: null argument");
    if (!s->built && s->n) return fail(CPT_ERR_NOT_BUILT, "cpt_render: build the LBVH first");
    if (p->spp <= 0) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render: spp must be positive");
    if (p->estimator != CPT_ESTIMATOR_REFERENCE && p->estimator != CPT_ESTIMATOR_CONFIG)
        return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render: unknown estimator");
    if (p->integrator != CPT_INTEGRATOR_MEGAKERNEL && p->integrator != CPT_INTEGRATOR_WAVEFRONT)
        return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render: unknown integrator");
    if (p->integrator == CPT_INTEGRATOR_WAVEFRONT && p->estimator != CPT_ESTIMATOR_CONFIG)
        return fail(CPT_ERR_UNSUPPORTED, "cpt_render: the wavefront integrator runs the config estimator");
    if (p->estimator == CPT_ESTIMATOR_CONFIG && !(p->rr_prob > 0.f && p->rr_prob <= 1.f))
        return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render: rr_prob must be in (0, 1]");
    int W = s->cam.width, H = s->cam.height;
    int r0 = p->row_begin, r1 = p->row_end;
    if (r0 == 0 && r1 == 0) r1 = H;
    if (r0 < 0 || r1 > H || r0 > r1) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render: bad row range");
    cudaStream_t stream = (cudaStream_t)stream_;
    CPT_CUDA(cudaSetDevice(s->ctx->device));
    size_t np = (size_t)W * H;
    float* rgb = out->rgb;
    uint8_t* rgba8 = out->rgba8;
    float* gbuf = out->gbuffer;
    bool host = !out->on_device;
    if (host) {
        CPT_CUDA(cudaMallocAsync((void**)&rgb, np * 12, stream));
        if (p->flags & CPT_RENDER_ACCUMULATE)
            CPT_CUDA(cudaMemcpyAsync(rgb, out->rgb, np * 12, cudaMemcpyHostToDevice, stream));
        if (out->rgba8) CPT_CUDA(cudaMallocAsync((void**)&rgba8, np * 4, stream));
        if (out->gbuffer) CPT_CUDA(cudaMallocAsync((void**)&gbuf, np * 32, stream));
    }
    RenderArgs a;
    a.spp = p->spp;
    a.estimator = p->estimator;
    a.max_depth = p->max_depth;
    a.rr_depth = p->rr_depth;
    a.rr_prob = p->rr_prob;
    a.seed = p->seed;
    a.row_begin = r0;
    a.row_end = r1;
    a.flags = p->flags;
    a.rgb = rgb;
    a.rgba8 = rgba8;
    a.gbuf = gbuf;
    a.ray_counter = s->ray_counter;
    a.err = s->err;
    a.iter_limit = s->ctx->iter_limit;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (stats) {
        CPT_CUDA(cudaEventCreate(&e0));
        CPT_CUDA(cudaEventCreate(&e1));
    }
    CPT_CUDA(cudaMemsetAsync(s->ray_counter, 0, sizeof(unsigned long long), stream));
    if (stats) CPT_CUDA(cudaEventRecord(e0, stream));
    cpt_status st = CPT_OK;
    if (p->integrator == CPT_INTEGRATOR_WAVEFRONT) {
        cpt_context* c = s->ctx;
        if (!c->wf_grids_ready) {
            st = wavefront_grids(c->sm_count, c->wf.block_trace, c->wf.block_shade, c->wf.short_stack, &c->wf.grid_trace, &c->wf.grid_trace_wide,
                                 &c->wf.grid_shade);
            c->wf_grids_ready = st == CPT_OK;
        }
        if (st == CPT_OK) st = launch_render_wavefront(view_of(s), a, stream, c->wf);
    } else {
        st = launch_render_megakernel(view_of(s), a, stream, s->ctx->render_block_x, s->ctx->render_block_y);
    }
    if (stats) CPT_CUDA(cudaEventRecord(e1, stream));
    if (st == CPT_OK && host) {
        size_t off = (size_t)r0 * W, cnt = (size_t)(r1 - r0) * W;
        CPT_CUDA(cudaMemcpyAsync(out->rgb + 3 * off, rgb + 3 * off, cnt * 12, cudaMemcpyDeviceToHost, stream));
        if (out->rgba8) CPT_CUDA(cudaMemcpyAsync(out->rgba8 + 4 * off, rgba8 + 4 * off, cnt * 4, cudaMemcpyDeviceToHost, stream));
        if (out->gbuffer) CPT_CUDA(cudaMemcpyAsync(out->gbuffer + 8 * off, gbuf + 8 * off, cnt * 32, cudaMemcpyDeviceToHost, stream));
    }
    if (host) {
        cudaFreeAsync(rgb, stream);
        if (out->rgba8) cudaFreeAsync(rgba8, stream);
        if (out->gbuffer) cudaFreeAsync(gbuf, stream);
    }
    if (st != CPT_OK) return st;
    if (stats) {
        unsigned long long rays = 0;
        CPT_CUDA(cudaMemcpyAsync(&rays, s->ray_counter, sizeof rays, cudaMemcpyDeviceToHost, stream));
        CPT_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        CPT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        CPT_CUDA(cudaStreamSynchronize(stream));
        stats->rays = rays;
        stats->paths = (uint64_t)(r1 - r0) * W * p->spp;
        stats->ms = ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    if (host || stats) return check_device_error(s, stream);
    return CPT_OK;
}

// Several renders in one wavefront (see cpt.h).
CPT_EXPORT cpt_status cpt_render_batch(cpt_context* ctx, const cpt_render_job* jobs, uint32_t count, void* stream_,
                                       cpt_render_stats* stats)
{
    if (!ctx || (count && !jobs)) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render_batch: null argument");
    if (count == 0) return CPT_OK;
    if (count > 4096) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render_batch: at most 4096 jobs");
    std::vector<int> r0(count), r1(count);
    cpt_scene* s0 = jobs[0].scene;
    for (uint32_t i = 0; i < count; ++i) {
        const cpt_render_job& j = jobs[i];
        cpt_scene* s = j.scene;
        if (!s || !j.output.rgb) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render_batch: job without scene or rgb");
        if (s->ctx != ctx) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render_batch: scene of another context");
        if (!s->built && s->n) return fail(CPT_ERR_NOT_BUILT, "cpt_render_batch: build the LBVH first");
        const cpt_render_params* p = &j.params;
        if (p->spp <= 0) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render_batch: spp must be positive");
        if (p->estimator != CPT_ESTIMATOR_CONFIG)
            return fail(CPT_ERR_UNSUPPORTED, "cpt_render_batch: the wavefront integrator runs the config estimator");
        if (!(p->rr_prob > 0.f && p->rr_prob <= 1.f))
            return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render_batch: rr_prob must be in (0, 1]");
        if (s->width != s0->width)
            return fail(CPT_ERR_UNSUPPORTED, "cpt_render_batch: all scenes must use the same BVH width");
        int H = s->cam.height;
        r0[i] = p->row_begin;
        r1[i] = p->row_end;
        if (r0[i] == 0 && r1[i] == 0) r1[i] = H;
        if (r0[i] < 0 || r1[i] > H || r0[i] > r1[i]) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_render_batch: bad row range");
    }
    cudaStream_t stream = (cudaStream_t)stream_;
    CPT_CUDA(cudaSetDevice(ctx->device));
    std::vector<SceneView> views(count);
    std::vector<RenderArgs> args(count);
    std::vector<void*> temps;
    auto release = [&]() {
        for (void* t : temps) cudaFreeAsync(t, stream);
    };
    cpt_status st = CPT_OK;
    uint64_t paths = 0;
    for (uint32_t i = 0; i < count && st == CPT_OK; ++i) {
        const cpt_render_job& j = jobs[i];
        cpt_scene* s = j.scene;
        const size_t np = (size_t)s->cam.width * s->cam.height;
        RenderArgs& a = args[i];
        a.spp = j.params.spp;
        a.estimator = j.params.estimator;
        a.max_depth = j.params.max_depth;
        a.rr_depth = j.params.rr_depth;
        a.rr_prob = j.params.rr_prob;
        a.seed = j.params.seed;
        a.row_begin = r0[i];
        a.row_end = r1[i];
        a.flags = j.params.flags;
        a.rgb = j.output.rgb;
        a.rgba8 = j.output.rgba8;
        a.gbuf = j.output.gbuffer;
        a.ray_counter = s0->ray_counter;
        a.err = s0->err;
        a.iter_limit = ctx->iter_limit;
        if (!j.output.on_device) {   // device copies of host outputs for the duration of the call
            auto tmp = [&](auto** dst, size_t bytes, const void* init) {
                void* d = nullptr;
                cudaError_t e = cudaMallocAsync(&d, bytes, stream);
                if (e == cudaSuccess && init) e = cudaMemcpyAsync(d, init, bytes, cudaMemcpyHostToDevice, stream);
                if (e != cudaSuccess) {
                    if (d) cudaFreeAsync(d, stream);
                    st = cuda_fail(e, "cpt_render_batch: device output");
                    return;
                }
                temps.push_back(d);
                *dst = static_cast<std::remove_pointer_t<decltype(dst)>>(d);
            };
            tmp(&a.rgb, np * 12, (j.params.flags & CPT_RENDER_ACCUMULATE) ? j.output.rgb : nullptr);
            if (st == CPT_OK && j.output.rgba8) tmp(&a.rgba8, np * 4, nullptr);
            if (st == CPT_OK && j.output.gbuffer) tmp(&a.gbuf, np * 32, nullptr);
        }
        views[i] = view_of(s);
        paths += (uint64_t)(r1[i] - r0[i]) * s->cam.width * j.params.spp;
    }
    if (st != CPT_OK) {
        release();
        return st;
    }
    if (!ctx->wf_grids_ready) {
        st = wavefront_grids(ctx->sm_count, ctx->wf.block_trace, ctx->wf.block_shade, ctx->wf.short_stack,
                             &ctx->wf.grid_trace, &ctx->wf.grid_trace_wide, &ctx->wf.grid_shade);
        ctx->wf_grids_ready = st == CPT_OK;
        if (st != CPT_OK) {
            release();
            return st;
        }
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (stats) {
        CPT_CUDA(cudaEventCreate(&e0));
        CPT_CUDA(cudaEventCreate(&e1));
    }
    CPT_CUDA(cudaMemsetAsync(s0->ray_counter, 0, sizeof(unsigned long long), stream));
    if (stats) CPT_CUDA(cudaEventRecord(e0, stream));
    st = launch_render_wavefront_batch(views.data(), args.data(), (int)count, stream, ctx->wf);
    if (stats) CPT_CUDA(cudaEventRecord(e1, stream));
    for (uint32_t i = 0; i < count && st == CPT_OK; ++i) {
        const cpt_render_job& j = jobs[i];
        if (j.output.on_device) continue;
        const int W = j.scene->cam.width;
        const size_t off = (size_t)r0[i] * W, cnt = (size_t)(r1[i] - r0[i]) * W;
        cudaError_t e = cudaMemcpyAsync(j.output.rgb + 3 * off, args[i].rgb + 3 * off, cnt * 12, cudaMemcpyDeviceToHost,
                                        stream);
        if (e == cudaSuccess && j.output.rgba8)
            e = cudaMemcpyAsync(j.output.rgba8 + 4 * off, args[i].rgba8 + 4 * off, cnt * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess && j.output.gbuffer)
            e = cudaMemcpyAsync(j.output.gbuffer + 8 * off, args[i].gbuf + 8 * off, cnt * 32, cudaMemcpyDeviceToHost,
                                stream);
        if (e != cudaSuccess) st = cuda_fail(e, "cpt_render_batch: read-back");
    }
    release();
    if (st != CPT_OK) return st;
    if (stats) {
        unsigned long long rays = 0;
        CPT_CUDA(cudaMemcpyAsync(&rays, s0->ray_counter, sizeof rays, cudaMemcpyDeviceToHost, stream));
        CPT_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        CPT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        CPT_CUDA(cudaStreamSynchronize(stream));
        stats->rays = rays;
        stats->paths = paths;
        stats->ms = ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return check_device_error(s0, stream);
}

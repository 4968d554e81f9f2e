/*
 * ref_harness.cpp — TEST INFRASTRUCTURE ONLY.
 *
 * Drives the reference's OWN source (BVH.cuh, Hittable.cuh, Material.cuh, HitRecord.cuh,
 * Camera.cuh/.cu, Render.cu, IniParser.cpp), compiled as host C++ by oracle/Makefile
 * from the files where they lie, into oracle/_ref/libcpt_ref.so.  It is used here, where
 * the reference is mounted, to pin the restated oracle (cpt_oracle.cpp) and to generate
 * the golden fixtures under tests/golden/.  Nothing of the reference is copied.
 *
 * What the harness itself restates (because the reference's file also contains
 * <<<>>> launches that only nvcc parses): the object placement of
 * Device::allocate*OnDevice (Device.cuh:29-59) and the orchestration of
 * Device::buildBVH (Device.cuh:169-195).  The sort there is thrust::sort_by_key on unique
 * keys; std::sort of the same keys yields the same permutation.
 */
#include "Render.cuh"
#include "IniParser.h"
#include "cpt.h"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
uint64_t cpt_ref_seed = 0;

// The reference calls these only to load a sky-box image into device memory (Camera.cu:33-39).
// Here "device memory" is host memory: stbi_load hands out the image the harness staged for the
// camera being constructed (3 channels), or fails (NULL) like a missing file; cudaMalloc and
// cudaMemcpy are malloc and memcpy.  They have hidden visibility, so they never shadow the CUDA
// runtime of another library in the process.
static thread_local const cpt_image* g_staged_image = nullptr;
extern "C" unsigned char* stbi_load(char const*, int* w, int* h, int* c, int)
{
    const cpt_image* im = g_staged_image;
    if (!im || !im->rgb) return nullptr;
    size_t bytes = 3 * (size_t)im->width * im->height;
    unsigned char* p = (unsigned char*)std::malloc(bytes);
    std::memcpy(p, im->rgb, bytes);
    *w = im->width;
    *h = im->height;
    *c = 3;
    return p;
}
extern "C" cudaError_t cudaMalloc(void** p, size_t bytes)
{
    if (!p) return cudaErrorInvalidValue;
    *p = std::malloc(bytes ? bytes : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
extern "C" cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, enum cudaMemcpyKind)
{
    std::memcpy(dst, src, bytes);
    return cudaSuccess;
}

#define REF_API extern "C" __attribute__((visibility("default")))

namespace {

struct RefScene {
    Hittable* objs = nullptr;
    int n = 0;
    int nLights = 0;
    std::vector<unsigned> lightsIndex;
    std::vector<Node> leaf, internal;
    std::vector<uint64_t> mortons;
    std::vector<unsigned> objIdx;
    Camera* cam = nullptr;
    int W = 0, H = 0;
    double3 minB, maxB;
    ~RefScene()
    {
        std::free(objs);
        if (cam) { cam->~Camera(); std::free(cam); }
    }
};

inline double3 d3(const double* p) { return make_double3(p[0], p[1], p[2]); }

MaterialType refType(int t)
{
    // IniParser::ParseMaterialType maps unknown names (e.g. a Lambertian) to Opaque (IniParser.cpp:127).
    if (t >= (int)M_LIGHT && t <= (int)M_VOLUME) return (MaterialType)t;
    return M_OPAQUE;
}

// Device::buildBVH (Device.cuh:169-195) with the reference's own morton3D,
// generateHierarchy and constructAABB.
void buildBVH(RefScene& s)
{
    int size = s.n;
    double3 expand = make_double3(1.0, 1.0, 1.0);
    double3 sceneMin = s.minB - expand;
    double3 sceneMax = s.maxB + expand;
    if (sceneMin.x > sceneMax.x) {
        sceneMin = make_double3(-20.0, -20.0, -20.0);
        sceneMax = make_double3(20.0, 20.0, 20.0);
    }
    s.mortons.assign(size, 0);
    s.objIdx.assign(size, 0);
    for (int i = 0; i < size; ++i) {   // generateMortonCodes (Device.cuh:134-142)
        s.mortons[i] = morton3D(s.objs[i].center, sceneMin, sceneMax, i);
        s.objIdx[i] = i;
    }
    std::vector<unsigned> perm(size);
    for (int i = 0; i < size; ++i) perm[i] = i;
    std::sort(perm.begin(), perm.end(), [&](unsigned a, unsigned b) { return s.mortons[a] < s.mortons[b]; });
    std::vector<uint64_t> k2(size);
    std::vector<unsigned> v2(size);
    for (int i = 0; i < size; ++i) { k2[i] = s.mortons[perm[i]]; v2[i] = s.objIdx[perm[i]]; }
    s.mortons.swap(k2);
    s.objIdx.swap(v2);
    s.leaf.assign(size, Node());
    s.internal.assign(size > 1 ? size - 1 : 1, Node());
    for (int idx = 0; idx < size; ++idx)   // generateBVH (Device.cuh:144-150)
        generateHierarchy(s.objs, s.leaf.data(), s.internal.data(), s.mortons.data(), s.objIdx.data(), size, idx);
    if (size > 1) constructAABB(s.internal.data());
}

int encodeChild(const RefScene& s, const Node* c)
{
    if (c >= s.leaf.data() && c < s.leaf.data() + s.leaf.size()) return ~(int)(c - s.leaf.data());
    return (int)(c - s.internal.data());
}

void setupCamera(RefScene& s, const cpt_camera& c, const cpt_image* sky = nullptr)
{
    s.cam = (Camera*)std::malloc(sizeof(Camera));
    // A sky image goes in through the reference's own loading path (Camera.cu:33-39): a non-empty
    // skyBox name makes the constructor call stbi_load, which returns the staged image.
    g_staged_image = sky && sky->rgb ? sky : nullptr;
    new (s.cam) Camera(c.width, c.aspect_ratio, d3(c.background), d3(c.look_from), d3(c.look_at), c.vfov_deg,
                       g_staged_image ? std::string("sky") : std::string());
    g_staged_image = nullptr;
    s.W = c.width;
    s.H = (int)(c.width / c.aspect_ratio);
}

}  // namespace

// Scene from a cpt_scene_desc, objects placed in the reference's order (lights, spheres,
// triangles) exactly as Device::allocate*OnDevice constructs them.
REF_API void* ref_scene_create(const cpt_scene_desc* d)
{
    RefScene* s = new RefScene();
    s->n = (int)(d->num_lights + d->num_spheres + d->num_triangles);
    s->objs = (Hittable*)std::aligned_alloc(64, ((sizeof(Hittable) * (size_t)std::max(1, s->n) + 63) / 64) * 64);
    int k = 0;
    for (uint32_t i = 0; i < d->num_lights; ++i) {
        const cpt_light& L = d->lights[i];
        new (&s->objs[k]) Hittable(Light(d3(L.center), L.width, L.height, d3(L.normal), d3(L.color), L.visible != 0));
        s->lightsIndex.push_back(k++);
    }
    for (uint32_t i = 0; i < d->num_spheres; ++i) {
        const cpt_sphere& S = d->spheres[i];
        const cpt_material& m = d->materials[S.material];
        new (&s->objs[k++]) Hittable(Sphere(d3(S.center), S.radius, d3(m.color), m.alpha_x, m.alpha_y, refType(m.type)));
    }
    for (uint32_t i = 0; i < d->num_triangles; ++i) {
        double3 p[3], nn[3];
        for (int v = 0; v < 3; ++v) {
            if (d->tri_vertices_f64)
                p[v] = d3(d->tri_vertices_f64 + 9 * i + 3 * v);
            else
                p[v] = make_double3(d->tri_vertices[9 * i + 3 * v], d->tri_vertices[9 * i + 3 * v + 1],
                                    d->tri_vertices[9 * i + 3 * v + 2]);
            nn[v] = d->tri_normals ? make_double3(d->tri_normals[9 * i + 3 * v], d->tri_normals[9 * i + 3 * v + 1],
                                                  d->tri_normals[9 * i + 3 * v + 2])
                                   : make_double3(0.0, 0.0, 0.0);
        }
        const cpt_material& m = d->materials[d->tri_material ? d->tri_material[i] : 0];
        double2 uv[3];
        for (int v = 0; v < 3; ++v)
            uv[v] = d->tri_uvs ? make_double2(d->tri_uvs[6 * i + 2 * v], d->tri_uvs[6 * i + 2 * v + 1])
                               : make_double2(0.0, 0.0);
        // allocateMeshesOnDevice passes the mesh's image with its width, height and channel count
        // (Device.cuh:56-79); the texels are host memory here.
        const cpt_image* tx = m.texture > 0 ? &d->textures[m.texture - 1] : nullptr;
        new (&s->objs[k++]) Hittable(Triangle(p[0], p[1], p[2], d3(m.color), m.alpha_x, m.alpha_y, refType(m.type),
                                              uv[0], uv[1], uv[2], nn[0], nn[1], nn[2],
                                              tx ? const_cast<unsigned char*>(tx->rgb) : NULL, tx ? tx->width : 0,
                                              tx ? tx->height : 0, tx ? 3 : 0));
    }
    s->nLights = (int)d->num_lights;
    s->minB = d3(d->bounds_min);
    s->maxB = d3(d->bounds_max);
    setupCamera(*s, d->camera, &d->sky);
    buildBVH(*s);
    return s;
}

// Scene from an INI file through the reference's IniParser, assembled as Scene::init does
// (Scene.cuh:72-99): lights, spheres, floors (two triangles per quad, Device.cuh:42-43).
// [Mesh] sections need OBJ assets and are rejected (returns NULL).
REF_API void* ref_scene_create_ini(const char* path)
{
    IniParser parser;
    parser.Parse(path);
    if (!parser.meshes.empty() || parser.hasCloth) return nullptr;
    std::vector<cpt_light> lights;
    std::vector<cpt_sphere> spheres;
    std::vector<cpt_material> mats;
    std::vector<double> tris;
    std::vector<uint32_t> tmat;
    for (auto& L : parser.lights) {
        cpt_light l = {};
        l.center[0] = L.center.x; l.center[1] = L.center.y; l.center[2] = L.center.z;
        l.normal[0] = L.normal.x; l.normal[1] = L.normal.y; l.normal[2] = L.normal.z;
        l.width = L.width; l.height = L.height;
        l.color[0] = L.color.x; l.color[1] = L.color.y; l.color[2] = L.color.z;
        l.visible = L.visible ? 1 : 0;
        lights.push_back(l);
    }
    auto addMat = [&](double3 c, double ax, double ay, MaterialType t) {
        cpt_material m = {};
        m.color[0] = c.x; m.color[1] = c.y; m.color[2] = c.z;
        m.alpha_x = ax; m.alpha_y = ay; m.type = (int)t; m.eta = 1.51;
        mats.push_back(m);
        return (uint32_t)(mats.size() - 1);
    };
    for (auto& S : parser.spheres) {
        cpt_sphere sp = {};
        sp.center[0] = S.center.x; sp.center[1] = S.center.y; sp.center[2] = S.center.z;
        sp.radius = S.radius;
        sp.material = addMat(S.color, S.alphaX, S.alphaY, S.type);
        spheres.push_back(sp);
    }
    for (auto& F : parser.floors) {
        uint32_t mi = addMat(F.color, F.alphaX, F.alphaY, F.type);
        double3 q[6] = {F.lt, F.lb, F.rt, F.rt, F.lb, F.rb};
        for (int t = 0; t < 6; ++t) { tris.push_back(q[t].x); tris.push_back(q[t].y); tris.push_back(q[t].z); }
        tmat.push_back(mi);
        tmat.push_back(mi);
    }
    if (mats.empty()) addMat(make_double3(1, 1, 1), 0.5, 0.5, M_OPAQUE);
    cpt_scene_desc d = {};
    d.num_lights = (uint32_t)lights.size();
    d.lights = lights.data();
    d.num_spheres = (uint32_t)spheres.size();
    d.spheres = spheres.data();
    d.num_triangles = (uint32_t)tmat.size();
    d.tri_vertices_f64 = tris.data();
    d.tri_material = tmat.data();
    d.num_materials = (uint32_t)mats.size();
    d.materials = mats.data();
    for (int a = 0; a < 3; ++a) { d.bounds_min[a] = INF; d.bounds_max[a] = -INF; }   // Scene.cuh:61-62
    d.camera.width = (int)parser.camera.width;
    d.camera.aspect_ratio = parser.camera.aspectRatio;
    d.camera.height = (int)(d.camera.width / d.camera.aspect_ratio);
    d.camera.look_from[0] = parser.camera.lookFrom.x; d.camera.look_from[1] = parser.camera.lookFrom.y;
    d.camera.look_from[2] = parser.camera.lookFrom.z;
    d.camera.look_at[0] = parser.camera.lookAt.x; d.camera.look_at[1] = parser.camera.lookAt.y;
    d.camera.look_at[2] = parser.camera.lookAt.z;
    d.camera.vfov_deg = parser.camera.vFov;
    d.camera.background[0] = parser.camera.background.x; d.camera.background[1] = parser.camera.background.y;
    d.camera.background[2] = parser.camera.background.z;
    return ref_scene_create(&d);
}

REF_API void ref_scene_destroy(void* p) { delete (RefScene*)p; }

REF_API int ref_scene_size(void* p, int* w, int* h)
{
    RefScene* s = (RefScene*)p;
    if (w) *w = s->W;
    if (h) *h = s->H;
    return s->n;
}

REF_API void ref_lbvh_export(void* p, uint64_t* keys, uint32_t* order, int32_t* ca, int32_t* cb, double* nodeBoxes,
                             double* leafBoxes, double* centroids)
{
    RefScene* s = (RefScene*)p;
    for (int i = 0; i < s->n; ++i) {
        if (keys) keys[i] = s->mortons[i];
        if (order) order[i] = s->objIdx[i];
        const AABB& b = s->leaf[i].aabb;
        if (leafBoxes) {
            double v[6] = {b.min.x, b.min.y, b.min.z, b.max.x, b.max.y, b.max.z};
            std::memcpy(leafBoxes + 6 * i, v, sizeof v);
        }
        if (centroids) {
            centroids[3 * i] = s->objs[i].center.x;
            centroids[3 * i + 1] = s->objs[i].center.y;
            centroids[3 * i + 2] = s->objs[i].center.z;
        }
    }
    for (int i = 0; i + 1 < s->n; ++i) {
        if (ca) ca[i] = encodeChild(*s, s->internal[i].childA);
        if (cb) cb[i] = encodeChild(*s, s->internal[i].childB);
        const AABB& b = s->internal[i].aabb;
        if (nodeBoxes) {
            double v[6] = {b.min.x, b.min.y, b.min.z, b.max.x, b.max.y, b.max.z};
            std::memcpy(nodeBoxes + 6 * i, v, sizeof v);
        }
    }
}

// Closest hit of each ray (8 doubles: origin, tmin, direction, tmax) with traverseIterative.
REF_API void ref_trace(void* p, const double* rays, int64_t n, int32_t* outId, double* outT)
{
    RefScene* s = (RefScene*)p;
    for (int64_t i = 0; i < n; ++i) {
        const double* r = rays + 8 * i;
        Ray ray(make_double3(r[0], r[1], r[2]), make_double3(r[4], r[5], r[6]), 0.0);
        HitRecord rec;
        int id = traverseIterative(s->internal.data(), s->objs, ray, rec, r[7], r[3]);
        outId[i] = id;
        if (outT) outT[i] = id >= 0 ? rec.t : -1.0;
    }
}

// The reference's render kernel in STATIC mode, one call per pixel (Render.cu:16).
// rgb: W*H*3 doubles (pic), rgba8: W*H*4 (devPtr), rows [r0, r1).
REF_API void ref_render(void* p, int spp, uint64_t seed, int r0, int r1, double* rgb, uint8_t* rgba8, int threads)
{
    RefScene* s = (RefScene*)p;
    cpt_ref_seed = seed;
    if (r0 == 0 && r1 == 0) r1 = s->H;
    size_t np = (size_t)s->W * s->H;
    std::vector<double3> pic(np), prev(np), before(np), gpos(np);
    std::vector<double4> gbuf(np);
    std::vector<uchar4> dev(np);
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next(r0);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            blockDim = dim3(1, 1, 1);
            threadIdx = make_uint3(0, 0, 0);
            for (;;) {
                int j = next.fetch_add(1);
                if (j >= r1) break;
                for (int i = 0; i < s->W; ++i) {
                    blockIdx = make_uint3(i, j, 0);
                    render(dev.data(), pic.data(), prev.data(), before.data(), gbuf.data(), gpos.data(), s->cam,
                           s->lightsIndex.data(), s->objs, s->internal.data(), s->nLights, s->W, s->H, spp, 0.0,
                           RenderType::STATIC);
                }
            }
        });
    for (auto& th : pool) th.join();
    for (int j = r0; j < r1; ++j)
        for (int i = 0; i < s->W; ++i) {
            size_t o = (size_t)j * s->W + i;
            rgb[3 * o] = pic[o].x; rgb[3 * o + 1] = pic[o].y; rgb[3 * o + 2] = pic[o].z;
            if (rgba8) { rgba8[4 * o] = dev[o].x; rgba8[4 * o + 1] = dev[o].y; rgba8[4 * o + 2] = dev[o].z; rgba8[4 * o + 3] = dev[o].w; }
        }
}

// The reference's getObject kernel (Render.cu:485-496) as a host call: the object under pixel
// (x, y), or -1.
REF_API int ref_pick(void* p, int x, int y)
{
    RefScene* s = (RefScene*)p;
    int sel = -1;
    getObject(s->objs, s->cam, s->internal.data(), &sel, x, y);
    return sel;
}

// The reference's changeMaterial kernel (Render.cu:498-522) over [first, end), one call per
// thread of the launch Window.cu:333-338 makes (512 threads per block).
REF_API void ref_change_material(void* p, int first, int end, double alphaX, double alphaY, int glass)
{
    RefScene* s = (RefScene*)p;
    const int threads = 512;
    const int blocks = (end - first + threads - 1) / threads;
    blockDim = dim3(threads, 1, 1);
    for (int b = 0; b < blocks; ++b)
        for (int t = 0; t < threads; ++t) {
            blockIdx = make_uint3(b, 0, 0);
            threadIdx = make_uint3(t, 0, 0);
            changeMaterial(s->objs, first, end, alphaX, alphaY, glass != 0);
        }
}

// IniParser::Parse flattened: returns the number of doubles written.
// Layout: camera[bg3, width, aspect, lookFrom3, lookAt3, vFov], nL, L*[center3, w, h, normal3, color3, visible],
// nS, S*[center3, r, color3, ax, ay, type], nF, F*[lt3, rt3, lb3, rb3, color3, ax, ay, type],
// nM, M*[center3, color3, ax, ay, type, rotation, scale], hasCloth.
REF_API int ref_ini_dump(const char* path, double* out, int cap)
{
    IniParser p;
    p.Parse(path);
    std::vector<double> v;
    auto put3 = [&](double3 a) { v.push_back(a.x); v.push_back(a.y); v.push_back(a.z); };
    put3(p.camera.background); v.push_back(p.camera.width); v.push_back(p.camera.aspectRatio);
    put3(p.camera.lookFrom); put3(p.camera.lookAt); v.push_back(p.camera.vFov);
    v.push_back((double)p.lights.size());
    for (auto& L : p.lights) { put3(L.center); v.push_back(L.width); v.push_back(L.height); put3(L.normal); put3(L.color); v.push_back(L.visible ? 1 : 0); }
    v.push_back((double)p.spheres.size());
    for (auto& S : p.spheres) { put3(S.center); v.push_back(S.radius); put3(S.color); v.push_back(S.alphaX); v.push_back(S.alphaY); v.push_back((double)S.type); }
    v.push_back((double)p.floors.size());
    for (auto& F : p.floors) { put3(F.lt); put3(F.rt); put3(F.lb); put3(F.rb); put3(F.color); v.push_back(F.alphaX); v.push_back(F.alphaY); v.push_back((double)F.type); }
    v.push_back((double)p.meshes.size());
    for (auto& M : p.meshes) { put3(M.center); put3(M.color); v.push_back(M.alphaX); v.push_back(M.alphaY); v.push_back((double)M.type); v.push_back(M.rotation); v.push_back(M.scale); }
    v.push_back(p.hasCloth ? 1 : 0);
    int n = (int)v.size();
    if (n <= cap) std::memcpy(out, v.data(), sizeof(double) * n);
    return n;
}

// The reference's real-time filters run as plain loops over their own kernels
// (gaussianSeparate, Render.cu:356-398; addPrevious, Render.cu:400-420).  Images are W*H
// double3; gbuf4 is W*H double4 (normal, depth); gpos W*H double3 (INF on a miss).
REF_API void ref_gaussian_separate(double* pic, double* before, const double* gbuf4, double sg, double sr, double sn,
                                   double sd, int W, int H, int horizontal)
{
    blockDim = dim3(1, 1, 1);
    threadIdx = make_uint3(0, 0, 0);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            blockIdx = make_uint3(x, y, 0);
            gaussianSeparate((double3*)pic, (double3*)before, (double4*)gbuf4, sg, sr, sn, sd, W, H, horizontal != 0);
        }
}

REF_API void ref_add_previous(double* pic, double* prev, double* gpos, const cpt_camera* cur, const double* pre_from,
                              const double* pre_at, int moving)
{
    Camera* cam = (Camera*)std::malloc(sizeof(Camera));
    new (cam) Camera(cur->width, cur->aspect_ratio, d3(cur->background), d3(cur->look_from), d3(cur->look_at),
                     cur->vfov_deg, std::string());
    cam->preLookFrom = make_double3(pre_from[0], pre_from[1], pre_from[2]);
    cam->preLookAt = make_double3(pre_at[0], pre_at[1], pre_at[2]);
    cam->isMoving = moving != 0;
    blockDim = dim3(1, 1, 1);
    threadIdx = make_uint3(0, 0, 0);
    for (int y = 0; y < cam->height; ++y)
        for (int x = 0; x < cam->width; ++x) {
            blockIdx = make_uint3(x, y, 0);
            addPrevious((double3*)pic, (double3*)prev, (double3*)gpos, cam, cam->width, cam->height);
        }
    cam->~Camera();
    std::free(cam);
}

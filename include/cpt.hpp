/* cpt.hpp — header-only C++ wrappers over the C ABI (cpt.h) named after the reference's classes,
 * so its call sites map one to one:
 *
 *   Device::Device / ~Device      -> cpt::Context          (Device.cuh:161-168)
 *   Scene::init(IniParser)        -> cpt::Scene(ctx, path) (Scene.cuh:72)
 *   Device::buildBVH              -> Scene::buildBVH       (Device.cuh:169-195)
 *   Scene::Update                 -> Scene::Update         (Scene.cuh:147-173)
 *   render<<<>>> (STATIC)         -> Scene::render         (Render.cu:16-261)
 *   traverseIterative (batched)   -> Scene::trace          (BVH.cuh:282-332)
 *   getObject / changeMaterial    -> Scene::pick / Scene::changeMaterial (Render.cu:485-522)
 *   Camera (ctor, getSampleRay, getRandomSampleRay)  -> cpt::Camera   (Camera.cu:5-40, Camera.cuh:37-48)
 *   Material(color, alphaX, alphaY, type)            -> cpt::Material (Material.cuh:5-22)
 *   Hittable(Light | Sphere | Triangle)              -> cpt::Hittable (Hittable.cuh:402-503)
 *   Scene::addOneLight / addOneSphere / addFloor / addMeshes
 *                                 -> cpt::SceneBuilder    (Scene.cuh:175-270)
 *   render<<<grid, block>>>(devPtr, pic, ...)        -> cpt::render   (Render.cu:16, main.cu:78-80)
 *
 * Errors: the wrappers throw cpt::Error (status + cpt_last_error_string()) where the reference
 * called exit(99) (Device.cuh:9-19).  Objects own their handles (move-only). */
#ifndef CPT_HPP
#define CPT_HPP

#include <cmath>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cpt.h"

namespace cpt {

class Error : public std::runtime_error {
public:
    Error(cpt_status s, const std::string& where)
        : std::runtime_error(where + ": " + cpt_last_error_string()), status(s) {}
    cpt_status status;
};

inline void check(cpt_status s, const char* where)
{
    if (s != CPT_OK) throw Error(s, where);
}

/* double3 of the reference's host code (rtmath.cuh), as a plain aggregate. */
struct Vec3 {
    double x, y, z;
};

/* The reference's MaterialType (rtmath.cuh:15), plus the Lambertian extension. */
enum MaterialType {
    M_NONE = CPT_M_NONE,
    M_LIGHT = CPT_M_LIGHT,
    M_OPAQUE = CPT_M_OPAQUE,
    M_SPECULAR_DIELECTRIC = CPT_M_SPECULAR_DIELECTRIC,
    M_ROUGH_DIELECTRIC = CPT_M_ROUGH_DIELECTRIC,
    M_VOLUME = CPT_M_VOLUME,
    M_LAMBERTIAN = CPT_M_LAMBERTIAN
};

/* Material (Material.cuh:5-22): colour, anisotropic roughness, type; eta 1.51 as in the
 * reference.  sigma_t / albedo / texture are the config estimator's extensions. */
struct Material {
    Vec3 color{0.0, 0.0, 0.0};
    double alphaX = 0.5, alphaY = 0.5;
    MaterialType type = M_OPAQUE;
    double eta = 1.51;
    double sigmaT = 0.0, albedo = 0.0;
    int32_t texture = 0;   /* 0: none, k: SceneBuilder texture k */

    Material() = default;
    Material(Vec3 c, double ax, double ay, MaterialType t) : color(c), alphaX(ax), alphaY(ay), type(t) {}

    cpt_material to_c() const
    {
        cpt_material m{};
        m.color[0] = color.x; m.color[1] = color.y; m.color[2] = color.z;
        m.alpha_x = alphaX; m.alpha_y = alphaY;
        m.type = type;
        m.texture = texture;
        m.eta = eta; m.sigma_t = sigmaT; m.albedo = albedo;
        return m;
    }
};

/* Camera (Camera.cu:5-40): the constructor's arguments; height follows the reference's rule
 * (int)(width / aspectRatio), at least 1.  getSampleRay / getRandomSampleRay build the same rays
 * as Camera.cuh:37-48 in double (image row 0 at the bottom). */
class Camera {
public:
    int width, height;
    double aspectRatio;
    Vec3 background, lookFrom, lookAt;
    double vFov;

    Camera(int w, double aspect, Vec3 bg, Vec3 from, Vec3 at, double vfov)
        : width(w), height(w / aspect < 1 ? 1 : (int)(w / aspect)), aspectRatio(aspect), background(bg),
          lookFrom(from), lookAt(at), vFov(vfov)
    {
        const double pi = 3.14159265358979323846;
        Vec3 d = sub(from, at);
        double focal = std::sqrt(dot(d, d));
        double vh = 2.0 * std::tan(vfov * pi / 180.0 / 2) * focal;
        double vw = (double)width / height * vh;
        Vec3 wv = unit(d);
        Vec3 u = unit(cross(Vec3{0, 1, 0}, wv));
        Vec3 v = cross(wv, u);
        dh_ = scale(u, vw / width);
        dv_ = scale(v, vh / height);
        Vec3 ul = sub(sub(sub(from, scale(u, vw / 2)), scale(v, vh / 2)), scale(wv, focal));
        pc_ = add(ul, add(scale(dh_, 0.5), scale(dv_, 0.5)));
    }

    cpt_camera to_c() const
    {
        cpt_camera c{};
        c.width = width; c.height = height; c.aspect_ratio = aspectRatio;
        c.look_from[0] = lookFrom.x; c.look_from[1] = lookFrom.y; c.look_from[2] = lookFrom.z;
        c.look_at[0] = lookAt.x; c.look_at[1] = lookAt.y; c.look_at[2] = lookAt.z;
        c.vfov_deg = vFov;
        c.background[0] = background.x; c.background[1] = background.y; c.background[2] = background.z;
        return c;
    }
    /* Ray through the centre of pixel (x, y) (Camera.cuh:44-48), traverseIterative's interval. */
    cpt_ray getSampleRay(int x, int y) const { return getRandomSampleRay(x, y, 0.5, 0.5); }
    /* Ray through (x - 0.5 + randx, y - 0.5 + randy) (Camera.cuh:37-43). */
    cpt_ray getRandomSampleRay(int x, int y, double randx, double randy) const
    {
        Vec3 p = add(pc_, add(scale(dh_, randx - 0.5 + x), scale(dv_, randy - 0.5 + y)));
        Vec3 d = sub(p, lookFrom);
        cpt_ray r{};
        r.origin[0] = (float)lookFrom.x; r.origin[1] = (float)lookFrom.y; r.origin[2] = (float)lookFrom.z;
        r.direction[0] = (float)d.x; r.direction[1] = (float)d.y; r.direction[2] = (float)d.z;
        r.tmin = 0.001f;
        r.tmax = 999999.0f;
        return r;
    }

private:
    Vec3 pc_{}, dh_{}, dv_{};
    static Vec3 add(Vec3 a, Vec3 b) { return Vec3{a.x + b.x, a.y + b.y, a.z + b.z}; }
    static Vec3 sub(Vec3 a, Vec3 b) { return Vec3{a.x - b.x, a.y - b.y, a.z - b.z}; }
    static Vec3 scale(Vec3 a, double t) { return Vec3{a.x * t, a.y * t, a.z * t}; }
    static double dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
    static Vec3 cross(Vec3 a, Vec3 b) { return Vec3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
    static Vec3 unit(Vec3 a) { return scale(a, 1.0 / std::sqrt(dot(a, a))); }
};

/* Hittable (Hittable.cuh:402-503): one primitive of the tagged union {Light, Sphere, Triangle}. */
struct Hittable {
    enum Type { LIGHT, SPHERE, TRIANGLE } type;
    /* Light: centre, width, height, normal, emitted colour, visibility (Hittable.cuh:346-366) */
    Vec3 center{}, normal{};
    double width = 0, height = 0;
    bool visible = true;
    /* Sphere: centre, radius */
    double radius = 0;
    /* Triangle: vertices, optional vertex normals and texture coordinates (Hittable.cuh:57-83) */
    Vec3 p0{}, p1{}, p2{}, n0{}, n1{}, n2{};
    double uv[6] = {0, 0, 0, 0, 0, 0};
    Material material;   /* for a light: material.color is the emitted radiance */

    explicit Hittable(Type t) : type(t) {}

    static Hittable Light(Vec3 c, double w, double h, Vec3 n, Vec3 color, bool vis = true)
    {
        Hittable o(LIGHT);
        o.center = c; o.width = w; o.height = h; o.normal = n; o.visible = vis;
        o.material.color = color;
        o.material.type = M_LIGHT;
        return o;
    }
    static Hittable Sphere(Vec3 c, double r, const Material& m)
    {
        Hittable o(SPHERE);
        o.center = c; o.radius = r; o.material = m;
        return o;
    }
    static Hittable Triangle(Vec3 a, Vec3 b, Vec3 c, const Material& m)
    {
        Hittable o(TRIANGLE);
        o.p0 = a; o.p1 = b; o.p2 = c; o.material = m;
        return o;
    }
};

/* Assembles a scene description the way Scene::init adds objects (Scene.cuh:72-99 and
 * 175-270): lights first, then spheres, then triangles (floors as the two triangles
 * (lt, lb, rt), (rt, lb, rb) of Device.cuh:42-43, then meshes), whatever the order of the calls.
 * Each add takes its own material copy, as the reference's objects do.  Mesh-vertex bounds for
 * the Morton quantisation are updated by addMeshes only, as in ObjLoader.cuh:107-112. */
class SceneBuilder {
public:
    explicit SceneBuilder(const Camera& cam) : camera_(cam) {}

    void add(const Hittable& h)
    {
        switch (h.type) {
        case Hittable::LIGHT: addOneLight(h.center, h.width, h.height, h.normal, h.material.color, h.visible); break;
        case Hittable::SPHERE: addOneSphere(h.center, h.radius, h.material); break;
        case Hittable::TRIANGLE: push_tri(h, material(h.material)); break;
        }
    }
    void addOneLight(Vec3 position, double width, double height, Vec3 normal, Vec3 color, bool visible = true)
    {
        cpt_light l{};
        set3(l.center, position); set3(l.normal, normal); set3(l.color, color);
        l.width = width; l.height = height; l.visible = visible ? 1 : 0;
        lights_.push_back(l);
    }
    void addOneSphere(Vec3 position, double radius, const Material& m)
    {
        cpt_sphere s{};
        set3(s.center, position);
        s.radius = radius;
        s.material = material(m);
        spheres_.push_back(s);
    }
    void addFloor(Vec3 lt, Vec3 rt, Vec3 lb, Vec3 rb, const Material& m)
    {
        uint32_t mi = material(m);
        push_tri(Hittable::Triangle(lt, lb, rt, m), mi);
        push_tri(Hittable::Triangle(rt, lb, rb, m), mi);
    }
    /* A mesh already loaded and transformed (Mesh::loadFromFile + transform): its vertices before
     * the translation `position` feed the scene bounds. */
    void addMeshes(const std::vector<Hittable>& triangles, Vec3 position, const Material& m)
    {
        uint32_t mi = material(m);
        for (const Hittable& t : triangles) {
            for (const Vec3& p : {t.p0, t.p1, t.p2}) {
                bmin_ = Vec3{std::fmin(bmin_.x, p.x), std::fmin(bmin_.y, p.y), std::fmin(bmin_.z, p.z)};
                bmax_ = Vec3{std::fmax(bmax_.x, p.x), std::fmax(bmax_.y, p.y), std::fmax(bmax_.z, p.z)};
            }
            Hittable moved = t;
            for (Vec3* p : {&moved.p0, &moved.p1, &moved.p2}) *p = Vec3{p->x + position.x, p->y + position.y, p->z + position.z};
            push_tri(moved, mi);
        }
    }
    /* An RGB8 image (rows in file order) for Material::texture; returns its number (1-based). */
    int32_t addTexture(int width, int height, const uint8_t* rgb)
    {
        textures_.push_back(cpt_image{width, height, rgb});
        return (int32_t)textures_.size();
    }
    void setSkyBox(int width, int height, const uint8_t* rgb) { sky_ = cpt_image{width, height, rgb}; }

    /* The description; valid while the builder (and the images it points to) lives. */
    const cpt_scene_desc& desc()
    {
        d_ = cpt_scene_desc{};
        d_.num_lights = (uint32_t)lights_.size();
        d_.lights = lights_.data();
        d_.num_spheres = (uint32_t)spheres_.size();
        d_.spheres = spheres_.data();
        d_.num_triangles = (uint32_t)tri_mat_.size();
        d_.tri_vertices_f64 = tri_.empty() ? nullptr : tri_.data();
        d_.tri_normals = any_normal_ ? tri_n_.data() : nullptr;
        d_.tri_uvs = any_uv_ ? tri_uv_.data() : nullptr;
        d_.tri_material = tri_mat_.empty() ? nullptr : tri_mat_.data();
        if (mats_.empty()) mats_.push_back(Material().to_c());
        d_.num_materials = (uint32_t)mats_.size();
        d_.materials = mats_.data();
        d_.num_textures = (uint32_t)textures_.size();
        d_.textures = textures_.empty() ? nullptr : textures_.data();
        d_.sky = sky_;
        d_.bounds_min[0] = bmin_.x; d_.bounds_min[1] = bmin_.y; d_.bounds_min[2] = bmin_.z;
        d_.bounds_max[0] = bmax_.x; d_.bounds_max[1] = bmax_.y; d_.bounds_max[2] = bmax_.z;
        d_.camera = camera_.to_c();
        return d_;
    }

private:
    Camera camera_;
    std::vector<cpt_light> lights_;
    std::vector<cpt_sphere> spheres_;
    std::vector<cpt_material> mats_;
    std::vector<double> tri_;
    std::vector<float> tri_n_, tri_uv_;
    std::vector<uint32_t> tri_mat_;
    std::vector<cpt_image> textures_;
    cpt_image sky_{0, 0, nullptr};
    bool any_normal_ = false, any_uv_ = false;
    Vec3 bmin_{999999.0, 999999.0, 999999.0}, bmax_{-999999.0, -999999.0, -999999.0};   /* Scene.cuh:61-62 */
    cpt_scene_desc d_{};

    static void set3(double* dst, Vec3 v) { dst[0] = v.x; dst[1] = v.y; dst[2] = v.z; }
    uint32_t material(const Material& m)
    {
        mats_.push_back(m.to_c());
        return (uint32_t)(mats_.size() - 1);
    }
    void push_tri(const Hittable& t, uint32_t mi)
    {
        for (const Vec3& p : {t.p0, t.p1, t.p2}) { tri_.push_back(p.x); tri_.push_back(p.y); tri_.push_back(p.z); }
        for (const Vec3& n : {t.n0, t.n1, t.n2}) {
            tri_n_.push_back((float)n.x); tri_n_.push_back((float)n.y); tri_n_.push_back((float)n.z);
            any_normal_ = any_normal_ || n.x != 0 || n.y != 0 || n.z != 0;
        }
        for (double u : t.uv) { tri_uv_.push_back((float)u); any_uv_ = any_uv_ || u != 0; }
        tri_mat_.push_back(mi);
    }
};

class Context {
public:
    explicit Context(int device = 0) { check(cpt_context_create(device, &h_), "cpt_context_create"); }
    ~Context() { if (h_) cpt_context_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    Context(Context&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    cpt_context* get() const { return h_; }

private:
    cpt_context* h_ = nullptr;
};

class Scene {
public:
    /* Scene::init from an INI file: parse, upload, build the LBVH. */
    Scene(Context& ctx, const char* ini_path, void* stream = nullptr)
    {
        check(cpt_scene_load_ini(ctx.get(), ini_path, &h_), "cpt_scene_load_ini");
        buildBVH(stream);
    }
    /* Scene from a caller-assembled description (reference object order). */
    Scene(Context& ctx, const cpt_scene_desc& desc, void* stream = nullptr)
    {
        check(cpt_scene_create(ctx.get(), &desc, &h_), "cpt_scene_create");
        buildBVH(stream);
    }
    ~Scene() { if (h_) cpt_scene_destroy(h_); }
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;
    Scene(Scene&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    cpt_scene* get() const { return h_; }

    cpt_bvh_stats buildBVH(void* stream = nullptr)
    {
        cpt_bvh_stats st{};
        check(cpt_lbvh_build(h_, stream, &st), "cpt_lbvh_build");
        return st;
    }
    /* Scene::Update: new vertices for triangles [first, first + count), then a rebuild (or a refit
     * that keeps the topology). */
    void Update(const float* vertices, uint32_t first, uint32_t count, bool rebuild = true, void* stream = nullptr)
    {
        check(cpt_scene_update_triangles(h_, vertices, first, count, stream), "cpt_scene_update_triangles");
        if (rebuild) buildBVH(stream);
        else check(cpt_lbvh_refit(h_, stream, nullptr), "cpt_lbvh_refit");
    }
    cpt_render_stats render(const cpt_render_params& p, const cpt_render_output& out, void* stream = nullptr)
    {
        cpt_render_stats st{};
        check(cpt_render(h_, &p, &out, stream, &st), "cpt_render");
        return st;
    }
    void trace(const cpt_ray* rays, uint64_t n, cpt_hit* hits, bool on_device, void* stream = nullptr)
    {
        check(cpt_trace_closest(h_, rays, n, hits, on_device ? 1 : 0, stream), "cpt_trace_closest");
    }
    int32_t pick(int32_t x, int32_t y)
    {
        int32_t prim = -1;
        check(cpt_pick(h_, x, y, &prim), "cpt_pick");
        return prim;
    }
    void changeMaterial(uint32_t first, uint32_t end, double alpha_x, double alpha_y, bool glass)
    {
        check(cpt_scene_set_material(h_, first, end, alpha_x, alpha_y, glass ? 1 : 0), "cpt_scene_set_material");
    }

private:
    cpt_scene* h_ = nullptr;
};

/* render<<<>>>(devPtr, pic, ...) in STATIC mode (Render.cu:16-261, launched by main.cu:78-80):
 * rgb (pic) = mean radiance per pixel, W*H*3 floats, row 0 at the bottom; rgba8 (devPtr,
 * optional) = the display bytes.  on_device: the buffers are device pointers.  The reference
 * estimator unless params say otherwise; returns the ray count and device time. */
inline cpt_render_stats render(Scene& scene, float* rgb, uint8_t* rgba8, int spp, uint64_t seed = 0,
                               bool on_device = false, void* stream = nullptr)
{
    cpt_render_params p{};
    p.spp = spp;
    p.estimator = CPT_ESTIMATOR_REFERENCE;
    p.integrator = CPT_INTEGRATOR_MEGAKERNEL;
    p.rr_prob = 0.7f;
    p.seed = seed;
    cpt_render_output o{};
    o.rgb = rgb;
    o.rgba8 = rgba8;
    o.on_device = on_device ? 1 : 0;
    return scene.render(p, o, stream);
}

inline cpt_render_stats render(Scene& scene, const cpt_render_params& params, float* rgb, uint8_t* rgba8 = nullptr,
                               bool on_device = false, void* stream = nullptr)
{
    cpt_render_output o{};
    o.rgb = rgb;
    o.rgba8 = rgba8;
    o.on_device = on_device ? 1 : 0;
    return scene.render(params, o, stream);
}

}  // namespace cpt

#endif /* CPT_HPP */

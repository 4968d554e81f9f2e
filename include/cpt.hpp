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
 *
 * Errors: the wrappers throw cpt::Error (status + cpt_last_error_string()) where the reference
 * called exit(99) (Device.cuh:9-19).  Objects own their handles (move-only). */
#ifndef CPT_HPP
#define CPT_HPP

#include <stdexcept>
#include <string>
#include <utility>

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

}  // namespace cpt

#endif /* CPT_HPP */

/*
 * cpt.h — C ABI of the GB300 path-tracing library (libcpt.so).
 *
 * The library replaces the hot path of CudaPathTracing: LBVH construction
 * (Morton codes, radix sort, Karras hierarchy emission, bounding-box refit) and the
 * trace loop (closest-hit traversal, primitive intersection, shading, next-event
 * estimation, Russian roulette).  Every entry point is `extern "C"`, takes plain
 * pointers and sizes, returns a cpt_status, never exits the process and never frees
 * a buffer it did not allocate.  The reference interface each entry point replaces is
 * cited as file:line within the CudaPathTracing project.
 *
 * Threading: a context may be used by one host thread at a time.  Work is ordered on
 * the CUDA stream passed in (NULL = the legacy default stream).
 * Errors: the text of the last failure on the calling thread is returned by
 * cpt_last_error_string().
 */
#ifndef CPT_H
#define CPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPT_ABI_VERSION 1

typedef enum cpt_status {
    CPT_OK = 0,
    CPT_ERR_INVALID_ARGUMENT = 1,
    CPT_ERR_CUDA = 2,
    CPT_ERR_OUT_OF_MEMORY = 3,
    CPT_ERR_TIMEOUT = 4,        /* a device loop hit its iteration limit */
    CPT_ERR_STACK_OVERFLOW = 5, /* a traversal stack or tree depth limit was exceeded */
    CPT_ERR_PARSE = 6,          /* malformed INI / OBJ input */
    CPT_ERR_NOT_BUILT = 7,      /* the scene has no BVH yet */
    CPT_ERR_UNSUPPORTED = 8,
    CPT_ERR_IO = 9
} cpt_status;

/* Material kinds.  Values 0..5 are the reference's MaterialType (rtmath.cuh:15);
 * CPT_M_LAMBERTIAN is new (the reference only has it as commented-out code,
 * Material.cuh:177-188) and falls back to CPT_M_OPAQUE under the reference estimator,
 * exactly as IniParser::ParseMaterialType (IniParser.cpp:120-127) maps unknown names. */
typedef enum cpt_material_type {
    CPT_M_NONE = 0,
    CPT_M_LIGHT = 1,
    CPT_M_OPAQUE = 2,               /* anisotropic GGX conductor (Material.cuh:71-92) */
    CPT_M_SPECULAR_DIELECTRIC = 3,  /* Fresnel-weighted delta reflect/refract (:32-50) */
    CPT_M_ROUGH_DIELECTRIC = 4,     /* GGX BTDF (:51-70, :118-174) */
    CPT_M_VOLUME = 5,               /* boundary of a homogeneous medium (Render.cu:64-135) */
    CPT_M_LAMBERTIAN = 6
} cpt_material_type;

/* Material (Material.cuh:5-22).  Colours are linear RGB.  eta, sigma_t and albedo are
 * used by the config estimator only; the reference estimator uses eta = 1.51
 * (Material.cuh:12) and the reference's volume constants (Render.cu:66,87). */
typedef struct cpt_material {
    double color[3];
    double alpha_x, alpha_y;
    int32_t type;    /* cpt_material_type */
    int32_t texture; /* 0: none; k >= 1: image k-1 of cpt_scene_desc.textures, whose texel at the hit's
                        interpolated UV replaces color on triangles (HitRecord::sampleTexture,
                        HitRecord.cuh:38-49; Triangle::hit, Hittable.cuh:123-125) */
    double eta;
    double sigma_t;
    double albedo;
} cpt_material;

/* An 8-bit RGB image, 3 bytes per texel, rows in file order (the first row is v = 0), as
 * stbi_load returns it and as the reference indexes it (HitRecord.cuh:44-48, Camera.cuh:56-61). */
typedef struct cpt_image {
    int32_t width;
    int32_t height;
    const uint8_t* rgb;
} cpt_image;

/* Rectangular one-sided area light (Light, Hittable.cuh:346-399; LightInfo, IniParser.h:26-34). */
typedef struct cpt_light {
    double center[3];
    double normal[3];
    double width, height;
    double color[3]; /* emitted radiance */
    int32_t visible; /* 0: the light is sampled by NEE but never hit by rays */
    int32_t reserved;
} cpt_light;

/* Sphere (Sphere, Hittable.cuh:10-55). */
typedef struct cpt_sphere {
    double center[3];
    double radius;
    uint32_t material;
    uint32_t reserved;
} cpt_sphere;

/* Pinhole camera (Camera.cu:5-40).  height must equal the reference rule
 * max(1, (int)(width / aspect_ratio)) (Camera.cu:11, main.cu:26-27). Image row 0 is the
 * bottom row, as in the reference (Camera.cu:29). */
typedef struct cpt_camera {
    int32_t width;
    int32_t height;
    double aspect_ratio;
    double look_from[3];
    double look_at[3];
    double vfov_deg;
    double background[3]; /* colour returned for rays that miss (Camera.cuh:50-53) */
} cpt_camera;

/* Scene description.  Primitives are indexed in the reference's object order
 * (Scene.cuh:72-99): lights [0, L), spheres [L, L+S), triangles [L+S, L+S+T); that index
 * is the one encoded in the low 32 bits of each Morton key (Device.cuh:138). */
typedef struct cpt_scene_desc {
    uint32_t num_lights;
    const cpt_light* lights;
    uint32_t num_spheres;
    const cpt_sphere* spheres;
    uint32_t num_triangles;
    const float* tri_vertices;      /* 9 floats per triangle (p0, p1, p2), or NULL */
    const double* tri_vertices_f64; /* 9 doubles per triangle, or NULL; exactly one is set when T > 0 */
    const float* tri_normals;       /* optional: 9 floats per triangle (n0, n1, n2), Hittable.cuh:123-137 */
    const uint32_t* tri_material;   /* T material indices */
    uint32_t num_materials;
    const cpt_material* materials;
    /* Mesh-vertex bounds before the +-1 expansion of Device::buildBVH (Device.cuh:174-181).
     * If min > max on x the reference's [-20, 20]^3 fallback applies. */
    double bounds_min[3];
    double bounds_max[3];
    cpt_camera camera;
    const float* tri_uvs;         /* optional: 6 floats per triangle (uv0, uv1, uv2), Hittable.cuh:60;
                                     NULL = all zero, as for OBJ faces without vt (ObjLoader.cuh:119-134) */
    uint32_t num_textures;
    const cpt_image* textures;    /* images referenced by cpt_material.texture */
    cpt_image sky;                /* equirectangular sky returned for rays that miss (Camera::getSkyBox,
                                     Camera.cuh:50-63); sky.rgb NULL = the camera's background colour */
} cpt_scene_desc;

typedef struct cpt_ray {
    float origin[3];
    float tmin; /* lower limit of the box tests (traverseIterative's tMin, BVH.cuh:282) */
    float direction[3];
    float tmax; /* upper limit (traverseIterative's tMax; the reference default is 999999) */
} cpt_ray;

/* Closest hit: prim = primitive index in the order above, -1 on a miss. */
typedef struct cpt_hit {
    float t;
    int32_t prim;
    float u, v; /* barycentrics for triangles, 0 otherwise */
} cpt_hit;

typedef struct cpt_bvh_stats {
    uint32_t num_prims;
    uint32_t max_depth;  /* deepest leaf of the binary LBVH (constructAABB's p_max, BVH.cuh:279) */
    uint32_t num_wide_nodes;
    uint32_t reserved;
    float ms_prep;       /* centroids, leaf boxes and Morton keys */
    float ms_sort;
    float ms_emit;       /* Karras hierarchy emission */
    float ms_refit;
    float ms_collapse;   /* traversal layout */
    float ms_total;
} cpt_bvh_stats;

typedef enum cpt_estimator {
    /* The reference's STATIC render (Render.cu:16-261): RR 0.7 from the first bounce,
     * unbounded depth, NEE only on Opaque, emission ignored after the first NEE,
     * light pdf 1/(width*width), volume with sigma_maj = 25. */
    CPT_ESTIMATOR_REFERENCE = 0,
    /* Config estimator: Lambertian, per-material IOR, homogeneous media with sigma_t and
     * albedo, maximum depth, RR from rr_depth on, NEE on Opaque and Lambertian. */
    CPT_ESTIMATOR_CONFIG = 1
} cpt_estimator;

typedef enum cpt_integrator {
    CPT_INTEGRATOR_MEGAKERNEL = 0,
    CPT_INTEGRATOR_WAVEFRONT = 1
} cpt_integrator;

enum {
    CPT_RENDER_ACCUMULATE = 1 /* add into rgb instead of overwriting (progressive) */
};

typedef struct cpt_render_params {
    int32_t spp;
    int32_t estimator;  /* cpt_estimator */
    int32_t integrator; /* cpt_integrator */
    int32_t max_depth;  /* config estimator; <= 0: unbounded */
    int32_t rr_depth;   /* config estimator: Russian roulette from this depth on */
    float rr_prob;      /* survival probability (reference: 0.7, Render.cu:202) */
    uint64_t seed;      /* PCG32 seed; stream = pixel offset j*W+i (Render.cu:25,32) */
    int32_t row_begin;  /* render rows [row_begin, row_end); 0,0 = the whole image */
    int32_t row_end;
    int32_t flags;
    int32_t reserved;
} cpt_render_params;

typedef struct cpt_render_output {
    float* rgb;        /* W*H*3 mean radiance per pixel (pic, Render.cu:222-225); required */
    uint8_t* rgba8;    /* optional W*H*4: sqrt gamma, x254.99, clamp (Render.cu:229-260) */
    float* gbuffer;    /* optional W*H*8: first-hit normal xyz, distance, albedo rgb, and (config
                          estimator) the variance of the pixel mean's luminance over its samples
                          (one sample: its squared luminance); 0 under the reference estimator */
    int32_t on_device; /* 1: the pointers above are device pointers, 0: host */
    int32_t reserved;
} cpt_render_output;

typedef struct cpt_render_stats {
    uint64_t rays;      /* closest-hit queries traced (camera, bounce, shadow, volume) */
    uint64_t paths;
    double ms;          /* device time of the render */
} cpt_render_stats;

/* Joint-bilateral filter parameters (gaussianSeparate, Render.cu:356-398).  Defaults (NULL
 * params): sigma_g 8, sigma_r 5, sigma_n 0.1, sigma_d 0.2 (Window.cu:11-14), radius 16
 * (KERNEL_RADIUS, Render.cuh:8). */
typedef struct cpt_filter_params {
    float sigma_g, sigma_r, sigma_n, sigma_d;
    int32_t radius;
} cpt_filter_params;

typedef struct cpt_context cpt_context;
typedef struct cpt_scene cpt_scene;

/* ---- library ------------------------------------------------------------------ */
int cpt_abi_version(void);
/* Number of CUDA kernels this library has launched since it was loaded (all threads). */
uint64_t cpt_launch_count(void);
const char* cpt_last_error_string(void);

/* Creates a context on a CUDA device (the reference's Device ctor, Device.cuh:161-168,
 * without its fixed 2,000,000-object pool). */
cpt_status cpt_context_create(int device, cpt_context** out);
cpt_status cpt_context_destroy(cpt_context* ctx);

/* Render tuning used by the autotuner: megakernel thread-block shape (bx*by a multiple of 32,
 * at most 512).  The defaults are 16 x 8. */
cpt_status cpt_context_set_render_block(cpt_context* ctx, int block_x, int block_y);
/* Wavefront integrator tuning: number of path slots (>= 1024; the wavefront size), thread-block
 * sizes of the trace and shade kernels (multiples of 32, at most 256), and whether iterations
 * are replayed from a captured CUDA graph.  Defaults: 2,097,152 slots, 128, 128, graphs on. */
cpt_status cpt_context_set_wavefront(cpt_context* ctx, int slots, int block_trace, int block_shade, int use_graph);
/* Depth of the wavefront trace kernels' shared-memory short stack (8, 16, 24 or 32 entries; the
 * rest of the traversal stack is in local memory).  Default 16. */
cpt_status cpt_context_set_short_stack(cpt_context* ctx, int entries);
/* Traversal layout built by later cpt_lbvh_build / cpt_lbvh_refit calls: 2 = binary nodes with
 * both child boxes per 64-byte node (the default), 8 = the compressed 8-wide BVH (96-byte nodes,
 * 8-bit quantised child boxes, direction-ordered slots). */
cpt_status cpt_context_set_bvh_width(cpt_context* ctx, int width);
/* BVH2 node format of later cpt_lbvh_build / cpt_lbvh_refit calls: 0 = 64-byte nodes with both
 * child boxes in FP32 (the default), 1 = 32-byte nodes (one memory sector per visit) with both
 * child boxes quantised outwards to 8 bits on a grid spanning the node, and the children as the
 * Karras split index.  Closest hits are the same up to exact ties; the quantised boxes are larger,
 * so a traversal may test a few more nodes. */
cpt_status cpt_context_set_bvh_compression(cpt_context* ctx, int on);
/* Wavefront integrator: when on, every iteration files the traced paths into bins by the material
 * their ray hit (miss / light / medium, Opaque and Lambertian, specular dielectric, rough
 * dielectric) and shades the bins in order, so that a warp's lanes run one BSDF.  The image is
 * the same either way.  Default off. */
cpt_status cpt_context_set_material_sort(cpt_context* ctx, int on);
/* Bounds of the device loops that replace the reference's unbounded `while (true)` bounce loop
 * (Render.cu:58) and its exit(99) on failure (Device.cuh:9-19): max_trips = loop trips per sample
 * (bounces plus volume steps) after which a path is stopped and the render returns
 * CPT_ERR_TIMEOUT; max_replays = wavefront iteration chunks (8 iterations each) replayed before a
 * render that has not drained returns CPT_ERR_TIMEOUT.  Defaults and maxima: 65536 and 1048576. */
cpt_status cpt_context_set_loop_limits(cpt_context* ctx, int32_t max_trips, int32_t max_replays);

/* ---- scene files (host only, no GPU needed) ------------------------------------------ */
/* Parses an INI scene (IniParser::Parse, IniParser.cpp:3-96) and assembles it in the
 * reference's object order (Scene::init, Scene.cuh:72-99: lights, spheres, floors as two
 * triangles each, OBJ meshes).  cpt_ini_describe fills a description whose pointers stay
 * valid until cpt_ini_free. */
typedef struct cpt_ini_scene cpt_ini_scene;
cpt_status cpt_ini_load(const char* path, cpt_ini_scene** out);
cpt_status cpt_ini_describe(const cpt_ini_scene* ini, cpt_scene_desc* out);
cpt_status cpt_ini_free(cpt_ini_scene* ini);

/* ---- scene ---------------------------------------------------------------------- */
/* Uploads a scene (replaces Scene::init's per-object <<<1,1>>> allocation kernels,
 * Scene.cuh:72-99,175-230, and Device::allocate*OnDevice, Device.cuh:29-79). */
cpt_status cpt_scene_create(cpt_context* ctx, const cpt_scene_desc* desc, cpt_scene** out);
/* Parses an INI scene file and uploads it (IniParser::Parse, IniParser.cpp:3-96, then
 * Scene::init, Scene.cuh:72).  [Mesh] sections load Wavefront OBJ files. */
cpt_status cpt_scene_load_ini(cpt_context* ctx, const char* path, cpt_scene** out);
cpt_status cpt_scene_destroy(cpt_scene* scene);
/* Counts and camera of a created scene. */
cpt_status cpt_scene_info(const cpt_scene* scene, uint32_t* num_lights, uint32_t* num_spheres,
                          uint32_t* num_triangles, cpt_camera* camera);
/* Replaces triangle vertices [first, first+count) (host pointer, 9 floats each) before a
 * rebuild or refit; the cloth update path (updateClothToDevice, Device.cuh:109-131). */
cpt_status cpt_scene_update_triangles(cpt_scene* scene, const float* tri_vertices, uint32_t first,
                                      uint32_t count, void* stream);

/* ---- LBVH ----------------------------------------------------------------------- */
/* Builds the LBVH and the traversal layout (Device::buildBVH, Device.cuh:169-195).
 * Morton keys, order and topology are bit-identical to the reference's. */
cpt_status cpt_lbvh_build(cpt_scene* scene, void* stream, cpt_bvh_stats* stats);
/* Recomputes boxes for moved vertices keeping the topology (the refit half of the
 * per-frame rebuild in Scene::Update, Scene.cuh:147-173). */
cpt_status cpt_lbvh_refit(cpt_scene* scene, void* stream, cpt_bvh_stats* stats);
/* Copies the binary LBVH to host buffers (any may be NULL): keys[N] sorted Morton keys
 * (code << 32 | index, Device.cuh:138-141), order[N] primitive index of each leaf,
 * child_a/child_b[N-1] children of each internal node (>= 0 internal node index,
 * < 0 leaf ~k, BVH.cuh:213-229), node_boxes[(N-1)*6] and leaf_boxes[N*6] as
 * min xyz, max xyz in FP32 rounded outwards from the reference's FP64 boxes. */
cpt_status cpt_lbvh_export(const cpt_scene* scene, uint64_t* keys, uint32_t* order, int32_t* child_a,
                           int32_t* child_b, float* node_boxes, float* leaf_boxes);

/* Low-level, caller-owned buffers: the same build on device pointers (the shape of
 * Device::buildBVH(d_objs, leaf, internal, d_mortons, d_objIdx, N, min, max), Device.cuh:169).
 *   extra_centroids: num_extra*3 doubles (light and sphere centres, Hittable.cuh:419,425)
 *   extra_boxes:     num_extra*8 floats (min xyz, 0, max xyz, 0; their leaf boxes rounded outwards)
 *   tri_vertices:    num_tri*9 floats; triangle i is primitive num_extra + i
 *   scene_min/max:   mesh bounds before the +-1 expansion (applied here, Device.cuh:174-181)
 * Outputs (N = num_extra + num_tri):
 *   out_keys[N]            sorted Morton keys (code << 32 | index); may be NULL
 *   out_order[N]           primitive index of each sorted leaf
 *   out_children[2*(N-1)]  (child A, child B) per internal node, leaf k encoded as ~k
 *   out_node_range[2*(N-1)] (first, last) sorted-leaf range of each internal node
 *   out_node_boxes[8*(N-1)], out_leaf_boxes[8*N]  min xyz, 0, max xyz, 0
 *   scratch: cpt_lbvh_scratch_bytes(N) bytes, 256-byte aligned; work is ordered on stream. */
size_t cpt_lbvh_scratch_bytes(uint32_t num_prims);
cpt_status cpt_lbvh_build_device(uint32_t num_extra, const double* extra_centroids, const float* extra_boxes,
                                 uint32_t num_tri, const float* tri_vertices, const double scene_min[3],
                                 const double scene_max[3], uint64_t* out_keys, uint32_t* out_order,
                                 int32_t* out_children, int32_t* out_node_range, float* out_node_boxes,
                                 float* out_leaf_boxes, void* scratch, size_t scratch_bytes, void* stream);

/* No counterpart in the reference.  The same build as cpt_lbvh_build_device for callers that
 * cannot allocate device memory — e.g. a host that has divided all of its HBM among its own
 * pools at start-up, or code in a frame loop or callback where a cudaMalloc (and the device
 * synchronisation it implies) is not allowed.  The caller passes inputs and outputs only; the
 * scratch is a 3 MiB array compiled into this library, which every GPU that loads it keeps
 * until the process exits.  At most CPT_LBVH_STATIC_MAX_PRIMS primitives; more is rejected with
 * CPT_ERR_INVALID_ARGUMENT.  The call allocates nothing.  Its first call on a device looks up the
 * array's device address in the current CUDA context (do that first call before any stream
 * capture); the address is cached per context, so after cudaDeviceReset the next call looks it up
 * again.  All calls share the one array: calls whose work overlaps on the GPU (other streams,
 * other host threads) race. */
#define CPT_LBVH_STATIC_MAX_PRIMS 65536u
cpt_status cpt_lbvh_build_device_static(uint32_t num_extra, const double* extra_centroids, const float* extra_boxes,
                                        uint32_t num_tri, const float* tri_vertices, const double scene_min[3],
                                        const double scene_max[3], uint64_t* out_keys, uint32_t* out_order,
                                        int32_t* out_children, int32_t* out_node_range, float* out_node_boxes,
                                        float* out_leaf_boxes, void* stream);

/* ---- trace ---------------------------------------------------------------------- */
/* Closest hit for n rays (traverseIterative, BVH.cuh:282-332, and Hittable::hit,
 * Hittable.cuh:487-503).  rays/hits are device pointers when on_device != 0, else host
 * buffers that are copied in and out on `stream` (the call then synchronises it). */
cpt_status cpt_trace_closest(cpt_scene* scene, const cpt_ray* rays, uint64_t n, cpt_hit* hits,
                             int on_device, void* stream);

/* ---- render --------------------------------------------------------------------- */
/* The reference's real-time denoiser on device buffers (W*H float3 images, row 0 at the
 * bottom; gbuf = the renderer's G-buffer, 2 float4 per pixel).
 * cpt_filter_bilateral: separable joint-bilateral filter, horizontal then vertical pass
 *   (gaussianSeparate, Render.cu:356-398, as run by main.cu:99-103); out must not alias rgb.
 * cpt_filter_temporal: rgb = alpha * rgb + (1 - alpha) * prev_rgb at the pixel where the
 *   previous camera saw this pixel's first hit (addPrevious, Render.cu:400-420;
 *   Camera::getPrePositionInImg, Camera.cuh:103-132); the reference uses alpha 0.1, or 0.4
 *   while the camera moves.  The hit position is rebuilt from the G-buffer depth along the
 *   pixel-centre ray. */
cpt_status cpt_filter_bilateral(cpt_context* ctx, const float* rgb, const float* gbuf, float* out, int32_t width,
                                int32_t height, const cpt_filter_params* params, void* stream);
cpt_status cpt_filter_temporal(cpt_context* ctx, float* rgb, const float* prev_rgb, const float* gbuf,
                               const cpt_camera* camera, const cpt_camera* prev_camera, float alpha, void* stream);

/* Picking and live material edit (getObject / changeMaterial, Render.cu:485-522, driven by
 * Window.cu:313-346).  cpt_pick: the primitive (reference numbering, a light included) hit by the
 * ray through the centre of pixel (x, y), row 0 at the bottom; -1 on a miss or outside the image.
 * cpt_scene_set_material: primitives [first, end) keep their colours and take roughness
 * (alpha_x, alpha_y) and the Opaque type, or SpecularDielectric when glass != 0 (lights are
 * skipped); primitives outside the range are unchanged. */
cpt_status cpt_pick(cpt_scene* scene, int32_t x, int32_t y, int32_t* prim);
cpt_status cpt_scene_set_material(cpt_scene* scene, uint32_t first, uint32_t end, double alpha_x, double alpha_y,
                                  int32_t glass);

/* ---- learned denoiser (no counterpart in the reference) --------------------------------
 * Kernel-predicting U-Net (5 levels, 32-64-96-128-160 channels, 3x3 convolutions, a predicted
 * 5x5 filter per pixel applied to the noisy radiance), trained and run on the library's own
 * BF16 tensor-core kernels with FP32 accumulation.  Parameters are one FP32 array
 * (cpt_denoiser_num_params floats: per convolution W[9][cin][cout] then b[cout]).
 * Images are device buffers: rgb and target [n][h][w][3] f32, gbuf [n][h][w][8] f32 (the
 * renderer's G-buffer).  Training crops must be multiples of 16; cpt_denoise takes any size. */
typedef struct cpt_denoiser cpt_denoiser;
cpt_status cpt_denoiser_create(int device, uint64_t seed, cpt_denoiser** out);
cpt_status cpt_denoiser_destroy(cpt_denoiser* d);
uint64_t cpt_denoiser_num_params(const cpt_denoiser* d);
cpt_status cpt_denoiser_get_params(cpt_denoiser* d, float* host_out);
cpt_status cpt_denoiser_set_params(cpt_denoiser* d, const float* host_in); /* also resets Adam */
cpt_status cpt_denoiser_get_grads(cpt_denoiser* d, float* host_out);      /* of the last train step */
/* Copies an internal tensor of the last pass (activations "X0", "A0a", "cat0", ..., "logits",
 * "out"; gradients "G_D0b", ...) as floats into host (if capacity suffices); *count = elements.
 * cpt_denoise on the default engine applies the predicted kernels inside the last convolution and
 * does not store "logits" (asking for them then fails with CPT_ERR_UNSUPPORTED);
 * cpt_denoiser_train_step stores every tensor. */
cpt_status cpt_denoiser_export(cpt_denoiser* d, const char* name, float* host, uint64_t capacity, uint64_t* count);
/* One step: forward, loss = mean |sqrt(out + 1e-3) - sqrt(target + 1e-3)|, backward, and (update != 0)
 * an Adam step with learning rate lr.  *loss (optional) receives the loss before the update. */
cpt_status cpt_denoiser_train_step(cpt_denoiser* d, int32_t n, int32_t h, int32_t w, const float* rgb,
                                   const float* gbuf, const float* target, float lr, int32_t update, float* loss,
                                   void* stream);
cpt_status cpt_denoise(cpt_denoiser* d, int32_t n, int32_t h, int32_t w, const float* rgb, const float* gbuf,
                       float* out, void* stream);
/* Convolution engine for the forward and input-gradient convolutions: 2 = TMA-fed warp-specialised
 * persistent tcgen05 kernels (the default: row tiles with halo reuse where the padded width is a
 * multiple of 128, im2col tiles elsewhere), 1 = tcgen05 kernel with cp.async copies, 0 = warp-level
 * mma.sync kernel. */
cpt_status cpt_denoiser_set_backend(cpt_denoiser* d, int32_t backend);
/* CPT_ERR_TIMEOUT if a tensor-core barrier wait of the passes since the last check timed out. */
cpt_status cpt_denoiser_check(cpt_denoiser* d);
/* Diagnostic: runs the bounded barrier wait of the tensor-core kernels on a barrier that nothing
 * arrives on, so that it gives up (after about one second) and sets the error word; the next
 * cpt_denoiser_check returns CPT_ERR_TIMEOUT and the denoiser stays usable.  Nothing is copied or
 * computed while it waits. */
cpt_status cpt_denoiser_wait_selftest(cpt_denoiser* d);

/* Renders the scene's camera view (render, Render.cu:16-261, STATIC mode). */
cpt_status cpt_render(cpt_scene* scene, const cpt_render_params* params, const cpt_render_output* out,
                      void* stream, cpt_render_stats* stats);

/* One render of a batch. */
typedef struct cpt_render_job {
    cpt_scene* scene;
    cpt_render_params params; /* config estimator; integrator is ignored (the batch is a wavefront) */
    cpt_render_output output;
} cpt_render_job;

/* No counterpart in the reference (its render kernel draws one image per launch, Render.cu:16).
 * Renders several jobs — scenes of one context, any image sizes, sample counts, depth settings
 * and seeds — in one wavefront: paths of all jobs share the path slots, queues and persistent
 * kernels, so small jobs fill the GPU together.  Each job's outputs are exactly what cpt_render
 * gives for it alone with the wavefront integrator.  All scenes must use the same BVH width.
 * stats (optional) sums rays and paths over the jobs; ms is the batch's device time. */
cpt_status cpt_render_batch(cpt_context* ctx, const cpt_render_job* jobs, uint32_t count, void* stream,
                            cpt_render_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* CPT_H */

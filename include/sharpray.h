/*
 * sharpray.h — C ABI of the GB300 (sm_103a) render hot path of SharpRay.
 *
 * The library replaces the CPU render call of the C# reference: scene construction
 * (Scene/Object/Mesh/Texture/SkyTexture/Fog), the Renderer (per-pixel path loop with
 * adaptive sampling and seven AOVs) and the Compositor (joint bilateral denoise, fog blur,
 * tonemap).  Every entry point is plain C: blittable structs, raw pointers and sizes,
 * int status codes (SR_OK == 0) and a thread-local message from sr_last_error_message().
 *
 * Each declaration names the reference interface it replaces (file:line within the
 * SharpRay project).  Struct layouts are fixed (all fields 4 bytes) so that a C# host can
 * mirror them with [StructLayout(LayoutKind.Sequential)].
 *
 * Threading: one SrContext per host thread.  All device work of a context runs on the
 * context's CUDA stream unless a *_device entry point is given an explicit stream.
 */
#ifndef SHARPRAY_H
#define SHARPRAY_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SR_API __attribute__((visibility("default")))
#else
#define SR_API
#endif

/* ---- status codes ------------------------------------------------------------------ */
enum {
    SR_OK = 0,
    SR_ERR_INVALID_ARG = 1,   /* bad pointer, size or id (reference: Debug.Assert)        */
    SR_ERR_STATE = 2,         /* build-state misuse (reference: InvalidOperationException)*/
    SR_ERR_CUDA = 3,          /* a CUDA runtime call failed                                */
    SR_ERR_OUT_OF_MEMORY = 4, /* device allocation failed                                  */
    SR_ERR_DEVICE = 5,        /* a kernel reported an error word (e.g. traversal stack)   */
    SR_ERR_IO = 6             /* asset parse failure (reference: Exception in obj/image)  */
};

/* ---- handles ------------------------------------------------------------------------- */
typedef struct SrContext SrContext;
typedef struct SrScene SrScene;

/* ---- plain data ---------------------------------------------------------------------- */

/* One triangle exactly as Mesh(IReadOnlyList<Triangle>) consumes it: the lean form
 * (PosA, PosB-PosA, PosC-PosA) and the per-corner attributes.
 * Reference: Triangle math.cs:1491-1528, TriangleLean math.cs:1336-1344, mesh.cs:6-11. */
typedef struct SrTriangle {
    float pos_a[3], ab[3], ac[3];
    float norm_a[3], norm_b[3], norm_c[3];
    float tan_a[4], tan_b[4], tan_c[4]; /* xyz tangent, w bitangent handedness */
    float uv_a[2], uv_b[2], uv_c[2];
} SrTriangle;

/* Reference: Transform math.cs:773-879 (Pos, Rot quaternion x,y,z,w, Scale). */
typedef struct SrTransform {
    float pos[3];
    float rot[4];
    float scale[3];
} SrTransform;

/* Reference: Material scene.cs:161-187.  Texture ids are from sr_texture_create, -1 = none. */
typedef struct SrMaterial {
    float albedo[3];
    float roughness;
    float metallic;
    float transparency;
    float ior;
    float radiance[3];
    int32_t color_texture;
    int32_t roughness_texture;
    int32_t metallic_texture;
    int32_t normal_texture;
} SrMaterial;

enum { SR_SHAPE_MESH = 0, SR_SHAPE_SPHERE = 1, SR_SHAPE_AABOX = 2 };

/* Texel encodings of image files (sr_texture_load): Texture.FromSrgb, FromLinear (Image.Load .tga),
 * FromHdr (ImageHdr.Load .hdr) texture.cs:138-163. */
enum { SR_TEXTURE_SRGB = 0, SR_TEXTURE_LINEAR = 1, SR_TEXTURE_HDR = 2 };

/* Where BVHs are built (sr_ctx_set_bvh_build, sr_bvh_build). */
enum { SR_BVH_BUILD_HOST = 0, SR_BVH_BUILD_DEVICE = 1 };

/* Reference: IShape implementations Mesh (mesh.cs:4), Sphere (math.cs:1179), AABox (math.cs:936).
 * sphere: params = {cx, cy, cz, radius}; aabox: params = {minx, miny, minz, maxx, maxy, maxz}. */
typedef struct SrShape {
    int32_t kind;
    int32_t mesh;
    float params[6];
} SrShape;

/* Reference: Fog scene.cs:438-442: exponential height fog, density * exp(-height_falloff * y), for
 * height_falloff > 0 (top_height is then ignored).  An extension without a reference counterpart:
 * height_falloff == 0 gives a homogeneous medium of constant density below top_height (finite) and
 * none above it -- bounded, because through an unbounded homogeneous medium no sky light would reach
 * any point.  Its optical depth is density x the length of the segment below the top, and its
 * free-flight draw is the reference's single exponential per segment. */
typedef struct SrFog {
    float density;
    float color[3];
    float anisotropy;
    float height_falloff;
    float top_height;
} SrFog;

/* Reference: SkyProcedural ctor scene.cs:341-354 + SunProcedural scene.cs:281-298. */
typedef struct SrSkyProcedural {
    float top[3];
    float middle[3];
    float bottom[3];
    float sun_dir[3];
    float sun_radiance[3];
    float sun_angle;
} SrSkyProcedural;

/* Reference: View math.cs:1582-1611 (fov in radians, near plane distance). */
typedef struct SrView {
    SrTransform transform;
    float fov;
    float near_plane;
} SrView;

/* Reference: Renderer ctor arguments renderer.cs:40-51. */
typedef struct SrRenderParams {
    uint32_t width;
    uint32_t height;
    uint32_t block_size;
    uint32_t min_samples;
    uint32_t max_samples;
    float variance_threshold;
    uint32_t bounces;
    float indirect_clamp;
} SrRenderParams;

/* The seven AOV planes of Renderer (renderer.cs:14-20), width*height entries each:
 * radiance/radiance_fog/normals float3, uv float2, depth float (+inf = none),
 * samples uint32, variance float.  Host or device pointers depending on the entry point. */
typedef struct SrAovs {
    float* radiance;
    float* radiance_fog;
    float* normals;
    float* uv;
    float* depth;
    uint32_t* samples;
    float* variance;
} SrAovs;

enum { SR_TONEMAP_REINHARD = 0, SR_TONEMAP_LINEAR_SMOOTH = 1 };

/* Reference: Compositor ctor compose.cs:22-48. */
typedef struct SrComposeParams {
    int32_t tonemapper;
    float exposure;
    float denoise_radius;
    float denoise_strength;
    float denoise_strength_max;
    float denoise_luminance_boost;
    float denoise_luminance_limit;
    float denoise_normal_limit;
    float denoise_depth_limit;
    float denoise_fog_radius;
    float denoise_fog_strength;
} SrComposeParams;

/* Work counters of one render (reference Counters.Type, counters.cs:24-79), collected only
 * when requested.  Index names: */
enum {
    SR_COUNTER_SAMPLE = 0,        /* Scene.Sample calls                 (scene.cs:640)   */
    SR_COUNTER_SAMPLE_BOUNCE,     /* path segments                      (scene.cs:652)   */
    SR_COUNTER_SCENE_TRACE,       /* closest-hit rays                   (scene.cs:606)   */
    SR_COUNTER_SCENE_OCCLUDE,     /* shadow rays                        (scene.cs:581)   */
    SR_COUNTER_TLAS_NODE,         /* scene BVH box tests                (bvh.cs:189)     */
    SR_COUNTER_TLAS_SHAPE,        /* object tests                       (bvh.cs:203)     */
    SR_COUNTER_BLAS_NODE,         /* mesh BVH box tests                 (bvh.cs:189)     */
    SR_COUNTER_BLAS_SHAPE,        /* triangle tests                     (bvh.cs:203)     */
    SR_COUNTER_HIT_INFLATE,       /* closest hits inflated              (mesh.cs:57)     */
    SR_COUNTER_TEX_SAMPLE,        /* material Texture.Sample calls      (texture.cs:39)  */
    SR_COUNTER_CDF_PROBE,         /* Cdf1 search probes performed       (cdf.cs:40-52)   */
    SR_COUNTER_LIGHT_SAMPLE,      /* sky-texture light samples (Cdf2)   (scene.cs:408)   */
    SR_COUNTER_ENV_LOOKUP,        /* SkyTexture.Radiance lookups        (scene.cs:406)   */
    SR_COUNTER_COUNT
};

/* ---- errors / version ----------------------------------------------------------------- */
SR_API const char* sr_version(void);
/* Message of the last failed call on this host thread ("" if none). */
SR_API const char* sr_last_error_message(void);

/* ---- context ---------------------------------------------------------------------------- */
/* Binds CUDA device `device` and creates the context's stream.  No reference counterpart
 * (the reference has no device); owns every texture/mesh/scene created from it.
 * device == -1 creates a host-only context: meshes, BVH builds/exports and scene BVH builds
 * work, every entry point that needs the GPU returns SR_ERR_STATE. */
SR_API int sr_ctx_create(int device, SrContext** out_ctx);
/* Scenes still alive keep the context alive: it is freed when the last of them is destroyed (the
 * context itself must not be used after this call). */
SR_API int sr_ctx_destroy(SrContext* ctx);

/* ---- host-side ingest (no device work) --------------------------------------------------- */
/* Builds `count` SrTriangles from triangle-corner positions (count*9 floats), optional
 * corner uvs (count*6, NULL = (0,0),(1,0),(0,1)) and optional corner normals (count*9, NULL =
 * face normal), then, if smooth_normals != 0 and normals == NULL, replaces the normals by
 * area-weighted vertex normals.  Replaces the Triangle constructors (math.cs:1498-1527) as
 * TriangulateFace uses them (obj.cs:403-443) followed by Mesh.ComputeSmoothNormals
 * (mesh.cs:99-123), i.e. the ObjLoader BuildObject path (obj.cs:170-190). */
SR_API int sr_triangles_from_corners(const float* positions, const float* uvs, const float* normals,
                                     uint32_t count, int32_t smooth_normals, SrTriangle* out);

/* ---- textures ---------------------------------------------------------------------------- */
/* Float3 texels (width*height*3, row-major, row 0 = top), filter 0 = bilinear, 1 = point.
 * Replaces Texture (texture.cs:6-37) as built by FromSrgb/FromLinear/FromHdr (texture.cs:138-163). */
SR_API int sr_texture_create(SrContext* ctx, const float* texels_rgb, uint32_t width, uint32_t height,
                             int32_t filter, float tiling_x, float tiling_y, int32_t* out_id);

/* ---- meshes ------------------------------------------------------------------------------ */
/* Builds the mesh BVH on the host (binned SAH, 8 bins, intersect cost 0.5; node order and item
 * permutation identical to bvh.cs) and uploads triangles + attributes.  Replaces
 * Mesh(IReadOnlyList<Triangle>) mesh.cs:18-45. */
SR_API int sr_mesh_create(SrContext* ctx, const SrTriangle* triangles, uint32_t count, int32_t* out_id);
/* Where sr_mesh_create and sr_scene_build build their BVHs: SR_BVH_BUILD_HOST (default) or
 * SR_BVH_BUILD_DEVICE (level by level on the context's GPU; node order, item permutation and bounds
 * bit-identical to the host build).  No counterpart in the reference, which builds on the CPU
 * (bvh.cs:58-75). */
SR_API int sr_ctx_set_bvh_build(SrContext* ctx, int32_t where);
/* The reference's Bvh over arbitrary shape bounds (Bvh ctor bvh.cs:58-75 with InsertRoot/Subdivide
 * :285-459): `bounds` holds {min xyz, max xyz} per shape; built on the host or, with
 * SR_BVH_BUILD_DEVICE, on the context's GPU.  Outputs as sr_mesh_bvh_export, sized for 2*count
 * nodes (node_links and items may be NULL); `node_count` receives the nodes used. */
SR_API int sr_bvh_build(SrContext* ctx, const float* bounds, uint32_t count, float cost_traverse,
                        float cost_intersect, int32_t bins, int32_t where, float* node_bounds, int32_t* node_links,
                        int32_t* items, uint32_t* node_count);
/* Node count of a mesh BVH (for sizing sr_mesh_bvh_export buffers). */
SR_API int sr_mesh_bvh_size(SrContext* ctx, int32_t mesh, uint32_t* node_count, uint32_t* item_count);
/* Exports the BVH exactly as bvh.cs stores it: per node {min xyz, max xyz} floats (6 per node)
 * and {child, shapeCount} ints (2 per node), plus the item permutation.  Replaces the private
 * Bvh._nodes/_items arrays (bvh.cs:53-55); used by parity tests. */
SR_API int sr_mesh_bvh_export(SrContext* ctx, int32_t mesh, float* node_bounds, int32_t* node_links,
                              int32_t* items);

/* ---- scenes ------------------------------------------------------------------------------ */
/* Replaces `new Scene()` (scene.cs:507). */
SR_API int sr_scene_create(SrContext* ctx, SrScene** out_scene);
SR_API int sr_scene_destroy(SrScene* scene);
/* Replaces Scene.SetSky(new SkyTexture(texture, multiplier, rotYaw)) scene.cs:543-551,389-404. */
SR_API int sr_scene_set_sky_texture(SrScene* scene, int32_t texture, float multiplier, float rot_yaw);
/* Replaces Scene.SetSky(new SkyProcedural(...)) scene.cs:543-551,334-356. */
SR_API int sr_scene_set_sky_procedural(SrScene* scene, const SrSkyProcedural* sky);
/* Replaces Scene.SetFog(Fog) scene.cs:553-561. */
SR_API int sr_scene_set_fog(SrScene* scene, const SrFog* fog);
/* Replaces Scene.AddObject(new Object(name, transform, material, shape)) scene.cs:563-571,214-225.
 * out_index receives the object index (the order of AddObject calls). */
SR_API int sr_scene_add_object(SrScene* scene, const SrTransform* transform, const SrMaterial* material,
                               const SrShape* shape, int32_t* out_index);
/* Builds the scene BVH over objects (32 bins, intersect cost 10) and uploads the scene.
 * Replaces Scene.Build scene.cs:517-541 (same errors: a sky is required). */
SR_API int sr_scene_build(SrScene* scene);
SR_API int sr_scene_bvh_size(SrScene* scene, uint32_t* node_count, uint32_t* item_count);
SR_API int sr_scene_bvh_export(SrScene* scene, float* node_bounds, int32_t* node_links, int32_t* items);

/* Closest hit of `count` world rays (origin xyz, dir xyz; dir unit length) on the GPU, host
 * buffers in and out.  Outputs per ray: object index (-1 = miss), triangle index within the
 * object's mesh (-1 for analytic shapes), world distance, barycentric u, v.  Replaces the
 * traversal of Scene.Trace (scene.cs:602-625 -> Bvh.Intersect bvh.cs:165-216 ->
 * Mesh.Intersect mesh.cs:51-62 -> TriangleLean.Intersect math.cs:1407-1435); used for the
 * bit-exact hit parity test.  The traversal is the wavefront renderer's persistent loop, or, in
 * the megakernel render mode (sr_scene_set_render_mode), the megakernel's per-ray traversal. */
SR_API int sr_scene_trace(SrScene* scene, const float* rays, uint32_t count, int32_t* out_object,
                          int32_t* out_triangle, float* out_dist, float* out_uv);

/* ---- rendering --------------------------------------------------------------------------- */
/* Renders the full image and copies the AOVs into the caller's host arrays (any of the seven
 * pointers may be NULL to skip that plane).  Replaces `new Renderer(...)` + the Tick() loop
 * until Step == Total (renderer.cs:40-151) and reading its public AOV arrays. */
SR_API int sr_render(SrScene* scene, const SrView* view, const SrRenderParams* params, const SrAovs* host_out);
/* Same, writing device arrays (all seven required, each width*height entries) on `stream`
 * (a cudaStream_t, NULL = the context stream).  Asynchronous: returns after the launches. */
SR_API int sr_render_device(SrScene* scene, const SrView* view, const SrRenderParams* params,
                            const SrAovs* device_out, void* stream);
/* Render + Compose in one call, the program.cs flow (program.cs:159-202 then 276-282): renders on
 * the device, denoises/tonemaps there, and copies back the RGB8 image (host_rgb8, width*height*3
 * bytes, may be NULL) and whichever AOV planes host_aovs requests (host_aovs or any plane may be
 * NULL).  Replaces `new Renderer(...)`, the Tick() loop and Compositor.Compose. */
SR_API int sr_render_compose(SrScene* scene, const SrView* view, const SrRenderParams* params,
                             const SrComposeParams* compose, const SrAovs* host_aovs, uint8_t* host_rgb8);
/* Render implementation used by this scene's renders (no reference counterpart; all produce the
 * same image): SR_RENDER_MEGAKERNEL = one thread per pixel running the whole sample loop;
 * SR_RENDER_WAVEFRONT = per-bounce extend/shade/resolve kernels driven by a host loop;
 * SR_RENDER_WAVEFRONT_GRAPH = the same kernels repeated on the device by a CUDA-graph
 * conditional loop (no host round trip per bounce).  SR_RENDER_AUTO picks the fastest (graph). */
enum { SR_RENDER_AUTO = 0, SR_RENDER_MEGAKERNEL = 1, SR_RENDER_WAVEFRONT = 2, SR_RENDER_WAVEFRONT_GRAPH = 3 };
SR_API int sr_scene_set_render_mode(SrScene* scene, int32_t mode);
/* Kernel launches and wavefront bounce iterations of the last completed render on this scene
 * (synchronises with it).  No reference counterpart. */
SR_API int sr_scene_render_info(SrScene* scene, uint32_t* kernel_launches, uint32_t* bounce_iterations);
/* Reads the work counters of the last render on this scene (device counting is enabled by
 * sr_scene_set_counting); counters_out has SR_COUNTER_COUNT entries. */
SR_API int sr_scene_set_counting(SrScene* scene, int32_t enabled);
SR_API int sr_scene_counters(SrScene* scene, uint64_t* counters_out);
/* Traversal-kernel timing (no reference counterpart; the reference's Counters.TimeRender times
 * whole renders): with timing enabled, a render in SR_RENDER_WAVEFRONT mode (the host loop)
 * records CUDA events on its stream right before and after every bounce's traversal kernel.
 * sr_scene_trace_time (synchronises) returns their summed duration in milliseconds and the number
 * of traversal launches of the last such render or adjoint replay; 0 and 0 when the last render
 * ran in another mode or without timing.  Other kernels of a bounce may run beside the traversal
 * kernel on parallel branches, as in an untimed render. */
SR_API int sr_scene_set_kernel_timing(SrScene* scene, int32_t enabled);
SR_API int sr_scene_trace_time(SrScene* scene, float* total_ms, uint32_t* launches);

/* ---- compositing ------------------------------------------------------------------------- */
/* Joint bilateral denoise + fog blur + tonemap to RGB8 (width*height*3 bytes), host AOVs in,
 * host pixels out.  Replaces Compositor.Compose compose.cs:74-99 (Filter :101-204,
 * FilterFog :206-245, Tonemap :247-266, Color.ToPixel math.cs:127-136). */
SR_API int sr_compose(SrContext* ctx, const SrAovs* host_aovs, uint32_t width, uint32_t height,
                      const SrComposeParams* params, uint8_t* host_rgb8);
/* Filter + FilterFog without the tonemap: the denoised linear radiance + fog (the colour that
 * Tonemap receives, compose.cs:93) into `device_linear` (width*height*3 floats), and the RGB8
 * image into `device_rgb8` too unless it is NULL.  Device AOVs as sr_compose_device, on `stream`. */
SR_API int sr_compose_float_device(SrContext* ctx, const SrAovs* device_aovs, uint32_t width, uint32_t height,
                                   const SrComposeParams* params, float* device_linear, uint8_t* device_rgb8,
                                   void* stream);
/* Same on device buffers (radiance, radiance_fog, normals, depth, variance are read) on `stream`. */
SR_API int sr_compose_device(SrContext* ctx, const SrAovs* device_aovs, uint32_t width, uint32_t height,
                             const SrComposeParams* params, uint8_t* device_rgb8, void* stream);
/* sr_compose_device that allocates no device memory: for hosts that cannot allocate when they
 * composite (a service whose device memory is fully committed to its own pools under a quota, a
 * latency-critical loop that cannot afford cudaMalloc's device-wide synchronisation).  No
 * counterpart in the reference.  Its scratch is a fixed
 * 32 MiB device array that every GPU loading the library holds until the process exits; the image
 * is filtered in row bands, and a call fails with SR_ERR_INVALID_ARG when one band with its filter
 * halo does not fit, i.e. when (2 * max(radius, fog radius) + 2) * width * 48 bytes > 32 MiB.
 * The first call on a device looks up the array's address there (make that first call before any
 * stream capture).  All calls share the array: calls that overlap on the GPU race and corrupt each
 * other's images, so run them one after another.  Spatial weights are evaluated per tap on the
 * device, so results can differ from sr_compose_device by one code value in rare pixels. */
SR_API int sr_compose_device_static(SrContext* ctx, const SrAovs* device_aovs, uint32_t width, uint32_t height,
                                    const SrComposeParams* params, uint8_t* device_rgb8, void* stream);
/* Tonemap of radiance + radiance_fog without denoise.  Replaces Compositor.Preview compose.cs:57-65. */
SR_API int sr_preview(SrContext* ctx, const SrAovs* host_aovs, uint32_t width, uint32_t height,
                      const SrComposeParams* params, uint8_t* host_rgb8);

/* Renderer.Tick (renderer.cs:98-105) without blocking: (finished pixels, pixels) of the scene's
 * last render launch (sr_render_device, sr_render_compose, sr_render_batch; sr_render returns
 * finished).  The wavefront renderer publishes the count every two bounces; the megakernel render
 * mode reports 0 until it completes.  Never waits for the GPU. */
SR_API int sr_render_progress(SrScene* scene, uint32_t* done, uint32_t* total);

/* Batched rendering (no counterpart in the reference, which renders one scene at a time): `count`
 * distinct built scenes of one context, each with its view, parameters and device AOV planes
 * (as sr_render_device), rendered by one CUDA graph launch on `stream` that holds one bounce
 * loop per scene, run side by side.  Each scene's AOVs equal what sr_render_device gives it.  The
 * graph is kept on the context and reused while the batch's scenes, views, parameters and
 * buffers stay the same. */
SR_API int sr_render_batch(SrScene* const* scenes, const SrView* views, const SrRenderParams* params,
                           const SrAovs* device_outs, uint32_t count, void* stream);

/* Random-number stream of the scene's renders and adjoints (an extension; the reference seeds
 * Rng(x, y) per pixel): 0, the default, is the reference's stream; any other value gives every
 * pixel an independent stream, e.g. fresh samples for each step of stochastic inverse rendering or
 * for progressive accumulation.  An adjoint replays the stream the scene has when it runs. */
SR_API int sr_scene_set_seed(SrScene* scene, uint32_t seed);
/* The scene's current random-number stream (what sr_scene_set_seed last set; 0 by default), e.g.
 * for a wrapper that must replay a render with the stream it was made with. */
SR_API int sr_scene_get_seed(SrScene* scene, uint32_t* seed);

/* Launch geometry of the wavefront kernels (no counterpart in the reference): threads per block of
 * the traversal kernel (64, 128 or 256; 0 = 128), blocks per SM of the traversal, fog-shade and
 * surface-shade kernels (0 = as many as fit; never more) and the live-path count slots /
 * tail_divisor at which the tail kernel takes over (0 = the built-in 16).  Results do not depend
 * on it.
 * Two loop caps (0 = the built-in runaway guards) bound the work of one render: the iterations of
 * the wavefront bounce loop and the actions (node visits, leaf steps) of one traversal.  A render
 * or trace that reaches either ends early and returns SR_ERR_DEVICE naming the loop cap (error
 * word 2); the kernels return normally and the context stays usable.  The reference has no such
 * guard (its Tick loop waits without a timeout, renderer.cs:98-105); lowering them is how failure
 * detection is exercised without a fault. */
typedef struct SrTuning {
    int32_t trace_blocks_per_sm;
    int32_t fog_shade_blocks_per_sm;
    int32_t surface_shade_blocks_per_sm;
    uint32_t tail_divisor;
    float ms;          /* sr_scene_autotune: trial render time of the chosen setting */
    float default_ms;  /* sr_scene_autotune: trial render time of the defaults */
    uint32_t max_bounce_iterations; /* wavefront bounce-loop cap (0 = (max_samples + 1) * (bounces + 2) * 2 + 8) */
    uint32_t max_traversal_steps;   /* per-traversal action cap (0 = 2^24) */
    uint32_t trace_block_threads;   /* traversal kernel block size: 64, 128 or 256 (0 = 128) */
    uint32_t max_slots;             /* path slots in flight, the wavefront queues' capacity, rounded up to
                                     * 32 (0 = one per pixel).  With fewer slots than pixels a slot takes
                                     * the next unclaimed pixel when its pixel is done: less path-state
                                     * memory, fewer paths per bounce; results are unchanged.  Not applied
                                     * to sr_render_checkpointed (its vertices are indexed by slot). */
} SrTuning;
SR_API int sr_scene_set_tuning(SrScene* scene, const SrTuning* tuning); /* NULL = defaults */
SR_API int sr_scene_get_tuning(SrScene* scene, SrTuning* tuning);
/* Autotuner: renders `params` at trial_spp samples per pixel under candidate launch geometries, one
 * dimension after another from the defaults -- traversal block size (128, 64, 256), traversal
 * blocks per SM (all that fit, one or two fewer), fog-shade blocks per SM (all, two fewer), tail
 * hand-over (slots / 16, 8, 32), slot capacity (every pixel, a half, a quarter) -- keeping the
 * fastest of each, and leaves the result on the scene
 * (ms: its trial time; default_ms: the defaults').  The BVH node width is not a dimension: the
 * traversal walks the reference's binary tree, whose child order the bit-exact hits rest on. */
SR_API int sr_scene_autotune(SrScene* scene, const SrView* view, const SrRenderParams* params, uint32_t trial_spp,
                             SrTuning* chosen);

/* ---- derivatives (no counterpart in the reference, which renders forward only) ------------- */
/* Path-replay adjoint: for the image I = radiance + radiance_fog that sr_render_device produced
 * with the same scene, view and params (`forward`: its radiance, radiance_fog and samples planes,
 * device pointers) and the gradient d_image = dL/dI of any loss L (device, width x height x 3;
 * for L = sum (I - target)^2 it is 2 (I - target)), ADDS dL/d(texels of albedo texture
 * `texture`) into `grad` (device, texture width x height x 3).  `replay` (device, width x height x 3,
 * may be NULL) receives the replayed image, which equals I.  Sampled directions, roulette
 * decisions, pdfs and MIS weights are held fixed (detached); the BRDF values and scatter weights
 * are differentiated.  Scenes with transparent materials and params->bounces > 16 are refused.
 * Runs asynchronously on `stream`. */
SR_API int sr_adjoint_albedo(SrScene* scene, const SrView* view, const SrRenderParams* params,
                             const SrAovs* forward, const float* d_image, int32_t texture, float* grad,
                             float* replay, void* stream);
/* The same for SR_ADJOINT_ALBEDO (a texture as the colour lookup; the gradient fills all three
 * channels), SR_ADJOINT_ROUGHNESS (a texture as the roughness lookup, which reads the red channel;
 * the gradient fills channel 0) or SR_ADJOINT_FOG_DENSITY (the scene's fog density; `texture` is
 * ignored and `grad` is one float).  The roughness moves the sampled specular directions and the
 * density the sampled scatter distances, so for these two the detached gradient is the derivative
 * of the expected image (score terms for the density), not of each sample. */
enum { SR_ADJOINT_ALBEDO = 0, SR_ADJOINT_ROUGHNESS = 1, SR_ADJOINT_FOG_DENSITY = 2 };
SR_API int sr_adjoint_texture(SrScene* scene, const SrView* view, const SrRenderParams* params,
                              const SrAovs* forward, const float* d_image, int32_t texture, int32_t parameter,
                              float* grad, float* replay, void* stream);
/* All three from one replay (one kernel launch instead of three): the albedo texture's gradient
 * into albedo_grad, the roughness texture's into roughness_grad (channel 0) and the fog density's
 * into fog_density_grad[0]; a NULL gradient skips its part. */
SR_API int sr_adjoint_all(SrScene* scene, const SrView* view, const SrRenderParams* params, const SrAovs* forward,
                          const float* d_image, int32_t albedo_texture, float* albedo_grad, int32_t roughness_texture,
                          float* roughness_grad, float* fog_density_grad, float* replay, void* stream);
/* How the adjoint entry points above replay a render's paths (no reference counterpart):
 * SR_ADJOINT_REPLAY_WAVEFRONT (the default) renders them again with the wavefront kernels -- the
 * same traversal, event queues and shading as sr_render_device -- recording each sample's path
 * vertices in a device buffer (slots x (bounces + 1) x 128 bytes) and sweeping them back into the
 * gradients when the sample ends; SR_ADJOINT_REPLAY_PIXEL replays each pixel's samples in one
 * thread.  Both give the same gradients up to the order of float additions. */
enum { SR_ADJOINT_REPLAY_WAVEFRONT = 0, SR_ADJOINT_REPLAY_PIXEL = 1 };
SR_API int sr_scene_set_adjoint_replay(SrScene* scene, int32_t form);
/* Path-vertex checkpointing (no reference counterpart): sr_render_device that also keeps every
 * sample's path vertices on the device, so that sr_adjoint_checkpointed can differentiate this
 * image without tracing it again.  The vertices take slots x max_samples x (bounces + 1) x 128 bytes
 * (slots: width x height rounded up to 8 x 4 tiles), reported in *bytes_kept (may be NULL), and stay
 * until the next checkpointed render or sr_scene_release_checkpoint.  The gradients are those of the
 * rendered samples themselves (replay with another seed decorrelates them instead). */
SR_API int sr_render_checkpointed(SrScene* scene, const SrView* view, const SrRenderParams* params,
                                  const SrAovs* device_out, void* stream, uint64_t* bytes_kept);
/* The adjoint of the last checkpointed render's image for dL/dI = d_image (device, width x height x 3):
 * adds the gradients as sr_adjoint_all does, sweeping the kept vertices (no traversal).  That
 * render's output planes must still hold it (its sample counts are read). */
SR_API int sr_adjoint_checkpointed(SrScene* scene, const float* d_image, int32_t albedo_texture, float* albedo_grad,
                                   int32_t roughness_texture, float* roughness_grad, float* fog_density_grad,
                                   void* stream);
/* Frees the vertices kept by sr_render_checkpointed. */
SR_API int sr_scene_release_checkpoint(SrScene* scene);
/* Sets the fog density of a built scene with fog (> 0), e.g. one step of inverse rendering. */
SR_API int sr_scene_update_fog_density(SrScene* scene, float density);
/* Replaces the texels of texture `texture` (rgb floats, its width x height) in a built scene's
 * device copy, e.g. one step of inverse rendering.  The context's texture and other scenes are left
 * as they are.  The scene's sky texture is refused (its light distribution is built from it). */
SR_API int sr_scene_update_texture(SrScene* scene, int32_t texture, const float* texels_rgb);
/* The same from device memory, asynchronously on `stream`. */
SR_API int sr_scene_update_texture_device(SrScene* scene, int32_t texture, const float* d_texels_rgb,
                                          void* stream);

/* ---- asset ingest (host-side file parsing) ------------------------------------------------- */
/* Image.Load (image.cs:214-273: uncompressed 24-bit TrueColor / 8-bit Grayscale .tga, rows top-down)
 * or ImageHdr.Load (image.cs:307-382: Radiance .hdr, "-Y h +X w", new-style RLE or flat): sizes
 * always; pixels (RGB8, or RGBE8 for .hdr: `channels` 3 or 4) when `pixels` is non-NULL and
 * `capacity` suffices.  Parse failures return SR_ERR_IO with the reference's message. */
SR_API int sr_image_load(const char* path, uint32_t* width, uint32_t* height, uint32_t* channels, uint8_t* pixels,
                         uint64_t capacity);
/* Texture.FromSrgb / FromLinear (Image.Load(path)) or FromHdr(ImageHdr.Load(path), max_luminance)
 * (texture.cs:138-163) as a texture of the context (filter and tiling as sr_texture_create). */
SR_API int sr_texture_load(SrContext* ctx, const char* path, int32_t encoding, float max_luminance, int32_t filter,
                           float tiling_x, float tiling_y, int32_t* out_id);
/* ObjLoader.Load(path, scene, config) obj.cs:139-259: parses the OBJ and its mtllib files (MTL
 * textures via sr_texture_load rules), makes one mesh + object per `o`/`g`/`usemtl` group with the
 * reference's names ("<file>_<name>" or "<file>_<n>"), triangle fans, V flipped, smooth normals
 * when the file has no `vn` and smooth_normals is set.  `transform` NULL = identity; `material`
 * NULL = Material(White, 1) for groups without an MTL material.  Unlike the reference, a parse error
 * adds nothing to the scene. */
SR_API int sr_obj_load(SrScene* scene, const char* path, const SrTransform* transform, const SrMaterial* material,
                       int32_t smooth_normals, uint32_t* objects_added);
/* Inspection (no reference counterpart): a texture's texels (3 floats each), a mesh's triangles,
 * a scene object's description and name (objects from sr_obj_load are named). */
SR_API int sr_texture_export(SrContext* ctx, int32_t texture, uint32_t* width, uint32_t* height, float* texels);
SR_API int sr_mesh_export(SrContext* ctx, int32_t mesh, uint32_t* count, SrTriangle* triangles);
SR_API int sr_scene_object_count(SrScene* scene, uint32_t* count);
SR_API int sr_scene_object_info(SrScene* scene, uint32_t index, SrTransform* transform, SrMaterial* material,
                                SrShape* shape, char* name, uint32_t name_capacity);

/* ---- AOV images, debug overlay, image files ------------------------------------------------ */
/* AOV visualisations of program.cs:211-263 (the normal.bmp / depth.bmp / variance.bmp /
 * samples.bmp / uv.bmp dumps) as RGB8: normal (n * 0.5 + 0.5) * 255; depth clamp(d / 25) * 255 grey,
 * red where infinite; variance clamp(v / (2 * variance_threshold)) * 255 grey; samples
 * log2(s / min) / log2(max / min) * 255 grey; uv |uv mod 1| * 255 in red and green.  Float to byte
 * conversions follow .NET 8: truncation, low 8 bits, 0 for NaN and values outside the int range. */
enum { SR_AOV_NORMAL = 0, SR_AOV_DEPTH = 1, SR_AOV_VARIANCE = 2, SR_AOV_SAMPLES = 3, SR_AOV_UV = 4 };
typedef struct SrAovImageParams {
    float variance_threshold; /* SR_AOV_VARIANCE */
    uint32_t min_samples;     /* SR_AOV_SAMPLES */
    uint32_t max_samples;
} SrAovImageParams;
SR_API int sr_aov_image(SrContext* ctx, const SrAovs* host_aovs, uint32_t width, uint32_t height, int32_t kind,
                        const SrAovImageParams* params, uint8_t* host_rgb8);
SR_API int sr_aov_image_device(SrContext* ctx, const SrAovs* device_aovs, uint32_t width, uint32_t height,
                               int32_t kind, const SrAovImageParams* params, uint8_t* device_rgb8, void* stream);

/* Overlay.Draw (overlay.cs:54-96): world-space lines (Bresenham, perspective-correct depth test
 * against the render's depth with a relative bias, overlay.cs:102-149) and text (8x8 bitmap font,
 * '\n' separated lines, top-left or centred, overlay.cs:151-196) drawn into an RGB8 image.  The
 * reference's draw order holds: every line, then every world-space text, then every screen-space
 * text, each in array order; later entries overwrite earlier ones.  Text is one byte per character;
 * characters outside the font's range are skipped but count for centring.  The font is the
 * caller's: `glyphs` holds 8 bytes per character from first_char to last_char, one byte per row
 * top to bottom, the most significant bit leftmost (the reference's Font table layout; no font
 * ships with the library).  Lines whose projected end points lie outside the int range or that
 * span more than 2^24 pixels fail with SR_ERR_INVALID_ARG. */
enum { SR_ALIGN_TOP_LEFT = 0, SR_ALIGN_CENTER = 1 };
typedef struct SrOverlayLine {
    float a[3], b[3];
    float color[3];     /* linear colour, encoded with Color.ToPixel */
    int32_t depth_test; /* 1: hidden behind nearer surfaces of the depth plane */
    float depth_bias;   /* fraction of the depth pulled towards the camera (reference default 0.005) */
} SrOverlayLine;
typedef struct SrOverlayText {
    const char* text;      /* NUL-terminated */
    int32_t in_world;      /* 1: world_pos projected through the view; 0: screen_pos in pixels */
    float world_pos[3];
    int32_t screen_pos[2];
    float color[3];
    int32_t align;         /* SR_ALIGN_*; the reference defaults to centred in world, top-left on screen */
} SrOverlayText;
typedef struct SrFont {
    const uint8_t* glyphs;
    int32_t first_char, last_char;
} SrFont;
SR_API int sr_overlay_draw(SrContext* ctx, uint8_t* host_rgb8, uint32_t width, uint32_t height, const SrView* view,
                           const float* host_depth, const SrOverlayLine* lines, uint32_t line_count,
                           const SrOverlayText* texts, uint32_t text_count, const SrFont* font);
/* Same on a device image and depth plane (depth may be NULL: no depth test) on `stream`. */
SR_API int sr_overlay_draw_device(SrContext* ctx, uint8_t* device_rgb8, uint32_t width, uint32_t height,
                                  const SrView* view, const float* device_depth, const SrOverlayLine* lines,
                                  uint32_t line_count, const SrOverlayText* texts, uint32_t text_count,
                                  const SrFont* font, void* stream);
/* Image.Save (image.cs:88-212): RGB8 rows top-down written as .tga (24-bit, top-left origin), .ppm
 * (P6) or .bmp (24-bit, top-down, rows padded to 4 bytes) by the path's extension; other
 * extensions or write failures return SR_ERR_IO. */
SR_API int sr_image_save(const char* path, uint32_t width, uint32_t height, const uint8_t* rgb8);

#ifdef __cplusplus
}
#endif

#endif /* SHARPRAY_H */

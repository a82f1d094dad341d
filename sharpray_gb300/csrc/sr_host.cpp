// sr_host.cpp — the C ABI (include/sharpray.h): contexts, textures, meshes, scene build and
// upload, render and compose entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sharpray.h"
#include "sr_bvh.h"
#include "sr_bvh_build.h"
#include "sr_image.h"
#include "sr_ingest.h"
#include "sr_kernels.h"
#include "sr_layout.h"
#include "sr_wavefront.h"

using namespace sr;
using namespace sr::host;

namespace {

thread_local std::string g_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    int code = e == cudaErrorMemoryAllocation ? SR_ERR_OUT_OF_MEMORY : SR_ERR_CUDA;
    return fail(code, "%s: %s", what, cudaGetErrorString(e));
}

#define SR_CUDA(call, what)                          \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

// Owning device buffer.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    cudaError_t reserve(size_t n) {
        if (n <= bytes) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    template <typename T>
    T* as() const {
        return (T*)ptr;
    }
};

cudaError_t upload(DevBuf& buf, const void* src, size_t bytes, cudaStream_t s) {
    cudaError_t e = buf.reserve(bytes > 0 ? bytes : 16);
    if (e != cudaSuccess) return e;
    if (bytes) e = cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyHostToDevice, s);
    return e;
}

struct TextureHost {
    uint32_t width, height;
    int32_t filter;
    float tiling_x, tiling_y;
    std::vector<float> texels;  // rgb
    float texel_lum(uint32_t x, uint32_t y) const {
        const float* t = &texels[((size_t)y * width + x) * 3];
        return 0.2126f * t[0] + 0.7152f * t[1] + 0.0722f * t[2];
    }
};

struct MeshHost {
    std::vector<SrTriangle> tris;
    BvhHost bvh;
    Box bounds;
};

}  // namespace

struct SrContext {
    int device = 0;
    cudaStream_t stream = nullptr;
    int32_t bvh_build = SR_BVH_BUILD_HOST;
    std::vector<std::unique_ptr<TextureHost>> textures;
    std::vector<std::unique_ptr<MeshHost>> meshes;
    // compose resources
    DevBuf compose_scratch, compose_tables, compose_io;
    std::vector<float> table_host;
    // AOV images and overlay (host-buffer entry points stage through image_io)
    DevBuf image_io, overlay_scratch;
    // batched rendering: the graph of the last batch and the launch descriptions baked into it
    cudaStream_t batch_capture = nullptr;
    cudaGraphExec_t batch_exec = nullptr;
    std::vector<WaveLaunch> batch_launch;
    // live scenes; sr_ctx_destroy with scenes still alive only marks the context closed, and the
    // last sr_scene_destroy frees it (finalisers may run in any order)
    std::vector<SrScene*> scenes;
    bool closed = false;
};

struct SrScene {
    SrContext* ctx;
    // description
    struct Obj {
        SrTransform tr;
        SrMaterial mat;
        SrShape shape;
        Box bounds;
    };
    std::vector<Obj> objects;
    std::vector<std::string> object_names;  // names of objects from sr_obj_load (others empty)
    int sky_kind = -1;
    int32_t sky_texture = -1;
    float sky_multiplier = 1, sky_yaw = 0;
    SrSkyProcedural sky_proc{};
    bool has_fog = false;
    SrFog fog{};
    bool built = false;
    BvhHost tlas;
    // device state
    DevScene dev{};
    DevBuf nodes, tris, attrs, objs, mats, texs, texels, cdf_marginal, cdf_cond, guide_marginal, guide_cond, sky_center;
    DevBuf err, counters;
    DevBuf aovs;  // staging for sr_render
    DevBuf rays_io;
    bool counting = false;
    uint64_t last_counters[SR_COUNTER_COUNT] = {};
    // wavefront renderer state
    int32_t render_mode = SR_RENDER_AUTO;
    DevBuf wave;
    uint32_t wave_slots = 0;
    WaveState ws[kWaveGroups]{};
    cudaStream_t capture_stream = nullptr;
    cudaStream_t side_streams[kSideStreams] = {};  // a bounce's parallel branches (or groups 1..)
    cudaEvent_t fork_events[kForkEvents] = {};      // forks and joins
    cudaGraphExec_t graph_exec = nullptr;
    WaveLaunch graph_launch{};  // launch parameters baked into graph_exec
    uint32_t* counts_host = nullptr;  // pinned
    // render progress (sr_render_progress): finished pixels published by the device loop into a
    // host-mapped word, and an event after the last render's launches
    uint32_t* progress_host = nullptr;
    uint32_t* progress_dev = nullptr;
    cudaEvent_t progress_event = nullptr;
    uint32_t progress_total = 0;
    int sms = 0;
    WaveTune tune{};  // launch geometry (sr_scene_set_tuning / sr_scene_autotune)
    uint32_t seed = 0;  // random-number stream of renders and adjoints (sr_scene_set_seed)
    DevBuf tune_aovs;  // autotune's scratch AOV planes
    std::vector<uint64_t> tex_offset;  // first texel of each texture in `texels` (textures present at build)
    DevBuf tex_stage;                   // sr_scene_update_texture staging
    int last_mode = 0;                // render mode of the last render
    uint32_t last_host_iters = 0;     // bounces run by the host loop
    bool last_tail = false;           // the host loop launched the tail kernel
    // traversal-kernel timing of host-loop renders (sr_scene_set_kernel_timing)
    bool kernel_timing = false;
    cudaEvent_t trace_ev[2] = {};
    double trace_ms = 0.0;         // summed duration of the last host-loop render's traversal kernels
    uint32_t trace_launches = 0;   // ... and their number
    // adjoint passes of the wavefront kernels (sr_wave_adjoint.cu)
    int32_t adjoint_replay = SR_ADJOINT_REPLAY_WAVEFRONT;  // sr_scene_set_adjoint_replay
    DevBuf adj_vbuf, adj_pass;     // replay: vertex records (one sample per slot), the device AdjPass
    DevBuf ckpt_vbuf, ckpt_vcount, ckpt_pass_dev;  // record: every sample's vertex records and counts
    cudaGraphExec_t adj_graph_exec = nullptr;
    WaveLaunch adj_graph_launch{};
    // the last checkpointed render (sr_render_checkpointed), swept by sr_adjoint_checkpointed
    bool ckpt_valid = false;
    WaveLaunch ckpt_launch{};
    AdjPass ckpt_pass{};
    ~SrScene() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (adj_graph_exec) cudaGraphExecDestroy(adj_graph_exec);
        if (capture_stream) cudaStreamDestroy(capture_stream);
        for (cudaStream_t& st : side_streams)
            if (st) cudaStreamDestroy(st);
        for (cudaEvent_t& e : fork_events)
            if (e) cudaEventDestroy(e);
        if (counts_host) cudaFreeHost(counts_host);
        if (progress_host) cudaFreeHost(progress_host);
        if (progress_event) cudaEventDestroy(progress_event);
        for (cudaEvent_t& e : trace_ev)
            if (e) cudaEventDestroy(e);
    }
};

namespace {

F3 f3(const float* p) { return {p[0], p[1], p[2]}; }
Quat quat(const float* p) { return {p[0], p[1], p[2], p[3]}; }
float4 mk4(float x, float y, float z, float w) {
    float4 r;
    r.x = x, r.y = y, r.z = z, r.w = w;
    return r;
}
float ibits(int32_t v) {
    float f;
    std::memcpy(&f, &v, 4);
    return f;
}

// Bounds of a triangle from its lean form (TriangleLean.Bounds math.cs:1356-1362).
Box tri_bounds(const SrTriangle& t) {
    F3 a = f3(t.pos_a), b = a + f3(t.ab), c = a + f3(t.ac);
    return {{net_min(a.x, net_min(b.x, c.x)), net_min(a.y, net_min(b.y, c.y)), net_min(a.z, net_min(b.z, c.z))},
            {net_max(a.x, net_max(b.x, c.x)), net_max(a.y, net_max(b.y, c.y)), net_max(a.z, net_max(b.z, c.z))}};
}

// Object world bounds: AABox.Transform -> Box, then Box.Bounds (scene.cs:219-220,
// math.cs:960-961,1100-1113).
Box object_bounds(const SrTransform& tr, const Box& local) {
    F3 pos = f3(tr.pos), scale = f3(tr.scale);
    Quat rot = quat(tr.rot);
    F3 center = pos + rotate(rot, local.center() * scale);
    F3 size = local.size() * scale;
    Box oriented{center - size * 0.5f, center + size * 0.5f};
    F3 c = oriented.center();
    F3 h = oriented.size() * 0.5f;
    F3 ax = rotate(rot, {h.x, 0, 0}), ay = rotate(rot, {0, h.y, 0}), az = rotate(rot, {0, 0, h.z});
    F3 ext{std::fabs(ax.x) + std::fabs(ay.x) + std::fabs(az.x), std::fabs(ax.y) + std::fabs(ay.y) + std::fabs(az.y),
           std::fabs(ax.z) + std::fabs(ay.z) + std::fabs(az.z)};
    F3 full = ext * 2.0f;
    return {c - full * 0.5f, c + full * 0.5f};
}

void export_bvh(const BvhHost& b, float* bounds, int32_t* links, int32_t* items) {
    for (int i = 0; i < b.node_count; ++i) {
        const BvhNodeHost& n = b.nodes[i];
        float* o = bounds + (size_t)i * 6;
        o[0] = n.bounds.lo.x, o[1] = n.bounds.lo.y, o[2] = n.bounds.lo.z;
        o[3] = n.bounds.hi.x, o[4] = n.bounds.hi.y, o[5] = n.bounds.hi.z;
        if (links) links[2 * i] = n.child, links[2 * i + 1] = n.count;
    }
    if (items) std::memcpy(items, b.items.data(), b.items.size() * sizeof(int32_t));
}

// Appends one tree to the node slot array.  Slot base is kept even so node pairs (c, c+1) with c
// odd land on 64-byte boundaries; node i goes to slot base + 1 + i.  Leaves point at
// `leaf_base + child`, interior nodes (count == 0, including the zero-count leaves the reference
// can create) at `base + 1 + child`.  Returns the root slot.
int32_t append_tree(std::vector<float4>& slots, const BvhHost& b, int32_t leaf_base) {
    if (slots.size() % 4 != 0) slots.resize(slots.size() + 2);  // keep (base) even in node units
    int32_t base = (int32_t)(slots.size() / 2);
    slots.resize(slots.size() + 2);  // padding slot
    for (const BvhNodeHost& n : b.nodes) {
        int32_t child = n.count > 0 ? leaf_base + n.child : base + 1 + n.child;
        slots.push_back(mk4(n.bounds.lo.x, n.bounds.lo.y, n.bounds.lo.z, ibits(child)));
        slots.push_back(mk4(n.bounds.hi.x, n.bounds.hi.y, n.bounds.hi.z, ibits(n.count)));
    }
    return b.node_count > 0 ? base + 1 : -1;
}

// Reference search (Cdf1.Sample cdf.cs:37-55) without the final clamp: #{j : cdf[j+1] <= u}.
uint32_t cdf_lower_bound(const float* cdf, uint32_t n, float u) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (cdf[mid + 1] <= u)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Bucket guide of one Cdf1 for the device search: guide[k] = lower bound at the smallest float u
// with (int)(u * n) >= k; guide[n] = n.
void build_guide(const float* cdf, uint32_t n, uint32_t* guide) {
    const float fn = (float)n;
    guide[0] = cdf_lower_bound(cdf, n, 0.0f);
    for (uint32_t k = 1; k < n; ++k) {
        float f = (float)((double)k / (double)n);
        while (f > 0.0f && (int)(f * fn) >= (int)k) f = std::nextafter(f, 0.0f);
        while ((int)(f * fn) < (int)k) f = std::nextafter(f, 2.0f);
        guide[k] = cdf_lower_bound(cdf, n, f);
    }
    guide[n] = n;
}

bool valid_texture(SrContext* ctx, int32_t id) { return id == -1 || (id >= 0 && id < (int32_t)ctx->textures.size()); }

}  // namespace

extern "C" {

SR_API const char* sr_version(void) { return "sharpray-gb300 0.1 (sm_103a)"; }
SR_API const char* sr_last_error_message(void) { return g_error.c_str(); }

SR_API int sr_ctx_create(int device, SrContext** out_ctx) {
    if (!out_ctx) return fail(SR_ERR_INVALID_ARG, "sr_ctx_create: out_ctx is NULL");
    if (device == -1) {  // host-only context: ingest and BVH builds, no device work
        auto ctx = std::make_unique<SrContext>();
        ctx->device = -1;
        *out_ctx = ctx.release();
        return SR_OK;
    }
    int n = 0;
    SR_CUDA(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (device < 0 || device >= n) return fail(SR_ERR_INVALID_ARG, "sr_ctx_create: device %d out of range (%d)", device, n);
    SR_CUDA(cudaSetDevice(device), "cudaSetDevice");
    auto ctx = std::make_unique<SrContext>();
    ctx->device = device;
    SR_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    *out_ctx = ctx.release();
    return SR_OK;
}

static void ctx_free(SrContext* ctx) {
    if (ctx->device >= 0) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        if (ctx->batch_exec) cudaGraphExecDestroy(ctx->batch_exec);
        if (ctx->batch_capture) cudaStreamDestroy(ctx->batch_capture);
        cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
}

SR_API int sr_ctx_destroy(SrContext* ctx) {
    if (!ctx) return SR_OK;
    ctx->closed = true;
    if (ctx->scenes.empty()) ctx_free(ctx);
    return SR_OK;
}

// A BVH built where `where` says (device builds need a device context); bit-identical either way.
static int build_tree(SrContext* ctx, const std::vector<Box>& bounds, float ct, float ci, int bins, int32_t where,
                      BvhHost& out) {
    if (where == SR_BVH_BUILD_DEVICE) {
        if (ctx->device < 0) return fail(SR_ERR_STATE, "device BVH build on a host-only context");
        SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
        SR_CUDA(build_bvh_device(bounds, ct, ci, bins, ctx->stream, out), "device BVH build");
    } else {
        out = build_bvh(bounds, ct, ci, bins);
    }
    if (out.overflow) return fail(SR_ERR_INVALID_ARG, "BVH needs more than 2N nodes (degenerate bounds)");
    return SR_OK;
}

SR_API int sr_ctx_set_bvh_build(SrContext* ctx, int32_t where) {
    if (!ctx) return fail(SR_ERR_INVALID_ARG, "context is NULL");
    if (where != SR_BVH_BUILD_HOST && where != SR_BVH_BUILD_DEVICE) return fail(SR_ERR_INVALID_ARG, "bad BVH build %d", where);
    if (where == SR_BVH_BUILD_DEVICE && ctx->device < 0) return fail(SR_ERR_STATE, "host-only context has no device");
    ctx->bvh_build = where;
    return SR_OK;
}

SR_API int sr_bvh_build(SrContext* ctx, const float* bounds, uint32_t count, float cost_traverse, float cost_intersect,
                        int32_t bins, int32_t where, float* node_bounds, int32_t* node_links, int32_t* items,
                        uint32_t* node_count) {
    if (!ctx || (!bounds && count) || !node_bounds || !node_count) return fail(SR_ERR_INVALID_ARG, "sr_bvh_build: NULL argument");
    if (bins < 2 || bins > 32) return fail(SR_ERR_INVALID_ARG, "sr_bvh_build: bins must be 2..32");
    if (where != SR_BVH_BUILD_HOST && where != SR_BVH_BUILD_DEVICE) return fail(SR_ERR_INVALID_ARG, "bad BVH build %d", where);
    std::vector<Box> b(count);
    for (uint32_t i = 0; i < count; ++i) {
        const float* p = bounds + 6 * (size_t)i;
        b[i] = {{p[0], p[1], p[2]}, {p[3], p[4], p[5]}};
    }
    BvhHost t;
    if (int rc = build_tree(ctx, b, cost_traverse, cost_intersect, bins, where, t)) return rc;
    export_bvh(t, node_bounds, node_links, items);
    *node_count = (uint32_t)t.node_count;
    return SR_OK;
}

SR_API int sr_triangles_from_corners(const float* positions, const float* uvs, const float* normals, uint32_t count,
                                     int32_t smooth_normals, SrTriangle* out) {
    if ((!positions || !out) && count) return fail(SR_ERR_INVALID_ARG, "sr_triangles_from_corners: NULL array");
    triangles_from_corners(positions, uvs, normals, count, smooth_normals != 0, out);
    return SR_OK;
}

SR_API int sr_texture_create(SrContext* ctx, const float* texels_rgb, uint32_t width, uint32_t height, int32_t filter,
                             float tiling_x, float tiling_y, int32_t* out_id) {
    if (!ctx || !texels_rgb || !out_id) return fail(SR_ERR_INVALID_ARG, "sr_texture_create: NULL argument");
    if (width == 0 || height == 0) return fail(SR_ERR_INVALID_ARG, "sr_texture_create: empty texture");
    if (filter != 0 && filter != 1) return fail(SR_ERR_INVALID_ARG, "sr_texture_create: bad filter %d", filter);
    auto t = std::make_unique<TextureHost>();
    t->width = width;
    t->height = height;
    t->filter = filter;
    t->tiling_x = tiling_x;
    t->tiling_y = tiling_y;
    t->texels.assign(texels_rgb, texels_rgb + (size_t)width * height * 3);
    ctx->textures.push_back(std::move(t));
    *out_id = (int32_t)ctx->textures.size() - 1;
    return SR_OK;
}

SR_API int sr_mesh_create(SrContext* ctx, const SrTriangle* triangles, uint32_t count, int32_t* out_id) {
    if (!ctx || (!triangles && count) || !out_id) return fail(SR_ERR_INVALID_ARG, "sr_mesh_create: NULL argument");
    auto m = std::make_unique<MeshHost>();
    m->tris.assign(triangles, triangles + count);
    std::vector<Box> bounds(count);
    for (uint32_t i = 0; i < count; ++i) bounds[i] = tri_bounds(m->tris[i]);
    if (int rc = build_tree(ctx, bounds, 1.0f, 0.5f, 8, ctx->bvh_build, m->bvh)) return rc;  // mesh.cs:40-41
    m->bounds = m->bvh.node_count > 0 ? m->bvh.nodes[0].bounds : Box::inverted();
    ctx->meshes.push_back(std::move(m));
    *out_id = (int32_t)ctx->meshes.size() - 1;
    return SR_OK;
}

SR_API int sr_mesh_bvh_size(SrContext* ctx, int32_t mesh, uint32_t* node_count, uint32_t* item_count) {
    if (!ctx || mesh < 0 || mesh >= (int32_t)ctx->meshes.size()) return fail(SR_ERR_INVALID_ARG, "bad mesh id");
    if (node_count) *node_count = (uint32_t)ctx->meshes[mesh]->bvh.node_count;
    if (item_count) *item_count = (uint32_t)ctx->meshes[mesh]->bvh.items.size();
    return SR_OK;
}

SR_API int sr_mesh_bvh_export(SrContext* ctx, int32_t mesh, float* node_bounds, int32_t* node_links, int32_t* items) {
    if (!ctx || mesh < 0 || mesh >= (int32_t)ctx->meshes.size()) return fail(SR_ERR_INVALID_ARG, "bad mesh id");
    if (!node_bounds) return fail(SR_ERR_INVALID_ARG, "node_bounds is NULL");
    export_bvh(ctx->meshes[mesh]->bvh, node_bounds, node_links, items);
    return SR_OK;
}

SR_API int sr_scene_create(SrContext* ctx, SrScene** out_scene) {
    if (!ctx || !out_scene) return fail(SR_ERR_INVALID_ARG, "sr_scene_create: NULL argument");
    if (ctx->closed) return fail(SR_ERR_STATE, "context destroyed");
    SrScene* s = new SrScene();
    s->ctx = ctx;
    ctx->scenes.push_back(s);
    *out_scene = s;
    return SR_OK;
}

SR_API int sr_scene_destroy(SrScene* scene) {
    if (!scene) return SR_OK;
    SrContext* ctx = scene->ctx;
    if (ctx->device >= 0) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    if (ctx->batch_exec) {  // the cached batch graph may hold this scene's buffers
        cudaGraphExecDestroy(ctx->batch_exec);
        ctx->batch_exec = nullptr;
        ctx->batch_launch.clear();
    }
    delete scene;
    ctx->scenes.erase(std::find(ctx->scenes.begin(), ctx->scenes.end(), scene));
    if (ctx->closed && ctx->scenes.empty()) ctx_free(ctx);
    return SR_OK;
}

SR_API int sr_scene_set_sky_texture(SrScene* s, int32_t texture, float multiplier, float rot_yaw) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "scene is NULL");
    if (s->built) return fail(SR_ERR_STATE, "Scene already built");
    if (texture < 0 || texture >= (int32_t)s->ctx->textures.size()) return fail(SR_ERR_INVALID_ARG, "bad texture id");
    s->sky_kind = 0;
    s->sky_texture = texture;
    s->sky_multiplier = multiplier;
    s->sky_yaw = rot_yaw;
    return SR_OK;
}

SR_API int sr_scene_set_sky_procedural(SrScene* s, const SrSkyProcedural* sky) {
    if (!s || !sky) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (s->built) return fail(SR_ERR_STATE, "Scene already built");
    s->sky_kind = 1;
    s->sky_proc = *sky;
    return SR_OK;
}

SR_API int sr_scene_set_fog(SrScene* s, const SrFog* fog) {
    if (!s || !fog) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (s->built) return fail(SR_ERR_STATE, "Scene already built");
    if (!(fog->height_falloff >= 0.0f) || std::isinf(fog->height_falloff))
        return fail(SR_ERR_INVALID_ARG, "Fog height_falloff must be finite and >= 0");
    if (fog->height_falloff == 0.0f && !std::isfinite(fog->top_height))
        return fail(SR_ERR_INVALID_ARG,
                    "a homogeneous fog (height_falloff 0) needs a finite top_height: through an unbounded medium "
                    "no sky light reaches the scene");
    if (!(fog->density > 0.0f) || !std::isfinite(fog->density)) return fail(SR_ERR_INVALID_ARG, "Fog density must be > 0");
    if (!(fog->anisotropy > -1.0f && fog->anisotropy < 1.0f))
        return fail(SR_ERR_INVALID_ARG, "Fog anisotropy must be in (-1, 1)");
    s->has_fog = true;
    s->fog = *fog;
    return SR_OK;
}

SR_API int sr_scene_add_object(SrScene* s, const SrTransform* tr, const SrMaterial* mat, const SrShape* shape,
                               int32_t* out_index) {
    if (!s || !tr || !mat || !shape) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (s->built) return fail(SR_ERR_STATE, "Scene already built");
    SrContext* ctx = s->ctx;
    if (!valid_texture(ctx, mat->color_texture) || !valid_texture(ctx, mat->roughness_texture) ||
        !valid_texture(ctx, mat->metallic_texture) || !valid_texture(ctx, mat->normal_texture))
        return fail(SR_ERR_INVALID_ARG, "material references an unknown texture");
    if (tr->scale[0] == 0.0f || tr->scale[1] == 0.0f || tr->scale[2] == 0.0f)
        return fail(SR_ERR_INVALID_ARG, "Scale cannot be zero");
    Box local;
    switch (shape->kind) {
        case SR_SHAPE_MESH:
            if (shape->mesh < 0 || shape->mesh >= (int32_t)ctx->meshes.size()) return fail(SR_ERR_INVALID_ARG, "bad mesh id");
            local = ctx->meshes[shape->mesh]->bounds;
            break;
        case SR_SHAPE_SPHERE: {
            if (!(shape->params[3] > 0.0f)) return fail(SR_ERR_INVALID_ARG, "Radius must be positive");
            F3 c = f3(shape->params), r{shape->params[3], shape->params[3], shape->params[3]};
            local = {c - r, c + r};
            break;
        }
        case SR_SHAPE_AABOX:
            local = {f3(shape->params), f3(shape->params + 3)};
            break;
        default:
            return fail(SR_ERR_INVALID_ARG, "unknown shape kind %d", shape->kind);
    }
    s->objects.push_back({*tr, *mat, *shape, object_bounds(*tr, local)});
    if (out_index) *out_index = (int32_t)s->objects.size() - 1;
    return SR_OK;
}

SR_API int sr_scene_build(SrScene* s) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "scene is NULL");
    if (s->built) return SR_OK;
    if (s->sky_kind < 0) return fail(SR_ERR_STATE, "Scene sky is required");
    SrContext* ctx = s->ctx;

    // Scene BVH over the objects (scene.cs:530-532).
    std::vector<Box> ob(s->objects.size());
    for (size_t i = 0; i < ob.size(); ++i) ob[i] = s->objects[i].bounds;
    if (int rc = build_tree(ctx, ob, 1.0f, 10.0f, 32, ctx->bvh_build, s->tlas)) return rc;
    if (ctx->device < 0) {  // host-only context: the BVH is inspectable, nothing is uploaded
        s->built = true;
        return SR_OK;
    }
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;

    // Meshes used by the scene, each uploaded once however many objects instance it.
    std::vector<int32_t> mesh_slot(ctx->meshes.size(), -2), mesh_root(ctx->meshes.size(), -1);
    std::vector<float4> node_slots, tri_rec, attr_rec;
    for (const auto& o : s->objects) {
        if (o.shape.kind != SR_SHAPE_MESH || mesh_slot[o.shape.mesh] != -2) continue;
        const MeshHost& m = *ctx->meshes[o.shape.mesh];
        int32_t tri_base = (int32_t)(tri_rec.size() / 3);
        mesh_slot[o.shape.mesh] = tri_base;
        for (int32_t j = 0; j < (int32_t)m.bvh.items.size(); ++j) {
            int32_t idx = m.bvh.items[j];
            const SrTriangle& t = m.tris[idx];
            tri_rec.push_back(mk4(t.pos_a[0], t.pos_a[1], t.pos_a[2], ibits(idx)));
            tri_rec.push_back(mk4(t.ab[0], t.ab[1], t.ab[2], 0.0f));
            tri_rec.push_back(mk4(t.ac[0], t.ac[1], t.ac[2], 0.0f));
            const float a[28] = {t.norm_a[0], t.norm_a[1], t.norm_a[2], t.norm_b[0], t.norm_b[1], t.norm_b[2],
                                 t.norm_c[0], t.norm_c[1], t.norm_c[2], t.tan_a[0],  t.tan_a[1],  t.tan_a[2],
                                 t.tan_a[3],  t.tan_b[0],  t.tan_b[1],  t.tan_b[2],  t.tan_b[3],  t.tan_c[0],
                                 t.tan_c[1],  t.tan_c[2],  t.tan_c[3],  t.uv_a[0],   t.uv_a[1],   t.uv_b[0],
                                 t.uv_b[1],   t.uv_c[0],   t.uv_c[1],   0.0f};
            for (int k = 0; k < 7; ++k) attr_rec.push_back(mk4(a[4 * k], a[4 * k + 1], a[4 * k + 2], a[4 * k + 3]));
        }
        mesh_root[o.shape.mesh] = append_tree(node_slots, m.bvh, tri_base);
    }
    // Objects in scene-BVH leaf order.
    std::vector<DevObject> objs(s->objects.size());
    std::vector<DevMaterial> mats(s->objects.size());
    bool has_transparent = false;
    for (size_t p = 0; p < s->objects.size(); ++p) {
        int32_t idx = s->tlas.items[p];
        const SrScene::Obj& o = s->objects[idx];
        DevObject& d = objs[p];
        std::memset(&d, 0, sizeof(d));
        d.pos_kind = mk4(o.tr.pos[0], o.tr.pos[1], o.tr.pos[2], ibits(o.shape.kind));
        d.rot = mk4(o.tr.rot[0], o.tr.rot[1], o.tr.rot[2], o.tr.rot[3]);
        int32_t root = o.shape.kind == SR_SHAPE_MESH ? mesh_root[o.shape.mesh] : -1;
        d.scale_root = mk4(o.tr.scale[0], o.tr.scale[1], o.tr.scale[2], ibits(root));
        d.shape0 = mk4(o.shape.params[0], o.shape.params[1], o.shape.params[2], o.shape.params[3]);
        d.shape1 = mk4(o.shape.params[3], o.shape.params[4], o.shape.params[5], 0.0f);
        d.index = idx;
        if (o.shape.kind == SR_SHAPE_AABOX) d.shape0.w = 0.0f;
    }
    for (size_t i = 0; i < s->objects.size(); ++i) {
        const SrMaterial& m = s->objects[i].mat;
        DevMaterial& d = mats[i];
        float r = (m.ior - 1.0f) / (m.ior + 1.0f);
        float f0 = std::pow(r, 2.0f);  // Brdf.BaseReflectivity brdf.cs:12-16
        d.albedo_rough = mk4(m.albedo[0], m.albedo[1], m.albedo[2], m.roughness);
        d.params = mk4(m.metallic, m.transparency, m.ior, f0);
        d.radiance = mk4(m.radiance[0], m.radiance[1], m.radiance[2], 0.0f);
        d.tex[0] = m.color_texture, d.tex[1] = m.roughness_texture, d.tex[2] = m.metallic_texture, d.tex[3] = m.normal_texture;
        if (m.transparency > 0.0f) has_transparent = true;
    }
    int32_t tlas_root = append_tree(node_slots, s->tlas, 0);

    // Textures (all of the context's, so ids stay valid).
    std::vector<DevTexture> texs(ctx->textures.size());
    std::vector<float4> texels;
    s->tex_offset.assign(ctx->textures.size(), 0);
    for (size_t i = 0; i < ctx->textures.size(); ++i) {
        const TextureHost& t = *ctx->textures[i];
        DevTexture& d = texs[i];
        std::memset(&d, 0, sizeof(d));
        d.width = t.width, d.height = t.height, d.filter = t.filter, d.tiling_x = t.tiling_x, d.tiling_y = t.tiling_y;
        d.offset = texels.size();
        s->tex_offset[i] = texels.size();
        for (size_t k = 0; k < (size_t)t.width * t.height; ++k)
            texels.push_back(mk4(t.texels[3 * k], t.texels[3 * k + 1], t.texels[3 * k + 2], 0.0f));
    }

    // Sky (SkyTexture ctor scene.cs:389-404 builds a Cdf2 with sin(theta) weights, cdf.cs:62-84).
    DevSky sky;
    std::memset(&sky, 0, sizeof(sky));
    sky.kind = s->sky_kind;
    std::vector<float> marginal, cond;
    std::vector<uint32_t> gmarginal, gcond;
    const float pi = 3.14159265358979323846f;
    if (s->sky_kind == 0) {
        const TextureHost& t = *ctx->textures[s->sky_texture];
        uint32_t w = t.width, h = t.height;
        cond.assign((size_t)h * (w + 1), 0.0f);
        std::vector<float> row_w(h);
        for (uint32_t y = 0; y < h; ++y) {
            float* c = &cond[(size_t)y * (w + 1)];
            float sin_w = std::sin(pi * ((float)(int)y + 0.5f) / (float)(int)h);
            c[0] = 0.0f;
            for (uint32_t x = 0; x < w; ++x) c[x + 1] = c[x] + t.texel_lum(x, y) * sin_w;
            float total = c[w];
            if (total > 0.0f)
                for (uint32_t x = 1; x <= w; ++x) c[x] /= total;
            row_w[y] = total;
        }
        marginal.assign(h + 1, 0.0f);
        for (uint32_t y = 0; y < h; ++y) marginal[y + 1] = marginal[y] + row_w[y];
        float total = marginal[h];
        if (total > 0.0f)
            for (uint32_t y = 1; y <= h; ++y) marginal[y] /= total;
        gmarginal.resize(h + 1);
        build_guide(marginal.data(), h, gmarginal.data());
        gcond.resize((size_t)h * (w + 1));
        for (uint32_t y = 0; y < h; ++y) build_guide(&cond[(size_t)y * (w + 1)], w, &gcond[(size_t)y * (w + 1)]);
        sky.texture = s->sky_texture;
        sky.multiplier = s->sky_multiplier;
        sky.cdf_total = total;
        sky.pdf_scale = (float)(int)(w * h) / (total * 2.0f * pi * pi);
        float half = s->sky_yaw * 0.5f;
        float sh = std::sin(half);
        Quat q{0.0f * sh, 1.0f * sh, 0.0f * sh, std::cos(half)};  // Quat.AngleAxis(yaw, Up)
        sky.rot = mk4(q.x, q.y, q.z, q.w);
        sky.rot_inv = mk4(-q.x, -q.y, -q.z, q.w);
    } else {
        const SrSkyProcedural& p = s->sky_proc;
        sky.top = mk4(p.top[0], p.top[1], p.top[2], 0);
        sky.middle = mk4(p.middle[0], p.middle[1], p.middle[2], 0);
        sky.bottom = mk4(p.bottom[0], p.bottom[1], p.bottom[2], 0);
        sky.sun_dir = mk4(p.sun_dir[0], p.sun_dir[1], p.sun_dir[2], 0);
        sky.sun_radiance = mk4(p.sun_radiance[0], p.sun_radiance[1], p.sun_radiance[2], 0);
        sky.sun_cos = std::cos(p.sun_angle);
        sky.sun_pdf_denom = pi * (1.0f - sky.sun_cos);
        // Quat.Look(dir, Up) = FromMat4(Mat4.RotateLook(dir, Up)) (math.cs:641-665, 736-751).
        F3 c0{1, 0, 0}, c1{0, 1, 0}, c2{0, 0, 1};
        F3 fwd_in = f3(p.sun_dir), up{0, 1, 0};
        if (!(mag_sqr(fwd_in) <= 1e-6f)) {
            F3 fwd = normalize(fwd_in);
            F3 right = cross(up, fwd);
            right = mag_sqr(right) > 1e-6f ? normalize(right) : F3{1, 0, 0};
            c0 = right, c1 = cross(fwd, right), c2 = fwd;
        }
        float trace = c0.x + c1.y + c2.z;
        Quat q;
        if (trace > 1e-6f) {
            float sq = std::sqrt(trace + 1) * 2;
            q = {(c1.z - c2.y) / sq, (c2.x - c0.z) / sq, (c0.y - c1.x) / sq, sq * 0.25f};
        } else if (c0.x > c1.y && c0.x > c2.z) {
            float sq = std::sqrt(1 + c0.x - c1.y - c2.z) * 2;
            q = {sq * 0.25f, (c1.x + c0.y) / sq, (c2.x + c0.z) / sq, (c1.z - c2.y) / sq};
        } else if (c1.y > c2.z) {
            float sq = std::sqrt(1 + c1.y - c0.x - c2.z) * 2;
            q = {(c1.x + c0.y) / sq, sq * 0.25f, (c2.y + c1.z) / sq, (c2.x - c0.z) / sq};
        } else {
            float sq = std::sqrt(1 + c2.z - c0.x - c1.y) * 2;
            q = {(c2.x + c0.z) / sq, (c2.y + c1.z) / sq, sq * 0.25f, (c0.y - c1.x) / sq};
        }
        sky.sun_rot = mk4(q.x, q.y, q.z, q.w);
        sky.rot = mk4(0, 0, 0, 1);
        sky.rot_inv = mk4(0, 0, 0, 1);
    }

    SR_CUDA(upload(s->nodes, node_slots.data(), node_slots.size() * sizeof(float4), st), "upload nodes");
    SR_CUDA(upload(s->tris, tri_rec.data(), tri_rec.size() * sizeof(float4), st), "upload triangles");
    SR_CUDA(upload(s->attrs, attr_rec.data(), attr_rec.size() * sizeof(float4), st), "upload attributes");
    SR_CUDA(upload(s->objs, objs.data(), objs.size() * sizeof(DevObject), st), "upload objects");
    SR_CUDA(upload(s->mats, mats.data(), mats.size() * sizeof(DevMaterial), st), "upload materials");
    SR_CUDA(upload(s->texs, texs.data(), texs.size() * sizeof(DevTexture), st), "upload textures");
    SR_CUDA(upload(s->texels, texels.data(), texels.size() * sizeof(float4), st), "upload texels");
    SR_CUDA(upload(s->cdf_marginal, marginal.data(), marginal.size() * sizeof(float), st), "upload cdf");
    SR_CUDA(upload(s->cdf_cond, cond.data(), cond.size() * sizeof(float), st), "upload cdf");
    SR_CUDA(upload(s->guide_marginal, gmarginal.data(), gmarginal.size() * sizeof(uint32_t), st), "upload cdf guide");
    SR_CUDA(upload(s->guide_cond, gcond.data(), gcond.size() * sizeof(uint32_t), st), "upload cdf guide");
    SR_CUDA(s->err.reserve(sizeof(uint32_t)), "alloc error word");
    SR_CUDA(cudaMemsetAsync(s->err.ptr, 0, sizeof(uint32_t), st), "clear error word");
    SR_CUDA(s->counters.reserve(SR_COUNTER_COUNT * sizeof(unsigned long long)), "alloc counters");
    SR_CUDA(cudaStreamSynchronize(st), "scene upload");

    sky.cdf_marginal = s->cdf_marginal.as<float>();
    sky.cdf_cond = s->cdf_cond.as<float>();
    sky.guide_marginal = s->guide_marginal.as<uint32_t>();
    sky.guide_cond = s->guide_cond.as<uint32_t>();
    DevScene& d = s->dev;
    std::memset(&d, 0, sizeof(d));
    d.nodes = s->nodes.as<float4>();
    d.tris = s->tris.as<float4>();
    d.attrs = s->attrs.as<float4>();
    d.objects = s->objs.as<DevObject>();
    d.materials = s->mats.as<DevMaterial>();
    d.textures = s->texs.as<DevTexture>();
    d.texels = s->texels.as<float4>();
    d.sky = sky;
    d.tlas_root = tlas_root;
    d.has_fog = s->has_fog ? 1 : 0;
    d.has_transparent = has_transparent ? 1 : 0;
    d.object_count = (int32_t)s->objects.size();
    bool general = has_transparent || s->sky_kind != 0;
    for (const auto& o : s->objects)
        if (o.shape.kind != SR_SHAPE_MESH || o.mat.normal_texture >= 0) general = true;
    d.general = general ? 1 : 0;
    d.max_actions = kDefaultMaxActions;
    if (s->has_fog) {
        d.fog_density = s->fog.density;
        d.fog_falloff = s->fog.height_falloff;
        d.fog_top = s->fog.height_falloff == 0.0f ? s->fog.top_height : __builtin_inff();
        d.fog_g = s->fog.anisotropy;
        d.fog_color = mk4(s->fog.color[0], s->fog.color[1], s->fog.color[2], 0);
    }
    d.sky.center = nullptr;
    if (ctx->device >= 0 && s->sky_kind == 0 && sky.cdf_total > 0.0f) {
        const TextureHost& t = *ctx->textures[s->sky_texture];
        const size_t n = (size_t)t.width * t.height;
        SR_CUDA(s->sky_center.reserve(n * sizeof(float4)), "alloc sky table");
        SR_CUDA(launch_sky_table(d, s->sky_center.as<float4>(), (uint32_t)n, st), "sky table");
        SR_CUDA(cudaStreamSynchronize(st), "sky table");
        d.sky.center = s->sky_center.as<float4>();
    }
    s->built = true;
    return SR_OK;
}

SR_API int sr_scene_bvh_size(SrScene* s, uint32_t* node_count, uint32_t* item_count) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "scene is NULL");
    if (!s->built) return fail(SR_ERR_STATE, "Scene not built");
    if (node_count) *node_count = (uint32_t)s->tlas.node_count;
    if (item_count) *item_count = (uint32_t)s->tlas.items.size();
    return SR_OK;
}

SR_API int sr_scene_bvh_export(SrScene* s, float* node_bounds, int32_t* node_links, int32_t* items) {
    if (!s || !node_bounds) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (!s->built) return fail(SR_ERR_STATE, "Scene not built");
    export_bvh(s->tlas, node_bounds, node_links, items);
    return SR_OK;
}

// The scene as a kernel argument: its device description with the tuned traversal cap.
static DevScene launch_scene(const SrScene* s) {
    DevScene d = s->dev;
    if (s->tune.max_actions) d.max_actions = s->tune.max_actions;
    return d;
}

static int need_device(SrScene* s) {
    if (!s->built) return fail(SR_ERR_STATE, "Scene not built");
    if (s->ctx->device < 0) return fail(SR_ERR_STATE, "host-only context (device -1) cannot run device work");
    return SR_OK;
}

static int check_device_error(SrScene* s) {
    uint32_t word = 0;
    SR_CUDA(cudaMemcpy(&word, s->err.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost), "read error word");
    if (word) {
        cudaMemset(s->err.ptr, 0, sizeof(uint32_t));
        return fail(SR_ERR_DEVICE, "kernel error word 0x%x (1 = traversal stack overflow, 2 = loop cap)", word);
    }
    return SR_OK;
}

SR_API int sr_scene_trace(SrScene* s, const float* rays, uint32_t count, int32_t* out_object, int32_t* out_triangle,
                          float* out_dist, float* out_uv) {
    if (!s || (!rays && count) || !out_object || !out_triangle || !out_dist || !out_uv)
        return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    // rays, then the four outputs, then (persistent form) ray-queue entries on 256 bytes and a cursor
    size_t in_b = (size_t)count * 6 * 4, out_b = (size_t)count * 5 * 4;
    const size_t q_off = (in_b + out_b + 255) & ~(size_t)255, q_b = (size_t)count * sizeof(Rec);
    SR_CUDA(s->rays_io.reserve(q_off + q_b + 256), "alloc ray buffers");
    char* base = s->rays_io.as<char>();
    float* d_rays = (float*)base;
    int32_t* d_obj = (int32_t*)(base + in_b);
    int32_t* d_tri = d_obj + count;
    float* d_dist = (float*)(d_tri + count);
    float* d_uv = d_dist + count;
    SR_CUDA(cudaMemcpyAsync(d_rays, rays, in_b, cudaMemcpyHostToDevice, st), "copy rays");
    if (s->render_mode == SR_RENDER_MEGAKERNEL) {
        // one thread per ray through the megakernel's traversal
        SR_CUDA(launch_trace(launch_scene(s), d_rays, count, d_obj, d_tri, d_dist, d_uv, s->err.as<uint32_t>(), st),
                "trace launch");
    } else {
        // the wavefront renderer's persistent traversal loop
        if (!s->sms) SR_CUDA(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->ctx->device), "device query");
        const DevScene S = launch_scene(s);
        SR_CUDA(launch_trace_persistent(S, S.general != 0, d_rays, count, (Rec*)(base + q_off),
                                        (uint32_t*)(base + q_off + q_b), d_obj, d_tri, d_dist, d_uv,
                                        s->err.as<uint32_t>(), s->sms, st),
                "trace launch");
    }
    SR_CUDA(cudaMemcpyAsync(out_object, d_obj, count * 4, cudaMemcpyDeviceToHost, st), "copy hits");
    SR_CUDA(cudaMemcpyAsync(out_triangle, d_tri, count * 4, cudaMemcpyDeviceToHost, st), "copy hits");
    SR_CUDA(cudaMemcpyAsync(out_dist, d_dist, count * 4, cudaMemcpyDeviceToHost, st), "copy hits");
    SR_CUDA(cudaMemcpyAsync(out_uv, d_uv, count * 8, cudaMemcpyDeviceToHost, st), "copy hits");
    SR_CUDA(cudaStreamSynchronize(st), "trace");
    return check_device_error(s);
}

static int make_view(const SrView* v, const SrRenderParams* p, DevView& dv, DevParams& dp) {
    if (!v || !p) return fail(SR_ERR_INVALID_ARG, "NULL view or params");
    if (p->width == 0 || p->height == 0) return fail(SR_ERR_INVALID_ARG, "width and height must be > 0");
    if (p->min_samples == 0 || p->min_samples > p->max_samples)
        return fail(SR_ERR_INVALID_ARG, "need 0 < min_samples <= max_samples");
    if (!(v->fov > 0.0f && v->fov < 3.14159265f)) return fail(SR_ERR_INVALID_ARG, "Invalid fov");
    if (!(v->near_plane > 0.0f)) return fail(SR_ERR_INVALID_ARG, "Invalid near plane");
    float aspect = (float)p->width / (float)p->height;
    float th, tv;
    if (aspect >= 1.0f) {
        th = std::tan(v->fov * 0.5f);
        tv = th / aspect;
    } else {
        tv = std::tan(v->fov * 0.5f);
        th = tv * aspect;
    }
    Quat rot = quat(v->transform.rot);
    F3 origin = f3(v->transform.pos) + rotate(rot, F3{0.0f, 0.0f, v->near_plane});
    dv.origin = mk4(origin.x, origin.y, origin.z, 0);
    dv.rot = mk4(rot.x, rot.y, rot.z, rot.w);
    dv.tan_h = th;
    dv.tan_v = tv;
    dv.pad0 = dv.pad1 = 0;
    dp.width = p->width;
    dp.height = p->height;
    dp.min_samples = p->min_samples;
    dp.max_samples = p->max_samples;
    dp.bounces = p->bounces;
    dp.variance_threshold = p->variance_threshold;
    dp.indirect_clamp = p->indirect_clamp;
    dp.aspect = aspect;
    dp.seed = 0;
    dp.pad[0] = dp.pad[1] = dp.pad[2] = 0;
    return SR_OK;
}

static int compose_impl(SrContext* ctx, const DevAovs& in, uint32_t w, uint32_t h, const SrComposeParams* p,
                        bool denoise, uint8_t* rgb8, cudaStream_t st,
                        float* linear = nullptr);

// Closest-hit queries a traversal launch may set aside (per group and parity): 1/32 of the slots,
// between 256 and 16384; kDeferBytes each (the query's state and a full traversal stack).
static uint32_t defer_capacity(size_t slots) {
    const size_t c = slots / 32;
    return (uint32_t)(c < 256 ? 256 : (c > 16384 ? 16384 : c));
}

// Allocates the wavefront path state for `tiles` tiles of 32 slots over an image of pixel_tiles
// 8x4 pixel tiles (tiles_x per row): the records of every slot, then each group's queues, then
// every group's counters (one block, carved).  Fewer slot tiles than pixel tiles: slots claim the
// pixels left over as theirs finish.
static int wave_reserve(SrScene* s, uint32_t tiles_x, uint32_t pixel_tiles, uint32_t tiles) {
    const size_t n = (size_t)tiles * 32;
    uint32_t group_slots[kWaveGroups];
    for (int g = 0; g < kWaveGroups; ++g) group_slots[g] = (uint32_t)(tiles > (uint32_t)g ? (tiles - g + kWaveGroups - 1) / kWaveGroups : 0) * 32;
    if (s->wave_slots < n || !s->wave.ptr) {
        // 32-byte sectors: path records (6 per slot), pixel records (4 per slot); 16-byte medium;
        // queues per group slot: ray entries (32 B) trace x2 + shadow x2, 4-byte event 3 x2 + late x2 +
        // resolve x2 + sorted 3; arrays start on 256 bytes
        const size_t rec = sizeof(Rec);
        size_t bytes = n * (10 * rec + 16 + 4 * rec + 13 * 4 + 1) + (4 + 13 * kWaveGroups) * 256 +
                       kWaveGroups * (kWaveCounters * sizeof(uint32_t) + 2 * (size_t)defer_capacity(n) * kDeferBytes);
        SR_CUDA(s->wave.reserve(bytes), "alloc wavefront state");
        s->wave_slots = (uint32_t)n;
    }
    char* p = s->wave.as<char>();
    auto take = [&](size_t count, size_t elem_bytes) {
        char* r = p;
        p += (count * elem_bytes + 255) & ~(size_t)255;
        return r;
    };
    const size_t rec = sizeof(Rec);
    Rec* recs = (Rec*)take(n, 6 * rec);
    Rec* pix = (Rec*)take(n, 4 * rec);
    float4* medium = (float4*)take(n, 16);
    uint8_t* ev_mark = (uint8_t*)take(n, 1);
    for (int g = 0; g < kWaveGroups; ++g) {
        WaveState& w = s->ws[g];
        const size_t m = group_slots[g];
        w.slots = group_slots[g];
        w.tiles_x = tiles_x;
        w.pixel_tiles = pixel_tiles;
        w.dynamic = tiles < pixel_tiles ? 1u : 0u;
        w.group = (uint32_t)g;
        w.groups = kWaveGroups;
        w.rec = recs;
        w.pix = pix;
        w.medium = medium;
        w.q_trace[0] = (Rec*)take(m, rec);
        w.q_trace[1] = (Rec*)take(m, rec);
        w.q_event[0] = (uint32_t*)take(m, 3 * 4);
        w.q_event[1] = (uint32_t*)take(m, 3 * 4);
        w.q_resolve[0] = (uint32_t*)take(m, 4);
        w.q_resolve[1] = (uint32_t*)take(m, 4);
        w.q_shadow[0] = (Rec*)take(m, rec);
        w.q_shadow[1] = (Rec*)take(m, rec);
        w.q_late[0] = (uint32_t*)take(m, 4);
        w.q_late[1] = (uint32_t*)take(m, 4);
        w.q_sorted = (uint32_t*)take(m, 3 * 4);
        w.defer_cap = defer_capacity(n);
        w.defer[0] = (float4*)take(w.defer_cap, kDeferBytes);
        w.defer[1] = (float4*)take(w.defer_cap, kDeferBytes);
        w.rec_stride = (uint32_t)n;
        w.ev_mark = ev_mark;
    }
    for (int g = 0; g < kWaveGroups; ++g) {
        s->ws[g].counts = (uint32_t*)p + g * kWaveCounters;
        s->ws[g].pixel_cursor = (uint32_t*)p + kCountPixel;  // group 0's
    }
    return SR_OK;
}

// The wavefront state of scene s reserved and initialised on `st` (first camera rays) for one
// render, and the launch description of its bounce kernels in L.
// `slot_cap`: whether the scene's slot capacity (WaveTune::max_slots) applies (not for renders that
// keep every sample's vertices, which are indexed by slot).
static int wave_prepare(SrScene* s, const DevView& dv, const DevParams& dp, const DevAovs& out,
                        unsigned long long* ctr, cudaStream_t st, WaveLaunch& L, bool slot_cap = true) {
    const uint32_t tiles_x = (dp.width + 7) / 8, tiles_y = (dp.height + 3) / 4, pixel_tiles = tiles_x * tiles_y;
    uint32_t tiles = pixel_tiles;
    if (slot_cap && s->tune.max_slots) {
        const uint32_t cap = (s->tune.max_slots + 31) / 32;
        if (cap < tiles) tiles = cap;
    }
    int rc = wave_reserve(s, tiles_x, pixel_tiles, tiles);
    if (rc) return rc;
    // side streams: the other groups' bounces, or (one group) the ready phase of each bounce
    for (cudaStream_t& side : s->side_streams)
        if (!side) SR_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking), "stream");
    for (cudaEvent_t& e : s->fork_events)
        if (!e) SR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    if (!s->sms) {
        SR_CUDA(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->ctx->device), "device query");
    }
    std::memset(&L, 0, sizeof(L));  // padding bytes take part in the graph-reuse comparison
    for (int g = 0; g < kWaveGroups; ++g) L.W[g] = s->ws[g];
    L.groups = kWaveGroups;
    L.S = launch_scene(s);
    L.V = dv;
    L.P = dp;
    L.out = out;
    L.err = s->err.as<uint32_t>();
    L.counters = ctr;
    L.general = s->dev.general;
    wave_grid_sizes(L, s->sms, &s->tune);
    // a runaway guard, not a budget: a pixel's samples run one after another, each taking up to
    // bounces + 2 iterations (the last segment's shadow ray is traced one bounce later), and a
    // slot runs the pixels it claims one after another
    const uint64_t rounds = (pixel_tiles + tiles - 1) / tiles;
    uint64_t cap = (((uint64_t)dp.max_samples + 1) * ((uint64_t)dp.bounces + 2) * 2 + 8) * rounds;
    if (s->tune.max_iters && s->tune.max_iters < cap) cap = s->tune.max_iters;
    L.max_iters = (uint32_t)(cap > 0x7fffffffull ? 0x7fffffffull : cap);
    uint32_t all_slots = 0;
    for (int g = 0; g < kWaveGroups; ++g) all_slots += s->ws[g].slots;
    const uint32_t tail_div = s->tune.tail_div ? s->tune.tail_div : (uint32_t)SR_TAIL_DIV;
    L.tail_paths = tail_div > 0 ? all_slots / tail_div : 0;
    L.progress = s->progress_dev;
    SR_CUDA(wave_init(L, st, s->seed), "wavefront init");
    return SR_OK;
}

// A wavefront render of scene s; `adj` (with adj_mode kAdjReplay or kAdjRecord) makes it an adjoint
// pass, whose AdjPass goes to the scene's device copy before the launches.  Forward renders and
// adjoint passes keep separate cached graphs.
static int render_wavefront(SrScene* s, const DevView& dv, const DevParams& dp, const DevAovs& out,
                            unsigned long long* ctr, cudaStream_t st, bool graph, int adj_mode = kAdjNone,
                            AdjPass* adj = nullptr, WaveLaunch* launch_out = nullptr) {
    WaveLaunch L;
    if (int rc = wave_prepare(s, dv, dp, out, ctr, st, L, adj_mode != kAdjRecord)) return rc;
    if (adj_mode != kAdjNone) {
        // vertex records: one sample per slot (replay) or every sample (record, kept apart so that
        // a replay pass does not overwrite a checkpoint)
        const bool record = adj_mode == kAdjRecord;
        const uint64_t kept = record ? dp.max_samples : 1u;
        adj->vper = dp.bounces + 1;
        adj->samples_kept = (uint32_t)kept;
        const uint64_t recs = (uint64_t)s->wave_slots * kept * adj->vper;
        DevBuf& vbuf = record ? s->ckpt_vbuf : s->adj_vbuf;
        DevBuf& pass = record ? s->ckpt_pass_dev : s->adj_pass;
        SR_CUDA(vbuf.reserve(recs * kAdjVertexF4 * sizeof(float4)), "alloc adjoint vertex records");
        adj->vbuf = vbuf.as<float4>();
        if (record) {
            SR_CUDA(s->ckpt_vcount.reserve((size_t)s->wave_slots * kept), "alloc adjoint vertex counts");
            adj->vcount = s->ckpt_vcount.as<uint8_t>();
        }
        SR_CUDA(pass.reserve(sizeof(AdjPass)), "alloc adjoint pass");
        SR_CUDA(cudaMemcpyAsync(pass.ptr, adj, sizeof(AdjPass), cudaMemcpyHostToDevice, st), "upload adjoint pass");
        L.adj_mode = adj_mode;
        L.adj = pass.as<AdjPass>();
        wave_adj_grid_sizes(L, s->sms);
    }
    if (launch_out) *launch_out = L;
    if (graph) {
        cudaGraphExec_t& exec = adj_mode != kAdjNone ? s->adj_graph_exec : s->graph_exec;
        WaveLaunch& baked = adj_mode != kAdjNone ? s->adj_graph_launch : s->graph_launch;
        if (!s->capture_stream) SR_CUDA(cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking), "stream");
        if (exec && std::memcmp(&baked, &L, sizeof(L)) != 0) {
            SR_CUDA(cudaStreamSynchronize(st), "sync before graph rebuild");
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        if (!exec) {
            SR_CUDA(wave_build_graph(L, s->capture_stream, s->side_streams, s->fork_events, &exec),
                    "build bounce-loop graph");
            std::memcpy(&baked, &L, sizeof(L));
        }
        SR_CUDA(cudaGraphLaunch(exec, st), "launch bounce-loop graph");
        return SR_OK;
    }
    const size_t count_bytes = kWaveGroups * kWaveCounters * sizeof(uint32_t);
    if (!s->counts_host) SR_CUDA(cudaMallocHost(&s->counts_host, count_bytes), "pinned alloc");
    s->trace_ms = 0.0;
    s->trace_launches = 0;
    if (s->kernel_timing) {  // an event pair around every bounce's traversal kernel, read after the bounce
        for (cudaEvent_t& e : s->trace_ev)
            if (!e) SR_CUDA(cudaEventCreate(&e), "event");
        L.trace_ev[0] = s->trace_ev[0];
        L.trace_ev[1] = s->trace_ev[1];
    }
    for (uint32_t it = 0;; ++it) {
        if (it >= L.max_iters)
            return fail(SR_ERR_DEVICE, "wavefront loop exceeded %u bounces (error word 0x2, loop cap)", L.max_iters);
        int cur = (int)(it & 1u);
        SR_CUDA(wave_bounce(L, cur, st, s->side_streams, s->fork_events), "wavefront bounce");
        SR_CUDA(cudaMemcpyAsync(s->counts_host, s->ws[0].counts, count_bytes, cudaMemcpyDeviceToHost, st), "read live count");
        SR_CUDA(cudaStreamSynchronize(st), "wavefront bounce");
        if (L.trace_ev[0]) {
            float ms = 0.0f;
            SR_CUDA(cudaEventElapsedTime(&ms, L.trace_ev[0], L.trace_ev[1]), "traversal kernel time");
            s->trace_ms += ms;
            ++s->trace_launches;
        }
        uint32_t live = 0, done = 0;
        for (int g = 0; g < kWaveGroups; ++g) {
            live += wave_live(s->counts_host + g * kWaveCounters, cur ^ 1, s->ws[g].defer_cap);
            done += s->counts_host[g * kWaveCounters + kCountDone];
        }
        if (s->progress_host) *(volatile uint32_t*)s->progress_host = done;
        if (live <= L.tail_paths) {
            s->last_host_iters = it + 1;
            s->last_tail = live > 0;
            if (live > 0) SR_CUDA(wave_tail(L, cur ^ 1, st), "wavefront tail");
            break;
        }
    }
    return SR_OK;
}

// Progress of the render about to be launched on scene s: the host-mapped word cleared, the total.
static int progress_begin(SrScene* s, uint32_t pixels) {
    if (!s->progress_host) {
        SR_CUDA(cudaHostAlloc(&s->progress_host, sizeof(uint32_t), cudaHostAllocMapped), "pinned alloc");
        SR_CUDA(cudaHostGetDevicePointer((void**)&s->progress_dev, s->progress_host, 0), "mapped pointer");
    }
    if (!s->progress_event) SR_CUDA(cudaEventCreateWithFlags(&s->progress_event, cudaEventDisableTiming), "event");
    *(volatile uint32_t*)s->progress_host = 0;
    s->progress_total = pixels;
    return SR_OK;
}

static int render_into(SrScene* s, const SrView* view, const SrRenderParams* params, const DevAovs& out, cudaStream_t st) {
    DevView dv;
    DevParams dp;
    int rc = make_view(view, params, dv, dp);
    if (rc) return rc;
    unsigned long long* ctr = nullptr;
    if (s->counting) {
        ctr = s->counters.as<unsigned long long>();
        SR_CUDA(cudaMemsetAsync(ctr, 0, SR_COUNTER_COUNT * sizeof(unsigned long long), st), "clear counters");
    }
    int mode = s->render_mode == SR_RENDER_AUTO ? SR_RENDER_WAVEFRONT_GRAPH : s->render_mode;
    s->last_mode = mode;
    if (int rc = progress_begin(s, dp.width * dp.height)) return rc;
    if (mode == SR_RENDER_MEGAKERNEL) {
        DevParams pm = dp;
        pm.seed = s->seed;
        SR_CUDA(launch_render(launch_scene(s), dv, pm, out, ctr, s->err.as<uint32_t>(), st), "render launch");
    } else if (int rc = render_wavefront(s, dv, dp, out, ctr, st, mode == SR_RENDER_WAVEFRONT_GRAPH)) {
        return rc;
    }
    SR_CUDA(cudaEventRecord(s->progress_event, st), "progress event");
    return SR_OK;
}

SR_API int sr_render_progress(SrScene* s, uint32_t* done, uint32_t* total) {
    if (!s || !done || !total) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    *total = s->progress_total;
    *done = 0;
    if (!s->progress_event) return SR_OK;  // nothing rendered yet
    cudaError_t q = cudaEventQuery(s->progress_event);
    if (q == cudaSuccess) {
        *done = s->progress_total;
    } else if (q == cudaErrorNotReady) {
        uint32_t d = *(volatile uint32_t*)s->progress_host;
        *done = d < s->progress_total ? d : s->progress_total;
    } else {
        SR_CUDA(q, "progress query");
    }
    return SR_OK;
}

SR_API int sr_render_device(SrScene* s, const SrView* view, const SrRenderParams* params, const SrAovs* out,
                            void* stream) {
    if (!s || !out) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    if (!out->radiance || !out->radiance_fog || !out->normals || !out->uv || !out->depth || !out->samples || !out->variance)
        return fail(SR_ERR_INVALID_ARG, "sr_render_device needs all seven AOV planes");
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : s->ctx->stream;
    DevAovs d{out->radiance, out->radiance_fog, out->normals, out->uv, out->depth, out->samples, out->variance};
    return render_into(s, view, params, d, st);
}

SR_API int sr_render_batch(SrScene* const* scenes, const SrView* views, const SrRenderParams* params,
                           const SrAovs* outs, uint32_t count, void* stream) {
    if (!scenes || !views || !params || !outs) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (count == 0) return SR_OK;
    SrContext* ctx = scenes[0] ? scenes[0]->ctx : nullptr;
    for (uint32_t i = 0; i < count; ++i) {
        SrScene* s = scenes[i];
        if (!s) return fail(SR_ERR_INVALID_ARG, "scene %u is NULL", i);
        if (s->ctx != ctx) return fail(SR_ERR_INVALID_ARG, "scene %u belongs to another context", i);
        if (int rc = need_device(s)) return rc;
        for (uint32_t j = 0; j < i; ++j)
            if (scenes[j] == s) return fail(SR_ERR_INVALID_ARG, "scene %u appears twice in the batch", i);
        const SrAovs& o = outs[i];
        if (!o.radiance || !o.radiance_fog || !o.normals || !o.uv || !o.depth || !o.samples || !o.variance)
            return fail(SR_ERR_INVALID_ARG, "batch entry %u needs all seven AOV planes", i);
    }
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    std::vector<WaveLaunch> Ls(count);
    for (uint32_t i = 0; i < count; ++i) {
        SrScene* s = scenes[i];
        DevView dv;
        DevParams dp;
        if (int rc = make_view(&views[i], &params[i], dv, dp)) return rc;
        unsigned long long* ctr = nullptr;
        if (s->counting) {
            ctr = s->counters.as<unsigned long long>();
            SR_CUDA(cudaMemsetAsync(ctr, 0, SR_COUNTER_COUNT * sizeof(unsigned long long), st), "clear counters");
        }
        const SrAovs& o = outs[i];
        DevAovs d{o.radiance, o.radiance_fog, o.normals, o.uv, o.depth, o.samples, o.variance};
        std::memset(&Ls[i], 0, sizeof(WaveLaunch));
        if (int rc = progress_begin(s, dp.width * dp.height)) return rc;
        if (int rc = wave_prepare(s, dv, dp, d, ctr, st, Ls[i])) return rc;
        s->last_mode = SR_RENDER_WAVEFRONT_GRAPH;
    }
    if (!ctx->batch_capture) SR_CUDA(cudaStreamCreateWithFlags(&ctx->batch_capture, cudaStreamNonBlocking), "stream");
    const bool same = ctx->batch_exec && ctx->batch_launch.size() == count &&
                      std::memcmp(ctx->batch_launch.data(), Ls.data(), count * sizeof(WaveLaunch)) == 0;
    if (!same) {
        if (ctx->batch_exec) {
            SR_CUDA(cudaStreamSynchronize(st), "sync before graph rebuild");
            cudaGraphExecDestroy(ctx->batch_exec);
            ctx->batch_exec = nullptr;
        }
        SrScene* s0 = scenes[0];  // side streams and fork events (used only with several slot groups)
        SR_CUDA(wave_build_graph_batch(Ls.data(), (int)count, ctx->batch_capture, s0->side_streams, s0->fork_events,
                                       &ctx->batch_exec),
                "build batch graph");
        ctx->batch_launch = Ls;
    }
    SR_CUDA(cudaGraphLaunch(ctx->batch_exec, st), "launch batch graph");
    for (uint32_t i = 0; i < count; ++i) SR_CUDA(cudaEventRecord(scenes[i]->progress_event, st), "progress event");
    return SR_OK;
}

SR_API int sr_scene_set_seed(SrScene* s, uint32_t seed) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    s->seed = seed;
    return SR_OK;
}

SR_API int sr_scene_get_seed(SrScene* s, uint32_t* seed) {
    if (!s || !seed) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    *seed = s->seed;
    return SR_OK;
}

SR_API int sr_scene_set_tuning(SrScene* s, const SrTuning* t) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "scene is NULL");
    if (t && (t->trace_blocks_per_sm < 0 || t->fog_shade_blocks_per_sm < 0 || t->surface_shade_blocks_per_sm < 0))
        return fail(SR_ERR_INVALID_ARG, "blocks per SM must be >= 0");
    if (t && t->trace_block_threads != 0 && t->trace_block_threads != 64 && t->trace_block_threads != 128 &&
        t->trace_block_threads != 256)
        return fail(SR_ERR_INVALID_ARG, "trace_block_threads must be 64, 128 or 256 (or 0)");
    s->tune = t ? WaveTune{t->trace_blocks_per_sm, t->fog_shade_blocks_per_sm, t->surface_shade_blocks_per_sm,
                           t->tail_divisor, t->max_bounce_iterations, t->max_traversal_steps,
                           (int)t->trace_block_threads, t->max_slots}
                : WaveTune{};
    return SR_OK;
}

SR_API int sr_scene_get_tuning(SrScene* s, SrTuning* t) {
    if (!s || !t) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    std::memset(t, 0, sizeof(*t));
    t->trace_blocks_per_sm = s->tune.trace_per_sm;
    t->fog_shade_blocks_per_sm = s->tune.fog_per_sm;
    t->surface_shade_blocks_per_sm = s->tune.surface_per_sm;
    t->tail_divisor = s->tune.tail_div;
    t->max_bounce_iterations = s->tune.max_iters;
    t->max_traversal_steps = s->tune.max_actions;
    t->trace_block_threads = (uint32_t)s->tune.trace_block;
    t->max_slots = s->tune.max_slots;
    return SR_OK;
}

// Times `params` at trial_spp samples per pixel under candidate launch geometries, one dimension at a
// time from the defaults (coordinate search): traversal block size, traversal blocks per SM,
// fog-shade blocks per SM, tail hand-over, slot capacity; keeps the fastest of each dimension and
// leaves the result on the scene.
SR_API int sr_scene_autotune(SrScene* s, const SrView* view, const SrRenderParams* params, uint32_t trial_spp,
                             SrTuning* out) {
    if (!s || !view || !params) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    if (trial_spp == 0) return fail(SR_ERR_INVALID_ARG, "trial_spp must be > 0");
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    SrRenderParams p = *params;
    p.min_samples = p.max_samples = trial_spp;
    const size_t n = (size_t)p.width * p.height;
    SR_CUDA(s->tune_aovs.reserve(n * 56 + 256), "alloc autotune AOVs");
    char* b = s->tune_aovs.as<char>();
    DevAovs d;
    d.radiance = (float*)b;
    d.radiance_fog = d.radiance + 3 * n;
    d.normals = d.radiance_fog + 3 * n;
    d.uv = d.normals + 3 * n;
    d.depth = d.uv + 2 * n;
    d.samples = (uint32_t*)(d.depth + n);
    d.variance = (float*)(d.samples + n);
    int tr = 0, fog = 0, surf = 0;
    wave_occupancy(s->dev.general != 0, &tr, &fog, &surf);
    cudaEvent_t e0, e1;
    SR_CUDA(cudaEventCreate(&e0), "event");
    SR_CUDA(cudaEventCreate(&e1), "event");
    const int32_t saved_mode = s->render_mode;
    const WaveTune saved = s->tune;
    s->render_mode = SR_RENDER_WAVEFRONT_GRAPH;
    int rc = SR_OK;
    // one trial: a warm-up render (builds the graph), then two timed renders
    auto trial = [&](const WaveTune& t, float& ms) {
        s->tune = t;
        rc = render_into(s, view, &p, d, st);
        if (!rc) rc = cudaEventRecord(e0, st) == cudaSuccess ? SR_OK : fail(SR_ERR_CUDA, "event");
        for (int k = 0; k < 2 && !rc; ++k) rc = render_into(s, view, &p, d, st);
        if (!rc) rc = cudaEventRecord(e1, st) == cudaSuccess ? SR_OK : fail(SR_ERR_CUDA, "event");
        if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = fail(SR_ERR_CUDA, "autotune render");
        ms = 0.0f;
        if (!rc) cudaEventElapsedTime(&ms, e0, e1);
        ms *= 0.5f;
        return rc == SR_OK;
    };
    WaveTune best{0, 0, 0, 16, saved.max_iters, saved.max_actions, 128, 0};
    float best_ms = 0.0f, default_ms = 0.0f;
    if (trial(best, default_ms)) best_ms = default_ms;
    auto consider = [&](WaveTune t) {
        float ms = 0.0f;
        if (!rc && trial(t, ms) && ms < best_ms) best_ms = ms, best = t;
    };
    for (int blk : {64, 256}) {  // traversal block size
        WaveTune t = best;
        t.trace_block = blk;
        consider(t);
    }
    const int fit = best.trace_block == 128 ? tr : wave_trace_occupancy(s->dev.general != 0, best.trace_block);
    for (int fewer : {1, 2}) {  // traversal blocks per SM: one or two fewer than fit
        WaveTune t = best;
        t.trace_per_sm = fit - fewer;
        if (t.trace_per_sm >= 1) consider(t);
    }
    if (fog - 2 >= 1) {  // fog-shade blocks per SM
        WaveTune t = best;
        t.fog_per_sm = fog - 2;
        consider(t);
    }
    for (uint32_t div : {8u, 32u}) {  // tail hand-over
        WaveTune t = best;
        t.tail_div = div;
        consider(t);
    }
    for (uint32_t part : {2u, 4u}) {  // slot capacity: half or a quarter of the pixels in flight
        WaveTune t = best;
        t.max_slots = (uint32_t)((n + part - 1) / part);
        if (t.max_slots >= 32) consider(t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->render_mode = saved_mode;
    if (rc) {
        s->tune = saved;
        return rc;
    }
    if (int erc = check_device_error(s)) {
        s->tune = saved;
        return erc;
    }
    s->tune = best;
    if (out) {
        sr_scene_get_tuning(s, out);
        out->ms = best_ms;
        out->default_ms = default_ms;
    }
    return SR_OK;
}

// Device AOV planes (56 B per pixel) plus an RGB8 image, cached on the scene.
static cudaError_t stage_aovs(SrScene* s, size_t n, DevAovs& d, uint8_t** rgb) {
    cudaError_t e = s->aovs.reserve(n * 59 + 256);
    if (e != cudaSuccess) return e;
    char* b = s->aovs.as<char>();
    d.radiance = (float*)b;
    d.radiance_fog = d.radiance + 3 * n;
    d.normals = d.radiance_fog + 3 * n;
    d.uv = d.normals + 3 * n;
    d.depth = d.uv + 2 * n;
    d.samples = (uint32_t*)(d.depth + n);
    d.variance = (float*)(d.samples + n);
    if (rgb) *rgb = (uint8_t*)(d.variance + n);
    return cudaSuccess;
}

static int copy_aovs_to_host(const DevAovs& d, size_t n, const SrAovs& host_out, cudaStream_t st) {
    struct Plane {
        void* dst;
        const void* src;
        size_t bytes;
    } planes[] = {{host_out.radiance, d.radiance, n * 12},  {host_out.radiance_fog, d.radiance_fog, n * 12},
                  {host_out.normals, d.normals, n * 12},    {host_out.uv, d.uv, n * 8},
                  {host_out.depth, d.depth, n * 4},         {host_out.samples, d.samples, n * 4},
                  {host_out.variance, d.variance, n * 4}};
    for (const Plane& p : planes)
        if (p.dst) SR_CUDA(cudaMemcpyAsync(p.dst, p.src, p.bytes, cudaMemcpyDeviceToHost, st), "copy AOVs");
    return SR_OK;
}

SR_API int sr_render(SrScene* s, const SrView* view, const SrRenderParams* params, const SrAovs* host_out) {
    if (!s || !host_out || !params) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    size_t n = (size_t)params->width * params->height;
    DevAovs d;
    SR_CUDA(stage_aovs(s, n, d, nullptr), "alloc AOVs");
    int rc = render_into(s, view, params, d, st);
    if (rc) return rc;
    rc = copy_aovs_to_host(d, n, *host_out, st);
    if (rc) return rc;
    SR_CUDA(cudaStreamSynchronize(st), "render");
    if (s->counting)
        SR_CUDA(cudaMemcpy(s->last_counters, s->counters.ptr, sizeof(s->last_counters), cudaMemcpyDeviceToHost),
                "read counters");
    return check_device_error(s);
}

SR_API int sr_scene_set_render_mode(SrScene* s, int32_t mode) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "scene is NULL");
    if (mode < SR_RENDER_AUTO || mode > SR_RENDER_WAVEFRONT_GRAPH) return fail(SR_ERR_INVALID_ARG, "bad render mode %d", mode);
    s->render_mode = mode;
    return SR_OK;
}

SR_API int sr_scene_render_info(SrScene* s, uint32_t* kernel_launches, uint32_t* bounce_iterations) {
    if (!s || !kernel_launches || !bounce_iterations) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    SR_CUDA(cudaDeviceSynchronize(), "sync");
    if (s->last_mode == SR_RENDER_MEGAKERNEL) {
        *kernel_launches = 1;
        *bounce_iterations = 0;
        return SR_OK;
    }
    uint32_t iters = s->last_host_iters;
    if (s->last_mode == SR_RENDER_WAVEFRONT_GRAPH) {
        SR_CUDA(cudaMemcpy(&iters, s->ws[0].counts + kCountIter, sizeof(uint32_t), cudaMemcpyDeviceToHost), "read bounce count");
        // init and bounce kernels per group, one loop condition per loop body, the tail kernel
        *kernel_launches = kWaveGroups * (1 + kWaveKernelsPerBounce * iters) + iters / kGraphBounces + 1;
    } else {
        *kernel_launches = kWaveGroups * (1 + kWaveKernelsPerBounce * iters) + (s->last_tail ? 1 : 0);
    }
    *bounce_iterations = iters;
    return SR_OK;
}

SR_API int sr_scene_set_kernel_timing(SrScene* s, int32_t enabled) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "scene is NULL");
    s->kernel_timing = enabled != 0;
    return SR_OK;
}

SR_API int sr_scene_trace_time(SrScene* s, float* total_ms, uint32_t* launches) {
    if (!s || !total_ms || !launches) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    SR_CUDA(cudaDeviceSynchronize(), "sync");
    const bool timed = s->last_mode == SR_RENDER_WAVEFRONT;
    *total_ms = timed ? (float)s->trace_ms : 0.0f;
    *launches = timed ? s->trace_launches : 0u;
    return SR_OK;
}

SR_API int sr_scene_set_counting(SrScene* s, int32_t enabled) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "scene is NULL");
    s->counting = enabled != 0;
    return SR_OK;
}

SR_API int sr_scene_counters(SrScene* s, uint64_t* counters_out) {
    if (!s || !counters_out) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    SR_CUDA(cudaDeviceSynchronize(), "sync");
    SR_CUDA(cudaMemcpy(counters_out, s->counters.ptr, SR_COUNTER_COUNT * sizeof(uint64_t), cudaMemcpyDeviceToHost),
            "read counters");
    return check_device_error(s);
}

// ---- compose ------------------------------------------------------------------------------------
static void build_table(std::vector<float>& out, int radius, float inv, float scale) {
    // (2R+1)^2 spatial weights scale*exp(-d^2*inv), then per-row half widths.
    int side = 2 * radius + 1;
    size_t base = out.size();
    out.resize(base + (size_t)side * side + side);
    for (int ky = -radius; ky <= radius; ++ky)
        for (int kx = -radius; kx <= radius; ++kx) {
            float kd = (float)(kx * kx + ky * ky);
            out[base + (size_t)(ky + radius) * side + (kx + radius)] = scale * std::exp(-kd * inv);
        }
    for (int ky = -radius; ky <= radius; ++ky) {
        int hw = 0;
        while ((hw + 1) * (hw + 1) + ky * ky <= radius * radius) ++hw;
        out[base + (size_t)side * side + (ky + radius)] = (float)hw;
    }
}

static int compose_impl(SrContext* ctx, const DevAovs& in, uint32_t w, uint32_t h, const SrComposeParams* p,
                        bool denoise, uint8_t* rgb8, cudaStream_t st, float* linear) {
    if (!p) return fail(SR_ERR_INVALID_ARG, "params is NULL");
    if (ctx->device < 0) return fail(SR_ERR_STATE, "host-only context (device -1) cannot run device work");
    if (w == 0 || h == 0) return fail(SR_ERR_INVALID_ARG, "empty image");
    if (p->tonemapper != SR_TONEMAP_REINHARD && p->tonemapper != SR_TONEMAP_LINEAR_SMOOTH)
        return fail(SR_ERR_INVALID_ARG, "Unknown tonemapper: %d", p->tonemapper);
    ComposeConsts k;
    k.tonemapper = p->tonemapper;
    k.exposure = p->exposure;
    k.strength = p->denoise_strength;
    k.strength_max = p->denoise_strength_max;
    k.lum_boost = p->denoise_luminance_boost;
    k.lum_limit_inv = 1.0f / (p->denoise_luminance_limit * p->denoise_luminance_limit * 2.0f);
    k.normal_limit_inv = 1.0f / (p->denoise_normal_limit * p->denoise_normal_limit * 2.0f);
    k.depth_limit_inv = 1.0f / (p->denoise_depth_limit * p->denoise_depth_limit * 2.0f);
    // Filter / FilterFog radii (compose.cs:112-115, 210-213).
    float area_sqrt = std::sqrt((float)(int)(w * h));
    float rp = p->denoise_radius * area_sqrt;
    float rp_inv = 1.0f / (rp * rp * 2.0f);
    float rpf = p->denoise_fog_radius * area_sqrt;
    float rpf_inv = 1.0f / (rpf * rpf * 2.0f);
    k.radius = (int)std::ceil(rp * 3.0f);
    k.fog_radius = (int)std::ceil(rpf * 3.0f);
    if (k.radius < 0 || k.fog_radius < 0 || k.radius > 4096 || k.fog_radius > 4096)
        return fail(SR_ERR_INVALID_ARG, "denoise radius out of range");
    std::vector<float>& tab = ctx->table_host;
    tab.clear();
    build_table(tab, k.radius, rp_inv, 1.0f);
    size_t fog_off = tab.size();
    build_table(tab, k.fog_radius, rpf_inv, p->denoise_fog_strength);
    SR_CUDA(upload(ctx->compose_tables, tab.data(), tab.size() * sizeof(float), st), "upload tables");
    size_t n = (size_t)w * h;
    SR_CUDA(ctx->compose_scratch.reserve(n * 3 * sizeof(float4)), "alloc compose scratch");
    const float* d_tab = ctx->compose_tables.as<float>();
    SR_CUDA(launch_compose(in, w, h, k, d_tab, d_tab + fog_off, denoise, rgb8, ctx->compose_scratch.as<float4>(), st,
                           linear),
            "compose launch");
    return SR_OK;
}

SR_API int sr_compose_float_device(SrContext* ctx, const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* p,
                                   float* device_linear, uint8_t* device_rgb8, void* stream) {
    if (!ctx || !a || !device_linear) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (!a->radiance || !a->radiance_fog || !a->normals || !a->depth || !a->variance)
        return fail(SR_ERR_INVALID_ARG, "compose needs radiance, radiance_fog, normals, depth and variance");
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    DevAovs d{a->radiance, a->radiance_fog, a->normals, a->uv, a->depth, a->samples, a->variance};
    return compose_impl(ctx, d, w, h, p, true, device_rgb8, st, device_linear);
}

SR_API int sr_compose_device(SrContext* ctx, const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* p,
                             uint8_t* device_rgb8, void* stream) {
    if (!ctx || !a || !device_rgb8) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (!a->radiance || !a->radiance_fog || !a->normals || !a->depth || !a->variance)
        return fail(SR_ERR_INVALID_ARG, "compose needs radiance, radiance_fog, normals, depth and variance");
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    DevAovs d{a->radiance, a->radiance_fog, a->normals, a->uv, a->depth, a->samples, a->variance};
    return compose_impl(ctx, d, w, h, p, true, device_rgb8, st);
}

SR_API int sr_compose_device_static(SrContext* ctx, const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* p,
                                    uint8_t* device_rgb8, void* stream) {
    if (!ctx || !a || !p || !device_rgb8) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (!a->radiance || !a->radiance_fog || !a->normals || !a->depth || !a->variance)
        return fail(SR_ERR_INVALID_ARG, "compose needs radiance, radiance_fog, normals, depth and variance");
    if (ctx->device < 0) return fail(SR_ERR_STATE, "host-only context (device -1) cannot run device work");
    if (w == 0 || h == 0) return fail(SR_ERR_INVALID_ARG, "empty image");
    if (p->tonemapper != SR_TONEMAP_REINHARD && p->tonemapper != SR_TONEMAP_LINEAR_SMOOTH)
        return fail(SR_ERR_INVALID_ARG, "Unknown tonemapper: %d", p->tonemapper);
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    ComposeConsts k;
    k.tonemapper = p->tonemapper;
    k.exposure = p->exposure;
    k.strength = p->denoise_strength;
    k.strength_max = p->denoise_strength_max;
    k.lum_boost = p->denoise_luminance_boost;
    k.lum_limit_inv = 1.0f / (p->denoise_luminance_limit * p->denoise_luminance_limit * 2.0f);
    k.normal_limit_inv = 1.0f / (p->denoise_normal_limit * p->denoise_normal_limit * 2.0f);
    k.depth_limit_inv = 1.0f / (p->denoise_depth_limit * p->denoise_depth_limit * 2.0f);
    float area_sqrt = std::sqrt((float)(int)(w * h));
    float rp = p->denoise_radius * area_sqrt;
    float rpf = p->denoise_fog_radius * area_sqrt;
    k.radius = (int)std::ceil(rp * 3.0f);
    k.fog_radius = (int)std::ceil(rpf * 3.0f);
    if (k.radius < 0 || k.fog_radius < 0 || k.radius > 4096 || k.fog_radius > 4096)
        return fail(SR_ERR_INVALID_ARG, "denoise radius out of range");
    DevAovs d{a->radiance, a->radiance_fog, a->normals, a->uv, a->depth, a->samples, a->variance};
    size_t needed = 0;
    bool too_large = false;
    cudaError_t e = launch_compose_static(ctx->device, d, w, h, k, 1.0f / (rp * rp * 2.0f), 1.0f / (rpf * rpf * 2.0f),
                                          p->denoise_fog_strength, device_rgb8, st, &needed, &too_large);
    if (too_large)
        return fail(SR_ERR_INVALID_ARG,
                    "sr_compose_device_static: a %u-pixel-wide image with filter radius %d needs %zu bytes of "
                    "scratch per band, more than the fixed %zu-byte scratch array",
                    w, k.radius > k.fog_radius ? k.radius : k.fog_radius, needed, compose_static_capacity());
    SR_CUDA(e, "compose (static scratch)");
    return SR_OK;
}

static int compose_host(SrContext* ctx, const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* p,
                        uint8_t* rgb, bool denoise) {
    if (!ctx || !a || !rgb || !a->radiance || !a->radiance_fog) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (denoise && (!a->normals || !a->depth || !a->variance))
        return fail(SR_ERR_INVALID_ARG, "compose needs radiance, radiance_fog, normals, depth and variance");
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    size_t n = (size_t)w * h;
    SR_CUDA(ctx->compose_io.reserve(n * (12 + 12 + 12 + 4 + 4 + 3) + 256), "alloc compose io");
    char* b = ctx->compose_io.as<char>();
    DevAovs d{};
    d.radiance = (float*)b;
    d.radiance_fog = d.radiance + 3 * n;
    d.normals = d.radiance_fog + 3 * n;
    d.depth = d.normals + 3 * n;
    d.variance = d.depth + n;
    uint8_t* d_rgb = (uint8_t*)(d.variance + n);
    SR_CUDA(cudaMemcpyAsync(d.radiance, a->radiance, n * 12, cudaMemcpyHostToDevice, st), "copy AOVs");
    SR_CUDA(cudaMemcpyAsync(d.radiance_fog, a->radiance_fog, n * 12, cudaMemcpyHostToDevice, st), "copy AOVs");
    if (denoise) {
        SR_CUDA(cudaMemcpyAsync(d.normals, a->normals, n * 12, cudaMemcpyHostToDevice, st), "copy AOVs");
        SR_CUDA(cudaMemcpyAsync(d.depth, a->depth, n * 4, cudaMemcpyHostToDevice, st), "copy AOVs");
        SR_CUDA(cudaMemcpyAsync(d.variance, a->variance, n * 4, cudaMemcpyHostToDevice, st), "copy AOVs");
    } else {
        SR_CUDA(cudaMemsetAsync(d.normals, 0, n * 20, st), "clear AOVs");
    }
    int rc = compose_impl(ctx, d, w, h, p, denoise, d_rgb, st);
    if (rc) return rc;
    SR_CUDA(cudaMemcpyAsync(rgb, d_rgb, n * 3, cudaMemcpyDeviceToHost, st), "copy pixels");
    SR_CUDA(cudaStreamSynchronize(st), "compose");
    return SR_OK;
}

SR_API int sr_compose(SrContext* ctx, const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* p, uint8_t* rgb) {
    return compose_host(ctx, a, w, h, p, rgb, true);
}

SR_API int sr_render_compose(SrScene* s, const SrView* view, const SrRenderParams* params, const SrComposeParams* cp,
                             const SrAovs* host_out, uint8_t* host_rgb8) {
    if (!s || !params || !cp) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    size_t n = (size_t)params->width * params->height;
    DevAovs d;
    uint8_t* d_rgb;
    SR_CUDA(stage_aovs(s, n, d, &d_rgb), "alloc AOVs");
    int rc = render_into(s, view, params, d, st);
    if (rc) return rc;
    rc = compose_impl(s->ctx, d, params->width, params->height, cp, true, d_rgb, st);
    if (rc) return rc;
    if (host_out) {
        rc = copy_aovs_to_host(d, n, *host_out, st);
        if (rc) return rc;
    }
    if (host_rgb8) SR_CUDA(cudaMemcpyAsync(host_rgb8, d_rgb, n * 3, cudaMemcpyDeviceToHost, st), "copy pixels");
    SR_CUDA(cudaStreamSynchronize(st), "render_compose");
    if (s->counting)
        SR_CUDA(cudaMemcpy(s->last_counters, s->counters.ptr, sizeof(s->last_counters), cudaMemcpyDeviceToHost),
                "read counters");
    return check_device_error(s);
}

SR_API int sr_preview(SrContext* ctx, const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* p, uint8_t* rgb) {
    return compose_host(ctx, a, w, h, p, rgb, false);
}

}  // extern "C"

// ---- asset ingest (sr_ingest.cpp) ------------------------------------------------------------------

SR_API int sr_image_load(const char* path, uint32_t* width, uint32_t* height, uint32_t* channels, uint8_t* pixels,
                         uint64_t capacity) {
    if (!path || !width || !height || !channels) return fail(SR_ERR_INVALID_ARG, "sr_image_load: NULL argument");
    try {
        std::string p(path);
        std::vector<uint8_t> data;
        uint32_t w = 0, h = 0, ch = 3;
        size_t dot = p.find_last_of('.');
        if (dot != std::string::npos && p.substr(dot) == ".hdr") {
            load_hdr(p, w, h, data);
            ch = 4;
        } else {
            load_image(p, w, h, data);
        }
        *width = w, *height = h, *channels = ch;
        if (pixels) {
            if (capacity < data.size()) return fail(SR_ERR_INVALID_ARG, "sr_image_load: buffer of %llu bytes, need %zu",
                                                    (unsigned long long)capacity, data.size());
            std::memcpy(pixels, data.data(), data.size());
        }
    } catch (const IngestError& e) {
        return fail(SR_ERR_IO, "%s", e.what());
    }
    return SR_OK;
}

static int texture_from_file(SrContext* ctx, const std::string& path, int32_t encoding, float max_luminance,
                             int32_t filter, float tiling_x, float tiling_y, int32_t* out_id) {
    std::vector<uint8_t> data;
    uint32_t w = 0, h = 0;
    std::vector<float> texels;
    if (encoding == SR_TEXTURE_HDR) {
        load_hdr(path, w, h, data);
        texels.resize((size_t)w * h * 3);
        rgbe_to_texels(data.data(), (size_t)w * h, max_luminance, texels.data());
    } else {
        load_image(path, w, h, data);
        texels.resize((size_t)w * h * 3);
        rgb8_to_texels(data.data(), (size_t)w * h, encoding == SR_TEXTURE_SRGB, texels.data());
    }
    return sr_texture_create(ctx, texels.data(), w, h, filter, tiling_x, tiling_y, out_id);
}

SR_API int sr_texture_load(SrContext* ctx, const char* path, int32_t encoding, float max_luminance, int32_t filter,
                           float tiling_x, float tiling_y, int32_t* out_id) {
    if (!ctx || !path || !out_id) return fail(SR_ERR_INVALID_ARG, "sr_texture_load: NULL argument");
    if (encoding != SR_TEXTURE_SRGB && encoding != SR_TEXTURE_LINEAR && encoding != SR_TEXTURE_HDR)
        return fail(SR_ERR_INVALID_ARG, "sr_texture_load: bad encoding %d", encoding);
    try {
        return texture_from_file(ctx, path, encoding, max_luminance, filter, tiling_x, tiling_y, out_id);
    } catch (const IngestError& e) {
        return fail(SR_ERR_IO, "%s", e.what());
    }
}

SR_API int sr_obj_load(SrScene* s, const char* path, const SrTransform* transform, const SrMaterial* material,
                       int32_t smooth_normals, uint32_t* objects_added) {
    if (!s || !path) return fail(SR_ERR_INVALID_ARG, "sr_obj_load: NULL argument");
    if (s->built) return fail(SR_ERR_STATE, "Scene already built");
    SrContext* ctx = s->ctx;
    const SrTransform identity{{0, 0, 0}, {0, 0, 0, 1}, {1, 1, 1}};
    const SrMaterial fallback{{1, 1, 1}, 1.0f, 0.0f, 0.0f, 1.5f, {0, 0, 0}, -1, -1, -1, -1};  // Material(White, 1)
    const SrTransform& tr = transform ? *transform : identity;
    ObjResult r;
    std::vector<SrMaterial> mats;  // per object
    try {
        r = parse_obj(path, smooth_normals != 0);
        std::map<const ObjImage*, int32_t> uploaded;  // one texture per decoded map
        for (const ObjObject& o : r.objects) {
            const ObjMaterial& m = o.material;
            SrMaterial sm = material ? *material : fallback;
            if (o.has_material) {
                sm = SrMaterial{{m.albedo[0], m.albedo[1], m.albedo[2]}, m.roughness, m.metallic, m.transparency, m.ior,
                                {m.radiance[0], m.radiance[1], m.radiance[2]}, -1, -1, -1, -1};
                const ObjImagePtr* maps[4] = {&m.color_map, &m.roughness_map, &m.metallic_map, &m.normal_map};
                int32_t* ids[4] = {&sm.color_texture, &sm.roughness_texture, &sm.metallic_texture, &sm.normal_texture};
                for (int k = 0; k < 4; ++k) {
                    const ObjImage* img = maps[k]->get();
                    if (!img) continue;
                    auto it = uploaded.find(img);
                    if (it == uploaded.end()) {
                        int32_t id = -1;  // Texture defaults: bilinear, tiling (1, 1) (texture.cs:17-30)
                        if (int rc = sr_texture_create(ctx, img->texels.data(), img->width, img->height, 0, 1.0f, 1.0f, &id))
                            return rc;
                        it = uploaded.emplace(img, id).first;
                    }
                    *ids[k] = it->second;
                }
            }
            mats.push_back(sm);
        }
    } catch (const IngestError& e) {
        return fail(SR_ERR_IO, "%s", e.what());
    }
    uint32_t added = 0;
    for (const ObjObject& o : r.objects) {
        int32_t mesh = -1, index = -1;
        if (int rc = sr_mesh_create(ctx, o.triangles.data(), (uint32_t)o.triangles.size(), &mesh)) return rc;
        SrShape shape{SR_SHAPE_MESH, mesh, {0, 0, 0, 0, 0, 0}};
        if (int rc = sr_scene_add_object(s, &tr, &mats[added], &shape, &index)) return rc;
        s->object_names.resize(s->objects.size());
        s->object_names[index] = o.name;
        ++added;
    }
    if (objects_added) *objects_added = added;
    return SR_OK;
}

SR_API int sr_texture_export(SrContext* ctx, int32_t id, uint32_t* width, uint32_t* height, float* texels) {
    if (!ctx || !valid_texture(ctx, id) || id < 0) return fail(SR_ERR_INVALID_ARG, "bad texture id");
    const TextureHost& t = *ctx->textures[id];
    if (width) *width = t.width;
    if (height) *height = t.height;
    if (texels) std::memcpy(texels, t.texels.data(), t.texels.size() * sizeof(float));
    return SR_OK;
}

SR_API int sr_mesh_export(SrContext* ctx, int32_t mesh, uint32_t* count, SrTriangle* triangles) {
    if (!ctx || mesh < 0 || mesh >= (int32_t)ctx->meshes.size()) return fail(SR_ERR_INVALID_ARG, "bad mesh id");
    const MeshHost& m = *ctx->meshes[mesh];
    if (count) *count = (uint32_t)m.tris.size();
    if (triangles) std::memcpy(triangles, m.tris.data(), m.tris.size() * sizeof(SrTriangle));
    return SR_OK;
}

SR_API int sr_scene_object_info(SrScene* s, uint32_t index, SrTransform* transform, SrMaterial* material,
                                SrShape* shape, char* name, uint32_t name_capacity) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "scene is NULL");
    if (index >= s->objects.size()) return fail(SR_ERR_INVALID_ARG, "object index %u of %zu", index, s->objects.size());
    const SrScene::Obj& o = s->objects[index];
    if (transform) *transform = o.tr;
    if (material) *material = o.mat;
    if (shape) *shape = o.shape;
    if (name && name_capacity) {
        std::string n = index < s->object_names.size() ? s->object_names[index] : std::string();
        std::snprintf(name, name_capacity, "%s", n.c_str());
    }
    return SR_OK;
}

SR_API int sr_scene_object_count(SrScene* s, uint32_t* count) {
    if (!s || !count) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    *count = (uint32_t)s->objects.size();
    return SR_OK;
}

// ---- AOV images, overlay, image files (sr_image.cpp, sr_overlay.cu) --------------------------------

static int aov_image_impl(SrContext* ctx, const DevAovs& d, uint32_t w, uint32_t h, int32_t kind,
                          const SrAovImageParams* p, uint8_t* d_rgb, uint8_t* d_lut, cudaStream_t st) {
    float var_div = 1.0f, min_s = 1.0f, log_range = 1.0f;
    uint32_t lut_n = 0;
    if (kind == SR_AOV_VARIANCE) var_div = p->variance_threshold * 2.0f;
    if (kind == SR_AOV_SAMPLES) {
        std::vector<uint8_t> lut = samples_table(p->min_samples, p->max_samples, &log_range);
        lut_n = (uint32_t)lut.size();
        min_s = (float)p->min_samples;
        SR_CUDA(cudaMemcpyAsync(d_lut, lut.data(), lut.size(), cudaMemcpyHostToDevice, st), "copy samples table");
    }
    SR_CUDA(launch_aov_image(d, w * h, kind, var_div, d_lut, lut_n, min_s, log_range, d_rgb, st), "aov image");
    (void)ctx;
    return SR_OK;
}

static int aov_image_check(const SrAovs* a, int32_t kind, const SrAovImageParams* p) {
    if (!a) return fail(SR_ERR_INVALID_ARG, "NULL AOVs");
    const void* plane = kind == SR_AOV_NORMAL ? (const void*)a->normals
                      : kind == SR_AOV_DEPTH ? (const void*)a->depth
                      : kind == SR_AOV_VARIANCE ? (const void*)a->variance
                      : kind == SR_AOV_SAMPLES ? (const void*)a->samples
                      : kind == SR_AOV_UV ? (const void*)a->uv : nullptr;
    if (kind < SR_AOV_NORMAL || kind > SR_AOV_UV) return fail(SR_ERR_INVALID_ARG, "bad AOV kind %d", kind);
    if (!plane) return fail(SR_ERR_INVALID_ARG, "the AOV plane of kind %d is NULL", kind);
    if ((kind == SR_AOV_VARIANCE || kind == SR_AOV_SAMPLES) && !p)
        return fail(SR_ERR_INVALID_ARG, "AOV kind %d needs parameters", kind);
    if (kind == SR_AOV_SAMPLES && (p->min_samples == 0 || p->max_samples < p->min_samples || p->max_samples > (1u << 24)))
        return fail(SR_ERR_INVALID_ARG, "need 0 < min_samples <= max_samples <= 2^24");
    return SR_OK;
}

SR_API int sr_aov_image(SrContext* ctx, const SrAovs* a, uint32_t w, uint32_t h, int32_t kind,
                        const SrAovImageParams* p, uint8_t* rgb) {
    if (!ctx || !rgb) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = aov_image_check(a, kind, p)) return rc;
    if (ctx->device < 0) return fail(SR_ERR_STATE, "context has no device");
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    const size_t n = (size_t)w * h;
    const size_t lut_bytes = kind == SR_AOV_SAMPLES ? (size_t)p->max_samples + 2 : 0;
    SR_CUDA(ctx->image_io.reserve(n * 12 + n * 3 + lut_bytes + 256), "alloc AOV image io");
    char* b = ctx->image_io.as<char>();
    DevAovs d{};
    size_t plane_bytes = 0;
    const void* src = nullptr;
    switch (kind) {
        case SR_AOV_NORMAL: d.normals = (float*)b, src = a->normals, plane_bytes = n * 12; break;
        case SR_AOV_DEPTH: d.depth = (float*)b, src = a->depth, plane_bytes = n * 4; break;
        case SR_AOV_VARIANCE: d.variance = (float*)b, src = a->variance, plane_bytes = n * 4; break;
        case SR_AOV_SAMPLES: d.samples = (uint32_t*)b, src = a->samples, plane_bytes = n * 4; break;
        default: d.uv = (float*)b, src = a->uv, plane_bytes = n * 8; break;
    }
    uint8_t* d_rgb = (uint8_t*)(b + n * 12);
    uint8_t* d_lut = d_rgb + n * 3;
    if (n) SR_CUDA(cudaMemcpyAsync(b, src, plane_bytes, cudaMemcpyHostToDevice, st), "copy AOV plane");
    if (int rc = aov_image_impl(ctx, d, w, h, kind, p, d_rgb, d_lut, st)) return rc;
    if (n) SR_CUDA(cudaMemcpyAsync(rgb, d_rgb, n * 3, cudaMemcpyDeviceToHost, st), "copy pixels");
    SR_CUDA(cudaStreamSynchronize(st), "aov image");
    return SR_OK;
}

SR_API int sr_aov_image_device(SrContext* ctx, const SrAovs* a, uint32_t w, uint32_t h, int32_t kind,
                               const SrAovImageParams* p, uint8_t* d_rgb, void* stream) {
    if (!ctx || !d_rgb) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = aov_image_check(a, kind, p)) return rc;
    if (ctx->device < 0) return fail(SR_ERR_STATE, "context has no device");
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    DevAovs d{a->radiance, a->radiance_fog, a->normals, a->uv, a->depth, a->samples, a->variance};
    const size_t lut_bytes = kind == SR_AOV_SAMPLES ? (size_t)p->max_samples + 2 : 16;
    SR_CUDA(ctx->overlay_scratch.reserve(lut_bytes), "alloc samples table");
    return aov_image_impl(ctx, d, w, h, kind, p, d_rgb, ctx->overlay_scratch.as<uint8_t>(), st);
}

// Plans on the host, then stages ops, colours and the font next to the owner plane in `scratch`.
static int overlay_impl(SrContext* ctx, DevBuf& scratch, uint8_t* d_rgb, uint32_t w, uint32_t h, const SrView* view,
                        const float* d_depth, const SrOverlayLine* lines, uint32_t nl, const SrOverlayText* texts,
                        uint32_t nt, const SrFont* font, cudaStream_t st) {
    OverlayPlan plan;
    try {
        plan = plan_overlay(w, h, *view, lines, nl, texts, nt, font);
    } catch (const ImageError& e) {
        return fail(SR_ERR_INVALID_ARG, "%s", e.what());
    }
    const size_t n = (size_t)w * h;
    const size_t font_bytes = font && font->glyphs ? (size_t)(font->last_char - font->first_char + 1) * 8 : 0;
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_owner = 0, o_lines = up(n * 4), o_glyphs = o_lines + up(plan.lines.size() * sizeof(OverlayLineOp));
    const size_t o_colors = o_glyphs + up(plan.glyphs.size() * sizeof(OverlayGlyphOp));
    const size_t o_font = o_colors + up(plan.colors.size() * 4), total = o_font + up(font_bytes) + 256;
    SR_CUDA(scratch.reserve(total), "alloc overlay scratch");
    char* b = scratch.as<char>();
    if (!plan.lines.empty())
        SR_CUDA(cudaMemcpyAsync(b + o_lines, plan.lines.data(), plan.lines.size() * sizeof(OverlayLineOp),
                                cudaMemcpyHostToDevice, st), "copy overlay lines");
    if (!plan.glyphs.empty())
        SR_CUDA(cudaMemcpyAsync(b + o_glyphs, plan.glyphs.data(), plan.glyphs.size() * sizeof(OverlayGlyphOp),
                                cudaMemcpyHostToDevice, st), "copy overlay glyphs");
    if (!plan.colors.empty())
        SR_CUDA(cudaMemcpyAsync(b + o_colors, plan.colors.data(), plan.colors.size() * 4, cudaMemcpyHostToDevice, st),
                "copy overlay colours");
    if (font_bytes)
        SR_CUDA(cudaMemcpyAsync(b + o_font, font->glyphs, font_bytes, cudaMemcpyHostToDevice, st), "copy font");
    SR_CUDA(launch_overlay((const OverlayLineOp*)(b + o_lines), (uint32_t)plan.lines.size(),
                           (const OverlayGlyphOp*)(b + o_glyphs), (uint32_t)plan.glyphs.size(),
                           (const uint8_t*)(b + o_font), (const uint32_t*)(b + o_colors), d_depth, w, h,
                           (int32_t*)(b + o_owner), d_rgb, st),
            "overlay");
    (void)ctx;
    return SR_OK;
}

static int overlay_check(SrContext* ctx, const void* rgb, uint32_t w, uint32_t h, const SrView* view,
                         const SrOverlayLine* lines, uint32_t nl, const SrOverlayText* texts, uint32_t nt,
                         const SrFont* font) {
    if (!ctx || !rgb || !view) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (w == 0 || h == 0) return fail(SR_ERR_INVALID_ARG, "empty image");
    if ((nl && !lines) || (nt && !texts)) return fail(SR_ERR_INVALID_ARG, "NULL overlay entries");
    if (nt && (!font || !font->glyphs)) return fail(SR_ERR_INVALID_ARG, "overlay text needs a font");
    if (font && font->glyphs && !(0 <= font->first_char && font->first_char <= font->last_char && font->last_char <= 255))
        return fail(SR_ERR_INVALID_ARG, "font range must be 0 <= first_char <= last_char <= 255");
    for (uint32_t i = 0; i < nt; ++i)
        if (!texts[i].text) return fail(SR_ERR_INVALID_ARG, "overlay text %u is NULL", i);
    if (ctx->device < 0) return fail(SR_ERR_STATE, "context has no device");
    return SR_OK;
}

SR_API int sr_overlay_draw(SrContext* ctx, uint8_t* rgb, uint32_t w, uint32_t h, const SrView* view,
                           const float* depth, const SrOverlayLine* lines, uint32_t nl, const SrOverlayText* texts,
                           uint32_t nt, const SrFont* font) {
    if (int rc = overlay_check(ctx, rgb, w, h, view, lines, nl, texts, nt, font)) return rc;
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    const size_t n = (size_t)w * h;
    SR_CUDA(ctx->image_io.reserve(n * 3 + n * 4 + 512), "alloc overlay io");
    uint8_t* d_rgb = ctx->image_io.as<uint8_t>();
    float* d_depth = depth ? (float*)(d_rgb + ((n * 3 + 255) & ~(size_t)255)) : nullptr;
    SR_CUDA(cudaMemcpyAsync(d_rgb, rgb, n * 3, cudaMemcpyHostToDevice, st), "copy image");
    if (depth) SR_CUDA(cudaMemcpyAsync(d_depth, depth, n * 4, cudaMemcpyHostToDevice, st), "copy depth");
    if (int rc = overlay_impl(ctx, ctx->overlay_scratch, d_rgb, w, h, view, d_depth, lines, nl, texts, nt, font, st))
        return rc;
    SR_CUDA(cudaMemcpyAsync(rgb, d_rgb, n * 3, cudaMemcpyDeviceToHost, st), "copy image");
    SR_CUDA(cudaStreamSynchronize(st), "overlay");
    return SR_OK;
}

SR_API int sr_overlay_draw_device(SrContext* ctx, uint8_t* d_rgb, uint32_t w, uint32_t h, const SrView* view,
                                  const float* d_depth, const SrOverlayLine* lines, uint32_t nl,
                                  const SrOverlayText* texts, uint32_t nt, const SrFont* font, void* stream) {
    if (int rc = overlay_check(ctx, d_rgb, w, h, view, lines, nl, texts, nt, font)) return rc;
    SR_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return overlay_impl(ctx, ctx->overlay_scratch, d_rgb, w, h, view, d_depth, lines, nl, texts, nt, font, st);
}

SR_API int sr_image_save(const char* path, uint32_t w, uint32_t h, const uint8_t* rgb) {
    if (!path || (!rgb && w && h)) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    try {
        save_image(path, w, h, rgb);
    } catch (const ImageError& e) {
        return fail(SR_ERR_IO, "%s", e.what());
    }
    return SR_OK;
}

// Checks shared by the adjoint entry points; dv / dp / st out.
static int adjoint_prepare(SrScene* s, const SrView* view, const SrRenderParams* params, const SrAovs* fwd,
                           const float* d_image, void* stream, DevView& dv, DevParams& dp, cudaStream_t& st) {
    if (!s || !fwd || !d_image) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    if (!fwd->radiance || !fwd->radiance_fog || !fwd->samples)
        return fail(SR_ERR_INVALID_ARG, "the adjoint needs the forward radiance, radiance_fog and samples planes");
    if (s->dev.has_transparent) return fail(SR_ERR_STATE, "the adjoint does not support transparent materials");
    if (int rc = make_view(view, params, dv, dp)) return rc;
    if (dp.bounces > 16) return fail(SR_ERR_INVALID_ARG, "the adjoint supports at most 16 bounces");
    dp.seed = s->seed;  // replay the forward render's random numbers
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    st = stream ? (cudaStream_t)stream : s->ctx->stream;
    return SR_OK;
}

static bool scene_texture(SrScene* s, int32_t texture) {
    return texture >= 0 && (size_t)texture < s->tex_offset.size();
}

// The adjoint of a finished render (forward planes f) in the scene's replay form: the wavefront
// replay (sr_wave_adjoint.cu; host loop when the scene renders with one, else the graph) or the
// per-pixel replay kernel (sr_adjoint.cu).  parameter 0-2 names one gradient, 3 all of them.
static int run_adjoint(SrScene* s, const DevView& dv, const DevParams& dp, const DevAovs& f, const float* d_image,
                       int parameter, int tex_a, float* grad_a, int tex_r, float* grad_r, float* grad_f,
                       float* replay, cudaStream_t st) {
    if (s->adjoint_replay == SR_ADJOINT_REPLAY_PIXEL) {
        SR_CUDA(launch_adjoint(launch_scene(s), dv, dp, f, d_image, parameter, tex_a, grad_a, tex_r, grad_r, grad_f,
                               replay, s->err.as<uint32_t>(), st),
                "adjoint launch");
        return SR_OK;
    }
    AdjPass a{};
    a.d_image = d_image;
    a.fwd_samples = f.samples;
    a.replay = replay;
    a.tex_a = grad_a ? tex_a : -1;
    a.grad_a = grad_a;
    a.tex_r = grad_r ? tex_r : -1;
    a.grad_r = grad_r;
    a.grad_f = grad_f;
    const DevAovs none{};  // a replay writes no AOVs
    return render_wavefront(s, dv, dp, none, nullptr, st, s->render_mode != SR_RENDER_WAVEFRONT, kAdjReplay, &a);
}

SR_API int sr_adjoint_texture(SrScene* s, const SrView* view, const SrRenderParams* params, const SrAovs* fwd,
                              const float* d_image, int32_t texture, int32_t parameter, float* grad, float* replay,
                              void* stream) {
    if (!grad) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (parameter != SR_ADJOINT_ALBEDO && parameter != SR_ADJOINT_ROUGHNESS && parameter != SR_ADJOINT_FOG_DENSITY)
        return fail(SR_ERR_INVALID_ARG, "unknown adjoint parameter %d", parameter);
    DevView dv;
    DevParams dp;
    cudaStream_t st;
    if (int rc = adjoint_prepare(s, view, params, fwd, d_image, stream, dv, dp, st)) return rc;
    if (parameter == SR_ADJOINT_FOG_DENSITY) {
        if (!s->dev.has_fog) return fail(SR_ERR_STATE, "the scene has no fog");
    } else if (!scene_texture(s, texture)) {
        return fail(SR_ERR_INVALID_ARG, "texture %d is not part of the scene", texture);
    }
    DevAovs f{fwd->radiance, fwd->radiance_fog, nullptr, nullptr, nullptr, fwd->samples, nullptr};
    const bool a = parameter == SR_ADJOINT_ALBEDO, r = parameter == SR_ADJOINT_ROUGHNESS;
    return run_adjoint(s, dv, dp, f, d_image, parameter, a ? texture : -1, a ? grad : nullptr, r ? texture : -1,
                       r ? grad : nullptr, a || r ? nullptr : grad, replay, st);
}

SR_API int sr_adjoint_all(SrScene* s, const SrView* view, const SrRenderParams* params, const SrAovs* fwd,
                          const float* d_image, int32_t albedo_texture, float* albedo_grad, int32_t roughness_texture,
                          float* roughness_grad, float* fog_density_grad, float* replay, void* stream) {
    DevView dv;
    DevParams dp;
    cudaStream_t st;
    if (int rc = adjoint_prepare(s, view, params, fwd, d_image, stream, dv, dp, st)) return rc;
    if (albedo_grad && !scene_texture(s, albedo_texture))
        return fail(SR_ERR_INVALID_ARG, "albedo texture %d is not part of the scene", albedo_texture);
    if (roughness_grad && !scene_texture(s, roughness_texture))
        return fail(SR_ERR_INVALID_ARG, "roughness texture %d is not part of the scene", roughness_texture);
    if (fog_density_grad && !s->dev.has_fog) return fail(SR_ERR_STATE, "the scene has no fog");
    if (!albedo_grad && !roughness_grad && !fog_density_grad) return SR_OK;
    DevAovs f{fwd->radiance, fwd->radiance_fog, nullptr, nullptr, nullptr, fwd->samples, nullptr};
    return run_adjoint(s, dv, dp, f, d_image, 3, albedo_grad ? albedo_texture : -1, albedo_grad,
                       roughness_grad ? roughness_texture : -1, roughness_grad, fog_density_grad, replay, st);
}

SR_API int sr_adjoint_albedo(SrScene* s, const SrView* view, const SrRenderParams* params, const SrAovs* fwd,
                             const float* d_image, int32_t texture, float* grad, float* replay, void* stream) {
    return sr_adjoint_texture(s, view, params, fwd, d_image, texture, SR_ADJOINT_ALBEDO, grad, replay, stream);
}

SR_API int sr_scene_set_adjoint_replay(SrScene* s, int32_t form) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (form != SR_ADJOINT_REPLAY_WAVEFRONT && form != SR_ADJOINT_REPLAY_PIXEL)
        return fail(SR_ERR_INVALID_ARG, "unknown adjoint replay form %d", form);
    s->adjoint_replay = form;
    return SR_OK;
}

SR_API int sr_render_checkpointed(SrScene* s, const SrView* view, const SrRenderParams* params, const SrAovs* out,
                                  void* stream, uint64_t* bytes_kept) {
    if (!s || !out || !params) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    if (!out->radiance || !out->radiance_fog || !out->normals || !out->uv || !out->depth || !out->samples || !out->variance)
        return fail(SR_ERR_INVALID_ARG, "sr_render_checkpointed needs all seven AOV planes");
    if (s->dev.has_transparent) return fail(SR_ERR_STATE, "the adjoint does not support transparent materials");
    DevView dv;
    DevParams dp;
    if (int rc = make_view(view, params, dv, dp)) return rc;
    if (dp.bounces > 16) return fail(SR_ERR_INVALID_ARG, "the adjoint supports at most 16 bounces");
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : s->ctx->stream;
    if (int rc = progress_begin(s, dp.width * dp.height)) return rc;
    s->ckpt_valid = false;
    DevAovs d{out->radiance, out->radiance_fog, out->normals, out->uv, out->depth, out->samples, out->variance};
    AdjPass a{};
    WaveLaunch L;
    if (int rc = render_wavefront(s, dv, dp, d, nullptr, st, s->render_mode != SR_RENDER_WAVEFRONT, kAdjRecord, &a, &L))
        return rc;
    SR_CUDA(cudaEventRecord(s->progress_event, st), "progress event");
    a.fwd_samples = out->samples;  // the sweep's sample counts
    s->ckpt_valid = true;
    s->ckpt_launch = L;
    s->ckpt_pass = a;
    if (bytes_kept)
        *bytes_kept = (uint64_t)s->wave_slots * a.samples_kept * (a.vper * kAdjVertexF4 * sizeof(float4) + 1);
    return SR_OK;
}

SR_API int sr_adjoint_checkpointed(SrScene* s, const float* d_image, int32_t albedo_texture, float* albedo_grad,
                                   int32_t roughness_texture, float* roughness_grad, float* fog_density_grad,
                                   void* stream) {
    if (!s || !d_image) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = need_device(s)) return rc;
    if (!s->ckpt_valid) return fail(SR_ERR_STATE, "no checkpointed render on this scene (sr_render_checkpointed)");
    if (albedo_grad && !scene_texture(s, albedo_texture))
        return fail(SR_ERR_INVALID_ARG, "albedo texture %d is not part of the scene", albedo_texture);
    if (roughness_grad && !scene_texture(s, roughness_texture))
        return fail(SR_ERR_INVALID_ARG, "roughness texture %d is not part of the scene", roughness_texture);
    if (fog_density_grad && !s->dev.has_fog) return fail(SR_ERR_STATE, "the scene has no fog");
    if (!albedo_grad && !roughness_grad && !fog_density_grad) return SR_OK;
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : s->ctx->stream;
    AdjPass a = s->ckpt_pass;
    a.d_image = d_image;
    a.tex_a = albedo_grad ? albedo_texture : -1;
    a.grad_a = albedo_grad;
    a.tex_r = roughness_grad ? roughness_texture : -1;
    a.grad_r = roughness_grad;
    a.grad_f = fog_density_grad;
    SR_CUDA(cudaMemcpyAsync(s->ckpt_pass_dev.ptr, &a, sizeof(AdjPass), cudaMemcpyHostToDevice, st), "upload adjoint pass");
    SR_CUDA(launch_adjoint_checkpoint(s->ckpt_launch, d_image, a.fwd_samples, st), "checkpoint sweep");
    return SR_OK;
}

SR_API int sr_scene_release_checkpoint(SrScene* s) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (s->ctx->device >= 0) cudaSetDevice(s->ctx->device);
    s->ckpt_valid = false;
    s->ckpt_vbuf.release();
    s->ckpt_vcount.release();
    return SR_OK;
}

SR_API int sr_scene_update_fog_density(SrScene* s, float density) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (!s->built) return fail(SR_ERR_STATE, "Scene not built");
    if (!s->has_fog) return fail(SR_ERR_STATE, "the scene has no fog");
    if (!(density > 0.0f) || !std::isfinite(density)) return fail(SR_ERR_INVALID_ARG, "fog density must be > 0");
    s->fog.density = density;
    s->dev.fog_density = density;  // kernels take the scene by value; a cached graph is rebuilt
    return SR_OK;
}

static int updatable_texture(SrScene* s, int32_t texture) {
    if (int rc = need_device(s)) return rc;
    if (texture < 0 || (size_t)texture >= s->tex_offset.size())
        return fail(SR_ERR_INVALID_ARG, "texture %d is not part of the scene", texture);
    if (s->sky_kind == 0 && s->sky_texture == texture)
        return fail(SR_ERR_INVALID_ARG, "texture %d is the sky texture", texture);
    return SR_OK;
}

SR_API int sr_scene_update_texture(SrScene* s, int32_t texture, const float* texels_rgb) {
    if (!s || !texels_rgb) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = updatable_texture(s, texture)) return rc;
    const TextureHost& t = *s->ctx->textures[texture];
    const size_t n = (size_t)t.width * t.height;
    std::vector<float4> rec(n);
    for (size_t k = 0; k < n; ++k) rec[k] = mk4(texels_rgb[3 * k], texels_rgb[3 * k + 1], texels_rgb[3 * k + 2], 0.0f);
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    SR_CUDA(cudaMemcpyAsync(s->texels.as<float4>() + s->tex_offset[texture], rec.data(), n * sizeof(float4),
                            cudaMemcpyHostToDevice, st),
            "upload texels");
    SR_CUDA(cudaStreamSynchronize(st), "upload texels");
    return SR_OK;
}

SR_API int sr_scene_update_texture_device(SrScene* s, int32_t texture, const float* d_texels_rgb, void* stream) {
    if (!s || !d_texels_rgb) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (int rc = updatable_texture(s, texture)) return rc;
    const TextureHost& t = *s->ctx->textures[texture];
    SR_CUDA(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : s->ctx->stream;
    SR_CUDA(launch_texels_from_rgb(d_texels_rgb, s->texels.as<float4>() + s->tex_offset[texture],
                                   (size_t)t.width * t.height, st),
            "update texels");
    return SR_OK;
}

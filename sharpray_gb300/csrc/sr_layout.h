// sr_layout.h — device-resident scene layout shared by the host builder (sr_host.cpp) and the
// kernels.  All records are 16-byte aligned so that every field is fetched with 128-bit loads.
//
// HBM layout of one built scene:
//   nodes   : float4[2 * N]   every BVH node of every mesh plus the scene BVH, 32 B per node:
//             {min.xyz, child}, {max.xyz, count} (child/count stored as int bits).  Node order
//             inside each tree is the reference's (bvh.cs), shifted by one slot so that the two
//             children of a node (always consecutive) start on a 64-byte boundary.  `child` is
//             the global node slot for interior nodes and the global triangle (or object)
//             position for leaves.
//   tris    : float4[3 * T]   triangles in BVH-leaf order: {A.xyz, original index}, {B-A}, {C-A}.
//   attrs   : float4[7 * T]   per-corner normals, tangents and uvs in the same order (108 B + pad).
//   objects : DevObject[O]    objects in scene-BVH leaf order.
//   texels  : float4[...]     all textures, one float4 per texel (rgb + pad).
#pragma once

#include <cstdint>

#include "../../include/sharpray.h"

#if defined(__CUDACC__)
#define SR_ALIGN16 __align__(16)
#else
#define SR_ALIGN16 alignas(16)
#include <vector_types.h>
#endif

namespace sr {

enum : uint32_t {
    SR_DEVERR_STACK = 1u,  // traversal stack would exceed its capacity
    SR_DEVERR_LOOP = 2u,   // a traversal, shadow or bounce loop exceeded its iteration cap
};
// Default cap on the actions (node visits, leaf steps) of one traversal.  A well-formed tree of N
// nodes needs at most about 2N; the cap turns a malformed tree into an error word instead of a
// hang.  A scene's tuning can lower it (SrTuning::max_traversal_steps).
constexpr uint32_t kDefaultMaxActions = 1u << 24;

struct SR_ALIGN16 DevObject {
    float4 pos_kind;    // transform position, shape kind (int bits)
    float4 rot;         // transform rotation quaternion
    float4 scale_root;  // transform scale, mesh BVH root slot (int bits)
    float4 shape0;      // sphere center + radius | box min
    float4 shape1;      // box max
    int32_t index;      // original object index (AddObject order)
    int32_t pad[3];
};

struct SR_ALIGN16 DevMaterial {
    float4 albedo_rough;  // albedo.rgb, roughness
    float4 params;        // metallic, transparency, ior, f0 = ((ior-1)/(ior+1))^2
    float4 radiance;      // emitted radiance.rgb, pad
    int32_t tex[4];       // color, roughness, metallic, normal texture ids (-1 = none)
};

struct SR_ALIGN16 DevTexture {
    uint32_t width, height;
    int32_t filter;
    float tiling_x, tiling_y;
    uint32_t pad;
    uint64_t offset;  // first texel in the texel array
};

struct SR_ALIGN16 DevSky {
    int32_t kind;  // 0 texture, 1 procedural
    int32_t texture;
    float multiplier;
    float pdf_scale;
    float cdf_total;
    float sun_cos;
    float sun_pdf_denom;
    float pad;
    float4 rot, rot_inv;
    const float* cdf_marginal;       // height + 1 floats
    const float* cdf_cond;           // height * (width + 1) floats
    const uint32_t* guide_marginal;  // height + 1 bucket bounds of the marginal search
    const uint32_t* guide_cond;      // height * (width + 1) bucket bounds of the row searches
    const float4* center;            // per texel: the sky radiance toward its centre (xyz) and its light
                                     // pdf (w), evaluated on the device at scene build (null: none)
    float4 top, middle, bottom, sun_dir, sun_radiance, sun_rot;
};

struct SR_ALIGN16 DevScene {
    const float4* nodes;
    const float4* tris;
    const float4* attrs;
    const DevObject* objects;
    const DevMaterial* materials;  // indexed by original object index
    const DevTexture* textures;
    const float4* texels;
    DevSky sky;
    int32_t tlas_root;  // slot of the scene-BVH root, -1 = no objects
    int32_t has_fog;
    int32_t has_transparent;
    int32_t object_count;
    int32_t general;  // needs the general kernels (analytic shapes, transparency, normal maps,
                      // procedural sky); 0 = meshes + texture sky only
    uint32_t max_actions;  // cap on the actions of one traversal (kDefaultMaxActions unless tuned)
    int32_t pad1[2];
    float fog_density, fog_falloff, fog_g;
    float fog_top;  // homogeneous fog (falloff 0): the medium's top height; +inf for the height fog
    float4 fog_color;
};

// Camera constants of View.Ray (math.cs:1613-1636) that do not depend on the sample.
struct SR_ALIGN16 DevView {
    float4 origin;  // Pos + Rot * (0, 0, near)
    float4 rot;
    float tan_h, tan_v, pad0, pad1;
};

struct SR_ALIGN16 DevParams {
    uint32_t width, height, min_samples, max_samples;
    uint32_t bounces;
    float variance_threshold, indirect_clamp, aspect;
    uint32_t seed;  // random-number stream of the render (0: the reference's Rng(x, y))
    uint32_t pad[3];
};

}  // namespace sr

// sr_path.cuh — path-level pieces of Scene.Sample shared by the megakernel and the wavefront
// kernels: surface lookup after a hit, shadow transmittance, sky-light sampling, Russian roulette,
// the adaptive-sampling statistic and the camera ray.
#pragma once

#include "sr_device.cuh"
#include "sr_kernels.h"

namespace sr {

struct Fragment {
    Col radiance, radiance_fog;
    bool has_primary;  // normal / uv / depth of the primary hit are set
    V3 normal;
    V2 uv;
    float depth;
};

struct SurfHit {
    Surface surf;
    float dist;
    int32_t material;  // index into DevScene::materials
};

// The Surface of a scene hit: Scene.Trace after the BVH query (scene.cs:608-621): inflate the
// winning hit, then the material's texture lookups, normal map and re-orthogonalised tangent.
template <bool COUNT, bool GENERAL = true>
__device__ __forceinline__ void surface_from_hit(const DevScene& S, const Ray& ray, const Hit& hit, SurfHit& out,
                                                 Ctr& c) {
    ShapeHit h = world_hit<COUNT, GENERAL>(S, ray, hit, c);
    const DevObject& o = S.objects[hit.obj];
    const DevMaterial& m = S.materials[o.index];
    float4 ar = m.albedo_rough;
    float4 mp = m.params;
    Col albedo = (m.tex[0] >= 0 ? tex_sample<COUNT>(S, m.tex[0], h.uv, c) : white()) * col3(ar);
    float roughness = (m.tex[1] >= 0 ? tex_sample<COUNT>(S, m.tex[1], h.uv, c).r : 1.0f) * ar.w;
    float metallic = (m.tex[2] >= 0 ? tex_sample<COUNT>(S, m.tex[2], h.uv, c).r : 1.0f) * mp.x;
    V3 normal = h.norm;
    if (GENERAL && m.tex[3] >= 0) {
        Col nc = tex_sample<COUNT>(S, m.tex[3], h.uv, c);
        V3 tn = normalize_or(V3{nc.r * 2.0f - 1.0f, -(nc.g * 2.0f - 1.0f), nc.b * 2.0f - 1.0f}, up3());
        normal = normalize_or(from_tangent_space(tn, h.tan, h.norm), h.norm);
    }
    V3 txyz = xyz(h.tan);
    V3 tdir = normalize_or(txyz - dot(txyz, normal) * normal, txyz);
    Surface& s = out.surf;
    s.radiance = col3(m.radiance);
    s.albedo = albedo;
    s.roughness = roughness;
    s.metallic = metallic;
    s.transparency = mp.y;
    s.ior = mp.z;
    s.f0 = mp.w;
    s.normal = normal;
    s.normal_geo = h.norm_geo;
    s.tangent = {tdir.x, tdir.y, tdir.z, h.tan.w};
    s.uv = h.uv;
    out.dist = h.dist;
    out.material = o.index;
}

// Scene.Trace scene.cs:602-625.
template <bool COUNT, bool GENERAL = true>
__device__ bool trace_surface(const DevScene& S, const Ray& ray, SurfHit& out, Ctr& c, uint32_t* err) {
    SR_COUNT(c, SR_COUNTER_SCENE_TRACE, 1);
    Hit hit = scene_closest<COUNT, GENERAL>(S, ray, c, err);
    if (hit.obj < 0) return false;
    surface_from_hit<COUNT, GENERAL>(S, ray, hit, out, c);
    return true;
}

// Scene.ShadowTransmittance scene.cs:576-600.  In scenes without transparent materials the first
// hit is always opaque, so the answer is "any hit -> black, else white".
template <bool COUNT, bool GENERAL = true>
__device__ Col shadow_transmittance(const DevScene& S, Ray ray, Ctr& c, uint32_t* err) {
    if (!GENERAL || !S.has_transparent) {
        SR_COUNT(c, SR_COUNTER_SCENE_OCCLUDE, 1);
        return scene_any<COUNT, GENERAL>(S, ray, c, err) ? black() : white();
    }
    Col tr = white();
    int steps = 0;
    do {
        if (++steps > 4096) {  // the ray advances every step; the cap only guards degenerate scenes
            atomicOr(err, SR_DEVERR_LOOP);
            return black();
        }
        SR_COUNT(c, SR_COUNTER_SCENE_OCCLUDE, 1);
        Hit hit = scene_closest<COUNT>(S, ray, c, err);
        if (hit.obj < 0) return tr;
        const DevObject& o = S.objects[hit.obj];
        const DevMaterial& m = S.materials[o.index];
        if (m.params.y <= 0.0f) return black();
        ShapeHit h = world_hit<COUNT>(S, ray, hit, c);
        Col albedo = (m.tex[0] >= 0 ? tex_sample<COUNT>(S, m.tex[0], h.uv, c) : white()) * col3(m.albedo_rough);
        float ndv = fabsf(dot(h.norm_geo, ray.d));
        Col f = fresnel(ndv, base_reflectivity(m.params.w, albedo, m.params.x));
        tr = tr * (albedo * m.params.y * (white() - f));
        ray = make_ray(ray_at(ray, h.dist + fmaxf(1e-4f, h.dist * 1e-4f)), ray.d);
    } while (max_component(tr) > 1e-4f);
    return tr;
}

// Scene.SampleSkyLight scene.cs:758-772.
template <bool COUNT, bool GENERAL = true>
__device__ bool sample_sky_light(const DevScene& S, V3 pos, Rng& rng, V3& ldir, float& lpdf, Col& tr, Ctr& c,
                                 uint32_t* err) {
    if (!sky_light_rand<COUNT, GENERAL>(S, rng, ldir, lpdf, c) || lpdf <= 0.0f) return false;
    Ray shadow = make_ray(pos, ldir);
    tr = shadow_transmittance<COUNT, GENERAL>(S, shadow, c, err);
    if (max_component(tr) <= 0.0f) return false;
    if (S.has_fog) tr = tr * fog_transmittance_inf(S, shadow);
    return true;
}

// Scene.SampleSkyDirect scene.cs:774-794.
template <bool COUNT>
__device__ Col sample_sky_direct(const DevScene& S, const Surface& s, V3 pos, V3 view, Rng& rng, Ctr& c, uint32_t* err) {
    V3 ldir;
    float lpdf;
    Col tr;
    if (!sample_sky_light<COUNT>(S, pos, rng, ldir, lpdf, tr, c, err)) return black();
    V3 n = dot(s.normal, view) >= 0.0f ? s.normal : -s.normal;
    if (dot(n, ldir) <= 0.0f) return black();
    V3 ng = dot(s.normal_geo, view) >= 0.0f ? s.normal_geo : -s.normal_geo;
    if (dot(ng, ldir) <= 0.0f) return black();
    Col refl = opaque_eval(s, view, ldir);
    float spdf = opaque_pdf(s, view, ldir, specular_probability(s, view));
    float mis = power_heuristic(lpdf, spdf);
    return sky_radiance<COUNT>(S, ldir, c) * tr * refl * mis / lpdf;
}

// Scene.SampleSkyDirectFog scene.cs:796-810.
template <bool COUNT, bool GENERAL = true>
__device__ Col sample_sky_direct_fog(const DevScene& S, V3 pos, V3 rdir, Rng& rng, Ctr& c, uint32_t* err) {
    V3 ldir;
    float lpdf;
    Col tr;
    if (!sample_sky_light<COUNT, GENERAL>(S, pos, rng, ldir, lpdf, tr, c, err)) return black();
    float fog_pdf = hg_pdf(dot(rdir, ldir), S.fog_g);
    float mis = power_heuristic(lpdf, fog_pdf);
    return sky_radiance<COUNT, GENERAL>(S, ldir, c) * tr * fog_pdf * mis / lpdf;
}

// Scene.RussianRoulette scene.cs:744-756.
__device__ __forceinline__ bool russian_roulette(Col& energy, uint32_t bounce, Rng& rng) {
    if (bounce < 3) return false;
    float survive = fminf(1.0f, max_component(energy));
    if (rng_float(rng) >= survive) return true;
    energy = energy / survive;
    return false;
}


// Renderer.RelativeStdErr renderer.cs:232-237.
__device__ __forceinline__ float relative_std_err(float sum, float sum_sqr, uint32_t n) {
    float fn = (float)n;
    float mean = sum / fn;
    float var = fmaxf(0.0f, sum_sqr / fn - mean * mean);
    return sqrtf(var / fn) / fmaxf(mean, 1e-4f);
}

template <bool COUNT>
__device__ __forceinline__ void flush_counters(Ctr& c, unsigned long long* counters) {
    if constexpr (COUNT) {
#pragma unroll
        for (int i = 0; i < SR_COUNTER_COUNT; ++i) {
            unsigned long long v = c.v[i];
            // warp reduction keeps the atomics to one per warp and counter
            for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
            if ((threadIdx.x & 31) == 0 && v) atomicAdd(counters + i, v);
            c.v[i] = 0;
        }
    }
}


// View.Ray math.cs:1613-1636 for pixel (x, y); draws the x then y jitter (renderer.cs:175).
__device__ __forceinline__ Ray camera_ray(const DevView& V, const DevParams& P, uint32_t x, uint32_t y, Rng& rng) {
    float jx = rng_float(rng);
    float px = ((float)x + jx) / (float)P.width;
    float jy = rng_float(rng);
    float py = ((float)y + jy) / (float)P.height;
    float ndc_x = px * 2.0f - 1.0f;
    float ndc_y = -py * 2.0f + 1.0f;
    V3 local{ndc_x * V.tan_h, ndc_y * V.tan_v, 1.0f};
    return make_ray(v3(V.origin), quat_rotate(V.rot, normalize(local)));
}

}  // namespace sr

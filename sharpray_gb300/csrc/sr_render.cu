// sr_render.cu — the per-pixel path loop (Renderer.Render renderer.cs:153-229 over
// Scene.Sample scene.cs:627-741) as CUDA kernels for sm_103a, plus the ray-query kernel used by
// the closest-hit parity test.
//
// Each pixel owns one RNG stream that all of its samples consume in order (Rng(x, y),
// renderer.cs:156), so the samples of a pixel are sequential by construction; parallelism is
// across pixels.  A warp covers an 8x4 pixel tile so that its primary rays are coherent.
#include <cuda_runtime.h>

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
};

// Scene.Trace scene.cs:602-625.
template <bool COUNT>
__device__ bool trace_surface(const DevScene& S, const Ray& ray, SurfHit& out, Ctr& c, uint32_t* err) {
    SR_COUNT(c, SR_COUNTER_SCENE_TRACE, 1);
    Hit hit = scene_closest<COUNT>(S, ray, c, err);
    if (hit.obj < 0) return false;
    ShapeHit h = world_hit<COUNT>(S, ray, hit, c);
    const DevObject& o = S.objects[hit.obj];
    const DevMaterial& m = S.materials[o.index];
    float4 ar = m.albedo_rough;
    float4 mp = m.params;
    Col albedo = (m.tex[0] >= 0 ? tex_sample<COUNT>(S, m.tex[0], h.uv, c) : white()) * col3(ar);
    float roughness = (m.tex[1] >= 0 ? tex_sample<COUNT>(S, m.tex[1], h.uv, c).r : 1.0f) * ar.w;
    float metallic = (m.tex[2] >= 0 ? tex_sample<COUNT>(S, m.tex[2], h.uv, c).r : 1.0f) * mp.x;
    V3 normal = h.norm;
    if (m.tex[3] >= 0) {
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
    return true;
}

// Scene.ShadowTransmittance scene.cs:576-600.  In scenes without transparent materials the first
// hit is always opaque, so the answer is "any hit -> black, else white".
template <bool COUNT>
__device__ Col shadow_transmittance(const DevScene& S, Ray ray, Ctr& c, uint32_t* err) {
    if (!S.has_transparent) {
        SR_COUNT(c, SR_COUNTER_SCENE_OCCLUDE, 1);
        return scene_any<COUNT>(S, ray, c, err) ? black() : white();
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
template <bool COUNT>
__device__ bool sample_sky_light(const DevScene& S, V3 pos, Rng& rng, V3& ldir, float& lpdf, Col& tr, Ctr& c,
                                 uint32_t* err) {
    if (!sky_light_rand<COUNT>(S, rng, ldir, lpdf, c) || lpdf <= 0.0f) return false;
    Ray shadow = make_ray(pos, ldir);
    tr = shadow_transmittance<COUNT>(S, shadow, c, err);
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
template <bool COUNT>
__device__ Col sample_sky_direct_fog(const DevScene& S, V3 pos, V3 rdir, Rng& rng, Ctr& c, uint32_t* err) {
    V3 ldir;
    float lpdf;
    Col tr;
    if (!sample_sky_light<COUNT>(S, pos, rng, ldir, lpdf, tr, c, err)) return black();
    float fog_pdf = hg_pdf(dot(rdir, ldir), S.fog_g);
    float mis = power_heuristic(lpdf, fog_pdf);
    return sky_radiance<COUNT>(S, ldir, c) * tr * fog_pdf * mis / lpdf;
}

// Scene.RussianRoulette scene.cs:744-756.
__device__ __forceinline__ bool russian_roulette(Col& energy, uint32_t bounce, Rng& rng) {
    if (bounce < 3) return false;
    float survive = fminf(1.0f, max_component(energy));
    if (rng_float(rng) >= survive) return true;
    energy = energy / survive;
    return false;
}

// Scene.Sample scene.cs:627-741.
template <bool COUNT>
__device__ Fragment sample_path(const DevScene& S, Ray ray, Rng& rng, uint32_t bounces, float indirect_clamp, Ctr& c,
                                uint32_t* err) {
    SR_COUNT(c, SR_COUNTER_SAMPLE, 1);
    Fragment frag;
    frag.has_primary = false;
    Col radiance = black(), radiance_fog = black(), energy = white();
    bool has_spdf = false;
    float spdf = 0.0f;
    bool has_medium = false;
    Col medium = black();
    const float inf = __int_as_float(0x7f800000);
    for (uint32_t i = 0; i != bounces + 1; ++i) {
        SR_COUNT(c, SR_COUNTER_SAMPLE_BOUNCE, 1);
        SurfHit hit;
        bool has_hit = trace_surface<COUNT>(S, ray, hit, c, err);
        float sdist;
        if (S.has_fog && fog_scatter_distance(S, ray, has_hit ? hit.dist : inf, rng, sdist)) {
            energy = energy * col3(S.fog_color);
            Col srad = sample_sky_direct_fog<COUNT>(S, ray_at(ray, sdist), ray.d, rng, c, err) * energy;
            if (i == 0)
                radiance_fog = radiance_fog + srad;
            else
                radiance = radiance + srad;
            if (russian_roulette(energy, i, rng)) break;
            V3 sdir = hg_scatter_dir(ray.d, S.fog_g, rng);
            has_spdf = true;
            spdf = hg_pdf(dot(ray.d, sdir), S.fog_g);
            ray = make_ray(ray_at(ray, sdist), sdir);
        } else if (has_hit) {
            const Surface& s = hit.surf;
            float dist = hit.dist;
            V3 view = -ray.d;
            float bias = fmaxf(1e-4f, dist * 1e-4f);
            V3 pos = ray_at(ray, dist - bias);
            if (has_medium) energy = energy * beer_law(medium, dist);
            radiance = radiance + s.radiance * energy;
            if (i == 0) {
                frag.has_primary = true;
                frag.normal = s.normal;
                frag.uv = s.uv;
                frag.depth = dist;
            }
            radiance = radiance + sample_sky_direct<COUNT>(S, s, pos, view, rng, c, err) * energy;
            if (russian_roulette(energy, i, rng)) break;
            Scatter sc = surface_scatter(s, ray.d, view, rng);
            energy = energy * sc.weight;
            energy = clamp_luminance(energy, indirect_clamp);
            bool enter = dot(sc.dir, s.normal_geo) < 0.0f;
            if (sc.refracted) {
                has_medium = enter;
                if (enter) medium = s.albedo;
            } else if (!enter) {
                has_medium = false;
            }
            has_spdf = sc.has_pdf;
            spdf = sc.pdf;
            ray = make_ray(ray_at(ray, dist) + sc.dir * bias, sc.dir);
        } else {
            float mis = has_spdf ? power_heuristic(spdf, sky_light_pdf(S, ray.d)) : 1.0f;
            radiance = radiance + sky_radiance<COUNT>(S, ray.d, c) * mis * energy;
            break;
        }
    }
    frag.radiance = radiance;
    frag.radiance_fog = radiance_fog;
    return frag;
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
    if (!COUNT) return;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) {
        unsigned long long v = c.v[i];
        // warp reduction keeps the atomics to one per warp and counter
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(counters + i, v);
        c.v[i] = 0;
    }
}

// Renderer.Render for one pixel (renderer.cs:153-229); writes the seven AOV planes.
template <bool COUNT>
__device__ void render_pixel(const DevScene& S, const DevView& V, const DevParams& P, const DevAovs& out, uint32_t x,
                             uint32_t y, Ctr& c, uint32_t* err) {
    Rng rng = rng_seed(x, y);
    Col rad_sum = black(), fog_sum = black();
    float lum_sum = 0.f, lum_sqr = 0.f, surf_sum = 0.f, surf_sqr = 0.f;
    V3 nsum{0.f, 0.f, 0.f}, nfb{0.f, 0.f, 0.f};
    uint32_t ncount = 0;
    bool has_uv = false;
    V2 uv{0.f, 0.f};
    float dsum = 0.f;
    uint32_t dcount = 0;
    uint32_t si = 0;
    V3 vorigin = v3(V.origin);
    for (; si != P.max_samples; ++si) {
        float jx = rng_float(rng);
        float px = ((float)x + jx) / (float)P.width;
        float jy = rng_float(rng);
        float py = ((float)y + jy) / (float)P.height;
        // View.Ray math.cs:1613-1636
        float ndc_x = px * 2.0f - 1.0f;
        float ndc_y = -py * 2.0f + 1.0f;
        V3 local{ndc_x * V.tan_h, ndc_y * V.tan_v, 1.0f};
        Ray ray = make_ray(vorigin, quat_rotate(V.rot, normalize(local)));
        Fragment f = sample_path<COUNT>(S, ray, rng, P.bounces, P.indirect_clamp, c, err);
        rad_sum = rad_sum + f.radiance;
        fog_sum = fog_sum + f.radiance_fog;
        float lum = luminance(f.radiance) + luminance(f.radiance_fog);
        lum_sum += lum;
        lum_sqr += lum * lum;
        float ls = luminance(f.radiance);
        surf_sum += ls;
        surf_sqr += ls * ls;
        if (f.has_primary) {
            nsum = nsum + f.normal;
            nfb = f.normal;
            ncount++;
            dsum += f.depth;
            dcount++;
            if (!has_uv) {
                has_uv = true;
                uv = f.uv;
            }
        }
        if (si >= P.min_samples - 1) {
            if (relative_std_err(lum_sum, lum_sqr, si + 1) < P.variance_threshold) break;
        }
    }
    uint32_t count = si + 1;
    float var = relative_std_err(surf_sum, surf_sqr, count);
    Col radiance = rad_sum / (float)count;
    Col radiance_fog = fog_sum / (float)count;
    V3 n = ncount > 0 ? normalize_or(nsum, nfb) : V3{0.f, 0.f, 0.f};
    size_t i = (size_t)y * P.width + x;
    out.radiance[i * 3 + 0] = radiance.r;
    out.radiance[i * 3 + 1] = radiance.g;
    out.radiance[i * 3 + 2] = radiance.b;
    out.radiance_fog[i * 3 + 0] = radiance_fog.r;
    out.radiance_fog[i * 3 + 1] = radiance_fog.g;
    out.radiance_fog[i * 3 + 2] = radiance_fog.b;
    out.normals[i * 3 + 0] = n.x;
    out.normals[i * 3 + 1] = n.y;
    out.normals[i * 3 + 2] = n.z;
    out.uv[i * 2 + 0] = uv.x;
    out.uv[i * 2 + 1] = uv.y;
    out.depth[i] = dcount > 0 ? dsum / (float)dcount : __int_as_float(0x7f800000);
    out.samples[i] = count;
    out.variance[i] = var;
}

// One thread per pixel; a 32x4 block covers four 8x4 warp tiles side by side.
template <bool COUNT>
__global__ void __launch_bounds__(128) k_render_pixels(DevScene S, DevView V, DevParams P, DevAovs out,
                                                       unsigned long long* counters, uint32_t* err) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = blockIdx.x * 32 + warp * 8 + (lane & 7);
    uint32_t y = blockIdx.y * 4 + (lane >> 3);
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    if (x < P.width && y < P.height) render_pixel<COUNT>(S, V, P, out, x, y, c, err);
    flush_counters<COUNT>(c, counters);
}

// Closest hit of world rays, for the bit-exact hit parity test.
__global__ void k_trace_rays(DevScene S, const float* rays, uint32_t n, int32_t* obj, int32_t* tri, float* dist,
                             float* uv, uint32_t* err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rays + (size_t)i * 6;
    Ray ray = make_ray(V3{r[0], r[1], r[2]}, V3{r[3], r[4], r[5]});
    Ctr c;
    Hit h = scene_closest<false>(S, ray, c, err);
    if (h.obj < 0) {
        obj[i] = -1;
        tri[i] = -1;
        dist[i] = __int_as_float(0x7f800000);
        uv[2 * i] = 0.f;
        uv[2 * i + 1] = 0.f;
        return;
    }
    obj[i] = S.objects[h.obj].index;
    tri[i] = h.tri >= 0 ? __float_as_int(__ldg(S.tris + 3 * h.tri).w) : -1;
    dist[i] = h.dist;
    uv[2 * i] = h.u;
    uv[2 * i + 1] = h.v;
}

cudaError_t launch_render(const DevScene& S, const DevView& V, const DevParams& P, const DevAovs& out,
                          unsigned long long* counters, uint32_t* err, cudaStream_t stream) {
    dim3 block(128);
    dim3 grid((P.width + 31) / 32, (P.height + 3) / 4);
    if (counters)
        k_render_pixels<true><<<grid, block, 0, stream>>>(S, V, P, out, counters, err);
    else
        k_render_pixels<false><<<grid, block, 0, stream>>>(S, V, P, out, counters, err);
    return cudaGetLastError();
}

cudaError_t launch_trace(const DevScene& S, const float* rays, uint32_t n, int32_t* obj, int32_t* tri, float* dist,
                         float* uv, uint32_t* err, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    k_trace_rays<<<(n + 127) / 128, 128, 0, stream>>>(S, rays, n, obj, tri, dist, uv, err);
    return cudaGetLastError();
}

}  // namespace sr

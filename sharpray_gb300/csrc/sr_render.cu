// sr_render.cu — the per-pixel path loop (Renderer.Render renderer.cs:153-229 over
// Scene.Sample scene.cs:627-741) as CUDA kernels for sm_103a, plus the ray-query kernel used by
// the closest-hit parity test.
//
// Each pixel owns one RNG stream that all of its samples consume in order (Rng(x, y),
// renderer.cs:156), so the samples of a pixel are sequential by construction; parallelism is
// across pixels.  A warp covers an 8x4 pixel tile so that its primary rays are coherent.
#include <cuda_runtime.h>

#include "sr_path.cuh"

namespace sr {

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

// Renderer.Render for one pixel (renderer.cs:153-229); writes the seven AOV planes.
template <bool COUNT>
__device__ void render_pixel(const DevScene& S, const DevView& V, const DevParams& P, const DevAovs& out, uint32_t x,
                             uint32_t y, Ctr& c, uint32_t* err) {
    Rng rng = rng_seed(x, y, P.seed);
    Col rad_sum = black(), fog_sum = black();
    float lum_sum = 0.f, lum_sqr = 0.f, surf_sum = 0.f, surf_sqr = 0.f;
    V3 nsum{0.f, 0.f, 0.f}, nfb{0.f, 0.f, 0.f};
    uint32_t ncount = 0;
    bool has_uv = false;
    V2 uv{0.f, 0.f};
    float dsum = 0.f;
    uint32_t dcount = 0;
    uint32_t si = 0;
    for (; si != P.max_samples; ++si) {
        Ray ray = camera_ray(V, P, x, y, rng);
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

// Per texel of a texture sky: the radiance toward the texel's centre -- the direction a light
// sample of that texel takes -- and the texel's light pdf (SkyTexture.LightDirRand scene.cs:408-416),
// with the functions the path code uses, so a light sample reads one record instead of a bilinear
// lookup.
__global__ void k_sky_table(DevScene S, float4* out) {
    const DevSky& k = S.sky;
    const DevTexture& t = S.textures[k.texture];
    const uint32_t n = t.width * t.height;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t x = i % t.width, y = i / t.width;
        Ctr c;
        const Col L = sky_radiance<false, true>(S, sky_texel_dir(k, t, x, y), c);
        const float pdf = luminance(col3(ldg4(S.texels + t.offset + (size_t)y * t.width + x))) * k.pdf_scale;
        out[i] = make_float4(L.r, L.g, L.b, pdf);
    }
}

cudaError_t launch_sky_table(const DevScene& S, float4* out, uint32_t texels, cudaStream_t stream) {
    if (texels == 0) return cudaSuccess;
    k_sky_table<<<(texels + 255) / 256 < 4096 ? (texels + 255) / 256 : 4096, 256, 0, stream>>>(S, out);
    return cudaGetLastError();
}

cudaError_t launch_trace(const DevScene& S, const float* rays, uint32_t n, int32_t* obj, int32_t* tri, float* dist,
                         float* uv, uint32_t* err, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    k_trace_rays<<<(n + 127) / 128, 128, 0, stream>>>(S, rays, n, obj, tri, dist, uv, err);
    return cudaGetLastError();
}

}  // namespace sr

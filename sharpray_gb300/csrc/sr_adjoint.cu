// sr_adjoint.cu — path-replay adjoint of a rendered image with respect to the texels of an albedo
// (colour) or roughness texture and the fog density: given dL/dI for the image I = radiance +
// radiance_fog of a render, the gradients dL/d(texels) and dL/d(density), one parameter per launch
// or all three from one replay.  No counterpart in the reference (it has no derivatives).
//
// One thread per pixel replays the pixel's samples exactly as the per-pixel path loop renders
// them (the same RNG stream and the same functions, so the same paths and the same radiance --
// the kernel also returns the replayed image for the caller to check), recording per vertex the
// throughput, what the vertex adds to the radiance and the scatter weight.  A reverse sweep over
// the vertices then carries the adjoint of the throughput back to the camera: through the scatter
// weights, the luminance clamp of the indirect throughput and the Russian-roulette division (both
// differentiated as functions of the throughput), and into the parameter of each surface vertex,
// whose texture lookup passes it on to the four bilinear texels (atomic adds).
//
// Differentiated: the BRDF values of the light samples and the scatter weights with respect to
// the parameter (albedo: the diffuse term and, for metallic surfaces, the Fresnel base;
// roughness: the GGX distribution and Smith terms).  Held fixed ("detached"), as path replay does:
// the sampled directions, lobe choices, Russian-roulette decisions and the pdfs and MIS weights.
// For the albedo of non-metallic surfaces none of these depends on the parameter, so the gradient
// is the exact derivative of the renderer's own estimator at fixed random numbers wherever no
// roulette decision or clamp threshold is crossed.  The roughness moves the sampled specular
// directions and the density the sampled scatter distances, so there the gradient is exact in
// expectation (d/dθ of the expected image) rather than per sample; for the density it carries the
// score terms of the free-flight sampling.  Scenes with transparent materials are refused by the
// host entry point.
#include <cuda_runtime.h>

#include "sr_adjoint.cuh"
#include "sr_kernels.h"

namespace sr {

// sample_path (sr_render.cu) recording the vertices; rad / fog as the forward pass sums them.
template <bool GENERAL, int PARAM>
__device__ int replay_sample(const DevScene& S, Ray ray, Rng& rng, uint32_t bounces, float indirect_clamp,
                             AdjVertex<PARAM>* v, Col& radiance, Col& radiance_fog, Ctr& c, uint32_t* err) {
    radiance = black();
    radiance_fog = black();
    Col energy = white();
    bool has_spdf = false;
    float spdf = 0.0f;
    const float inf = __int_as_float(0x7f800000);
    int n = 0;
    for (uint32_t i = 0; i != bounces + 1; ++i) {
        SurfHit hit;
        bool has_hit = trace_surface<false, GENERAL>(S, ray, hit, c, err);
        float sdist;
        AdjVertex<PARAM>& x = v[n++];
        x.e_in = energy;
        x.rr = 1.0f;
        x.clamp_max = indirect_clamp;
        x.dadd = black();
        x.ds = black();
        if constexpr (PARAM == ADJ_ALL) x.ex = AdjExtra{black(), black(), black(), 0.0f};
        if (S.has_fog && fog_scatter_distance(S, ray, has_hit ? hit.dist : inf, rng, sdist)) {
            x.kind = AV_FOG;
            if constexpr (kAdjFog<PARAM>)  // score of a scatter at sdist: 1/density - depth
                set_score(x, 1.0f / S.fog_density - fog_depth_unit(S, ray, sdist));
            energy = energy * col3(S.fog_color);
            x.e_rr = energy;
            Col dfog;
            x.add = sample_sky_direct_fog_adj<GENERAL, PARAM>(S, ray_at(ray, sdist), ray.d, rng, c, err, dfog);
            if constexpr (PARAM == ADJ_ALL)
                x.ex.dadd_f = dfog;
            else if constexpr (PARAM == ADJ_FOG_DENSITY)
                x.dadd = dfog;
            Col srad = x.add * energy;
            if (i == 0)
                radiance_fog = radiance_fog + srad;
            else
                radiance = radiance + srad;
            if (i >= 3) x.rr = fminf(1.0f, max_component(energy));
            if (russian_roulette(energy, i, rng)) {
                x.kind = AV_FOG_END;
                break;
            }
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
            x.kind = AV_SURF;
            x.uv = s.uv;
            x.material = hit.material;
            if constexpr (kAdjFog<PARAM>)  // score of passing the fog up to the surface
                if (S.has_fog) set_score(x, -fog_depth_unit(S, ray, dist));
            radiance = radiance + s.radiance * energy;
            NeeDeriv dn;
            Col nee = sample_sky_direct_adj<GENERAL, PARAM>(S, s, pos, view, rng, c, err, dn);
            radiance = radiance + nee * energy;
            x.add = s.radiance + nee;
            if constexpr (PARAM == ADJ_ALL) {
                x.dadd = dn.a;
                x.ex.dadd_r = dn.r;
                x.ex.dadd_f = dn.f;
            } else {
                x.dadd = PARAM == ADJ_ALBEDO ? dn.a : (PARAM == ADJ_ROUGHNESS ? dn.r : dn.f);
            }
            if (i >= 3) x.rr = fminf(1.0f, max_component(energy));
            if (russian_roulette(energy, i, rng)) {
                x.kind = AV_SURF_END;
                break;
            }
            x.e_rr = energy;
            Scatter sc = surface_scatter<GENERAL>(s, ray.d, view, rng);
            x.s = sc.weight;
            const float ipdf = 1.0f / fmaxf(sc.pdf, 1e-6f);
            if constexpr (kAdjAlbedo<PARAM>) x.ds = opaque_eval_dalbedo(s, view, sc.dir) * ipdf;
            if constexpr (PARAM == ADJ_ROUGHNESS) x.ds = opaque_eval_droughness(s, view, sc.dir) * ipdf;
            if constexpr (PARAM == ADJ_ALL) x.ex.ds_r = opaque_eval_droughness(s, view, sc.dir) * ipdf;
            energy = energy * sc.weight;
            x.pre = energy;
            energy = clamp_luminance(energy, indirect_clamp);
            has_spdf = sc.has_pdf;
            spdf = sc.pdf;
            ray = make_ray(ray_at(ray, dist) + sc.dir * bias, sc.dir);
        } else {
            x.kind = AV_SKY;
            if constexpr (kAdjFog<PARAM>)
                if (S.has_fog) {
                    const float depth = fog_depth_unit(S, ray, inf);
                    set_score(x, isfinite(depth) ? -depth : 0.0f);  // an escape needs a finite depth
                }
            float mis = has_spdf ? power_heuristic(spdf, sky_light_pdf<GENERAL>(S, ray.d)) : 1.0f;
            x.add = sky_radiance<false, GENERAL>(S, ray.d, c) * mis;
            radiance = radiance + x.add * energy;
            break;
        }
    }
    return n;
}

// One thread per pixel: replay, then the reverse sweep.  Register caps: 128 for the lean
// instantiation (8 blocks of 64 per SM), 168 for the general one.
template <bool GENERAL, int PARAM>
__global__ void __launch_bounds__(64, GENERAL ? 6 : 8)
    k_adjoint(DevScene S, DevView V, DevParams P, DevAovs fwd, const float* d_image, AdjTargets T, float* replay,
              uint32_t* err) {
    const uint32_t x = blockIdx.x * 8 + (threadIdx.x & 7), y = blockIdx.y * 8 + (threadIdx.x >> 3);
    if (x >= P.width || y >= P.height) return;
    const size_t i = (size_t)y * P.width + x;
    const uint32_t count = fwd.samples[i];
    const uint32_t taken = count < P.max_samples ? count : P.max_samples;  // the loop's off-by-one
    const float inv = 1.0f / (float)count;
    Col G{d_image[3 * i] * inv, d_image[3 * i + 1] * inv, d_image[3 * i + 2] * inv};
    Ctr c;
    AdjVertex<PARAM> v[kAdjMaxVertices];
    Rng rng = rng_seed(x, y, P.seed);
    Col rad_sum = black(), fog_sum = black();
    float g_density = 0.0f;  // this pixel's d loss / d fog density
    for (uint32_t si = 0; si < taken; ++si) {
        Ray ray = camera_ray(V, P, x, y, rng);
        Col rad, fog;
        const int n = replay_sample<GENERAL, PARAM>(S, ray, rng, P.bounces, P.indirect_clamp, v, rad, fog, c, err);
        rad_sum = rad_sum + rad;
        fog_sum = fog_sum + fog;
        adjoint_sweep<PARAM>(S, [&](int k) -> const AdjVertex<PARAM>& { return v[k]; }, n, G, T, g_density);
    }
    if constexpr (kAdjFog<PARAM>)
        if (T.grad_f && g_density != 0.0f) atomicAdd(T.grad_f, g_density);
    if (replay) {
        const Col r = rad_sum / (float)count, f = fog_sum / (float)count;
        replay[3 * i] = r.r + f.r;
        replay[3 * i + 1] = r.g + f.g;
        replay[3 * i + 2] = r.b + f.b;
    }
}

cudaError_t launch_adjoint(const DevScene& S, const DevView& V, const DevParams& P, const DevAovs& fwd,
                           const float* d_image, int parameter, int tex_a, float* grad_a, int tex_r, float* grad_r,
                           float* grad_f, float* replay, uint32_t* err, cudaStream_t stream) {
    dim3 grid((P.width + 7) / 8, (P.height + 7) / 8);
    const AdjTargets T{tex_a, grad_a, tex_r, grad_r, grad_f};
    // scenes of meshes under a texture sky without transparency or normal maps take the lean
    // instantiation, as the wavefront kernels do (same results, far less code)
#define SR_ADJ_LAUNCH(PR)                                                                           \
    do {                                                                                            \
        if (S.general)                                                                              \
            k_adjoint<true, PR><<<grid, 64, 0, stream>>>(S, V, P, fwd, d_image, T, replay, err);    \
        else                                                                                        \
            k_adjoint<false, PR><<<grid, 64, 0, stream>>>(S, V, P, fwd, d_image, T, replay, err);   \
    } while (0)
    switch (parameter) {
    case ADJ_ALBEDO: SR_ADJ_LAUNCH(ADJ_ALBEDO); break;
    case ADJ_ROUGHNESS: SR_ADJ_LAUNCH(ADJ_ROUGHNESS); break;
    case ADJ_FOG_DENSITY: SR_ADJ_LAUNCH(ADJ_FOG_DENSITY); break;
    default: SR_ADJ_LAUNCH(ADJ_ALL); break;
    }
#undef SR_ADJ_LAUNCH
    return cudaGetLastError();
}

// rgb float triples -> the texel records (rgb + pad) of one texture.
__global__ void k_texels_from_rgb(const float* __restrict__ rgb, float4* __restrict__ out, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        float4 t;
        t.x = rgb[3 * k], t.y = rgb[3 * k + 1], t.z = rgb[3 * k + 2], t.w = 0.0f;
        out[k] = t;
    }
}

cudaError_t launch_texels_from_rgb(const float* rgb, float4* out, size_t n, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    size_t blocks = (n + 255) / 256;
    k_texels_from_rgb<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, stream>>>(rgb, out, n);
    return cudaGetLastError();
}

}  // namespace sr

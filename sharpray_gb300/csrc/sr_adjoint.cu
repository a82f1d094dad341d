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

#include <type_traits>

#include "sr_kernels.h"
#include "sr_path.cuh"

namespace sr {

constexpr int kAdjMaxVertices = 17;  // bounces <= 16

enum : int { AV_FOG = 0, AV_SURF = 1, AV_SURF_END = 2, AV_SKY = 3, AV_FOG_END = 4 };

enum : int { ADJ_ALBEDO = 0, ADJ_ROUGHNESS = 1, ADJ_FOG_DENSITY = 2, ADJ_ALL = 3 };

// The roughness and fog-density derivatives of a vertex, kept besides the albedo ones when one
// replay serves all three parameters.
struct AdjExtra {
    Col dadd_r;   // d add / d roughness
    Col ds_r;     // d s / d roughness
    Col dadd_f;   // d add / d fog density
    float score;  // d log(sampling weight of the segment into the vertex) / d fog density
};
struct AdjNone {};

template <int PARAM>
struct AdjVertex {
    Col e_in;   // throughput entering the vertex
    Col e_rr;   // throughput after the Russian roulette (surface), or after the fog colour (fog)
    Col add;    // radiance added per unit throughput (emission + light sample; fog light sample; sky)
    Col dadd;   // d add / d parameter (albedo: per channel; roughness, density: the rgb of d add / d p)
    Col s;      // scatter weight (surface)
    Col ds;     // d s / d parameter, likewise (fog density: ds.r holds the score of the segment into
                // the vertex, d log(its sampling weight) / d density; s does not depend on it)
    Col pre;    // e_rr * s before the luminance clamp
    float rr;   // survival probability divided by (1: none)
    float clamp_max;
    V2 uv;
    int kind;
    int material;
    std::conditional_t<PARAM == ADJ_ALL, AdjExtra, AdjNone> ex;
};

template <int PARAM> constexpr bool kAdjAlbedo = PARAM == ADJ_ALBEDO || PARAM == ADJ_ALL;
template <int PARAM> constexpr bool kAdjRough = PARAM == ADJ_ROUGHNESS || PARAM == ADJ_ALL;
template <int PARAM> constexpr bool kAdjFog = PARAM == ADJ_FOG_DENSITY || PARAM == ADJ_ALL;

// Where each parameter's derivatives sit in a record.
template <int PARAM>
__device__ __forceinline__ Col dadd_rough(const AdjVertex<PARAM>& q) {
    if constexpr (PARAM == ADJ_ALL) return q.ex.dadd_r; else return q.dadd;
}
template <int PARAM>
__device__ __forceinline__ Col ds_rough(const AdjVertex<PARAM>& q) {
    if constexpr (PARAM == ADJ_ALL) return q.ex.ds_r; else return q.ds;
}
template <int PARAM>
__device__ __forceinline__ Col dadd_fog(const AdjVertex<PARAM>& q) {
    if constexpr (PARAM == ADJ_ALL) return q.ex.dadd_f; else return q.dadd;
}
template <int PARAM>
__device__ __forceinline__ float score_of(const AdjVertex<PARAM>& q) {
    if constexpr (PARAM == ADJ_ALL) return q.ex.score; else return q.ds.r;
}
template <int PARAM>
__device__ __forceinline__ void set_score(AdjVertex<PARAM>& x, float score) {
    if constexpr (PARAM == ADJ_ALL) x.ex.score = score; else x.ds.r = score;
}

// d opaque_eval / d albedo (per channel), pdfs held fixed.
__device__ Col opaque_eval_dalbedo(const Surface& s, V3 view, V3 light) {
    float ndl = dot(s.normal, light);
    if (ndl <= 0.0f) return black();
    float ndv = fmaxf(1e-4f, dot(s.normal, view));
    float rs = fmaxf(s.roughness * s.roughness, 1e-4f);
    Col base = base_reflectivity(s.f0, s.albedo, s.metallic);
    V3 half = normalize_or(view + light, s.normal);
    float ndh = dot(s.normal, half);
    float hdv = dot(half, view);
    // fresnel(x, base) = base + (1 - base) (1 - x)^5, base = f0 + (albedo - f0) metallic
    float xh = 1.0f - hdv, xv = 1.0f - ndv;
    float dfh = s.metallic * (1.0f - xh * xh * xh * xh * xh);
    float dfv = s.metallic * (1.0f - xv * xv * xv * xv * xv);
    float g = smith_g1(ndv, rs) * smith_g1(ndl, rs);
    float dspec = ggx_d(ndh, rs) * dfh * g / (4.0f * ndv);
    Col fv = fresnel(ndv, base);
    float k = (1.0f - s.metallic) * (ndl / kPi);
    Col ddiff{((1.0f - fv.r) - s.albedo.r * dfv) * k, ((1.0f - fv.g) - s.albedo.g * dfv) * k,
              ((1.0f - fv.b) - s.albedo.b * dfv) * k};
    return (gray(dspec) + ddiff) * (1.0f - s.transparency);
}

// d opaque_eval / d roughness, pdfs held fixed: only the specular term depends on it, through
// rs = max(roughness^2, 1e-4) in the GGX distribution D = a2 / (pi d^2) (a2 = rs^2,
// d = 1 - (n.h)^2 + (n.h)^2 a2) and in both Smith terms G1(x) = x / (x (1 - k) + k), k = rs / 2.
__device__ Col opaque_eval_droughness(const Surface& s, V3 view, V3 light) {
    float ndl = dot(s.normal, light);
    if (ndl <= 0.0f) return black();
    float rs = s.roughness * s.roughness;
    if (!(rs > 1e-4f)) return black();  // rs sits at its floor
    float ndv = fmaxf(1e-4f, dot(s.normal, view));
    Col base = base_reflectivity(s.f0, s.albedo, s.metallic);
    V3 half = normalize_or(view + light, s.normal);
    float ndh = dot(s.normal, half);
    float hdv = dot(half, view);
    Col f = fresnel(hdv, base);
    float a2 = rs * rs, nh2 = ndh * ndh;
    float dd = (1.0f - nh2) + nh2 * a2;
    float d_ggx = a2 / (kPi * dd * dd);
    float dd_ggx = (dd - 2.0f * a2 * nh2) / (kPi * dd * dd * dd) * (2.0f * rs);  // d D / d rs
    float k = rs * 0.5f;
    float qv = ndv * (1.0f - k) + k, ql = ndl * (1.0f - k) + k;
    float gv = ndv / qv, gl = ndl / ql;
    float dgv = -0.5f * ndv * (1.0f - ndv) / (qv * qv), dgl = -0.5f * ndl * (1.0f - ndl) / (ql * ql);
    float dspec = (dd_ggx * gv * gl + d_ggx * (dgv * gl + gv * dgl)) / (4.0f * ndv) * (2.0f * s.roughness);
    return f * (dspec * (1.0f - s.transparency));
}

// Optical depth per unit fog density along r over [0, t] (t may be +inf): the integral of
// exp(-falloff * height) that Fog.OpticalDepth scales by the density (fog_transmittance_inf).
__device__ float fog_depth_unit(const DevScene& S, const Ray& r, float t) {
    const float hd = r.d.y, hs = r.o.y;
    const float es = sr_exp(-S.fog_falloff * hs);
    if (fabsf(hd) < 1e-6f) return es * t;
    return (es - sr_exp(-S.fog_falloff * (hs + t * hd))) / (S.fog_falloff * hd);
}

// d/d density of a quantity proportional to exp(-density * depth): -depth times it; zero where the
// depth is infinite (the quantity is then exactly zero and so is the limit of its derivative).
__device__ __forceinline__ Col fog_depth_derivative(Col value, float depth) {
    return isfinite(depth) ? value * -depth : black();
}

// d nee / d albedo (per channel), d roughness, d fog density.
struct NeeDeriv {
    Col a, r, f;
};

// Scene.SampleSkyDirect (sample_sky_direct in sr_path.cuh) returning also its derivatives.
template <bool GENERAL, int PARAM>
__device__ Col sample_sky_direct_adj(const DevScene& S, const Surface& s, V3 pos, V3 view, Rng& rng, Ctr& c,
                                     uint32_t* err, NeeDeriv& dn) {
    dn.a = dn.r = dn.f = black();
    V3 ldir;
    float lpdf;
    Col tr;
    if (!sample_sky_light<false, GENERAL>(S, pos, rng, ldir, lpdf, tr, c, err)) return black();
    V3 n = dot(s.normal, view) >= 0.0f ? s.normal : -s.normal;
    if (dot(n, ldir) <= 0.0f) return black();
    V3 ng = dot(s.normal_geo, view) >= 0.0f ? s.normal_geo : -s.normal_geo;
    if (dot(ng, ldir) <= 0.0f) return black();
    Col refl = opaque_eval(s, view, ldir);
    float spdf = opaque_pdf(s, view, ldir, specular_probability(s, view));
    float mis = power_heuristic(lpdf, spdf);
    Col sky = sky_radiance<false, GENERAL>(S, ldir, c);
    Col nee = sky * tr * refl * mis / lpdf;
    if constexpr (kAdjAlbedo<PARAM>) dn.a = sky * tr * opaque_eval_dalbedo(s, view, ldir) * mis / lpdf;
    if constexpr (kAdjRough<PARAM>) dn.r = sky * tr * opaque_eval_droughness(s, view, ldir) * mis / lpdf;
    if constexpr (kAdjFog<PARAM>) {  // the shadow ray's fog transmittance exp(-density * depth)
        if (S.has_fog)
            dn.f = fog_depth_derivative(nee, fog_depth_unit(S, make_ray(pos, ldir), __int_as_float(0x7f800000)));
    }
    return nee;
}

// Scene.SampleSkyDirectFog (sample_sky_direct_fog in sr_path.cuh) returning also d/d density.
template <bool GENERAL, int PARAM>
__device__ Col sample_sky_direct_fog_adj(const DevScene& S, V3 pos, V3 rdir, Rng& rng, Ctr& c, uint32_t* err,
                                         Col& dadd) {
    dadd = black();
    V3 ldir;
    float lpdf;
    Col tr;
    if (!sample_sky_light<false, GENERAL>(S, pos, rng, ldir, lpdf, tr, c, err)) return black();
    float fog_pdf = hg_pdf(dot(rdir, ldir), S.fog_g);
    float mis = power_heuristic(lpdf, fog_pdf);
    Col out = sky_radiance<false, GENERAL>(S, ldir, c) * tr * fog_pdf * mis / lpdf;
    if constexpr (kAdjFog<PARAM>)
        dadd = fog_depth_derivative(out, fog_depth_unit(S, make_ray(pos, ldir), __int_as_float(0x7f800000)));
    return out;
}

__device__ __forceinline__ float sum3(Col c) { return c.r + c.g + c.b; }

// Adjoint of x -> x / p, p = min(1, max component of x), at x (when p < 1).
__device__ Col rr_adjoint(Col x, float p, Col a) {
    if (!(p < 1.0f)) return a;
    int m = (x.r >= x.g && x.r >= x.b) ? 0 : (x.g >= x.b ? 1 : 2);
    float d = (x.r * a.r + x.g * a.g + x.b * a.b) / (p * p);
    Col r = a / p;
    if (m == 0) r.r -= d;
    else if (m == 1) r.g -= d;
    else r.b -= d;
    return r;
}

// Adjoint of x -> x * (max / lum(x)) when lum(x) > max.
__device__ Col clamp_adjoint(Col x, float max, Col a) {
    float lum = luminance(x);
    if (!(lum > max)) return a;
    float k = max / lum;
    float d = (x.r * a.r + x.g * a.g + x.b * a.b) / lum;
    return Col{k * (a.r - 0.2126f * d), k * (a.g - 0.7152f * d), k * (a.b - 0.0722f * d)};
}

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

// Passes the derivative at a surface vertex to the texels of the texture lookup that set the
// parameter (the bilinear or point lookup of Texture.Sample texture.cs:39-69): for the albedo
// g = dL/d(albedo) per channel, times the material's albedo; for the roughness (the lookup's red
// channel times the material's roughness) the sum of g's components times the material's roughness,
// into the red channel.
template <int PARAM>
__device__ void scatter_texel_grad(const DevScene& S, int material, V2 uv, Col g, int tex, float* grad) {
    if (tex < 0 || !grad) return;
    const DevMaterial& m = S.materials[material];
    if (m.tex[PARAM == ADJ_ALBEDO ? 0 : 1] != tex) return;
    const DevTexture& t = S.textures[tex];
    const Col ga = PARAM == ADJ_ALBEDO ? g * col3(m.albedo_rough)
                                       : Col{(g.r + g.g + g.b) * m.albedo_rough.w, 0.0f, 0.0f};
    float u = uv.x * t.tiling_x;
    u -= floorf(u);
    float vv = uv.y * t.tiling_y;
    vv -= floorf(vv);
    const uint32_t w = t.width, h = t.height;
    auto add = [&](uint32_t x, uint32_t y, float wt) {
        float* p = grad + 3 * ((size_t)y * w + x);
        atomicAdd(p, ga.r * wt);
        if (PARAM == ADJ_ALBEDO) {
            atomicAdd(p + 1, ga.g * wt);
            atomicAdd(p + 2, ga.b * wt);
        }
    };
    if (t.filter == 1) {
        add((uint32_t)(u * (float)w) % w, (uint32_t)(vv * (float)h) % h, 1.0f);
        return;
    }
    float fx = u * (float)(w - 1), fy = vv * (float)(h - 1);
    uint32_t x0 = (uint32_t)fx, y0 = (uint32_t)fy;
    uint32_t x1 = (x0 + 1) % w, y1 = (y0 + 1) % h;
    float tx = fx - (float)x0, ty = fy - (float)y0;
    add(x0, y0, (1.0f - tx) * (1.0f - ty));
    add(x1, y0, tx * (1.0f - ty));
    add(x0, y1, (1.0f - tx) * ty);
    add(x1, y1, tx * ty);
}

// Where the gradients go: an albedo texture and its gradient, a roughness texture and its
// gradient, the fog density's gradient (one float); texture -1 or a null pointer skips a part.
struct AdjTargets {
    int tex_a;
    float* grad_a;
    int tex_r;
    float* grad_r;
    float* grad_f;
};

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
        // reverse sweep: a = d loss / d (throughput leaving the vertex)
        Col a = black();
        for (int k = n - 1; k >= 0; --k) {
            const AdjVertex<PARAM>& q = v[k];
            Col a_in;
            if (q.kind == AV_SKY) {
                a_in = G * q.add;
            } else if (q.kind == AV_FOG || q.kind == AV_FOG_END) {
                // e_rr = e_in * fog colour; add * e_rr; then the roulette divides e_rr
                Col a_rr = (q.kind == AV_FOG ? rr_adjoint(q.e_rr, q.rr, a) : black()) + G * q.add;
                a_in = a_rr * col3(S.fog_color);
                if constexpr (kAdjFog<PARAM>) g_density += sum3(G * q.e_rr * dadd_fog(q));
            } else {
                const Col ge = G * q.e_in;
                Col a_s = black();  // d loss / d (scatter weight); none after a roulette end
                if (q.kind == AV_SURF_END) {
                    a_in = G * q.add;
                } else {
                    const Col a_pre = clamp_adjoint(q.pre, q.clamp_max, a);
                    a_s = q.e_rr * a_pre;
                    a_in = rr_adjoint(q.e_in, q.rr, q.s * a_pre) + G * q.add;
                }
                if constexpr (kAdjAlbedo<PARAM>)
                    scatter_texel_grad<ADJ_ALBEDO>(S, q.material, q.uv, a_s * q.ds + ge * q.dadd, T.tex_a, T.grad_a);
                if constexpr (kAdjRough<PARAM>)
                    scatter_texel_grad<ADJ_ROUGHNESS>(S, q.material, q.uv, a_s * ds_rough(q) + ge * dadd_rough(q),
                                                      T.tex_r, T.grad_r);
                if constexpr (kAdjFog<PARAM>) g_density += sum3(ge * dadd_fog(q));
            }
            // the segment into the vertex scales e_in by its sampling weight, whose derivative is
            // the weight times the score
            if constexpr (kAdjFog<PARAM>) g_density += score_of(q) * sum3(a_in * q.e_in);
            a = a_in;
        }
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

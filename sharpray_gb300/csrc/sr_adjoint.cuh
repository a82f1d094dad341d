// sr_adjoint.cuh — the path-replay adjoint's vertex records, derivatives and reverse sweep, shared
// by the per-pixel replay kernel (sr_adjoint.cu) and the wavefront replay (sr_wave_adjoint.cu).
#pragma once

#include <type_traits>

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
__device__ __forceinline__ Col opaque_eval_dalbedo(const Surface& s, V3 view, V3 light) {
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
__device__ __forceinline__ Col opaque_eval_droughness(const Surface& s, V3 view, V3 light) {
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
__device__ __forceinline__ float fog_depth_unit(const DevScene& S, const Ray& r, float t) {
    if (S.fog_falloff == 0.0f) {  // homogeneous: the length of [0, t] below the top
        float enter, exit;
        if (!fog_slab_span(S, r, enter, exit)) return 0.0f;
        const float e = fminf(t, exit);
        return e > enter ? e - enter : 0.0f;
    }
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
__device__ __forceinline__ Col sample_sky_direct_adj(const DevScene& S, const Surface& s, V3 pos, V3 view, Rng& rng, Ctr& c,
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
__device__ __forceinline__ Col sample_sky_direct_fog_adj(const DevScene& S, V3 pos, V3 rdir, Rng& rng, Ctr& c, uint32_t* err,
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
__device__ __forceinline__ Col rr_adjoint(Col x, float p, Col a) {
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
__device__ __forceinline__ Col clamp_adjoint(Col x, float max, Col a) {
    float lum = luminance(x);
    if (!(lum > max)) return a;
    float k = max / lum;
    float d = (x.r * a.r + x.g * a.g + x.b * a.b) / lum;
    return Col{k * (a.r - 0.2126f * d), k * (a.g - 0.7152f * d), k * (a.b - 0.0722f * d)};
}

// Passes the derivative at a surface vertex to the texels of the texture lookup that set the
// parameter (the bilinear or point lookup of Texture.Sample texture.cs:39-69): for the albedo
// g = dL/d(albedo) per channel, times the material's albedo; for the roughness (the lookup's red
// channel times the material's roughness) the sum of g's components times the material's roughness,
// into the red channel.
template <int PARAM>
__device__ __forceinline__ void scatter_texel_grad(const DevScene& S, int material, V2 uv, Col g, int tex, float* grad) {
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

// Reverse sweep over one sample's vertices v[0, n) carrying a = d loss / d (throughput leaving the
// vertex) back to the camera: through the scatter weights, the luminance clamp of the indirect
// throughput and the Russian-roulette division (both differentiated as functions of the
// throughput), into the parameters of each vertex (texel gradients by atomic adds, the fog density
// into g_density).  G = dL/dI of the pixel divided by its sample count.
// `vertex(k)` gives vertex k (a record of a local array, or one decoded from a global buffer).
template <int PARAM, typename Vertex>
__device__ __forceinline__ void adjoint_sweep(const DevScene& S, Vertex vertex, int n, Col G, const AdjTargets& T,
                                              float& g_density) {
    Col a = black();
    for (int k = n - 1; k >= 0; --k) {
        const auto& q = vertex(k);  // a reference into an array, or a decoded temporary
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

}  // namespace sr

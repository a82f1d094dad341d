// sr_wavefront.cu — wavefront form of the per-pixel path loop.
//
// Renderer.Render (renderer.cs:153-229) + Scene.Sample (scene.cs:627-741) are split into four
// kernels per bounce over structure-of-arrays path state, one slot per pixel:
//
//   extend   : closest hit of every live path ray            (Scene.Trace -> Bvh.Intersect)
//   shade    : surface/fog/miss logic of one segment, light sample, Russian roulette, scatter;
//              the NEE shadow ray and the end of a sample are deferred
//   shadow   : shadow rays (ShadowTransmittance, scene.cs:576-600) times the fog transmittance
//   finalize : NEE contributions, then, for finished samples, the pixel statistics, the adaptive
//              stop, and the next camera ray or the AOV write
//
// extend and shadow are persistent: a lane that finishes its ray takes the next one from the
// queue at once (refilled per warp with one atomic), so warps stay full although ray lengths
// differ by orders of magnitude.
//
// Live paths are compacted between kernels with warp-aggregated atomics (ballot + popc), so every
// launch works on dense queues.  Every per-path operation -- RNG draws, float operation order,
// the order in which contributions are added -- is the megakernel's (sr_path.cuh), so the two
// forms produce identical images; the wavefront form keeps each kernel's register footprint
// small so the latency-bound traversals run at high occupancy.
//
// The bounce loop runs either as a host loop (one launch per kernel per bounce, the host reads the
// live-path count after every bounce) or as a CUDA graph whose conditional WHILE node repeats the
// bounce kernels on the device until no path is left (no host round trip per bounce).
#include <cuda_runtime.h>

#include "sr_path.cuh"
#include "sr_wavefront.h"

namespace sr {

enum : uint32_t { PF_SPDF = 1u, PF_MEDIUM = 2u, PF_PRIMARY = 4u };
enum : uint32_t { RF_SHADOW = 1u, RF_TERMINATE = 2u, RF_FOG = 4u };

__device__ __forceinline__ void slot_pixel(const WaveState& W, uint32_t slot, uint32_t& x, uint32_t& y) {
    // slots are laid out in 8x4 pixel tiles so that a warp's primary rays are neighbours
    uint32_t tile = slot >> 5, lane = slot & 31u;
    x = (tile % W.tiles_x) * 8u + (lane & 7u);
    y = (tile / W.tiles_x) * 4u + (lane >> 3);
}

// Warp-aggregated append of `value` to queue q when pred holds (all 32 lanes must call).
__device__ __forceinline__ void push(uint32_t* q, uint32_t* count, uint32_t value, bool pred) {
    unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (!mask) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) q[base + __popc(mask & ((1u << lane) - 1u))] = value;
}

__device__ __forceinline__ Rng load_rng(const WaveState& W, uint32_t s) {
    uint4 a = W.rng[s];
    return {a.x, a.y, a.z, a.w, W.rng_c[s]};
}
__device__ __forceinline__ void store_rng(const WaveState& W, uint32_t s, const Rng& r) {
    W.rng[s] = make_uint4(r.s0, r.s1, r.s2, r.s3);
    W.rng_c[s] = r.s4;
}

// Start of a sample: the camera ray and a reset path (scene.cs:633-638).
__device__ __forceinline__ void begin_sample(const WaveState& W, uint32_t s, const Ray& ray) {
    W.ray_o[s] = make_float4(ray.o.x, ray.o.y, ray.o.z, __int_as_float(0));
    W.ray_d[s] = make_float4(ray.d.x, ray.d.y, ray.d.z, __int_as_float(0));
    W.rad[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    W.fog[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    W.energy[s] = make_float4(1.f, 1.f, 1.f, 0.f);
}

__global__ void __launch_bounds__(128) k_wave_init(WaveState W, DevView V, DevParams P) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = false;
    if (s < W.slots) {
        uint32_t x, y;
        slot_pixel(W, s, x, y);
        valid = x < P.width && y < P.height;
        if (valid) {
            Rng rng = rng_seed(x, y);
            Ray ray = camera_ray(V, P, x, y, rng);
            store_rng(W, s, rng);
            begin_sample(W, s, ray);
            float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            W.acc0[s] = z;
            W.acc1[s] = z;
            W.acc2[s] = z;
            W.acc3[s] = z;
            W.acc4[s] = z;  // depth sum, normal count, depth count, sample index (int bits 0)
            W.acc5[s] = z;  // first uv, has-uv flag
        }
    }
    push(W.q_active[0], &W.counts[0], s, valid);
}

// A warp refills its idle lanes once at least this many are idle (or all are).
#ifndef SR_REFILL
#define SR_REFILL 8
#endif
constexpr int kRefill = SR_REFILL;
// Minimum resident blocks per SM requested for the traversal kernels (caps their registers).
#ifndef SR_TRACE_MIN_BLOCKS
#define SR_TRACE_MIN_BLOCKS 6
#endif

// Persistent ray loop shared by extend and shadow: lanes take queue entries [fetch counter) until
// the queue is exhausted; `start(slot)` begins a query, `finish(slot)` stores its answer.
template <bool COUNT, bool ANY, bool GENERAL, typename Start, typename Finish>
__device__ __forceinline__ void persistent_queries(const DevScene& S, const uint32_t* q, uint32_t n, uint32_t* fetch,
                                                   Ctr& c, uint32_t* err, Start start, Finish finish) {
    StackEntry stack[kSceneStack];
    SceneQuery<ANY, GENERAL> sq;
    bool busy = false, exhausted = false;
    uint32_t slot = 0;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned idle = __ballot_sync(0xffffffffu, !busy);
        int nidle = __popc(idle);
        if (!exhausted && nidle >= kRefill) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, (uint32_t)nidle);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + (uint32_t)nidle >= n) exhausted = true;
            if (!busy) {
                uint32_t idx = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (idx < n) {
                    slot = q[idx];
                    sq.init(S, start(slot), stack);
                    busy = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, busy)) {
            if (exhausted) break;
            continue;
        }
        if (busy && sq.template step<COUNT>(S, stack, c, err)) {
            finish(slot, sq.best);
            busy = false;
        }
    }
}

template <bool COUNT, bool GENERAL>
__global__ void __launch_bounds__(128, SR_TRACE_MIN_BLOCKS) k_wave_extend(WaveState W, DevScene S, int cur, uint32_t* err,
                                                     unsigned long long* counters) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counts[2] = 0;        // deferred-work queue of this bounce starts empty
        W.counts[6] = 0;        // shadow queue of this bounce starts empty
        W.counts[cur ^ 1] = 0;  // next live queue starts empty
    }
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    persistent_queries<COUNT, false, GENERAL>(
        S, W.q_active[cur], W.counts[cur], &W.counts[4], c, err,
        [&](uint32_t s) {
            SR_COUNT(c, SR_COUNTER_SCENE_TRACE, 1);
            float4 o = W.ray_o[s], d = W.ray_d[s];
            return make_ray(V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z});
        },
        [&](uint32_t s, const Hit& h) {
            W.hit[s] = make_float4(__int_as_float(h.obj), __int_as_float(h.tri), h.dist, h.tl);
            W.hit_uv[s] = make_float2(h.u, h.v);
        });
    flush_counters<COUNT>(c, counters);
}

// Shadow rays of the bounce: transmittance (any hit -> black in opaque scenes) times the fog
// transmittance, as SampleSkyLight forms it (scene.cs:758-772); written over the ray origin.
template <bool COUNT, bool GENERAL>
__global__ void __launch_bounds__(128, SR_TRACE_MIN_BLOCKS) k_wave_shadow(WaveState W, DevScene S, uint32_t* err,
                                                     unsigned long long* counters) {
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    if (!GENERAL || !S.has_transparent) {
        persistent_queries<COUNT, true, GENERAL>(
            S, W.q_shadow, W.counts[6], &W.counts[5], c, err,
            [&](uint32_t s) {
                SR_COUNT(c, SR_COUNTER_SCENE_OCCLUDE, 1);
                float4 o = W.sh0[s], d = W.sh1[s];
                return make_ray(V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z});
            },
            [&](uint32_t s, const Hit& h) {
                float4 o = W.sh0[s], d = W.sh1[s];
                float tr = 0.0f;
                if (h.obj < 0) {
                    tr = 1.0f;
                    if (S.has_fog) tr = 1.0f * fog_transmittance_inf(S, make_ray(V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}));
                }
                W.sh0[s] = make_float4(tr, tr, tr, o.w);
            });
    } else {
        const uint32_t n = W.counts[6];
        for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
            uint32_t s = W.q_shadow[k];
            float4 o = W.sh0[s], d = W.sh1[s];
            Ray shadow = make_ray(V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z});
            Col tr = shadow_transmittance<COUNT, GENERAL>(S, shadow, c, err);
            if (max_component(tr) > 0.0f && S.has_fog) tr = tr * fog_transmittance_inf(S, shadow);
            W.sh0[s] = make_float4(tr.r, tr.g, tr.b, o.w);
        }
    }
    flush_counters<COUNT>(c, counters);
}

template <bool COUNT, bool GENERAL>
__global__ void __launch_bounds__(128) k_wave_shade(WaveState W, DevScene S, DevParams P, int cur, uint32_t* err,
                                                    unsigned long long* counters) {
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counts[5] = 0;  // shadow kernel's fetch counter
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    const int nxt = cur ^ 1;
    const uint32_t n = W.counts[cur];
    const uint32_t stride = gridDim.x * blockDim.x;
    const float inf = __int_as_float(0x7f800000);
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        uint32_t k = base + threadIdx.x;
        bool valid = k < n;
        uint32_t s = valid ? W.q_active[cur][k] : 0u;
        uint32_t rflags = 0;
        if (valid) {
            SR_COUNT(c, SR_COUNTER_SAMPLE_BOUNCE, 1);
            Rng rng = load_rng(W, s);
            float4 o4 = W.ray_o[s], d4 = W.ray_d[s];
            uint32_t bounce = (uint32_t)__float_as_int(o4.w);
            uint32_t pflags = (uint32_t)__float_as_int(d4.w);
            if (bounce == 0) SR_COUNT(c, SR_COUNTER_SAMPLE, 1);
            Ray ray = make_ray(V3{o4.x, o4.y, o4.z}, V3{d4.x, d4.y, d4.z});
            float4 rad4 = W.rad[s];
            Col radiance{rad4.x, rad4.y, rad4.z};
            float spdf = rad4.w;
            Col energy = col3(W.energy[s]);
            float4 h0 = W.hit[s];
            float2 huv = W.hit_uv[s];
            Hit hit{__float_as_int(h0.x), __float_as_int(h0.y), h0.z, h0.w, huv.x, huv.y};
            bool has_hit = hit.obj >= 0;
            SurfHit sh;
            if (has_hit) surface_from_hit<COUNT, GENERAL>(S, ray, hit, sh, c);
            float sdist;
            // Event of this segment (scene.cs:654-738): fog scatter (free-flight distance drawn first
            // when fog is set), surface hit, or miss.  Fog and surface events share one light sample,
            // one Russian-roulette draw and then scatter, in that RNG order, so those calls exist once.
            bool fog_event = S.has_fog && fog_scatter_distance(S, ray, has_hit ? sh.dist : inf, rng, sdist);
            if (fog_event || has_hit) {
                const Surface& su = sh.surf;
                const float dist = sh.dist;
                const V3 view = -ray.d;
                float bias = 0.0f;
                V3 pos;
                if (fog_event) {
                    energy = energy * col3(S.fog_color);
                    pos = ray_at(ray, sdist);
                } else {
                    bias = fmaxf(1e-4f, dist * 1e-4f);
                    pos = ray_at(ray, dist - bias);
                    if (GENERAL && (pflags & PF_MEDIUM)) energy = energy * beer_law(col3(W.medium[s]), dist);
                    radiance = radiance + su.radiance * energy;
                    if (bounce == 0) {
                        pflags |= PF_PRIMARY;
                        W.prim[s] = make_float4(su.normal.x, su.normal.y, su.normal.z, dist);
                        W.prim_uv[s] = make_float2(su.uv.x, su.uv.y);
                    }
                }
                // NEE toward the sky (SampleSkyDirectFog scene.cs:796-810 / SampleSkyDirect :774-794);
                // the shadow ray and the contribution are deferred
                V3 ldir;
                float lpdf;
                if (sky_light_rand<COUNT, GENERAL>(S, rng, ldir, lpdf, c) && lpdf > 0.0f) {
                    bool emit = true;
                    Col w3;
                    float mis;
                    if (fog_event) {
                        float fog_pdf = hg_pdf(dot(ray.d, ldir), S.fog_g);
                        mis = power_heuristic(lpdf, fog_pdf);
                        w3 = gray(fog_pdf);
                    } else {
                        V3 nn = dot(su.normal, view) >= 0.0f ? su.normal : -su.normal;
                        V3 ng = dot(su.normal_geo, view) >= 0.0f ? su.normal_geo : -su.normal_geo;
                        emit = dot(nn, ldir) > 0.0f && dot(ng, ldir) > 0.0f;
                        if (emit) {
                            w3 = opaque_eval(su, view, ldir);
                            mis = power_heuristic(lpdf, opaque_pdf(su, view, ldir, specular_probability(su, view)));
                        }
                    }
                    if (emit) {
                        rflags |= RF_SHADOW | ((fog_event && bounce == 0) ? RF_FOG : 0u);
                        W.sh0[s] = make_float4(pos.x, pos.y, pos.z, 0.f);
                        W.sh1[s] = make_float4(ldir.x, ldir.y, ldir.z, lpdf);
                        W.sh2[s] = make_float4(w3.r, w3.g, w3.b, mis);
                        W.sh3[s] = make_float4(energy.r, energy.g, energy.b, 0.f);
                    }
                }
                if (russian_roulette(energy, bounce, rng)) {
                    rflags |= RF_TERMINATE;
                } else if (fog_event) {
                    V3 sdir = hg_scatter_dir(ray.d, S.fog_g, rng);
                    pflags |= PF_SPDF;
                    spdf = hg_pdf(dot(ray.d, sdir), S.fog_g);
                    ray = make_ray(pos, sdir);
                } else {
                    Scatter sc = surface_scatter<GENERAL>(su, ray.d, view, rng);
                    energy = energy * sc.weight;
                    energy = clamp_luminance(energy, P.indirect_clamp);
                    bool enter = dot(sc.dir, su.normal_geo) < 0.0f;
                    if (GENERAL && sc.refracted) {
                        if (enter) {
                            pflags |= PF_MEDIUM;
                            W.medium[s] = make_float4(su.albedo.r, su.albedo.g, su.albedo.b, 0.f);
                        } else {
                            pflags &= ~PF_MEDIUM;
                        }
                    } else if (!enter) {
                        pflags &= ~PF_MEDIUM;
                    }
                    pflags = sc.has_pdf ? (pflags | PF_SPDF) : (pflags & ~PF_SPDF);
                    spdf = sc.pdf;
                    ray = make_ray(ray_at(ray, dist) + sc.dir * bias, sc.dir);
                }
            } else {
                // miss: sky radiance with the MIS weight of the last scatter (scene.cs:728-738)
                float mis = (pflags & PF_SPDF) ? power_heuristic(spdf, sky_light_pdf<GENERAL>(S, ray.d)) : 1.0f;
                radiance = radiance + sky_radiance<COUNT, GENERAL>(S, ray.d, c) * mis * energy;
                rflags |= RF_TERMINATE;
            }
            if (!(rflags & RF_TERMINATE) && ++bounce == P.bounces + 1) rflags |= RF_TERMINATE;
            store_rng(W, s, rng);
            W.ray_o[s] = make_float4(ray.o.x, ray.o.y, ray.o.z, __int_as_float((int)bounce));
            W.ray_d[s] = make_float4(ray.d.x, ray.d.y, ray.d.z, __int_as_float((int)pflags));
            W.rad[s] = make_float4(radiance.r, radiance.g, radiance.b, spdf);
            W.energy[s] = make_float4(energy.r, energy.g, energy.b, 0.f);
            if (rflags) W.sh0[s].w = __int_as_float((int)rflags);
        }
        push(W.q_active[nxt], &W.counts[nxt], s, valid && rflags == 0);
        push(W.q_resolve, &W.counts[2], s, valid && rflags != 0);
        push(W.q_shadow, &W.counts[6], s, valid && (rflags & RF_SHADOW));
    }
    flush_counters<COUNT>(c, counters);
}

template <bool COUNT, bool GENERAL>
__global__ void __launch_bounds__(128) k_wave_finalize(WaveState W, DevScene S, DevView V, DevParams P, DevAovs out,
                                                       int cur, uint32_t* err, unsigned long long* counters) {
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counts[4] = 0;  // next extend's fetch counter
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    const int nxt = cur ^ 1;
    const uint32_t n = W.counts[2];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        uint32_t k = base + threadIdx.x;
        bool valid = k < n;
        uint32_t s = valid ? W.q_resolve[k] : 0u;
        bool live = false;
        if (valid) {
            float4 s0 = W.sh0[s];
            uint32_t rflags = (uint32_t)__float_as_int(s0.w);
            if (rflags & RF_SHADOW) {
                // the rest of SampleSkyDirect / SampleSkyDirectFog (scene.cs:774-810) once the
                // shadow kernel has left the transmittance (incl. fog) in sh0.xyz
                Col tr = col3(s0);
                if (max_component(tr) > 0.0f) {
                    float4 s1 = W.sh1[s], s2 = W.sh2[s], s3 = W.sh3[s];
                    V3 ldir{s1.x, s1.y, s1.z};
                    Col contrib = sky_radiance<COUNT, GENERAL>(S, ldir, c) * tr * col3(s2) * s2.w / s1.w;
                    Col add = contrib * col3(s3);
                    if (rflags & RF_FOG) {
                        float4 f = W.fog[s];
                        W.fog[s] = make_float4(f.x + add.r, f.y + add.g, f.z + add.b, f.w);
                    } else {
                        float4 r = W.rad[s];
                        W.rad[s] = make_float4(r.x + add.r, r.y + add.g, r.z + add.b, r.w);
                    }
                }
            }
            // clear the request flags so a later bounce without a request is not re-resolved
            W.sh0[s].w = __int_as_float(0);
            live = !(rflags & RF_TERMINATE);
            if (!live) {
                // end of a sample: pixel statistics and the adaptive stop (renderer.cs:173-212)
                Col radiance = col3(W.rad[s]);
                Col radiance_fog = col3(W.fog[s]);
                uint32_t pflags = (uint32_t)__float_as_int(W.ray_d[s].w);
                float4 a0 = W.acc0[s], a1 = W.acc1[s], a2 = W.acc2[s], a3 = W.acc3[s], a4 = W.acc4[s], a5 = W.acc5[s];
                a0.x += radiance.r, a0.y += radiance.g, a0.z += radiance.b;
                a1.x += radiance_fog.r, a1.y += radiance_fog.g, a1.z += radiance_fog.b;
                float lum = luminance(radiance) + luminance(radiance_fog);
                a0.w += lum;
                a1.w += lum * lum;
                float ls = luminance(radiance);
                a2.w += ls;
                a3.w += ls * ls;
                uint32_t ncount = (uint32_t)__float_as_int(a4.y), dcount = (uint32_t)__float_as_int(a4.z);
                uint32_t si = (uint32_t)__float_as_int(a4.w);
                if (pflags & PF_PRIMARY) {
                    float4 pr = W.prim[s];
                    a2.x += pr.x, a2.y += pr.y, a2.z += pr.z;
                    a3.x = pr.x, a3.y = pr.y, a3.z = pr.z;
                    ncount++;
                    a4.x += pr.w;
                    dcount++;
                    if (__float_as_int(a5.z) == 0) {
                        float2 uv = W.prim_uv[s];
                        a5 = make_float4(uv.x, uv.y, __int_as_float(1), 0.f);
                    }
                }
                bool done = false;
                uint32_t count = 0;
                if (si >= P.min_samples - 1 && relative_std_err(a0.w, a1.w, si + 1) < P.variance_threshold) {
                    done = true;
                    count = si + 1;
                } else if (++si == P.max_samples) {
                    done = true;
                    count = si + 1;  // loop ran out: normalised by maxSamples + 1 (renderer.cs:215)
                }
                uint32_t x, y;
                slot_pixel(W, s, x, y);
                if (done) {
                    float var = relative_std_err(a2.w, a3.w, count);
                    Col r = col3(a0) / (float)count;
                    Col f = col3(a1) / (float)count;
                    V3 nsum{a2.x, a2.y, a2.z}, nfb{a3.x, a3.y, a3.z};
                    V3 nrm = ncount > 0 ? normalize_or(nsum, nfb) : V3{0.f, 0.f, 0.f};
                    size_t i = (size_t)y * P.width + x;
                    out.radiance[3 * i] = r.r, out.radiance[3 * i + 1] = r.g, out.radiance[3 * i + 2] = r.b;
                    out.radiance_fog[3 * i] = f.r, out.radiance_fog[3 * i + 1] = f.g, out.radiance_fog[3 * i + 2] = f.b;
                    out.normals[3 * i] = nrm.x, out.normals[3 * i + 1] = nrm.y, out.normals[3 * i + 2] = nrm.z;
                    out.uv[2 * i] = a5.x, out.uv[2 * i + 1] = a5.y;
                    out.depth[i] = dcount > 0 ? a4.x / (float)dcount : __int_as_float(0x7f800000);
                    out.samples[i] = count;
                    out.variance[i] = var;
                } else {
                    Rng rng = load_rng(W, s);
                    Ray ray = camera_ray(V, P, x, y, rng);
                    store_rng(W, s, rng);
                    begin_sample(W, s, ray);
                    live = true;
                }
                a4.y = __int_as_float((int)ncount), a4.z = __int_as_float((int)dcount), a4.w = __int_as_float((int)si);
                W.acc0[s] = a0, W.acc1[s] = a1, W.acc2[s] = a2, W.acc3[s] = a3, W.acc4[s] = a4, W.acc5[s] = a5;
            }
        }
        push(W.q_active[nxt], &W.counts[nxt], s, valid && live);
    }
    flush_counters<COUNT>(c, counters);
}

// Condition of the device-side bounce loop: continue while paths are live and the bounce cap
// (max_samples * (bounces + 1) per pixel, plus slack) is not reached.
__global__ void k_wave_continue(cudaGraphConditionalHandle handle, uint32_t* counts, uint32_t max_iters, uint32_t* err) {
    uint32_t it = counts[3] + 2;  // two bounces per loop body
    counts[3] = it;
    bool more = counts[0] > 0;
    if (more && it >= max_iters) {
        atomicOr(err, SR_DEVERR_LOOP);
        more = false;
    }
    cudaGraphSetConditional(handle, more ? 1u : 0u);
}

// ---- launchers ------------------------------------------------------------------------------------
template <bool COUNT, bool GENERAL>
static void launch_bounce(const WaveLaunch& L, int cur, cudaStream_t st) {
    k_wave_extend<COUNT, GENERAL><<<L.grid_extend, 128, 0, st>>>(L.W, L.S, cur, L.err, L.counters);
    k_wave_shade<COUNT, GENERAL><<<L.grid_shade, 128, 0, st>>>(L.W, L.S, L.P, cur, L.err, L.counters);
    k_wave_shadow<COUNT, GENERAL><<<L.grid_shadow, 128, 0, st>>>(L.W, L.S, L.err, L.counters);
    k_wave_finalize<COUNT, GENERAL><<<L.grid_resolve, 128, 0, st>>>(L.W, L.S, L.V, L.P, L.out, cur, L.err,
                                                                    L.counters);
}

void wave_grid_sizes(WaveLaunch& L, int sms) {
    int b0 = 0, b1 = 0, b2 = 0, b3 = 0;
    if (L.general) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b0, k_wave_extend<false, true>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_wave_shade<false, true>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_wave_finalize<false, true>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b3, k_wave_shadow<false, true>, 128, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b0, k_wave_extend<false, false>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_wave_shade<false, false>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_wave_finalize<false, false>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b3, k_wave_shadow<false, false>, 128, 0);
    }
    L.grid_extend = sms * (b0 > 0 ? b0 : 1);
    L.grid_shade = sms * (b1 > 0 ? b1 : 1);
    L.grid_resolve = sms * (b2 > 0 ? b2 : 1);
    L.grid_shadow = sms * (b3 > 0 ? b3 : 1);
}

cudaError_t wave_init(const WaveLaunch& L, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(L.W.counts, 0, 8 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    k_wave_init<<<(L.W.slots + 127) / 128, 128, 0, st>>>(L.W, L.V, L.P);
    return cudaGetLastError();
}

cudaError_t wave_bounce(const WaveLaunch& L, int cur, cudaStream_t st) {
    if (L.general) {
        if (L.counters)
            launch_bounce<true, true>(L, cur, st);
        else
            launch_bounce<false, true>(L, cur, st);
    } else {
        if (L.counters)
            launch_bounce<true, false>(L, cur, st);
        else
            launch_bounce<false, false>(L, cur, st);
    }
    return cudaGetLastError();
}

cudaError_t wave_build_graph(const WaveLaunch& L, cudaStream_t capture_stream, cudaGraphExec_t* exec_out) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle handle;
    e = cudaGraphConditionalHandleCreate(&handle, graph, 1u, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) {
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
        if (e == cudaSuccess) {
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            e = cudaStreamBeginCaptureToGraph(capture_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
            if (e == cudaSuccess) {
                wave_bounce(L, 0, capture_stream);
                wave_bounce(L, 1, capture_stream);
                k_wave_continue<<<1, 1, 0, capture_stream>>>(handle, L.W.counts, L.max_iters, L.err);
                cudaGraph_t captured = nullptr;
                cudaError_t e2 = cudaStreamEndCapture(capture_stream, &captured);
                e = e2 != cudaSuccess ? e2 : cudaGetLastError();
            }
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec_out, graph, 0);
    cudaGraphDestroy(graph);
    return e;
}

}  // namespace sr

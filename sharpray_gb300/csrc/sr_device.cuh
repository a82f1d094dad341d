// sr_device.cuh — device-side scene layout and the per-path arithmetic of SharpRay's hot path.
//
// Everything here is compiled with -fmad=false and IEEE division/sqrt so that every float
// operation matches the C# reference's single-precision evaluation order (left to right, no
// FMA contraction).  Integer work (RNG, BVH indices) is exact by construction; the BVH
// traversal is bit-exact, so closest-hit results equal the reference's.  The transcendental
// calls (sinf, cosf, expf, logf, powf, atan2f, asinf) are CUDA's, which differ from the C
// runtime by at most a few ulp; images are therefore compared statistically.
#pragma once

#include <cstdint>

#include "sr_layout.h"

namespace sr {

#define SR_DEV __device__ __forceinline__

constexpr float kPi = 3.14159265358979323846f;

// Transcendentals go through one non-inlined copy each: inlining every call site multiplies the
// kernels' machine code (the shading kernel exceeded the instruction cache), while the calls are
// few per path segment.  The functions are CUDA's own sinf/cosf/expf/logf/powf/atan2f/asinf.
static __device__ __noinline__ void sr_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
static __device__ __noinline__ float sr_exp(float x) { return expf(x); }
static __device__ __noinline__ float sr_log(float x) { return logf(x); }
static __device__ __noinline__ float sr_pow(float x, float y) { return powf(x, y); }
static __device__ __noinline__ float sr_atan2(float y, float x) { return atan2f(y, x); }
static __device__ __noinline__ float sr_asin(float x) { return asinf(x); }

// IEEE division and square root expand to ~17 instructions per call site; with SR_OUTLINE_DIV the
// vector helpers below share one out-of-line copy of each (same correctly rounded results), which
// keeps the shading kernels' machine code small enough for the instruction cache.
#ifndef SR_OUTLINE_DIV
#define SR_OUTLINE_DIV 0
#endif
#if SR_OUTLINE_DIV
static __device__ __noinline__ float sr_fdiv(float a, float b) { return a / b; }
static __device__ __noinline__ float sr_fsqrt(float a) { return sqrtf(a); }
#else
static __device__ __forceinline__ float sr_fdiv(float a, float b) { return a / b; }
static __device__ __forceinline__ float sr_fsqrt(float a) { return sqrtf(a); }
#endif

// ---- small vector types ------------------------------------------------------------------------
struct V2 {
    float x, y;
};
struct V3 {
    float x, y, z;
};
struct V4 {
    float x, y, z, w;
};
struct Col {
    float r, g, b;
};

SR_DEV V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
SR_DEV V2 operator*(V2 v, float s) { return {v.x * s, v.y * s}; }
SR_DEV V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
SR_DEV V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
SR_DEV V3 operator-(V3 v) { return {-v.x, -v.y, -v.z}; }
SR_DEV V3 operator*(V3 a, float b) { return {a.x * b, a.y * b, a.z * b}; }
SR_DEV V3 operator*(float a, V3 b) { return {a * b.x, a * b.y, a * b.z}; }
SR_DEV V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
SR_DEV V3 operator/(V3 a, float b) { return {sr_fdiv(a.x, b), sr_fdiv(a.y, b), sr_fdiv(a.z, b)}; }
SR_DEV V3 operator/(V3 a, V3 b) { return {sr_fdiv(a.x, b.x), sr_fdiv(a.y, b.y), sr_fdiv(a.z, b.z)}; }
SR_DEV float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SR_DEV V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
SR_DEV float mag_sqr(V3 v) { return dot(v, v); }
SR_DEV float magnitude(V3 v) { return sr_fsqrt(mag_sqr(v)); }
SR_DEV V3 normalize(V3 v) { return v / magnitude(v); }
SR_DEV V3 normalize_or(V3 v, V3 fb) {
    float m = mag_sqr(v);
    return m >= 1e-12f ? v / sr_fsqrt(m) : fb;
}
SR_DEV V3 up3() { return {0.f, 1.f, 0.f}; }
SR_DEV V3 right3() { return {1.f, 0.f, 0.f}; }
SR_DEV V4 operator+(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
SR_DEV V4 operator*(V4 a, float b) { return {a.x * b, a.y * b, a.z * b, a.w * b}; }
SR_DEV V3 xyz(V4 v) { return {v.x, v.y, v.z}; }
SR_DEV V3 v3(float4 f) { return {f.x, f.y, f.z}; }

SR_DEV Col operator+(Col a, Col b) { return {a.r + b.r, a.g + b.g, a.b + b.b}; }
SR_DEV Col operator-(Col a, Col b) { return {a.r - b.r, a.g - b.g, a.b - b.b}; }
SR_DEV Col operator*(Col a, Col b) { return {a.r * b.r, a.g * b.g, a.b * b.b}; }
SR_DEV Col operator*(Col c, float s) { return {c.r * s, c.g * s, c.b * s}; }
SR_DEV Col operator*(float s, Col c) { return {c.r * s, c.g * s, c.b * s}; }
SR_DEV Col operator/(Col c, float s) { return {sr_fdiv(c.r, s), sr_fdiv(c.g, s), sr_fdiv(c.b, s)}; }
SR_DEV Col operator/(Col a, Col b) { return {sr_fdiv(a.r, b.r), sr_fdiv(a.g, b.g), sr_fdiv(a.b, b.b)}; }
SR_DEV Col gray(float v) { return {v, v, v}; }
SR_DEV Col black() { return {0.f, 0.f, 0.f}; }
SR_DEV Col white() { return {1.f, 1.f, 1.f}; }
SR_DEV float luminance(Col c) { return 0.2126f * c.r + 0.7152f * c.g + 0.0722f * c.b; }
SR_DEV float max_component(Col c) { return fmaxf(c.r, fmaxf(c.g, c.b)); }
SR_DEV Col clamp_luminance(Col c, float max) {
    float lum = luminance(c);
    return lum > max ? c * (max / lum) : c;
}
SR_DEV Col lerp(Col a, Col b, float t) { return {a.r + (b.r - a.r) * t, a.g + (b.g - a.g) * t, a.b + (b.b - a.b) * t}; }
SR_DEV Col bilerp(Col c1, Col c2, Col c3, Col c4, float tx, float ty) { return lerp(lerp(c1, c2, tx), lerp(c3, c4, tx), ty); }
SR_DEV float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
SR_DEV Col col3(float4 f) { return {f.x, f.y, f.z}; }

// ---- quaternions (Quat * Vec3, math.cs:609-617) ------------------------------------------------
SR_DEV V3 quat_rotate(float4 q, V3 v) {
    V3 axis{q.x, q.y, q.z};
    float sqr = mag_sqr(axis);
    V3 a = axis * (dot(axis, v) * 2.0f);
    V3 b = v * (q.w * q.w - sqr);
    V3 c = cross(axis, v) * (q.w * 2.0f);
    return a + b + c;
}
SR_DEV float4 quat_inverse(float4 q) { return make_float4(-q.x, -q.y, -q.z, q.w); }

// ---- rays (Ray ctor math.cs:846-857) -------------------------------------------------------------
struct Ray {
    V3 o, d, inv;
};
SR_DEV float safe_comp(float d) { return fabsf(d) >= 1e-8f ? d : copysignf(1e-8f, d); }
SR_DEV Ray make_ray(V3 o, V3 d) {
    Ray r;
    r.o = o;
    r.d = d;
    r.inv = {1.0f / safe_comp(d.x), 1.0f / safe_comp(d.y), 1.0f / safe_comp(d.z)};
    return r;
}
SR_DEV V3 ray_at(const Ray& r, float t) { return r.o + r.d * t; }

// ---- RNG: xorwow-style generator seeded by splitmix64 (math.cs:1665-1743) -------------------------
struct Rng {
    uint32_t s0, s1, s2, s3, s4;
};
SR_DEV uint64_t split_mix64(uint64_t& state) {
    uint64_t r = state += 0x9e3779b97f4a7c15ULL;
    r = (r ^ (r >> 30)) * 0xbf58476d1ce4e5b9ULL;
    r = (r ^ (r >> 27)) * 0x94d049bb133111ebULL;
    return r ^ (r >> 31);
}
// Rng(a, b) (math.cs:1665-1743); `stream` != 0 selects another, independent stream per (a, b) (an
// extension: 0 is the reference's seeding).
SR_DEV Rng rng_seed(uint32_t a, uint32_t b, uint32_t stream = 0) {
    uint64_t seed = ((uint64_t)a << 32) | b;
    if (stream) seed ^= (uint64_t)stream * 0x9E3779B97F4A7C15ull;
    uint64_t v1 = split_mix64(seed);
    uint64_t v2 = split_mix64(seed);
    return {(uint32_t)v1, (uint32_t)(v1 >> 32), (uint32_t)v2, (uint32_t)(v2 >> 32), 0u};
}
SR_DEV uint32_t rng_uint(Rng& r) {
    uint32_t t = r.s3;
    uint32_t s = r.s0;
    r.s3 = r.s2;
    r.s2 = r.s1;
    r.s1 = s;
    t ^= t >> 2;
    t ^= t << 1;
    t ^= s ^ (s << 4);
    r.s0 = t;
    r.s4 += 362437u;
    return t + r.s4;
}
SR_DEV float rng_float(Rng& r) {
    const float to_float = 1.0f / (4294967296.0f + 512.0f);
    return __uint2float_rn(rng_uint(r)) * to_float;
}
SR_DEV float rng_exponential(Rng& r) {
    float u;
    do {
        u = rng_float(r);
    } while (u <= 1e-8f);
    return -sr_log(u);
}
SR_DEV void rng_gauss(Rng& r, float& a_out, float& b_out) {
    float a;
    do {
        a = rng_float(r);
    } while (a <= 1e-8f);
    float b = (kPi * 2.0f) * rng_float(r);
    float mag = sqrtf(-2.0f * sr_log(a));
    float sb, cb;
    sr_sincos(b, &sb, &cb);
    a_out = mag * cb;
    b_out = mag * sb;
}
SR_DEV V2 rand_v2(Rng& r) {
    float x = rng_float(r);
    float y = rng_float(r);
    return {x, y};
}
SR_DEV V3 rand_on_sphere(Rng& r) {
    while (true) {
        float x, y, z, unused;
        rng_gauss(r, x, y);
        rng_gauss(r, z, unused);
        float m = x * x + y * y + z * z;
        if (m > 1e-6f) return V3{x, y, z} / sqrtf(m);
    }
}

// ---- work counters (per thread, flushed once per warp) --------------------------------------------
struct Ctr {
    uint32_t v[SR_COUNTER_COUNT];
};
#define SR_COUNT(c, idx, n)            \
    do {                               \
        if (COUNT) (c).v[(idx)] += (n); \
    } while (0)

// ---- AABB slab test (AABox.IntersectDist math.cs:983-1004) ----------------------------------------
SR_DEV bool slab(float4 lo, float4 hi, const Ray& r, float& t_out) {
    float t1 = (lo.x - r.o.x) * r.inv.x;
    float t2 = (hi.x - r.o.x) * r.inv.x;
    float t3 = (lo.y - r.o.y) * r.inv.y;
    float t4 = (hi.y - r.o.y) * r.inv.y;
    float t5 = (lo.z - r.o.z) * r.inv.z;
    float t6 = (hi.z - r.o.z) * r.inv.z;
    float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
    float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
    if (tmax < 0.0f || tmin > tmax) return false;
    t_out = fmaxf(0.0f, tmin);
    return true;
}

// ---- Moller-Trumbore (TriangleLean.Intersect math.cs:1407-1435) ------------------------------------
SR_DEV bool tri_hit(V3 a, V3 ab, V3 ac, const Ray& r, float& t_out, float& u_out, float& v_out) {
    V3 h = cross(r.d, ac);
    float det = dot(ab, h);
    if (fabsf(det) <= 1e-7f) return false;
    float inv_det = 1.0f / det;
    const float eps = 1e-7f;
    V3 ao = r.o - a;
    float u = dot(ao, h) * inv_det;
    if (u < -eps || u > (1.0f + eps)) return false;
    V3 q = cross(ao, ab);
    float v = dot(r.d, q) * inv_det;
    if (v < -eps || (u + v) > (1.0f + eps)) return false;
    float t = dot(ac, q) * inv_det;
    if (t < 0.0f) return false;
    t_out = t;
    u_out = u;
    v_out = v;
    return true;
}

// Traversal stack entry: the pushed node's own (child, count) record and its entry distance.
struct StackEntry {
    int child;
    int count;
    float t;
};
constexpr int kStackSize = 128;  // bvh.cs:172 stackalloc size; depth cap 64 keeps use <= 65.

// Traversal stacks.  LocalStack is a per-thread array in local memory.  SplitStack keeps the first
// N entries of each thread's stack in shared memory and the rest in a per-thread local array.  Its
// shared words are laid out [entry][word][thread of the block], so the 32 lanes of a warp always
// touch 32 different banks, whatever stack depth each lane is at; local memory interleaves the
// threads of a warp word by word, so lanes at different depths touch different 128-byte lines.
struct LocalStack {
    StackEntry* a;
    SR_DEV StackEntry get(int i) const { return a[i]; }
    SR_DEV void set(int i, const StackEntry& e) { a[i] = e; }
};
template <int N, int BLOCK>
struct SplitStack {
    uint32_t* sm;   // this thread's first word: the block's shared array + threadIdx.x
    StackEntry* a;  // entries N and up
    SR_DEV StackEntry get(int i) const {
        if (i >= N) return a[i - N];
        const uint32_t* p = sm + (size_t)i * 3 * BLOCK;
        return {(int)p[0], (int)p[BLOCK], __uint_as_float(p[2 * BLOCK])};
    }
    SR_DEV void set(int i, const StackEntry& e) {
        if (i >= N) {
            a[i - N] = e;
            return;
        }
        uint32_t* p = sm + (size_t)i * 3 * BLOCK;
        p[0] = (uint32_t)e.child;
        p[BLOCK] = (uint32_t)e.count;
        p[2 * BLOCK] = __float_as_uint(e.t);
    }
};

// Read-only scene data (BVH nodes, triangles, attributes, texels, CDF tables) goes through the
// non-coherent path.  SR_SCENE_HINT = 1 adds the L2 eviction priority evict_last so that the path
// state streaming through L2 every bounce evicts it last; measured on GB300 at 1080p it did not
// help (the traversal is latency-bound on L1/L2 hits already), so it is off by default.
#ifndef SR_SCENE_HINT
#define SR_SCENE_HINT 0
#endif
#if SR_SCENE_HINT
SR_DEV uint64_t scene_policy() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
SR_DEV float4 ldg4(const float4* ptr) {
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(ptr), "l"(scene_policy()));
    return v;
}
SR_DEV float ldg1(const float* ptr) {
    float v;
    asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(ptr), "l"(scene_policy()));
    return v;
}
SR_DEV uint32_t ldgu(const uint32_t* ptr) {
    uint32_t v;
    asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(ptr), "l"(scene_policy()));
    return v;
}
#else
SR_DEV float4 ldg4(const float4* p) { return __ldg(p); }
SR_DEV float ldg1(const float* p) { return __ldg(p); }
SR_DEV uint32_t ldgu(const uint32_t* p) { return __ldg(p); }
#endif

// ---- shape hits ---------------------------------------------------------------------------------
struct ShapeHit {
    float dist;
    V3 norm, norm_geo;
    V4 tan;
    V2 uv;
};

// Transform.TransformRayInv math.cs:816-822.
SR_DEV Ray to_local(const DevObject& o, const Ray& r, float& scale) {
    float4 inv = quat_inverse(o.rot);
    V3 s = v3(o.scale_root);
    V3 origin = quat_rotate(inv, r.o - v3(o.pos_kind)) / s;
    V3 dir_raw = quat_rotate(inv, r.d) / s;
    scale = magnitude(dir_raw);
    return make_ray(origin, dir_raw / scale);
}

// Sphere.Intersect math.cs:1210-1234.
SR_DEV bool sphere_hit(float4 sc, const Ray& r, ShapeHit& h, bool full) {
    V3 c = v3(sc);
    float rad = sc.w;
    V3 tc = c - r.o;
    float ds = mag_sqr(tc);
    float a = dot(tc, r.d);
    float disc = rad * rad - ds + a * a;
    if (disc < 0.0f) return false;
    float f = sqrtf(disc);
    float t = ds < rad * rad ? a + f : a - f;
    if (t < 0.0f) return false;
    h.dist = t;
    if (full) {
        V3 n = normalize(ray_at(r, t) - c);
        V3 txyz = normalize_or(V3{-n.z, 0.0f, n.x}, right3());
        h.norm = n;
        h.norm_geo = n;
        h.tan = {txyz.x, txyz.y, txyz.z, 1.0f};
        h.uv = {0.5f + sr_atan2(n.z, n.x) / (2.0f * kPi), 0.5f - sr_asin(clampf(n.y, -1.0f, 1.0f)) / kPi};
    }
    return true;
}

// AABox.Intersect math.cs:1006-1059.
SR_DEV bool box_hit(float4 lo, float4 hi, const Ray& r, ShapeHit& h, bool full) {
    float t1 = (lo.x - r.o.x) * r.inv.x;
    float t2 = (hi.x - r.o.x) * r.inv.x;
    float t3 = (lo.y - r.o.y) * r.inv.y;
    float t4 = (hi.y - r.o.y) * r.inv.y;
    float t5 = (lo.z - r.o.z) * r.inv.z;
    float t6 = (hi.z - r.o.z) * r.inv.z;
    float mina = fminf(t1, t2), minb = fminf(t3, t4), minc = fminf(t5, t6);
    float maxa = fmaxf(t1, t2), maxb = fmaxf(t3, t4), maxc = fmaxf(t5, t6);
    float tmin = fmaxf(fmaxf(mina, minb), minc);
    float tmax = fminf(fminf(maxa, maxb), maxc);
    if (tmax < 0.0f || tmin > tmax) return false;
    bool inside = tmin < 0.0f;
    float t = inside ? tmax : tmin;
    h.dist = t;
    if (full) {
        V3 p = ray_at(r, t);
        V3 n;
        V4 tan;
        V2 face;
        if (mina >= minb && mina >= minc) {
            bool neg = t1 <= t2;
            n = neg ? V3{-1.f, 0.f, 0.f} : V3{1.f, 0.f, 0.f};
            tan = {0.f, 1.f, 0.f, neg ? -1.0f : 1.0f};
            face = {(p.y - lo.y) / (hi.y - lo.y), (p.z - lo.z) / (hi.z - lo.z)};
        } else if (minb >= mina && minb >= minc) {
            bool neg = t3 <= t4;
            n = neg ? V3{0.f, -1.f, 0.f} : V3{0.f, 1.f, 0.f};
            tan = {1.f, 0.f, 0.f, neg ? 1.0f : -1.0f};
            face = {(p.x - lo.x) / (hi.x - lo.x), (p.z - lo.z) / (hi.z - lo.z)};
        } else {
            bool neg = t5 <= t6;
            n = neg ? V3{0.f, 0.f, -1.f} : V3{0.f, 0.f, 1.f};
            tan = {1.f, 0.f, 0.f, neg ? -1.0f : 1.0f};
            face = {(p.x - lo.x) / (hi.x - lo.x), (p.y - lo.y) / (hi.y - lo.y)};
        }
        V3 nn = inside ? -n : n;
        h.norm = nn;
        h.norm_geo = nn;
        h.tan = tan;
        h.uv = face;
    }
    return true;
}

// TriangleLean.Inflate math.cs:1437-1459 for the triangle at reordered position `pos`.
SR_DEV ShapeHit inflate(const DevScene& S, int pos, float dist, float u, float v) {
    const float4* tp = S.tris + 3 * pos;
    V3 ab = v3(ldg4(tp + 1)), ac = v3(ldg4(tp + 2));
    const float4* ap = S.attrs + 7 * pos;
    float4 q0 = ldg4(ap), q1 = ldg4(ap + 1), q2 = ldg4(ap + 2), q3 = ldg4(ap + 3), q4 = ldg4(ap + 4), q5 = ldg4(ap + 5),
           q6 = ldg4(ap + 6);
    // attribute record: na.xyz nb.x | nb.yz nc.xy | nc.z ta.xyz | ta.w tb.xyz | tb.w tc.xyz | tc.w uva.xy uvb.x | uvb.y uvc.xy -
    V3 na{q0.x, q0.y, q0.z}, nb{q0.w, q1.x, q1.y}, nc{q1.z, q1.w, q2.x};
    V4 ta{q2.y, q2.z, q2.w, q3.x}, tb{q3.y, q3.z, q3.w, q4.x}, tc{q4.y, q4.z, q4.w, q5.x};
    V2 uva{q5.y, q5.z}, uvb{q5.w, q6.x}, uvc{q6.y, q6.z};
    float w = 1.0f - u - v;
    V3 face = normalize_or(cross(ab, ac), up3());
    V3 ni = na * w + nb * u + nc * v;
    V3 norm = mag_sqr(ni) >= 1e-12f ? normalize(ni) : face;
    V4 ti = ta * w + tb * u + tc * v;
    V3 txyz = xyz(ti);
    V3 tan_xyz = normalize_or(txyz - dot(txyz, norm) * norm, right3());
    ShapeHit h;
    h.dist = dist;
    h.norm = norm;
    h.norm_geo = face;
    h.tan = {tan_xyz.x, tan_xyz.y, tan_xyz.z, ti.w >= 0.0f ? 1.0f : -1.0f};
    h.uv = uva * w + uvb * u + uvc * v;
    return h;
}

// Result of a scene closest-hit query before inflation.
struct Hit {
    int obj;     // position of the object in the scene-BVH item order, -1 = miss
    int tri;     // reordered triangle position (meshes), -1 otherwise
    float dist;  // world distance (hit.Dist / localRayScale)
    float tl;    // local distance (meshes)
    float u, v;  // barycentrics (meshes)
};

// Scene-level closest hit (ANY = false) or occlusion test (ANY = true) as ONE loop over a shared
// stack (SceneQuery below).  The reference nests two traversals: Bvh<Object>.Intersect
// (bvh.cs:165-216) calls, for each object of a scene-BVH leaf, Object.Intersect (math.cs:67-79)
// which runs a complete, unpruned mesh BVH traversal in the object's local space.  Here the mesh
// traversal of the current object pushes its entries above the scene entries (above `mesh_base`);
// the query swaps the traversal ray and the pruning distance when it enters and leaves an object.
// Visit order, pruning (`t >= best` on pop, `t <= best` on push), tie-breaking (first strictly
// closer hit) and the per-object comparison `hit.Dist / localRayScale < bestDist` are the
// reference's, so results are bit-exact.  With ANY the search stops at the first hit found and
// prunes nothing, which gives the same yes/no answer as the closest-hit query.
constexpr int kSceneStack = 192;  // scene (<= 65) + mesh (<= 65) entries, with margin

// Resumable traversal state.  init() starts a ray; the query is then a sequence of actions, each
// chosen by `state`:
//   QS_NODE : visit the next node -- the nearer child kept from the last visit (the reference
//             pushes it last and pops it next, so it never needs to go through the stack) or the
//             stack top; an interior node tests its two children, a leaf moves to QS_TRI / QS_OBJ
//   QS_TRI  : test the triangles of a mesh leaf (bvh.cs:203-212)
//   QS_OBJ  : enter the next object of a scene leaf (to its local ray and mesh root)
//   QS_EXIT : an object's mesh traversal is complete: compare its hit with the scene's best
//   QS_DONE : `best` holds the answer
// Node actions and leaf actions are separate so that persistent kernels can run the node actions
// of all lanes together and batch the (long, divergent) leaf actions.  GENERAL = false compiles
// only what scenes of meshes need (no analytic shapes).  DYN = true (with ANY = false) makes the
// query kind a run-time choice (init's `any`), so one loop can serve closest-hit and occlusion
// queries: an occlusion query keeps its pruning distance at +inf, which makes every node test and
// push/pop decision the same as the ANY form's, and stops at its first hit.
enum : int { QS_NODE = 0, QS_TRI = 1, QS_OBJ = 2, QS_EXIT = 3, QS_DONE = 4 };

template <bool ANY, bool GENERAL, bool DYN = false>
struct SceneQuery {
    // The traversal stack lives outside the struct (a separate local array passed to the actions):
    // keeping the dynamically indexed array out lets the scalar state stay in registers.
    Ray wr;              // world ray
    Ray cr;              // ray of the current level (world, or the current object's local ray)
    float cur_best;      // pruning distance of the current level
    float lscale;        // local-ray scale of the current object
    float ob_u, ob_v;    // best hit inside the current object
    Hit best;
    StackEntry node;     // next node to visit when has_node (instead of the stack top)
    int sp, mesh_base, leaf_next, leaf_left, tri_next, tri_left, obj_pos, ob_tri;
    uint32_t pops;
    int state;
    bool in_mesh, has_node;
    bool any_hit;  // DYN: this query is an occlusion query

    SR_DEV bool is_any() const { return ANY || (DYN && any_hit); }

    // The query's state as kQueryWords words (and back), field by field so that it stays in
    // registers; ray reciprocals are recomputed by make_ray, which gives the same bits.
    static constexpr int kQueryWords = 36;
    SR_DEV void save(uint32_t* w) const {
        const float f[] = {wr.o.x, wr.o.y, wr.o.z, wr.d.x, wr.d.y, wr.d.z, cr.o.x, cr.o.y, cr.o.z, cr.d.x, cr.d.y,
                           cr.d.z, cur_best, lscale, ob_u, ob_v, best.dist, best.tl, best.u, best.v, node.t};
#pragma unroll
        for (int i = 0; i < 21; ++i) w[i] = __float_as_uint(f[i]);
        const int n[] = {best.obj, best.tri, node.child, node.count, sp, mesh_base, leaf_next, leaf_left, tri_next,
                         tri_left, obj_pos, ob_tri, (int)pops, state,
                         (in_mesh ? 1 : 0) | (has_node ? 2 : 0) | (any_hit ? 4 : 0)};
#pragma unroll
        for (int i = 0; i < 15; ++i) w[21 + i] = (uint32_t)n[i];
    }
    SR_DEV void load(const uint32_t* w) {
        auto f = [&](int i) { return __uint_as_float(w[i]); };
        wr = make_ray(V3{f(0), f(1), f(2)}, V3{f(3), f(4), f(5)});
        cr = make_ray(V3{f(6), f(7), f(8)}, V3{f(9), f(10), f(11)});
        cur_best = f(12), lscale = f(13), ob_u = f(14), ob_v = f(15);
        best = Hit{(int)w[21], (int)w[22], f(16), f(17), f(18), f(19)};
        node = StackEntry{(int)w[23], (int)w[24], f(20)};
        sp = (int)w[25], mesh_base = (int)w[26], leaf_next = (int)w[27], leaf_left = (int)w[28];
        tri_next = (int)w[29], tri_left = (int)w[30], obj_pos = (int)w[31], ob_tri = (int)w[32];
        pops = w[33];
        state = (int)w[34];
        in_mesh = (w[35] & 1u) != 0, has_node = (w[35] & 2u) != 0, any_hit = (w[35] & 4u) != 0;
    }

    SR_DEV void init(const DevScene& S, const Ray& r, bool any = false) {
        any_hit = any;
        const float inf = __int_as_float(0x7f800000);
        best = Hit{-1, -1, inf, 0.f, 0.f, 0.f};
        wr = r;
        cr = r;
        cur_best = inf;
        lscale = 1.0f;
        ob_u = ob_v = 0.f;
        mesh_base = leaf_next = leaf_left = tri_next = tri_left = 0;
        obj_pos = ob_tri = -1;
        pops = 0;
        in_mesh = false;
        sp = 0;
        has_node = false;
        state = QS_DONE;
        if (S.tlas_root >= 0) {
            float4 rn0 = ldg4(S.nodes + 2 * S.tlas_root);
            float4 rn1 = ldg4(S.nodes + 2 * S.tlas_root + 1);
            node = {__float_as_int(rn0.w), __float_as_int(rn1.w), 0.0f};
            has_node = true;
            state = QS_NODE;
        }
    }

    // The action after the current one, in the reference's order: finish the current mesh, then
    // the remaining objects of the current scene leaf, then the stack.
    SR_DEV void next_state() {
        if (in_mesh)
            state = (has_node || sp > mesh_base) ? QS_NODE : QS_EXIT;
        else if (leaf_left > 0)
            state = QS_OBJ;
        else
            state = (has_node || sp > 0) ? QS_NODE : QS_DONE;
    }

    // Every action counts against the scene's cap (DevScene::max_actions); past it the query ends
    // with the error word set, so a malformed tree (or a test's low cap) ends in an error, not a hang.
    SR_DEV bool count_action(const DevScene& S, uint32_t* err) {
        if (++pops > S.max_actions) {
            atomicOr(err, SR_DEVERR_LOOP);
            state = QS_DONE;
            return false;
        }
        return true;
    }

    template <bool COUNT, typename STK>
    SR_DEV void node_action(const DevScene& S, STK& stack, Ctr& c, uint32_t* err) {
        if (!count_action(S, err)) return;
        StackEntry e = has_node ? node : stack.get(--sp);
        has_node = false;
        if (!ANY && e.t >= cur_best) {
            next_state();
            return;
        }
        if (e.count == 0) {
            if (in_mesh)
                SR_COUNT(c, SR_COUNTER_BLAS_NODE, 2);
            else
                SR_COUNT(c, SR_COUNTER_TLAS_NODE, 2);
            const float4* n = S.nodes + 2 * e.child;
            float4 a0 = ldg4(n), a1 = ldg4(n + 1), b0 = ldg4(n + 2), b1 = ldg4(n + 3);
            float ta = 0.f, tb = 0.f;
            bool pa = slab(a0, a1, cr, ta) && (ANY || ta <= cur_best);
            bool pb = slab(b0, b1, cr, tb) && (ANY || tb <= cur_best);
            StackEntry ea{__float_as_int(a0.w), __float_as_int(a1.w), ta};
            StackEntry eb{__float_as_int(b0.w), __float_as_int(b1.w), tb};
            if (pa && pb) {
                // the nearer child is visited first; on a tie the second child is (bvh.cs:196-197)
                if (sp + 1 > kSceneStack) {
                    atomicOr(err, SR_DEVERR_STACK);
                    state = QS_DONE;
                    return;
                }
                bool a_first = ta < tb;
                stack.set(sp++, a_first ? eb : ea);
                node = a_first ? ea : eb;
                has_node = true;
            } else if (pa || pb) {
                node = pa ? ea : eb;
                has_node = true;
            }
            next_state();
        } else if (in_mesh) {
            SR_COUNT(c, SR_COUNTER_BLAS_SHAPE, (uint32_t)e.count);
            tri_next = e.child;
            tri_left = e.count;
            state = QS_TRI;
        } else {
            SR_COUNT(c, SR_COUNTER_TLAS_SHAPE, (uint32_t)e.count);
            leaf_next = e.child;
            leaf_left = e.count;
            next_state();
        }
    }

    template <bool COUNT, typename STK>
    SR_DEV void leaf_action(const DevScene& S, STK& stack, Ctr& c, uint32_t* err) {
        const float inf = __int_as_float(0x7f800000);
        if (!count_action(S, err)) return;
        if (state == QS_TRI) {
            // the whole mesh leaf, in leaf order (bvh.cs:203-212)
            for (; tri_left > 0; ++tri_next, --tri_left) {
                const float4* tp = S.tris + 3 * tri_next;
                float4 q0 = ldg4(tp), q1 = ldg4(tp + 1), q2 = ldg4(tp + 2);
                float t, u, v;
                if (tri_hit(v3(q0), v3(q1), v3(q2), cr, t, u, v) && (is_any() || t < cur_best)) {
                    if (is_any()) {
                        best = {obj_pos, tri_next, 0.f, 0.f, 0.f, 0.f};
                        tri_left = 0;
                        state = QS_DONE;
                        return;
                    }
                    cur_best = t;
                    ob_tri = tri_next;
                    ob_u = u;
                    ob_v = v;
                }
            }
            next_state();
        } else if (state == QS_EXIT) {
            // the object's mesh traversal is complete: Bvh<Object> leaf comparison (bvh.cs:207)
            if (ob_tri >= 0) {
                float d = cur_best / lscale;
                if (d < best.dist) best = {obj_pos, ob_tri, d, cur_best, ob_u, ob_v};
            }
            in_mesh = false;
            cr = wr;
            cur_best = is_any() ? inf : best.dist;
            next_state();
        } else if (state == QS_OBJ) {
            const DevObject& o = S.objects[leaf_next];
            obj_pos = leaf_next;
            ++leaf_next;
            --leaf_left;
            Ray l = to_local(o, wr, lscale);
            int kind = GENERAL ? __float_as_int(o.pos_kind.w) : SR_SHAPE_MESH;
            if (kind == SR_SHAPE_MESH) {
                int root = __float_as_int(o.scale_root.w);
                if (root >= 0) {  // an empty mesh never hits
                    float4 rn0 = ldg4(S.nodes + 2 * root);
                    float4 rn1 = ldg4(S.nodes + 2 * root + 1);
                    mesh_base = sp;
                    node = {__float_as_int(rn0.w), __float_as_int(rn1.w), 0.0f};
                    has_node = true;
                    in_mesh = true;
                    cr = l;
                    cur_best = inf;
                    ob_tri = -1;
                }
            } else if (GENERAL) {
                ShapeHit h;
                bool ok = kind == SR_SHAPE_SPHERE ? sphere_hit(o.shape0, l, h, false)
                                                  : box_hit(o.shape0, o.shape1, l, h, false);
                if (ok) {
                    if (is_any()) {
                        best = {obj_pos, -1, 0.f, 0.f, 0.f, 0.f};
                        state = QS_DONE;
                        return;
                    }
                    float d = h.dist / lscale;
                    if (d < best.dist) best = {obj_pos, -1, d, 0.f, 0.f, 0.f};
                    cur_best = best.dist;
                }
            }
            next_state();
        }
    }

    // One action of whatever kind is next; true when the query is answered.
    template <bool COUNT, typename STK>
    SR_DEV bool step(const DevScene& S, STK& stack, Ctr& c, uint32_t* err) {
        if (state == QS_NODE)
            node_action<COUNT>(S, stack, c, err);
        else if (state != QS_DONE)
            leaf_action<COUNT>(S, stack, c, err);
        return state == QS_DONE;
    }
};

// True when a query's first step -- the two children of the scene BVH's root -- already decides it
// (neither box is hit, so there is no hit), without a traversal; counts what that step counts.
// False when the root is a leaf or a child box is hit.
template <bool COUNT, bool ANY>
SR_DEV bool misses_scene(const DevScene& S, const Ray& r, Ctr& c) {
    if (S.tlas_root < 0) return true;
    const float4* root = S.nodes + 2 * S.tlas_root;
    float4 rn0 = ldg4(root), rn1 = ldg4(root + 1);
    if (__float_as_int(rn1.w) != 0) return false;
    SR_COUNT(c, SR_COUNTER_TLAS_NODE, 2);
    const float4* n = S.nodes + 2 * __float_as_int(rn0.w);
    float4 a0 = ldg4(n), a1 = ldg4(n + 1), b0 = ldg4(n + 2), b1 = ldg4(n + 3);
    const float inf = __int_as_float(0x7f800000);
    float ta = 0.f, tb = 0.f;
    bool pa = slab(a0, a1, r, ta) && (ANY || ta <= inf);
    bool pb = slab(b0, b1, r, tb) && (ANY || tb <= inf);
    return !pa && !pb;
}

template <bool COUNT, bool ANY, bool GENERAL = true>
SR_DEV Hit scene_traverse(const DevScene& S, const Ray& wr, Ctr& c, uint32_t* err) {
    StackEntry entries[kSceneStack];
    LocalStack stack{entries};
    SceneQuery<ANY, GENERAL> q;
    q.init(S, wr);
    while (!q.template step<COUNT>(S, stack, c, err)) {
    }
    return q.best;
}

template <bool COUNT, bool GENERAL = true>
SR_DEV Hit scene_closest(const DevScene& S, const Ray& r, Ctr& c, uint32_t* err) {
    return scene_traverse<COUNT, false, GENERAL>(S, r, c, err);
}

template <bool COUNT, bool GENERAL = true>
SR_DEV bool scene_any(const DevScene& S, const Ray& r, Ctr& c, uint32_t* err) {
    return scene_traverse<COUNT, true, GENERAL>(S, r, c, err).obj >= 0;
}

// The world-space ShapeHit of a scene hit (ShapeExtensions.Intersect math.cs:67-79).
template <bool COUNT, bool GENERAL = true>
SR_DEV ShapeHit world_hit(const DevScene& S, const Ray& r, const Hit& hit, Ctr& c) {
    const DevObject& o = S.objects[hit.obj];
    float scale;
    Ray lr = to_local(o, r, scale);
    int kind = GENERAL ? __float_as_int(o.pos_kind.w) : SR_SHAPE_MESH;
    ShapeHit h;
    if (!GENERAL || kind == SR_SHAPE_MESH) {
        SR_COUNT(c, SR_COUNTER_HIT_INFLATE, 1);
        h = inflate(S, hit.tri, hit.tl, hit.u, hit.v);
    } else if (kind == SR_SHAPE_SPHERE) {
        sphere_hit(o.shape0, lr, h, true);
    } else {
        box_hit(o.shape0, o.shape1, lr, h, true);
    }
    V3 s = v3(o.scale_root);
    V3 wn = normalize(quat_rotate(o.rot, h.norm / s));
    V3 wng = normalize(quat_rotate(o.rot, h.norm_geo / s));
    V3 wt = normalize(quat_rotate(o.rot, xyz(h.tan)));
    ShapeHit w;
    w.dist = h.dist / scale;
    w.norm = wn;
    w.norm_geo = wng;
    w.tan = {wt.x, wt.y, wt.z, h.tan.w};
    w.uv = h.uv;
    return w;
}

// ---- textures (Texture.Sample texture.cs:39-69) ----------------------------------------------------
template <bool COUNT>
SR_DEV Col tex_sample(const DevScene& S, int id, V2 coord, Ctr& c) {
    SR_COUNT(c, SR_COUNTER_TEX_SAMPLE, 1);
    const DevTexture& t = S.textures[id];
    float u = coord.x * t.tiling_x;
    u -= floorf(u);
    float v = coord.y * t.tiling_y;
    v -= floorf(v);
    const float4* tx = S.texels + t.offset;
    uint32_t w = t.width, hgt = t.height;
    if (t.filter == 1) {
        uint32_t x = (uint32_t)(u * (float)w) % w;
        uint32_t y = (uint32_t)(v * (float)hgt) % hgt;
        return col3(ldg4(tx + (size_t)y * w + x));
    }
    float fx = u * (float)(w - 1);
    float fy = v * (float)(hgt - 1);
    uint32_t x0 = (uint32_t)fx;
    uint32_t y0 = (uint32_t)fy;
    uint32_t x1 = (x0 + 1) % w;
    uint32_t y1 = (y0 + 1) % hgt;
    float txf = fx - (float)x0;
    float tyf = fy - (float)y0;
    return bilerp(col3(ldg4(tx + (size_t)y0 * w + x0)), col3(ldg4(tx + (size_t)y0 * w + x1)),
                  col3(ldg4(tx + (size_t)y1 * w + x0)), col3(ldg4(tx + (size_t)y1 * w + x1)), txf, tyf);
}

// ---- sky ----------------------------------------------------------------------------------------
SR_DEV V2 equirect_uv(V3 d) {
    float u = sr_atan2(d.z, d.x) / (kPi * 2.0f) + 0.5f;
    float v = 0.5f - sr_asin(clampf(d.y, -1.0f, 1.0f)) / kPi;
    return {u, v};
}
SR_DEV V3 from_equirect_uv(V2 uv) {
    float phi = (uv.x - 0.5f) * 2.0f * kPi;
    float st, ct, sp, cp;
    sr_sincos(kPi * uv.y, &st, &ct);
    sr_sincos(phi, &sp, &cp);
    return {st * cp, ct, st * sp};
}

template <bool COUNT, bool GENERAL = true>
SR_DEV Col sky_radiance(const DevScene& S, V3 dir, Ctr& c) {
    const DevSky& k = S.sky;
    if (!GENERAL || k.kind == 0) {
        SR_COUNT(c, SR_COUNTER_ENV_LOOKUP, 1);
        return tex_sample<false>(S, k.texture, equirect_uv(quat_rotate(k.rot_inv, dir)), c) * k.multiplier;
    }
    const float bias = 0.0001f;
    float top_b = 1.0f - sr_pow(fminf(1.0f, 1.0f + bias - dir.y), 4.0f);
    float bot_b = 1.0f - sr_pow(fminf(1.0f, 1.0f + bias + dir.y), 40.0f);
    float mid_b = 1.0f - top_b - bot_b;
    Col ambient = col3(k.top) * top_b + col3(k.middle) * mid_b + col3(k.bottom) * bot_b;
    float blend = fmaxf(0.0f, (dot(dir, v3(k.sun_dir)) - k.sun_cos) / (1.0f - k.sun_cos));
    return ambient + col3(k.sun_radiance) * blend;
}

// SkyTexture.LightDir / SunProcedural.LightDir (point-lookup pdf for MIS); 0 = null.
template <bool GENERAL = true>
SR_DEV float sky_light_pdf(const DevScene& S, V3 dir) {
    const DevSky& k = S.sky;
    if (!GENERAL || k.kind == 0) {
        if (k.cdf_total <= 0.0f) return 0.0f;
        V2 uv = equirect_uv(quat_rotate(k.rot_inv, dir));
        const DevTexture& t = S.textures[k.texture];
        int cx = (int)(uv.x * (float)t.width) % (int)t.width;
        int cy = (int)(uv.y * (float)t.height) % (int)t.height;
        cx = min(max(cx, 0), (int)t.width - 1);  // in range for every finite direction; guards NaN input
        cy = min(max(cy, 0), (int)t.height - 1);
        float pdf = luminance(col3(ldg4(S.texels + t.offset + (size_t)cy * t.width + cx))) * k.pdf_scale;
        return pdf > 0.0f ? pdf : 0.0f;
    }
    float ct = dot(dir, v3(k.sun_dir));
    if (ct < k.sun_cos) return 0.0f;
    float blend = (ct - k.sun_cos) / (1.0f - k.sun_cos);
    return blend / k.sun_pdf_denom;
}

// Cdf1.Sample cdf.cs:37-55 over cdf[0..n], accelerated by a bucket guide.  The reference's loop is
// a lower bound over the non-decreasing cdf[1..n] (prefix sums of non-negative weights divided by
// their total), i.e. r(u) = #{j : cdf[j+1] <= u}, clamped to n-1.  guide[k] holds r() at the
// smallest float u that falls into bucket k = (int)(u * n), so for any u in bucket k the answer
// lies in [guide[k], guide[k+1]]; bisecting that range with the same predicate returns exactly
// the reference's index while touching ~1-2 cdf entries instead of ~log2(n).
template <bool COUNT>
SR_DEV uint32_t cdf_sample(const float* cdf, const uint32_t* guide, uint32_t n, float norm, Ctr& c) {
    uint32_t k = min((uint32_t)(int)(norm * (float)n), n - 1);
    uint32_t lo = ldgu(guide + k), hi = ldgu(guide + k + 1);
    while (lo < hi) {
        SR_COUNT(c, SR_COUNTER_CDF_PROBE, 1);
        uint32_t mid = (lo + hi) >> 1;
        if (ldg1(cdf + mid + 1) <= norm)
            lo = mid + 1;
        else
            hi = mid;
    }
    return min(lo, n - 1);
}

// The direction toward the centre of sky texel (x, y) (SkyTexture.LightDirRand scene.cs:412-415).
SR_DEV V3 sky_texel_dir(const DevSky& k, const DevTexture& t, uint32_t x, uint32_t y) {
    V2 uv{((float)(int)x + 0.5f) / (float)(int)t.width, ((float)(int)y + 0.5f) / (float)(int)t.height};
    return quat_rotate(k.rot, from_equirect_uv(uv));
}

// ISky.LightDirRand (SkyTexture scene.cs:408-416, SunProcedural scene.cs:314-323).  `texel` is the
// sampled texel of a texture sky (-1 otherwise), whose radiance sky_light_radiance then reads.
template <bool COUNT, bool GENERAL = true>
SR_DEV bool sky_light_rand(const DevScene& S, Rng& rng, V3& dir, float& pdf, int& texel, Ctr& c) {
    const DevSky& k = S.sky;
    if (!GENERAL || k.kind == 0) {
        if (k.cdf_total <= 0.0f) return false;
        V2 u = rand_v2(rng);
        const DevTexture& t = S.textures[k.texture];
        SR_COUNT(c, SR_COUNTER_LIGHT_SAMPLE, 1);
        uint32_t y = cdf_sample<COUNT>(k.cdf_marginal, k.guide_marginal, t.height, u.y, c);
        size_t row = (size_t)y * (t.width + 1);
        uint32_t x = cdf_sample<COUNT>(k.cdf_cond + row, k.guide_cond + row, t.width, u.x, c);
        dir = sky_texel_dir(k, t, x, y);
        texel = (int)((size_t)y * t.width + x);
        pdf = k.center ? ldg4(k.center + texel).w
                       : luminance(col3(ldg4(S.texels + t.offset + (size_t)y * t.width + x))) * k.pdf_scale;
        return pdf > 0.0f;
    }
    texel = -1;
    float phi = (kPi * 2.0f) * rng_float(rng);
    float blend = sqrtf(rng_float(rng));
    float z = k.sun_cos + (1.0f - k.sun_cos) * blend;
    float st = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float sp, cp;
    sr_sincos(phi, &sp, &cp);
    dir = quat_rotate(k.sun_rot, V3{cp * st, sp * st, z});
    pdf = blend / k.sun_pdf_denom;
    return true;
}

template <bool COUNT, bool GENERAL = true>
SR_DEV bool sky_light_rand(const DevScene& S, Rng& rng, V3& dir, float& pdf, Ctr& c) {
    int texel;
    return sky_light_rand<COUNT, GENERAL>(S, rng, dir, pdf, texel, c);
}

// Sky radiance toward a light sample's direction: for a sampled texel of a texture sky the value
// evaluated at scene build (the same sky_radiance of the same direction, so the same bits), one
// 16-byte load next to the pdf just read instead of a bilinear lookup.
template <bool COUNT, bool GENERAL = true>
SR_DEV Col sky_light_radiance(const DevScene& S, int texel, V3 dir, Ctr& c) {
    if (texel >= 0 && S.sky.center) {
        SR_COUNT(c, SR_COUNTER_ENV_LOOKUP, 1);
        return col3(ldg4(S.sky.center + texel));
    }
    return sky_radiance<COUNT, GENERAL>(S, dir, c);
}

// ---- fog (scene.cs:445-496) -----------------------------------------------------------------------
SR_DEV float fog_density_at(const DevScene& S, float y) { return S.fog_density * sr_exp(-S.fog_falloff * y); }
// Homogeneous fog (an extension for falloff 0, no reference counterpart): the part [enter, exit) of
// ray r (t >= 0) below the medium's top height; false when the ray never is below it.
SR_DEV bool fog_slab_span(const DevScene& S, const Ray& r, float& enter, float& exit) {
    const float inf = __int_as_float(0x7f800000);
    const float hd = r.d.y, ho = r.o.y;
    enter = 0.0f;
    exit = inf;
    if (hd == 0.0f) return ho < S.fog_top;
    const float tc = (S.fog_top - ho) / hd;  // where the ray crosses the top
    if (hd > 0.0f) {
        exit = tc;
        return tc > 0.0f;
    }
    enter = fmaxf(0.0f, tc);
    return true;
}
SR_DEV float fog_transmittance_inf(const DevScene& S, const Ray& r) {
    if (S.fog_falloff == 0.0f) {  // homogeneous: density x the length below the top
        float enter, exit;
        if (!fog_slab_span(S, r, enter, exit)) return 1.0f;
        return sr_exp(-(S.fog_density * (exit - enter)));
    }
    // OpticalDepth over [0, +inf).
    float hd = r.d.y;
    float inf = __int_as_float(0x7f800000);
    float hs = r.o.y + 0.0f * hd;
    float he = r.o.y + inf * hd;
    float ds = fog_density_at(S, hs);
    float de = fog_density_at(S, he);
    float od = fabsf(hd) < 1e-6f ? ds * (inf - 0.0f) : (ds - de) / (S.fog_falloff * hd);
    return sr_exp(-od);
}
SR_DEV bool fog_scatter_distance(const DevScene& S, const Ray& r, float end, Rng& rng, float& t_out) {
    float hd = r.d.y;
    float ho = r.o.y;
    float hs = ho + 0.0f * hd;
    float u = rng_exponential(rng);
    float t;
    if (S.fog_falloff == 0.0f) {  // homogeneous: the optical-depth budget spent at constant density
        float enter, exit;
        if (!fog_slab_span(S, r, enter, exit)) return false;
        t = enter + u / S.fog_density;
        if (t < exit && t < end) {
            t_out = t;
            return true;
        }
        return false;
    }
    if (fabsf(hd) < 1e-6f) {
        float ds = fog_density_at(S, hs);
        if (ds <= 0.0f) return false;
        t = 0.0f + u / ds;
    } else {
        float rhs = sr_exp(-S.fog_falloff * hs) - u * S.fog_falloff * hd / S.fog_density;
        if (rhs <= 0.0f) return false;
        float yt = -sr_log(rhs) / S.fog_falloff;
        t = (yt - ho) / hd;
    }
    if (t < end) {
        t_out = t;
        return true;
    }
    return false;
}

// ---- BRDF (brdf.cs) ----------------------------------------------------------------------------------
SR_DEV Col base_reflectivity(float f0, Col albedo, float metallic) { return lerp(gray(f0), albedo, metallic); }
SR_DEV Col fresnel(float n_dot_v, Col base) {
    float x = 1.0f - n_dot_v;
    float x2 = x * x;
    float x5 = x2 * x2 * x;
    return base + (white() - base) * x5;
}
SR_DEV float ggx_d(float n_dot_h, float rs) {
    float a2 = rs * rs;
    float nh2 = n_dot_h * n_dot_h;
    float d = (1.0f - nh2) + nh2 * a2;
    return a2 / (kPi * d * d);
}
SR_DEV float smith_g1(float n_dot_x, float rs) {
    float k = rs / 2.0f;
    return n_dot_x / (n_dot_x * (1.0f - k) + k);
}
SR_DEV V3 ggx_sample_local(float rs, V2 u) {
    float ct = sqrtf((1.0f - u.x) / (u.x * (rs * rs - 1.0f) + 1.0f));
    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    float phi = (2.0f * kPi) * u.y;
    float sp, cp;
    sr_sincos(phi, &sp, &cp);
    return {st * cp, st * sp, ct};
}
SR_DEV float power_heuristic(float p1, float p2) {
    float a = p1 * p1;
    float b = p2 * p2;
    return a + b > 0.0f ? a / (a + b) : 0.0f;
}
SR_DEV float hg_pdf(float r_dot_l, float g) {
    float gs = g * g;
    float d = 1.0f + gs - 2.0f * g * r_dot_l;
    return (1.0f - gs) / ((4.0f * kPi) * d * sqrtf(d));
}
SR_DEV bool refract(V3 in, V3 n, float ratio, V3& out) {
    float ci = -dot(in, n);
    float s2t = ratio * ratio * (1.0f - ci * ci);
    if (s2t >= 1.0f) return false;
    float ctt = sqrtf(1.0f - s2t);
    out = ratio * in + (ratio * ci - ctt) * n;
    return true;
}
SR_DEV Col beer_law(Col a, float dist) {
    return {sr_pow(fmaxf(a.r, 0.0f), dist), sr_pow(fmaxf(a.g, 0.0f), dist), sr_pow(fmaxf(a.b, 0.0f), dist)};
}
SR_DEV V3 perp(V3 v) {
    V3 up = fabsf(v.y) < 0.9f ? up3() : right3();
    return normalize(cross(up, v));
}
SR_DEV V3 hg_scatter_dir(V3 fwd, float g, Rng& rng) {
    V2 u = rand_v2(rng);
    float ct;
    if (fabsf(g) < 1e-3f) {
        ct = 1.0f - 2.0f * u.x;
    } else {
        float s = (1.0f - g * g) / (1.0f - g + 2.0f * g * u.x);
        ct = (1.0f + g * g - s * s) / (2.0f * g);
    }
    ct = clampf(ct, -1.0f, 1.0f);
    float st = sqrtf(1.0f - ct * ct);
    float phi = (2.0f * kPi) * u.y;
    V3 t = perp(fwd);
    V3 b = cross(fwd, t);
    float sp, cp;
    sr_sincos(phi, &sp, &cp);
    return ct * fwd + (st * cp) * t + (st * sp) * b;
}
SR_DEV V3 from_tangent_space(V3 d, V4 tangent, V3 n) {
    V3 t = xyz(tangent);
    V3 b = tangent.w * cross(n, t);
    return d.x * t + d.y * b + d.z * n;
}
SR_DEV V3 reflect(V3 v, V3 n) { return v - (2.0f * dot(v, n)) * n; }

// ---- Surface (scene.cs:15-151) --------------------------------------------------------------------
struct Surface {
    Col radiance, albedo;
    float roughness, metallic, transparency, ior, f0;
    V3 normal, normal_geo;
    V4 tangent;
    V2 uv;
};
struct Scatter {
    V3 dir;
    Col weight;
    bool has_pdf;
    float pdf;
    bool refracted;
};

SR_DEV V3 clamp_to_geo_side(const Surface& s, V3 dir, V3 side) {
    float d = dot(dir, s.normal_geo);
    if (d * dot(side, s.normal_geo) < 0.0f) dir = normalize_or(dir - (2.0f * d) * s.normal_geo, side);
    return dir;
}
SR_DEV float specular_probability(const Surface& s, V3 view) {
    float ndv = fmaxf(1e-4f, dot(s.normal, view));
    float f = luminance(fresnel(ndv, base_reflectivity(s.f0, s.albedo, s.metallic)));
    return clampf(fmaxf(f, s.metallic), 0.001f, 0.999f);
}
// Surface.OpaqueEval / OpaquePdf are evaluated for the light sample and again for the scattered
// direction.  SR_NOINLINE_BRDF = 1 compiles one out-of-line copy each (smaller shading kernels);
// it stays off: with it the megakernel recorded wrong primary-hit depths in a transparent/fog
// scene on this toolchain (caught by the render-mode identity test), while the inlined build
// matches the oracle bit for bit.
#ifndef SR_NOINLINE_BRDF
#define SR_NOINLINE_BRDF 0
#endif
#if SR_NOINLINE_BRDF
#define SR_BRDF static __device__ __noinline__
#else
#define SR_BRDF SR_DEV
#endif
SR_BRDF Col opaque_eval(const Surface& s, V3 view, V3 light) {
    float ndl = dot(s.normal, light);
    if (ndl <= 0.0f) return black();
    float ndv = fmaxf(1e-4f, dot(s.normal, view));
    float rs = fmaxf(s.roughness * s.roughness, 1e-4f);
    Col base = base_reflectivity(s.f0, s.albedo, s.metallic);
    V3 half = normalize_or(view + light, s.normal);
    float ndh = dot(s.normal, half);
    float hdv = dot(half, view);
    Col f = fresnel(hdv, base);
    float g = smith_g1(ndv, rs) * smith_g1(ndl, rs);
    Col spec = ggx_d(ndh, rs) * f * g / (4.0f * ndv);
    Col diff = (white() - fresnel(ndv, base)) * s.albedo * (1.0f - s.metallic) * (ndl / kPi);
    return (spec + diff) * (1.0f - s.transparency);
}
SR_BRDF float opaque_pdf(const Surface& s, V3 view, V3 light, float spec_p) {
    float ndl = dot(s.normal, light);
    if (ndl <= 0.0f) return 0.0f;
    V3 half = normalize_or(view + light, s.normal);
    float ndh = fmaxf(0.0f, dot(s.normal, half));
    float hdv = fmaxf(1e-6f, dot(half, view));
    float rs = fmaxf(s.roughness * s.roughness, 1e-4f);
    float ps = ggx_d(ndh, rs) * ndh / (4.0f * hdv);
    float pd = ndl / kPi;
    return (spec_p * ps + (1.0f - spec_p) * pd) * (1.0f - s.transparency);
}
template <bool GENERAL = true>
SR_DEV Scatter surface_scatter(const Surface& s, V3 in, V3 view, Rng& rng) {
    if (rng_float(rng) < s.transparency && GENERAL) {
        // TransparentScatter scene.cs:119-144
        bool entering = dot(in, s.normal_geo) < 0.0f;
        V3 rn = entering ? s.normal_geo : -s.normal_geo;
        float ratio = entering ? 1.0f / s.ior : s.ior;
        float rs = fmaxf(s.roughness * s.roughness, 1e-4f);
        V3 half = from_tangent_space(ggx_sample_local(rs, rand_v2(rng)), s.tangent, s.normal);
        if (!entering) half = -half;
        if (dot(in, half) > 0.0f) half = rn;
        float hdv = fmaxf(1e-4f, dot(half, view));
        float f = luminance(fresnel(hdv, base_reflectivity(s.f0, s.albedo, s.metallic)));
        V3 rdir;
        if (rng_float(rng) >= f && refract(in, half, ratio, rdir))
            return {clamp_to_geo_side(s, rdir, -rn), white(), false, 0.0f, true};
        return {clamp_to_geo_side(s, reflect(in, half), rn), white(), false, 0.0f, false};
    }
    // OpaqueScatter scene.cs:103-117
    float spec_p = specular_probability(s, view);
    V3 dir;
    if (rng_float(rng) < spec_p) {
        float rs = fmaxf(s.roughness * s.roughness, 1e-4f);
        V3 hl = ggx_sample_local(rs, rand_v2(rng));
        V3 hw = from_tangent_space(hl, s.tangent, s.normal);
        dir = reflect(in, hw);
    } else {
        dir = normalize_or(s.normal + rand_on_sphere(rng), s.normal);
    }
    dir = clamp_to_geo_side(s, dir, s.normal_geo);
    float pdf = opaque_pdf(s, view, dir, spec_p);
    return {dir, opaque_eval(s, view, dir) / fmaxf(pdf, 1e-6f), true, pdf, false};
}

}  // namespace sr

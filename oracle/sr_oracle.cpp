// sr_oracle.cpp — CPU restatement of SharpRay's render hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests, the smoke check and the
// CPU-baseline leg of bench.py call it to check and time the GPU library.  Nothing in the
// product (sharpray_gb300/, include/) links or calls it.
//
// It restates, in scalar single-threaded-deterministic C++17, the C# reference path:
//   Rng                           math.cs:1665-1743
//   Vec/Color/Quat/Transform/Ray  math.cs:88-879
//   AABox / Sphere / triangles    math.cs:936-1579
//   Bvh build + traversal         bvh.cs:58-476
//   Mesh + ingest helpers         mesh.cs:4-123, math.cs:1491-1579, obj.cs:403-443
//   Texture / Cdf1 / Cdf2         texture.cs:39-75, cdf.cs:7-98
//   SkyTexture / SkyProcedural    scene.cs:281-435
//   Fog / Brdf / Surface          scene.cs:15-151,438-505, brdf.cs:12-122
//   Scene.Sample + helpers        scene.cs:576-810
//   Renderer.Render + scheduling  renderer.cs:107-237
//   Compositor                    compose.cs:57-266
//   AOV dumps, Overlay            program.cs:211-263, overlay.cs:54-196, math.cs:261,1638-1663
// in the reference's exact floating-point operation order: C# evaluates left to right, RyuJIT
// never contracts a*b+c into an FMA (this file must be compiled with -ffp-contract=off), and
// MathF.Min/Max follow IEEE 754:2019 minimum/maximum (NaN-propagating, -0 < +0), restated in
// net_min/net_max.  MathF transcendentals map to the C runtime's sinf/cosf/... as .NET does on
// Linux.  Parity against the C# binary itself is unpinned (no .NET runtime is available to run
// it); the restatement is pinned by published-algorithm known answers (splitmix64) and by the
// analytic checks in tests/.
#include "../include/sharpray.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <optional>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

constexpr float kPi = 3.14159265358979323846f;  // MathF.PI
constexpr float kFloatMax = std::numeric_limits<float>::max();
constexpr float kInf = std::numeric_limits<float>::infinity();

// ---- .NET MathF semantics ------------------------------------------------------------------
inline float net_max(float x, float y) {
    if (x != y) {
        if (!std::isnan(x)) return y < x ? x : y;
        return x;
    }
    return std::signbit(y) ? x : y;
}
inline float net_min(float x, float y) {
    if (x != y) {
        if (!std::isnan(x)) return x < y ? x : y;
        return x;
    }
    return std::signbit(x) ? x : y;
}
// Math.Clamp(float) / float.Clamp
inline float net_clamp(float v, float lo, float hi) {
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}

// ---- vectors (math.cs) ---------------------------------------------------------------------
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

inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator*(V2 v, float s) { return {v.x * s, v.y * s}; }

inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 v) { return {-v.x, -v.y, -v.z}; }
inline V3 operator*(V3 a, float b) { return {a.x * b, a.y * b, a.z * b}; }
inline V3 operator*(float a, V3 b) { return {a * b.x, a * b.y, a * b.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, float b) { return {a.x / b, a.y / b, a.z / b}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float comp(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float mag_sqr(V3 v) { return dot(v, v); }
inline float magnitude(V3 v) { return std::sqrt(mag_sqr(v)); }
inline V3 normalize(V3 v) { return v / magnitude(v); }
inline V3 normalize_or(V3 v, V3 fallback) {
    float m = mag_sqr(v);
    return m >= 1e-12f ? v / std::sqrt(m) : fallback;
}
const V3 kUp{0, 1, 0};
const V3 kRight{1, 0, 0};

inline V4 operator+(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline V4 operator*(V4 a, float b) { return {a.x * b, a.y * b, a.z * b, a.w * b}; }
inline V3 xyz(V4 v) { return {v.x, v.y, v.z}; }

inline Col operator+(Col a, Col b) { return {a.r + b.r, a.g + b.g, a.b + b.b}; }
inline Col operator-(Col a, Col b) { return {a.r - b.r, a.g - b.g, a.b - b.b}; }
inline Col operator*(Col a, Col b) { return {a.r * b.r, a.g * b.g, a.b * b.b}; }
inline Col operator*(Col c, float s) { return {c.r * s, c.g * s, c.b * s}; }
inline Col operator*(float s, Col c) { return {c.r * s, c.g * s, c.b * s}; }
inline Col operator/(Col c, float s) { return {c.r / s, c.g / s, c.b / s}; }
inline Col operator/(Col a, Col b) { return {a.r / b.r, a.g / b.g, a.b / b.b}; }
inline Col col(float v) { return {v, v, v}; }
const Col kBlack{0, 0, 0};
const Col kWhite{1, 1, 1};
inline float luminance(Col c) { return 0.2126f * c.r + 0.7152f * c.g + 0.0722f * c.b; }
inline float max_component(Col c) { return net_max(c.r, net_max(c.g, c.b)); }
inline Col clamp_luminance(Col c, float max) {
    float lum = luminance(c);
    return lum > max ? c * (max / lum) : c;
}
inline Col lerp(Col a, Col b, float t) {
    return {a.r + (b.r - a.r) * t, a.g + (b.g - a.g) * t, a.b + (b.b - a.b) * t};
}
inline Col bilerp(Col c1, Col c2, Col c3, Col c4, float tx, float ty) {
    return lerp(lerp(c1, c2, tx), lerp(c3, c4, tx), ty);
}
inline bool is_finite(Col c) { return std::isfinite(c.r) && std::isfinite(c.g) && std::isfinite(c.b); }

// ---- quaternion / transform (math.cs:551-879) ------------------------------------------------
struct Quat {
    float x, y, z, w;
};
inline Quat quat_inverse(Quat q) { return {-q.x, -q.y, -q.z, q.w}; }
inline V3 operator*(Quat q, V3 v) {
    V3 axis{q.x, q.y, q.z};
    float sqr = mag_sqr(axis);
    V3 a = axis * (dot(axis, v) * 2);
    V3 b = v * (q.w * q.w - sqr);
    V3 c = cross(axis, v) * (q.w * 2);
    return a + b + c;
}
inline Quat quat_angle_axis(float angle, V3 axis) {
    V3 v = axis * std::sin(angle * 0.5f);
    return {v.x, v.y, v.z, std::cos(angle * 0.5f)};
}
// Quat.FromMat4(Mat4.RotateLook(forward, upRef)) math.cs:641-665,736-751; columns c0,c1,c2.
inline Quat quat_look(V3 forward, V3 up_ref) {
    V3 c0{1, 0, 0}, c1{0, 1, 0}, c2{0, 0, 1};
    if (!(mag_sqr(forward) <= 1e-6f) && !(mag_sqr(up_ref) <= 1e-6f)) {
        V3 fwd = normalize(forward);
        V3 right = cross(up_ref, fwd);
        right = mag_sqr(right) > 1e-6f ? normalize(right) : V3{1, 0, 0};
        V3 up = cross(fwd, right);
        c0 = right;
        c1 = up;
        c2 = fwd;
    }
    float trace = c0.x + c1.y + c2.z;
    if (trace > 1e-6f) {
        float s = std::sqrt(trace + 1) * 2;
        return {(c1.z - c2.y) / s, (c2.x - c0.z) / s, (c0.y - c1.x) / s, s * 0.25f};
    }
    if (c0.x > c1.y && c0.x > c2.z) {
        float s = std::sqrt(1 + c0.x - c1.y - c2.z) * 2;
        return {s * 0.25f, (c1.x + c0.y) / s, (c2.x + c0.z) / s, (c1.z - c2.y) / s};
    }
    if (c1.y > c2.z) {
        float s = std::sqrt(1 + c1.y - c0.x - c2.z) * 2;
        return {(c1.x + c0.y) / s, s * 0.25f, (c2.y + c1.z) / s, (c2.x - c0.z) / s};
    }
    float s = std::sqrt(1 + c2.z - c0.x - c1.y) * 2;
    return {(c2.x + c0.z) / s, (c2.y + c1.z) / s, s * 0.25f, (c0.y - c1.x) / s};
}

struct Transform {
    V3 pos;
    Quat rot;
    V3 scale;
};
inline V3 transform_point(const Transform& t, V3 p) { return t.pos + t.rot * (p * t.scale); }

// ---- ray (math.cs:840-861) ------------------------------------------------------------------
struct Ray {
    V3 origin, dir, dir_inv;
};
inline float safe_comp(float d) {
    const float min_comp = 1e-8f;
    return std::fabs(d) >= min_comp ? d : std::copysign(min_comp, d);
}
inline Ray make_ray(V3 origin, V3 dir) {
    Ray r;
    r.origin = origin;
    r.dir = dir;
    r.dir_inv = {1.0f / safe_comp(dir.x), 1.0f / safe_comp(dir.y), 1.0f / safe_comp(dir.z)};
    return r;
}
inline V3 ray_at(const Ray& r, float t) { return r.origin + r.dir * t; }

// Transform.TransformRayInv math.cs:816-822.
inline Ray transform_ray_inv(const Transform& t, const Ray& ray, float* out_scale) {
    Quat inv = quat_inverse(t.rot);
    V3 origin = (inv * (ray.origin - t.pos)) / t.scale;
    V3 dir_raw = (inv * ray.dir) / t.scale;
    float scale = magnitude(dir_raw);
    *out_scale = scale;
    return make_ray(origin, dir_raw / scale);
}

// ---- RNG (math.cs:1665-1743) ---------------------------------------------------------------
uint64_t split_mix64(uint64_t& state) {
    uint64_t result = state += 0x9e3779b97f4a7c15ULL;
    result = (result ^ (result >> 30)) * 0xbf58476d1ce4e5b9ULL;
    result = (result ^ (result >> 27)) * 0x94d049bb133111ebULL;
    return result ^ (result >> 31);
}

struct Rng {
    uint32_t s0, s1, s2, s3, s4;
    Rng(uint32_t seed_a, uint32_t seed_b) {
        uint64_t seed = ((uint64_t)seed_a << 32) | seed_b;
        uint64_t v1 = split_mix64(seed);
        uint64_t v2 = split_mix64(seed);
        s0 = (uint32_t)v1;
        s1 = (uint32_t)(v1 >> 32);
        s2 = (uint32_t)v2;
        s3 = (uint32_t)(v2 >> 32);
        s4 = 0;
    }
    uint32_t next_uint() {
        uint32_t t = s3;
        uint32_t s = s0;
        s3 = s2;
        s2 = s1;
        s1 = s;
        t ^= t >> 2;
        t ^= t << 1;
        t ^= s ^ (s << 4);
        s0 = t;
        s4 += 362437u;
        return t + s4;
    }
    float next_float() {
        const float to_float = 1.0f / (4294967296.0f + 512.0f);
        return (float)next_uint() * to_float;
    }
    float next_exponential() {
        float u;
        do {
            u = next_float();
        } while (u <= 1e-8f);
        return -std::log(u);
    }
    void next_gauss(float* a_out, float* b_out) {
        float a;
        do {
            a = next_float();
        } while (a <= 1e-8f);
        float b = (kPi * 2.0f) * next_float();
        float mag = std::sqrt(-2.0f * std::log(a));
        *a_out = mag * std::cos(b);
        *b_out = mag * std::sin(b);
    }
};

inline V2 rand_v2(Rng& rng) {
    float x = rng.next_float();
    float y = rng.next_float();
    return {x, y};
}
inline V3 rand_on_sphere(Rng& rng) {
    while (true) {
        float x, y, z, unused;
        rng.next_gauss(&x, &y);
        rng.next_gauss(&z, &unused);
        float m = x * x + y * y + z * z;
        if (m > 1e-6f) return V3{x, y, z} / std::sqrt(m);
    }
}

// ---- counters ---------------------------------------------------------------------------------
struct Counters {
    uint64_t v[SR_COUNTER_COUNT] = {};
    void add(int i, uint64_t n = 1) { v[i] += n; }
};

// ---- AABox (math.cs:936-1070) ---------------------------------------------------------------
struct AABox {
    V3 min, max;
};
inline AABox aabox_inverted() { return {{kFloatMax, kFloatMax, kFloatMax}, {-kFloatMax, -kFloatMax, -kFloatMax}}; }
inline V3 box_center(const AABox& b) { return (b.min + b.max) * 0.5f; }
inline V3 box_size(const AABox& b) { return b.max - b.min; }
inline float surface_area(const AABox& b) {
    V3 s = box_size(b);
    return 2.0f * (s.x * s.y + s.x * s.z + s.y * s.z);
}
inline bool is_inverted(const AABox& b) { return b.min.x > b.max.x || b.min.y > b.max.y || b.min.z > b.max.z; }
inline void encapsulate(AABox& b, V3 p) {
    b.min = {net_min(b.min.x, p.x), net_min(b.min.y, p.y), net_min(b.min.z, p.z)};
    b.max = {net_max(b.max.x, p.x), net_max(b.max.y, p.y), net_max(b.max.z, p.z)};
}
inline void encapsulate(AABox& b, const AABox& o) {
    b.min = {net_min(b.min.x, o.min.x), net_min(b.min.y, o.min.y), net_min(b.min.z, o.min.z)};
    b.max = {net_max(b.max.x, o.max.x), net_max(b.max.y, o.max.y), net_max(b.max.z, o.max.z)};
}
inline AABox from_center(V3 c, V3 size) { return {c - size * 0.5f, c + size * 0.5f}; }

// AABox.IntersectDist math.cs:983-1004; returns false for "null".
inline bool box_intersect_dist(const AABox& b, const Ray& ray, float* t_out) {
    float t1 = (b.min.x - ray.origin.x) * ray.dir_inv.x;
    float t2 = (b.max.x - ray.origin.x) * ray.dir_inv.x;
    float t3 = (b.min.y - ray.origin.y) * ray.dir_inv.y;
    float t4 = (b.max.y - ray.origin.y) * ray.dir_inv.y;
    float t5 = (b.min.z - ray.origin.z) * ray.dir_inv.z;
    float t6 = (b.max.z - ray.origin.z) * ray.dir_inv.z;
    float min_a = net_min(t1, t2), min_b = net_min(t3, t4), min_c = net_min(t5, t6);
    float max_a = net_max(t1, t2), max_b = net_max(t3, t4), max_c = net_max(t5, t6);
    float t_min = net_max(net_max(min_a, min_b), min_c);
    float t_max = net_min(net_min(max_a, max_b), max_c);
    if (t_max < 0.0f || t_min > t_max) return false;
    *t_out = net_max(0.0f, t_min);
    return true;
}

// ---- shape hits --------------------------------------------------------------------------------
struct ShapeHit {
    float dist;
    V3 norm, norm_geo;
    V4 tan;
    V2 uv;
};

// AABox.Intersect math.cs:1006-1059 (analytic box shape).
bool aabox_intersect(const AABox& b, const Ray& ray, ShapeHit* out) {
    float t1 = (b.min.x - ray.origin.x) * ray.dir_inv.x;
    float t2 = (b.max.x - ray.origin.x) * ray.dir_inv.x;
    float t3 = (b.min.y - ray.origin.y) * ray.dir_inv.y;
    float t4 = (b.max.y - ray.origin.y) * ray.dir_inv.y;
    float t5 = (b.min.z - ray.origin.z) * ray.dir_inv.z;
    float t6 = (b.max.z - ray.origin.z) * ray.dir_inv.z;
    float min_a = net_min(t1, t2), min_b = net_min(t3, t4), min_c = net_min(t5, t6);
    float max_a = net_max(t1, t2), max_b = net_max(t3, t4), max_c = net_max(t5, t6);
    float t_min = net_max(net_max(min_a, min_b), min_c);
    float t_max = net_min(net_min(max_a, max_b), max_c);
    if (t_max < 0.0f || t_min > t_max) return false;
    bool inside = t_min < 0.0f;
    float t = inside ? t_max : t_min;
    V3 hit = ray_at(ray, t);
    V3 norm;
    V4 tan;
    V2 face;
    if (min_a >= min_b && min_a >= min_c) {
        bool neg = t1 <= t2;
        norm = neg ? V3{-1, 0, 0} : V3{1, 0, 0};
        tan = {0, 1, 0, neg ? -1.0f : 1.0f};
        face = {(hit.y - b.min.y) / (b.max.y - b.min.y), (hit.z - b.min.z) / (b.max.z - b.min.z)};
    } else if (min_b >= min_a && min_b >= min_c) {
        bool neg = t3 <= t4;
        norm = neg ? V3{0, -1, 0} : V3{0, 1, 0};
        tan = {1, 0, 0, neg ? 1.0f : -1.0f};
        face = {(hit.x - b.min.x) / (b.max.x - b.min.x), (hit.z - b.min.z) / (b.max.z - b.min.z)};
    } else {
        bool neg = t5 <= t6;
        norm = neg ? V3{0, 0, -1} : V3{0, 0, 1};
        tan = {1, 0, 0, neg ? -1.0f : 1.0f};
        face = {(hit.x - b.min.x) / (b.max.x - b.min.x), (hit.y - b.min.y) / (b.max.y - b.min.y)};
    }
    V3 n = inside ? -norm : norm;
    *out = {t, n, n, tan, face};
    return true;
}

// Sphere.Intersect math.cs:1210-1234.
struct SphereShape {
    V3 center;
    float radius;
};
bool sphere_intersect(const SphereShape& s, const Ray& ray, ShapeHit* out) {
    V3 to_center = s.center - ray.origin;
    float dist_sqr = mag_sqr(to_center);
    float a = dot(to_center, ray.dir);
    float disc = s.radius * s.radius - dist_sqr + a * a;
    if (disc < 0.0f) return false;
    float f = std::sqrt(disc);
    float t = dist_sqr < s.radius * s.radius ? a + f : a - f;
    if (t < 0.0f) return false;
    V3 norm = normalize(ray_at(ray, t) - s.center);
    V4 tan{0, 0, 0, 1};
    V3 txyz = normalize_or(V3{-norm.z, 0.0f, norm.x}, kRight);
    tan = {txyz.x, txyz.y, txyz.z, 1.0f};
    float tex_u = 0.5f + std::atan2(norm.z, norm.x) / (2.0f * kPi);
    float tex_v = 0.5f - std::asin(net_clamp(norm.y, -1.0f, 1.0f)) / kPi;
    *out = {t, norm, norm, tan, {tex_u, tex_v}};
    return true;
}

// ---- triangles (math.cs:1336-1579) ---------------------------------------------------------
struct TriLean {
    V3 a, ab, ac;
    V3 pos_b() const { return a + ab; }
    V3 pos_c() const { return a + ac; }
    V3 normal() const { return normalize_or(cross(ab, ac), kUp); }
    AABox bounds() const {
        V3 b = pos_b(), c = pos_c();
        return {{net_min(a.x, net_min(b.x, c.x)), net_min(a.y, net_min(b.y, c.y)), net_min(a.z, net_min(b.z, c.z))},
                {net_max(a.x, net_max(b.x, c.x)), net_max(a.y, net_max(b.y, c.y)), net_max(a.z, net_max(b.z, c.z))}};
    }
};
inline TriLean make_lean(V3 a, V3 b, V3 c) { return {a, b - a, c - a}; }

// TriangleLean.Intersect (Moller-Trumbore) math.cs:1407-1435.
inline bool tri_intersect(const TriLean& tri, const Ray& ray, float* t_out, float* u_out, float* v_out) {
    V3 h = cross(ray.dir, tri.ac);
    float det = dot(tri.ab, h);
    if (std::fabs(det) <= 1e-7f) return false;
    float inv_det = 1.0f / det;
    const float edge_eps = 1e-7f;
    V3 ao = ray.origin - tri.a;
    float u = dot(ao, h) * inv_det;
    if (u < -edge_eps || u > (1.0f + edge_eps)) return false;
    V3 q = cross(ao, tri.ab);
    float v = dot(ray.dir, q) * inv_det;
    if (v < -edge_eps || (u + v) > (1.0f + edge_eps)) return false;
    float t = dot(tri.ac, q) * inv_det;
    if (t < 0.0f) return false;
    *t_out = t;
    *u_out = u;
    *v_out = v;
    return true;
}

struct TriAttr {
    V3 na, nb, nc;
    V4 ta, tb, tc;
    V2 uva, uvb, uvc;
};

// TriangleLean.Inflate math.cs:1437-1459.
ShapeHit tri_inflate(const TriLean& tri, const TriAttr& at, float dist, float u, float v) {
    float w = 1.0f - u - v;
    V3 n_interp = at.na * w + at.nb * u + at.nc * v;
    V3 norm = mag_sqr(n_interp) >= 1e-12f ? normalize(n_interp) : tri.normal();
    V3 norm_face = tri.normal();
    V4 t_interp = at.ta * w + at.tb * u + at.tc * v;
    V3 txyz = xyz(t_interp);
    V3 tan_xyz = normalize_or(txyz - dot(txyz, norm) * norm, kRight);
    V4 tan{tan_xyz.x, tan_xyz.y, tan_xyz.z, t_interp.w >= 0.0f ? 1.0f : -1.0f};
    V2 uv = at.uva * w + at.uvb * u + at.uvc * v;
    return {dist, norm, norm_face, tan, uv};
}

// Triangle.ComputeTangent math.cs:1553-1579.
V4 compute_tangent(V3 pa, V3 pb, V3 pc, V2 uva, V2 uvb, V2 uvc, V3 norm) {
    V3 pd1 = pb - pa;
    V3 pd2 = pc - pa;
    V2 ud1{uvb.x - uva.x, uvb.y - uva.y};
    V2 ud2{uvc.x - uva.x, uvc.y - uva.y};
    float f = ud1.x * ud2.y - ud2.x * ud1.y;
    if (std::fabs(f) < 1e-8f) {
        V3 t = normalize_or(pd1 - dot(pd1, norm) * norm, kRight);
        return {t.x, t.y, t.z, 1.0f};
    }
    float inv_f = 1.0f / f;
    V3 tangent = (ud2.y * pd1 - ud1.y * pd2) * inv_f;
    V3 bitangent = (-ud2.x * pd1 + ud1.x * pd2) * inv_f;
    tangent = normalize_or(tangent - dot(tangent, norm) * norm, kRight);
    float w = dot(cross(norm, tangent), bitangent) < 0.0f ? -1.0f : 1.0f;
    return {tangent.x, tangent.y, tangent.z, w};
}

// Full Triangle (lean + attributes) as the C# struct holds it.
struct Triangle {
    TriLean lean;
    TriAttr attr;
};
// Triangle(posA, posB, posC, uvA, uvB, uvC) math.cs:1510-1517.
Triangle make_triangle_uv(V3 pa, V3 pb, V3 pc, V2 uva, V2 uvb, V2 uvc) {
    Triangle t;
    t.lean = make_lean(pa, pb, pc);
    V3 n = t.lean.normal();
    t.attr.na = t.attr.nb = t.attr.nc = n;
    V4 tan = compute_tangent(pa, pb, pc, uva, uvb, uvc, n);
    t.attr.ta = t.attr.tb = t.attr.tc = tan;
    t.attr.uva = uva;
    t.attr.uvb = uvb;
    t.attr.uvc = uvc;
    return t;
}
// Triangle(posA, posB, posC, normA, normB, normC, uvA, uvB, uvC) math.cs:1519-1531.
Triangle make_triangle_full(V3 pa, V3 pb, V3 pc, V3 na, V3 nb, V3 nc, V2 uva, V2 uvb, V2 uvc) {
    Triangle t;
    t.lean = make_lean(pa, pb, pc);
    t.attr.na = na;
    t.attr.nb = nb;
    t.attr.nc = nc;
    t.attr.uva = uva;
    t.attr.uvb = uvb;
    t.attr.uvc = uvc;
    V3 geo = normalize_or(cross(pb - pa, pc - pa), kUp);
    V3 avg = normalize_or((na + nb + nc) / 3.0f, geo);
    V4 tan = compute_tangent(pa, pb, pc, uva, uvb, uvc, avg);
    t.attr.ta = t.attr.tb = t.attr.tc = tan;
    return t;
}

// Mesh.ComputeSmoothNormals mesh.cs:99-123 with Vec3Comparer(1e-6) math.cs:396-403.
struct QKey {
    int64_t x, y, z;
    bool operator==(const QKey& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct QKeyHash {
    size_t operator()(const QKey& k) const {
        uint64_t h = (uint64_t)k.x * 0x9E3779B97F4A7C15ULL;
        h ^= (uint64_t)k.y + 0x7F4A7C159E3779B9ULL + (h << 6) + (h >> 2);
        h ^= (uint64_t)k.z + 0x94D049BB133111EBULL + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};
void compute_smooth_normals(std::vector<Triangle>& tris) {
    const float inv_eps = 1.0f / 1e-6f;
    auto quant = [&](float v) { return (int64_t)std::nearbyint(v * inv_eps); };
    auto key = [&](V3 p) { return QKey{quant(p.x), quant(p.y), quant(p.z)}; };
    std::unordered_map<QKey, V3, QKeyHash> accum;
    accum.reserve(tris.size() * 2);
    for (const Triangle& t : tris) {
        V3 c = cross(t.lean.ab, t.lean.ac);
        float area = magnitude(c) * 0.5f;
        V3 nw = t.lean.normal() * area;
        V3 p[3] = {t.lean.a, t.lean.pos_b(), t.lean.pos_c()};
        for (int k = 0; k < 3; ++k) {
            auto it = accum.find(key(p[k]));
            if (it == accum.end())
                accum.emplace(key(p[k]), V3{0, 0, 0} + nw);
            else
                it->second = it->second + nw;
        }
    }
    for (Triangle& t : tris) {
        V3 pa = t.lean.a, pb = t.lean.pos_b(), pc = t.lean.pos_c();
        V3 face = t.lean.normal();
        V3 na = normalize_or(accum[key(pa)], face);
        V3 nb = normalize_or(accum[key(pb)], face);
        V3 nc = normalize_or(accum[key(pc)], face);
        t = make_triangle_full(pa, pb, pc, na, nb, nc, t.attr.uva, t.attr.uvb, t.attr.uvc);
    }
}

// ---- BVH (bvh.cs) ------------------------------------------------------------------------------
struct BvhNode {
    AABox bounds;
    int32_t child;
    int32_t count;
};

// Binned-SAH BVH restated from bvh.cs:58-476.  `BoundsOf(i)` returns shape i's AABox.
template <typename BoundsFn>
struct BvhBuilder {
    int bins;
    float cost_traverse, cost_intersect;
    int shape_count;
    BoundsFn bounds_of;
    std::vector<BvhNode> nodes;
    std::vector<int32_t> items;
    int node_count = 0;

    BvhBuilder(int n, BoundsFn fn, float ct, float ci, int nb)
        : bins(nb), cost_traverse(ct), cost_intersect(ci), shape_count(n), bounds_of(fn) {
        nodes.assign(std::max(n * 2, 1), BvhNode{{{0, 0, 0}, {0, 0, 0}}, 0, 0});
        items.resize(n);
        for (int i = 0; i < n; ++i) items[i] = i;
        if (n > 0) subdivide(insert_root(), 0);
    }
    float sah_leaf(float sa, int count) const { return cost_intersect * sa * (float)count; }
    float sah_split(float psa, float lsa, int lc, float rsa, int rc) const {
        return cost_traverse * psa + sah_leaf(lsa, lc) + sah_leaf(rsa, rc);
    }
    int insert_root() {
        int idx = node_count++;
        BvhNode& n = nodes[idx];
        n.bounds = aabox_inverted();
        n.child = 0;
        n.count = shape_count;
        for (int i = 0; i < shape_count; ++i) encapsulate(n.bounds, bounds_of(items[i]));
        return idx;
    }
    int insert(int begin, int count) {
        int idx = node_count++;
        BvhNode& n = nodes[idx];
        n.bounds = aabox_inverted();
        n.child = begin;
        n.count = count;
        for (int i = 0; i < count; ++i) encapsulate(n.bounds, bounds_of(items[begin + i]));
        return idx;
    }
    AABox centroid_bounds(int begin, int count) const {
        AABox b = aabox_inverted();
        for (int i = 0; i < count; ++i) encapsulate(b, box_center(bounds_of(items[begin + i])));
        return b;
    }
    bool split_pick(int node_idx, int* axis_out, float* pos_out) {
        const BvhNode& node = nodes[node_idx];
        int begin = node.child, count = node.count;
        AABox cb = centroid_bounds(begin, count);
        float parent_sa = surface_area(node.bounds);
        float best_cost = sah_leaf(parent_sa, count);
        int best_axis = -1;
        float best_pos = 0.0f;
        std::vector<AABox> bin_bounds(bins);
        std::vector<int> bin_count(bins);
        std::vector<float> left_sa(bins - 1);
        std::vector<int> left_count(bins - 1);
        for (int axis = 0; axis != 3; ++axis) {
            float cmin = comp(cb.min, axis), cmax = comp(cb.max, axis);
            if (cmax - cmin < 1e-6f) continue;
            for (int b = 0; b != bins; ++b) {
                bin_bounds[b] = aabox_inverted();
                bin_count[b] = 0;
            }
            float scale = (float)bins / (cmax - cmin);
            for (int i = 0; i != count; ++i) {
                AABox sb = bounds_of(items[begin + i]);
                int bin = std::min((int)((comp(box_center(sb), axis) - cmin) * scale), bins - 1);
                encapsulate(bin_bounds[bin], sb);
                ++bin_count[bin];
            }
            AABox lb = aabox_inverted();
            int lc = 0;
            for (int b = 0; b != bins - 1; ++b) {
                encapsulate(lb, bin_bounds[b]);
                lc += bin_count[b];
                left_sa[b] = is_inverted(lb) ? 0.0f : surface_area(lb);
                left_count[b] = lc;
            }
            AABox rb = aabox_inverted();
            int rc = 0;
            for (int b = bins - 1; b != 0; --b) {
                encapsulate(rb, bin_bounds[b]);
                rc += bin_count[b];
                float rsa = is_inverted(rb) ? 0.0f : surface_area(rb);
                float cost = sah_split(parent_sa, left_sa[b - 1], left_count[b - 1], rsa, rc);
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_pos = cmin + (float)b * (cmax - cmin) / (float)bins;
                }
            }
        }
        if (best_axis < 0) return false;
        *axis_out = best_axis;
        *pos_out = best_pos;
        return true;
    }
    int partition(int node_idx, int axis, float split_pos) {
        BvhNode& node = nodes[node_idx];
        int left = node.child;
        int right = node.child + node.count - 1;
        while (true) {
            AABox lb = bounds_of(items[left]);
            float center = (comp(lb.min, axis) + comp(lb.max, axis)) * 0.5f;
            if (center < split_pos) {
                ++left;
                if (left > right) break;
            } else {
                if (left == right) break;
                std::swap(items[left], items[right]);
                --right;
            }
        }
        return left;
    }
    void subdivide(int node_idx, int depth) {
        if (depth >= 64) return;
        int axis;
        float pos;
        if (!split_pick(node_idx, &axis, &pos)) return;
        int p = partition(node_idx, axis, pos);
        int count_a = p - nodes[node_idx].child;
        int count_b = nodes[node_idx].count - count_a;
        int child_a = insert(nodes[node_idx].child, count_a);
        int child_b = insert(p, count_b);
        (void)child_b;
        nodes[node_idx].child = child_a;
        nodes[node_idx].count = 0;
        subdivide(child_a, depth + 1);
        subdivide(child_a + 1, depth + 1);
    }
};

// Bvh.Intersect bvh.cs:165-216.  LeafFn(shape_index, best_dist) returns true + dist when the
// shape is hit (the shape's own hit record is kept by the callback).
template <typename LeafFn>
bool bvh_intersect(const std::vector<BvhNode>& nodes, int node_count, const std::vector<int32_t>& items,
                   const Ray& ray, LeafFn leaf, int* best_idx, Counters* ctr, int ctr_node, int ctr_shape) {
    if (node_count == 0) return false;
    struct Entry {
        int idx;
        float t;
    };
    Entry queue[128];
    int qc = 1;
    queue[0] = {0, 0.0f};
    bool found = false;
    float best = kInf;
    while (qc > 0) {
        Entry e = queue[--qc];
        if (e.t >= best) continue;
        const BvhNode& node = nodes[e.idx];
        if (node.count == 0) {
            if (ctr) ctr->add(ctr_node, 2);
            float ta = 0, tb = 0;
            bool ha = box_intersect_dist(nodes[node.child].bounds, ray, &ta);
            bool hb = box_intersect_dist(nodes[node.child + 1].bounds, ray, &tb);
            bool pa = ha && ta <= best, pb = hb && tb <= best;
            if (pa) queue[qc++] = {node.child, ta};
            if (pb) queue[qc++] = {node.child + 1, tb};
            if (pa && pb && ta < tb) std::swap(queue[qc - 2], queue[qc - 1]);
        } else {
            if (ctr) ctr->add(ctr_shape, (uint64_t)node.count);
            for (int i = 0; i != node.count; ++i) {
                int idx = items[node.child + i];
                float d;
                if (leaf(idx, &d) && d < best) {
                    best = d;
                    *best_idx = idx;
                    found = true;
                }
            }
        }
    }
    return found;
}

// ---- Texture (texture.cs) ------------------------------------------------------------------
struct Texture {
    uint32_t width = 0, height = 0;
    int filter = 0;  // 0 bilinear, 1 point
    V2 tiling{1, 1};
    std::vector<Col> texels;
    Col get(int x, int y) const { return texels[(uint32_t)y * width + (uint32_t)x]; }
    Col sample(V2 coord, Counters* ctr) const {
        if (ctr) ctr->add(SR_COUNTER_TEX_SAMPLE);
        float u = coord.x * tiling.x;
        u -= std::floor(u);
        float v = coord.y * tiling.y;
        v -= std::floor(v);
        if (filter == 1) {
            uint32_t x = (uint32_t)(u * (float)width) % width;
            uint32_t y = (uint32_t)(v * (float)height) % height;
            return texels[y * width + x];
        }
        float fx = u * (float)(width - 1);
        float fy = v * (float)(height - 1);
        uint32_t x0 = (uint32_t)fx;
        uint32_t y0 = (uint32_t)fy;
        uint32_t x1 = (x0 + 1) % width;
        uint32_t y1 = (y0 + 1) % height;
        float tx = fx - (float)x0;
        float ty = fy - (float)y0;
        return bilerp(texels[y0 * width + x0], texels[y0 * width + x1], texels[y1 * width + x0],
                      texels[y1 * width + x1], tx, ty);
    }
    V3 sample_normal(V2 coord, Counters* ctr) const {
        Col c = sample(coord, ctr);
        return normalize_or(V3{c.r * 2.0f - 1.0f, -(c.g * 2.0f - 1.0f), c.b * 2.0f - 1.0f}, kUp);
    }
};

// ---- CDF (cdf.cs) ---------------------------------------------------------------------------
struct Cdf1 {
    std::vector<float> cdf;  // n + 1
    float total = 0;
    void init(const float* w, int n) {
        cdf.assign(n + 1, 0.0f);
        cdf[0] = 0.0f;
        for (int i = 0; i != n; ++i) cdf[i + 1] = cdf[i] + w[i];
        total = cdf[n];
        if (total > 0.0f)
            for (int i = 1; i != n + 1; ++i) cdf[i] /= total;
    }
    uint32_t count() const { return (uint32_t)cdf.size() - 1; }
    uint32_t sample(float norm, Counters* ctr) const {
        uint32_t lo = 0, hi = count();
        while (lo < hi) {
            if (ctr) ctr->add(SR_COUNTER_CDF_PROBE);
            uint32_t mid = (lo + hi) >> 1;
            if (cdf[mid + 1] <= norm)
                lo = mid + 1;
            else
                hi = mid;
        }
        return std::min(lo, count() - 1);
    }
};
struct Cdf2 {
    Cdf1 marginal;
    std::vector<Cdf1> conditionals;
};

// ---- Sky ------------------------------------------------------------------------------------
struct SampleLight {
    V3 dir;
    float pdf;
};

// V3.EquirectUv math.cs:390-398; V3.FromEquirectUv math.cs:493-500.
inline V2 equirect_uv(V3 d) {
    float u = std::atan2(d.z, d.x) / (kPi * 2.0f) + 0.5f;
    float v = 0.5f - std::asin(net_clamp(d.y, -1.0f, 1.0f)) / kPi;
    return {u, v};
}
inline V3 from_equirect_uv(V2 uv) {
    float phi = (uv.x - 0.5f) * 2.0f * kPi;
    float sin_theta = std::sin(kPi * uv.y);
    float y = std::cos(kPi * uv.y);
    return {sin_theta * std::cos(phi), y, sin_theta * std::sin(phi)};
}

struct Sky {
    int kind = -1;  // 0 texture, 1 procedural
    // SkyTexture scene.cs:379-435
    const Texture* tex = nullptr;
    Cdf2 cdf;
    float pdf_scale = 0, multiplier = 1;
    Quat rot{0, 0, 0, 1}, rot_inv{0, 0, 0, 1};
    // SkyProcedural + SunProcedural scene.cs:281-377
    Col top, middle, bottom;
    V3 sun_dir;
    Col sun_radiance;
    float sun_angle_cos = 1, sun_pdf_denom = 0;
    Quat sun_rot{0, 0, 0, 1};

    void init_texture(const Texture* t, float mult, float rot_yaw) {
        kind = 0;
        tex = t;
        int w = (int)t->width, h = (int)t->height;
        std::vector<float> row_w(h), col_w(w);
        cdf.conditionals.resize(h);
        for (int y = 0; y != h; ++y) {
            for (int x = 0; x != w; ++x)
                col_w[x] = luminance(t->get(x, y)) * std::sin(kPi * ((float)y + 0.5f) / (float)h);
            cdf.conditionals[y].init(col_w.data(), w);
            row_w[y] = cdf.conditionals[y].total;
        }
        cdf.marginal.init(row_w.data(), h);
        pdf_scale = (float)(w * h) / (cdf.marginal.total * 2.0f * kPi * kPi);
        multiplier = mult;
        rot = quat_angle_axis(rot_yaw, kUp);
        rot_inv = quat_inverse(rot);
    }
    void init_procedural(const SrSkyProcedural& p) {
        kind = 1;
        top = {p.top[0], p.top[1], p.top[2]};
        middle = {p.middle[0], p.middle[1], p.middle[2]};
        bottom = {p.bottom[0], p.bottom[1], p.bottom[2]};
        sun_dir = {p.sun_dir[0], p.sun_dir[1], p.sun_dir[2]};
        sun_radiance = {p.sun_radiance[0], p.sun_radiance[1], p.sun_radiance[2]};
        sun_angle_cos = std::cos(p.sun_angle);
        sun_rot = quat_look(sun_dir, kUp);
        sun_pdf_denom = kPi * (1.0f - sun_angle_cos);
    }
    Col radiance(V3 dir, Counters* ctr) const {
        if (kind == 0) {
            if (ctr) ctr->add(SR_COUNTER_ENV_LOOKUP);
            return tex->sample(equirect_uv(rot_inv * dir), nullptr) * multiplier;
        }
        const float bias = 0.0001f;
        float top_b = 1.0f - std::pow(net_min(1.0f, 1.0f + bias - dir.y), 4.0f);
        float bot_b = 1.0f - std::pow(net_min(1.0f, 1.0f + bias + dir.y), 40.0f);
        float mid_b = 1.0f - top_b - bot_b;
        Col ambient = top * top_b + middle * mid_b + bottom * bot_b;
        float blend = net_max(0.0f, (dot(dir, sun_dir) - sun_angle_cos) / (1.0f - sun_angle_cos));
        return ambient + sun_radiance * blend;
    }
    std::optional<SampleLight> light_dir(V3 dir) const {
        if (kind == 0) {
            if (cdf.marginal.total <= 0.0f) return std::nullopt;
            V2 uv = equirect_uv(rot_inv * dir);
            int cx = (int)(uv.x * (float)tex->width) % (int)tex->width;
            int cy = (int)(uv.y * (float)tex->height) % (int)tex->height;
            float pdf = luminance(tex->get(cx, cy)) * pdf_scale;
            if (pdf > 0.0f) return SampleLight{dir, pdf};
            return std::nullopt;
        }
        float cos_theta = dot(dir, sun_dir);
        if (cos_theta < sun_angle_cos) return std::nullopt;
        float blend = (cos_theta - sun_angle_cos) / (1.0f - sun_angle_cos);
        return SampleLight{dir, blend / sun_pdf_denom};
    }
    std::optional<SampleLight> light_dir_rand(Rng& rng, Counters* ctr) const {
        if (kind == 0) {
            if (cdf.marginal.total <= 0.0f) return std::nullopt;
            if (ctr) ctr->add(SR_COUNTER_LIGHT_SAMPLE);
            V2 c = rand_v2(rng);
            int y = (int)cdf.marginal.sample(c.y, ctr);
            int x = (int)cdf.conditionals[y].sample(c.x, ctr);
            V2 uv{((float)x + 0.5f) / (float)tex->width, ((float)y + 0.5f) / (float)tex->height};
            V3 dir = rot * from_equirect_uv(uv);
            float pdf = luminance(tex->get(x, y)) * pdf_scale;
            if (pdf > 0.0f) return SampleLight{dir, pdf};
            return std::nullopt;
        }
        float phi = (kPi * 2.0f) * rng.next_float();
        float blend = std::sqrt(rng.next_float());
        float z = sun_angle_cos + (1.0f - sun_angle_cos) * blend;
        float sin_t = std::sqrt(net_max(0.0f, 1.0f - z * z));
        V3 dir = sun_rot * V3{std::cos(phi) * sin_t, std::sin(phi) * sin_t, z};
        return SampleLight{dir, blend / sun_pdf_denom};
    }
};

// ---- Fog (scene.cs:438-505) -----------------------------------------------------------------
struct Fog {
    float density;
    Col color;
    float anisotropy;
    float height_falloff;
    float top_height;  // the homogeneous extension (height_falloff 0): the medium's top
    float density_at(float y) const { return density * std::exp(-height_falloff * y); }
    // Homogeneous fog (height_falloff 0; an extension, no counterpart in the reference, whose
    // formulas divide by the falloff): the part [enter, exit) of the ray below the top height.
    bool slab_span(const Ray& ray, float* enter, float* exit) const {
        const float hd = ray.dir.y, ho = ray.origin.y;
        *enter = 0.0f;
        *exit = kInf;
        if (hd == 0.0f) return ho < top_height;
        const float tc = (top_height - ho) / hd;
        if (hd > 0.0f) {
            *exit = tc;
            return tc > 0.0f;
        }
        *enter = net_max(0.0f, tc);
        return true;
    }
    float optical_depth(const Ray& ray, float start, float end) const {
        if (height_falloff == 0.0f) {  // density x the length of [start, end] below the top
            float enter, exit;
            if (!slab_span(ray, &enter, &exit)) return 0.0f;
            const float a = net_max(start, enter), b = net_min(end, exit);
            return b > a ? density * (b - a) : 0.0f;
        }
        float hd = ray.dir.y;
        float hs = ray.origin.y + start * hd;
        float he = ray.origin.y + end * hd;
        float ds = density_at(hs);
        float de = density_at(he);
        if (std::fabs(hd) < 1e-6f) return ds * (end - start);
        return (ds - de) / (height_falloff * hd);
    }
    float transmittance(const Ray& ray, float start, float end) const { return std::exp(-optical_depth(ray, start, end)); }
    bool scatter_distance(const Ray& ray, float start, float end, Rng& rng, float* t_out) const {
        float hd = ray.dir.y;
        float ho = ray.origin.y;
        float hs = ho + start * hd;
        float u = rng.next_exponential();
        float t;
        if (height_falloff == 0.0f) {  // the optical-depth budget spent at constant density
            float enter, exit;
            if (!slab_span(ray, &enter, &exit)) return false;
            t = net_max(start, enter) + u / density;
            if (t < exit && t < end) {
                *t_out = t;
                return true;
            }
            return false;
        }
        if (std::fabs(hd) < 1e-6f) {
            float ds = density_at(hs);
            if (ds <= 0.0f) return false;
            t = start + u / ds;
        } else {
            float rhs = std::exp(-height_falloff * hs) - u * height_falloff * hd / density;
            if (rhs <= 0.0f) return false;
            float yt = -std::log(rhs) / height_falloff;
            t = (yt - ho) / hd;
        }
        if (t < end) {
            *t_out = t;
            return true;
        }
        return false;
    }
};

// ---- BRDF (brdf.cs) ---------------------------------------------------------------------------
inline Col base_reflectivity(float ior, Col albedo, float metallic) {
    float f0 = std::pow((ior - 1.0f) / (ior + 1.0f), 2.0f);
    return lerp(col(f0), albedo, metallic);
}
inline Col fresnel(float n_dot_v, Col base) {
    float x = 1.0f - n_dot_v;
    float x2 = x * x;
    float x5 = x2 * x2 * x;
    return base + (kWhite - base) * x5;
}
inline float ggx_d(float n_dot_h, float rs) {
    float a2 = rs * rs;
    float nh2 = n_dot_h * n_dot_h;
    float d = (1.0f - nh2) + nh2 * a2;
    return a2 / (kPi * d * d);
}
inline float smith_g1(float n_dot_x, float rs) {
    float k = rs / 2.0f;
    return n_dot_x / (n_dot_x * (1.0f - k) + k);
}
inline V3 ggx_sample_local(float rs, V2 u) {
    float cos_t = std::sqrt((1.0f - u.x) / (u.x * (rs * rs - 1.0f) + 1.0f));
    float sin_t = std::sqrt(net_max(0.0f, 1.0f - cos_t * cos_t));
    float phi = (2.0f * kPi) * u.y;
    return {sin_t * std::cos(phi), sin_t * std::sin(phi), cos_t};
}
inline float power_heuristic(float p1, float p2) {
    float a = p1 * p1;
    float b = p2 * p2;
    return a + b > 0.0f ? a / (a + b) : 0.0f;
}
inline float hg_pdf(float r_dot_l, float g) {
    float gs = g * g;
    float d = 1.0f + gs - 2.0f * g * r_dot_l;
    return (1.0f - gs) / ((4.0f * kPi) * d * std::sqrt(d));
}
inline bool refract(V3 incoming, V3 normal, float ior_ratio, V3* out) {
    float cos_i = -dot(incoming, normal);
    float sin2t = ior_ratio * ior_ratio * (1.0f - cos_i * cos_i);
    if (sin2t >= 1.0f) return false;
    float cos_t = std::sqrt(1.0f - sin2t);
    *out = ior_ratio * incoming + (ior_ratio * cos_i - cos_t) * normal;
    return true;
}
inline Col beer_law(Col albedo, float distance) {
    return {std::pow(net_max(albedo.r, 0.0f), distance), std::pow(net_max(albedo.g, 0.0f), distance),
            std::pow(net_max(albedo.b, 0.0f), distance)};
}
inline V3 perp(V3 v) {
    V3 up = std::fabs(v.y) < 0.9f ? kUp : kRight;
    return normalize(cross(up, v));
}
inline V3 hg_scatter_dir(V3 forward, float g, Rng& rng) {
    V2 u = rand_v2(rng);
    float cos_t;
    if (std::fabs(g) < 1e-3f) {
        cos_t = 1.0f - 2.0f * u.x;
    } else {
        float s = (1.0f - g * g) / (1.0f - g + 2.0f * g * u.x);
        cos_t = (1.0f + g * g - s * s) / (2.0f * g);
    }
    cos_t = net_clamp(cos_t, -1.0f, 1.0f);
    float sin_t = std::sqrt(1.0f - cos_t * cos_t);
    float phi = (2.0f * kPi) * u.y;
    V3 tangent = perp(forward);
    V3 bitangent = cross(forward, tangent);
    return cos_t * forward + (sin_t * std::cos(phi)) * tangent + (sin_t * std::sin(phi)) * bitangent;
}
inline V3 from_tangent_space(V3 dir, V4 tangent, V3 normal) {
    V3 tan = xyz(tangent);
    V3 bitan = tangent.w * cross(normal, tan);
    return dir.x * tan + dir.y * bitan + dir.z * normal;
}
inline V3 reflect(V3 v, V3 n) { return v - (2.0f * dot(v, n)) * n; }

// ---- Surface (scene.cs:15-151) ----------------------------------------------------------------
struct SampleScatter {
    V3 dir;
    Col weight;
    bool has_pdf;
    float pdf;
    bool refracted;
};

struct Surface {
    Col radiance, albedo;
    float roughness, metallic, transparency, ior;
    V3 normal, normal_geo;
    V4 tangent;
    V2 uv;

    V3 clamp_to_geo_side(V3 dir, V3 side) const {
        float d = dot(dir, normal_geo);
        if (d * dot(side, normal_geo) < 0.0f) dir = normalize_or(dir - (2.0f * d) * normal_geo, side);
        return dir;
    }
    float specular_probability(V3 view) const {
        float n_dot_v = net_max(1e-4f, dot(normal, view));
        float f = luminance(fresnel(n_dot_v, base_reflectivity(ior, albedo, metallic)));
        return net_clamp(net_max(f, metallic), 0.001f, 0.999f);
    }
    V3 specular_dir(V3 incoming, Rng& rng) const {
        float rs = net_max(roughness * roughness, 1e-4f);
        V3 h_local = ggx_sample_local(rs, rand_v2(rng));
        V3 h_world = from_tangent_space(h_local, tangent, normal);
        return reflect(incoming, h_world);
    }
    Col opaque_eval(V3 view, V3 light) const {
        float n_dot_l = dot(normal, light);
        if (n_dot_l <= 0.0f) return kBlack;
        float n_dot_v = net_max(1e-4f, dot(normal, view));
        float rs = net_max(roughness * roughness, 1e-4f);
        Col base = base_reflectivity(ior, albedo, metallic);
        V3 half = normalize_or(view + light, normal);
        float n_dot_h = dot(normal, half);
        float h_dot_v = dot(half, view);
        Col f = fresnel(h_dot_v, base);
        float g = smith_g1(n_dot_v, rs) * smith_g1(n_dot_l, rs);
        Col specular = ggx_d(n_dot_h, rs) * f * g / (4.0f * n_dot_v);
        Col diffuse = (kWhite - fresnel(n_dot_v, base)) * albedo * (1.0f - metallic) * (n_dot_l / kPi);
        return (specular + diffuse) * (1.0f - transparency);
    }
    float opaque_pdf(V3 view, V3 light, float spec_p) const {
        float n_dot_l = dot(normal, light);
        if (n_dot_l <= 0.0f) return 0.0f;
        V3 half = normalize_or(view + light, normal);
        float n_dot_h = net_max(0.0f, dot(normal, half));
        float h_dot_v = net_max(1e-6f, dot(half, view));
        float rs = net_max(roughness * roughness, 1e-4f);
        float pdf_spec = ggx_d(n_dot_h, rs) * n_dot_h / (4.0f * h_dot_v);
        float pdf_diff = n_dot_l / kPi;
        return (spec_p * pdf_spec + (1.0f - spec_p) * pdf_diff) * (1.0f - transparency);
    }
    float opaque_pdf(V3 view, V3 light) const { return opaque_pdf(view, light, specular_probability(view)); }
    SampleScatter opaque_scatter(V3 incoming, V3 view, Rng& rng) const {
        float spec_p = specular_probability(view);
        V3 dir;
        if (rng.next_float() < spec_p)
            dir = specular_dir(incoming, rng);
        else
            dir = normalize_or(normal + rand_on_sphere(rng), normal);
        dir = clamp_to_geo_side(dir, normal_geo);
        float pdf = opaque_pdf(view, dir, spec_p);
        return {dir, opaque_eval(view, dir) / net_max(pdf, 1e-6f), true, pdf, false};
    }
    SampleScatter transparent_scatter(V3 incoming, V3 view, Rng& rng) const {
        bool entering = dot(incoming, normal_geo) < 0.0f;
        V3 refract_normal = entering ? normal_geo : -normal_geo;
        float ior_ratio = entering ? 1.0f / ior : ior;
        float rs = net_max(roughness * roughness, 1e-4f);
        V3 half = from_tangent_space(ggx_sample_local(rs, rand_v2(rng)), tangent, normal);
        if (!entering) half = -half;
        if (dot(incoming, half) > 0.0f) half = refract_normal;
        float h_dot_v = net_max(1e-4f, dot(half, view));
        float f = luminance(fresnel(h_dot_v, base_reflectivity(ior, albedo, metallic)));
        V3 rdir;
        if (rng.next_float() >= f && refract(incoming, half, ior_ratio, &rdir))
            return {clamp_to_geo_side(rdir, -refract_normal), kWhite, false, 0.0f, true};
        return {clamp_to_geo_side(reflect(incoming, half), refract_normal), kWhite, false, 0.0f, false};
    }
    SampleScatter scatter(V3 incoming, V3 view, Rng& rng) const {
        if (rng.next_float() < transparency) return transparent_scatter(incoming, view, rng);
        return opaque_scatter(incoming, view, rng);
    }
};

// ---- scene ---------------------------------------------------------------------------------
struct Mesh {
    std::vector<TriLean> tris;
    std::vector<TriAttr> attrs;
    std::vector<BvhNode> nodes;
    std::vector<int32_t> items;
    int node_count = 0;
    AABox bounds;
};

struct Material {
    Col albedo;
    float roughness, metallic, transparency, ior;
    Col radiance;
    int color_tex, rough_tex, metal_tex, normal_tex;
};

struct Object {
    Transform trans;
    Material mat;
    int kind;
    int mesh;
    SphereShape sphere;
    AABox box;
    AABox bounds;
};

struct Fragment {
    Col radiance, radiance_fog;
    bool has_normal;
    V3 normal;
    bool has_uv;
    V2 uv;
    bool has_depth;
    float depth;
};

struct SurfaceHit {
    Surface surf;
    float dist;
};

struct Scene {
    std::vector<std::unique_ptr<Texture>> textures;
    std::vector<std::unique_ptr<Mesh>> meshes;
    std::vector<Object> objects;
    Sky sky;
    bool has_sky = false;
    bool has_fog = false;
    Fog fog{};
    bool built = false;
    std::vector<BvhNode> nodes;
    std::vector<int32_t> items;
    int node_count = 0;

    const Texture* tex(int id) const { return id >= 0 ? textures[id].get() : nullptr; }

    // Object.Intersect -> ShapeExtensions.Intersect math.cs:67-79 (closest hit in world space).
    bool object_intersect(const Object& o, const Ray& ray, ShapeHit* out, int* tri_out, Counters* ctr) const {
        float scale;
        Ray local = transform_ray_inv(o.trans, ray, &scale);
        ShapeHit hit;
        *tri_out = -1;
        bool ok = false;
        if (o.kind == SR_SHAPE_MESH) {
            const Mesh& m = *meshes[o.mesh];
            // The BVH loop accepts a candidate iff its distance is strictly below the best so far;
            // the callback applies the same test to keep the accepted record.
            struct Accept {
                float t, u, v;
                int idx;
            } acc{kInf, 0, 0, -1};
            auto leaf = [&](int idx, float* d) {
                float t, u, v;
                if (!tri_intersect(m.tris[idx], local, &t, &u, &v)) return false;
                *d = t;
                if (t < acc.t) acc = {t, u, v, idx};
                return true;
            };
            int bidx = -1;
            ok = bvh_intersect(m.nodes, m.node_count, m.items, local, leaf, &bidx, ctr, SR_COUNTER_BLAS_NODE,
                               SR_COUNTER_BLAS_SHAPE);
            if (ok) {
                if (ctr) ctr->add(SR_COUNTER_HIT_INFLATE);
                hit = tri_inflate(m.tris[acc.idx], m.attrs[acc.idx], acc.t, acc.u, acc.v);
                *tri_out = acc.idx;
            }
        } else if (o.kind == SR_SHAPE_SPHERE) {
            ok = sphere_intersect(o.sphere, local, &hit);
        } else {
            ok = aabox_intersect(o.box, local, &hit);
        }
        if (!ok) return false;
        V3 wn = normalize(o.trans.rot * (hit.norm / o.trans.scale));
        V3 wng = normalize(o.trans.rot * (hit.norm_geo / o.trans.scale));
        V3 wt = normalize(o.trans.rot * xyz(hit.tan));
        *out = {hit.dist / scale, wn, wng, {wt.x, wt.y, wt.z, hit.tan.w}, hit.uv};
        return true;
    }

    // Scene-level Bvh<Object>.Intersect: closest object hit.
    bool intersect(const Ray& ray, ShapeHit* out, int* obj_out, int* tri_out, Counters* ctr) const {
        struct Accept {
            float d;
            ShapeHit h;
            int tri;
        } acc{kInf, {}, -1};
        auto leaf = [&](int idx, float* d) {
            ShapeHit h;
            int tri;
            if (!object_intersect(objects[idx], ray, &h, &tri, ctr)) return false;
            *d = h.dist;
            if (h.dist < acc.d) acc = {h.dist, h, tri};
            return true;
        };
        int best = -1;
        if (!bvh_intersect(nodes, node_count, items, ray, leaf, &best, ctr, SR_COUNTER_TLAS_NODE,
                           SR_COUNTER_TLAS_SHAPE))
            return false;
        *out = acc.h;
        *obj_out = best;
        *tri_out = acc.tri;
        return true;
    }

    // Material.Sample* scene.cs:173-187.
    Col sample_albedo(const Material& m, V2 uv, Counters* ctr) const {
        const Texture* t = tex(m.color_tex);
        return (t ? t->sample(uv, ctr) : kWhite) * m.albedo;
    }

    // Scene.ShadowTransmittance scene.cs:576-600.
    Col shadow_transmittance(Ray ray, Counters* ctr) const {
        Col tr = kWhite;
        do {
            if (ctr) ctr->add(SR_COUNTER_SCENE_OCCLUDE);
            ShapeHit hit;
            int idx, tri;
            if (!intersect(ray, &hit, &idx, &tri, ctr)) return tr;
            const Material& mat = objects[idx].mat;
            if (mat.transparency <= 0.0f) return kBlack;
            Col albedo = sample_albedo(mat, hit.uv, ctr);
            float n_dot_v = std::fabs(dot(hit.norm_geo, ray.dir));
            Col f = fresnel(n_dot_v, base_reflectivity(mat.ior, albedo, mat.metallic));
            tr = tr * (albedo * mat.transparency * (kWhite - f));
            ray = make_ray(ray_at(ray, hit.dist + net_max(1e-4f, hit.dist * 1e-4f)), ray.dir);
        } while (max_component(tr) > 1e-4f);
        return tr;
    }

    // Scene.Trace scene.cs:602-625.
    bool trace(const Ray& ray, SurfaceHit* out, Counters* ctr, int* obj_out = nullptr) const {
        if (ctr) ctr->add(SR_COUNTER_SCENE_TRACE);
        ShapeHit hit;
        int idx, tri;
        if (!intersect(ray, &hit, &idx, &tri, ctr)) return false;
        if (obj_out) *obj_out = idx;
        const Material& mat = objects[idx].mat;
        Col albedo = sample_albedo(mat, hit.uv, ctr);
        const Texture* rt = tex(mat.rough_tex);
        float roughness = (rt ? rt->sample(hit.uv, ctr).r : 1.0f) * mat.roughness;
        const Texture* mt = tex(mat.metal_tex);
        float metallic = (mt ? mt->sample(hit.uv, ctr).r : 1.0f) * mat.metallic;
        const Texture* nt = tex(mat.normal_tex);
        V3 normal = nt ? normalize_or(from_tangent_space(nt->sample_normal(hit.uv, ctr), hit.tan, hit.norm), hit.norm)
                       : hit.norm;
        V3 txyz = xyz(hit.tan);
        V3 tdir = normalize_or(txyz - dot(txyz, normal) * normal, txyz);
        out->surf = {mat.radiance, albedo, roughness, metallic, mat.transparency, mat.ior, normal, hit.norm_geo,
                     {tdir.x, tdir.y, tdir.z, hit.tan.w}, hit.uv};
        out->dist = hit.dist;
        return true;
    }

    // Scene.RussianRoulette scene.cs:744-756.
    static bool russian_roulette(Col& energy, uint32_t bounce, Rng& rng) {
        if (bounce < 3) return false;
        float survive = net_min(1.0f, max_component(energy));
        if (rng.next_float() >= survive) return true;
        energy = energy / survive;
        return false;
    }

    // Scene.SampleSkyLight scene.cs:758-772.
    bool sample_sky_light(V3 pos, Rng& rng, SampleLight* light_out, Col* tr_out, Counters* ctr) const {
        auto light = sky.light_dir_rand(rng, ctr);
        if (!light || light->pdf <= 0.0f) return false;
        Ray shadow = make_ray(pos, light->dir);
        Col tr = shadow_transmittance(shadow, ctr);
        if (max_component(tr) <= 0.0f) return false;
        if (has_fog) tr = tr * fog.transmittance(shadow, 0.0f, kInf);
        *light_out = *light;
        *tr_out = tr;
        return true;
    }

    // Scene.SampleSkyDirect scene.cs:774-794.
    Col sample_sky_direct(const Surface& surf, V3 hit_pos, V3 view, Rng& rng, Counters* ctr) const {
        SampleLight light;
        Col tr;
        if (!sample_sky_light(hit_pos, rng, &light, &tr, ctr)) return kBlack;
        V3 n = dot(surf.normal, view) >= 0.0f ? surf.normal : -surf.normal;
        if (dot(n, light.dir) <= 0.0f) return kBlack;
        V3 ng = dot(surf.normal_geo, view) >= 0.0f ? surf.normal_geo : -surf.normal_geo;
        if (dot(ng, light.dir) <= 0.0f) return kBlack;
        Col refl = surf.opaque_eval(view, light.dir);
        float surf_pdf = surf.opaque_pdf(view, light.dir);
        float mis = power_heuristic(light.pdf, surf_pdf);
        return sky.radiance(light.dir, ctr) * tr * refl * mis / light.pdf;
    }

    // Scene.SampleSkyDirectFog scene.cs:796-810.
    Col sample_sky_direct_fog(V3 pos, V3 ray_dir, Rng& rng, Counters* ctr) const {
        SampleLight light;
        Col tr;
        if (!sample_sky_light(pos, rng, &light, &tr, ctr)) return kBlack;
        float r_dot_l = dot(ray_dir, light.dir);
        float fog_pdf = hg_pdf(r_dot_l, fog.anisotropy);
        float mis = power_heuristic(light.pdf, fog_pdf);
        return sky.radiance(light.dir, ctr) * tr * fog_pdf * mis / light.pdf;
    }

    // Scene.Sample scene.cs:627-741.
    Fragment sample(Ray ray, Rng& rng, uint32_t bounces, float indirect_clamp, Counters* ctr) const {
        if (ctr) ctr->add(SR_COUNTER_SAMPLE);
        Col radiance = kBlack, radiance_fog = kBlack, energy = kWhite;
        Fragment frag{};
        bool has_scatter_pdf = false;
        float scatter_pdf = 0.0f;
        bool has_medium = false;
        Col medium_albedo = kBlack;
        for (uint32_t i = 0; i != bounces + 1; ++i) {
            if (ctr) ctr->add(SR_COUNTER_SAMPLE_BOUNCE);
            bool primary = i == 0;
            SurfaceHit hit;
            bool has_hit = trace(ray, &hit, ctr);
            float scatter_dist;
            if (has_fog && fog.scatter_distance(ray, 0.0f, has_hit ? hit.dist : kInf, rng, &scatter_dist)) {
                energy = energy * fog.color;
                Col scatter_rad = sample_sky_direct_fog(ray_at(ray, scatter_dist), ray.dir, rng, ctr) * energy;
                if (primary)
                    radiance_fog = radiance_fog + scatter_rad;
                else
                    radiance = radiance + scatter_rad;
                if (russian_roulette(energy, i, rng)) break;
                V3 sdir = hg_scatter_dir(ray.dir, fog.anisotropy, rng);
                has_scatter_pdf = true;
                scatter_pdf = hg_pdf(dot(ray.dir, sdir), fog.anisotropy);
                ray = make_ray(ray_at(ray, scatter_dist), sdir);
            } else if (has_hit) {
                const Surface& surf = hit.surf;
                float dist = hit.dist;
                V3 view = -ray.dir;
                float dist_bias = net_max(1e-4f, dist * 1e-4f);
                V3 hit_pos = ray_at(ray, dist - dist_bias);
                if (has_medium) energy = energy * beer_law(medium_albedo, dist);
                radiance = radiance + surf.radiance * energy;
                if (i == 0) {
                    frag.has_normal = true;
                    frag.normal = surf.normal;
                    frag.has_uv = true;
                    frag.uv = surf.uv;
                    frag.has_depth = true;
                    frag.depth = dist;
                }
                radiance = radiance + sample_sky_direct(surf, hit_pos, view, rng, ctr) * energy;
                if (russian_roulette(energy, i, rng)) break;
                SampleScatter sc = surf.scatter(ray.dir, view, rng);
                energy = energy * sc.weight;
                energy = clamp_luminance(energy, indirect_clamp);
                bool enter = dot(sc.dir, surf.normal_geo) < 0.0f;
                if (sc.refracted) {
                    has_medium = enter;
                    if (enter) medium_albedo = surf.albedo;
                } else if (!enter) {
                    has_medium = false;
                }
                has_scatter_pdf = sc.has_pdf;
                scatter_pdf = sc.pdf;
                ray = make_ray(ray_at(ray, dist) + sc.dir * dist_bias, sc.dir);
            } else {
                float mis = 1.0f;
                if (has_scatter_pdf) {
                    auto l = sky.light_dir(ray.dir);
                    mis = power_heuristic(scatter_pdf, l ? l->pdf : 0.0f);
                }
                radiance = radiance + sky.radiance(ray.dir, ctr) * mis * energy;
                break;
            }
        }
        frag.radiance = radiance;
        frag.radiance_fog = radiance_fog;
        return frag;
    }
};

// View.Ray math.cs:1613-1636.
struct View {
    Transform trans;
    float fov, near_plane;
    Ray ray(V2 screen, float aspect) const {
        float ndc_x = screen.x * 2.0f - 1.0f;
        float ndc_y = -screen.y * 2.0f + 1.0f;
        float thh, thv;
        if (aspect >= 1.0f) {
            thh = std::tan(fov * 0.5f);
            thv = thh / aspect;
        } else {
            thv = std::tan(fov * 0.5f);
            thh = thv * aspect;
        }
        V3 local{ndc_x * thh, ndc_y * thv, 1.0f};
        V3 origin = trans.pos + trans.rot * V3{0.0f, 0.0f, near_plane};
        V3 dir = trans.rot * normalize(local);
        return make_ray(origin, dir);
    }
};

Transform to_transform(const SrTransform& t) {
    return {{t.pos[0], t.pos[1], t.pos[2]}, {t.rot[0], t.rot[1], t.rot[2], t.rot[3]}, {t.scale[0], t.scale[1], t.scale[2]}};
}

// Renderer.RelativeStdErr renderer.cs:232-237.
inline float relative_std_err(float sum, float sum_sqr, uint32_t n) {
    float mean = sum / (float)n;
    float variance = net_max(0.0f, sum_sqr / (float)n - mean * mean);
    return std::sqrt(variance / (float)n) / net_max(mean, 1e-4f);
}

// Renderer.Render renderer.cs:153-229 for one pixel; writes the seven AOVs.
void render_pixel(const Scene& scene, const View& view, const SrRenderParams& p, float aspect, uint32_t x, uint32_t y,
                  const SrAovs& out, Counters* ctr) {
    Rng rng(x, y);
    Col rad_sum = kBlack, fog_sum = kBlack;
    float lum_sum = 0, lum_sqr = 0, surf_sum = 0, surf_sqr = 0;
    V3 normal_sum{0, 0, 0}, normal_fallback{0, 0, 0};
    uint32_t normal_count = 0;
    bool has_uv = false;
    V2 uv{0, 0};
    float depth_sum = 0;
    uint32_t depth_count = 0;
    uint32_t si = 0;
    for (; si != p.max_samples; ++si) {
        float jx = rng.next_float();
        float px = ((float)x + jx) / (float)p.width;
        float jy = rng.next_float();
        float py = ((float)y + jy) / (float)p.height;
        Ray ray = view.ray({px, py}, aspect);
        Fragment f = scene.sample(ray, rng, p.bounces, p.indirect_clamp, ctr);
        rad_sum = rad_sum + f.radiance;
        fog_sum = fog_sum + f.radiance_fog;
        float lum = luminance(f.radiance) + luminance(f.radiance_fog);
        lum_sum += lum;
        lum_sqr += lum * lum;
        float ls = luminance(f.radiance);
        surf_sum += ls;
        surf_sqr += ls * ls;
        if (f.has_normal) {
            normal_sum = normal_sum + f.normal;
            normal_fallback = f.normal;
            normal_count++;
        }
        if (f.has_depth) {
            depth_sum += f.depth;
            depth_count++;
        }
        if (!has_uv && f.has_uv) {
            has_uv = true;
            uv = f.uv;
        }
        if (si >= p.min_samples - 1) {
            if (relative_std_err(lum_sum, lum_sqr, si + 1) < p.variance_threshold) break;
        }
    }
    uint32_t count = si + 1;
    float var = relative_std_err(surf_sum, surf_sqr, count);
    Col radiance = rad_sum / (float)count;
    Col radiance_fog = fog_sum / (float)count;
    size_t i = (size_t)y * p.width + x;
    if (out.radiance) {
        out.radiance[i * 3 + 0] = radiance.r;
        out.radiance[i * 3 + 1] = radiance.g;
        out.radiance[i * 3 + 2] = radiance.b;
    }
    if (out.radiance_fog) {
        out.radiance_fog[i * 3 + 0] = radiance_fog.r;
        out.radiance_fog[i * 3 + 1] = radiance_fog.g;
        out.radiance_fog[i * 3 + 2] = radiance_fog.b;
    }
    V3 n = normal_count > 0 ? normalize_or(normal_sum, normal_fallback) : V3{0, 0, 0};
    if (out.normals) {
        out.normals[i * 3 + 0] = n.x;
        out.normals[i * 3 + 1] = n.y;
        out.normals[i * 3 + 2] = n.z;
    }
    if (out.uv) {
        out.uv[i * 2 + 0] = has_uv ? uv.x : 0.0f;
        out.uv[i * 2 + 1] = has_uv ? uv.y : 0.0f;
    }
    if (out.depth) out.depth[i] = depth_count > 0 ? depth_sum / (float)depth_count : kInf;
    if (out.samples) out.samples[i] = count;
    if (out.variance) out.variance[i] = var;
}

// ---- Compositor (compose.cs) ------------------------------------------------------------------
struct Compositor {
    SrComposeParams p;
    float lum_limit_inv, normal_limit_inv, depth_limit_inv;
    explicit Compositor(const SrComposeParams& cp) : p(cp) {
        lum_limit_inv = 1.0f / (p.denoise_luminance_limit * p.denoise_luminance_limit * 2.0f);
        normal_limit_inv = 1.0f / (p.denoise_normal_limit * p.denoise_normal_limit * 2.0f);
        depth_limit_inv = 1.0f / (p.denoise_depth_limit * p.denoise_depth_limit * 2.0f);
    }
    static Col load3(const float* a, size_t i) { return {a[i * 3], a[i * 3 + 1], a[i * 3 + 2]}; }
    static V3 load3v(const float* a, size_t i) { return {a[i * 3], a[i * 3 + 1], a[i * 3 + 2]}; }

    Col filter(const SrAovs& a, int w, int h, int cx, int cy) const {
        float rp = p.denoise_radius * std::sqrt((float)(w * h));
        float rp_inv = 1.0f / (rp * rp * 2.0f);
        int kr = (int)std::ceil(rp * 3.0f);
        size_t ci = (size_t)cy * w + cx;
        Col c_rad = load3(a.radiance, ci);
        V3 c_n = load3v(a.normals, ci);
        float c_d = a.depth[ci];
        bool has_n = mag_sqr(c_n) > 0.0f;
        bool has_d = !std::isinf(c_d);
        float lum = luminance(c_rad);
        float boost = 1.0f + lum * p.denoise_luminance_boost;
        float dw = net_min(a.variance[ci] * boost * p.denoise_strength, p.denoise_strength_max);
        if (dw < 1e-4f) return c_rad;
        float wsum = 1.0f;
        Col rsum = c_rad;
        for (int ky = -kr; ky <= kr; ++ky) {
            int ky2 = ky * ky;
            for (int kx = -kr; kx <= kr; ++kx) {
                if (kx == 0 && ky == 0) continue;
                float kd = (float)(kx * kx + ky2);
                if (kd > (float)(kr * kr)) continue;
                int nx = cx + kx, ny = cy + ky;
                if (nx < 0 || nx >= w || ny < 0 || ny >= h) continue;
                size_t ni = (size_t)ny * w + nx;
                Col n_rad = load3(a.radiance, ni);
                V3 n_n = load3v(a.normals, ni);
                float n_d = a.depth[ni];
                bool nh_n = mag_sqr(n_n) > 0.0f;
                bool nh_d = !std::isinf(n_d);
                if (has_n != nh_n || has_d != nh_d) continue;
                float wgt = dw * std::exp(-kd * rp_inv);
                if (has_n && wgt > 0.0f) {
                    V3 nd = c_n - n_n;
                    wgt *= std::exp(-mag_sqr(nd) * normal_limit_inv);
                }
                if (has_d && wgt > 0.0f) {
                    float dd = c_d - n_d;
                    wgt *= std::exp(-(dd * dd) * depth_limit_inv);
                }
                if (wgt > 0.0f) {
                    float ld = net_max(0.0f, luminance(n_rad) - lum);
                    wgt *= std::exp(-(ld * ld) * lum_limit_inv);
                }
                wsum += wgt;
                rsum = rsum + n_rad * wgt;
            }
        }
        return rsum / wsum;
    }
    Col filter_fog(const SrAovs& a, int w, int h, int cx, int cy) const {
        float rp = p.denoise_fog_radius * std::sqrt((float)(w * h));
        float rp_inv = 1.0f / (rp * rp * 2.0f);
        int kr = (int)std::ceil(rp * 3.0f);
        float wsum = 1.0f;
        Col rsum = load3(a.radiance_fog, (size_t)cy * w + cx);
        for (int ky = -kr; ky <= kr; ++ky) {
            int ky2 = ky * ky;
            for (int kx = -kr; kx <= kr; ++kx) {
                if (kx == 0 && ky == 0) continue;
                float kd = (float)(kx * kx + ky2);
                if (kd > (float)(kr * kr)) continue;
                int nx = cx + kx, ny = cy + ky;
                if (nx < 0 || nx >= w || ny < 0 || ny >= h) continue;
                float wgt = p.denoise_fog_strength * std::exp(-kd * rp_inv);
                wsum += wgt;
                rsum = rsum + load3(a.radiance_fog, (size_t)ny * w + nx) * wgt;
            }
        }
        return rsum / wsum;
    }
    static void to_pixel(Col c, uint8_t* out) {
        Col cc{net_clamp(c.r, 0.0f, 1.0f), net_clamp(c.g, 0.0f, 1.0f), net_clamp(c.b, 0.0f, 1.0f)};
        float r = net_max(1.055f * std::pow(cc.r, 0.416666667f) - 0.055f, 0.0f);
        float g = net_max(1.055f * std::pow(cc.g, 0.416666667f) - 0.055f, 0.0f);
        float b = net_max(1.055f * std::pow(cc.b, 0.416666667f) - 0.055f, 0.0f);
        out[0] = (uint8_t)(int)(r * 255.0f + 0.5f);
        out[1] = (uint8_t)(int)(g * 255.0f + 0.5f);
        out[2] = (uint8_t)(int)(b * 255.0f + 0.5f);
    }
    void tonemap(Col radiance, uint8_t* out) const {
        Col x = radiance * p.exposure;
        if (p.tonemapper == SR_TONEMAP_REINHARD) {
            to_pixel(x / (x + col(1.0f)), out);
        } else {
            const float a = 1.8f, b = 1.4f, c = 0.5f, d = 1.5f;
            to_pixel((x * (a * x + col(b))) / (x * (a * x + col(c)) + col(d)), out);
        }
    }
};

thread_local char g_err[512];
int fail(int code, const char* msg) {
    std::snprintf(g_err, sizeof(g_err), "%s", msg);
    return code;
}

template <typename Fn>
void parallel_for(int n, int threads, Fn fn) {
    if (threads <= 1 || n <= 1) {
        for (int i = 0; i < n; ++i) fn(i, 0);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t] {
            for (;;) {
                int i = next.fetch_add(1);
                if (i >= n) break;
                fn(i, t);
            }
        });
    for (auto& th : pool) th.join();
}

// ---- FP64 path-replay adjoint ------------------------------------------------------------------
//
// The double-precision reference for the GPU's path-replay adjoint.  The reference renderer has no
// derivatives; this restates the replay estimator of dL/dθ, for θ = the texels of an albedo texture,
// the texels of a roughness texture (its red channel) and the fog density, given dL/dI for the
// image I = radiance + radiance_fog.  Paths are replayed in float with the reference's arithmetic --
// the same random numbers and the same paths as Scene::sample -- while every derivative is taken in
// double by forward-mode dual numbers through the reference's formulas: OpaqueEval (scene.cs:76-101
// with brdf.cs:12-57), the fog's optical depth and free-flight density (scene.cs:445-496),
// ClampLuminance (math.cs:121-125) and RussianRoulette (scene.cs:744-756).  The chain from the
// camera to every vertex runs backwards in double.  Held fixed, as path replay does: the sampled
// directions, lobe choices, roulette decisions, pdfs and MIS weights.  The free-flight sampling of
// every segment contributes the score d log p / d density of its sampled event (a scatter at t,
// reaching a surface, or escaping to the sky).  Scenes with transparent materials are not covered
// (the GPU adjoint refuses them).

struct Dual {
    double v, d;
};
inline Dual dual(double v, double d = 0.0) { return {v, d}; }
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline Dual dexp(Dual a) {
    double e = std::exp(a.v);
    return {e, a.d * e};
}
inline Dual dlog(Dual a) { return {std::log(a.v), a.d / a.v}; }
struct DCol {
    Dual c[3];
};
inline DCol dcol(Col x) { return {{dual(x.r), dual(x.g), dual(x.b)}}; }
inline double cval(Col x, int i) { return i == 0 ? x.r : (i == 1 ? x.g : x.b); }

struct V3d {
    double x, y, z;
};
inline V3d v3d(V3 v) { return {v.x, v.y, v.z}; }
inline double dotd(V3d a, V3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3d normalize_or_d(V3d v, V3d fb) {
    double m = dotd(v, v);
    if (!(m >= 1e-12)) return fb;
    double k = 1.0 / std::sqrt(m);
    return {v.x * k, v.y * k, v.z * k};
}

// Brdf.Fresnel, GgxD, SmithG1 (brdf.cs:22-57) over duals.
inline Dual fresnel_dual(double n_dot_v, Dual base) {
    double x = 1.0 - n_dot_v;
    double x5 = x * x * x * x * x;
    return base + (dual(1.0) - base) * dual(x5);
}
inline Dual ggx_d_dual(double n_dot_h, Dual rs) {
    Dual a2 = rs * rs;
    double nh2 = n_dot_h * n_dot_h;
    Dual d = dual(1.0 - nh2) + dual(nh2) * a2;
    return a2 / (dual(M_PI) * d * d);
}
inline Dual smith_g1_dual(double n_dot_x, Dual rs) {
    Dual k = rs / dual(2.0);
    return dual(n_dot_x) / (dual(n_dot_x) * (dual(1.0) - k) + k);
}

// Surface.OpaqueEval (scene.cs:76-101) in double over a dual albedo and roughness; the branch
// decisions (light behind the surface, the roughness floor) are the float surface's.
DCol opaque_eval_dual(const Surface& s, V3 view, V3 light, const DCol& albedo, Dual roughness) {
    DCol out{{dual(0), dual(0), dual(0)}};
    if (dot(s.normal, light) <= 0.0f) return out;
    const V3d n = v3d(s.normal), v = v3d(view), l = v3d(light);
    const double n_dot_l = dotd(n, l);
    const double n_dot_v = std::max(1e-4, dotd(n, v));
    Dual r2 = roughness * roughness;
    Dual rs = s.roughness * s.roughness > 1e-4f ? r2 : dual(1e-4);
    const double f0 = std::pow(((double)s.ior - 1.0) / ((double)s.ior + 1.0), 2.0);
    const V3d half = normalize_or_d({v.x + l.x, v.y + l.y, v.z + l.z}, n);
    const double n_dot_h = dotd(n, half), h_dot_v = dotd(half, v);
    Dual g = smith_g1_dual(n_dot_v, rs) * smith_g1_dual(n_dot_l, rs);
    Dual dterm = ggx_d_dual(n_dot_h, rs) * g / dual(4.0 * n_dot_v);
    const double m = s.metallic, tr = 1.0 - (double)s.transparency;
    for (int i = 0; i < 3; ++i) {
        Dual base = dual(f0) + (albedo.c[i] - dual(f0)) * dual(m);  // Color.Lerp(f0, albedo, metallic)
        Dual spec = dterm * fresnel_dual(h_dot_v, base);
        Dual diff = (dual(1.0) - fresnel_dual(n_dot_v, base)) * albedo.c[i] * dual((1.0 - m) * (n_dot_l / M_PI));
        out.c[i] = (spec + diff) * dual(tr);
    }
    return out;
}

// Fog.OpticalDepth (scene.cs:452-467) over [start, end] in double with a dual density.
Dual optical_depth_dual(const Fog& f, const Ray& r, double start, double end, Dual density) {
    if (f.height_falloff == 0.0f) {  // homogeneous: density x the length of [start, end] below the top
        float enter, exit;
        if (!f.slab_span(r, &enter, &exit)) return dual(0.0);
        const double a = std::max(start, (double)enter), b = std::min(end, (double)exit);
        return density * dual(b > a ? b - a : 0.0);
    }
    const double hd = r.dir.y, ho = r.origin.y, k = f.height_falloff;
    const double hs = ho + start * hd;
    const double es = std::exp(-k * hs);
    if (std::fabs(r.dir.y) < 1e-6f) return density * dual(es * (end - start));
    const double ee = std::isinf(end) ? (end * hd > 0 ? 0.0 : INFINITY) : std::exp(-k * (ho + end * hd));
    return density * dual((es - ee) / (k * hd));
}

// Albedo + roughness derivatives of one BRDF evaluation: d eval / d albedo (channel i only moves
// channel i of eval: this takes the diagonal) and d eval / d roughness, both in double.
void eval_derivatives(const Surface& s, V3 view, V3 light, double d_alb[3], double d_rough[3]) {
    for (int i = 0; i < 3; ++i) {
        DCol a = dcol(s.albedo);
        a.c[i].d = 1.0;
        d_alb[i] = opaque_eval_dual(s, view, light, a, dual(s.roughness)).c[i].d;
    }
    DCol e = opaque_eval_dual(s, view, light, dcol(s.albedo), dual(s.roughness, 1.0));
    for (int i = 0; i < 3; ++i) d_rough[i] = e.c[i].d;
}

enum { AJ_FOG = 0, AJ_SURF = 1, AJ_SURF_END = 2, AJ_SKY = 3, AJ_FOG_END = 4 };
struct AdjVertex64 {
    int kind;
    uint32_t bounce;
    Col e_in;       // throughput entering the vertex (float, as the forward has it)
    Col s;          // scatter weight (surface)
    double add[3];  // radiance added per unit throughput
    double dadd_a[3], dadd_r[3], dadd_f[3];  // d add / d albedo channel, d roughness, d density
    double ds_a[3], ds_r[3];                 // d s / d albedo channel, d roughness
    double score;   // d log(density of the sampled segment into the vertex) / d fog density
    float clamp_max;
    V2 uv;
    int object;
};

// Scene.RussianRoulette's division (scene.cs:744-756) over duals: x / min(1, max component of x)
// from bounce 3 on; the survival value's branch is the float forward's.
inline DCol roulette_dual(const DCol& x, Col xf, uint32_t bounce) {
    if (bounce < 3) return x;
    float p = net_min(1.0f, max_component(xf));
    if (!(p < 1.0f)) return x;
    const int m = (xf.r >= xf.g && xf.r >= xf.b) ? 0 : (xf.g >= xf.b ? 1 : 2);
    Dual pd = x.c[m];
    return {{x.c[0] / pd, x.c[1] / pd, x.c[2] / pd}};
}
// Color.ClampLuminance (math.cs:121-125) over duals; the branch is the float forward's.
inline DCol clamp_dual(const DCol& x, Col xf, float max) {
    if (!(luminance(xf) > max)) return x;
    Dual lum = dual(0.2126) * x.c[0] + dual(0.7152) * x.c[1] + dual(0.0722) * x.c[2];
    Dual k = dual(max) / lum;
    return {{x.c[0] * k, x.c[1] * k, x.c[2] * k}};
}

struct Adjoint64 {
    const Scene& sc;
    Dual density;  // the fog density, as a dual seeded 1 (d / d density)

    // d log p / d density of a segment's free flight (scene.cs:469-496 samples t with density
    // sigma(t) exp(-tau(0, t))): a scatter at t, or no scatter before `end` (a surface or the sky).
    double score_scatter(const Ray& r, float t) const {
        const double y = r.origin.y + (double)t * r.dir.y;
        Dual log_sigma = dlog(density) - dual(sc.fog.height_falloff * y);
        return (log_sigma - optical_depth_dual(sc.fog, r, 0.0, t, density)).d;
    }
    double score_pass(const Ray& r, double end) const {
        Dual tau = optical_depth_dual(sc.fog, r, 0.0, end, density);
        return std::isfinite(tau.v) ? -tau.d : 0.0;
    }
    // d/d density of the shadow ray's fog transmittance exp(-tau(0, inf)), relative to its value.
    double transmittance_log_derivative(const Ray& shadow) const {
        Dual tau = optical_depth_dual(sc.fog, shadow, 0.0, INFINITY, density);
        return std::isfinite(tau.v) ? -tau.d : 0.0;
    }

    // Scene::sample replayed, recording the vertices (returns their number); the float arithmetic
    // and RNG draws are sample()'s, so radiance / radiance_fog come out the same.
    int replay(Ray ray, Rng& rng, uint32_t bounces, float indirect_clamp, AdjVertex64* v, Col& radiance,
               Col& radiance_fog) const {
        radiance = kBlack;
        radiance_fog = kBlack;
        Col energy = kWhite;
        bool has_scatter_pdf = false;
        float scatter_pdf = 0.0f;
        int n = 0;
        for (uint32_t i = 0; i != bounces + 1; ++i) {
            SurfaceHit hit;
            int obj = -1;
            bool has_hit = sc.trace(ray, &hit, nullptr, &obj);
            float scatter_dist;
            AdjVertex64& x = v[n++];
            x = AdjVertex64{};
            x.bounce = i;
            x.e_in = energy;
            x.clamp_max = indirect_clamp;
            if (sc.has_fog && sc.fog.scatter_distance(ray, 0.0f, has_hit ? hit.dist : kInf, rng, &scatter_dist)) {
                x.kind = AJ_FOG;
                x.score = score_scatter(ray, scatter_dist);
                energy = energy * sc.fog.color;
                // Scene.SampleSkyDirectFog scene.cs:796-810
                V3 pos = ray_at(ray, scatter_dist);
                Col nee = kBlack;
                SampleLight light;
                Col tr;
                if (sc.sample_sky_light(pos, rng, &light, &tr, nullptr)) {
                    float fog_pdf = hg_pdf(dot(ray.dir, light.dir), sc.fog.anisotropy);
                    float mis = power_heuristic(light.pdf, fog_pdf);
                    nee = sc.sky.radiance(light.dir, nullptr) * tr * fog_pdf * mis / light.pdf;
                    const double dl = transmittance_log_derivative(make_ray(pos, light.dir));
                    for (int c = 0; c < 3; ++c) x.dadd_f[c] = cval(nee, c) * dl;
                }
                for (int c = 0; c < 3; ++c) x.add[c] = cval(nee, c);
                Col scatter_rad = nee * energy;
                if (i == 0)
                    radiance_fog = radiance_fog + scatter_rad;
                else
                    radiance = radiance + scatter_rad;
                if (Scene::russian_roulette(energy, i, rng)) {
                    x.kind = AJ_FOG_END;
                    break;
                }
                V3 sdir = hg_scatter_dir(ray.dir, sc.fog.anisotropy, rng);
                has_scatter_pdf = true;
                scatter_pdf = hg_pdf(dot(ray.dir, sdir), sc.fog.anisotropy);
                ray = make_ray(ray_at(ray, scatter_dist), sdir);
            } else if (has_hit) {
                const Surface& surf = hit.surf;
                float dist = hit.dist;
                V3 view = -ray.dir;
                float dist_bias = net_max(1e-4f, dist * 1e-4f);
                V3 hit_pos = ray_at(ray, dist - dist_bias);
                x.kind = AJ_SURF;
                x.uv = surf.uv;
                x.object = obj;
                if (sc.has_fog) x.score = score_pass(ray, dist);
                radiance = radiance + surf.radiance * energy;
                // Scene.SampleSkyDirect scene.cs:774-794
                Col nee = kBlack;
                SampleLight light;
                Col tr;
                if (sc.sample_sky_light(hit_pos, rng, &light, &tr, nullptr)) {
                    V3 nn = dot(surf.normal, view) >= 0.0f ? surf.normal : -surf.normal;
                    V3 ng = dot(surf.normal_geo, view) >= 0.0f ? surf.normal_geo : -surf.normal_geo;
                    if (dot(nn, light.dir) > 0.0f && dot(ng, light.dir) > 0.0f) {
                        Col refl = surf.opaque_eval(view, light.dir);
                        float mis = power_heuristic(light.pdf, surf.opaque_pdf(view, light.dir));
                        Col sky = sc.sky.radiance(light.dir, nullptr);
                        nee = sky * tr * refl * mis / light.pdf;
                        double da[3], dr[3];
                        eval_derivatives(surf, view, light.dir, da, dr);
                        const double dl = sc.has_fog ? transmittance_log_derivative(make_ray(hit_pos, light.dir)) : 0.0;
                        for (int c = 0; c < 3; ++c) {
                            const double k = cval(sky, c) * cval(tr, c) * (double)mis / (double)light.pdf;
                            x.dadd_a[c] = k * da[c];
                            x.dadd_r[c] = k * dr[c];
                            x.dadd_f[c] = cval(nee, c) * dl;
                        }
                    }
                }
                radiance = radiance + nee * energy;
                for (int c = 0; c < 3; ++c) x.add[c] = cval(surf.radiance, c) + cval(nee, c);
                if (Scene::russian_roulette(energy, i, rng)) {
                    x.kind = AJ_SURF_END;
                    break;
                }
                SampleScatter scat = surf.scatter(ray.dir, view, rng);
                x.s = scat.weight;
                double da[3], dr[3];
                eval_derivatives(surf, view, scat.dir, da, dr);
                const double ipdf = 1.0 / (double)net_max(scat.pdf, 1e-6f);
                for (int c = 0; c < 3; ++c) {
                    x.ds_a[c] = da[c] * ipdf;
                    x.ds_r[c] = dr[c] * ipdf;
                }
                energy = energy * scat.weight;
                energy = clamp_luminance(energy, indirect_clamp);
                has_scatter_pdf = scat.has_pdf;
                scatter_pdf = scat.pdf;
                ray = make_ray(ray_at(ray, dist) + scat.dir * dist_bias, scat.dir);
            } else {
                x.kind = AJ_SKY;
                if (sc.has_fog) x.score = score_pass(ray, INFINITY);
                float mis = 1.0f;
                if (has_scatter_pdf) {
                    auto l = sc.sky.light_dir(ray.dir);
                    mis = power_heuristic(scatter_pdf, l ? l->pdf : 0.0f);
                }
                Col add = sc.sky.radiance(ray.dir, nullptr) * mis;
                for (int c = 0; c < 3; ++c) x.add[c] = cval(add, c);
                radiance = radiance + add * energy;
                break;
            }
        }
        return n;
    }
};

// The texels (and bilinear weights) Texture.Sample (texture.cs:39-69) reads at uv.
int texel_footprint(const Texture& t, V2 coord, uint32_t idx[4], double w[4]) {
    float u = coord.x * t.tiling.x;
    u -= std::floor(u);
    float v = coord.y * t.tiling.y;
    v -= std::floor(v);
    if (t.filter == 1) {
        uint32_t x = (uint32_t)(u * (float)t.width) % t.width;
        uint32_t y = (uint32_t)(v * (float)t.height) % t.height;
        idx[0] = y * t.width + x;
        w[0] = 1.0;
        return 1;
    }
    float fx = u * (float)(t.width - 1), fy = v * (float)(t.height - 1);
    uint32_t x0 = (uint32_t)fx, y0 = (uint32_t)fy;
    uint32_t x1 = (x0 + 1) % t.width, y1 = (y0 + 1) % t.height;
    double tx = (double)fx - (double)x0, ty = (double)fy - (double)y0;
    idx[0] = y0 * t.width + x0, w[0] = (1 - tx) * (1 - ty);
    idx[1] = y0 * t.width + x1, w[1] = tx * (1 - ty);
    idx[2] = y1 * t.width + x0, w[2] = (1 - tx) * ty;
    idx[3] = y1 * t.width + x1, w[3] = tx * ty;
    return 4;
}

// Per-thread gradient sums.
struct AdjSums {
    std::vector<double> a, r;
    double f = 0.0;
};

// Reverse sweep over one sample's vertices; G = dL/dI / sample count of the pixel.
void adjoint_sweep(const Scene& sc, const AdjVertex64* v, int n, const double G[3], int tex_a, int tex_r,
                   AdjSums& out) {
    double a[3] = {0, 0, 0};  // d loss / d (throughput leaving the vertex)
    for (int k = n - 1; k >= 0; --k) {
        const AdjVertex64& q = v[k];
        double a_in[3];
        for (int c = 0; c < 3; ++c) a_in[c] = G[c] * q.add[c];
        if (q.kind == AJ_FOG || q.kind == AJ_FOG_END) {
            const Col fc = sc.fog.color;
            const Col ef = q.e_in * fc;
            double a_f[3] = {a_in[0], a_in[1], a_in[2]};  // d loss / d (throughput after the fog colour)
            if (q.kind == AJ_FOG)
                for (int j = 0; j < 3; ++j) {  // column j of d roulette(ef) / d ef
                    DCol x = dcol(ef);
                    x.c[j].d = 1.0;
                    DCol y = roulette_dual(x, ef, q.bounce);
                    for (int c = 0; c < 3; ++c) a_f[j] += a[c] * y.c[c].d;
                }
            for (int c = 0; c < 3; ++c) {
                a_in[c] = a_f[c] * cval(fc, c);
                out.f += G[c] * cval(ef, c) * q.dadd_f[c];
            }
        } else if (q.kind == AJ_SURF || q.kind == AJ_SURF_END) {
            const bool scatters = q.kind == AJ_SURF;
            Col rr_f = q.e_in;  // the roulette's float output (as the forward divides)
            if (q.bounce >= 3) {
                float p = net_min(1.0f, max_component(q.e_in));
                if (p < 1.0f) rr_f = q.e_in / p;
            }
            const Col pre_f = rr_f * q.s;
            if (scatters)
                for (int j = 0; j < 3; ++j) {  // column j of d clamp(roulette(e) * s) / d e
                    DCol x = dcol(q.e_in);
                    x.c[j].d = 1.0;
                    DCol y = roulette_dual(x, q.e_in, q.bounce);
                    for (int c = 0; c < 3; ++c) y.c[c] = y.c[c] * dual(cval(q.s, c));
                    y = clamp_dual(y, pre_f, q.clamp_max);
                    for (int c = 0; c < 3; ++c) a_in[j] += a[c] * y.c[c].d;
                }
            // d loss / d parameter at this vertex: through the light sample and the scatter weight
            auto through_scatter = [&](const double ds[3]) {
                if (!scatters) return 0.0;
                DCol y;
                for (int c = 0; c < 3; ++c) y.c[c] = dual(cval(rr_f, c)) * dual(cval(q.s, c), ds[c]);
                y = clamp_dual(y, pre_f, q.clamp_max);
                return a[0] * y.c[0].d + a[1] * y.c[1].d + a[2] * y.c[2].d;
            };
            const Material& m = sc.objects[q.object].mat;
            uint32_t idx[4];
            double w[4];
            if (tex_a >= 0 && m.color_tex == tex_a) {
                const int nt = texel_footprint(*sc.textures[tex_a], q.uv, idx, w);
                for (int c = 0; c < 3; ++c) {
                    double ds[3] = {0, 0, 0};
                    ds[c] = q.ds_a[c];
                    const double g = G[c] * cval(q.e_in, c) * q.dadd_a[c] + through_scatter(ds);
                    for (int t = 0; t < nt; ++t) out.a[3 * idx[t] + c] += g * cval(m.albedo, c) * w[t];
                }
            }
            if (tex_r >= 0 && m.rough_tex == tex_r) {
                const int nt = texel_footprint(*sc.textures[tex_r], q.uv, idx, w);
                double g = through_scatter(q.ds_r);
                for (int c = 0; c < 3; ++c) g += G[c] * cval(q.e_in, c) * q.dadd_r[c];
                for (int t = 0; t < nt; ++t) out.r[3 * idx[t]] += g * m.roughness * w[t];
            }
            for (int c = 0; c < 3; ++c) out.f += G[c] * cval(q.e_in, c) * q.dadd_f[c];
        }
        // the segment into the vertex: its sampling density's score times everything downstream
        out.f += q.score * (a_in[0] * q.e_in.r + a_in[1] * q.e_in.g + a_in[2] * q.e_in.b);
        for (int c = 0; c < 3; ++c) a[c] = a_in[c];
    }
}

}  // namespace

// =====================================================================================================
// C API for the Python test harness (ctypes).
// =====================================================================================================
extern "C" {

const char* oracle_last_error(void) { return g_err; }

// First `n` outputs of Rng(seed_a, seed_b): NextUInt values, and (from a fresh generator) NextFloat values.
void oracle_rng_stream(uint32_t seed_a, uint32_t seed_b, uint32_t n, uint32_t* out_u32, float* out_f32) {
    Rng a(seed_a, seed_b);
    for (uint32_t i = 0; i < n; ++i) out_u32[i] = a.next_uint();
    Rng b(seed_a, seed_b);
    for (uint32_t i = 0; i < n; ++i) out_f32[i] = b.next_float();
}

// splitmix64 sequence from `seed` (for the published known-answer check).
void oracle_splitmix64(uint64_t seed, uint32_t n, uint64_t* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = split_mix64(seed);
}

int oracle_triangles_from_corners(const float* pos, const float* uvs, const float* normals, uint32_t count,
                                  int32_t smooth, SrTriangle* out) {
    if (!pos || !out) return fail(SR_ERR_INVALID_ARG, "null pointer");
    std::vector<Triangle> tris(count);
    for (uint32_t i = 0; i < count; ++i) {
        const float* p = pos + (size_t)i * 9;
        V3 a{p[0], p[1], p[2]}, b{p[3], p[4], p[5]}, c{p[6], p[7], p[8]};
        V2 ua{0, 0}, ub{1, 0}, uc{0, 1};
        if (uvs) {
            const float* u = uvs + (size_t)i * 6;
            ua = {u[0], u[1]};
            ub = {u[2], u[3]};
            uc = {u[4], u[5]};
        }
        if (normals) {
            const float* n = normals + (size_t)i * 9;
            tris[i] = make_triangle_full(a, b, c, {n[0], n[1], n[2]}, {n[3], n[4], n[5]}, {n[6], n[7], n[8]}, ua, ub, uc);
        } else {
            tris[i] = make_triangle_uv(a, b, c, ua, ub, uc);
        }
    }
    if (smooth && !normals) compute_smooth_normals(tris);
    for (uint32_t i = 0; i < count; ++i) {
        const Triangle& t = tris[i];
        SrTriangle& o = out[i];
        auto put3 = [](float* d, V3 v) { d[0] = v.x, d[1] = v.y, d[2] = v.z; };
        auto put4 = [](float* d, V4 v) { d[0] = v.x, d[1] = v.y, d[2] = v.z, d[3] = v.w; };
        put3(o.pos_a, t.lean.a);
        put3(o.ab, t.lean.ab);
        put3(o.ac, t.lean.ac);
        put3(o.norm_a, t.attr.na);
        put3(o.norm_b, t.attr.nb);
        put3(o.norm_c, t.attr.nc);
        put4(o.tan_a, t.attr.ta);
        put4(o.tan_b, t.attr.tb);
        put4(o.tan_c, t.attr.tc);
        o.uv_a[0] = t.attr.uva.x, o.uv_a[1] = t.attr.uva.y;
        o.uv_b[0] = t.attr.uvb.x, o.uv_b[1] = t.attr.uvb.y;
        o.uv_c[0] = t.attr.uvc.x, o.uv_c[1] = t.attr.uvc.y;
    }
    return SR_OK;
}

void* oracle_scene_create(void) { return new Scene(); }
void oracle_scene_destroy(void* s) { delete (Scene*)s; }

int oracle_texture_create(void* sp, const float* texels, uint32_t w, uint32_t h, int32_t filter, float tx, float ty) {
    Scene* s = (Scene*)sp;
    auto t = std::make_unique<Texture>();
    t->width = w;
    t->height = h;
    t->filter = filter;
    t->tiling = {tx, ty};
    t->texels.resize((size_t)w * h);
    for (size_t i = 0; i < (size_t)w * h; ++i) t->texels[i] = {texels[i * 3], texels[i * 3 + 1], texels[i * 3 + 2]};
    s->textures.push_back(std::move(t));
    return (int)s->textures.size() - 1;
}

int oracle_mesh_create(void* sp, const SrTriangle* tris, uint32_t count) {
    Scene* s = (Scene*)sp;
    auto m = std::make_unique<Mesh>();
    m->tris.resize(count);
    m->attrs.resize(count);
    for (uint32_t i = 0; i < count; ++i) {
        const SrTriangle& t = tris[i];
        m->tris[i] = {{t.pos_a[0], t.pos_a[1], t.pos_a[2]}, {t.ab[0], t.ab[1], t.ab[2]}, {t.ac[0], t.ac[1], t.ac[2]}};
        m->attrs[i] = {{t.norm_a[0], t.norm_a[1], t.norm_a[2]},
                       {t.norm_b[0], t.norm_b[1], t.norm_b[2]},
                       {t.norm_c[0], t.norm_c[1], t.norm_c[2]},
                       {t.tan_a[0], t.tan_a[1], t.tan_a[2], t.tan_a[3]},
                       {t.tan_b[0], t.tan_b[1], t.tan_b[2], t.tan_b[3]},
                       {t.tan_c[0], t.tan_c[1], t.tan_c[2], t.tan_c[3]},
                       {t.uv_a[0], t.uv_a[1]},
                       {t.uv_b[0], t.uv_b[1]},
                       {t.uv_c[0], t.uv_c[1]}};
    }
    const Mesh* mp = m.get();
    auto bounds_of = [mp](int i) { return mp->tris[i].bounds(); };
    BvhBuilder<decltype(bounds_of)> b((int)count, bounds_of, 1.0f, 0.5f, 8);
    m->nodes = std::move(b.nodes);
    m->items = std::move(b.items);
    m->node_count = b.node_count;
    m->bounds = m->node_count > 0 ? m->nodes[0].bounds : aabox_inverted();
    s->meshes.push_back(std::move(m));
    return (int)s->meshes.size() - 1;
}

static void export_bvh(const std::vector<BvhNode>& nodes, int node_count, const std::vector<int32_t>& items,
                       float* bounds, int32_t* links, int32_t* out_items) {
    for (int i = 0; i < node_count; ++i) {
        const BvhNode& n = nodes[i];
        float* b = bounds + (size_t)i * 6;
        b[0] = n.bounds.min.x, b[1] = n.bounds.min.y, b[2] = n.bounds.min.z;
        b[3] = n.bounds.max.x, b[4] = n.bounds.max.y, b[5] = n.bounds.max.z;
        links[i * 2] = n.child;
        links[i * 2 + 1] = n.count;
    }
    for (size_t i = 0; i < items.size(); ++i) out_items[i] = items[i];
}

void oracle_mesh_bvh_size(void* sp, int32_t mesh, uint32_t* nodes, uint32_t* items) {
    const Mesh& m = *((Scene*)sp)->meshes[mesh];
    *nodes = (uint32_t)m.node_count;
    *items = (uint32_t)m.items.size();
}
void oracle_mesh_bvh_export(void* sp, int32_t mesh, float* bounds, int32_t* links, int32_t* items) {
    const Mesh& m = *((Scene*)sp)->meshes[mesh];
    export_bvh(m.nodes, m.node_count, m.items, bounds, links, items);
}

void oracle_scene_set_sky_texture(void* sp, int32_t tex, float mult, float yaw) {
    Scene* s = (Scene*)sp;
    s->sky.init_texture(s->textures[tex].get(), mult, yaw);
    s->has_sky = true;
}
void oracle_scene_set_sky_procedural(void* sp, const SrSkyProcedural* p) {
    Scene* s = (Scene*)sp;
    s->sky.init_procedural(*p);
    s->has_sky = true;
}
void oracle_scene_set_fog(void* sp, const SrFog* f) {
    Scene* s = (Scene*)sp;
    s->has_fog = true;
    s->fog = {f->density, {f->color[0], f->color[1], f->color[2]}, f->anisotropy, f->height_falloff,
              f->height_falloff == 0.0f ? f->top_height : kInf};
}

// Object ctor scene.cs:214-225: world bounds from the rotated local bounds.
int oracle_scene_add_object(void* sp, const SrTransform* tr, const SrMaterial* m, const SrShape* sh) {
    Scene* s = (Scene*)sp;
    Object o{};
    o.trans = to_transform(*tr);
    o.mat = {{m->albedo[0], m->albedo[1], m->albedo[2]},
             m->roughness,
             m->metallic,
             m->transparency,
             m->ior,
             {m->radiance[0], m->radiance[1], m->radiance[2]},
             m->color_texture,
             m->roughness_texture,
             m->metallic_texture,
             m->normal_texture};
    o.kind = sh->kind;
    o.mesh = sh->mesh;
    AABox local;
    if (sh->kind == SR_SHAPE_MESH) {
        local = s->meshes[sh->mesh]->bounds;
    } else if (sh->kind == SR_SHAPE_SPHERE) {
        o.sphere = {{sh->params[0], sh->params[1], sh->params[2]}, sh->params[3]};
        V3 r{o.sphere.radius, o.sphere.radius, o.sphere.radius};
        local = {o.sphere.center - r, o.sphere.center + r};
    } else {
        o.box = {{sh->params[0], sh->params[1], sh->params[2]}, {sh->params[3], sh->params[4], sh->params[5]}};
        local = o.box;
    }
    // AABox.Transform -> Box(FromCenter(TransformPoint(Center), Size * Scale), Rot); Box.Bounds().
    AABox rot_local = from_center(transform_point(o.trans, box_center(local)), box_size(local) * o.trans.scale);
    V3 c = box_center(rot_local);
    V3 hh = box_size(rot_local) * 0.5f;
    V3 ax = o.trans.rot * V3{hh.x, 0, 0};
    V3 ay = o.trans.rot * V3{0, hh.y, 0};
    V3 az = o.trans.rot * V3{0, 0, hh.z};
    V3 ext{std::fabs(ax.x) + std::fabs(ay.x) + std::fabs(az.x), std::fabs(ax.y) + std::fabs(ay.y) + std::fabs(az.y),
           std::fabs(ax.z) + std::fabs(ay.z) + std::fabs(az.z)};
    o.bounds = from_center(c, ext * 2.0f);
    s->objects.push_back(o);
    return (int)s->objects.size() - 1;
}

int oracle_scene_build(void* sp) {
    Scene* s = (Scene*)sp;
    if (s->built) return SR_OK;
    if (!s->has_sky) return fail(SR_ERR_STATE, "Scene sky is required");
    s->built = true;
    const Scene* cs = s;
    auto bounds_of = [cs](int i) { return cs->objects[i].bounds; };
    BvhBuilder<decltype(bounds_of)> b((int)s->objects.size(), bounds_of, 1.0f, 10.0f, 32);
    s->nodes = std::move(b.nodes);
    s->items = std::move(b.items);
    s->node_count = b.node_count;
    return SR_OK;
}

void oracle_scene_bvh_size(void* sp, uint32_t* nodes, uint32_t* items) {
    Scene* s = (Scene*)sp;
    *nodes = (uint32_t)s->node_count;
    *items = (uint32_t)s->items.size();
}
void oracle_scene_bvh_export(void* sp, float* bounds, int32_t* links, int32_t* items) {
    Scene* s = (Scene*)sp;
    export_bvh(s->nodes, s->node_count, s->items, bounds, links, items);
}

// Closest hit per ray: object, triangle (mesh-local index), world distance, barycentric (u, v).
void oracle_scene_trace(void* sp, const float* rays, uint32_t n, int32_t* obj, int32_t* tri, float* dist, float* uv,
                        int32_t threads) {
    const Scene* s = (Scene*)sp;
    int chunks = (int)((n + 4095) / 4096);
    parallel_for(chunks, threads, [&](int c, int) {
        uint32_t b = (uint32_t)c * 4096, e = std::min<uint32_t>(n, b + 4096);
        for (uint32_t i = b; i < e; ++i) {
            const float* r = rays + (size_t)i * 6;
            Ray ray = make_ray({r[0], r[1], r[2]}, {r[3], r[4], r[5]});
            ShapeHit h;
            int o, t;
            // Re-derive the barycentrics of the accepted triangle for reporting.
            if (s->intersect(ray, &h, &o, &t, nullptr)) {
                obj[i] = o;
                tri[i] = t;
                dist[i] = h.dist;
                float u = 0, v = 0;
                if (t >= 0) {
                    const Object& ob = s->objects[o];
                    float sc;
                    Ray local = transform_ray_inv(ob.trans, ray, &sc);
                    float tt;
                    tri_intersect(s->meshes[ob.mesh]->tris[t], local, &tt, &u, &v);
                }
                uv[i * 2] = u;
                uv[i * 2 + 1] = v;
            } else {
                obj[i] = -1;
                tri[i] = -1;
                dist[i] = kInf;
                uv[i * 2] = 0;
                uv[i * 2 + 1] = 0;
            }
        }
    });
}

// Renderer: rows [y_begin, y_end) of the image on `threads` worker threads, pulling
// block_size^2 tiles from an atomic counter as RenderWorker does (renderer.cs:107-151).
int oracle_render(void* sp, const SrView* v, const SrRenderParams* p, int32_t threads, uint32_t y_begin, uint32_t y_end,
                  const SrAovs* out, uint64_t* counters) {
    const Scene* s = (Scene*)sp;
    if (!s->built) return fail(SR_ERR_STATE, "Scene not built");
    View view{to_transform(v->transform), v->fov, v->near_plane};
    float aspect = (float)p->width / (float)p->height;
    uint32_t bs = p->block_size ? p->block_size : 32;
    uint32_t bx = (p->width + bs - 1) / bs;
    uint32_t by0 = y_begin / bs, by1 = (y_end + bs - 1) / bs;
    int blocks = (int)(bx * (by1 - by0));
    int nt = threads > 0 ? threads : 1;
    std::vector<Counters> ctrs(nt);
    parallel_for(blocks, nt, [&](int blk, int t) {
        uint32_t bxi = (uint32_t)blk % bx, byi = (uint32_t)blk / bx + by0;
        uint32_t x0 = bxi * bs, y0 = std::max(byi * bs, y_begin);
        uint32_t x1 = std::min(x0 + bs, p->width), y1 = std::min(byi * bs + bs, std::min(y_end, p->height));
        for (uint32_t y = y0; y < y1; ++y)
            for (uint32_t x = x0; x < x1; ++x) render_pixel(*s, view, *p, aspect, x, y, *out, counters ? &ctrs[t] : nullptr);
    });
    if (counters) {
        for (int i = 0; i < SR_COUNTER_COUNT; ++i) {
            counters[i] = 0;
            for (auto& c : ctrs) counters[i] += c.v[i];
        }
    }
    return SR_OK;
}

// Compositor.Compose: denoise + fog blur + tonemap -> RGB8; rows in parallel (compose.cs:77-96).
void oracle_compose(const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* cp, uint8_t* rgb, int32_t threads) {
    Compositor c(*cp);
    parallel_for((int)h, threads, [&](int y, int) {
        for (int x = 0; x < (int)w; ++x) {
            Col main = c.filter(*a, (int)w, (int)h, x, y);
            Col fog = c.filter_fog(*a, (int)w, (int)h, x, y);
            c.tonemap(main + fog, rgb + ((size_t)y * w + x) * 3);
        }
    });
}

// Compositor.Preview compose.cs:57-65.
void oracle_preview(const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* cp, uint8_t* rgb) {
    Compositor c(*cp);
    for (size_t i = 0; i < (size_t)w * h; ++i)
        c.tonemap(Compositor::load3(a->radiance, i) + Compositor::load3(a->radiance_fog, i), rgb + i * 3);
}

// Filter only (float output before tonemap) for tolerance checks of the denoiser.
void oracle_denoise(const SrAovs* a, uint32_t w, uint32_t h, const SrComposeParams* cp, float* out_rgb, int32_t threads) {
    Compositor c(*cp);
    parallel_for((int)h, threads, [&](int y, int) {
        for (int x = 0; x < (int)w; ++x) {
            Col m = c.filter(*a, (int)w, (int)h, x, y) + c.filter_fog(*a, (int)w, (int)h, x, y);
            float* o = out_rgb + ((size_t)y * w + x) * 3;
            o[0] = m.r, o[1] = m.g, o[2] = m.b;
        }
    });
}

// ---- AOV dumps (program.cs:211-263) and the debug overlay (overlay.cs:54-196) ------------------------

// (byte)f as .NET 8 on x64 compiles it: cvttss2si to int (0x80000000 for NaN and out-of-range
// values), then the low byte.
static uint8_t dotnet_byte(float f) {
    int32_t i = (f >= -2147483648.0f && f < 2147483648.0f) ? (int32_t)f : INT32_MIN;
    return (uint8_t)(uint32_t)i;
}

void oracle_aov_image(const SrAovs* a, uint32_t w, uint32_t h, int32_t kind, const SrAovImageParams* p, uint8_t* rgb) {
    const uint32_t n = w * h;
    for (uint32_t i = 0; i != n; ++i) {
        uint8_t* px = rgb + 3 * (size_t)i;
        if (kind == SR_AOV_NORMAL) {
            px[0] = dotnet_byte((a->normals[3 * i] * 0.5f + 0.5f) * 255.0f);
            px[1] = dotnet_byte((a->normals[3 * i + 1] * 0.5f + 0.5f) * 255.0f);
            px[2] = dotnet_byte((a->normals[3 * i + 2] * 0.5f + 0.5f) * 255.0f);
        } else if (kind == SR_AOV_DEPTH) {
            const float depth_max_inv = 1.0f / 25.0f;
            float depth = a->depth[i];
            if (std::isinf(depth)) {
                px[0] = 255, px[1] = 0, px[2] = 0;  // Pixel.Red
            } else {
                px[0] = px[1] = px[2] = dotnet_byte(net_clamp(depth * depth_max_inv, 0.0f, 1.0f) * 255.0f);
            }
        } else if (kind == SR_AOV_VARIANCE) {
            float t = a->variance[i] / (p->variance_threshold * 2.0f);
            px[0] = px[1] = px[2] = dotnet_byte(net_clamp(t, 0.0f, 1.0f) * 255.0f);
        } else if (kind == SR_AOV_SAMPLES) {
            float log_range = std::log2(p->max_samples / (float)p->min_samples);
            float frac = std::log2(a->samples[i] / (float)p->min_samples) / log_range;
            px[0] = px[1] = px[2] = dotnet_byte(frac * 255.0f);
        } else {
            px[0] = dotnet_byte(std::fabs(std::fmod(a->uv[2 * i], 1.0f)) * 255.0f);
            px[1] = dotnet_byte(std::fabs(std::fmod(a->uv[2 * i + 1], 1.0f)) * 255.0f);
            px[2] = 0;
        }
    }
}

// View.Project math.cs:1638-1663.
static bool oracle_view_project(const SrView& v, V3 world, float aspect, float& sx, float& sy, float& depth) {
    Quat rot{v.transform.rot[0], v.transform.rot[1], v.transform.rot[2], v.transform.rot[3]};
    V3 pos{v.transform.pos[0], v.transform.pos[1], v.transform.pos[2]};
    V3 scale{v.transform.scale[0], v.transform.scale[1], v.transform.scale[2]};
    V3 local = quat_inverse(rot) * (world - pos) / scale;
    if (local.z <= v.near_plane) return false;
    float tan_half_hor, tan_half_ver;
    if (aspect >= 1.0f) {
        tan_half_hor = std::tan(v.fov * 0.5f);
        tan_half_ver = tan_half_hor / aspect;
    } else {
        tan_half_ver = std::tan(v.fov * 0.5f);
        tan_half_hor = tan_half_ver * aspect;
    }
    V3 local_from_near{local.x, local.y, local.z - v.near_plane};
    float ndc_x = (local_from_near.x / local_from_near.z) / tan_half_hor;
    float ndc_y = (local_from_near.y / local_from_near.z) / tan_half_ver;
    sx = (ndc_x + 1.0f) * 0.5f;
    sy = (1.0f - ndc_y) * 0.5f;
    depth = magnitude(local_from_near);
    return true;
}

// Vec2.RoundToInt math.cs:261 (MathF.Round is round-half-even); false when (int) would overflow.
static bool oracle_round_to_int(float v, int32_t& out) {
    float r = std::rint(v);
    if (!(r >= -2147483648.0f && r < 2147483648.0f)) return false;
    out = (int32_t)r;
    return true;
}

static void oracle_put_pixel(uint8_t* rgb, uint32_t w, uint32_t h, int32_t x, int32_t y, const uint8_t* value,
                             const float* depth, float line_depth, bool test) {
    if ((uint32_t)x >= w || (uint32_t)y >= h) return;  // Overlay.PixelIndex
    size_t index = (size_t)y * w + x;
    if (test && !(line_depth <= depth[index])) return;
    std::memcpy(rgb + 3 * index, value, 3);
}

// RasterizeLine overlay.cs:102-149.
static void oracle_rasterize_line(uint8_t* rgb, uint32_t w, uint32_t h, const float* depth, int32_t sx, int32_t sy,
                                  int32_t ex, int32_t ey, float depth_a, float depth_b, const uint8_t* value) {
    float depth_a_inv = 1.0f / depth_a;
    float depth_b_inv = 1.0f / depth_b;
    int span_x = std::abs(ex - sx);
    int span_y = -std::abs(ey - sy);
    int step_x = sx < ex ? 1 : -1;
    int step_y = sy < ey ? 1 : -1;
    int error = span_x + span_y;
    int total_steps = std::max(span_x, -span_y);
    int step = -1;
    int cx = sx, cy = sy;
    while (true) {
        ++step;
        float line_frac = total_steps > 0 ? (float)step / total_steps : 0.0f;
        float line_depth = 1.0f / (depth_a_inv * (1.0f - line_frac) + depth_b_inv * line_frac);  // float.Lerp
        oracle_put_pixel(rgb, w, h, cx, cy, value, depth, line_depth, depth != nullptr);
        if (cx == ex && cy == ey) break;
        int err2 = 2 * error;
        if (err2 >= span_y) {
            error += span_y;
            cx += step_x;
        }
        if (err2 <= span_x) {
            error += span_x;
            cy += step_y;
        }
    }
}

// RasterizeText overlay.cs:151-196.
static void oracle_rasterize_text(uint8_t* rgb, uint32_t w, uint32_t h, const char* text, int32_t x, int32_t y,
                                  int32_t align, const SrFont& font, const uint8_t* value) {
    std::vector<std::pair<size_t, size_t>> lines;  // [begin, end) ranges; at most 64
    size_t len = std::strlen(text), begin = 0;
    for (size_t i = 0; i < len && lines.size() < 63; ++i) {
        if (text[i] == '\n') {
            lines.push_back({begin, i});
            begin = i + 1;
        }
    }
    lines.push_back({begin, len});
    if (align == SR_ALIGN_CENTER) {
        int width = 0;
        for (auto& r : lines) width = std::max(width, (int)(r.second - r.first));
        x -= width * 8 / 2;
        y -= (int)lines.size() * 8 / 2;
    }
    for (size_t li = 0; li < lines.size(); ++li) {
        for (size_t i = lines[li].first; i < lines[li].second; ++i) {
            int ch = (unsigned char)text[i];
            if (ch < font.first_char || ch > font.last_char) continue;
            int glyph_base = (ch - font.first_char) * 8;
            for (int row = 0; row != 8; ++row) {
                uint8_t bits = font.glyphs[glyph_base + row];
                for (int col = 0; col != 8; ++col) {
                    if ((bits & (0x80 >> col)) == 0) continue;
                    oracle_put_pixel(rgb, w, h, x + (int)(i - lines[li].first) * 8 + col, y + (int)li * 8 + row,
                                     value, nullptr, 0.0f, false);
                }
            }
        }
    }
}

// Overlay.Draw overlay.cs:54-96: lines, then world texts, then screen texts.  Returns 1 when a line
// end point does not fit an int (where the reference's Math.Abs would throw).
int oracle_overlay_draw(uint8_t* rgb, uint32_t w, uint32_t h, const SrView* view, const float* depth,
                        const SrOverlayLine* lines, uint32_t nl, const SrOverlayText* texts, uint32_t nt,
                        const SrFont* font) {
    float aspect = (float)w / h;
    for (uint32_t i = 0; i < nl; ++i) {
        const SrOverlayLine& l = lines[i];
        float ax, ay, da, bx, by, db;
        if (!oracle_view_project(*view, {l.a[0], l.a[1], l.a[2]}, aspect, ax, ay, da)) continue;
        if (!oracle_view_project(*view, {l.b[0], l.b[1], l.b[2]}, aspect, bx, by, db)) continue;
        int32_t cax, cay, cbx, cby;
        if (!oracle_round_to_int(ax * (float)w, cax) || !oracle_round_to_int(ay * (float)h, cay) ||
            !oracle_round_to_int(bx * (float)w, cbx) || !oracle_round_to_int(by * (float)h, cby))
            return 1;
        float bias = 1.0f - l.depth_bias;
        uint8_t value[3];
        Compositor::to_pixel({l.color[0], l.color[1], l.color[2]}, value);
        oracle_rasterize_line(rgb, w, h, l.depth_test ? depth : nullptr, cax, cay, cbx, cby, da * bias, db * bias,
                              value);
    }
    for (int world = 1; world >= 0; --world) {
        for (uint32_t i = 0; i < nt; ++i) {
            const SrOverlayText& t = texts[i];
            if ((t.in_world != 0) != (world == 1)) continue;
            int32_t x = t.screen_pos[0], y = t.screen_pos[1];
            if (world) {
                float sx, sy, d;
                if (!oracle_view_project(*view, {t.world_pos[0], t.world_pos[1], t.world_pos[2]}, aspect, sx, sy, d))
                    continue;
                if (!oracle_round_to_int(sx * (float)w, x) || !oracle_round_to_int(sy * (float)h, y)) continue;
            }
            uint8_t value[3];
            Compositor::to_pixel({t.color[0], t.color[1], t.color[2]}, value);
            oracle_rasterize_text(rgb, w, h, t.text, x, y, t.align, *font, value);
        }
    }
    return 0;
}

// FP64 path-replay adjoint (see "FP64 path-replay adjoint" above): for dL/dI = d_image (h x w x 3)
// of the image I = radiance + radiance_fog, with `samples` the forward render's sample counts (the
// normalisation of each pixel), ADDS dL/d(texels of albedo texture tex_a) into grad_a (its w x h x
// 3), dL/d(red texels of roughness texture tex_r) into grad_r (w x h x 3, channel 0) and dL/d(fog
// density) into grad_f[0]; -1 / NULL skip a part.  `replay` (optional, h x w x 3) receives the
// replayed image, which equals the render's radiance + radiance_fog.  Random-number stream 0 (the
// reference's Rng(x, y)).
int oracle_adjoint(void* sp, const SrView* v, const SrRenderParams* p, int32_t threads, const float* d_image,
                   const uint32_t* samples, int32_t tex_a, double* grad_a, int32_t tex_r, double* grad_r,
                   double* grad_f, float* replay) {
    const Scene* s = (Scene*)sp;
    if (!s->built) return fail(SR_ERR_STATE, "Scene not built");
    for (const Object& o : s->objects)
        if (o.mat.transparency > 0.0f) return fail(SR_ERR_STATE, "the adjoint does not cover transparent materials");
    if (p->bounces > 16) return fail(SR_ERR_INVALID_ARG, "bounces must be <= 16");
    const int nt = threads > 0 ? threads : 1;
    const size_t na = tex_a >= 0 && grad_a ? (size_t)s->textures[tex_a]->width * s->textures[tex_a]->height * 3 : 0;
    const size_t nr = tex_r >= 0 && grad_r ? (size_t)s->textures[tex_r]->width * s->textures[tex_r]->height * 3 : 0;
    std::vector<AdjSums> sums(nt);
    for (AdjSums& a : sums) {
        a.a.assign(na, 0.0);
        a.r.assign(nr, 0.0);
    }
    View view{to_transform(v->transform), v->fov, v->near_plane};
    const float aspect = (float)p->width / (float)p->height;
    Adjoint64 adj{*s, dual(s->has_fog ? s->fog.density : 1.0f, 1.0)};
    parallel_for((int)p->height, nt, [&](int yi, int t) {
        const uint32_t y = (uint32_t)yi;
        AdjVertex64 verts[17];
        for (uint32_t x = 0; x < p->width; ++x) {
            const size_t i = (size_t)y * p->width + x;
            const uint32_t count = samples[i];
            const uint32_t taken = count < p->max_samples ? count : p->max_samples;  // the loop's off-by-one
            double G[3];
            for (int c = 0; c < 3; ++c) G[c] = (double)d_image[3 * i + c] / (double)count;
            Rng rng(x, y);
            Col rad_sum = kBlack, fog_sum = kBlack;
            for (uint32_t si = 0; si < taken; ++si) {
                // Renderer.Render's jitter (renderer.cs:167-176): x first, then y
                float jx = rng.next_float();
                float px = ((float)x + jx) / (float)p->width;
                float jy = rng.next_float();
                float py = ((float)y + jy) / (float)p->height;
                Ray ray = view.ray({px, py}, aspect);
                Col rad, fog;
                const int n = adj.replay(ray, rng, p->bounces, p->indirect_clamp, verts, rad, fog);
                rad_sum = rad_sum + rad;
                fog_sum = fog_sum + fog;
                adjoint_sweep(*s, verts, n, G, na ? tex_a : -1, nr ? tex_r : -1, sums[t]);
            }
            if (replay) {
                Col r = rad_sum / (float)count, f = fog_sum / (float)count;
                replay[3 * i] = r.r + f.r;
                replay[3 * i + 1] = r.g + f.g;
                replay[3 * i + 2] = r.b + f.b;
            }
        }
    });
    for (const AdjSums& a : sums) {
        for (size_t k = 0; k < na; ++k) grad_a[k] += a.a[k];
        for (size_t k = 0; k < nr; ++k) grad_r[k] += a.r[k];
        if (grad_f) grad_f[0] += a.f;
    }
    return SR_OK;
}

}  // extern "C"

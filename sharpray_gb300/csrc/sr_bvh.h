// sr_bvh.h — host-side geometry and the binned-SAH BVH builder.
//
// The builder reproduces bvh.cs (Bvh ctor :58-75, InsertRoot :285-298, Insert :305-317,
// SplitPick :325-395, Partition :401-426, Subdivide :432-459): the same node order (children
// stored consecutively, allocated depth-first), the same in-place item permutation, and the same
// float arithmetic, so the node arrays are bit-identical to the reference's.  Unlike the
// reference it evaluates every shape's bounds and centroid once up front instead of on every
// visit; the values are identical because they are pure functions of the shape.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

namespace sr {
namespace host {

// .NET MathF.Min/Max semantics (IEEE 754:2019 minimum/maximum: NaN propagates, -0 < +0).
inline float net_max(float x, float y) {
    if (x != y) return std::isnan(x) ? x : (y < x ? x : y);
    return std::signbit(y) ? x : y;
}
inline float net_min(float x, float y) {
    if (x != y) return std::isnan(x) ? x : (x < y ? x : y);
    return std::signbit(x) ? x : y;
}

struct F3 {
    float x, y, z;
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline F3 operator*(F3 a, F3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline F3 operator/(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline F3 operator/(F3 a, F3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline F3 operator-(F3 a) { return {-a.x, -a.y, -a.z}; }
inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float mag_sqr(F3 v) { return dot(v, v); }
inline float magnitude(F3 v) { return std::sqrt(mag_sqr(v)); }
inline F3 normalize(F3 v) { return v / magnitude(v); }
inline F3 normalize_or(F3 v, F3 fb) {
    float m = mag_sqr(v);
    return m >= 1e-12f ? v / std::sqrt(m) : fb;
}

struct Quat {
    float x, y, z, w;
};
inline F3 rotate(Quat q, F3 v) {
    F3 axis{q.x, q.y, q.z};
    float sqr = mag_sqr(axis);
    F3 a = axis * (dot(axis, v) * 2.0f);
    F3 b = v * (q.w * q.w - sqr);
    F3 c = cross(axis, v) * (q.w * 2.0f);
    return a + b + c;
}

struct Box {
    F3 lo, hi;
    static Box inverted() {
        const float m = 3.40282347e+38f;
        return {{m, m, m}, {-m, -m, -m}};
    }
    void grow(const Box& o) {
        lo = {net_min(lo.x, o.lo.x), net_min(lo.y, o.lo.y), net_min(lo.z, o.lo.z)};
        hi = {net_max(hi.x, o.hi.x), net_max(hi.y, o.hi.y), net_max(hi.z, o.hi.z)};
    }
    void grow(F3 p) {
        lo = {net_min(lo.x, p.x), net_min(lo.y, p.y), net_min(lo.z, p.z)};
        hi = {net_max(hi.x, p.x), net_max(hi.y, p.y), net_max(hi.z, p.z)};
    }
    F3 center() const { return (lo + hi) * 0.5f; }
    F3 size() const { return hi - lo; }
    float area() const {
        F3 s = size();
        return 2.0f * (s.x * s.y + s.x * s.z + s.y * s.z);
    }
    bool is_inverted() const { return lo.x > hi.x || lo.y > hi.y || lo.z > hi.z; }
};

struct BvhNodeHost {
    Box bounds;
    int32_t child;
    int32_t count;
};

struct BvhHost {
    std::vector<BvhNodeHost> nodes;  // size max(2N, 1); nodes past node_count stay zero
    std::vector<int32_t> items;
    int32_t node_count = 0;
    bool overflow = false;  // more than 2N nodes were needed (the reference throws); tree unusable
};

// Builds over `n` shapes with the given bounds.  Reference parameters: meshes use
// (traverse 1, intersect 0.5, 8 bins), the scene uses (1, 10, 32).
BvhHost build_bvh(const std::vector<Box>& shape_bounds, float cost_traverse, float cost_intersect, int bins);

// Triangle construction + optional smooth normals (the ObjLoader mesh path); see
// sr_triangles_from_corners in sharpray.h.  `out` is an array of SrTriangle.
void triangles_from_corners(const float* positions, const float* uvs, const float* normals, uint32_t count,
                            bool smooth_normals, void* out);
// Mesh.ComputeSmoothNormals mesh.cs:99-123 over `count` SrTriangles in place.
void compute_smooth_normals(void* tris, uint32_t count);
// One SrTriangle from its corners (Triangle ctors math.cs:1510-1531); `normals` NULL gives the face
// normal at every corner.
void make_triangle_corners(const float* pa, const float* pb, const float* pc, const float* normals, const float* uva,
                           const float* uvb, const float* uvc, void* out);

}  // namespace host
}  // namespace sr

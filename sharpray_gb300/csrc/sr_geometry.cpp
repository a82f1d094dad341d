// sr_geometry.cpp — host geometry: the bit-exact binned-SAH BVH builder and triangle ingest.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "../../include/sharpray.h"
#include "sr_bvh.h"

namespace sr {
namespace host {

namespace {

struct Builder {
    const std::vector<Box>& bounds;
    std::vector<F3> centers;
    float ct, ci;
    int bins;
    BvhHost out;
    // scratch for SplitPick
    std::vector<Box> bin_box;
    std::vector<int> bin_cnt;
    std::vector<float> left_area;
    std::vector<int> left_cnt;

    Builder(const std::vector<Box>& b, float ct_, float ci_, int bins_) : bounds(b), ct(ct_), ci(ci_), bins(bins_) {
        centers.resize(b.size());
        for (size_t i = 0; i < b.size(); ++i) centers[i] = b[i].center();
        bin_box.resize(bins);
        bin_cnt.resize(bins);
        left_area.resize(bins - 1);
        left_cnt.resize(bins - 1);
    }

    float leaf_cost(float area, int count) const { return ci * area * (float)count; }

    int alloc(int begin, int count) {
        int idx = out.node_count++;
        BvhNodeHost& n = out.nodes[idx];
        n.bounds = Box::inverted();
        n.child = begin;
        n.count = count;
        for (int i = 0; i < count; ++i) n.bounds.grow(bounds[out.items[begin + i]]);
        return idx;
    }

    // SplitPick bvh.cs:325-395: best (axis, position) over all bin boundaries, or false when a leaf
    // is cheaper.
    bool pick(const BvhNodeHost& node, int& axis_out, float& pos_out) {
        const int begin = node.child, count = node.count;
        Box cb = Box::inverted();
        for (int i = 0; i < count; ++i) cb.grow(centers[out.items[begin + i]]);
        const float parent_area = node.bounds.area();
        float best = leaf_cost(parent_area, count);
        int best_axis = -1;
        float best_pos = 0.0f;
        for (int axis = 0; axis < 3; ++axis) {
            const float lo = cb.lo[axis], hi = cb.hi[axis];
            if (hi - lo < 1e-6f) continue;
            std::fill(bin_box.begin(), bin_box.end(), Box::inverted());
            std::fill(bin_cnt.begin(), bin_cnt.end(), 0);
            const float scale = (float)bins / (hi - lo);
            for (int i = 0; i < count; ++i) {
                int s = out.items[begin + i];
                int bin = std::min((int)((centers[s][axis] - lo) * scale), bins - 1);
                bin_box[bin].grow(bounds[s]);
                ++bin_cnt[bin];
            }
            Box acc = Box::inverted();
            int n = 0;
            for (int b = 0; b < bins - 1; ++b) {
                acc.grow(bin_box[b]);
                n += bin_cnt[b];
                left_area[b] = acc.is_inverted() ? 0.0f : acc.area();
                left_cnt[b] = n;
            }
            acc = Box::inverted();
            n = 0;
            for (int b = bins - 1; b > 0; --b) {
                acc.grow(bin_box[b]);
                n += bin_cnt[b];
                float right_area = acc.is_inverted() ? 0.0f : acc.area();
                float cost = ct * parent_area + leaf_cost(left_area[b - 1], left_cnt[b - 1]) + leaf_cost(right_area, n);
                if (cost < best) {
                    best = cost;
                    best_axis = axis;
                    best_pos = lo + (float)b * (hi - lo) / (float)bins;
                }
            }
        }
        if (best_axis < 0) return false;
        axis_out = best_axis;
        pos_out = best_pos;
        return true;
    }

    // Partition bvh.cs:401-426 (same swap sequence).
    int partition(const BvhNodeHost& node, int axis, float split) {
        int l = node.child, r = node.child + node.count - 1;
        for (;;) {
            if (centers[out.items[l]][axis] < split) {
                if (++l > r) break;
            } else {
                if (l == r) break;
                std::swap(out.items[l], out.items[r]);
                --r;
            }
        }
        return l;
    }

    void run() {
        const int n = (int)bounds.size();
        out.nodes.assign(std::max(2 * n, 1), BvhNodeHost{{{0, 0, 0}, {0, 0, 0}}, 0, 0});
        out.items.resize(n);
        std::iota(out.items.begin(), out.items.end(), 0);
        if (n == 0) return;
        int root = alloc(0, n);
        // Depth-first worklist: popping child A before child B reproduces the recursive
        // Subdivide order, so node slots are allocated exactly as the reference allocates them.
        struct Work {
            int node, depth;
        };
        std::vector<Work> stack;
        stack.push_back({root, 0});
        while (!stack.empty()) {
            Work w = stack.back();
            stack.pop_back();
            if (w.depth >= 64) continue;
            int axis;
            float pos;
            if (!pick(out.nodes[w.node], axis, pos)) continue;
            if (out.node_count + 2 > (int)out.nodes.size()) {
                // a split whose partition sends every item to one side repeats until the depth
                // cap and can outgrow the reference's 2N node array (bvh.cs would throw)
                out.overflow = true;
                return;
            }
            int p = partition(out.nodes[w.node], axis, pos);
            BvhNodeHost& node = out.nodes[w.node];
            int count_a = p - node.child;
            int count_b = node.count - count_a;
            int begin = node.child;
            int a = alloc(begin, count_a);
            alloc(p, count_b);
            out.nodes[w.node].child = a;
            out.nodes[w.node].count = 0;
            stack.push_back({a + 1, w.depth + 1});
            stack.push_back({a, w.depth + 1});
        }
    }
};

// Triangle.ComputeTangent math.cs:1553-1579.
void tangent_of(F3 pa, F3 pb, F3 pc, const float* ua, const float* ub, const float* uc, F3 n, float* out) {
    F3 d1 = pb - pa, d2 = pc - pa;
    float u1x = ub[0] - ua[0], u1y = ub[1] - ua[1];
    float u2x = uc[0] - ua[0], u2y = uc[1] - ua[1];
    float f = u1x * u2y - u2x * u1y;
    const F3 right{1, 0, 0};
    if (std::fabs(f) < 1e-8f) {
        F3 t = normalize_or(d1 - dot(d1, n) * n, right);
        out[0] = t.x, out[1] = t.y, out[2] = t.z, out[3] = 1.0f;
        return;
    }
    float inv = 1.0f / f;
    F3 t = (u2y * d1 - u1y * d2) * inv;
    F3 b = (-u2x * d1 + u1x * d2) * inv;
    t = normalize_or(t - dot(t, n) * n, right);
    float w = dot(cross(n, t), b) < 0.0f ? -1.0f : 1.0f;
    out[0] = t.x, out[1] = t.y, out[2] = t.z, out[3] = w;
}

void put3(float* d, F3 v) { d[0] = v.x, d[1] = v.y, d[2] = v.z; }
F3 get3(const float* s) { return {s[0], s[1], s[2]}; }

// Triangle(posA, posB, posC, [normA..C,] uvA..C) math.cs:1510-1531 into an SrTriangle.
void make_triangle(F3 pa, F3 pb, F3 pc, const F3* normals, const float* uva, const float* uvb, const float* uvc,
                   SrTriangle& t) {
    const F3 up{0, 1, 0};
    F3 ab = pb - pa, ac = pc - pa;
    put3(t.pos_a, pa);
    put3(t.ab, ab);
    put3(t.ac, ac);
    F3 tan_normal;
    if (normals) {
        put3(t.norm_a, normals[0]);
        put3(t.norm_b, normals[1]);
        put3(t.norm_c, normals[2]);
        F3 geo = normalize_or(cross(pb - pa, pc - pa), up);
        tan_normal = normalize_or((normals[0] + normals[1] + normals[2]) / 3.0f, geo);
    } else {
        F3 face = normalize_or(cross(ab, ac), up);
        put3(t.norm_a, face);
        put3(t.norm_b, face);
        put3(t.norm_c, face);
        tan_normal = face;
    }
    tangent_of(pa, pb, pc, uva, uvb, uvc, tan_normal, t.tan_a);
    std::memcpy(t.tan_b, t.tan_a, sizeof(t.tan_a));
    std::memcpy(t.tan_c, t.tan_a, sizeof(t.tan_a));
    t.uv_a[0] = uva[0], t.uv_a[1] = uva[1];
    t.uv_b[0] = uvb[0], t.uv_b[1] = uvb[1];
    t.uv_c[0] = uvc[0], t.uv_c[1] = uvc[1];
}

}  // namespace

void make_triangle_corners(const float* pa, const float* pb, const float* pc, const float* normals, const float* uva,
                           const float* uvb, const float* uvc, void* out) {
    F3 ns[3];
    if (normals) ns[0] = get3(normals), ns[1] = get3(normals + 3), ns[2] = get3(normals + 6);
    make_triangle(get3(pa), get3(pb), get3(pc), normals ? ns : nullptr, uva, uvb, uvc, *(SrTriangle*)out);
}

BvhHost build_bvh(const std::vector<Box>& shape_bounds, float cost_traverse, float cost_intersect, int bins) {
    Builder b(shape_bounds, cost_traverse, cost_intersect, bins);
    b.run();
    return std::move(b.out);
}

void triangles_from_corners(const float* positions, const float* uvs, const float* normals, uint32_t count,
                            bool smooth_normals, void* out_v) {
    SrTriangle* out = (SrTriangle*)out_v;
    static const float kUvA[2] = {0, 0}, kUvB[2] = {1, 0}, kUvC[2] = {0, 1};
    for (uint32_t i = 0; i < count; ++i) {
        const float* p = positions + (size_t)i * 9;
        const float* ua = uvs ? uvs + (size_t)i * 6 : kUvA;
        const float* ub = uvs ? uvs + (size_t)i * 6 + 2 : kUvB;
        const float* uc = uvs ? uvs + (size_t)i * 6 + 4 : kUvC;
        F3 ns[3];
        if (normals) {
            const float* n = normals + (size_t)i * 9;
            ns[0] = get3(n), ns[1] = get3(n + 3), ns[2] = get3(n + 6);
        }
        make_triangle(get3(p), get3(p + 3), get3(p + 6), normals ? ns : nullptr, ua, ub, uc, out[i]);
    }
    if (!smooth_normals || normals || count == 0) return;
    compute_smooth_normals(out, count);
}

void compute_smooth_normals(void* tris_v, uint32_t count) {
    SrTriangle* out = (SrTriangle*)tris_v;
    if (count == 0) return;
    // Mesh.ComputeSmoothNormals mesh.cs:99-123.  Corner positions are grouped by the quantised key
    // of Vec3Comparer(1e-6) (math.cs:396-403); each group's area-weighted face normals are summed in
    // corner order (triangle order, then A, B, C), which is the order the reference's dictionary
    // accumulates them in.
    const F3 up{0, 1, 0};
    const float inv_eps = 1.0f / 1e-6f;
    auto quant = [inv_eps](float v) { return (int64_t)std::nearbyint(v * inv_eps); };
    const size_t corners = (size_t)count * 3;
    std::vector<int64_t> keys(corners * 3);
    std::vector<F3> weighted(count), pos(corners);
    for (uint32_t i = 0; i < count; ++i) {
        const SrTriangle& t = out[i];
        F3 a = get3(t.pos_a), ab = get3(t.ab), ac = get3(t.ac);
        F3 c = cross(ab, ac);
        weighted[i] = normalize_or(c, up) * (magnitude(c) * 0.5f);
        pos[3 * i] = a;
        pos[3 * i + 1] = a + ab;
        pos[3 * i + 2] = a + ac;
    }
    for (size_t k = 0; k < corners; ++k) {
        keys[3 * k] = quant(pos[k].x);
        keys[3 * k + 1] = quant(pos[k].y);
        keys[3 * k + 2] = quant(pos[k].z);
    }
    std::vector<uint32_t> order(corners);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t l, uint32_t r) {
        const int64_t* kl = &keys[3 * (size_t)l];
        const int64_t* kr = &keys[3 * (size_t)r];
        if (kl[0] != kr[0]) return kl[0] < kr[0];
        if (kl[1] != kr[1]) return kl[1] < kr[1];
        return kl[2] < kr[2];
    });
    std::vector<F3> vertex_normal(corners);
    for (size_t g = 0; g < corners;) {
        size_t e = g + 1;
        const int64_t* kg = &keys[3 * (size_t)order[g]];
        while (e < corners && std::memcmp(&keys[3 * (size_t)order[e]], kg, 3 * sizeof(int64_t)) == 0) ++e;
        F3 sum{0, 0, 0};
        for (size_t j = g; j < e; ++j) sum = sum + weighted[order[j] / 3];
        for (size_t j = g; j < e; ++j) vertex_normal[order[j]] = sum;
        g = e;
    }
    for (uint32_t i = 0; i < count; ++i) {
        SrTriangle& t = out[i];
        F3 face = normalize_or(cross(get3(t.ab), get3(t.ac)), up);
        F3 ns[3] = {normalize_or(vertex_normal[3 * i], face), normalize_or(vertex_normal[3 * i + 1], face),
                    normalize_or(vertex_normal[3 * i + 2], face)};
        float ua[2] = {t.uv_a[0], t.uv_a[1]}, ub[2] = {t.uv_b[0], t.uv_b[1]}, uc[2] = {t.uv_c[0], t.uv_c[1]};
        make_triangle(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], ns, ua, ub, uc, t);
    }
}

}  // namespace host
}  // namespace sr

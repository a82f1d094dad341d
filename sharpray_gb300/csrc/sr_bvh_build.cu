// sr_bvh_build.cu — the binned-SAH BVH build of bvh.cs on the device, bit-identical to the host
// build (sr_geometry.cpp) and so to the reference: same node order, same `_items` permutation,
// same bounds bits.
//
// The reference builds recursively: Subdivide (bvh.cs:432-459) picks a split with SplitPick
// (:325-395), partitions the node's item range in place (Partition :401-426) and allocates the two
// children consecutively, depth first.  Here the tree is built level by level, one CTA per node of
// the level:
//   * node bounds and centroid bounds: block reductions (min/max are order-independent, with .NET
//     MathF.Min/Max semantics for -0 and +0, via an order-preserving integer key);
//   * SplitPick: bin boxes and counts per axis in shared memory (per-warp copies, merged), then the
//     reference's two sweeps and cost comparisons in its order, by one thread;
//   * Partition: the reference's loop moves items only between its two cursors, so its result has
//     a closed form -- with p items going left: a left-going item of [0, p) stays; the k-th
//     right-going item of [0, p) (from the left) goes just below the (k-1)-th left-going item of
//     [p, n) counted from the right end (the first to n - 1); the k-th left-going item of [p, n)
//     from the right takes the place of the k-th right-going item of [0, p); a right-going item of
//     [p, n) moves down one place, except the one at p, which goes just below the last left-going
//     item of [p, n) (or to n - 1).  Block scans give the ranks.
// Node numbers follow from the finished tree: the reference allocates a node's children when it
// subdivides it, in depth-first preorder, so the q-th internal node in preorder has its children
// at 2q + 1 and 2q + 2 -- subtree sizes (bottom-up) and preorder ranks (top-down) give q.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "sr_bvh.h"
#include "sr_bvh_build.h"

namespace sr {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxBins = 32;
constexpr int kMaxDepth = 64;  // bvh.cs Subdivide: no split at depth >= 64
constexpr float kFltMax = 3.40282347e+38f;

// Order-preserving integer key of a float (no NaN): -0 sorts below +0 as MathF.Min/Max order them.
__device__ __forceinline__ int fkey(float f) {
    int b = __float_as_int(f);
    return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float kfloat(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }
__device__ __forceinline__ int kmin(int a, int b) { return a < b ? a : b; }
__device__ __forceinline__ int kmax(int a, int b) { return a > b ? a : b; }

// A node of the build, in level order (temporary numbering).
struct BuildNode {
    int lo[3], hi[3];  // bounds as keys
    int begin, count, depth;
    int child;  // temporary number of child A (B = A + 1), -1 for a leaf
    int internal;  // internal nodes in the subtree (bottom-up pass)
    int rank;      // preorder rank among internal nodes (top-down pass)
    int final_index;
};

struct BuildArgs {
    BuildNode* nodes;
    int* total;  // nodes allocated so far (temporary numbering)
    int* error;  // 1: node array overflow (as the host build), 2: a partition index out of range
    int capacity;  // node slots (2N)
    const float* bounds;   // 6 per shape: lo.xyz, hi.xyz
    const float* centers;  // 3 per shape
    int* items;
    int* tmp;
    int* rx;     // positions of right-going items of [0, p), by rank from the left
    int* ly;     // positions of left-going items of [p, n), by rank from the left
    int* rank;   // per position: rank of the item in its class
    float ct, ci;
    int bins;
};

__global__ void k_centers(const float* bounds, float* centers, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* b = bounds + 6 * (size_t)i;
    // Box.Center = (min + max) * 0.5
    centers[3 * (size_t)i] = (b[0] + b[3]) * 0.5f;
    centers[3 * (size_t)i + 1] = (b[1] + b[4]) * 0.5f;
    centers[3 * (size_t)i + 2] = (b[2] + b[5]) * 0.5f;
}

// Block scan of a 0/1 predicate over kThreads threads: returns this thread's exclusive prefix and
// sets `total`.
__device__ __forceinline__ int block_excl(bool pred, int* warp_sums, int& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned m = __ballot_sync(0xffffffffu, pred);
    if (lane == 0) warp_sums[warp] = __popc(m);
    __syncthreads();
    int before = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        int v = warp_sums[w];
        if (w < warp) before += v;
        tot += v;
    }
    __syncthreads();
    total = tot;
    return before + __popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ float box_area(const float* lo, const float* hi) {
    // AABox.SurfaceArea math.cs:948: 2 (x y + x z + y z) of the size
    float sx = hi[0] - lo[0], sy = hi[1] - lo[1], sz = hi[2] - lo[2];
    return 2.0f * (sx * sy + sx * sz + sy * sz);
}

__global__ void __launch_bounds__(kThreads) k_level(BuildArgs A, int level_begin) {
    __shared__ int s_box[12];                      // node bounds lo/hi, centroid bounds lo/hi (keys)
    __shared__ int s_bin[kWarps][3][kMaxBins][7];  // per warp: lo.xyz, hi.xyz keys, count
    __shared__ int s_warp[kWarps];
    __shared__ float s_split[2];  // axis (as float bits), position
    __shared__ int s_p;

    BuildNode& nd = A.nodes[level_begin + blockIdx.x];
    const int b = nd.begin, c = nd.count;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int* items = A.items + b;

    // ---- node bounds (alloc: grow over the items' bounds) and centroid bounds ----
    int acc[12];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        acc[j] = fkey(kFltMax), acc[3 + j] = fkey(-kFltMax);
        acc[6 + j] = fkey(kFltMax), acc[9 + j] = fkey(-kFltMax);
    }
    for (int i = tid; i < c; i += kThreads) {
        const int s = items[i];
        const float* bb = A.bounds + 6 * (size_t)s;
        const float* cc = A.centers + 3 * (size_t)s;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            acc[j] = kmin(acc[j], fkey(bb[j]));
            acc[3 + j] = kmax(acc[3 + j], fkey(bb[3 + j]));
            acc[6 + j] = kmin(acc[6 + j], fkey(cc[j]));
            acc[9 + j] = kmax(acc[9 + j], fkey(cc[j]));
        }
    }
#pragma unroll
    for (int j = 0; j < 12; ++j) {
        const bool is_min = (j % 6) < 3;
        for (int off = 16; off > 0; off >>= 1) {
            int o = __shfl_down_sync(0xffffffffu, acc[j], off);
            acc[j] = is_min ? kmin(acc[j], o) : kmax(acc[j], o);
        }
    }
    if (tid < 12) s_box[tid] = (tid % 6) < 3 ? fkey(kFltMax) : fkey(-kFltMax);
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            if ((j % 6) < 3)
                atomicMin(&s_box[j], acc[j]);
            else
                atomicMax(&s_box[j], acc[j]);
        }
    }
    __syncthreads();
    if (tid == 0) {
        for (int j = 0; j < 3; ++j) nd.lo[j] = s_box[j], nd.hi[j] = s_box[3 + j];
        nd.child = -1;
    }
    if (nd.depth >= kMaxDepth) return;

    float cl[3], ch[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) cl[j] = kfloat(s_box[6 + j]), ch[j] = kfloat(s_box[9 + j]);
    const int bins = A.bins;

    // ---- SplitPick: bin boxes and counts per axis ----
    {
        int* flat = &s_bin[0][0][0][0];
        for (int i = tid; i < kWarps * 3 * kMaxBins * 7; i += kThreads) {
            int f = i % 7;
            flat[i] = f < 3 ? fkey(kFltMax) : (f < 6 ? fkey(-kFltMax) : 0);
        }
    }
    __syncthreads();
    float scale[3];
    bool use[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        use[ax] = !(ch[ax] - cl[ax] < 1e-6f);
        scale[ax] = use[ax] ? (float)bins / (ch[ax] - cl[ax]) : 0.0f;
    }
    for (int i = tid; i < c; i += kThreads) {
        const int s = items[i];
        const float* bb = A.bounds + 6 * (size_t)s;
        const float* cc = A.centers + 3 * (size_t)s;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            if (!use[ax]) continue;
            int bin = (int)((cc[ax] - cl[ax]) * scale[ax]);
            bin = bin < bins - 1 ? bin : bins - 1;
            int* e = s_bin[warp][ax][bin];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                atomicMin(&e[j], fkey(bb[j]));
                atomicMax(&e[3 + j], fkey(bb[3 + j]));
            }
            atomicAdd(&e[6], 1);
        }
    }
    __syncthreads();
    // merge the warp copies into copy 0
    for (int i = tid; i < 3 * kMaxBins * 7; i += kThreads) {
        int ax = i / (kMaxBins * 7), rem = i % (kMaxBins * 7), bin = rem / 7, f = rem % 7;
        int v = s_bin[0][ax][bin][f];
        for (int w = 1; w < kWarps; ++w) {
            int o = s_bin[w][ax][bin][f];
            v = f < 3 ? kmin(v, o) : (f < 6 ? kmax(v, o) : v + o);
        }
        s_bin[0][ax][bin][f] = v;
    }
    __syncthreads();
    if (tid == 0) {
        float nlo[3], nhi[3];
        for (int j = 0; j < 3; ++j) nlo[j] = kfloat(nd.lo[j]), nhi[j] = kfloat(nd.hi[j]);
        const float parent_area = box_area(nlo, nhi);
        float best = A.ci * parent_area * (float)c;  // leaf cost
        int best_axis = -1;
        float best_pos = 0.0f;
        float left_area[kMaxBins];
        int left_cnt[kMaxBins];
        for (int ax = 0; ax < 3; ++ax) {
            if (!use[ax]) continue;
            const float lo = cl[ax], hi = ch[ax];
            int blo[3], bhi[3];
            for (int j = 0; j < 3; ++j) blo[j] = fkey(kFltMax), bhi[j] = fkey(-kFltMax);
            int n = 0;
            for (int bn = 0; bn < bins - 1; ++bn) {
                const int* e = s_bin[0][ax][bn];
                for (int j = 0; j < 3; ++j) blo[j] = kmin(blo[j], e[j]), bhi[j] = kmax(bhi[j], e[3 + j]);
                n += e[6];
                float lo3[3], hi3[3];
                bool inv = false;
                for (int j = 0; j < 3; ++j) {
                    lo3[j] = kfloat(blo[j]), hi3[j] = kfloat(bhi[j]);
                    inv = inv || lo3[j] > hi3[j];
                }
                left_area[bn] = inv ? 0.0f : box_area(lo3, hi3);
                left_cnt[bn] = n;
            }
            for (int j = 0; j < 3; ++j) blo[j] = fkey(kFltMax), bhi[j] = fkey(-kFltMax);
            n = 0;
            for (int bn = bins - 1; bn > 0; --bn) {
                const int* e = s_bin[0][ax][bn];
                for (int j = 0; j < 3; ++j) blo[j] = kmin(blo[j], e[j]), bhi[j] = kmax(bhi[j], e[3 + j]);
                n += e[6];
                float lo3[3], hi3[3];
                bool inv = false;
                for (int j = 0; j < 3; ++j) {
                    lo3[j] = kfloat(blo[j]), hi3[j] = kfloat(bhi[j]);
                    inv = inv || lo3[j] > hi3[j];
                }
                const float right_area = inv ? 0.0f : box_area(lo3, hi3);
                const float cost = A.ct * parent_area + A.ci * left_area[bn - 1] * (float)left_cnt[bn - 1] +
                                   A.ci * right_area * (float)n;
                if (cost < best) {
                    best = cost;
                    best_axis = ax;
                    best_pos = lo + (float)bn * (hi - lo) / (float)bins;
                }
            }
        }
        s_split[0] = __int_as_float(best_axis);
        s_split[1] = best_pos;
    }
    __syncthreads();
    const int axis = __float_as_int(s_split[0]);
    if (axis < 0) return;
    const float pos = s_split[1];
    // the two children need slots; past 2N the build stops as the host build does
    if (tid == 0) s_p = atomicAdd(A.total, 2);
    __syncthreads();
    const int ch0 = s_p;
    if (ch0 + 2 > A.capacity) {
        if (tid == 0) atomicOr(A.error, 1);
        return;
    }
    __syncthreads();

    // ---- Partition: p, then ranks, then destinations ----
    int nl = 0;
    for (int i = tid; i < c; i += kThreads) nl += A.centers[3 * (size_t)items[i] + axis] < pos ? 1 : 0;
    for (int off = 16; off > 0; off >>= 1) nl += __shfl_down_sync(0xffffffffu, nl, off);
    if (tid == 0) s_p = 0;
    __syncthreads();
    if (lane == 0) atomicAdd(&s_p, nl);
    __syncthreads();
    const int p = s_p;
    int carry_r = 0, carry_l = 0;
    int* rx = A.rx + b;
    int* ly = A.ly + b;
    int* rk = A.rank + b;
    for (int base = 0; base < c; base += kThreads) {
        const int i = base + tid;
        const bool valid = i < c;
        const bool left = valid && A.centers[3 * (size_t)items[i] + axis] < pos;
        const bool r_left = valid && i < p && !left;  // right-going item of [0, p)
        const bool l_right = valid && i >= p && left;  // left-going item of [p, n)
        int tr, tl;
        const int er = block_excl(r_left, s_warp, tr);
        const int el = block_excl(l_right, s_warp, tl);
        if (r_left) {
            rx[carry_r + er] = i;
            rk[i] = carry_r + er;
        }
        if (l_right) {
            ly[carry_l + el] = i;
            rk[i] = carry_l + el;
        }
        carry_r += tr;
        carry_l += tl;
    }
    const int K = carry_l;  // = carry_r
    __syncthreads();                       // the rank arrays are complete
    const int last_l = K > 0 ? ly[0] : c;  // lowest left-going position of [p, n)
    for (int i = tid; i < c; i += kThreads) {
        const bool left = A.centers[3 * (size_t)items[i] + axis] < pos;
        int dest;
        if (i < p) {
            if (left) {
                dest = i;
            } else {
                const int k = rk[i];                   // k-th right-going of [0, p)
                dest = k == 0 ? c - 1 : ly[K - k] - 1;  // below the (k-1)-th left-going of [p, n) from the right
            }
        } else if (left) {
            dest = rx[K - 1 - rk[i]];  // rank from the right
        } else {
            dest = i == p ? last_l - 1 : i - 1;
        }
        if (dest < 0 || dest >= c) {  // cannot happen for a consistent rank pass; checked, not written
            atomicOr(A.error, 2);
            continue;
        }
        A.tmp[b + dest] = items[i];
    }
    __syncthreads();
    for (int i = tid; i < c; i += kThreads) A.items[b + i] = A.tmp[b + i];
    if (tid == 0) {
        BuildNode& na = A.nodes[ch0];
        BuildNode& nb = A.nodes[ch0 + 1];
        na.begin = b, na.count = p, na.depth = nd.depth + 1;
        nb.begin = b + p, nb.count = c - p, nb.depth = nd.depth + 1;
        nd.child = ch0;
    }
}

// Internal nodes per subtree, deepest level first.
__global__ void k_subtree(BuildNode* nodes, int begin, int count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    BuildNode& n = nodes[begin + i];
    n.internal = n.child < 0 ? 0 : 1 + nodes[n.child].internal + nodes[n.child + 1].internal;
}

// Preorder ranks and final numbers, top level first.
__global__ void k_number(BuildNode* nodes, int begin, int count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    BuildNode& n = nodes[begin + i];
    if (n.child < 0) return;
    BuildNode& a = nodes[n.child];
    BuildNode& b = nodes[n.child + 1];
    a.rank = n.rank + 1;
    b.rank = n.rank + 1 + a.internal;
    a.final_index = 2 * n.rank + 1;
    b.final_index = 2 * n.rank + 2;
}

// Nodes in the reference's layout: {min.xyz, max.xyz, child, count}.
__global__ void k_emit(const BuildNode* nodes, int count, host::BvhNodeHost* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const BuildNode& n = nodes[i];
    host::BvhNodeHost o;
    o.bounds.lo = {kfloat(n.lo[0]), kfloat(n.lo[1]), kfloat(n.lo[2])};
    o.bounds.hi = {kfloat(n.hi[0]), kfloat(n.hi[1]), kfloat(n.hi[2])};
    o.child = n.child < 0 ? n.begin : nodes[n.child].final_index;
    o.count = n.child < 0 ? n.count : 0;
    out[n.final_index] = o;
}

template <typename T>
struct DevArray {
    T* p = nullptr;
    ~DevArray() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, (n ? n : 1) * sizeof(T)); }
};

#define SR_TRY(x)                               \
    do {                                        \
        cudaError_t e_ = (x);                   \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)

}  // namespace

cudaError_t build_bvh_device(const std::vector<host::Box>& shape_bounds, float cost_traverse, float cost_intersect,
                             int bins, cudaStream_t st, host::BvhHost& out) {
    using host::BvhHost;
    const int n = (int)shape_bounds.size();
    out = BvhHost{};
    out.nodes.assign(n > 0 ? 2 * (size_t)n : 1, host::BvhNodeHost{{{0, 0, 0}, {0, 0, 0}}, 0, 0});
    out.items.resize(n);
    if (n == 0) return cudaSuccess;
    if (bins < 2 || bins > kMaxBins) return cudaErrorInvalidValue;
    static_assert(sizeof(host::Box) == 24 && sizeof(host::BvhNodeHost) == 32, "host layouts");

    DevArray<float> d_bounds, d_centers;
    DevArray<int> d_items, d_tmp, d_rx, d_ly, d_rank, d_total;
    DevArray<BuildNode> d_nodes;
    DevArray<host::BvhNodeHost> d_out;
    SR_TRY(d_bounds.alloc(6 * (size_t)n));
    SR_TRY(d_centers.alloc(3 * (size_t)n));
    SR_TRY(d_items.alloc(n));
    SR_TRY(d_tmp.alloc(n));
    SR_TRY(d_rx.alloc(n));
    SR_TRY(d_ly.alloc(n));
    SR_TRY(d_rank.alloc(n));
    SR_TRY(d_total.alloc(2));  // [0] nodes allocated, [1] error word
    SR_TRY(d_nodes.alloc(2 * (size_t)n));
    SR_TRY(d_out.alloc(2 * (size_t)n));
    SR_TRY(cudaMemcpyAsync(d_bounds.p, shape_bounds.data(), 6 * sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, st));
    std::vector<int> iota(n);
    for (int i = 0; i < n; ++i) iota[i] = i;
    SR_TRY(cudaMemcpyAsync(d_items.p, iota.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st));
    k_centers<<<(n + 255) / 256, 256, 0, st>>>(d_bounds.p, d_centers.p, n);
    BuildNode root{};
    root.begin = 0, root.count = n, root.depth = 0, root.child = -1, root.rank = 0, root.final_index = 0;
    SR_TRY(cudaMemcpyAsync(d_nodes.p, &root, sizeof(root), cudaMemcpyHostToDevice, st));
    const int init[2] = {1, 0};
    SR_TRY(cudaMemcpyAsync(d_total.p, init, sizeof(init), cudaMemcpyHostToDevice, st));

    BuildArgs A{d_nodes.p, d_total.p, d_total.p + 1, 2 * n, d_bounds.p, d_centers.p, d_items.p, d_tmp.p, d_rx.p, d_ly.p,
                d_rank.p, cost_traverse, cost_intersect, bins};
    std::vector<std::pair<int, int>> levels;  // [begin, count) of each level
    int begin = 0, count = 1;
    while (count > 0) {
        levels.push_back({begin, count});
        k_level<<<count, kThreads, 0, st>>>(A, begin);
        SR_TRY(cudaGetLastError());
        int state[2] = {0, 0};
        SR_TRY(cudaMemcpyAsync(state, d_total.p, sizeof(state), cudaMemcpyDeviceToHost, st));
        SR_TRY(cudaStreamSynchronize(st));
        if (state[1]) {
            out.overflow = true;
            return state[1] & 2 ? cudaErrorIllegalState : cudaSuccess;
        }
        begin += count;
        count = state[0] - begin;
    }
    const int node_count = begin;
    for (size_t l = levels.size(); l-- > 0;)
        k_subtree<<<(levels[l].second + 255) / 256, 256, 0, st>>>(d_nodes.p, levels[l].first, levels[l].second);
    for (size_t l = 0; l < levels.size(); ++l)
        k_number<<<(levels[l].second + 255) / 256, 256, 0, st>>>(d_nodes.p, levels[l].first, levels[l].second);
    k_emit<<<(node_count + 255) / 256, 256, 0, st>>>(d_nodes.p, node_count, d_out.p);
    SR_TRY(cudaGetLastError());
    SR_TRY(cudaMemcpyAsync(out.nodes.data(), d_out.p, sizeof(host::BvhNodeHost) * (size_t)node_count,
                           cudaMemcpyDeviceToHost, st));
    SR_TRY(cudaMemcpyAsync(out.items.data(), d_items.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st));
    SR_TRY(cudaStreamSynchronize(st));
    out.node_count = node_count;
    return cudaSuccess;
}

}  // namespace sr

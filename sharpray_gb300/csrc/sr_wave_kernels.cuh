// sr_wave_kernels.cuh — device code of the wavefront renderer: path-state records and queues, the
// persistent traversal loop, the shade / finalize / tail kernel templates.  Included by
// sr_wavefront.cu (the render's kernels and launchers) and sr_wave_adjoint.cu (the same kernels
// recording path vertices for the adjoint); each instantiates what it launches.
#pragma once

#include <cuda_runtime.h>

#include "sr_adjoint.cuh"
#include "sr_path.cuh"
#include "sr_wavefront.h"

namespace sr {

// path flags (Rec path.b.w)
enum : uint32_t {
    PF_SPDF = 1u,      // the last scatter has a pdf (MIS on a later sky hit)
    PF_MEDIUM = 2u,    // inside a refractive medium
    PF_PRIMARY = 4u,   // the sample's primary hit is recorded in `prim`
    PF_NEE = 8u,       // a traced shadow ray's contribution is pending
    PF_NEE_FOG = 16u,  // ... and it goes to the fog radiance (primary-segment fog scatter)
};
// segment events (queue index)
enum : int { EV_FOG = 0, EV_MISS = 1, EV_SURF = 2 };
// Event selector of a shade kernel that shades both fog-scatter and miss events in one launch
// (warps padded between the two queues so that each warp runs one event's logic).
constexpr int EV_FOG_MISS = 3;

// Sectors of a slot's path record (WaveState::rec, six per slot, 192 bytes on 64-byte boundaries:
// {ray, hit}, {path, rng} and the shadow request each fill one 64-byte DRAM burst) and of its pixel
// record (WaveState::pix, four per slot).
enum : int { R_RAY = 0, R_HIT = 1, R_PATH = 2, R_RNG = 3, R_SH0 = 4, R_SH1 = 5 };
enum : int { X_PRIM = 0, X_ACC = 1 };
__device__ __forceinline__ size_t rix(const WaveState& W, uint32_t s, int k) {
    return SR_REC_SOA ? (size_t)k * W.rec_stride + s : 6 * (size_t)s + k;
}
__device__ __forceinline__ size_t pix(const WaveState& W, uint32_t s, int k) {
    return SR_REC_SOA ? (size_t)k * W.rec_stride + s : 4 * (size_t)s + k;
}

// Tag of a slot whose event `ev` is shaded by the bounce of parity `parity` (0: none); `wait`: the
// event is decided by that bounce's traversal kernel or the path's shadow ray is traced there, so
// it is shaded after that kernel (else it is ready at the bounce's start).
__device__ __forceinline__ uint8_t event_mark(int ev, int parity, int wait) {
    return (uint8_t)(1 + ev + 3 * parity + 6 * wait);
}

// Record loads and stores (one place to change how path state is moved).
__device__ __forceinline__ Rec ld_rec(const Rec* p) { return *p; }
__device__ __forceinline__ void st_rec(Rec* p, const Rec& v) { *p = v; }
__device__ __forceinline__ void st4(float4* p, float4 v) { *p = v; }

__device__ __forceinline__ uint32_t ibits(float f) { return (uint32_t)__float_as_int(f); }
__device__ __forceinline__ float fbits(uint32_t u) { return __int_as_float((int)u); }

// Pixel of tile-order index p: pixels are numbered in 8x4 tiles, so that the 32 slots of a warp
// start on neighbouring pixels (slot s starts on pixel s).
__device__ __forceinline__ void pixel_xy(const WaveState& W, uint32_t p, uint32_t& x, uint32_t& y) {
    uint32_t tile = p >> 5, lane = p & 31u;
    x = (tile % W.tiles_x) * 8u + (lane & 7u);
    y = (tile / W.tiles_x) * 4u + (lane >> 3);
}
// The first pixel of a slot (every slot's pixel when there is one slot per pixel).
__device__ __forceinline__ void slot_pixel(const WaveState& W, uint32_t slot, uint32_t& x, uint32_t& y) {
    pixel_xy(W, slot, x, y);
}
// The next unclaimed pixel inside the image for a slot of a render with fewer slots than pixels
// (~0u: none left).
__device__ __forceinline__ uint32_t claim_pixel(const WaveState& W, const DevParams& P) {
    const uint32_t end = W.pixel_tiles * 32u;
    for (;;) {
        const uint32_t p = atomicAdd(W.pixel_cursor, 1u);
        if (p >= end) return ~0u;
        uint32_t x, y;
        pixel_xy(W, p, x, y);
        if (x < P.width && y < P.height) return p;
    }
}

// Appends of one grid-stride round to NQ queues (value to queue i where pred[i] holds), aggregated
// per block: one atomic per queue and block.  The queue lengths are single words that every block
// appends to; their atomics serialise in L2, so per-warp appends made them a bottleneck.  All
// threads of the 128-thread block call it in block-uniform control flow, passing shared scratch
// sh[2][NQ][5] and the round's parity (the scratch alternates so a round needs two barriers).
constexpr int kBlockWarps = 4;
template <int NQ>
__device__ __forceinline__ void block_offsets(uint32_t* const (&count)[NQ], const bool (&pred)[NQ],
                                              uint32_t (*sh)[NQ][kBlockWarps + 1], uint32_t round,
                                              uint32_t (&off)[NQ]) {
    uint32_t(&b)[NQ][kBlockWarps + 1] = sh[round & 1u];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned mask[NQ];
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        mask[i] = __ballot_sync(0xffffffffu, pred[i]);
        if (lane == 0) b[i][warp] = (uint32_t)__popc(mask[i]);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        if (threadIdx.x == (unsigned)i) {
            uint32_t tot = b[i][0] + b[i][1] + b[i][2] + b[i][3];
            b[i][kBlockWarps] = tot ? atomicAdd(count[i], tot) : 0u;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        uint32_t o = b[i][kBlockWarps];
        for (int w = 0; w < warp; ++w) o += b[i][w];
        off[i] = o + (uint32_t)__popc(mask[i] & ((1u << lane) - 1u));
    }
}
// block_offsets, then `value` written to queue i where pred[i] holds.
template <int NQ>
__device__ __forceinline__ void push_block(uint32_t* const (&q)[NQ], uint32_t* const (&count)[NQ], uint32_t value,
                                           const bool (&pred)[NQ], uint32_t (*sh)[NQ][kBlockWarps + 1],
                                           uint32_t round) {
    uint32_t off[NQ];
    block_offsets<NQ>(count, pred, sh, round, off);
#pragma unroll
    for (int i = 0; i < NQ; ++i)
        if (pred[i]) q[i][off[i]] = value;
}

// Ray-queue entries carry the ray itself (origin + slot, direction + the path ray's fog scatter
// distance), so that a traversal kernel starts a ray with one coalesced load instead of a queue
// load followed by a scattered record load.
__device__ __forceinline__ Rec ray_entry(uint32_t slot, V3 o, V3 d, float fog_t) {
    return {make_float4(o.x, o.y, o.z, __int_as_float((int)slot)), make_float4(d.x, d.y, d.z, fog_t)};
}

__device__ __forceinline__ Rng rng_of(const Rec& g) {
    return {ibits(g.a.x), ibits(g.a.y), ibits(g.a.z), ibits(g.a.w), ibits(g.b.x)};
}
__device__ __forceinline__ Rec rng_rec(const Rng& r, Col fog) {
    return {make_float4(fbits(r.s0), fbits(r.s1), fbits(r.s2), fbits(r.s3)), make_float4(fbits(r.s4), fog.r, fog.g, fog.b)};
}

// The fog free-flight draw of a path ray (Fog.ScatterDistance scene.cs:478-496 without its end
// test): the scatter distance, or +inf when the ray cannot scatter (or the scene has no fog, in
// which case nothing is drawn).  The segment scatters when this is nearer than its closest hit.
__device__ __forceinline__ float fog_scatter_t(const DevScene& S, const Ray& ray, Rng& rng) {
    const float inf = __int_as_float(0x7f800000);
    float t = inf;
    if (S.has_fog && !fog_scatter_distance(S, ray, inf, rng, t)) t = inf;
    return t;
}

// Start of a sample: the camera ray and a reset path (scene.cs:633-638).
// `flags`: the path flags a sample starts with (an adjoint pass that keeps every sample's vertices
// puts the sample index there).
__device__ __forceinline__ void begin_sample(const WaveState& W, uint32_t s, const Ray& ray, const Rng& rng,
                                             float sdist = 0.f, uint32_t flags = 0u) {
    st_rec(&W.rec[rix(W, s, R_RAY)], Rec{make_float4(ray.o.x, ray.o.y, ray.o.z, fbits(0u)), make_float4(ray.d.x, ray.d.y, ray.d.z, sdist)});
    st_rec(&W.rec[rix(W, s, R_PATH)], Rec{make_float4(0.f, 0.f, 0.f, 0.f), make_float4(1.f, 1.f, 1.f, fbits(flags))});
    st_rec(&W.rec[rix(W, s, R_RNG)], rng_rec(rng, black()));
}

// The event of a segment whose closest hit is known (scene.cs:654-738 decides in this order):
// with fog set, the free-flight distance is drawn first -- the segment's first RNG draw -- and wins
// if it is shorter than the hit; else a hit is a surface event and no hit a miss.
__device__ __forceinline__ int segment_event(float fog_t, bool has_hit, float hit_dist) {
    if (fog_t < (has_hit ? hit_dist : __int_as_float(0x7f800000))) return EV_FOG;
    return has_hit ? EV_SURF : EV_MISS;
}

// A new path ray (scatter or camera ray) with fog scatter distance fog_t: -1 when it needs the
// next trace kernel's traversal; when it misses both root children of the scene BVH -- the first
// thing the traversal tests -- it has no hit, and its segment's event is returned.
template <bool COUNT>
__device__ __forceinline__ int next_segment(const DevScene& S, const Ray& ray, float fog_t, Ctr& c) {
    if (!misses_scene<COUNT, false>(S, ray, c)) return -1;
    SR_COUNT(c, SR_COUNTER_SCENE_TRACE, 1);
    return segment_event(fog_t, false, 0.f);
}

// Per-warp staging of the persistent loop's appends to NQ queues: entries collect in a shared
// ring of 64 per queue and go out 32 at a time (one atomic and one coalesced write per 32
// entries).  All 32 lanes call add() and flush() together.
template <int NQ>
struct WarpStage {
    uint32_t* buf;  // this warp's [NQ][64] shared ring
    uint32_t head[NQ], cnt[NQ];

    __device__ __forceinline__ void init(uint32_t* ring) {
        buf = ring;
#pragma unroll
        for (int k = 0; k < NQ; ++k) head[k] = cnt[k] = 0;
    }
    // value goes to queue `which` (-1: nothing)
    __device__ __forceinline__ void add(uint32_t* const (&q)[NQ], uint32_t* const (&count)[NQ], uint32_t value,
                                        int which) {
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
            unsigned m = __ballot_sync(0xffffffffu, which == k);
            if (!m) continue;
            if (which == k) buf[k * 64 + ((head[k] + cnt[k] + (uint32_t)__popc(m & ((1u << lane) - 1u))) & 63u)] = value;
            cnt[k] += (uint32_t)__popc(m);
            if (cnt[k] >= 32u) {
                __syncwarp();
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(count[k], 32u);
                base = __shfl_sync(0xffffffffu, base, 0);
                q[k][base + lane] = buf[k * 64 + ((head[k] + lane) & 63u)];
                __syncwarp();
                head[k] = (head[k] + 32u) & 63u;
                cnt[k] -= 32u;
            }
        }
    }
    __device__ __forceinline__ void flush(uint32_t* const (&q)[NQ], uint32_t* const (&count)[NQ]) {
        const int lane = threadIdx.x & 31;
        __syncwarp();
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
            if (!cnt[k]) continue;
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(count[k], cnt[k]);
            base = __shfl_sync(0xffffffffu, base, 0);
            if ((uint32_t)lane < cnt[k]) q[k][base + lane] = buf[k * 64 + ((head[k] + lane) & 63u)];
            cnt[k] = 0;
        }
    }
};

// A warp refills its idle lanes once at least this many are idle (or all are).
#ifndef SR_REFILL
#define SR_REFILL 8
#endif
constexpr int kRefill = SR_REFILL;
// Minimum resident blocks per SM requested for the traversal kernels (caps their registers).
#ifndef SR_TRACE_MIN_BLOCKS
#define SR_TRACE_MIN_BLOCKS 7
#endif
// Node phase of the persistent loop: at most SR_NODE_BURST node visits per round, ended early
// once SR_LEAF_WAIT lanes wait for a leaf action (triangles, entering or leaving an object) or
// are done.  1 / 1 runs one action of each lane per round.
#ifndef SR_NODE_BURST
#define SR_NODE_BURST 8
#endif
#ifndef SR_LEAF_WAIT
#define SR_LEAF_WAIT 16
#endif
// The node burst takes one warp vote per node visit (1) or two (0: any lane with node work, then
// the lanes waiting for a leaf action); both make the same decisions.
#ifndef SR_BURST_ONE_VOTE
#define SR_BURST_ONE_VOTE 1
#endif
// Shading runs as one kernel per event (SR_SPLIT_SHADE = 1): fog scatter, the most frequent
// event in foggy scenes, then needs far fewer registers than surface shading and runs at higher
// occupancy.  Minimum resident blocks per SM requested for each (caps their registers).
#ifndef SR_SPLIT_SHADE
#define SR_SPLIT_SHADE 1
#endif
#ifndef SR_SHADE_MIN_BLOCKS
#define SR_SHADE_MIN_BLOCKS 5
#endif
#ifndef SR_SHADE_FOG_MIN_BLOCKS
#define SR_SHADE_FOG_MIN_BLOCKS 8
#endif
constexpr int shade_min_blocks(int ev) {
    return ev == EV_FOG || ev == EV_MISS || ev == EV_FOG_MISS ? SR_SHADE_FOG_MIN_BLOCKS : SR_SHADE_MIN_BLOCKS;
}
constexpr int kNodeBurst = SR_NODE_BURST;
// Order in which the persistent loop takes queries (bit 2: occlusion queue first; bits 0 / 1:
// closest-hit / occlusion queue from its end).  A bounce's traversal kernel ends with a ramp-down
// in which SMs run out of queries while a few long ones finish, so the order matters: the default
// 5 takes the shadow rays first, then the path rays from the end of their queue (camera rays and
// surface bounces first, fog scatters last) -- measured 2 % faster than queue order on C2.
#ifndef SR_TRACE_ORDER
#define SR_TRACE_ORDER 5
#endif
constexpr int kLeafWait = SR_LEAF_WAIT;
// Traversal stack entries per lane kept in shared memory (0: the whole stack in local memory).
// Shared words are laid out so that a warp's stack accesses never conflict; each entry costs
// 12 bytes per thread, 1.5 KB per block.  Measured on the 1080p fog workload: 8 or 16 entries
// within -0.7 % of none (the traversal is not bound by its stack accesses).
#ifndef SR_SMEM_STACK
#define SR_SMEM_STACK 0
#endif

// Persistent ray loop: lanes take entries [fetch counter) of the concatenation of two ray queues
// -- q0 closest-hit queries, q1 occlusion queries -- until both are exhausted; `start(any)` is
// called as a query begins, `finish(slot, tag, any, hit, ray)` (tag: the bits of the entry's fog
// scatter distance) stores its answer and returns an output code that `emit(slot, code)` (all
// lanes together, -1 = none) passes on.
// Each round runs the node visits of all lanes together (up to kNodeBurst), then one leaf action
// of each lane that waits for one: leaf actions are long and differ between lanes, so batching
// them keeps warps from running each one with a single lane.  Finished lanes are answered in a
// batch when the warp refills.  Every lane's own sequence of actions is unchanged, so results are
// those of a plain loop over SceneQuery::step.
// Closest-hit queries that are still running SR_DEFER_ROUNDS rounds after the queues ran out are
// set aside -- their complete state (SceneQuery::save and the used stack entries) goes to a defer
// buffer -- and the next bounce's traversal kernel resumes them before anything else, so that a
// launch ends soon after its queues do instead of waiting for its longest queries while most SMs
// idle.  A query's own sequence of actions is unchanged, so results are too; the path is shaded
// one or more bounces later.  Occlusion queries are never set aside (their answer is needed by
// this bounce's shading).  0: no deferral.  Measured on the 1080p fog workload (images identical):
// 16 rounds +1.6 % and 4 rounds -7 % with the events shaded in one phase; 16 rounds -2 % with split
// phases (SR_SPLIT_PHASES), whose ready phase already fills the ramp-down that deferral shortens.
#ifndef SR_DEFER_ROUNDS
#define SR_DEFER_ROUNDS 0
#endif
// A deferred query's record: slot, fog tag and the query's words, then its stack entries.
constexpr int kDeferHeadF4 = 10;  // 2 + SceneQuery::kQueryWords words, rounded up to float4s
constexpr int kDeferF4 = kDeferHeadF4 + (3 * kSceneStack + 3) / 4;
static_assert(kDeferF4 * sizeof(float4) == kDeferBytes, "host and device sizes of a defer record differ");

template <bool COUNT, bool GENERAL, typename Start, typename Finish, typename Emit>
__device__ __forceinline__ void persistent_queries(const DevScene& S, const Rec* q0, uint32_t n0, const Rec* q1,
                                                   uint32_t n1, uint32_t* fetch, Ctr& c, uint32_t* err, Start start,
                                                   Finish finish, Emit emit, const float4* din = nullptr,
                                                   uint32_t nd = 0, float4* dout = nullptr, uint32_t* dcount = nullptr,
                                                   uint32_t dcap = 0) {
#if SR_SMEM_STACK > 0
    // the first SR_SMEM_STACK entries of every lane's stack in shared memory, the rest local
    constexpr int kTraceBlock = 128;  // threads per block of the traversal kernel
    __shared__ uint32_t stack_words[SR_SMEM_STACK * 3 * kTraceBlock];
    StackEntry entries[kSceneStack - SR_SMEM_STACK];
    SplitStack<SR_SMEM_STACK, kTraceBlock> stack{stack_words + threadIdx.x, entries};
#else
    StackEntry entries[kSceneStack];
    LocalStack stack{entries};
#endif
    SceneQuery<false, GENERAL, true> sq;
    static_assert(2 + decltype(sq)::kQueryWords <= 4 * kDeferHeadF4, "defer record header");
    const uint32_t n = nd + n0 + n1;  // deferred queries first, then the two queues
    bool busy = false, pending = false, exhausted = false;
    uint32_t slot = 0, tag = 0;
    const int lane = threadIdx.x & 31;
    [[maybe_unused]] uint32_t rounds_after = 0;  // rounds since this warp found the queues empty
    for (;;) {
        unsigned idle = __ballot_sync(0xffffffffu, !busy);
        int nidle = __popc(idle);
        if (nidle >= kRefill || (exhausted && idle == 0xffffffffu)) {
            int code = -1;
            if (pending) {
                code = finish(slot, tag, sq.any_hit, sq.best, sq.wr);
                pending = false;
            }
            emit(slot, code);
        }
        if (!exhausted && nidle >= kRefill) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, (uint32_t)nidle);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + (uint32_t)nidle >= n) exhausted = true;
            if (!busy) {
                uint32_t idx = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (idx < nd) {  // a query set aside by the last launch: resumed where it stopped
                    const float4* r = din + (size_t)idx * kDeferF4;
                    const uint32_t* w = reinterpret_cast<const uint32_t*>(r);
                    slot = w[0];
                    tag = w[1];
                    sq.load(w + 2);
                    const uint32_t* se = reinterpret_cast<const uint32_t*>(r + kDeferHeadF4);
                    for (int i = 0; i < sq.sp; ++i)
                        stack.set(i, StackEntry{(int)se[3 * i], (int)se[3 * i + 1], __uint_as_float(se[3 * i + 2])});
                    busy = true;
                } else if (idx < n) {
                    idx -= nd;
                    // fetch order: bit 2 of SR_TRACE_ORDER puts the occlusion queue first, bits 0
                    // and 1 walk the closest-hit / occlusion queue from its end
                    const bool sfirst = (SR_TRACE_ORDER & 4) != 0;
                    const bool any = sfirst ? idx < n1 : idx >= n0;
                    const uint32_t j = sfirst ? (any ? idx : idx - n1) : (any ? idx - n0 : idx);
                    Rec e = any ? q1[(SR_TRACE_ORDER & 2) ? n1 - 1 - j : j] : q0[(SR_TRACE_ORDER & 1) ? n0 - 1 - j : j];
                    slot = (uint32_t)__float_as_int(e.a.w);
                    tag = (uint32_t)__float_as_int(e.b.w);
                    start(any);
                    sq.init(S, make_ray(V3{e.a.x, e.a.y, e.a.z}, V3{e.b.x, e.b.y, e.b.z}), any);
                    busy = true;
                }
            }
        }
        const unsigned busy_mask = __ballot_sync(0xffffffffu, busy);
        if (!busy_mask) {
            if (exhausted) break;
            continue;
        }
#if SR_BURST_ONE_VOTE
        // one vote per node visit: the lanes waiting for a leaf action (or done); the busy lanes
        // not among them have node work (a lane's busy flag does not change inside the burst)
        unsigned waiting = __ballot_sync(0xffffffffu, busy && sq.state != QS_NODE);
#pragma unroll 1
        for (int k = 0; k < kNodeBurst; ++k) {
            if (!(busy_mask & ~waiting)) break;
            if (busy && sq.state == QS_NODE) sq.template node_action<COUNT>(S, stack, c, err);
            waiting = __ballot_sync(0xffffffffu, busy && sq.state != QS_NODE);
            if (__popc(waiting) >= kLeafWait) break;
        }
#else
#pragma unroll 1
        for (int k = 0; k < kNodeBurst; ++k) {
            bool nodework = busy && sq.state == QS_NODE;
            if (!__any_sync(0xffffffffu, nodework)) break;
            if (nodework) sq.template node_action<COUNT>(S, stack, c, err);
            if (__popc(__ballot_sync(0xffffffffu, busy && sq.state != QS_NODE)) >= kLeafWait) break;
        }
#endif
        if (busy && sq.state != QS_NODE && sq.state != QS_DONE) sq.template leaf_action<COUNT>(S, stack, c, err);
        if (busy && sq.state == QS_DONE) {
            busy = false;
            pending = true;
        }
        if (SR_DEFER_ROUNDS > 0 && exhausted && ++rounds_after >= SR_DEFER_ROUNDS && busy && !sq.any_hit && dcap) {
            const uint32_t d = atomicAdd(dcount, 1u);
            if (d < dcap) {  // else the buffer is full and the query runs on here
                float4* r = dout + (size_t)d * kDeferF4;
                uint32_t* w = reinterpret_cast<uint32_t*>(r);
                w[0] = slot;
                w[1] = tag;
                sq.save(w + 2);
                uint32_t* se = reinterpret_cast<uint32_t*>(r + kDeferHeadF4);
                for (int i = 0; i < sq.sp; ++i) {
                    const StackEntry e = stack.get(i);
                    se[3 * i] = (uint32_t)e.child, se[3 * i + 1] = (uint32_t)e.count, se[3 * i + 2] = __float_as_uint(e.t);
                }
                busy = false;  // set aside: no answer this launch
            }
        }
    }
}

// The closest hit of slot s's path ray (fog scatter distance fog_t) is known: decide the
// segment's event and store the hit a surface event needs.  (The ray record was written when the
// ray was made.)
__device__ __forceinline__ int extend_answer(const WaveState& W, uint32_t s, const Hit& h, float fog_t) {
    const int ev = segment_event(fog_t, h.obj >= 0, h.dist);
    if (ev == EV_SURF)
        st_rec(&W.rec[rix(W, s, R_HIT)], Rec{make_float4(__int_as_float(h.obj), __int_as_float(h.tri), h.dist, h.tl),
                                          make_float4(h.u, h.v, 0.f, 0.f)});
    return ev;
}

// Traversals of the bounce: the closest hit of every queued path ray, then its segment's event
// (one event queue each), and -- WITH_SHADOW -- the shadow rays of the previous bounce's light
// samples in the same persistent loop (any hit -> black in opaque scenes, else the fog
// transmittance, written over the request's origin; SampleSkyLight scene.cs:758-772).  One loop
// for both keeps the SMs busy while either kind's last long rays finish.
// BLOCK: threads per block (64, 128 or 256, chosen at run time by the scene's tuning); the register
// cap keeps SR_TRACE_MIN_BLOCKS x 128 threads resident per SM whatever the block size.
template <bool COUNT, bool GENERAL, bool WITH_SHADOW, int BLOCK = 128>
__global__ void __launch_bounds__(BLOCK, SR_TRACE_MIN_BLOCKS * 128 / BLOCK)
    k_wave_trace(WaveState W, DevScene S, int cur, uint32_t* err, unsigned long long* counters) {
    // (the queues this kernel appends to were emptied by the last bounce's finalize kernel, so that
    // the ready phase's kernels can run beside this one)
    const int nxt = cur ^ 1;
    __shared__ uint32_t ring[BLOCK / 32][3 * 64];
    WarpStage<3> stage;
    stage.init(ring[threadIdx.x >> 5]);
    uint32_t* const eq[3] = {W.q_event[cur] + (size_t)EV_FOG * W.slots, W.q_event[cur] + (size_t)EV_MISS * W.slots,
                             W.q_event[cur] + (size_t)EV_SURF * W.slots};
    uint32_t* const ec[3] = {&W.counts[kCountEvent + 3 * cur + EV_FOG], &W.counts[kCountEvent + 3 * cur + EV_MISS],
                             &W.counts[kCountEvent + 3 * cur + EV_SURF]};
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    persistent_queries<COUNT, GENERAL>(
        S, W.q_trace[cur], W.counts[kCountTrace + cur], W.q_shadow[cur], WITH_SHADOW ? W.counts[kCountShadow + cur] : 0u,
        &W.counts[kCountTraceFetch], c, err,
        [&](bool any) { SR_COUNT(c, any ? SR_COUNTER_SCENE_OCCLUDE : SR_COUNTER_SCENE_TRACE, 1); },
        [&](uint32_t s, uint32_t bounce, bool any, const Hit& h, const Ray& ray) {
            (void)ray;
            if (!any) return extend_answer(W, s, h, __uint_as_float(bounce));
            float tr = 0.0f;
            if (h.obj < 0) {
                tr = 1.0f;
                if (S.has_fog) tr = 1.0f * fog_transmittance_inf(S, ray);
            }
            st4(&W.rec[rix(W, s, R_SH0)].a, make_float4(tr, tr, tr, 0.f));
            return -1;
        },
        [&](uint32_t s, int ev) {
            stage.add(eq, ec, s, ev);
            if (ev >= 0) W.ev_mark[s] = event_mark(ev, cur, 1);
        },
        W.defer[cur], wave_deferred(W.counts, W.defer_cap, cur), W.defer[nxt], &W.counts[kCountDefer + nxt],
        W.defer_cap);
    stage.flush(eq, ec);
    flush_counters<COUNT>(c, counters);
}

// The transmittance of slot s's shadow ray by the closest-hit loop (ShadowTransmittance,
// scene.cs:576-600), times the fog transmittance, written over the request's origin.
template <bool COUNT, bool GENERAL>
__device__ __forceinline__ void shadow_trace(const WaveState& W, const DevScene& S, uint32_t s, const Ray& shadow,
                                             Ctr& c, uint32_t* err) {
    Col tr = shadow_transmittance<COUNT, GENERAL>(S, shadow, c, err);
    if (max_component(tr) > 0.0f && S.has_fog) tr = tr * fog_transmittance_inf(S, shadow);
    st4(&W.rec[rix(W, s, R_SH0)].a, make_float4(tr.r, tr.g, tr.b, 0.f));
}

// Shadow rays of the previous bounce in scenes with transparent materials, where a shadow ray is a
// closest-hit loop through the transparent objects it meets.
template <bool COUNT, bool GENERAL>
__global__ void __launch_bounds__(128) k_wave_shadow_loop(WaveState W, DevScene S, int cur, uint32_t* err,
                                                         unsigned long long* counters) {
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    const uint32_t n = W.counts[kCountShadow + cur];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        Rec e = W.q_shadow[cur][k];
        shadow_trace<COUNT, GENERAL>(W, S, (uint32_t)__float_as_int(e.a.w),
                                     make_ray(V3{e.a.x, e.a.y, e.a.z}, V3{e.b.x, e.b.y, e.b.z}), c, err);
    }
    flush_counters<COUNT>(c, counters);
}

// ---- path-vertex records of the adjoint passes (ADJ != kAdjNone) ----------------------------------
// One record of 8 float4 per vertex (the quantities the reverse sweep needs, as adjoint_sweep's
// AdjVertex holds them, with the light sample kept apart from its shadow-ray transmittance, which
// a traced shadow ray only delivers a bounce later):
//   0: throughput in (rgb), kind | material << 3      4: d nee / d roughness, score of the segment in
//   1: emission or sky x MIS, transmittance            5: scatter weight, uv.x
//   2: light sample without transmittance, d log tr / d density   6: d s / d albedo, uv.y
//   3: d nee / d albedo, survival probability          7: d s / d roughness, -
__device__ __forceinline__ float4* adj_vertex(const AdjPass* A, uint32_t s, uint32_t sample, uint32_t k) {
    return A->vbuf + (((size_t)s * A->samples_kept + sample) * A->vper + k) * kAdjVertexF4;
}
// The slot's sample whose vertices the record holds: 0 when one sample is kept, else the index in
// the path flags.
__device__ __forceinline__ uint32_t adj_sample(const AdjPass* A, uint32_t pflags) {
    return A->samples_kept > 1 ? pflags >> kAdjSampleShift : 0u;
}
// A vertex record as adjoint_sweep reads it; the throughputs after the roulette (and the fog
// colour) and before the clamp are recomputed with the forward's float operations.
__device__ __forceinline__ AdjVertex<ADJ_ALL> adj_decode(const float4* r, const DevScene& S, float clamp_max) {
    const float4 r0 = r[0], r1 = r[1], r2 = r[2], r3 = r[3], r4 = r[4], r5 = r[5], r6 = r[6], r7 = r[7];
    AdjVertex<ADJ_ALL> q;
    const uint32_t km = __float_as_uint(r0.w);
    q.kind = (int)(km & 7u);
    q.material = (int)(km >> 3);
    q.e_in = col3(r0);
    const Col nee = col3(r2) * r1.w;
    q.add = col3(r1) + nee;
    q.dadd = col3(r3) * r1.w;
    q.rr = r3.w;
    q.s = col3(r5);
    q.ds = col3(r6);
    q.uv = V2{r5.w, r6.w};
    q.clamp_max = clamp_max;
    q.ex = AdjExtra{col3(r4) * r1.w, col3(r7), nee * r2.w, r4.w};
    if (q.kind == AV_FOG || q.kind == AV_FOG_END) {
        q.e_rr = q.e_in * col3(S.fog_color);
    } else {
        q.e_rr = q.rr < 1.0f ? q.e_in / q.rr : q.e_in;
        q.pre = q.e_rr * q.s;
    }
    return q;
}

// The rest of SampleSkyDirect / SampleSkyDirectFog (scene.cs:774-810) once the shadow kernel has
// left the transmittance (incl. fog) in the request record: the contribution of the light sample.
// Adjoint passes also complete the light-sample vertex's record `vrec` with the transmittance.
template <bool COUNT, bool GENERAL, int ADJ = kAdjNone>
__device__ __forceinline__ void add_nee(const WaveState& W, const DevScene& S, uint32_t s, uint32_t pflags,
                                        Col& radiance, Col& fog, Ctr& c, float4* vrec = nullptr) {
    Rec r0 = ld_rec(&W.rec[rix(W, s, R_SH0)]);
    Col tr = col3(r0.a);
    if constexpr (ADJ != kAdjNone) reinterpret_cast<float*>(vrec + 1)[3] = tr.r;  // opaque scenes: grey
    if (max_component(tr) > 0.0f) {
        Rec r1 = ld_rec(&W.rec[rix(W, s, R_SH1)]);
        V3 ldir{r0.b.x, r0.b.y, r0.b.z};
        Col contrib = sky_light_radiance<COUNT, GENERAL>(S, __float_as_int(r1.b.w), ldir, c) * tr * col3(r1.a) * r1.a.w /
                      r0.b.w;
        Col add = contrib * col3(r1.b);
        if (pflags & PF_NEE_FOG)
            fog = fog + add;
        else
            radiance = radiance + add;
    }
}

// The outcome of one path step: whether the path goes on, whether a shadow ray must be traced,
// and the next segment (its event, or -1 when its ray needs a traversal) with the rays to queue.
struct SegOut {
    bool live = false, shadow = false;
    int next = -1;
    V3 sh_o{0.f, 0.f, 0.f}, sh_d{0.f, 0.f, 0.f};  // the shadow ray, when traced
    V3 nx_o{0.f, 0.f, 0.f}, nx_d{0.f, 0.f, 0.f};  // the next ray, when traced
    float nx_t = 0.f;                              // ... and its fog scatter distance
};

// The state a path carries from segment to segment (its ray and fog scatter distance, bounce index,
// flags, accumulated radiance and fog radiance, throughput, last scatter pdf, random numbers), in
// registers while one shade call runs its segments.
struct PathRegs {
    Ray ray;
    float fog_t;
    uint32_t bounce, pflags;
    Col radiance, energy, fog;
    float spdf;
    Rng rng;
};

// A segment of path slot s whose event is ev (scene.cs:640-738), on the path state in p: the
// event's logic, then the next ray's fog free-flight draw and, when that ray misses the scene's
// root boxes, its segment's event (o.next).  FOG_OR_MISS = true compiles only what fog scatter
// and miss events need (the events a chained segment can have: its ray misses the root boxes).
template <bool COUNT, bool GENERAL, bool FOG_OR_MISS, int ADJ = kAdjNone>
__device__ __forceinline__ SegOut shade_event(const WaveState& W, const DevScene& S, const DevParams& P, uint32_t s,
                                              int ev, PathRegs& p, Ctr& c, const AdjPass* A = nullptr) {
    SegOut o;
    SR_COUNT(c, SR_COUNTER_SAMPLE_BOUNCE, 1);
    if (p.bounce == 0) SR_COUNT(c, SR_COUNTER_SAMPLE, 1);
    Ray& ray = p.ray;
    Col& energy = p.energy;
    const uint32_t bounce = p.bounce;
    bool terminate = false;
    // adjoint passes: this vertex's record (see adj_vertex), built up as the segment runs
    [[maybe_unused]] const Col e_in = energy;
    [[maybe_unused]] int vkind = AV_SKY, vmat = 0;
    [[maybe_unused]] Col vemit = black(), vnee = black(), vdnee_a = black(), vdnee_r = black(), vs = black(),
                         vds_a = black(), vds_r = black();
    [[maybe_unused]] float vtr = 0.0f, vdlogtr = 0.0f, vrr = 1.0f, vscore = 0.0f;
    [[maybe_unused]] V2 vuv{0.0f, 0.0f};
    if (ev != EV_MISS) {
        // Fog and surface events share one light sample, one Russian-roulette draw and then
        // scatter, in that RNG order (scene.cs:654-726).
        const bool fog_event = FOG_OR_MISS || ev == EV_FOG;
        SurfHit sh;
        if (!fog_event) {
            const Rec hr = ld_rec(&W.rec[rix(W, s, R_HIT)]);
            Hit hit{__float_as_int(hr.a.x), __float_as_int(hr.a.y), hr.a.z, hr.a.w, hr.b.x, hr.b.y};
            surface_from_hit<COUNT, GENERAL>(S, ray, hit, sh, c);
            if constexpr (ADJ != kAdjNone) vmat = S.objects[hit.obj].index;
        }
        const Surface& su = sh.surf;
        const float dist = sh.dist;
        const V3 view = -ray.d;
        float bias = 0.0f;
        V3 pos;
        if (fog_event) {
            energy = energy * col3(S.fog_color);
            pos = ray_at(ray, p.fog_t);  // the fog scatter distance
            if constexpr (ADJ != kAdjNone) {  // score of a scatter at t: 1/density - depth(t)/density
                vkind = AV_FOG;
                vscore = 1.0f / S.fog_density - fog_depth_unit(S, ray, p.fog_t);
            }
        } else {
            bias = fmaxf(1e-4f, dist * 1e-4f);
            pos = ray_at(ray, dist - bias);
            if (GENERAL && (p.pflags & PF_MEDIUM)) energy = energy * beer_law(col3(W.medium[s]), dist);
            p.radiance = p.radiance + su.radiance * energy;
            if constexpr (ADJ != kAdjNone) {
                vkind = AV_SURF;
                vemit = su.radiance;
                vuv = su.uv;
                if (S.has_fog) vscore = -fog_depth_unit(S, ray, dist);  // passing the fog up to the surface
            }
            if (bounce == 0) {
                p.pflags |= PF_PRIMARY;
                st_rec(&W.pix[pix(W, s, X_PRIM)], Rec{make_float4(su.normal.x, su.normal.y, su.normal.z, dist),
                                                     make_float4(su.uv.x, su.uv.y, 0.f, 0.f)});
            }
        }
        // NEE toward the sky (SampleSkyDirectFog scene.cs:796-810 / SampleSkyDirect :774-794);
        // a shadow ray that needs a traversal goes to the shadow kernel and its contribution is
        // added next segment (before anything of that segment touches the radiance)
        V3 ldir;
        float lpdf;
        int texel;
        if (sky_light_rand<COUNT, GENERAL>(S, p.rng, ldir, lpdf, texel, c) && lpdf > 0.0f) {
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
            if constexpr (ADJ != kAdjNone) {
                if (emit) {
                    const Col sky = sky_light_radiance<false, GENERAL>(S, texel, ldir, c) * mis / lpdf;
                    vnee = sky * w3;
                    if (!fog_event) {
                        vdnee_a = sky * opaque_eval_dalbedo(su, view, ldir);
                        vdnee_r = sky * opaque_eval_droughness(su, view, ldir);
                    }
                    if (S.has_fog) {  // d log(fog transmittance of the shadow ray) / d density
                        const float depth = fog_depth_unit(S, make_ray(pos, ldir), __int_as_float(0x7f800000));
                        vdlogtr = isfinite(depth) ? -depth : 0.0f;
                    }
                }
            }
            if (emit) {
                const bool to_fog = fog_event && bounce == 0;
                Ray shadow = make_ray(pos, ldir);
                const bool any = !GENERAL || !S.has_transparent;
                if (any ? misses_scene<COUNT, true>(S, shadow, c) : misses_scene<COUNT, false>(S, shadow, c)) {
                    // a shadow ray that misses the scene's root boxes is unoccluded: its
                    // transmittance is the fog's alone, and the light sample's contribution is
                    // added at once, as SampleSkyDirect(Fog) forms it
                    SR_COUNT(c, SR_COUNTER_SCENE_OCCLUDE, 1);
                    float t = 1.0f;
                    if (S.has_fog) t = 1.0f * fog_transmittance_inf(S, shadow);
                    Col tr = gray(t);
                    if constexpr (ADJ != kAdjNone) vtr = t;
                    if (max_component(tr) > 0.0f) {
                        Col contrib = sky_light_radiance<COUNT, GENERAL>(S, texel, ldir, c) * tr * w3 * mis / lpdf;
                        Col add = contrib * energy;
                        if (to_fog)
                            p.fog = p.fog + add;
                        else
                            p.radiance = p.radiance + add;
                    }
                } else {
                    // traced by the shadow kernel; the contribution is added next segment
                    p.pflags |= PF_NEE | (to_fog ? PF_NEE_FOG : 0u);
                    o.shadow = true;
                    o.sh_o = pos;
                    o.sh_d = ldir;
                    st_rec(&W.rec[rix(W, s, R_SH0)], Rec{make_float4(pos.x, pos.y, pos.z, 0.f),
                                                      make_float4(ldir.x, ldir.y, ldir.z, lpdf)});
                    st_rec(&W.rec[rix(W, s, R_SH1)], Rec{make_float4(w3.r, w3.g, w3.b, mis),
                                                      make_float4(energy.r, energy.g, energy.b, __int_as_float(texel))});
                }
            }
        }
        if constexpr (ADJ != kAdjNone)
            if (bounce >= 3) vrr = fminf(1.0f, max_component(energy));  // the roulette's survival probability
        if (russian_roulette(energy, bounce, p.rng)) {
            terminate = true;
            if constexpr (ADJ != kAdjNone) vkind = fog_event ? AV_FOG_END : AV_SURF_END;
        } else if (fog_event) {
            V3 sdir = hg_scatter_dir(ray.d, S.fog_g, p.rng);
            p.pflags |= PF_SPDF;
            p.spdf = hg_pdf(dot(ray.d, sdir), S.fog_g);
            ray = make_ray(pos, sdir);
        } else {
            Scatter sc = surface_scatter<GENERAL>(su, ray.d, view, p.rng);
            if constexpr (ADJ != kAdjNone) {  // the scatter weight and its derivatives (pdf held fixed)
                const float ipdf = 1.0f / fmaxf(sc.pdf, 1e-6f);
                vs = sc.weight;
                vds_a = opaque_eval_dalbedo(su, view, sc.dir) * ipdf;
                vds_r = opaque_eval_droughness(su, view, sc.dir) * ipdf;
            }
            energy = energy * sc.weight;
            energy = clamp_luminance(energy, P.indirect_clamp);
            bool enter = dot(sc.dir, su.normal_geo) < 0.0f;
            if (GENERAL && sc.refracted) {
                if (enter) {
                    p.pflags |= PF_MEDIUM;
                    W.medium[s] = make_float4(su.albedo.r, su.albedo.g, su.albedo.b, 0.f);
                } else {
                    p.pflags &= ~PF_MEDIUM;
                }
            } else if (!enter) {
                p.pflags &= ~PF_MEDIUM;
            }
            p.pflags = sc.has_pdf ? (p.pflags | PF_SPDF) : (p.pflags & ~PF_SPDF);
            p.spdf = sc.pdf;
            ray = make_ray(ray_at(ray, dist) + sc.dir * bias, sc.dir);
        }
    } else {
        // miss: sky radiance with the MIS weight of the last scatter (scene.cs:728-738)
        float mis = (p.pflags & PF_SPDF) ? power_heuristic(p.spdf, sky_light_pdf<GENERAL>(S, ray.d)) : 1.0f;
        p.radiance = p.radiance + sky_radiance<COUNT, GENERAL>(S, ray.d, c) * mis * energy;
        terminate = true;
        if constexpr (ADJ != kAdjNone) {
            vemit = sky_radiance<false, GENERAL>(S, ray.d, c) * mis;
            if (S.has_fog) {  // escaping: the fog's transmittance to infinity
                const float depth = fog_depth_unit(S, ray, __int_as_float(0x7f800000));
                vscore = isfinite(depth) ? -depth : 0.0f;
            }
        }
    }
    if constexpr (ADJ != kAdjNone) {
        float4* r = adj_vertex(A, s, adj_sample(A, p.pflags), bounce);
        r[0] = make_float4(e_in.r, e_in.g, e_in.b, __uint_as_float((uint32_t)vkind | ((uint32_t)vmat << 3)));
        r[1] = make_float4(vemit.r, vemit.g, vemit.b, vtr);
        r[2] = make_float4(vnee.r, vnee.g, vnee.b, vdlogtr);
        r[3] = make_float4(vdnee_a.r, vdnee_a.g, vdnee_a.b, vrr);
        r[4] = make_float4(vdnee_r.r, vdnee_r.g, vdnee_r.b, vscore);
        r[5] = make_float4(vs.r, vs.g, vs.b, vuv.x);
        r[6] = make_float4(vds_a.r, vds_a.g, vds_a.b, vuv.y);
        r[7] = make_float4(vds_r.r, vds_r.g, vds_r.b, 0.0f);
    }
    if (!terminate && ++p.bounce == P.bounces + 1) terminate = true;
    o.live = !terminate;
    if (o.live) {
        // the next segment's fog free-flight draw: the reference makes it right after the
        // traversal, which draws nothing, so drawing it now keeps the RNG sequence
        p.fog_t = fog_scatter_t(S, ray, p.rng);
        o.next = next_segment<COUNT>(S, ray, p.fog_t, c);
        o.nx_o = ray.o;
        o.nx_d = ray.d;
        o.nx_t = p.fog_t;
    }
    return o;
}

// Segments of a path whose next event is already known can run back to back: while a segment's
// new ray misses the scene's root boxes (its event is a fog scatter or a miss, decided on the spot)
// and no shadow ray waits for a traversal, the same shade call goes on with the next segment, with
// the path state in registers, instead of storing it and queueing the slot for the next bounce.
// A warp keeps chaining while at least SR_CHAIN_MIN_LANES of its lanes can (0: never), so that a
// few long chains do not hold a mostly idle warp.  Each path's operations and their order are
// unchanged, so images are identical either way; only the records stored and the bounces run
// change.  Measured on the 1080p fog workload: chaining every lane (1) was 7 % slower than none
// (0), with the bounces down from 352 to 156: the warps ran as long as their longest chain.
#ifndef SR_CHAIN_MIN_LANES
#define SR_CHAIN_MIN_LANES 0
#endif

// Path slot s from its stored state through its segment with event ev -- first the NEE
// contribution of the previous segment if its shadow ray was traced since -- and, chaining, the
// segments after it that need no traversal; then the new path state is stored.
template <bool COUNT, bool GENERAL, int ADJ = kAdjNone, bool FOG_OR_MISS = false>
__device__ __forceinline__ SegOut shade_segment(const WaveState& W, const DevScene& S, const DevParams& P, uint32_t s,
                                                int ev, Ctr& c, const AdjPass* A = nullptr) {
    const Rec rr = ld_rec(&W.rec[rix(W, s, R_RAY)]), pr = ld_rec(&W.rec[rix(W, s, R_PATH)]),
              gr = ld_rec(&W.rec[rix(W, s, R_RNG)]);
    PathRegs p;
    p.rng = rng_of(gr);
    p.fog = Col{gr.b.y, gr.b.z, gr.b.w};
    p.bounce = ibits(rr.a.w);
    p.pflags = ibits(pr.b.w);
    p.ray = make_ray(V3{rr.a.x, rr.a.y, rr.a.z}, V3{rr.b.x, rr.b.y, rr.b.z});
    p.fog_t = rr.b.w;
    p.radiance = col3(pr.a);
    p.spdf = pr.a.w;
    p.energy = col3(pr.b);
    if (p.pflags & PF_NEE) {  // the previous segment's light sample (that segment's vertex)
        float4* vrec = nullptr;
        if constexpr (ADJ != kAdjNone) vrec = adj_vertex(A, s, adj_sample(A, p.pflags), p.bounce - 1);
        add_nee<COUNT, GENERAL, ADJ>(W, S, s, p.pflags, p.radiance, p.fog, c, vrec);
    }
    p.pflags &= ~(PF_NEE | PF_NEE_FOG);
    SegOut o = shade_event<COUNT, GENERAL, FOG_OR_MISS, ADJ>(W, S, P, s, ev, p, c, A);
    if (SR_CHAIN_MIN_LANES > 0) {
        // at most bounces + 1 segments per sample: every segment advances the bounce index; the
        // lanes of the call vote each round, and all of them stop together
        const unsigned lanes = __activemask();
        for (;;) {
            const bool more = o.live && !o.shadow && o.next >= 0;
            if (__popc(__ballot_sync(lanes, more)) < SR_CHAIN_MIN_LANES) break;
            if (more) o = shade_event<COUNT, GENERAL, true, ADJ>(W, S, P, s, o.next, p, c, A);
        }
    }
    st_rec(&W.rec[rix(W, s, R_PATH)], Rec{make_float4(p.radiance.r, p.radiance.g, p.radiance.b, p.spdf),
                                          make_float4(p.energy.r, p.energy.g, p.energy.b, fbits(p.pflags))});
    if (o.live)
        st_rec(&W.rec[rix(W, s, R_RAY)], Rec{make_float4(p.ray.o.x, p.ray.o.y, p.ray.o.z, fbits(p.bounce)),
                                             make_float4(p.ray.d.x, p.ray.d.y, p.ray.d.z, p.fog_t)});
    st_rec(&W.rec[rix(W, s, R_RNG)], rng_rec(p.rng, p.fog));
    return o;
}

// Events of phase `phase` of the bounce (0: the ready events, 1: the others; see SR_SPLIT_PHASES)
// from the slot-ordered queues, or every event from the arrival-ordered ones (SR_SORT_EVENTS = 0).
// Returns the event count and sets *first, its first entry in the sorted queue.
__device__ __forceinline__ uint32_t phase_events(const WaveState& W, int cur, int phase, int ev, uint32_t* first) {
    *first = 0;
    if (!SR_SORT_EVENTS) return W.counts[kCountEvent + 3 * cur + ev];
    if (phase == 0) return W.counts[kCountSorted + ev];
    *first = W.counts[kCountSorted + ev];
    return W.counts[kCountSortedLate + ev];
}

// One segment of every live path of the phase with event EVK, or of all its live paths (EVK = -1)
// with warps sorted by event: the index space is then the fog queue, the miss queue and the surface
// queue, the first two padded to whole warps, so every warp runs one event's logic.  EVK =
// EV_FOG_MISS: the fog queue (padded) and the miss queue in one launch, compiled with only the
// fog and miss logic.
template <bool COUNT, bool GENERAL, int EVK, int ADJ = kAdjNone>
__global__ void __launch_bounds__(128, ADJ != kAdjNone ? 4 : shade_min_blocks(EVK))
    k_wave_shade(WaveState W, DevScene S, DevParams P, int cur, int phase, uint32_t* err,
                 unsigned long long* counters, const AdjPass* A) {
    __shared__ uint32_t sh[2][6][kBlockWarps + 1];
    uint32_t round = 0;
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    const int nxt = cur ^ 1;
    uint32_t first[3];
    const uint32_t nfog = phase_events(W, cur, phase, EV_FOG, &first[EV_FOG]);
    const uint32_t nmiss = phase_events(W, cur, phase, EV_MISS, &first[EV_MISS]);
    const uint32_t nsurf = phase_events(W, cur, phase, EV_SURF, &first[EV_SURF]);
    const uint32_t ecount[3] = {nfog, nmiss, nsurf};
    const uint32_t pfog = (nfog + 31u) & ~31u, pmiss = (nmiss + 31u) & ~31u;
    const uint32_t total = EVK == EV_FOG_MISS ? pfog + nmiss : EVK >= 0 ? ecount[EVK % 3] : pfog + pmiss + nsurf;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += stride) {
        const uint32_t k = base + threadIdx.x;
        int ev;
        uint32_t i, cnt;
        if (EVK >= 0 && EVK != EV_FOG_MISS) {
            ev = EVK, i = k, cnt = total;
        } else if (k < pfog) {
            ev = EV_FOG, i = k, cnt = nfog;
        } else if (EVK == EV_FOG_MISS || k < pfog + pmiss) {
            ev = EV_MISS, i = k - pfog, cnt = nmiss;
        } else {
            ev = EV_SURF, i = k - pfog - pmiss, cnt = nsurf;
        }
        const bool valid = i < cnt;
        const uint32_t* const q = SR_SORT_EVENTS ? W.q_sorted : W.q_event[cur];
        const uint32_t s = valid ? q[(size_t)ev * W.slots + first[ev] + i] : 0u;
        SegOut o;
        if (valid) {
            o = shade_segment<COUNT, GENERAL, ADJ, EVK == EV_FOG_MISS>(W, S, P, s, ev, c, A);
        }
        uint32_t* eq = W.q_event[nxt];
        // finished samples wait for their last shadow ray (traced next bounce) when it has one; so
        // does the next event of a path with a shadow ray queued
        const bool pred[6] = {valid && o.live && o.next < 0, valid && o.live && o.next == EV_FOG,
                              valid && o.live && o.next == EV_MISS, valid && !o.live && !o.shadow,
                              valid && !o.live && o.shadow, valid && o.shadow};
        uint32_t off[6];
        block_offsets<6>({&W.counts[kCountTrace + nxt], &W.counts[kCountEvent + 3 * nxt + EV_FOG],
                          &W.counts[kCountEvent + 3 * nxt + EV_MISS], &W.counts[count_resolve(cur)],
                          &W.counts[kCountLate + nxt], &W.counts[kCountShadow + nxt]},
                         pred, sh, round++, off);
        const int wait = o.shadow ? 1 : 0;
        if (pred[0]) W.q_trace[nxt][off[0]] = ray_entry(s, o.nx_o, o.nx_d, o.nx_t);
        if (pred[1]) eq[(size_t)EV_FOG * W.slots + off[1]] = s, W.ev_mark[s] = event_mark(EV_FOG, nxt, wait);
        if (pred[2]) eq[(size_t)EV_MISS * W.slots + off[2]] = s, W.ev_mark[s] = event_mark(EV_MISS, nxt, wait);
        if (pred[3]) W.q_resolve[cur][off[3]] = s;
        if (pred[4]) W.q_late[nxt][off[4]] = s;
        if (pred[5]) W.q_shadow[nxt][off[5]] = ray_entry(s, o.sh_o, o.sh_d, 0.f);
    }
    flush_counters<COUNT>(c, counters);
}

// One more finished pixel per calling thread (warp-aggregated: one atomic per converged group).
__device__ __forceinline__ void count_pixel_done(uint32_t* counter) {
    const unsigned m = __activemask();
    if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(counter, (uint32_t)__popc(m));
}

// End of the sample in slot s: the pending NEE contribution of its last segment, the pixel
// statistics and the adaptive stop (renderer.cs:173-212), then the next camera ray or the AOVs.
template <bool COUNT, bool GENERAL, int ADJ = kAdjNone>
__device__ __forceinline__ SegOut finalize_sample(const WaveState& W, const DevScene& S, const DevView& V,
                                                  const DevParams& P, const DevAovs& out, uint32_t s, Ctr& c,
                                                  const AdjPass* A = nullptr, float* g_density = nullptr) {
    SegOut o;
        Rec pr = ld_rec(&W.rec[rix(W, s, R_PATH)]), gr = ld_rec(&W.rec[rix(W, s, R_RNG)]);
        uint32_t pflags = ibits(pr.b.w);
        Col radiance = col3(pr.a);
        Col radiance_fog{gr.b.y, gr.b.z, gr.b.w};
        // adjoint passes: the sample's last segment (its vertex count - 1) and its record slot
        [[maybe_unused]] uint32_t last = 0, vsample = 0;
        if constexpr (ADJ != kAdjNone) {
            last = ibits(ld_rec(&W.rec[rix(W, s, R_RAY)]).a.w);
            vsample = adj_sample(A, pflags);
        }
        if (pflags & PF_NEE) {
            float4* vrec = nullptr;
            if constexpr (ADJ != kAdjNone) vrec = adj_vertex(A, s, vsample, last);
            add_nee<COUNT, GENERAL, ADJ>(W, S, s, pflags, radiance, radiance_fog, c, vrec);
        }
        Rec c0 = ld_rec(&W.pix[pix(W, s, X_ACC)]), c1 = ld_rec(&W.pix[pix(W, s, X_ACC + 1)]), c2 = ld_rec(&W.pix[pix(W, s, X_ACC + 2)]);
        float4 a0 = c0.a, a1 = c0.b, a2 = c1.a, a3 = c1.b, a4 = c2.a, a5 = c2.b;
        a0.x += radiance.r, a0.y += radiance.g, a0.z += radiance.b;
        a1.x += radiance_fog.r, a1.y += radiance_fog.g, a1.z += radiance_fog.b;
        float lum = luminance(radiance) + luminance(radiance_fog);
        a0.w += lum;
        a1.w += lum * lum;
        float ls = luminance(radiance);
        a2.w += ls;
        a3.w += ls * ls;
        uint32_t ncount = ibits(a4.y), dcount = ibits(a4.z);
        uint32_t si = ibits(a4.w);
        if (pflags & PF_PRIMARY) {
            Rec pm = ld_rec(&W.pix[pix(W, s, X_PRIM)]);
            float4 pn = pm.a;
            a2.x += pn.x, a2.y += pn.y, a2.z += pn.z;
            a3.x = pn.x, a3.y = pn.y, a3.z = pn.z;
            ncount++;
            a4.x += pn.w;
            dcount++;
            if (ibits(a5.z) == 0u) a5 = make_float4(pm.b.x, pm.b.y, fbits(1u), a5.w);
        }
        bool done = false;
        uint32_t count = 0;
        uint32_t x, y;
        const uint32_t pixel = W.dynamic ? ibits(a5.w) : s;
        pixel_xy(W, pixel, x, y);
        if constexpr (ADJ == kAdjReplay) {
            // the replayed render takes the samples the replayed one took (renderer.cs:215's
            // off-by-one: a pixel whose loop ran out counts max_samples + 1), and this sample's
            // vertices are swept back at once with G = dL/dI / count
            const size_t i = (size_t)y * P.width + x;
            count = A->fwd_samples[i];
            const uint32_t taken = count < P.max_samples ? count : P.max_samples;
            const float inv = 1.0f / (float)count;
            const Col G{A->d_image[3 * i] * inv, A->d_image[3 * i + 1] * inv, A->d_image[3 * i + 2] * inv};
            const float4* vb = adj_vertex(A, s, 0, 0);
            adjoint_sweep<ADJ_ALL>(
                S, [&](int k) { return adj_decode(vb + (size_t)k * kAdjVertexF4, S, P.indirect_clamp); },
                (int)last + 1, G, AdjTargets{A->tex_a, A->grad_a, A->tex_r, A->grad_r, A->grad_f}, *g_density);
            if (si + 1 >= taken)
                done = true;
            else
                ++si;
        } else {
            if constexpr (ADJ == kAdjRecord) A->vcount[(size_t)s * A->samples_kept + vsample] = (uint8_t)(last + 1);
            if (si >= P.min_samples - 1 && relative_std_err(a0.w, a1.w, si + 1) < P.variance_threshold) {
                done = true;
                count = si + 1;
            } else if (++si == P.max_samples) {
                done = true;
                count = si + 1;  // loop ran out: normalised by maxSamples + 1 (renderer.cs:215)
            }
        }
        if (ADJ == kAdjReplay && done) {
            if (A->replay) {
                const Col r = col3(a0) / (float)count, f = col3(a1) / (float)count;
                const size_t i = (size_t)y * P.width + x;
                A->replay[3 * i] = r.r + f.r, A->replay[3 * i + 1] = r.g + f.g, A->replay[3 * i + 2] = r.b + f.b;
            }
            count_pixel_done(W.counts + kCountDone);
        } else if (done) {
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
            count_pixel_done(W.counts + kCountDone);
        }
        // the pixel's next sample, or (fewer slots than pixels) the first sample of the next
        // unclaimed pixel, with that pixel's own random-number stream and fresh statistics
        bool start = !done;
        Rng rng = rng_of(gr);
        if (done && W.dynamic) {
            const uint32_t q = claim_pixel(W, P);
            if (q != ~0u) {
                pixel_xy(W, q, x, y);
                const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
                a0 = a1 = a2 = a3 = a4 = z;
                a5 = make_float4(0.f, 0.f, 0.f, fbits(q));
                ncount = dcount = si = 0;
                rng = rng_seed(x, y, W.pixel_cursor[kCountSeed - kCountPixel]);
                start = true;
            }
        }
        if (start) {
            Ray ray = camera_ray(V, P, x, y, rng);
            const float ft = fog_scatter_t(S, ray, rng);
            o.next = next_segment<COUNT>(S, ray, ft, c);
            begin_sample(W, s, ray, rng, ft, ADJ == kAdjRecord ? si << kAdjSampleShift : 0u);
            o.live = true;
            o.nx_o = ray.o;
            o.nx_d = ray.d;
            o.nx_t = ft;
        }
        a4.y = fbits(ncount), a4.z = fbits(dcount), a4.w = fbits(si);
        st_rec(&W.pix[pix(W, s, X_ACC)], Rec{a0, a1});
        st_rec(&W.pix[pix(W, s, X_ACC + 1)], Rec{a2, a3});
        st_rec(&W.pix[pix(W, s, X_ACC + 2)], Rec{a4, a5});
    return o;
}

// Finished samples: the pending NEE contribution of the last segment, then the pixel statistics
// and the adaptive stop (renderer.cs:173-212), then the next camera ray or the AOV write.
// LATE: the samples that finished last bounce with a shadow ray, traced since by this bounce's
// trace kernel; else the samples finished this bounce without one.
template <bool COUNT, bool GENERAL, bool LATE, int ADJ = kAdjNone>
__global__ void __launch_bounds__(128) k_wave_finalize(WaveState W, DevScene S, DevView V, DevParams P, DevAovs out,
                                                       int cur, uint32_t* err, unsigned long long* counters,
                                                       const AdjPass* A) {
    const int nxt = cur ^ 1;
    if (!LATE && blockIdx.x == 0 && threadIdx.x == 0) {
        // The queues of this bounce's parity are consumed: empty them for the bounce after next,
        // and the cursors and finished-sample queue of the next bounce (whose other queues this
        // bounce has filled).  Done here, at the end of a bounce, so that the next bounce's ready
        // phase and traversal kernel start together.
        W.counts[kCountTraceFetch] = 0;    // next trace's fetch cursor
        W.counts[kCountDefer + cur] = 0;  // this bounce's traversal resumed these; the next one fills them
        W.counts[kCountTrace + cur] = 0;
        W.counts[kCountShadow + cur] = 0;
        W.counts[kCountLate + cur] = 0;
        W.counts[kCountEvent + 3 * cur + EV_FOG] = 0;
        W.counts[kCountEvent + 3 * cur + EV_MISS] = 0;
        W.counts[kCountEvent + 3 * cur + EV_SURF] = 0;
        W.counts[count_resolve(nxt)] = 0;
        for (int e = 0; e < 3; ++e) W.counts[kCountSorted + e] = W.counts[kCountSortedLate + e] = 0;
    }
    __shared__ uint32_t sh[2][3][kBlockWarps + 1];
    uint32_t round = 0;
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    const uint32_t n = LATE ? W.counts[kCountLate + cur] : W.counts[count_resolve(cur)];
    const uint32_t* q = LATE ? W.q_late[cur] : W.q_resolve[cur];
    const uint32_t stride = gridDim.x * blockDim.x;
    float g_density = 0.0f;  // adjoint replay: this thread's d loss / d fog density
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        uint32_t k = base + threadIdx.x;
        bool valid = k < n;
        uint32_t s = valid ? q[k] : 0u;
        SegOut o;
        if (valid) {
            o = finalize_sample<COUNT, GENERAL, ADJ>(W, S, V, P, out, s, c, A, &g_density);
        }
        uint32_t* eq = W.q_event[nxt];
        const bool pred[3] = {valid && o.live && o.next < 0, valid && o.live && o.next == EV_FOG,
                              valid && o.live && o.next == EV_MISS};
        uint32_t off[3];
        block_offsets<3>({&W.counts[kCountTrace + nxt], &W.counts[kCountEvent + 3 * nxt + EV_FOG],
                          &W.counts[kCountEvent + 3 * nxt + EV_MISS]},
                         pred, sh, round++, off);
        if (pred[0]) W.q_trace[nxt][off[0]] = ray_entry(s, o.nx_o, o.nx_d, o.nx_t);
        if (pred[1]) eq[(size_t)EV_FOG * W.slots + off[1]] = s, W.ev_mark[s] = event_mark(EV_FOG, nxt, 0);
        if (pred[2]) eq[(size_t)EV_MISS * W.slots + off[2]] = s, W.ev_mark[s] = event_mark(EV_MISS, nxt, 0);
    }
    flush_counters<COUNT>(c, counters);
    if constexpr (ADJ == kAdjReplay) {  // every thread of the block gets here: one atomic per warp
        for (int d = 16; d > 0; d >>= 1) g_density += __shfl_xor_sync(0xffffffffu, g_density, d);
        if ((threadIdx.x & 31) == 0 && A->grad_f && g_density != 0.0f) atomicAdd(A->grad_f, g_density);
    }
}

constexpr int kTailFinalize = 16;  // tail-kernel state: the slot's sample is finished

// The last paths of a frame, one thread per slot run to completion.  When few paths are left the
// bounce kernels are bound by the latency of their few longest paths plus the launch gaps of
// every bounce, while one thread per slot runs the same steps back to back -- traversal, event,
// shading, shadow ray, end of sample -- in the same order, so results are identical.  The live
// slots of parity `cur` are those of every group's trace, event and late queues; a slot's shadow
// ray still queued is traced first.
template <bool COUNT, bool GENERAL, int ADJ = kAdjNone>
__global__ void __launch_bounds__(128) k_wave_tail(WaveGroups G, DevScene S, DevView V, DevParams P, DevAovs out,
                                                   int cur, uint32_t* err, unsigned long long* counters,
                                                   const AdjPass* A) {
    float g_density = 0.0f;  // adjoint replay: this thread's d loss / d fog density
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    int group = -1, ev = -1;
    bool resumed = false;  // a query set aside by the last traversal kernel
    uint32_t s = 0;
    float rt = 0.f;
    V3 ro{0.f, 0.f, 0.f}, rd{0.f, 0.f, 0.f};  // the ray of a segment that needs a traversal
    for (int g = 0; g < G.groups && group < 0; ++g) {
        const WaveState& Wg = G.W[g];
        const uint32_t nt = Wg.counts[kCountTrace + cur];
        if (k < nt) {
            group = g;
            Rec e = Wg.q_trace[cur][k];
            s = (uint32_t)__float_as_int(e.a.w);
            rt = e.b.w;
            ro = V3{e.a.x, e.a.y, e.a.z};
            rd = V3{e.b.x, e.b.y, e.b.z};
            break;
        }
        k -= nt;
        for (int e = 0; e < 3 && group < 0; ++e) {
            const uint32_t ne = Wg.counts[kCountEvent + 3 * cur + e];
            if (k < ne) {
                group = g, ev = e;
                s = Wg.q_event[cur][(size_t)e * Wg.slots + k];
                break;
            }
            k -= ne;
        }
        if (group >= 0) break;
        const uint32_t nl = Wg.counts[kCountLate + cur];
        if (k < nl) {
            group = g, ev = kTailFinalize;
            s = Wg.q_late[cur][k];
            break;
        }
        k -= nl;
        // queries set aside by the last traversal kernel: traced again from their ray (same answer)
        const uint32_t nd = wave_deferred(Wg.counts, Wg.defer_cap, cur);
        if (k < nd) {
            group = g;
            resumed = true;
            const uint32_t* w = reinterpret_cast<const uint32_t*>(Wg.defer[cur] + (size_t)k * kDeferF4);
            s = w[0];
            rt = __uint_as_float(w[1]);
            ro = V3{__uint_as_float(w[2]), __uint_as_float(w[3]), __uint_as_float(w[4])};
            rd = V3{__uint_as_float(w[5]), __uint_as_float(w[6]), __uint_as_float(w[7])};
            break;
        }
        k -= nd;
    }
    if (group >= 0) {
        const WaveState W = G.W[group];
        // the slot's shadow ray queued for the next bounce, if any: traced first (a set-aside
        // query's shadow ray was traced by the kernel that set it aside: its transmittance has
        // replaced the ray's origin)
        if (!resumed && (ibits(ld_rec(&W.rec[rix(W, s, R_PATH)]).b.w) & PF_NEE)) {
            Rec r0 = ld_rec(&W.rec[rix(W, s, R_SH0)]);
            shadow_trace<COUNT, GENERAL>(W, S, s, make_ray(V3{r0.a.x, r0.a.y, r0.a.z}, V3{r0.b.x, r0.b.y, r0.b.z}), c,
                                         err);
        }
        // every step advances a segment or ends a sample, so this bounds a well-formed frame
        const uint64_t cap = ((uint64_t)P.max_samples + 1) * ((uint64_t)P.bounces + 2) * 2 + 8;
        for (uint64_t step = 0;; ++step) {
            if (step > cap) {
                atomicOr(err, SR_DEVERR_LOOP);
                break;
            }
            SegOut o;
            if (ev == kTailFinalize) {
                o.live = false;
            } else {
                if (ev < 0) {
                    Ray ray = make_ray(ro, rd);
                    SR_COUNT(c, SR_COUNTER_SCENE_TRACE, 1);
                    ev = extend_answer(W, s, scene_closest<COUNT, GENERAL>(S, ray, c, err), rt);
                }
                o = shade_segment<COUNT, GENERAL, ADJ>(W, S, P, s, ev, c, A);
                if (o.shadow) shadow_trace<COUNT, GENERAL>(W, S, s, make_ray(o.sh_o, o.sh_d), c, err);
            }
            if (!o.live) {
                o = finalize_sample<COUNT, GENERAL, ADJ>(W, S, V, P, out, s, c, A, &g_density);
                if (!o.live) break;
            }
            ev = o.next;
            ro = o.nx_o, rd = o.nx_d, rt = o.nx_t;
        }
    }
    flush_counters<COUNT>(c, counters);
    if constexpr (ADJ == kAdjReplay)
        if (A->grad_f && g_density != 0.0f) atomicAdd(A->grad_f, g_density);
}

}  // namespace sr

// sr_wavefront.h — path state of the wavefront renderer (sr_wavefront.cu) and its launchers.
#pragma once

#include <cuda_runtime.h>

#include "sr_kernels.h"
#include "sr_layout.h"

namespace sr {

// One 32-byte sector.  Path state is stored as records of fields that the kernels read and write
// together, so that a lane touching a path moves whole DRAM bursts: the slots a warp visits are
// scattered (queues are compacted in arrival order), and 16-byte fields in separate planes would
// waste most of every burst read and turn every write into a partial write.
struct alignas(32) Rec {
    float4 a, b;
};

// The pixel slots can be split into independent groups (tile t belongs to group t % groups), each
// a complete wavefront with its own queues and counters whose bounce kernels run on parallel
// branches of the graph, so that while one group's kernel drains the other's fills the idle SMs.
// With shadow rays traced in the same persistent loop as path rays one group measured best
// (C2 1080p on GB300: 1 group 413, 2 groups 400 M samples/s).
#ifndef SR_WAVE_GROUPS
#define SR_WAVE_GROUPS 1
#endif
constexpr int kWaveGroups = SR_WAVE_GROUPS;

// Path state of one group, one slot per pixel (slots in 8x4 pixel tiles).
struct WaveState {
    uint32_t slots;    // this group's slots: its tiles x 32 (queue capacity)
    uint32_t tiles_x;  // ceil(width / 8)
    uint32_t group;    // this group's index
    uint32_t groups;   // number of groups
    // records of all groups, indexed by the global slot (tile * 32 + lane)
    Rec* rec;          // path records, six sectors per slot (192 bytes, 64-byte aligned):
                       //   ray  a: origin, bounce index (int bits)      b: direction, fog scatter distance
                       //   hit  a: object, triangle (int bits), world distance, local distance
                       //        b: barycentric u, v, -, -  (written for surface events only)
                       //   path a: radiance, pdf of the last scatter    b: throughput, path flags (int bits)
                       //   rng  a: RNG words s0..s3 (bits)              b: RNG counter s4 (bits), fog radiance
                       //   sh0  a: shadow origin (then transmittance)   b: shadow direction, light pdf
                       //   sh1  a: reflectance or phase pdf, MIS weight b: throughput at the light sample,
                       //                                                  sampled sky texel (int bits)
    Rec* pix;          // pixel records, four sectors per slot:
                       //   prim a: primary-hit normal, depth            b: primary-hit uv, -, -
                       //   acc0 a: radiance sum, luminance sum          b: fog radiance sum, luminance^2 sum
                       //   acc1 a: normal sum, surface lum sum          b: last normal, surface lum^2 sum
                       //   acc2 a: depth sum, normal count, depth count, sample index (int bits)
                       //        b: first uv, has-uv flag, -
    float4* medium;    // albedo of the medium the path is inside (scenes with refraction only)
    Rec* q_trace[2];        // rays that need a traversal (ping-pong by bounce parity): entries
                            // {origin, slot (int bits)}, {direction, -}
    uint32_t* q_event[2];   // paths whose next segment's event is known, three queues of `slots`
                            // entries each: fog scatter, miss, surface hit (ping-pong)
    Rec* q_shadow[2];       // shadow rays (ping-pong), entries as q_trace
    uint32_t* q_late[2];    // finished samples whose last shadow ray is still to trace (ping-pong)
    uint32_t* q_resolve[2]; // finished samples without a shadow ray to trace (ping-pong)
    uint32_t* counts;       // this group's counters, kCount* below
    uint32_t rec_stride;    // slots of all groups (record kind k of slot s at k * rec_stride + s)
    uint8_t* ev_mark;       // per global slot, its event tag (event_mark): the event, the parity of
                            // the bounce that shades it and whether it waits for that bounce's
                            // traversal kernel
    uint32_t* q_sorted;     // this bounce's event queues in slot order, three of `slots` entries:
                            // the ready events first, then the others
    uint32_t pixel_tiles;   // 8x4 pixel tiles covering the image (slots / 32 when every pixel has one)
    uint32_t dynamic;       // 1: fewer slots than pixels -- a slot whose pixel is done takes the next
                            // unclaimed pixel (its tile-order index in the pixel record, acc2.b.w)
    uint32_t* pixel_cursor; // next unclaimed pixel (tile-order index), shared by the groups; the
                            // render's random-number stream in the word after it
    float4* defer[2];       // closest-hit queries the traversal kernel set aside at the end of its
                            // launch (ping-pong by bounce parity), kDeferF4 float4 each: resumed
                            // first by the next bounce's traversal kernel
    uint32_t defer_cap;     // entries per defer buffer (0: no deferral)
};

// Path and pixel records as one array per record kind (SR_REC_SOA = 1) or six / four records per
// slot back to back (0).  With event queues in slot order (SR_SORT_EVENTS = 1) neighbouring
// threads of the shade and finalize kernels then touch neighbouring records.
#ifndef SR_REC_SOA
#define SR_REC_SOA 0
#endif
#ifndef SR_SORT_EVENTS
#define SR_SORT_EVENTS 1
#endif

// Bytes of one set-aside traversal (sr_wave_kernels.cuh, kDeferF4): the query's state and its stack.
constexpr size_t kDeferBytes = 16 * (10 + (3 * 192 + 3) / 4);

// Events of a bounce are shaded in two phases (SR_SPLIT_PHASES = 1).  Ready events -- those decided
// where their ray was made (it missed the scene's root boxes) whose path has no shadow ray waiting
// for a traversal -- need nothing from the bounce's traversal kernel, so they are sorted and shaded
// on a parallel branch while it runs; the events the traversal decides, and those that wait for one
// of its shadow rays, are sorted and shaded after it.  The phases touch disjoint slots, and every
// path's own operations keep their order, so images are those of one phase.  0: one phase after
// the traversal.  (Needs the slot-ordered queues, SR_SORT_EVENTS.)  Measured on the 1080p fog
// workload: 514 vs 492 M samples/s, images identical; the ready fog kernel limited to 2 or 4 blocks
// per SM (SR_READY_BLOCKS) -18 % / -0.6 %.
#ifndef SR_SPLIT_PHASES
#define SR_SPLIT_PHASES 1
#endif
constexpr bool kSplitPhases = SR_SPLIT_PHASES && SR_SORT_EVENTS;

// Number of 32-bit counters at WaveState::counts, and their layout.
constexpr int kWaveCounters = 27;
enum : int {
    kCountResolve = 0,     // samples finished this bounce without a shadow ray to trace (parity 0;
                           // parity 1: kCountResolve1)
    kCountIter = 1,        // bounces run by the device loop
    kCountTraceFetch = 2,  // the trace kernel's fetch cursor
    kCountDone = 3,        // pixels whose AOVs are written (render progress)
    kCountTrace = 4,       // + parity: trace-queue length
    kCountShadow = 6,      // + parity: shadow-queue length
    kCountLate = 8,        // + parity: late finished samples
    kCountEvent = 10,      // + 3 * parity + event: event-queue lengths
    kCountSorted = 16,     // + event: fill cursors of the slot-ordered queues, ready events
    kCountDefer = 19,      // + parity: queries set aside in defer[parity] (may exceed defer_cap)
    kCountResolve1 = 21,   // as kCountResolve, parity 1
    kCountSortedLate = 22, // + event: fill cursors of the slot-ordered queues, the other events
    kCountPixel = 25,      // group 0: next unclaimed pixel of a render with fewer slots than pixels
    kCountSeed = 26,       // group 0, same renders: the random-number stream of the render (the
                           // bounce kernels' parameters stay seed-independent for graph reuse)
};
#if defined(__CUDACC__)
__host__ __device__
#endif
constexpr int count_resolve(int parity) { return parity ? kCountResolve1 : kCountResolve; }
// Paths alive for the bounce of the given parity: queued for a traversal, with a known event,
// finished with their last shadow ray still to trace, or with a traversal set aside.
#if defined(__CUDACC__)
__host__ __device__
#endif
inline uint32_t wave_deferred(const uint32_t* counts, uint32_t cap, int parity) {
    const uint32_t n = counts[kCountDefer + parity];
    return n < cap ? n : cap;
}
#if defined(__CUDACC__)
__host__ __device__
#endif
inline uint32_t wave_live(const uint32_t* counts, int parity, uint32_t defer_cap) {
    return counts[kCountTrace + parity] + counts[kCountEvent + 3 * parity] + counts[kCountEvent + 3 * parity + 1] +
           counts[kCountEvent + 3 * parity + 2] + counts[kCountLate + parity] +
           wave_deferred(counts, defer_cap, parity);
}

// Adjoint modes of the wavefront kernels (instantiated in sr_wave_adjoint.cu).  kAdjReplay: the
// render replays the paths of a finished render (same random numbers), records each sample's path
// vertices in the slot's vertex buffer and, when the sample ends, sweeps them back into the
// parameter gradients (dL/dI known).  kAdjRecord: a normal render that also keeps every sample's
// vertices (path-vertex checkpointing), swept later by launch_adjoint_checkpoint.
enum : int { kAdjNone = 0, kAdjReplay = 1, kAdjRecord = 2 };
constexpr int kAdjVertexF4 = 8;     // float4s per vertex record
constexpr int kAdjSampleShift = 8;  // record mode: the sample index rides in the path flags above bit 8

// Where the adjoint kernels read and write, kept in device memory (one per scene) so that a cached
// graph stays valid while the buffers change from call to call.
struct AdjPass {
    float4* vbuf;                 // vertex records: ((slot * samples_kept + sample) * vper + k) * 8 float4
    uint32_t vper;                // vertices per sample (bounces + 1)
    uint32_t samples_kept;        // samples kept per slot (replay 1, record max_samples)
    uint8_t* vcount;              // record: vertices of each (slot, sample)
    const float* d_image;         // replay: dL/dI (width x height x 3)
    const uint32_t* fwd_samples;  // replay: sample counts of the render replayed
    float* replay;                // replay: the re-rendered image (optional)
    int32_t tex_a, tex_r;         // albedo / roughness texture (-1: none)
    float* grad_a;                // dL/d(albedo texels), texture w x h x 3
    float* grad_r;                // dL/d(roughness texels), texture w x h x 3 (channel 0)
    float* grad_f;                // dL/d(fog density), one float
};

struct WaveLaunch {
    WaveState W[kWaveGroups];
    int groups;
    DevScene S;
    DevView V;
    DevParams P;
    DevAovs out;
    uint32_t* err;
    unsigned long long* counters;
    int grid_trace, grid_shadow, grid_finalize;
    int trace_block;    // threads per block of the traversal kernel (64, 128 or 256)
    int grid_shade[3];  // per event kernel (fog, miss, surface), or [0] for the sorted kernel
    int grid_ready[2];  // fog and miss kernels of the ready phase (run beside the traversal kernel)
    int general;  // 1: kernels with analytic shapes, transparency/media, normal maps, procedural sky
    uint32_t max_iters;
    uint32_t tail_paths;  // the bounce loop stops when at most this many paths are live; the tail
                          // kernel then finishes them, one thread per slot
    uint32_t* progress;   // host-mapped word the device loop publishes finished pixels to (or null)
    int adj_mode;         // kAdj*: the kernels of an adjoint pass
    const AdjPass* adj;   // device AdjPass of an adjoint pass
    cudaEvent_t trace_ev[2];  // host-loop renders with kernel timing: recorded on the launching stream
                              // right before and after each bounce's traversal kernel (else null)
    int grid_adj_shade[3], grid_adj_finalize;  // their grids
};

// Every group's state, as one kernel argument.
struct WaveGroups {
    WaveState W[kWaveGroups];
    int groups;
};

// Bounces per body of the graph's device-side loop (even: the tail after the loop takes parity 0).
#ifndef SR_GRAPH_BOUNCES
#define SR_GRAPH_BOUNCES 2
#endif
constexpr int kGraphBounces = SR_GRAPH_BOUNCES;
static_assert(kGraphBounces % 2 == 0, "whole pairs of bounces per loop body");

// The bounce loop hands over to the tail kernel at slots / SR_TAIL_DIV live paths (0: never).
#ifndef SR_TAIL_DIV
#define SR_TAIL_DIV 16
#endif

// Kernels launched per bounce and group: trace, late finalize, event sort and shade per event,
// finalize, and with split phases the ready phase's sort and fog and miss shade kernels (plus a
// shadow-loop kernel in scenes with transparent materials).
#ifndef SR_SPLIT_SHADE
#define SR_SPLIT_SHADE 1
#endif
// Trace queue reordered by ray-direction octant within chunks of 256 entries before each traversal
// (1) or left in producer order (0).
#ifndef SR_TRACE_OCTANT_SORT
#define SR_TRACE_OCTANT_SORT 0
#endif
// Kernels of a bounce that touch disjoint slots run on parallel graph branches (SR_PAR_SHADE = 1):
// the late finalize beside the ready phase's join and the waiting phase's sort, and the surface
// shade beside the fog and miss shade kernels of the waiting phase.
#ifndef SR_PAR_SHADE
#define SR_PAR_SHADE 1
#endif
// Side streams and events a bounce's branches use (one group), or the other groups' streams.
constexpr int kSideStreams = kWaveGroups > 3 ? kWaveGroups - 1 : 3;
constexpr int kForkEvents = kWaveGroups + 1 > 6 ? kWaveGroups + 1 : 6;
// The fog-scatter and miss events of a phase are shaded by one launch (SR_FOG_MISS_ONE = 1: warps
// padded between the two queues) or by one launch each (0).
#ifndef SR_FOG_MISS_ONE
#define SR_FOG_MISS_ONE 1
#endif
constexpr int kShadeLaunches = SR_SPLIT_SHADE ? (SR_FOG_MISS_ONE ? 2 : 3) : 1;  // waiting phase
constexpr int kReadyShadeLaunches = SR_SPLIT_SHADE && !SR_FOG_MISS_ONE ? 2 : 1;
constexpr int kWaveKernelsPerBounce = 3 + kShadeLaunches + (SR_SORT_EVENTS ? 1 : 0) +
                                      (kSplitPhases ? 1 + kReadyShadeLaunches : 0) + (SR_TRACE_OCTANT_SORT ? 1 : 0);

// Launch geometry chosen at run time (0 = the default: as many blocks per SM as fit).
struct WaveTune {
    int trace_per_sm;     // persistent traversal kernel
    int fog_per_sm;       // fog-event shade kernel
    int surface_per_sm;   // surface-event shade kernel
    uint32_t tail_div;    // the tail kernel takes over at slots / tail_div live paths (0 = SR_TAIL_DIV)
    uint32_t max_iters;   // bounce-loop cap (0 = the runaway guard)
    uint32_t max_actions; // per-traversal action cap (0 = kDefaultMaxActions)
    int trace_block;      // threads per block of the traversal kernel: 64, 128 or 256 (0 = 128)
    uint32_t max_slots;   // path slots in flight (queue capacity; 0 = one per pixel)
};
// Resident blocks per SM of the traversal, fog-shade and surface-shade kernels.
void wave_occupancy(bool general, int* trace, int* fog, int* surface);
void wave_grid_sizes(WaveLaunch& L, int sms, const WaveTune* tune = nullptr);
// Counters of every group (contiguous, kWaveCounters per group) cleared, first camera rays.
// Counters cleared and the first camera rays of every slot, drawn from random-number stream `seed`.
cudaError_t wave_init(const WaveLaunch& L, cudaStream_t st, uint32_t seed = 0);
// One bounce of every group: group 0 on `st`, the others on `side` streams forked from and
// joined back to `st` with the events in `fork` (one per group).
cudaError_t wave_bounce(const WaveLaunch& L, int cur, cudaStream_t st, const cudaStream_t* side, const cudaEvent_t* fork);
// The tail kernel over the live paths of parity `cur` (at most L.tail_paths of them).
cudaError_t wave_tail(const WaveLaunch& L, int cur, cudaStream_t st);
cudaError_t wave_build_graph(const WaveLaunch& L, cudaStream_t capture_stream, const cudaStream_t* side,
                             const cudaEvent_t* fork, cudaGraphExec_t* exec_out);
// One graph with an independent bounce loop + tail per launch description (batched rendering).
cudaError_t wave_build_graph_batch(const WaveLaunch* Ls, int n, cudaStream_t capture_stream, const cudaStream_t* side,
                                   const cudaEvent_t* fork, cudaGraphExec_t* exec_out);

// The adjoint forms of a bounce's kernels other than the traversal and the sorts (sr_wave_adjoint.cu):
// the late finalize (late = true) or the finalize, the shade kernels of a phase, the tail; grids
// from their occupancy.
void wave_adj_finalize(const WaveLaunch& L, const WaveState& W, int cur, cudaStream_t st, bool late);
// `events`: bit 0 fog, bit 1 miss, bit 2 surface (phase 0 never has surface events).
void wave_adj_shade(const WaveLaunch& L, const WaveState& W, int cur, int phase, cudaStream_t st, int events = 7);
cudaError_t wave_adj_tail(const WaveLaunch& L, int cur, cudaStream_t st);
void wave_adj_grid_sizes(WaveLaunch& L, int sms);
// Closest hits of n world rays (6 floats each, device) through the persistent traversal loop of the
// wavefront renderer; `entries` (n ray-queue records) and `fetch` (one word) are scratch.
cudaError_t launch_trace_persistent(const DevScene& S, bool general, const float* rays, uint32_t n, Rec* entries,
                                    uint32_t* fetch, int32_t* obj, int32_t* tri, float* dist, float* uv,
                                    uint32_t* err, int sms, cudaStream_t st);
// The traversal kernel at 64 or 256 threads per block (sr_wave_trace.cu) and its resident blocks per SM.
void wave_trace_block(const WaveLaunch& L, const WaveState& W, int cur, cudaStream_t st, bool loop_shadows);
int wave_trace_occupancy(bool general, int block);
// Record mode's sweep: every kept sample of every slot, once dL/dI of the recorded render is known
// (`samples`: that render's sample counts).
cudaError_t launch_adjoint_checkpoint(const WaveLaunch& L, const float* d_image, const uint32_t* samples,
                                      cudaStream_t st);

}  // namespace sr

// sr_wavefront.cu — wavefront form of the per-pixel path loop.
//
// Renderer.Render (renderer.cs:153-229) + Scene.Sample (scene.cs:627-741) are split into kernels
// over per-path state records, one slot per pixel.  Per bounce:
//
//   trace    : one persistent traversal loop over two ray queues: the closest hit of every path
//              ray that enters the root boxes of the scene BVH (Scene.Trace -> Bvh.Intersect),
//              followed by its segment's event -- fog scatter (the free-flight distance is drawn
//              here, the segment's first RNG draw), surface hit or miss -- into one queue per
//              event; and the shadow rays of the previous bounce's light samples
//              (ShadowTransmittance scene.cs:576-600 x fog transmittance).  A ray that misses the
//              root boxes is decided where it is made: in foggy scenes most rays start far outside
//              the scene and leave it
//   late     : samples that finished last bounce with a shadow ray still to trace: its
//              contribution, the pixel statistics, the adaptive stop, the next camera ray
//   shade    : one kernel per event: first the NEE contribution of the previous segment if its
//              shadow ray was traced since, then the event's logic: light sample (a shadow ray that
//              misses the root boxes contributes at once, others are queued), Russian roulette,
//              scatter
//   finalize : samples that finished this bounce without a shadow ray to trace: pixel statistics,
//              adaptive stop, next camera ray or the AOV write
//
// Sorting paths by event makes every shade warp run one branch: fog scatter, surface and miss
// logic differ completely, and in foggy scenes most segments end in the fog while a few hit
// surfaces, so unsorted warps nearly always ran all three.
//
// The trace loop is persistent: a lane that finishes its ray takes the next one from the queues
// at once (refilled per warp with one atomic), so warps stay full although ray lengths differ by
// orders of magnitude, and shadow rays fill the SMs while the last long path rays finish.
//
// Paths are compacted into queues between kernels with aggregated atomics (per block in the
// grid-stride kernels, per warp and 32 entries in the persistent ones), so every launch works on
// dense queues.  Every per-path operation -- RNG draws, float operation order, the order in
// which contributions are added -- is the megakernel's (sr_path.cuh), so the two forms produce
// identical images: a segment's NEE contribution is added before anything of the next segment
// (or the end of its sample) touches the radiance, exactly where the megakernel adds it.
//
// The bounce loop runs either as a host loop (one launch per kernel per bounce, the host reads the
// live-path count after every bounce) or as a CUDA graph whose conditional WHILE node repeats the
// bounce kernels on the device (no host round trip per bounce).  Either hands the last few live
// paths to a tail kernel that runs each to completion.
#include <cuda_runtime.h>

#include "sr_wave_kernels.cuh"

namespace sr {

// The pixel cursor of a render with fewer slots than pixels -- the pixels after the slots' own --
// and the render's random-number stream, which the finalize kernels seed claimed pixels from.
__global__ void k_wave_cursor(uint32_t* cursor, uint32_t first, uint32_t seed) {
    cursor[0] = first;
    cursor[kCountSeed - kCountPixel] = seed;
}

__global__ void __launch_bounds__(128) k_wave_init(WaveState W, DevScene S, DevView V, DevParams P) {
    __shared__ uint32_t sh[2][1][kBlockWarps + 1];
    const uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;  // index among this group's slots
    const uint32_t s = ((li >> 5) * W.groups + W.group) * 32u + (li & 31u);
    bool valid = false;
    if (li < W.slots) {
        // slot s starts on pixel s (or, with fewer slots than pixels, on the next unclaimed pixel
        // when pixel s lies outside the image)
        uint32_t x, y, p = s;
        pixel_xy(W, p, x, y);
        valid = x < P.width && y < P.height;
        if (!valid && W.dynamic) {
            p = claim_pixel(W, P);
            valid = p != ~0u;
            if (valid) pixel_xy(W, p, x, y);
        }
        if (valid) {
            Rng rng = rng_seed(x, y, P.seed);
            Ray ray = camera_ray(V, P, x, y, rng);
            begin_sample(W, s, ray, rng, fog_scatter_t(S, ray, rng));
            float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            st_rec(&W.pix[pix(W, s, X_ACC)], Rec{z, z});
            st_rec(&W.pix[pix(W, s, X_ACC + 1)], Rec{z, z});
            // counts and sample index start at 0 (int bits); the pixel's tile-order index in the last word
            st_rec(&W.pix[pix(W, s, X_ACC + 2)], Rec{z, make_float4(0.f, 0.f, 0.f, fbits(p))});
        }
    }
    uint32_t off[1];
    block_offsets<1>({&W.counts[kCountTrace]}, {valid}, sh, 0u, off);
    if (valid) {
        Rec r = ld_rec(&W.rec[rix(W, s, R_RAY)]);
        W.q_trace[0][off[0]] = ray_entry(s, V3{r.a.x, r.a.y, r.a.z}, V3{r.b.x, r.b.y, r.b.z}, r.b.w);
    }
}

// The event queues of this bounce in slot order, so that the shade kernels' neighbouring threads
// work on neighbouring slots: every producer of an event also tags the slot with the event, the
// parity of the bounce that shades it and whether it waits for that bounce's traversal kernel
// (event_mark), and k_event_sort scans the slots in order -- four per thread -- appending each slot
// tagged for this bounce and phase to its event's sorted queue (one atomic per block and event;
// inside a block's run the order is the slot order) and clearing its tag.  Phase 0 takes the ready
// events (running beside the traversal kernel, which meanwhile tags other slots: a tag it has not
// written yet reads as 0 or as a waiting tag, both left alone); phase 1 takes the rest of the
// bounce's events and places them after phase 0's.  Tags for the next bounce (from a late finalize)
// are left in place.
//
// Slots one thread of k_event_sort scans (4, 8 or 16: consecutive slots of one 32-slot tile, their
// tags read as one vector when they are all inside the group; the tags it takes are cleared byte
// by byte, since the traversal kernel may be tagging the others).  Measured on the 1080p fog
// workload (graph mode): 4 per thread 527.7, 8 525.8, 16 523.1 M samples/s -- the kernel wants
// the parallelism more than fewer blocks and atomics.
#ifndef SR_SORT_PER_THREAD
#define SR_SORT_PER_THREAD 4
#endif
constexpr int kSortPerThread = SR_SORT_PER_THREAD;
static_assert(kSortPerThread == 4 || kSortPerThread == 8 || kSortPerThread == 16, "k_event_sort slots per thread");
constexpr int kSortBlock = 256;

__global__ void __launch_bounds__(kSortBlock) k_event_sort(WaveState W, int cur, int phase) {
    __shared__ uint32_t warp_n[3][kSortBlock / 32];
    __shared__ uint32_t base[3];
    constexpr int K = kSortPerThread;
    const uint32_t li = K * (blockIdx.x * blockDim.x + threadIdx.x);  // group-local slot index
    const uint32_t s0 = ((li >> 5) * W.groups + W.group) * 32u + (li & 31u);  // K consecutive slots
    // the K tags (one byte each)
    uint32_t tag[K / 4];
    if (li + K <= W.slots) {
        if constexpr (K == 16) {
            const uint4 v = *reinterpret_cast<const uint4*>(W.ev_mark + s0);
            tag[0] = v.x, tag[1] = v.y, tag[2] = v.z, tag[3] = v.w;
        } else if constexpr (K == 8) {
            const uint2 v = *reinterpret_cast<const uint2*>(W.ev_mark + s0);
            tag[0] = v.x, tag[1] = v.y;
        } else {
            tag[0] = *reinterpret_cast<const uint32_t*>(W.ev_mark + s0);
        }
    } else {
#pragma unroll
        for (int q = 0; q < K / 4; ++q) {
            tag[q] = 0u;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (li + 4 * q + j < W.slots) tag[q] |= (uint32_t)W.ev_mark[s0 + 4 * q + j] << (8 * j);
        }
    }
    uint32_t evs = 0;  // 2 bits per slot: the slot's event of this bounce and phase, 3 = none
    uint32_t cnt[3] = {0, 0, 0};
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const uint32_t m = (tag[j >> 2] >> (8 * (j & 3))) & 0xffu;
        // m = 1 + event + 3 x parity + 6 x wait: the event of this bounce and phase, else >= 3
        const uint32_t t = phase == 0 ? m - 1u - 3u * (uint32_t)cur : (m > 6u ? m - 7u : m - 1u) - 3u * (uint32_t)cur;
        const uint32_t e = m == 0u ? 3u : (t < 3u ? t : 3u);
        evs |= e << (2 * j);
        if (e < 3u) {
            W.ev_mark[s0 + j] = 0;  // byte stores: other slots' tags may be written meanwhile
            ++cnt[e];
        }
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t pre[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        uint32_t v = cnt[e];  // inclusive warp scan
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= (uint32_t)d) v += t;
        }
        pre[e] = v - cnt[e];
        if (lane == 31) warp_n[e][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        uint32_t t = 0;
        for (int w = 0; w < kSortBlock / 32; ++w) t += warp_n[threadIdx.x][w];
        const uint32_t first = phase == 0 ? 0u : W.counts[kCountSorted + threadIdx.x];
        base[threadIdx.x] =
            first + (t ? atomicAdd(&W.counts[(phase == 0 ? kCountSorted : kCountSortedLate) + threadIdx.x], t) : 0u);
    }
    __syncthreads();
    uint32_t off[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        off[e] = base[e] + pre[e];
        for (uint32_t w = 0; w < warp; ++w) off[e] += warp_n[e][w];
    }
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const uint32_t e = (evs >> (2 * j)) & 3u;
        if (e < 3u) W.q_sorted[(size_t)e * W.slots + off[e]++] = s0 + j;
    }
}

static unsigned sort_blocks(const WaveState& W) {
    return (W.slots + kSortBlock * kSortPerThread - 1) / (kSortBlock * kSortPerThread);
}

// Closest hits of world rays through the renderer's own persistent traversal loop (the ray
// query of sr_scene_trace outside the megakernel render mode): the rays become ray-queue entries,
// then one persistent launch answers them, each lane writing its query's result.
__global__ void k_pack_rays(const float* rays, uint32_t n, Rec* q) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rays + (size_t)i * 6;
    q[i] = ray_entry(i, V3{r[0], r[1], r[2]}, V3{r[3], r[4], r[5]}, 0.f);
}

template <bool GENERAL>
__global__ void __launch_bounds__(128, SR_TRACE_MIN_BLOCKS)
    k_trace_rays_persistent(DevScene S, const Rec* q, uint32_t n, uint32_t* fetch, int32_t* obj, int32_t* tri,
                            float* dist, float* uv, uint32_t* err) {
    Ctr c;
#pragma unroll
    for (int i = 0; i < SR_COUNTER_COUNT; ++i) c.v[i] = 0;
    persistent_queries<false, GENERAL>(
        S, q, n, nullptr, 0u, fetch, c, err, [&](bool) {},
        [&](uint32_t i, uint32_t, bool, const Hit& h, const Ray&) {
            if (h.obj < 0) {
                obj[i] = -1, tri[i] = -1, dist[i] = __int_as_float(0x7f800000), uv[2 * i] = 0.f, uv[2 * i + 1] = 0.f;
            } else {
                obj[i] = S.objects[h.obj].index;
                tri[i] = h.tri >= 0 ? __float_as_int(__ldg(S.tris + 3 * h.tri).w) : -1;
                dist[i] = h.dist, uv[2 * i] = h.u, uv[2 * i + 1] = h.v;
            }
            return -1;
        },
        [&](uint32_t, int) {});
}

cudaError_t launch_trace_persistent(const DevScene& S, bool general, const float* rays, uint32_t n, Rec* entries,
                                    uint32_t* fetch, int32_t* obj, int32_t* tri, float* dist, float* uv,
                                    uint32_t* err, int sms, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    k_pack_rays<<<(n + 127) / 128, 128, 0, st>>>(rays, n, entries);
    int per_sm = 0;
    if (general) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_rays_persistent<true>, 128, 0);
        k_trace_rays_persistent<true><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(S, entries, n, fetch, obj, tri,
                                                                                    dist, uv, err);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_rays_persistent<false>, 128, 0);
        k_trace_rays_persistent<false><<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(S, entries, n, fetch, obj,
                                                                                     tri, dist, uv, err);
    }
    return cudaGetLastError();
}

// Condition of the device-side bounce loop: continue while more than `tail` paths of all groups
// are live (the rest go to the tail kernel) and the bounce cap (a runaway guard of twice
// (max_samples + 1) * (bounces + 2) per pixel) is not reached.  `counts` holds the groups' counters one after another.
__global__ void k_wave_continue(cudaGraphConditionalHandle handle, uint32_t* counts, int groups, uint32_t tail,
                                uint32_t max_iters, uint32_t* err, uint32_t* progress, uint32_t defer_cap) {
    uint32_t it = counts[kCountIter] + kGraphBounces;  // bounces per loop body
    counts[kCountIter] = it;
    uint32_t live = 0, done = 0;
    for (int g = 0; g < groups; ++g) {
        live += wave_live(counts + g * kWaveCounters, 0, defer_cap);  // next bounce: parity 0
        done += counts[g * kWaveCounters + kCountDone];
    }
    if (progress) *(volatile uint32_t*)progress = done;  // host-mapped: read by sr_render_progress
    bool more = live > tail;
    if (more && it >= max_iters) {
        atomicOr(err, SR_DEVERR_LOOP);
        more = false;
    }
    cudaGraphSetConditional(handle, more ? 1u : 0u);
}

// ---- launchers ------------------------------------------------------------------------------------
// The trace queue of parity cur reordered in place by ray-direction octant (sign bits of d) within
// each chunk of 256 entries, keeping the producer order inside an octant, so that the lanes of a
// traversal warp take rays heading the same way.  Results are per slot, so the order of the queue
// does not change them.
__global__ void __launch_bounds__(256) k_trace_octant_sort(WaveState W, int cur) {
    __shared__ uint32_t wcount[8][8];  // [warp][octant]
    __shared__ uint32_t base[8][8];
    const uint32_t len = W.counts[kCountTrace + cur];
    const uint32_t start = blockIdx.x * 256u;
    if (start >= len) return;  // uniform over the block
    const uint32_t i = start + threadIdx.x;
    const bool valid = i < len;
    Rec e;
    int oct = 8;  // none
    if (valid) {
        e = ld_rec(&W.q_trace[cur][i]);
        oct = (e.b.x < 0.0f ? 1 : 0) | (e.b.y < 0.0f ? 2 : 0) | (e.b.z < 0.0f ? 4 : 0);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    uint32_t rank = 0;
    for (int o = 0; o < 8; ++o) {
        const unsigned m = __ballot_sync(0xffffffffu, oct == o);
        if (oct == o) rank = __popc(m & below);
        if (lane == 0) wcount[warp][o] = __popc(m);
    }
    __syncthreads();  // every entry of the chunk is in registers before any is written back
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int o = 0; o < 8; ++o)
            for (int w = 0; w < 8; ++w) {
                base[w][o] = acc;
                acc += wcount[w][o];
            }
    }
    __syncthreads();
    if (valid) st_rec(&W.q_trace[cur][start + base[warp][oct] + rank], e);
}

// The shade kernels of one phase of a bounce (phase 0: the ready events, fog and miss only; a
// surface event always comes from the traversal kernel); `events`: bit 0 fog, bit 1 miss, bit 2
// surface.
template <bool COUNT, bool GENERAL>
static void launch_shade(const WaveLaunch& L, const WaveState& W, int cur, int phase, cudaStream_t st, int events = 7) {
    if (L.adj_mode != kAdjNone) {
        wave_adj_shade(L, W, cur, phase, st, events);
        return;
    }
    if (SR_SPLIT_SHADE && SR_FOG_MISS_ONE && (events & 3) == 3) {
        k_wave_shade<COUNT, GENERAL, EV_FOG_MISS><<<phase == 0 ? L.grid_ready[0] : L.grid_shade[0], 128, 0, st>>>(
            W, L.S, L.P, cur, phase, L.err, L.counters, nullptr);
        if (phase == 1 && (events & 4))
            k_wave_shade<COUNT, GENERAL, EV_SURF>
                <<<L.grid_shade[2], 128, 0, st>>>(W, L.S, L.P, cur, phase, L.err, L.counters, nullptr);
    } else if (SR_SPLIT_SHADE) {
        if (events & 1)
            k_wave_shade<COUNT, GENERAL, EV_FOG><<<phase == 0 ? L.grid_ready[0] : L.grid_shade[0], 128, 0, st>>>(
                W, L.S, L.P, cur, phase, L.err, L.counters, nullptr);
        if (events & 2)
            k_wave_shade<COUNT, GENERAL, EV_MISS><<<phase == 0 ? L.grid_ready[1] : L.grid_shade[1], 128, 0, st>>>(
                W, L.S, L.P, cur, phase, L.err, L.counters, nullptr);
        if (phase == 1 && (events & 4))
            k_wave_shade<COUNT, GENERAL, EV_SURF>
                <<<L.grid_shade[2], 128, 0, st>>>(W, L.S, L.P, cur, phase, L.err, L.counters, nullptr);
    } else if (events == 7) {
        k_wave_shade<COUNT, GENERAL, -1>
            <<<phase == 0 ? L.grid_ready[0] : L.grid_shade[0], 128, 0, st>>>(W, L.S, L.P, cur, phase, L.err,
                                                                           L.counters, nullptr);
    }
}

// `to` waits for the work queued on `from` so far (event ev).
static cudaError_t stream_join(cudaStream_t to, cudaStream_t from, cudaEvent_t ev) {
    cudaError_t e = cudaEventRecord(ev, from);
    return e == cudaSuccess ? cudaStreamWaitEvent(to, ev, 0) : e;
}

// One bounce of group W on stream st.  With side streams (side[0..2], events fork[0..5]) its
// kernels form this graph of branches; without them they run in the same order on st:
//
//   st:      trace ----------> [late finalize on side[1]] ---+
//   side[0]:  sort + shade ready events ---+                  |
//   st:                                    +-> sort rest -> fog + miss shade -+-> finalize
//   side[2]:                                            +-> surface shade ----+
//
// Every branch touches its own slots (the ready events', the late samples', the waiting events'
// by event), so the order between branches does not change any path.
template <bool COUNT, bool GENERAL>
static cudaError_t launch_bounce(const WaveLaunch& L, const WaveState& W, int cur, cudaStream_t st,
                                 const cudaStream_t* side, const cudaEvent_t* fork) {
    cudaError_t e = cudaSuccess;
    if (kSplitPhases) {
        cudaStream_t sa = side ? side[0] : st;
        if (side && (e = stream_join(side[0], st, fork[0])) != cudaSuccess) return e;
        k_event_sort<<<sort_blocks(W), kSortBlock, 0, sa>>>(W, cur, 0);
        launch_shade<COUNT, GENERAL>(L, W, cur, 0, sa);
    }
    if (SR_TRACE_OCTANT_SORT) k_trace_octant_sort<<<(W.slots + 255) / 256, 256, 0, st>>>(W, cur);
    if (L.trace_ev[0] && (e = cudaEventRecord(L.trace_ev[0], st)) != cudaSuccess) return e;
    const bool loop_shadows = GENERAL && L.S.has_transparent;
    if (!COUNT && L.trace_block != 128) {
        wave_trace_block(L, W, cur, st, loop_shadows);
    } else if (loop_shadows) {
        k_wave_trace<COUNT, GENERAL, false><<<L.grid_trace, 128, 0, st>>>(W, L.S, cur, L.err, L.counters);
    } else {
        k_wave_trace<COUNT, GENERAL, true><<<L.grid_trace, 128, 0, st>>>(W, L.S, cur, L.err, L.counters);
    }
    if (loop_shadows) k_wave_shadow_loop<COUNT, GENERAL><<<L.grid_shadow, 128, 0, st>>>(W, L.S, cur, L.err, L.counters);
    if (L.trace_ev[1] && (e = cudaEventRecord(L.trace_ev[1], st)) != cudaSuccess) return e;
    // the late finalize: the samples whose last shadow ray the traversal kernel just traced
    const bool par = SR_PAR_SHADE && side != nullptr;
    cudaStream_t sl = par ? side[1] : st;
    if (par && (e = stream_join(side[1], st, fork[1])) != cudaSuccess) return e;
    if (L.adj_mode != kAdjNone)
        wave_adj_finalize(L, W, cur, sl, true);
    else
        k_wave_finalize<COUNT, GENERAL, true><<<L.grid_finalize, 128, 0, sl>>>(W, L.S, L.V, L.P, L.out, cur, L.err,
                                                                               L.counters, nullptr);
    if (kSplitPhases && side && (e = stream_join(st, side[0], fork[2])) != cudaSuccess) return e;
    if (SR_SORT_EVENTS) k_event_sort<<<sort_blocks(W), kSortBlock, 0, st>>>(W, cur, 1);
    if (par && SR_SPLIT_SHADE) {
        if ((e = stream_join(side[2], st, fork[3])) != cudaSuccess) return e;
        launch_shade<COUNT, GENERAL>(L, W, cur, 1, side[2], 4);
        launch_shade<COUNT, GENERAL>(L, W, cur, 1, st, 3);
        if ((e = stream_join(st, side[2], fork[4])) != cudaSuccess) return e;
    } else {
        launch_shade<COUNT, GENERAL>(L, W, cur, 1, st);
    }
    if (par && (e = stream_join(st, side[1], fork[5])) != cudaSuccess) return e;
    if (L.adj_mode != kAdjNone)
        wave_adj_finalize(L, W, cur, st, false);
    else
        k_wave_finalize<COUNT, GENERAL, false><<<L.grid_finalize, 128, 0, st>>>(W, L.S, L.V, L.P, L.out, cur, L.err,
                                                                                L.counters, nullptr);
    return cudaSuccess;
}

static cudaError_t launch_group_bounces(const WaveLaunch& L, const WaveState& W, int cur, int n, cudaStream_t st,
                                        const cudaStream_t* side, const cudaEvent_t* fork) {
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < n && e == cudaSuccess; ++i, cur ^= 1) {
        if (L.general)
            e = L.counters ? launch_bounce<true, true>(L, W, cur, st, side, fork)
                           : launch_bounce<false, true>(L, W, cur, st, side, fork);
        else
            e = L.counters ? launch_bounce<true, false>(L, W, cur, st, side, fork)
                           : launch_bounce<false, false>(L, W, cur, st, side, fork);
    }
    return e;
}

// n bounces of every group starting at parity cur.  One group: its bounces on st, their parallel
// branches on side[0..2] (events fork[0..5]).  Several groups: group 0 on st, group g on
// side[g - 1], forked from st by fork[0] and joined back by fork[g]; each group's kernels then run
// one after the other.
static cudaError_t launch_bounces(const WaveLaunch& L, int cur, int n, cudaStream_t st, const cudaStream_t* side,
                                  const cudaEvent_t* fork) {
    cudaError_t e = cudaSuccess;
    if (L.groups == 1) {
        e = launch_group_bounces(L, L.W[0], cur, n, st, side, fork);
        return e != cudaSuccess ? e : cudaGetLastError();
    }
    e = cudaEventRecord(fork[0], st);
    for (int g = 1; g < L.groups && e == cudaSuccess; ++g) e = cudaStreamWaitEvent(side[g - 1], fork[0], 0);
    if (e != cudaSuccess) return e;
    for (int g = 0; g < L.groups && e == cudaSuccess; ++g)
        e = launch_group_bounces(L, L.W[g], cur, n, g == 0 ? st : side[g - 1], nullptr, fork);
    for (int g = 1; g < L.groups && e == cudaSuccess; ++g) {
        e = cudaEventRecord(fork[g], side[g - 1]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, fork[g], 0);
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

#ifndef SR_READY_BLOCKS
#define SR_READY_BLOCKS 0
#endif

template <bool GENERAL>
static void occupancy(int* b) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[0], k_wave_trace<false, GENERAL, true>, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[1], k_wave_shadow_loop<false, GENERAL>, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[2], k_wave_finalize<false, GENERAL, false>, 128, 0);
    if (SR_SPLIT_SHADE) {
        if (SR_FOG_MISS_ONE)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[3], k_wave_shade<false, GENERAL, EV_FOG_MISS>, 128, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[3], k_wave_shade<false, GENERAL, EV_FOG>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[4], k_wave_shade<false, GENERAL, EV_MISS>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[5], k_wave_shade<false, GENERAL, EV_SURF>, 128, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[3], k_wave_shade<false, GENERAL, -1>, 128, 0);
    }
}

void wave_occupancy(bool general, int* trace, int* fog, int* surface) {
    int b[6] = {0, 0, 0, 0, 0, 0};
    if (general)
        occupancy<true>(b);
    else
        occupancy<false>(b);
    *trace = b[0], *fog = b[3], *surface = b[5];
}

void wave_grid_sizes(WaveLaunch& L, int sms, const WaveTune* tune) {
    int b[6] = {0, 0, 0, 0, 0, 0};
    if (L.general)
        occupancy<true>(b);
    else
        occupancy<false>(b);
    // the traversal kernel's block size (counting renders keep the default 128)
    L.trace_block = 128;
    if (tune && (tune->trace_block == 64 || tune->trace_block == 256) && !L.counters) {
        L.trace_block = tune->trace_block;
        b[0] = wave_trace_occupancy(L.general != 0, L.trace_block);
    }
    if (tune) {  // a tuned count never exceeds what fits
        auto pick = [](int want, int fit) { return want > 0 && want < fit ? want : fit; };
        b[0] = pick(tune->trace_per_sm, b[0]);
        b[3] = pick(tune->fog_per_sm, b[3]);
        b[5] = pick(tune->surface_per_sm, b[5]);
    }
    for (int& v : b) v = sms * (v > 0 ? v : 1);
    L.grid_trace = b[0];
    L.grid_shadow = b[1];
    L.grid_finalize = b[2];
    L.grid_shade[0] = b[3];
    L.grid_shade[1] = b[4];
    L.grid_shade[2] = b[5];
    // the ready phase's fog kernel shares the SMs with the traversal kernel: SR_READY_BLOCKS blocks
    // per SM (0: as many as fit alone)
    L.grid_ready[0] = SR_READY_BLOCKS > 0 && sms * SR_READY_BLOCKS < b[3] ? sms * SR_READY_BLOCKS : b[3];
    L.grid_ready[1] = b[4];
}

cudaError_t wave_init(const WaveLaunch& L, cudaStream_t st, uint32_t seed) {
    DevParams P = L.P;  // the seed only reaches the first camera rays, outside any cached graph
    P.seed = seed;
    cudaError_t e = cudaMemsetAsync(L.W[0].counts, 0, (size_t)L.groups * kWaveCounters * sizeof(uint32_t), st);
    if (e == cudaSuccess && SR_SORT_EVENTS) e = cudaMemsetAsync(L.W[0].ev_mark, 0, L.W[0].rec_stride, st);
    if (e != cudaSuccess) return e;
    if (L.W[0].dynamic) k_wave_cursor<<<1, 1, 0, st>>>(L.W[0].pixel_cursor, L.W[0].rec_stride, seed);
    for (int g = 0; g < L.groups; ++g)
        if (L.W[g].slots) k_wave_init<<<(L.W[g].slots + 127) / 128, 128, 0, st>>>(L.W[g], L.S, L.V, P);
    return cudaGetLastError();
}

cudaError_t wave_bounce(const WaveLaunch& L, int cur, cudaStream_t st, const cudaStream_t* side, const cudaEvent_t* fork) {
    return launch_bounces(L, cur, 1, st, side, fork);
}

cudaError_t wave_tail(const WaveLaunch& L, int cur, cudaStream_t st) {
    WaveGroups G;
    for (int g = 0; g < kWaveGroups; ++g) G.W[g] = L.W[g];
    G.groups = L.groups;
    const int grid = (int)((L.tail_paths + 127) / 128);
    if (grid == 0) return cudaSuccess;
    if (L.adj_mode != kAdjNone) return wave_adj_tail(L, cur, st);
    if (L.general) {
        if (L.counters)
            k_wave_tail<true, true><<<grid, 128, 0, st>>>(G, L.S, L.V, L.P, L.out, cur, L.err, L.counters, nullptr);
        else
            k_wave_tail<false, true><<<grid, 128, 0, st>>>(G, L.S, L.V, L.P, L.out, cur, L.err, L.counters, nullptr);
    } else {
        if (L.counters)
            k_wave_tail<true, false><<<grid, 128, 0, st>>>(G, L.S, L.V, L.P, L.out, cur, L.err, L.counters, nullptr);
        else
            k_wave_tail<false, false><<<grid, 128, 0, st>>>(G, L.S, L.V, L.P, L.out, cur, L.err, L.counters, nullptr);
    }
    return cudaGetLastError();
}

// One graph holding, per launch description, the device-side bounce loop (a conditional WHILE node
// whose body is two bounces and the loop condition) followed by its tail kernel.  The branches of
// different descriptions have no edges between them, so the GPU runs them side by side: one
// scene's small bounces and kernel ramp-downs overlap another's work.
cudaError_t wave_build_graph_batch(const WaveLaunch* Ls, int n, cudaStream_t capture_stream, const cudaStream_t* side,
                                   const cudaEvent_t* fork, cudaGraphExec_t* exec_out) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e != cudaSuccess) return e;
    for (int i = 0; i < n && e == cudaSuccess; ++i) {
        const WaveLaunch& L = Ls[i];
        cudaGraphConditionalHandle handle;
        e = cudaGraphConditionalHandleCreate(&handle, graph, 1u, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) break;
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
        if (e != cudaSuccess) break;
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(capture_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) break;
        // kGraphBounces bounces per group on parallel branches, joined before the loop condition
        cudaError_t e1 = launch_bounces(L, 0, kGraphBounces, capture_stream, side, fork);
        k_wave_continue<<<1, 1, 0, capture_stream>>>(handle, L.W[0].counts, L.groups, L.tail_paths, L.max_iters, L.err,
                                                     L.progress, L.W[0].defer_cap);
        cudaGraph_t captured = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(capture_stream, &captured);
        e = e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : cudaGetLastError());
        if (e != cudaSuccess) break;
        // after the loop: the tail kernel over the paths left (parity 0 after whole bodies)
        e = cudaStreamBeginCaptureToGraph(capture_stream, graph, &node, nullptr, 1, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) break;
        e1 = wave_tail(L, 0, capture_stream);
        e2 = cudaStreamEndCapture(capture_stream, &captured);
        e = e1 != cudaSuccess ? e1 : e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec_out, graph, 0);
    cudaGraphDestroy(graph);
    return e;
}

cudaError_t wave_build_graph(const WaveLaunch& L, cudaStream_t capture_stream, const cudaStream_t* side,
                             const cudaEvent_t* fork, cudaGraphExec_t* exec_out) {
    return wave_build_graph_batch(&L, 1, capture_stream, side, fork, exec_out);
}

}  // namespace sr

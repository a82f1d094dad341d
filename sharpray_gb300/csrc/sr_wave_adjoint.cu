// sr_wave_adjoint.cu — the wavefront renderer's kernels in their adjoint forms (no counterpart in the
// reference, which has no derivatives).
//
// An adjoint pass is a wavefront render whose shade, finalize and tail kernels also write one record
// per path vertex (sr_wave_kernels.cuh, adj_vertex): the throughput entering it, what it adds to the
// radiance and the derivatives of that and of its scatter weight with respect to the albedo and
// roughness lookups and the fog density, the score of the free flight into it.  The traversal kernel
// is the render's own (launched from sr_wavefront.cu).  Two forms:
//
//   replay (kAdjReplay): the paths of a finished render are rendered again with the same random
//     numbers, one sample at a time per slot; when a sample ends, the finalize (or tail) kernel
//     sweeps its vertices back to the camera (adjoint_sweep) with dL/dI of the pixel, adding into
//     the texel gradients by atomics.  Memory: slots x (bounces + 1) records.  This is the per-pixel
//     replay of sr_adjoint.cu with the traversal and shading organised as the render's wavefront,
//     so it runs at the render's speed instead of the divergent one-thread-per-pixel loop's.
//   record (kAdjRecord): a normal render that keeps every sample's vertices (path-vertex
//     checkpointing); once dL/dI of its image is known, k_adjoint_checkpoint sweeps them without
//     tracing anything again.  Memory: slots x max_samples x (bounces + 1) records, which the
//     GB300's HBM holds for a 768x768 view at 32 samples (21.7 GB).
//
// Both differentiate the same estimator as sr_adjoint.cu (sampling, roulette decisions, pdfs and MIS
// weights held fixed; score terms for the fog density).
#include <cuda_runtime.h>

#include "sr_wave_kernels.cuh"

namespace sr {

template <bool GENERAL, int ADJ>
static void adj_finalize(const WaveLaunch& L, const WaveState& W, int cur, cudaStream_t st, bool late) {
    if (late)
        k_wave_finalize<false, GENERAL, true, ADJ>
            <<<L.grid_adj_finalize, 128, 0, st>>>(W, L.S, L.V, L.P, L.out, cur, L.err, nullptr, L.adj);
    else
        k_wave_finalize<false, GENERAL, false, ADJ>
            <<<L.grid_adj_finalize, 128, 0, st>>>(W, L.S, L.V, L.P, L.out, cur, L.err, nullptr, L.adj);
}

void wave_adj_finalize(const WaveLaunch& L, const WaveState& W, int cur, cudaStream_t st, bool late) {
    if (L.general)
        L.adj_mode == kAdjReplay ? adj_finalize<true, kAdjReplay>(L, W, cur, st, late)
                                 : adj_finalize<true, kAdjRecord>(L, W, cur, st, late);
    else
        L.adj_mode == kAdjReplay ? adj_finalize<false, kAdjReplay>(L, W, cur, st, late)
                                 : adj_finalize<false, kAdjRecord>(L, W, cur, st, late);
}

// The shade kernels of one phase of a bounce (phase 0: the ready events, which are never surface
// events).
template <bool GENERAL, int ADJ>
static void adj_shade(const WaveLaunch& L, const WaveState& W, int cur, int phase, cudaStream_t st, int events) {
    if (events & 1)
        k_wave_shade<false, GENERAL, EV_FOG, ADJ>
            <<<L.grid_adj_shade[0], 128, 0, st>>>(W, L.S, L.P, cur, phase, L.err, nullptr, L.adj);
    if (events & 2)
        k_wave_shade<false, GENERAL, EV_MISS, ADJ>
            <<<L.grid_adj_shade[1], 128, 0, st>>>(W, L.S, L.P, cur, phase, L.err, nullptr, L.adj);
    if (phase == 1 && (events & 4))
        k_wave_shade<false, GENERAL, EV_SURF, ADJ>
            <<<L.grid_adj_shade[2], 128, 0, st>>>(W, L.S, L.P, cur, phase, L.err, nullptr, L.adj);
}

void wave_adj_shade(const WaveLaunch& L, const WaveState& W, int cur, int phase, cudaStream_t st, int events) {
    if (L.general)
        L.adj_mode == kAdjReplay ? adj_shade<true, kAdjReplay>(L, W, cur, phase, st, events)
                                 : adj_shade<true, kAdjRecord>(L, W, cur, phase, st, events);
    else
        L.adj_mode == kAdjReplay ? adj_shade<false, kAdjReplay>(L, W, cur, phase, st, events)
                                 : adj_shade<false, kAdjRecord>(L, W, cur, phase, st, events);
}

cudaError_t wave_adj_tail(const WaveLaunch& L, int cur, cudaStream_t st) {
    WaveGroups G;
    for (int g = 0; g < kWaveGroups; ++g) G.W[g] = L.W[g];
    G.groups = L.groups;
    const int grid = (int)((L.tail_paths + 127) / 128);
    if (grid == 0) return cudaSuccess;
#define SR_ADJ_TAIL(GEN, MODE) \
    k_wave_tail<false, GEN, MODE><<<grid, 128, 0, st>>>(G, L.S, L.V, L.P, L.out, cur, L.err, nullptr, L.adj)
    if (L.general) {
        if (L.adj_mode == kAdjReplay)
            SR_ADJ_TAIL(true, kAdjReplay);
        else
            SR_ADJ_TAIL(true, kAdjRecord);
    } else {
        if (L.adj_mode == kAdjReplay)
            SR_ADJ_TAIL(false, kAdjReplay);
        else
            SR_ADJ_TAIL(false, kAdjRecord);
    }
#undef SR_ADJ_TAIL
    return cudaGetLastError();
}

template <bool GENERAL, int ADJ>
static void adj_occupancy(int* shade, int* finalize) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shade[0], k_wave_shade<false, GENERAL, EV_FOG, ADJ>, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shade[1], k_wave_shade<false, GENERAL, EV_MISS, ADJ>, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shade[2], k_wave_shade<false, GENERAL, EV_SURF, ADJ>, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(finalize, k_wave_finalize<false, GENERAL, false, ADJ>, 128, 0);
}

void wave_adj_grid_sizes(WaveLaunch& L, int sms) {
    int sh[3] = {0, 0, 0}, fin = 0;
    if (L.general)
        L.adj_mode == kAdjReplay ? adj_occupancy<true, kAdjReplay>(sh, &fin) : adj_occupancy<true, kAdjRecord>(sh, &fin);
    else
        L.adj_mode == kAdjReplay ? adj_occupancy<false, kAdjReplay>(sh, &fin)
                                 : adj_occupancy<false, kAdjRecord>(sh, &fin);
    for (int e = 0; e < 3; ++e) L.grid_adj_shade[e] = sms * (sh[e] > 0 ? sh[e] : 1);
    L.grid_adj_finalize = sms * (fin > 0 ? fin : 1);
}

// Record mode's sweep: one thread per (slot, kept sample) -- every slot of every group, its pixel
// from the 8x4 tile layout -- over the samples the pixel took, with G = dL/dI / its sample count.
__global__ void __launch_bounds__(128) k_adjoint_checkpoint(WaveState W, DevScene S, DevParams P, const AdjPass* A,
                                                            const float* d_image, const uint32_t* samples) {
    const AdjTargets T{A->tex_a, A->grad_a, A->tex_r, A->grad_r, A->grad_f};
    const size_t total = (size_t)W.rec_stride * A->samples_kept;
    float g_density = 0.0f;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t s = (uint32_t)(t / A->samples_kept), sample = (uint32_t)(t % A->samples_kept);
        uint32_t x, y;
        slot_pixel(W, s, x, y);
        if (x >= P.width || y >= P.height) continue;
        const size_t i = (size_t)y * P.width + x;
        const uint32_t count = samples[i];
        const uint32_t taken = count < P.max_samples ? count : P.max_samples;
        if (sample >= taken) continue;
        const float inv = 1.0f / (float)count;
        const Col G{d_image[3 * i] * inv, d_image[3 * i + 1] * inv, d_image[3 * i + 2] * inv};
        const float4* vb = adj_vertex(A, s, sample, 0);
        adjoint_sweep<ADJ_ALL>(
            S, [&](int k) { return adj_decode(vb + (size_t)k * kAdjVertexF4, S, P.indirect_clamp); },
            (int)A->vcount[t], G, T, g_density);
    }
    for (int d = 16; d > 0; d >>= 1) g_density += __shfl_xor_sync(0xffffffffu, g_density, d);
    if ((threadIdx.x & 31) == 0 && A->grad_f && g_density != 0.0f) atomicAdd(A->grad_f, g_density);
}

cudaError_t launch_adjoint_checkpoint(const WaveLaunch& L, const float* d_image, const uint32_t* samples,
                                      cudaStream_t st) {
    int per_sm = 0, sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint_checkpoint, 128, 0);
    k_adjoint_checkpoint<<<sms * (per_sm > 0 ? per_sm : 1), 128, 0, st>>>(L.W[0], L.S, L.P, L.adj, d_image, samples);
    return cudaGetLastError();
}

}  // namespace sr

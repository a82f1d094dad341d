// sr_wavefront.h — path state of the wavefront renderer (sr_wavefront.cu) and its launchers.
#pragma once

#include <cuda_runtime.h>

#include "sr_kernels.h"
#include "sr_layout.h"

namespace sr {

// Structure-of-arrays path state, one slot per pixel (slots in 8x4 pixel tiles).
struct WaveState {
    uint32_t slots;    // tiles_x * tiles_y * 32
    uint32_t tiles_x;  // ceil(width / 8)
    uint4* rng;        // RNG words s0..s3
    uint32_t* rng_c;   // RNG Weyl counter s4
    float4* ray_o;     // ray origin, w = bounce index (int bits)
    float4* ray_d;     // ray direction, w = path flags (int bits)
    float4* rad;       // path radiance, w = pdf of the last scatter
    float4* fog;       // path fog radiance (primary-segment fog scatter)
    float4* energy;    // path throughput
    float4* medium;    // albedo of the medium the path is inside
    float4* prim;      // primary-hit normal, depth
    float2* prim_uv;   // primary-hit uv
    float4* acc0;      // pixel: radiance sum, luminance sum
    float4* acc1;      // pixel: fog radiance sum, luminance^2 sum
    float4* acc2;      // pixel: normal sum, surface luminance sum
    float4* acc3;      // pixel: last normal, surface luminance^2 sum
    float4* acc4;      // pixel: depth sum, normal count, depth count, sample index (int bits)
    float4* acc5;      // pixel: first uv, has-uv flag
    float4* hit;       // closest hit: object, triangle (int bits), world distance, local distance
    float2* hit_uv;    // closest hit barycentrics
    float4* sh0;       // deferred work: shadow origin (then its transmittance), request flags (int bits)
    float4* sh1;       // shadow direction, light pdf
    float4* sh2;       // reflectance (or phase pdf) rgb, MIS weight
    float4* sh3;       // throughput at the light sample
    uint32_t* q_active[2];  // live-path queues (ping-pong)
    uint32_t* q_resolve;    // deferred-work queue (shadow requests and finished samples)
    uint32_t* q_shadow;     // shadow-ray queue
    uint32_t* counts;       // [0],[1] live counts, [2] deferred count, [3] bounce counter,
                            // [4] extend fetch, [5] shadow fetch, [6] shadow count
};

struct WaveLaunch {
    WaveState W;
    DevScene S;
    DevView V;
    DevParams P;
    DevAovs out;
    uint32_t* err;
    unsigned long long* counters;
    int grid_extend, grid_shade, grid_resolve, grid_shadow;
    int general;  // 1: kernels with analytic shapes, transparency/media, normal maps, procedural sky
    uint32_t max_iters;
};

void wave_grid_sizes(WaveLaunch& L, int sms);
cudaError_t wave_init(const WaveLaunch& L, cudaStream_t st);
cudaError_t wave_bounce(const WaveLaunch& L, int cur, cudaStream_t st);
cudaError_t wave_build_graph(const WaveLaunch& L, cudaStream_t capture_stream, cudaGraphExec_t* exec_out);

}  // namespace sr

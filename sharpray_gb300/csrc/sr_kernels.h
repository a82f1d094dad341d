// sr_kernels.h — host-callable launchers of the CUDA kernels (implemented in the .cu files).
#pragma once

#include <cuda_runtime.h>

#include "sr_layout.h"

namespace sr {

struct DevAovs {
    float* radiance;
    float* radiance_fog;
    float* normals;
    float* uv;
    float* depth;
    uint32_t* samples;
    float* variance;
};

// Path loop over every pixel (sr_render.cu).
cudaError_t launch_render(const DevScene& S, const DevView& V, const DevParams& P, const DevAovs& out,
                          unsigned long long* counters, uint32_t* err, cudaStream_t stream);

// Sky table of a texture sky (DevSky::center), `texels` = width x height (sr_render.cu).
cudaError_t launch_sky_table(const DevScene& S, float4* out, uint32_t texels, cudaStream_t stream);

// Path-replay adjoint (sr_adjoint.cu) for dL/dI = d_image (width x height x 3, I = radiance +
// radiance_fog): parameter 0 adds dL/d(texels of albedo texture tex_a) into grad_a, 1 dL/d(texels
// of roughness texture tex_r) into grad_r (channel 0), 2 dL/d(fog density) into grad_f[0], 3 all
// three from one replay (a -1 texture or null gradient skips a part); replay (optional) gets the
// re-rendered image.
cudaError_t launch_adjoint(const DevScene& S, const DevView& V, const DevParams& P, const DevAovs& fwd,
                           const float* d_image, int parameter, int tex_a, float* grad_a, int tex_r, float* grad_r,
                           float* grad_f, float* replay, uint32_t* err, cudaStream_t stream);
// rgb float triples -> texel records (sr_adjoint.cu).
cudaError_t launch_texels_from_rgb(const float* rgb, float4* out, size_t n, cudaStream_t stream);

// Closest hit per world ray (sr_render.cu).
cudaError_t launch_trace(const DevScene& S, const float* rays, uint32_t n, int32_t* obj, int32_t* tri, float* dist,
                         float* uv, uint32_t* err, cudaStream_t stream);

// Denoise + fog blur + tonemap (sr_compose.cu).  `spatial` holds the (2r+1)^2 surface weights
// dw-independent exp(-d^2/(2 r^2)) and `fog_spatial` the fog weights strength*exp(...), both
// evaluated on the host.  `denoise` = false gives Compositor.Preview.
struct ComposeConsts {
    int32_t tonemapper;
    float exposure;
    float strength, strength_max, lum_boost;
    float lum_limit_inv, normal_limit_inv, depth_limit_inv;
    int32_t radius, fog_radius;
};
// `linear` (optional, width x height x 3): the filtered radiance + fog before exposure and tonemap;
// rgb8 may be null when only that is wanted.
cudaError_t launch_compose(const DevAovs& in, uint32_t width, uint32_t height, const ComposeConsts& k,
                           const float* spatial, const float* fog_spatial, bool denoise, uint8_t* rgb8,
                           float4* scratch, cudaStream_t stream, float* linear = nullptr);

// Compositing that allocates nothing: packed planes live in a fixed device array of sr_compose.cu
// (bands of rows); spatial weights are evaluated per tap.  When the image is too wide for the array
// it launches nothing, sets *too_large and returns cudaErrorInvalidValue (needed_bytes then holds
// the size one band would need); any other error is a CUDA failure of the lookup or a launch.
cudaError_t launch_compose_static(int device, const DevAovs& in, uint32_t width, uint32_t height,
                                  const ComposeConsts& k, float rp_inv, float rpf_inv, float fog_strength,
                                  uint8_t* rgb8, cudaStream_t stream, size_t* needed_bytes, bool* too_large);
// Bytes of the fixed array launch_compose_static works in.
size_t compose_static_capacity();

// AOV visualisation to RGB8 (sr_overlay.cu).  `lut` maps sample counts below lut_n to bytes.
cudaError_t launch_aov_image(const DevAovs& in, uint32_t n, int32_t kind, float variance_div, const uint8_t* lut,
                             uint32_t lut_n, float min_samples, float log_range, uint8_t* rgb8, cudaStream_t stream);

// Overlay draw (sr_overlay.cu): lines and glyphs prepared on the host; `entry` is the draw-order
// index, `colors[entry]` the packed RGB8 (r | g << 8 | b << 16); `owner` is a w*h int32 scratch.
struct OverlayLineOp {
    int32_t ax, ay, bx, by;
    float inv_a, inv_b;  // 1 / biased depth at a and b
    int32_t depth_test, entry;
};
struct OverlayGlyphOp {
    int32_t x, y;   // top-left pixel of the 8x8 cell
    int32_t glyph;  // row index into the font table
    int32_t entry;
};
cudaError_t launch_overlay(const OverlayLineOp* lines, uint32_t line_count, const OverlayGlyphOp* glyph_ops,
                           uint32_t glyph_count, const uint8_t* glyphs, const uint32_t* colors, const float* depth,
                           uint32_t width, uint32_t height, int32_t* owner, uint8_t* rgb8, cudaStream_t stream);

}  // namespace sr

// sr_overlay.cu — the image-side conveniences around a render: AOV visualisations (the normal /
// depth / variance / samples / uv dumps of program.cs:211-263) and the debug overlay
// (Overlay.Draw overlay.cs:54-196) drawn into an RGB8 image on the device.
//
// The overlay keeps the reference's sequential draw order without serialising the draw: every
// line (one thread walks its Bresenham steps) and every glyph row (one thread per row) records the
// index of the entry that covers a pixel with atomicMax into an owner plane, and a final pass
// paints each owned pixel with the colour of its highest entry, which is the entry the reference
// draws last there.  The depth plane is read-only during the draw, so the depth test of each step
// does not depend on the order.  End points, depths and colours are prepared on the host.
#include <cuda_runtime.h>

#include "../../include/sharpray.h"
#include "sr_kernels.h"

namespace sr {

// (byte)f in .NET 8: truncation to int (0 for NaN and outside the int range), low 8 bits.
__device__ __forceinline__ uint8_t net_byte(float f) {
    if (!(fabsf(f) < 2147483648.0f)) return 0;
    return (uint8_t)(uint32_t)(int32_t)f;
}

// Math.Clamp(x, 0, 1): NaN passes through.
__device__ __forceinline__ float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

__global__ void k_aov_image(DevAovs in, uint32_t n, int32_t kind, float variance_div, const uint8_t* lut,
                            uint32_t lut_n, float min_samples, float log_range, uint8_t* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint8_t r = 0, g = 0, b = 0;
    if (kind == SR_AOV_NORMAL) {
        r = net_byte((in.normals[3 * i] * 0.5f + 0.5f) * 255.0f);
        g = net_byte((in.normals[3 * i + 1] * 0.5f + 0.5f) * 255.0f);
        b = net_byte((in.normals[3 * i + 2] * 0.5f + 0.5f) * 255.0f);
    } else if (kind == SR_AOV_DEPTH) {
        const float depth_max_inv = 1.0f / 25.0f;
        float d = in.depth[i];
        if (isinf(d)) {
            r = 255;
        } else {
            r = g = b = net_byte(clamp01(d * depth_max_inv) * 255.0f);
        }
    } else if (kind == SR_AOV_VARIANCE) {
        r = g = b = net_byte(clamp01(in.variance[i] / variance_div) * 255.0f);
    } else if (kind == SR_AOV_SAMPLES) {
        uint32_t s = in.samples[i];
        // counts up to max_samples + 1 come from a host table of the C runtime's log2f
        r = g = b = s < lut_n ? lut[s] : net_byte(log2f((float)s / min_samples) / log_range * 255.0f);
    } else {
        r = net_byte(fabsf(fmodf(in.uv[2 * i], 1.0f)) * 255.0f);
        g = net_byte(fabsf(fmodf(in.uv[2 * i + 1], 1.0f)) * 255.0f);
    }
    out[3 * i] = r, out[3 * i + 1] = g, out[3 * i + 2] = b;
}

cudaError_t launch_aov_image(const DevAovs& in, uint32_t n, int32_t kind, float variance_div, const uint8_t* lut,
                             uint32_t lut_n, float min_samples, float log_range, uint8_t* rgb8, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    k_aov_image<<<(n + 255) / 256, 256, 0, stream>>>(in, n, kind, variance_div, lut, lut_n, min_samples, log_range,
                                                      rgb8);
    return cudaGetLastError();
}

// RasterizeLine overlay.cs:102-149: all-octant Bresenham from a to b; step k of `total` has depth
// 1 / lerp(1/depth_a, 1/depth_b, k / total) (float.Lerp: a * (1 - t) + b * t).
__global__ void k_overlay_lines(const OverlayLineOp* ops, uint32_t count, uint32_t width, uint32_t height,
                                const float* depth, int32_t* owner) {
    uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= count) return;
    const OverlayLineOp L = ops[li];
    const int span_x = abs(L.bx - L.ax), span_y = -abs(L.by - L.ay);
    const int step_x = L.ax < L.bx ? 1 : -1, step_y = L.ay < L.by ? 1 : -1;
    const int total = max(span_x, -span_y);
    int err = span_x + span_y;
    int x = L.ax, y = L.ay;
    // the walk reaches b after `total` moves; the bound only caps the loop
    for (int step = 0; step <= total; ++step) {
        if ((uint32_t)x < width && (uint32_t)y < height) {
            const uint32_t idx = (uint32_t)y * width + (uint32_t)x;
            const float frac = total > 0 ? (float)step / (float)total : 0.0f;
            const float line_depth = 1.0f / (L.inv_a * (1.0f - frac) + L.inv_b * frac);
            if (!L.depth_test || depth == nullptr || line_depth <= depth[idx]) atomicMax(owner + idx, L.entry);
        }
        if (x == L.bx && y == L.by) break;
        const int e2 = 2 * err;
        if (e2 >= span_y) err += span_y, x += step_x;
        if (e2 <= span_x) err += span_x, y += step_y;
    }
}

// RasterizeTextLine overlay.cs:151-170: one thread per glyph row.
__global__ void k_overlay_glyphs(const OverlayGlyphOp* ops, uint32_t count, const uint8_t* glyphs, uint32_t width,
                                 uint32_t height, int32_t* owner) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * 8u) return;
    const OverlayGlyphOp G = ops[t >> 3];
    const int row = (int)(t & 7u);
    const uint32_t bits = glyphs[(size_t)G.glyph * 8 + row];
    for (int col = 0; col < 8; ++col) {
        if (!(bits & (0x80u >> col))) continue;
        const int x = G.x + col, y = G.y + row;
        if ((uint32_t)x < width && (uint32_t)y < height) atomicMax(owner + (size_t)y * width + x, G.entry);
    }
}

__global__ void k_overlay_paint(const int32_t* owner, uint32_t n, const uint32_t* colors, uint8_t* rgb8) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t e = owner[i];
    if (e < 0) return;
    const uint32_t c = colors[e];
    rgb8[3 * i] = (uint8_t)(c & 255u), rgb8[3 * i + 1] = (uint8_t)((c >> 8) & 255u);
    rgb8[3 * i + 2] = (uint8_t)((c >> 16) & 255u);
}

cudaError_t launch_overlay(const OverlayLineOp* lines, uint32_t line_count, const OverlayGlyphOp* glyph_ops,
                           uint32_t glyph_count, const uint8_t* glyphs, const uint32_t* colors, const float* depth,
                           uint32_t width, uint32_t height, int32_t* owner, uint8_t* rgb8, cudaStream_t stream) {
    const uint32_t n = width * height;
    if (n == 0 || (line_count == 0 && glyph_count == 0)) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(owner, 0xff, (size_t)n * sizeof(int32_t), stream);
    if (e != cudaSuccess) return e;
    if (line_count) k_overlay_lines<<<(line_count + 63) / 64, 64, 0, stream>>>(lines, line_count, width, height, depth,
                                                                                 owner);
    if (glyph_count)
        k_overlay_glyphs<<<(glyph_count * 8 + 255) / 256, 256, 0, stream>>>(glyph_ops, glyph_count, glyphs, width,
                                                                           height, owner);
    k_overlay_paint<<<(n + 255) / 256, 256, 0, stream>>>(owner, n, colors, rgb8);
    return cudaGetLastError();
}

}  // namespace sr

// sr_compose.cu — Compositor.Compose (compose.cs:74-99) on the GPU: joint bilateral denoise of
// the surface radiance (Filter compose.cs:101-204), Gaussian blur of the fog radiance
// (FilterFog compose.cs:206-245) and tonemapping to RGB8 (Tonemap compose.cs:247-266,
// Color.ToPixel math.cs:127-136), fused into one pass per pixel.
//
// A packing pass first turns the AOV planes into two float4 planes, {radiance.rgb, luminance}
// and {normal.xyz, depth}, plus {fog.rgb, 0}, so that every filter tap is two 128-bit loads and
// the neighbour luminance is not recomputed per tap.  The taps of a pixel are visited in the
// reference order (rows top to bottom, columns left to right) so the weighted sums accumulate
// in the same order; the spatial weights exp(-d^2 / 2r^2) come from a host-evaluated table.
#include <cuda_runtime.h>

#include "sr_device.cuh"
#include "sr_kernels.h"

namespace sr {

__global__ void k_pack(DevAovs in, uint32_t n, float4* p_rad, float4* p_geo, float4* p_fog) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Col r{in.radiance[3 * i], in.radiance[3 * i + 1], in.radiance[3 * i + 2]};
    p_rad[i] = make_float4(r.r, r.g, r.b, luminance(r));
    p_geo[i] = make_float4(in.normals[3 * i], in.normals[3 * i + 1], in.normals[3 * i + 2], in.depth[i]);
    p_fog[i] = make_float4(in.radiance_fog[3 * i], in.radiance_fog[3 * i + 1], in.radiance_fog[3 * i + 2], 0.0f);
}

// Color.ToPixel math.cs:127-136.
__device__ __forceinline__ void to_pixel(Col c, uint8_t* out) {
    Col cc{clampf(c.r, 0.0f, 1.0f), clampf(c.g, 0.0f, 1.0f), clampf(c.b, 0.0f, 1.0f)};
    float r = fmaxf(1.055f * powf(cc.r, 0.416666667f) - 0.055f, 0.0f);
    float g = fmaxf(1.055f * powf(cc.g, 0.416666667f) - 0.055f, 0.0f);
    float b = fmaxf(1.055f * powf(cc.b, 0.416666667f) - 0.055f, 0.0f);
    out[0] = (uint8_t)(int)(r * 255.0f + 0.5f);
    out[1] = (uint8_t)(int)(g * 255.0f + 0.5f);
    out[2] = (uint8_t)(int)(b * 255.0f + 0.5f);
}

// Compositor.Tonemap compose.cs:247-266.
__device__ __forceinline__ void tonemap(const ComposeConsts& k, Col radiance, uint8_t* out) {
    Col x = radiance * k.exposure;
    if (k.tonemapper == SR_TONEMAP_REINHARD) {
        to_pixel(x / (x + gray(1.0f)), out);
    } else {
        const float a = 1.8f, b = 1.4f, c = 0.5f, d = 1.5f;
        to_pixel((x * (a * x + gray(b))) / (x * (a * x + gray(c)) + gray(d)), out);
    }
}

// Table layout (host-built): for radius R, (2R+1)^2 spatial weights followed by 2R+1 row half-widths
// (as floats) = the largest |kx| with kx^2 + ky^2 <= R^2.
__global__ void __launch_bounds__(128) k_compose(const float4* __restrict__ p_rad, const float4* __restrict__ p_geo,
                                                 const float4* __restrict__ p_fog, const float* __restrict__ variance,
                                                 uint32_t width, uint32_t height, ComposeConsts k,
                                                 const float* __restrict__ spatial, const float* __restrict__ fog_spatial,
                                                 int denoise, uint8_t* rgb8) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= (int)width || y >= (int)height) return;
    size_t ci = (size_t)y * width + x;
    float4 c0 = __ldg(p_rad + ci);
    Col main = col3(c0);
    Col fog = col3(__ldg(p_fog + ci));
    if (denoise) {
        // ---- Filter compose.cs:101-204 ----
        float4 c1 = __ldg(p_geo + ci);
        V3 cn = v3(c1);
        float cd = c1.w;
        bool has_n = mag_sqr(cn) > 0.0f;
        bool has_d = !isinf(cd);
        float lum = c0.w;
        float boost = 1.0f + lum * k.lum_boost;
        float dw = fminf(__ldg(variance + ci) * boost * k.strength, k.strength_max);
        if (!(dw < 1e-4f)) {
            int R = k.radius;
            int side = 2 * R + 1;
            const float* row_half = spatial + side * side;
            float wsum = 1.0f;
            Col rsum = main;
            int ky0 = max(-R, -y), ky1 = min(R, (int)height - 1 - y);
            for (int ky = ky0; ky <= ky1; ++ky) {
                int hw = (int)__ldg(row_half + ky + R);
                int kx0 = max(-hw, -x), kx1 = min(hw, (int)width - 1 - x);
                const float* wrow = spatial + (ky + R) * side + R;
                const float4* prow = p_rad + (size_t)(y + ky) * width + x;
                const float4* grow = p_geo + (size_t)(y + ky) * width + x;
                for (int kx = kx0; kx <= kx1; ++kx) {
                    if (kx == 0 && ky == 0) continue;
                    float4 q1 = __ldg(grow + kx);
                    V3 nn = v3(q1);
                    bool nh_n = mag_sqr(nn) > 0.0f;
                    bool nh_d = !isinf(q1.w);
                    if (has_n != nh_n || has_d != nh_d) continue;
                    float4 q0 = __ldg(prow + kx);
                    float w = dw * __ldg(wrow + kx);
                    if (has_n && w > 0.0f) {
                        V3 nd = cn - nn;
                        w *= expf(-mag_sqr(nd) * k.normal_limit_inv);
                    }
                    if (has_d && w > 0.0f) {
                        float dd = cd - q1.w;
                        w *= expf(-(dd * dd) * k.depth_limit_inv);
                    }
                    if (w > 0.0f) {
                        float ld = fmaxf(0.0f, q0.w - lum);
                        w *= expf(-(ld * ld) * k.lum_limit_inv);
                    }
                    wsum += w;
                    rsum = rsum + col3(q0) * w;
                }
            }
            main = rsum / wsum;
        }
        // ---- FilterFog compose.cs:206-245 ----
        {
            int R = k.fog_radius;
            int side = 2 * R + 1;
            const float* row_half = fog_spatial + side * side;
            float wsum = 1.0f;
            Col rsum = fog;
            int ky0 = max(-R, -y), ky1 = min(R, (int)height - 1 - y);
            for (int ky = ky0; ky <= ky1; ++ky) {
                int hw = (int)__ldg(row_half + ky + R);
                int kx0 = max(-hw, -x), kx1 = min(hw, (int)width - 1 - x);
                const float* wrow = fog_spatial + (ky + R) * side + R;
                const float4* frow = p_fog + (size_t)(y + ky) * width + x;
                for (int kx = kx0; kx <= kx1; ++kx) {
                    if (kx == 0 && ky == 0) continue;
                    float w = __ldg(wrow + kx);
                    wsum += w;
                    rsum = rsum + col3(__ldg(frow + kx)) * w;
                }
            }
            fog = rsum / wsum;
        }
    }
    tonemap(k, main + fog, rgb8 + ci * 3);
}

cudaError_t launch_compose(const DevAovs& in, uint32_t width, uint32_t height, const ComposeConsts& k,
                           const float* spatial, const float* fog_spatial, bool denoise, uint8_t* rgb8,
                           float4* scratch, cudaStream_t stream) {
    uint32_t n = width * height;
    if (n == 0) return cudaSuccess;
    float4* p_rad = scratch;
    float4* p_geo = scratch + n;
    float4* p_fog = scratch + 2 * (size_t)n;
    k_pack<<<(n + 255) / 256, 256, 0, stream>>>(in, n, p_rad, p_geo, p_fog);
    dim3 grid((width + 31) / 32, (height + 3) / 4);
    k_compose<<<grid, 128, 0, stream>>>(p_rad, p_geo, p_fog, in.variance, width, height, k, spatial, fog_spatial,
                                        denoise ? 1 : 0, rgb8);
    return cudaGetLastError();
}

}  // namespace sr

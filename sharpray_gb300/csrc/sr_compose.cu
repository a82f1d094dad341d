// sr_compose.cu — Compositor.Compose (compose.cs:74-99) on the GPU: joint bilateral denoise of
// the surface radiance (Filter compose.cs:101-204), Gaussian blur of the fog radiance
// (FilterFog compose.cs:206-245) and tonemapping to RGB8 (Tonemap compose.cs:247-266,
// Color.ToPixel math.cs:127-136), fused into one pass per pixel.
//
// A packing pass first turns the AOV planes into two float4 planes, {radiance.rgb, luminance}
// and {normal.xyz, depth}, plus {fog.rgb, 0}, so that every filter tap is two 128-bit loads and
// the neighbour luminance is not recomputed per tap.  The taps of a pixel are visited in the
// reference order (rows top to bottom, columns left to right) so the weighted sums accumulate
// in the same order; the spatial weights exp(-d^2 / 2r^2) come from a host-evaluated table.  Per
// tap the normal, depth and luminance Gaussians are one fast exponential of their summed
// exponents and the sums accumulate with fused multiply-adds: the filter is the reference's up to
// float rounding (images agree within one code value).
#include <atomic>
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
                                                 int denoise, uint8_t* rgb8, float* linear) {
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
                    // the normal, depth and luminance Gaussians of compose.cs:165-190 as one
                    // exponential of the summed exponents (equal up to rounding; a weight the
                    // reference zeroes by underflow stays zero)
                    if (w > 0.0f) {
                        float e = 0.0f;
                        if (has_n) {
                            V3 nd = cn - nn;
                            e = mag_sqr(nd) * k.normal_limit_inv;
                        }
                        if (has_d) {
                            float dd = cd - q1.w;
                            e = __fmaf_rn(dd * dd, k.depth_limit_inv, e);
                        }
                        float ld = fmaxf(0.0f, q0.w - lum);
                        e = __fmaf_rn(ld * ld, k.lum_limit_inv, e);
                        w *= __expf(-e);
                    }
                    wsum += w;
                    rsum = Col{__fmaf_rn(q0.x, w, rsum.r), __fmaf_rn(q0.y, w, rsum.g), __fmaf_rn(q0.z, w, rsum.b)};
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
                    float4 f = __ldg(frow + kx);
                    wsum += w;
                    rsum = Col{__fmaf_rn(f.x, w, rsum.r), __fmaf_rn(f.y, w, rsum.g), __fmaf_rn(f.z, w, rsum.b)};
                }
            }
            fog = rsum / wsum;
        }
    }
    const Col total = main + fog;
    if (linear) linear[3 * ci] = total.r, linear[3 * ci + 1] = total.g, linear[3 * ci + 2] = total.b;
    if (rgb8) tonemap(k, total, rgb8 + ci * 3);
}

// Two horizontally adjacent pixels per thread (SR_COMPOSE_PAIR = 1): the main filter walks the
// union of both pixels' tap columns row by row, so every tap column's two float4 loads serve both
// pixels; each pixel still takes exactly its own taps in the reference order, so the sums (and the
// image) are those of k_compose.  Measured 0.6 % slower at 1920x1080 (the filter is bound by the
// per-tap arithmetic, not by its loads), so it stays off.
#ifndef SR_COMPOSE_PAIR
#define SR_COMPOSE_PAIR 0
#endif

struct FilterPx {
    bool filter;  // the pixel's joint bilateral filter runs (weight above the early-out)
    bool has_n, has_d;
    V3 cn;
    float cd, lum, dw, wsum;
    Col rsum;
};

// One tap of Filter (compose.cs:150-198) for pixel p: neighbour q0 = {rgb, luminance},
// q1 = {normal, depth}, spatial weight ws.
__device__ __forceinline__ void filter_tap(FilterPx& p, const ComposeConsts& k, float4 q0, float4 q1, float ws) {
    V3 nn = v3(q1);
    bool nh_n = mag_sqr(nn) > 0.0f;
    bool nh_d = !isinf(q1.w);
    if (p.has_n != nh_n || p.has_d != nh_d) return;
    float w = p.dw * ws;
    if (w > 0.0f) {
        float e = 0.0f;
        if (p.has_n) {
            V3 nd = p.cn - nn;
            e = mag_sqr(nd) * k.normal_limit_inv;
        }
        if (p.has_d) {
            float dd = p.cd - q1.w;
            e = __fmaf_rn(dd * dd, k.depth_limit_inv, e);
        }
        float ld = fmaxf(0.0f, q0.w - p.lum);
        e = __fmaf_rn(ld * ld, k.lum_limit_inv, e);
        w *= __expf(-e);
    }
    p.wsum += w;
    p.rsum = Col{__fmaf_rn(q0.x, w, p.rsum.r), __fmaf_rn(q0.y, w, p.rsum.g), __fmaf_rn(q0.z, w, p.rsum.b)};
}

// FilterFog compose.cs:206-245 for pixel (x, y).
__device__ __forceinline__ Col filter_fog(const float4* __restrict__ p_fog, uint32_t width, uint32_t height,
                                          const ComposeConsts& k, const float* __restrict__ fog_spatial, int x, int y,
                                          Col fog) {
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
            float4 f = __ldg(frow + kx);
            wsum += w;
            rsum = Col{__fmaf_rn(f.x, w, rsum.r), __fmaf_rn(f.y, w, rsum.g), __fmaf_rn(f.z, w, rsum.b)};
        }
    }
    return rsum / wsum;
}

__global__ void __launch_bounds__(128) k_compose_pair(const float4* __restrict__ p_rad,
                                                      const float4* __restrict__ p_geo,
                                                      const float4* __restrict__ p_fog,
                                                      const float* __restrict__ variance, uint32_t width,
                                                      uint32_t height, ComposeConsts k,
                                                      const float* __restrict__ spatial,
                                                      const float* __restrict__ fog_spatial, int denoise,
                                                      uint8_t* rgb8, float* linear) {
    const int xa = 2 * (int)(blockIdx.x * 32 + (threadIdx.x & 31));
    const int y = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (xa >= (int)width || y >= (int)height) return;
    const bool b_live = xa + 1 < (int)width;
    FilterPx px[2];
    Col main[2], fog[2];
    for (int j = 0; j < 2; ++j) {
        px[j].filter = false;
        if (j == 1 && !b_live) continue;
        const size_t ci = (size_t)y * width + xa + j;
        const float4 c0 = __ldg(p_rad + ci);
        main[j] = col3(c0);
        fog[j] = col3(__ldg(p_fog + ci));
        if (!denoise) continue;
        const float4 c1 = __ldg(p_geo + ci);
        FilterPx& p = px[j];
        p.cn = v3(c1);
        p.cd = c1.w;
        p.has_n = mag_sqr(p.cn) > 0.0f;
        p.has_d = !isinf(p.cd);
        p.lum = c0.w;
        const float boost = 1.0f + p.lum * k.lum_boost;
        p.dw = fminf(__ldg(variance + ci) * boost * k.strength, k.strength_max);
        p.filter = !(p.dw < 1e-4f);
        p.wsum = 1.0f;
        p.rsum = main[j];
    }
    if (px[0].filter || px[1].filter) {
        // ---- Filter compose.cs:101-204, both pixels over the union of their tap columns ----
        const int R = k.radius;
        const int side = 2 * R + 1;
        const float* row_half = spatial + side * side;
        const int xb = xa + 1;
        const int ky0 = max(-R, -y), ky1 = min(R, (int)height - 1 - y);
        for (int ky = ky0; ky <= ky1; ++ky) {
            const int hw = (int)__ldg(row_half + ky + R);
            const int c_lo = max(0, (px[0].filter ? xa : xb) - hw);
            const int c_hi = min((int)width - 1, (px[1].filter ? xb : xa) + hw);
            const float* wrow = spatial + (ky + R) * side + R;
            const float4* prow = p_rad + (size_t)(y + ky) * width;
            const float4* grow = p_geo + (size_t)(y + ky) * width;
            for (int c = c_lo; c <= c_hi; ++c) {
                const float4 q1 = __ldg(grow + c);
                const float4 q0 = __ldg(prow + c);
                const int ka = c - xa, kb = c - xb;
                if (px[0].filter && ka <= hw && (ka != 0 || ky != 0)) filter_tap(px[0], k, q0, q1, __ldg(wrow + ka));
                if (px[1].filter && kb >= -hw && (kb != 0 || ky != 0))
                    filter_tap(px[1], k, q0, q1, __ldg(wrow + kb));
            }
        }
        for (int j = 0; j < 2; ++j)
            if (px[j].filter) main[j] = px[j].rsum / px[j].wsum;
    }
    for (int j = 0; j < 2; ++j) {
        if (j == 1 && !b_live) break;
        if (denoise) fog[j] = filter_fog(p_fog, width, height, k, fog_spatial, xa + j, y, fog[j]);
        const size_t ci = (size_t)y * width + xa + j;
        const Col total = main[j] + fog[j];
        if (linear) linear[3 * ci] = total.r, linear[3 * ci + 1] = total.g, linear[3 * ci + 2] = total.b;
        if (rgb8) tonemap(k, total, rgb8 + ci * 3);
    }
}

cudaError_t launch_compose(const DevAovs& in, uint32_t width, uint32_t height, const ComposeConsts& k,
                           const float* spatial, const float* fog_spatial, bool denoise, uint8_t* rgb8,
                           float4* scratch, cudaStream_t stream, float* linear) {
    uint32_t n = width * height;
    if (n == 0) return cudaSuccess;
    float4* p_rad = scratch;
    float4* p_geo = scratch + n;
    float4* p_fog = scratch + 2 * (size_t)n;
    k_pack<<<(n + 255) / 256, 256, 0, stream>>>(in, n, p_rad, p_geo, p_fog);
    if (SR_COMPOSE_PAIR) {
        dim3 grid((width + 63) / 64, (height + 3) / 4);
        k_compose_pair<<<grid, 128, 0, stream>>>(p_rad, p_geo, p_fog, in.variance, width, height, k, spatial,
                                                 fog_spatial, denoise ? 1 : 0, rgb8, linear);
    } else {
        dim3 grid((width + 31) / 32, (height + 3) / 4);
        k_compose<<<grid, 128, 0, stream>>>(p_rad, p_geo, p_fog, in.variance, width, height, k, spatial, fog_spatial,
                                            denoise ? 1 : 0, rgb8, linear);
    }
    return cudaGetLastError();
}

// ---- compositing without allocations ----------------------------------------------------------
//
// Some hosts cannot allocate device memory at the moment they want to composite: a render service
// whose device memory is already committed to its own frame pools under a hard quota, or a
// latency-critical loop that must not call cudaMalloc because an allocation can synchronise the
// whole device and stall its other streams.  For them sr_compose_device_static runs the same filter
// as sr_compose_device but keeps its packed planes in the fixed array below instead of a context
// buffer, and evaluates the spatial weights inline instead of uploading a weight table.
//
// Limits: the array is kStaticScratchBytes (32 MiB) on every GPU that loads the library, held until
// the process exits.  The image is filtered in bands of rows, each band packed together with its
// filter halo; a call fails when even a one-row band with its halo does not fit, i.e. when
// (2 * max(radius, fog radius) + 2) * width * 48 bytes exceeds 32 MiB.  All calls share the array:
// two calls that overlap on the GPU (e.g. on different streams) overwrite each other's bands and
// produce wrong images, so serialise them.  Every band is packed before it is read, so the array
// needs no clearing between calls.
static constexpr size_t kStaticScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch, resolved once per device with that device current.  Host
// threads making their first call on one device at the same time may both resolve it; they store
// the same value, and the atomic entries make that a benign race instead of a data race.
static constexpr int kMaxDevices = 64;
static std::atomic<float4*> g_static_scratch_addr[kMaxDevices];

static cudaError_t static_scratch(int device, float4** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    float4* addr = g_static_scratch_addr[device].load(std::memory_order_acquire);
    if (!addr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return e;
        addr = (float4*)p;
        g_static_scratch_addr[device].store(addr, std::memory_order_release);
    }
    *out = addr;
    return cudaSuccess;
}

size_t compose_static_capacity() { return kStaticScratchBytes; }

// Packs image rows [row0, row0 + rows) into band-local planes.
__global__ void k_pack_band(DevAovs in, uint32_t width, uint32_t row0, uint32_t rows, float4* p_rad, float4* p_geo,
                            float4* p_fog) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= width * rows) return;
    size_t g = (size_t)row0 * width + i;
    Col r{in.radiance[3 * g], in.radiance[3 * g + 1], in.radiance[3 * g + 2]};
    p_rad[i] = make_float4(r.r, r.g, r.b, luminance(r));
    p_geo[i] = make_float4(in.normals[3 * g], in.normals[3 * g + 1], in.normals[3 * g + 2], in.depth[g]);
    p_fog[i] = make_float4(in.radiance_fog[3 * g], in.radiance_fog[3 * g + 1], in.radiance_fog[3 * g + 2], 0.0f);
}

// Largest |kx| with kx^2 + ky^2 <= r^2 (the circular-kernel test of compose.cs:147-148).
__device__ __forceinline__ int half_width(int r, int ky) {
    int hw = (int)sqrtf((float)(r * r - ky * ky));
    while (hw > 0 && hw * hw + ky * ky > r * r) --hw;
    while ((hw + 1) * (hw + 1) + ky * ky <= r * r) ++hw;
    return hw;
}

// k_compose for output rows [y0, y1) reading band planes that start at image row `prow0`; spatial
// weights are evaluated per tap as the reference does (compose.cs:160, 236).
__global__ void __launch_bounds__(128) k_compose_band(const float4* __restrict__ p_rad, const float4* __restrict__ p_geo,
                                                      const float4* __restrict__ p_fog, const float* __restrict__ variance,
                                                      uint32_t width, uint32_t height, uint32_t y0, uint32_t y1,
                                                      uint32_t prow0, ComposeConsts k, float rp_inv, float rpf_inv,
                                                      float fog_strength, uint8_t* rgb8) {
    int x = blockIdx.x * 32 + (threadIdx.x & 31);
    int y = (int)y0 + blockIdx.y * 4 + (threadIdx.x >> 5);
    if (x >= (int)width || y >= (int)y1) return;
    size_t li = (size_t)(y - (int)prow0) * width + x;
    float4 c0 = __ldg(p_rad + li);
    Col main = col3(c0);
    Col fog = col3(__ldg(p_fog + li));
    float4 c1 = __ldg(p_geo + li);
    V3 cn = v3(c1);
    float cd = c1.w;
    bool has_n = mag_sqr(cn) > 0.0f;
    bool has_d = !isinf(cd);
    float lum = c0.w;
    float boost = 1.0f + lum * k.lum_boost;
    float dw = fminf(__ldg(variance + (size_t)y * width + x) * boost * k.strength, k.strength_max);
    if (!(dw < 1e-4f)) {
        int R = k.radius;
        float wsum = 1.0f;
        Col rsum = main;
        int ky0 = max(-R, -y), ky1 = min(R, (int)height - 1 - y);
        for (int ky = ky0; ky <= ky1; ++ky) {
            int hw = half_width(R, ky);
            int kx0 = max(-hw, -x), kx1 = min(hw, (int)width - 1 - x);
            const float4* prow = p_rad + (size_t)(y + ky - (int)prow0) * width + x;
            const float4* grow = p_geo + (size_t)(y + ky - (int)prow0) * width + x;
            for (int kx = kx0; kx <= kx1; ++kx) {
                if (kx == 0 && ky == 0) continue;
                float4 q1 = __ldg(grow + kx);
                V3 nn = v3(q1);
                bool nh_n = mag_sqr(nn) > 0.0f;
                bool nh_d = !isinf(q1.w);
                if (has_n != nh_n || has_d != nh_d) continue;
                float4 q0 = __ldg(prow + kx);
                float kd = (float)(kx * kx + ky * ky);
                float w = dw * sr_exp(-kd * rp_inv);
                if (has_n && w > 0.0f) {
                    V3 nd = cn - nn;
                    w *= sr_exp(-mag_sqr(nd) * k.normal_limit_inv);
                }
                if (has_d && w > 0.0f) {
                    float dd = cd - q1.w;
                    w *= sr_exp(-(dd * dd) * k.depth_limit_inv);
                }
                if (w > 0.0f) {
                    float ld = fmaxf(0.0f, q0.w - lum);
                    w *= sr_exp(-(ld * ld) * k.lum_limit_inv);
                }
                wsum += w;
                rsum = rsum + col3(q0) * w;
            }
        }
        main = rsum / wsum;
    }
    {
        int R = k.fog_radius;
        float wsum = 1.0f;
        Col rsum = fog;
        int ky0 = max(-R, -y), ky1 = min(R, (int)height - 1 - y);
        for (int ky = ky0; ky <= ky1; ++ky) {
            int hw = half_width(R, ky);
            int kx0 = max(-hw, -x), kx1 = min(hw, (int)width - 1 - x);
            const float4* frow = p_fog + (size_t)(y + ky - (int)prow0) * width + x;
            for (int kx = kx0; kx <= kx1; ++kx) {
                if (kx == 0 && ky == 0) continue;
                float kd = (float)(kx * kx + ky * ky);
                float w = fog_strength * sr_exp(-kd * rpf_inv);
                wsum += w;
                rsum = rsum + col3(__ldg(frow + kx)) * w;
            }
        }
        fog = rsum / wsum;
    }
    tonemap(k, main + fog, rgb8 + ((size_t)y * width + x) * 3);
}

cudaError_t launch_compose_static(int device, const DevAovs& in, uint32_t width, uint32_t height,
                                  const ComposeConsts& k, float rp_inv, float rpf_inv, float fog_strength,
                                  uint8_t* rgb8, cudaStream_t stream, size_t* needed_bytes, bool* too_large) {
    uint32_t halo = (uint32_t)(k.radius > k.fog_radius ? k.radius : k.fog_radius);
    const size_t row_bytes = (size_t)width * 3 * sizeof(float4);
    size_t rows_cap = kStaticScratchBytes / row_bytes;
    *needed_bytes = (size_t)(2 * halo + 2) * row_bytes;
    *too_large = rows_cap < 2 * (size_t)halo + 2;
    if (*too_large) return cudaErrorInvalidValue;  // nothing launched; the caller reports the limit
    float4* base = nullptr;
    cudaError_t e = static_scratch(device, &base);
    if (e != cudaSuccess) return e;
    uint32_t band = (uint32_t)(rows_cap - 2 * halo);
    for (uint32_t y0 = 0; y0 < height; y0 += band) {
        uint32_t y1 = y0 + band < height ? y0 + band : height;
        uint32_t p0 = y0 > halo ? y0 - halo : 0;
        uint32_t p1 = y1 + halo < height ? y1 + halo : height;
        uint32_t prows = p1 - p0;
        size_t plane = (size_t)prows * width;
        float4* p_rad = base;
        float4* p_geo = base + plane;
        float4* p_fog = base + 2 * plane;
        k_pack_band<<<(unsigned)((plane + 255) / 256), 256, 0, stream>>>(in, width, p0, prows, p_rad, p_geo, p_fog);
        dim3 grid((width + 31) / 32, (y1 - y0 + 3) / 4);
        k_compose_band<<<grid, 128, 0, stream>>>(p_rad, p_geo, p_fog, in.variance, width, height, y0, y1, p0, k,
                                                 rp_inv, rpf_inv, fog_strength, rgb8);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace sr

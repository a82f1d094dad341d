// sr_compose.cu — Compositor.Compose (compose.cs:74-99) on the GPU: joint bilateral denoise of
// the surface radiance (Filter compose.cs:101-204), Gaussian blur of the fog radiance
// (FilterFog compose.cs:206-245) and tonemapping to RGB8 (Tonemap compose.cs:247-266,
// Color.ToPixel math.cs:127-136), fused into one pass per pixel.
//
// A packing pass first turns the AOV planes into two float4 planes, {radiance.rgb, luminance}
// and {normal.xyz, depth}, plus {fog.rgb, 0}, so that every filter tap is two 128-bit loads and
// the neighbour luminance is not recomputed per tap.  The packed luminance, normal and depth are
// pre-scaled so that the normal, depth and luminance Gaussians of a tap are one base-2 exponential
// of a sum of three squares, and the two neighbour classes of compose.cs:154-158 (normal present,
// depth finite) ride in the sign bits of the packed luminance and depth.  The taps of a pixel are
// visited in the reference order (rows top to bottom, columns left to right) so the weighted sums
// accumulate in the same order; the spatial weights exp(-d^2 / 2r^2) come from a host-evaluated
// table.  The filter is the reference's up to float rounding (images agree within one code value).
#include <atomic>
#include <cuda_runtime.h>

#include "sr_device.cuh"
#include "sr_kernels.h"

namespace sr {

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

// Scale factors of the packed planes: the Gaussian exp(-x^2 * inv) of compose.cs:165-190 is
// 2^-((s x)^2) with s = sqrt(inv * log2(e)).
struct ComposeScales {
    float n, d, l;  // normal, depth and luminance
};
constexpr uint32_t kSignBit = 0x80000000u;

// Packed planes of pixel i: p_rad = {rgb, s_l * luminance}, p_geo = {s_n * normal, s_d * depth} and
// p_fog = {fog rgb, 0}.  A pixel without a normal (|n|^2 == 0, compose.cs:140) stores a zero normal
// and the luminance with its sign bit set; a pixel without a finite depth stores -0 as its depth.
// Accepted neighbours are always of the centre's class, so a zero normal or depth stands only
// where the reference skips that Gaussian, and luminance and depth are never negative, so their
// magnitudes stay intact.
__global__ void k_pack(DevAovs in, uint32_t n, ComposeScales sc, float4* p_rad, float4* p_geo, float4* p_fog) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Col r{in.radiance[3 * i], in.radiance[3 * i + 1], in.radiance[3 * i + 2]};
    V3 nv{in.normals[3 * i], in.normals[3 * i + 1], in.normals[3 * i + 2]};
    float d = in.depth[i];
    const bool has_n = mag_sqr(nv) > 0.0f, has_d = !isinf(d);
    const float l = sc.l * luminance(r);
    p_rad[i] = make_float4(r.r, r.g, r.b, has_n ? l : __uint_as_float(__float_as_uint(l) | kSignBit));
    const float gd = has_d ? sc.d * d : __uint_as_float(kSignBit);
    p_geo[i] = has_n ? make_float4(sc.n * nv.x, sc.n * nv.y, sc.n * nv.z, gd) : make_float4(0.f, 0.f, 0.f, gd);
    p_fog[i] = make_float4(in.radiance_fog[3 * i], in.radiance_fog[3 * i + 1], in.radiance_fog[3 * i + 2], 0.0f);
}

// 2^x (the hardware approximation; x <= 0 here).
__device__ __forceinline__ float exp2_fast(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The centre pixel of Filter (compose.cs:101-204) and its running sums.
struct FilterCentre {
    uint32_t cls_l, cls_d;  // sign-bit classes of the packed luminance and depth
    float nx, ny, nz, d, l; // packed normal, depth and luminance magnitudes
    float dw;               // denoise weight
    float wsum;
    Col rsum;
};

// One tap of Filter (compose.cs:150-198) for centre c: neighbour q0 = {rgb, packed luminance},
// q1 = {packed normal, packed depth}, spatial weight ws.
__device__ __forceinline__ void filter_tap(FilterCentre& c, const float4& q0, const float4& q1, float ws) {
    // neighbours of another class are rejected (compose.cs:154-158)
    if ((int)((__float_as_uint(q0.w) ^ c.cls_l) | (__float_as_uint(q1.w) ^ c.cls_d)) < 0) return;
    const float dx = c.nx - q1.x, dy = c.ny - q1.y, dz = c.nz - q1.z;
    const float dd = c.d - fabsf(q1.w);
    const float dl = fmaxf(0.0f, fabsf(q0.w) - c.l);
    float e = dx * dx;
    e = __fmaf_rn(dy, dy, e);
    e = __fmaf_rn(dz, dz, e);
    e = __fmaf_rn(dd, dd, e);
    e = __fmaf_rn(dl, dl, e);
    const float w = (c.dw * ws) * exp2_fast(-e);
    c.wsum += w;
    c.rsum = Col{__fmaf_rn(q0.x, w, c.rsum.r), __fmaf_rn(q0.y, w, c.rsum.g), __fmaf_rn(q0.z, w, c.rsum.b)};
}

// Taps kx in [kx0, kx1] of one kernel row: prow / grow point at the row's column x, wrow at its
// spatial weights (centre column at offset 0).
__device__ __forceinline__ void filter_row(FilterCentre& c, const float4* __restrict__ prow,
                                           const float4* __restrict__ grow, const float* __restrict__ wrow, int kx0,
                                           int kx1) {
#pragma unroll 1
    for (int kx = kx0; kx <= kx1; ++kx) filter_tap(c, __ldg(prow + kx), __ldg(grow + kx), __ldg(wrow + kx));
}

// Unroll factor of the two-row kernel's column loop and its minimum resident blocks per SM (the
// register cap).  Measured at 1920x1080: unroll 2 at 6 blocks (80 registers) 7.0 ms; unroll 1 at 6
// or 8 blocks 7.5 ms; unroll 2 at 8 blocks (64 registers, spills) 8.2 ms.
#ifndef SR_COMPOSE_COL_UNROLL
#define SR_COMPOSE_COL_UNROLL 2
#endif
#ifndef SR_COMPOSE_MIN_BLOCKS
#define SR_COMPOSE_MIN_BLOCKS 6
#endif
constexpr int kComposeColUnroll = SR_COMPOSE_COL_UNROLL;

// Columns kx in [kx0, kx1] of one image row for two vertically adjacent pixels a and b (MODE bit 0:
// the column is a tap of a, bit 1: of b), each tap column loaded once for both; wa / wb point at
// the row's spatial weights of each pixel's kernel.
template <int MODE>
__device__ __forceinline__ void filter_cols(FilterCentre& a, FilterCentre& b, const float4* __restrict__ prow,
                                            const float4* __restrict__ grow, const float* __restrict__ wa,
                                            const float* __restrict__ wb, int kx0, int kx1) {
#pragma unroll kComposeColUnroll
    for (int kx = kx0; kx <= kx1; ++kx) {
        const float4 q0 = __ldg(prow + kx), q1 = __ldg(grow + kx);
        if (MODE & 1) filter_tap(a, q0, q1, __ldg(wa + kx));
        if (MODE & 2) filter_tap(b, q0, q1, __ldg(wb + kx));
    }
}

// FilterFog compose.cs:206-245 for pixel (x, y) with fog radiance `fog`.
__device__ __forceinline__ Col filter_fog(const float4* __restrict__ p_fog, uint32_t width, uint32_t height,
                                          const ComposeConsts& k, const float* __restrict__ fog_spatial, int x, int y,
                                          Col fog) {
    const int R = k.fog_radius;
    const int side = 2 * R + 1;
    const float* row_half = fog_spatial + side * side;
    float wsum = 1.0f;
    Col rsum = fog;
    const int ky0 = max(-R, -y), ky1 = min(R, (int)height - 1 - y);
    for (int ky = ky0; ky <= ky1; ++ky) {
        const int hw = (int)__ldg(row_half + ky + R);
        const int kx0 = max(-hw, -x), kx1 = min(hw, (int)width - 1 - x);
        const float* wrow = fog_spatial + (ky + R) * side + R;
        const float4* frow = p_fog + (size_t)(y + ky) * width + x;
        for (int kx = kx0; kx <= kx1; ++kx) {
            if (kx == 0 && ky == 0) continue;
            const float w = __ldg(wrow + kx);
            const float4 f = __ldg(frow + kx);
            wsum += w;
            rsum = Col{__fmaf_rn(f.x, w, rsum.r), __fmaf_rn(f.y, w, rsum.g), __fmaf_rn(f.z, w, rsum.b)};
        }
    }
    return rsum / wsum;
}

// The centre of Filter for pixel ci (packed c0 = {rgb, packed luminance}, c1 = {packed normal,
// depth}); false when its denoise weight takes the early out (compose.cs:125-131).
__device__ __forceinline__ bool filter_centre(FilterCentre& c, const ComposeConsts& k, const float4& c0,
                                              const float4& c1, float variance) {
    const Col main = col3(c0);
    const float lum = luminance(main);
    const float boost = 1.0f + lum * k.lum_boost;
    c.dw = fminf(variance * boost * k.strength, k.strength_max);
    if (c.dw < 1e-4f) return false;
    c.cls_l = __float_as_uint(c0.w) & kSignBit;
    c.cls_d = __float_as_uint(c1.w) & kSignBit;
    c.nx = c1.x, c.ny = c1.y, c.nz = c1.z;
    c.d = fabsf(c1.w);
    c.l = fabsf(c0.w);
    c.wsum = 1.0f;
    c.rsum = main;
    return true;
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
        FilterCentre c;
        if (filter_centre(c, k, c0, __ldg(p_geo + ci), __ldg(variance + ci))) {
            const int R = k.radius;
            const int side = 2 * R + 1;
            const float* row_half = spatial + side * side;
            const int ky0 = max(-R, -y), ky1 = min(R, (int)height - 1 - y);
            for (int ky = ky0; ky <= ky1; ++ky) {
                const int hw = (int)__ldg(row_half + ky + R);
                const int kx0 = max(-hw, -x), kx1 = min(hw, (int)width - 1 - x);
                const float* wrow = spatial + (ky + R) * side + R;
                const float4* prow = p_rad + (size_t)(y + ky) * width + x;
                const float4* grow = p_geo + (size_t)(y + ky) * width + x;
                if (ky != 0) {
                    filter_row(c, prow, grow, wrow, kx0, kx1);
                } else {  // the centre itself is not a tap
                    filter_row(c, prow, grow, wrow, kx0, -1);
                    filter_row(c, prow, grow, wrow, 1, kx1);
                }
            }
            main = c.rsum / c.wsum;
        }
        fog = filter_fog(p_fog, width, height, k, fog_spatial, x, y, fog);
    }
    const Col total = main + fog;
    if (linear) linear[3 * ci] = total.r, linear[3 * ci + 1] = total.g, linear[3 * ci + 2] = total.b;
    if (rgb8) tonemap(k, total, rgb8 + ci * 3);
}

// Two vertically adjacent pixels per thread (SR_COMPOSE_ROWS = 2): a = (x, y) and b = (x, y + 1)
// walk the union of their kernel rows together, and each tap column of a row is loaded once for
// both.  Each pixel still takes exactly its own taps in the reference order (per row: the columns
// only the wider of the two kernels covers on the left, the shared columns, those on the right),
// so its sums -- and the image -- are those of k_compose.
#ifndef SR_COMPOSE_ROWS
#define SR_COMPOSE_ROWS 2
#endif

__global__ void __launch_bounds__(128, SR_COMPOSE_MIN_BLOCKS) k_compose_rows2(const float4* __restrict__ p_rad,
                                                       const float4* __restrict__ p_geo,
                                                       const float4* __restrict__ p_fog,
                                                       const float* __restrict__ variance, uint32_t width,
                                                       uint32_t height, ComposeConsts k,
                                                       const float* __restrict__ spatial,
                                                       const float* __restrict__ fog_spatial, int denoise,
                                                       uint8_t* rgb8, float* linear) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = 2 * (int)(blockIdx.y * 4 + (threadIdx.x >> 5));
    if (x >= (int)width || y >= (int)height) return;
    const bool b_in = y + 1 < (int)height;
    const size_t ca = (size_t)y * width + x, cb = ca + width;
    const float4 a0 = __ldg(p_rad + ca);
    float4 b0 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (b_in) b0 = __ldg(p_rad + cb);
    Col main_a = col3(a0), main_b = col3(b0);
    if (denoise) {
        // ---- Filter compose.cs:101-204 for both pixels ----
        FilterCentre A, B;
        const bool fa = filter_centre(A, k, a0, __ldg(p_geo + ca), __ldg(variance + ca));
        const bool fb = b_in && filter_centre(B, k, b0, __ldg(p_geo + cb), __ldg(variance + cb));
        if (fa || fb) {
            const int R = k.radius;
            const int side = 2 * R + 1;
            const float* row_half = spatial + side * side;
            const int colmin = -x, colmax = (int)width - 1 - x;
            // image rows y + ky for ky in [-R, R + 1]: row ky of a's kernel and row ky - 1 of b's
            const int ky0 = max(-R, -y), ky1 = min(R + 1, (int)height - 1 - y);
            for (int ky = ky0; ky <= ky1; ++ky) {
                const int ka = ky, kb = ky - 1;
                const int hwa = fa && ka <= R ? (int)__ldg(row_half + ka + R) : -1;
                const int hwb = fb && kb >= -R ? (int)__ldg(row_half + kb + R) : -1;
                const float* wa = spatial + (ka + R) * side + R;
                const float* wb = spatial + (kb + R) * side + R;
                const float4* prow = p_rad + (size_t)(y + ky) * width + x;
                const float4* grow = p_geo + (size_t)(y + ky) * width + x;
                // a pixel's own centre is not one of its taps
                const int skip = (ka == 0 ? 1 : 0) | (kb == 0 ? 2 : 0);
                auto run = [&](int mode, int k0, int k1) {
                    if (k0 > k1 || mode == 0) return;
                    auto cols = [&](int m, int c0, int c1) {
                        if (c0 > c1) return;
                        if (m == 1)
                            filter_cols<1>(A, B, prow, grow, wa, wb, c0, c1);
                        else if (m == 2)
                            filter_cols<2>(A, B, prow, grow, wa, wb, c0, c1);
                        else if (m == 3)
                            filter_cols<3>(A, B, prow, grow, wa, wb, c0, c1);
                    };
                    if ((mode & skip) && k0 <= 0 && 0 <= k1) {
                        cols(mode, k0, -1);
                        cols(mode & ~skip, 0, 0);
                        cols(mode, 1, k1);
                    } else {
                        cols(mode, k0, k1);
                    }
                };
                const int hmin = min(hwa, hwb), hmax = max(hwa, hwb);
                if (hmax < 0) continue;
                const int wide = hwa > hwb ? 1 : 2;  // the pixel whose kernel row is wider
                const int lo = max(-hmax, colmin), hi = min(hmax, colmax);
                if (hmin < 0) {
                    run(wide, lo, hi);
                } else {
                    const int clo = max(-hmin, colmin), chi = min(hmin, colmax);
                    run(wide, lo, clo - 1);
                    run(3, clo, chi);
                    run(wide, chi + 1, hi);
                }
            }
            if (fa) main_a = A.rsum / A.wsum;
            if (fb) main_b = B.rsum / B.wsum;
        }
    }
    auto finish = [&](size_t ci, int py, const Col& m) {
        Col fog = col3(__ldg(p_fog + ci));
        if (denoise) fog = filter_fog(p_fog, width, height, k, fog_spatial, x, py, fog);
        const Col total = m + fog;
        if (linear) linear[3 * ci] = total.r, linear[3 * ci + 1] = total.g, linear[3 * ci + 2] = total.b;
        if (rgb8) tonemap(k, total, rgb8 + ci * 3);
    };
    finish(ca, y, main_a);
    if (b_in) finish(cb, y + 1, main_b);
}

cudaError_t launch_compose(const DevAovs& in, uint32_t width, uint32_t height, const ComposeConsts& k,
                           const float* spatial, const float* fog_spatial, bool denoise, uint8_t* rgb8,
                           float4* scratch, cudaStream_t stream, float* linear) {
    uint32_t n = width * height;
    if (n == 0) return cudaSuccess;
    float4* p_rad = scratch;
    float4* p_geo = scratch + n;
    float4* p_fog = scratch + 2 * (size_t)n;
    const float log2e = 1.4426950408889634f;
    const ComposeScales sc{sqrtf(k.normal_limit_inv * log2e), sqrtf(k.depth_limit_inv * log2e),
                           sqrtf(k.lum_limit_inv * log2e)};
    k_pack<<<(n + 255) / 256, 256, 0, stream>>>(in, n, sc, p_rad, p_geo, p_fog);
    if (SR_COMPOSE_ROWS == 2) {
        dim3 grid((width + 31) / 32, (height + 7) / 8);
        k_compose_rows2<<<grid, 128, 0, stream>>>(p_rad, p_geo, p_fog, in.variance, width, height, k, spatial,
                                                  fog_spatial, denoise ? 1 : 0, rgb8, linear);
    } else {
        dim3 grid((width + 31) / 32, (height + 3) / 4);
        k_compose<<<grid, 128, 0, stream>>>(p_rad, p_geo, p_fog, in.variance, width, height, k, spatial,
                                            fog_spatial, denoise ? 1 : 0, rgb8, linear);
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

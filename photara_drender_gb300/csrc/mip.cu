// Mipmapped (trilinear) texture sampling and its adjoint, the filtering the reference lists as planned
// (README.md:141, docs/architecture.md:64): a box-filtered pyramid beside the caller's texture, an
// isotropic level of detail from the pixel-space uv derivatives, and per level the same texel-centre
// bilinear addressing as texture_forward.hlsl.
//
// * Level k+1 has max(1, size >> 1) texels per side; texel (x, y) is the mean of level k's texels
//   {2x, min(2x + 1, w - 1)} x {2y, min(2y + 1, h - 1)}, summed as ((a + b) + (c + d)) * 0.25.
// * With uv_da = (du/dx, du/dy, dv/dx, dv/dy) per pixel, lod = 0.5 log2(max(|(du/dx W, dv/dx H)|^2,
//   |(du/dy W, dv/dy H)|^2)) (W, H of level 0), clamped to [0, levels - 1]; the sample is
//   (1 - f) * bilinear(level l) + f * bilinear(level l + 1) with l = floor(lod), f = lod - l, and exactly
//   bilinear(level l) when f = 0 (so lod <= 0 equals texture_forward bit for bit).
// * The adjoint scatters into every level it sampled, then folds the pyramid's gradient down to level 0
//   (the transpose of the box filter, coarsest level first). The level of detail is a constant of the
//   adjoint: no gradient reaches uv_da.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr uint32_t kMaxLevels = 24;

struct MipLevels {
    uint32_t n;                 // levels including level 0
    uint32_t w[kMaxLevels], h[kMaxLevels];
    uint64_t off[kMaxLevels];   // texel offset of level k >= 1 in the pyramid buffer
};

MipLevels mip_levels(uint32_t w, uint32_t h, uint32_t max_level) {
    MipLevels L{};
    L.n = 1;
    L.w[0] = w;
    L.h[0] = h;
    uint64_t off = 0;
    while (L.n < kMaxLevels && (L.w[L.n - 1] > 1 || L.h[L.n - 1] > 1) && L.n - 1 < max_level) {
        const uint32_t k = L.n;
        L.w[k] = L.w[k - 1] > 1 ? L.w[k - 1] >> 1 : 1;
        L.h[k] = L.h[k - 1] > 1 ? L.h[k - 1] >> 1 : 1;
        L.off[k] = off;
        off += (uint64_t)L.w[k] * L.h[k];
        ++L.n;
    }
    L.off[0] = off;  // level 0 lives in the caller's texture; off[0] holds the pyramid's texel count
    return L;
}

__global__ void mip_down_kernel(const float* __restrict__ src, uint32_t sw, uint32_t sh, float* __restrict__ dst,
                                uint32_t dw, uint32_t dh, uint32_t C) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)dw * dh) return;
    const uint32_t x = (uint32_t)(i % dw), y = (uint32_t)(i / dw);
    const uint32_t x0 = 2 * x, x1 = min(2 * x + 1, sw - 1), y0 = 2 * y, y1 = min(2 * y + 1, sh - 1);
    for (uint32_t c = 0; c < C; ++c) {
        const float a = src[((uint64_t)y0 * sw + x0) * C + c], b = src[((uint64_t)y0 * sw + x1) * C + c];
        const float d = src[((uint64_t)y1 * sw + x0) * C + c], e = src[((uint64_t)y1 * sw + x1) * C + c];
        dst[i * C + c] = ((a + b) + (d + e)) * 0.25f;
    }
}

// level of detail of one pixel (NaN or -inf -> 0)
__device__ __forceinline__ float pixel_lod(float4 da, uint32_t w0, uint32_t h0, uint32_t n) {
    const float ux = da.x * (float)w0, vx = da.z * (float)h0, uy = da.y * (float)w0, vy = da.w * (float)h0;
    const float m = fmaxf(ux * ux + vx * vx, uy * uy + vy * vy);
    const float lod = 0.5f * log2f(m);
    return lod > 0.0f ? fminf(lod, (float)(n - 1)) : 0.0f;
}

struct LevelTaps {
    uint64_t o[4];
    float w[4];
    float fx, fy;
};

// texture_forward.hlsl's taps at one level (texel centres, address mode)
__device__ __forceinline__ LevelTaps level_taps(float2 uv, uint32_t w, uint32_t h, uint32_t mode) {
    LevelTaps t;
    const float tx = uv.x * (float)w - 0.5f, ty = uv.y * (float)h - 0.5f;
    const int32_t bx = f2i_sat(floorf(tx)), by = f2i_sat(floorf(ty));
    const float fx = tx - floorf(tx), fy = ty - floorf(ty);
    const int32_t x0 = address_coordinate(bx, w, mode), x1 = address_coordinate(add1(bx), w, mode);
    const int32_t y0 = address_coordinate(by, h, mode), y1 = address_coordinate(add1(by), h, mode);
    t.o[0] = (uint64_t)(uint32_t)y0 * w + (uint32_t)x0;
    t.o[1] = (uint64_t)(uint32_t)y0 * w + (uint32_t)x1;
    t.o[2] = (uint64_t)(uint32_t)y1 * w + (uint32_t)x0;
    t.o[3] = (uint64_t)(uint32_t)y1 * w + (uint32_t)x1;
    t.w[0] = (1.0f - fx) * (1.0f - fy);
    t.w[1] = fx * (1.0f - fy);
    t.w[2] = (1.0f - fx) * fy;
    t.w[3] = fx * fy;
    t.fx = fx;
    t.fy = fy;
    return t;
}

struct MipArgs {
    const float* tex0;
    const float* pyr;
    MipLevels L;
    uint32_t C, mode;
};

__device__ __forceinline__ const float* level_data(const MipArgs& a, uint32_t k) {
    return k == 0 ? a.tex0 : a.pyr + a.L.off[k] * a.C;
}

__global__ void mip_forward_kernel(MipArgs a, const float2* __restrict__ uv, const float4* __restrict__ uv_da,
                                   const float4* __restrict__ raster, size_t P, float* __restrict__ out) {
    const uint32_t view = blockIdx.y;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const uint32_t C = a.C;
    if (raster_id(raster[pix].w) == 0) {
        for (uint32_t c = 0; c < C; ++c) out[pix * C + c] = 0.0f;
        return;
    }
    const float lod = pixel_lod(uv_da[pix], a.L.w[0], a.L.h[0], a.L.n);
    const uint32_t l0 = (uint32_t)floorf(lod);
    const float f = lod - floorf(lod);
    const uint32_t l1 = min(l0 + 1, a.L.n - 1);
    const float2 u = uv[pix];
    const LevelTaps t0 = level_taps(u, a.L.w[l0], a.L.h[l0], a.mode);
    const float* d0 = level_data(a, l0);
    const bool blend = f > 0.0f;
    LevelTaps t1 = t0;
    const float* d1 = d0;
    if (blend) {
        t1 = level_taps(u, a.L.w[l1], a.L.h[l1], a.mode);
        d1 = level_data(a, l1);
    }
    for (uint32_t c = 0; c < C; ++c) {
        const float s0 = d0[t0.o[0] * C + c] * t0.w[0] + d0[t0.o[1] * C + c] * t0.w[1] + d0[t0.o[2] * C + c] * t0.w[2] +
                         d0[t0.o[3] * C + c] * t0.w[3];
        if (!blend) {
            out[pix * C + c] = s0;
            continue;
        }
        const float s1 = d1[t1.o[0] * C + c] * t1.w[0] + d1[t1.o[1] * C + c] * t1.w[1] + d1[t1.o[2] * C + c] * t1.w[2] +
                         d1[t1.o[3] * C + c] * t1.w[3];
        out[pix * C + c] = (1.0f - f) * s0 + f * s1;
    }
}

// grad_pyr has the pyramid's layout; grad_tex0 is level 0's gradient. grad_uv may be null.
__global__ void mip_backward_kernel(MipArgs a, const float2* __restrict__ uv, const float4* __restrict__ uv_da,
                                    const float4* __restrict__ raster, size_t P, const float* __restrict__ grad_out,
                                    float* __restrict__ grad_tex0, float* __restrict__ grad_pyr,
                                    float2* __restrict__ grad_uv) {
    const uint32_t view = blockIdx.y;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const uint32_t C = a.C;
    if (raster_id(raster[pix].w) == 0) {
        if (grad_uv) grad_uv[pix] = make_float2(0.0f, 0.0f);
        return;
    }
    const float lod = pixel_lod(uv_da[pix], a.L.w[0], a.L.h[0], a.L.n);
    const uint32_t l0 = (uint32_t)floorf(lod);
    const float f = lod - floorf(lod);
    const uint32_t levels[2] = {l0, min(l0 + 1, a.L.n - 1)};
    const float weights[2] = {f > 0.0f ? 1.0f - f : 1.0f, f};
    const float2 u = uv[pix];
    float gu = 0.0f, gv = 0.0f;
    for (int s = 0; s < 2; ++s) {
        if (weights[s] == 0.0f) continue;
        const uint32_t k = levels[s];
        const uint32_t w = a.L.w[k], h = a.L.h[k];
        const LevelTaps t = level_taps(u, w, h, a.mode);
        const float* d = level_data(a, k);
        float* g = k == 0 ? grad_tex0 : grad_pyr + a.L.off[k] * C;
        for (uint32_t c = 0; c < C; ++c) {
            const float gc = grad_out[pix * C + c] * weights[s];
            if (gc == 0.0f) continue;
#pragma unroll
            for (int q = 0; q < 4; ++q) atomicAdd(g + t.o[q] * C + c, t.w[q] * gc);
            const float c00 = d[t.o[0] * C + c], c10 = d[t.o[1] * C + c], c01 = d[t.o[2] * C + c];
            const float c11 = d[t.o[3] * C + c];
            gu += gc * (((1.0f - t.fy) * (c10 - c00) + t.fy * (c11 - c01)) * (float)w);
            gv += gc * (((1.0f - t.fx) * (c01 - c00) + t.fx * (c11 - c10)) * (float)h);
        }
    }
    if (grad_uv) grad_uv[pix] = make_float2(gu, gv);
}

// the box filter's transpose: every parent texel of level k + 1 adds a quarter of its gradient to each
// of its four children at level k (a child counted twice when a side is one texel wide)
__global__ void mip_up_kernel(const float* __restrict__ gparent, uint32_t pw, uint32_t ph, float* __restrict__ gchild,
                              uint32_t cw, uint32_t ch, uint32_t C) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)pw * ph) return;
    const uint32_t x = (uint32_t)(i % pw), y = (uint32_t)(i / pw);
    const uint32_t x0 = 2 * x, x1 = min(2 * x + 1, cw - 1), y0 = 2 * y, y1 = min(2 * y + 1, ch - 1);
    for (uint32_t c = 0; c < C; ++c) {
        const float g = gparent[i * C + c] * 0.25f;
        if (g == 0.0f) continue;
        atomicAdd(gchild + ((uint64_t)y0 * cw + x0) * C + c, g);
        atomicAdd(gchild + ((uint64_t)y0 * cw + x1) * C + c, g);
        atomicAdd(gchild + ((uint64_t)y1 * cw + x0) * C + c, g);
        atomicAdd(gchild + ((uint64_t)y1 * cw + x1) * C + c, g);
    }
}

// d attribute / d pixel from the barycentric derivatives [db0/dx, db0/dy, db1/dx, db1/dy]:
// a = b0 a0 + b1 a1 + (1 - b0 - b1) a2, so da/dx = db0/dx (a0 - a2) + db1/dx (a1 - a2).
__global__ void interpolate_derivatives_kernel(const float* __restrict__ attrs, uint32_t V, uint32_t A,
                                               const uint3* __restrict__ idx, uint32_t T,
                                               const float4* __restrict__ raster, const float4* __restrict__ deriv,
                                               size_t P, float* __restrict__ out) {
    const uint32_t view = blockIdx.y;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    float* o = out + pix * A * 2;
    const uint32_t id = raster_id(raster[pix].w);
    const uint3 vi = (id != 0 && id <= T) ? idx[id - 1] : make_uint3(0xffffffffu, 0, 0);
    if (id == 0 || id > T || vi.x >= V || vi.y >= V || vi.z >= V) {
        for (uint32_t k = 0; k < 2 * A; ++k) o[k] = 0.0f;
        return;
    }
    const float4 db = deriv[pix];
    for (uint32_t k = 0; k < A; ++k) {
        const float a0 = attrs[(size_t)vi.x * A + k], a1 = attrs[(size_t)vi.y * A + k];
        const float a2 = attrs[(size_t)vi.z * A + k];
        o[2 * k] = db.x * (a0 - a2) + db.z * (a1 - a2);
        o[2 * k + 1] = db.y * (a0 - a2) + db.w * (a1 - a2);
    }
}

uint32_t blocks(uint64_t n) { return (uint32_t)((n + 255) / 256); }

pdr_status check_mip(const float* tex, uint32_t w, uint32_t h, uint32_t C, uint32_t mode) {
    if (!tex || w == 0 || h == 0) return set_error(PDR_INVALID_ARGUMENT, "texture must have shape [height, width, channels]");
    if (C == 0 || C > 64) return set_error(PDR_INVALID_ARGUMENT, "texture channels must be 1..64");
    if (mode > 2) return set_error(PDR_INVALID_ARGUMENT, "address_mode must be clamp, wrap or mirror");
    return PDR_OK;
}

}  // namespace
}  // namespace pdr

using namespace pdr;

extern "C" {

pdr_status pdr_mip_pyramid_size(uint32_t width, uint32_t height, uint32_t max_level, uint32_t* levels,
                                uint64_t* pyramid_texels) {
    if (!levels || !pyramid_texels || width == 0 || height == 0)
        return set_error(PDR_INVALID_ARGUMENT, "mip pyramid size needs a positive texture size and outputs");
    const MipLevels L = mip_levels(width, height, max_level);
    *levels = L.n;
    *pyramid_texels = L.off[0];
    return PDR_OK;
}

pdr_status pdr_mip_build(const float* texture, uint32_t width, uint32_t height, uint32_t channels, uint32_t max_level,
                         float* pyramid, void* stream) {
    pdr_status st = check_mip(texture, width, height, channels, 0);
    if (st) return st;
    const MipLevels L = mip_levels(width, height, max_level);
    if (L.n > 1 && !pyramid) return set_error(PDR_INVALID_ARGUMENT, "the pyramid buffer is required");
    const cudaStream_t s = (cudaStream_t)stream;
    for (uint32_t k = 1; k < L.n; ++k) {
        const float* src = k == 1 ? texture : pyramid + L.off[k - 1] * channels;
        mip_down_kernel<<<blocks((uint64_t)L.w[k] * L.h[k]), 256, 0, s>>>(src, L.w[k - 1], L.h[k - 1],
                                                                         pyramid + L.off[k] * channels, L.w[k], L.h[k],
                                                                         channels);
    }
    return set_cuda_error(cudaGetLastError(), "mip_build");
}

pdr_status pdr_texture_forward_mip(const float* texture, const float* pyramid, uint32_t width, uint32_t height,
                                   uint32_t channels, uint32_t max_level, uint32_t address_mode, const float* uv,
                                   const float* uv_da, const float* raster, uint32_t views, uint64_t pixels_per_view,
                                   float* sampled, void* stream) {
    pdr_status st = check_mip(texture, width, height, channels, address_mode);
    if (st) return st;
    if (!uv || !uv_da || !raster || !sampled || views == 0 || views > 65535u)
        return set_error(PDR_INVALID_ARGUMENT, "uv, uv_da, raster and output are required");
    MipArgs a{texture, pyramid, mip_levels(width, height, max_level), channels, address_mode};
    if (a.L.n > 1 && !pyramid) return set_error(PDR_INVALID_ARGUMENT, "the pyramid buffer is required");
    if (pixels_per_view == 0) return PDR_OK;
    const dim3 grid(blocks(pixels_per_view), views);
    mip_forward_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(a, reinterpret_cast<const float2*>(uv),
                                                               reinterpret_cast<const float4*>(uv_da),
                                                               reinterpret_cast<const float4*>(raster),
                                                               pixels_per_view, sampled);
    return set_cuda_error(cudaGetLastError(), "texture_forward_mip");
}

pdr_status pdr_texture_backward_mip(const float* texture, const float* pyramid, uint32_t width, uint32_t height,
                                    uint32_t channels, uint32_t max_level, uint32_t address_mode, const float* uv,
                                    const float* uv_da, const float* raster, uint32_t views, uint64_t pixels_per_view,
                                    const float* grad_sampled, float* grad_texture, float* grad_pyramid, float* grad_uv,
                                    void* stream) {
    pdr_status st = check_mip(texture, width, height, channels, address_mode);
    if (st) return st;
    if (!uv || !uv_da || !raster || !grad_sampled || !grad_texture || views == 0 || views > 65535u)
        return set_error(PDR_INVALID_ARGUMENT, "uv, uv_da, raster, grad_sampled and grad_texture are required");
    MipArgs a{texture, pyramid, mip_levels(width, height, max_level), channels, address_mode};
    if (a.L.n > 1 && (!pyramid || !grad_pyramid))
        return set_error(PDR_INVALID_ARGUMENT, "the pyramid and its gradient buffer are required");
    const cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(grad_texture, 0, (size_t)width * height * channels * sizeof(float), s);
    if (!e && a.L.n > 1) e = cudaMemsetAsync(grad_pyramid, 0, (size_t)a.L.off[0] * channels * sizeof(float), s);
    if (e) return set_cuda_error(e, "texture_backward_mip");
    if (pixels_per_view) {
        const dim3 grid(blocks(pixels_per_view), views);
        mip_backward_kernel<<<grid, 256, 0, s>>>(a, reinterpret_cast<const float2*>(uv),
                                                 reinterpret_cast<const float4*>(uv_da),
                                                 reinterpret_cast<const float4*>(raster), pixels_per_view, grad_sampled,
                                                 grad_texture, grad_pyramid, reinterpret_cast<float2*>(grad_uv));
    }
    for (uint32_t k = a.L.n - 1; k >= 1; --k) {
        float* child = k == 1 ? grad_texture : grad_pyramid + a.L.off[k - 1] * channels;
        mip_up_kernel<<<blocks((uint64_t)a.L.w[k] * a.L.h[k]), 256, 0, s>>>(
            grad_pyramid + a.L.off[k] * channels, a.L.w[k], a.L.h[k], child, a.L.w[k - 1], a.L.h[k - 1], channels);
    }
    return set_cuda_error(cudaGetLastError(), "texture_backward_mip");
}

pdr_status pdr_interpolate_derivatives(const float* attributes, uint32_t vertex_count, uint32_t attribute_count,
                                       const uint32_t* indices, uint32_t triangle_count, const float* raster,
                                       const float* barycentric_derivatives, uint32_t views, uint64_t pixels_per_view,
                                       float* attribute_derivatives, void* stream) {
    if (!attributes || !indices || !raster || !barycentric_derivatives || !attribute_derivatives ||
        vertex_count == 0 || attribute_count == 0 || triangle_count == 0 || views == 0 || views > 65535u)
        return set_error(PDR_INVALID_ARGUMENT, "interpolate_derivatives needs attributes, indices, raster and outputs");
    if (pixels_per_view == 0) return PDR_OK;
    const dim3 grid(blocks(pixels_per_view), views);
    interpolate_derivatives_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
        attributes, vertex_count, attribute_count, reinterpret_cast<const uint3*>(indices), triangle_count,
        reinterpret_cast<const float4*>(raster), reinterpret_cast<const float4*>(barycentric_derivatives),
        pixels_per_view, attribute_derivatives);
    return set_cuda_error(cudaGetLastError(), "interpolate_derivatives");
}

}  // extern "C"

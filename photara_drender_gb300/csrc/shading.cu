// Attribute interpolation and bilinear texture sampling with their adjoints, many views per launch.
//
// Reference path: shaders/interpolate_forward.hlsl, interpolate_grad_attributes.hlsl,
// interpolate_grad_raster.hlsl, texture_forward.hlsl, texture_grad_texture.hlsl (+ the
// texel->sample table of src/rasterizer.cpp:187-258), texture_grad_uv.hlsl.
//
// The reference's attribute and texel gradients are gathers over host-built tables (an
// O(V*A*P) pixel loop for attributes). Here every pixel scatters its contributions with atomics;
// sums therefore differ from the reference only in summation order.
#include <cuda_runtime.h>

#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

__global__ void interpolate_forward_kernel(const float* __restrict__ attr_all, size_t attr_stride, uint32_t V,
                                           uint32_t A, const uint3* __restrict__ idx, uint32_t T,
                                           const float4* __restrict__ raster, size_t P, float* __restrict__ out) {
    const uint32_t view = blockIdx.y;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const float4 r = raster[pix];
    const uint32_t id = raster_id(r.w);
    float* o = out + pix * A;
    uint3 vi = make_uint3(0, 0, 0);
    bool ok = id != 0 && id <= T;
    if (ok) {
        vi = idx[id - 1];
        ok = vi.x < V && vi.y < V && vi.z < V;
    }
    if (!ok) {
        for (uint32_t a = 0; a < A; ++a) o[a] = 0.0f;
        return;
    }
    const float* attr = attr_all + (size_t)view * attr_stride;
    const float u = r.x, v = r.y, w = 1.0f - u - v;
    for (uint32_t a = 0; a < A; ++a) {
        const float a0 = attr[(size_t)vi.x * A + a], a1 = attr[(size_t)vi.y * A + a], a2 = attr[(size_t)vi.z * A + a];
        o[a] = u * a0 + v * a1 + w * a2;
    }
}

// grad_raster follows interpolate_grad_raster.hlsl; grad_attr receives weight * grad per distinct
// vertex of the pixel's triangle, the weight accumulated as interpolate_grad_attributes.hlsl:42-54.
__global__ void interpolate_backward_kernel(const float* __restrict__ attr_all, size_t attr_stride, uint32_t V,
                                            uint32_t A, const uint3* __restrict__ idx, uint32_t T,
                                            const float4* __restrict__ raster, size_t P,
                                            const float* __restrict__ grad_out, float* __restrict__ grad_attr_all,
                                            float4* __restrict__ grad_raster, bool accumulate) {
    const uint32_t view = blockIdx.y;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const float4 r = raster[pix];
    const uint32_t id = raster_id(r.w);
    if (id == 0 || id > T) {
        if (grad_raster && !accumulate) grad_raster[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const uint3 vi = idx[id - 1];
    const float* g = grad_out + pix * A;
    const float u = r.x, v = r.y;
    if (grad_attr_all) {
        float* grad_attr = grad_attr_all + (size_t)view * attr_stride;
        const uint32_t vs[3] = {vi.x, vi.y, vi.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint32_t vx = vs[k];
            bool first = true;
            for (int j = 0; j < k; ++j) first = first && vs[j] != vx;
            if (!first || vx >= V) continue;
            float wgt = 0.0f;
            if (vi.x == vx) wgt += u;
            if (vi.y == vx) wgt += v;
            if (vi.z == vx) wgt += 1.0f - u - v;
            for (uint32_t a = 0; a < A; ++a) atomicAdd(grad_attr + (size_t)vx * A + a, wgt * g[a]);
        }
    }
    if (grad_raster) {
        float gx = 0.0f, gy = 0.0f;
        if (vi.x < V && vi.y < V && vi.z < V) {
            const float* attr = attr_all + (size_t)view * attr_stride;
            for (uint32_t a = 0; a < A; ++a) {
                const float a0 = attr[(size_t)vi.x * A + a], a1 = attr[(size_t)vi.y * A + a];
                const float a2 = attr[(size_t)vi.z * A + a];
                gx += g[a] * (a0 - a2);
                gy += g[a] * (a1 - a2);
            }
        }
        if (accumulate) {
            const float4 o = grad_raster[pix];
            grad_raster[pix] = make_float4(o.x + gx, o.y + gy, o.z, o.w);
        } else {
            grad_raster[pix] = make_float4(gx, gy, 0.0f, 0.0f);
        }
    }
}

struct Taps {
    uint32_t o[4];  // texel indices (y * tw + x)
    float w[4];
};

// texture_forward.hlsl:55-73 in fp32.
__device__ __forceinline__ Taps taps_fp32(float2 uv, uint32_t tw, uint32_t th, uint32_t mode, float* fx_out,
                                          float* fy_out) {
    const float tx = uv.x * (float)tw - 0.5f;
    const float ty = uv.y * (float)th - 0.5f;
    const int32_t bx = f2i_sat(floorf(tx)), by = f2i_sat(floorf(ty));
    const float fx = tx - floorf(tx), fy = ty - floorf(ty);
    const int32_t x0 = address_coordinate(bx, tw, mode), x1 = address_coordinate(add1(bx), tw, mode);
    const int32_t y0 = address_coordinate(by, th, mode), y1 = address_coordinate(add1(by), th, mode);
    Taps t;
    t.o[0] = (uint32_t)y0 * tw + (uint32_t)x0;
    t.o[1] = (uint32_t)y0 * tw + (uint32_t)x1;
    t.o[2] = (uint32_t)y1 * tw + (uint32_t)x0;
    t.o[3] = (uint32_t)y1 * tw + (uint32_t)x1;
    t.w[0] = (1.0f - fx) * (1.0f - fy);
    t.w[1] = fx * (1.0f - fy);
    t.w[2] = (1.0f - fx) * fy;
    t.w[3] = fx * fy;
    *fx_out = fx;
    *fy_out = fy;
    return t;
}

template <int kC>
__global__ void texture_forward_kernel(const float* __restrict__ tex_all, size_t tex_stride, uint32_t tw, uint32_t th,
                                       uint32_t C, uint32_t mode, const float2* __restrict__ uv,
                                       const float4* __restrict__ raster, size_t P, float* __restrict__ out) {
    const uint32_t view = blockIdx.y;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const uint32_t nc = kC > 0 ? (uint32_t)kC : C;
    if (raster_id(raster[pix].w) == 0) {
        if (kC == 4) {
            reinterpret_cast<float4*>(out)[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            for (uint32_t c = 0; c < nc; ++c) out[pix * nc + c] = 0.0f;
        }
        return;
    }
    float fx, fy;
    const Taps t = taps_fp32(uv[pix], tw, th, mode, &fx, &fy);
    const float* tex = tex_all + (size_t)view * tex_stride;
    if (kC == 4) {
        const float4* t4 = reinterpret_cast<const float4*>(tex);
        const float4 c0 = __ldg(t4 + t.o[0]), c1 = __ldg(t4 + t.o[1]), c2 = __ldg(t4 + t.o[2]), c3 = __ldg(t4 + t.o[3]);
        float4 r;
        r.x = c0.x * t.w[0] + c1.x * t.w[1] + c2.x * t.w[2] + c3.x * t.w[3];
        r.y = c0.y * t.w[0] + c1.y * t.w[1] + c2.y * t.w[2] + c3.y * t.w[3];
        r.z = c0.z * t.w[0] + c1.z * t.w[1] + c2.z * t.w[2] + c3.z * t.w[3];
        r.w = c0.w * t.w[0] + c1.w * t.w[1] + c2.w * t.w[2] + c3.w * t.w[3];
        reinterpret_cast<float4*>(out)[pix] = r;
    } else {
        for (uint32_t c = 0; c < nc; ++c) {
            const float v0 = __ldg(tex + (size_t)t.o[0] * nc + c), v1 = __ldg(tex + (size_t)t.o[1] * nc + c);
            const float v2 = __ldg(tex + (size_t)t.o[2] * nc + c), v3 = __ldg(tex + (size_t)t.o[3] * nc + c);
            out[pix * nc + c] = v0 * t.w[0] + v1 * t.w[1] + v2 * t.w[2] + v3 * t.w[3];
        }
    }
}

// grad_texture: pixels with raster.w != 0 scatter weight * grad to their four texels, the
// weights computed from the double-precision texel position of src/rasterizer.cpp:207-229
// (reproduced exactly with integer arithmetic). grad_uv follows texture_grad_uv.hlsl in fp32.
template <int kC>
__global__ void texture_backward_kernel(const float* __restrict__ tex_all, size_t tex_stride, uint32_t tw,
                                        uint32_t th, uint32_t C, uint32_t mode, const float2* __restrict__ uv,
                                        const float4* __restrict__ raster, size_t P, const float* __restrict__ grad,
                                        float* __restrict__ grad_tex_all, float2* __restrict__ grad_uv,
                                        uint32_t* __restrict__ status) {
    const uint32_t view = blockIdx.y;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const uint32_t nc = kC > 0 ? (uint32_t)kC : C;
    const float rw = raster[pix].w;
    const float2 u = uv[pix];
    const float* g = grad + pix * nc;
    if (grad_tex_all && rw != 0.0f) {
        int32_t bx, by;
        float fx, fy;
        const int ex = exact_texel_coordinate(u.x, tw, &bx, &fx);
        const int ey = exact_texel_coordinate(u.y, th, &by, &fy);
        if (ex | ey) {
            const int code = ((ex | ey) & kTexelNonFinite) ? kTexelNonFinite : kTexelRange;
            atomicMax(status + kStatusTexelError, (uint32_t)code);
        } else {
            const int32_t xs[2] = {address_coordinate(bx, tw, mode), address_coordinate(bx + 1, tw, mode)};
            const int32_t ys[2] = {address_coordinate(by, th, mode), address_coordinate(by + 1, th, mode)};
            const float w[4] = {(1.0f - fx) * (1.0f - fy), fx * (1.0f - fy), (1.0f - fx) * fy, fx * fy};
            const uint32_t o[4] = {(uint32_t)ys[0] * tw + (uint32_t)xs[0], (uint32_t)ys[0] * tw + (uint32_t)xs[1],
                                   (uint32_t)ys[1] * tw + (uint32_t)xs[0], (uint32_t)ys[1] * tw + (uint32_t)xs[1]};
            float* gt = grad_tex_all + (size_t)view * tex_stride;
            if (kC == 4) {
                const float4 gg = reinterpret_cast<const float4*>(grad)[pix];
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    red_add_v4_texel(gt + (size_t)o[k] * 4, make_float4(w[k] * gg.x, w[k] * gg.y, w[k] * gg.z, w[k] * gg.w),
                                     (size_t)tw * th < P);
            } else {
                for (int k = 0; k < 4; ++k)
                    for (uint32_t c = 0; c < nc; ++c) atomicAdd(gt + (size_t)o[k] * nc + c, w[k] * g[c]);
            }
        }
    }
    if (grad_uv) {
        if (raster_id(rw) == 0) {
            grad_uv[pix] = make_float2(0.0f, 0.0f);
            return;
        }
        float fx, fy;
        const Taps t = taps_fp32(u, tw, th, mode, &fx, &fy);
        const float* tex = tex_all + (size_t)view * tex_stride;
        float gx = 0.0f, gy = 0.0f;
        for (uint32_t c = 0; c < nc; ++c) {
            const float c00 = __ldg(tex + (size_t)t.o[0] * nc + c), c10 = __ldg(tex + (size_t)t.o[1] * nc + c);
            const float c01 = __ldg(tex + (size_t)t.o[2] * nc + c), c11 = __ldg(tex + (size_t)t.o[3] * nc + c);
            const float dx = (1.0f - fy) * (c10 - c00) + fy * (c11 - c01);
            const float dy = (1.0f - fx) * (c01 - c00) + fx * (c11 - c10);
            gx += g[c] * (dx * (float)tw);
            gy += g[c] * (dy * (float)th);
        }
        grad_uv[pix] = make_float2(gx, gy);
    }
}

}  // namespace

cudaError_t launch_interpolate_forward(const float* attr, size_t attr_view_stride, uint32_t V, uint32_t A,
                                       const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                       size_t P, float* out, cudaStream_t stream) {
    const dim3 grid((uint32_t)((P + 255) / 256), views);
    interpolate_forward_kernel<<<grid, 256, 0, stream>>>(attr, attr_view_stride, V, A,
                                                         reinterpret_cast<const uint3*>(idx), T,
                                                         reinterpret_cast<const float4*>(raster), P, out);
    return cudaGetLastError();
}

cudaError_t launch_interpolate_backward(const float* attr, size_t attr_view_stride, uint32_t V, uint32_t A,
                                        const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                        size_t P, const float* grad_out, float* grad_attr, float* grad_raster,
                                        cudaStream_t stream, bool accumulate_raster) {
    if (grad_attr) {
        const size_t n = attr_view_stride == 0 ? (size_t)V * A : attr_view_stride * views;
        cudaError_t err = cudaMemsetAsync(grad_attr, 0, n * sizeof(float), stream);
        if (err != cudaSuccess) return err;
    }
    const dim3 grid((uint32_t)((P + 255) / 256), views);
    interpolate_backward_kernel<<<grid, 256, 0, stream>>>(attr, attr_view_stride, V, A,
                                                          reinterpret_cast<const uint3*>(idx), T,
                                                          reinterpret_cast<const float4*>(raster), P, grad_out,
                                                          grad_attr, reinterpret_cast<float4*>(grad_raster),
                                                          accumulate_raster);
    return cudaGetLastError();
}

cudaError_t launch_texture_forward(const float* tex, size_t tex_view_stride, uint32_t tw, uint32_t th, uint32_t C,
                                   uint32_t mode, const float* uv, const float* raster, uint32_t views, size_t P,
                                   float* out, cudaStream_t stream) {
    const dim3 grid((uint32_t)((P + 255) / 256), views);
    if (C == 4)
        texture_forward_kernel<4><<<grid, 256, 0, stream>>>(tex, tex_view_stride, tw, th, C, mode,
                                                            reinterpret_cast<const float2*>(uv),
                                                            reinterpret_cast<const float4*>(raster), P, out);
    else
        texture_forward_kernel<0><<<grid, 256, 0, stream>>>(tex, tex_view_stride, tw, th, C, mode,
                                                            reinterpret_cast<const float2*>(uv),
                                                            reinterpret_cast<const float4*>(raster), P, out);
    return cudaGetLastError();
}

cudaError_t launch_texture_backward(const float* tex, size_t tex_view_stride, uint32_t tw, uint32_t th, uint32_t C,
                                    uint32_t mode, const float* uv, const float* raster, uint32_t views, size_t P,
                                    const float* grad, float* grad_tex, float* grad_uv, uint32_t* status,
                                    cudaStream_t stream) {
    if (grad_tex) {
        const size_t n = tex_view_stride == 0 ? (size_t)tw * th * C : tex_view_stride * views;
        cudaError_t err = cudaMemsetAsync(grad_tex, 0, n * sizeof(float), stream);
        if (err != cudaSuccess) return err;
    }
    const dim3 grid((uint32_t)((P + 255) / 256), views);
    if (C == 4)
        texture_backward_kernel<4><<<grid, 256, 0, stream>>>(tex, tex_view_stride, tw, th, C, mode,
                                                             reinterpret_cast<const float2*>(uv),
                                                             reinterpret_cast<const float4*>(raster), P, grad,
                                                             grad_tex, reinterpret_cast<float2*>(grad_uv), status);
    else
        texture_backward_kernel<0><<<grid, 256, 0, stream>>>(tex, tex_view_stride, tw, th, C, mode,
                                                             reinterpret_cast<const float2*>(uv),
                                                             reinterpret_cast<const float4*>(raster), P, grad,
                                                             grad_tex, reinterpret_cast<float2*>(grad_uv), status);
    return cudaGetLastError();
}

}  // namespace pdr

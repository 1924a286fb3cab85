// Texture-atlas refinement: view preparation, masked Charbonnier photometric gradient, seam
// gradient, chart-aware total variation and the dense Adam update, plus the native driver that
// records the whole optimisation as one CUDA graph.
//
// Reference path: src/texture_refiner.cpp:174-454, shaders/atlas_photometric_gradient.hlsl,
// atlas_seam_gradient.hlsl, atlas_adam_update.hlsl; total variation from
// python/photara_drender/atlas.py:84-115 (the native reference refiner has none; weight 0 keeps
// the reference's objective).
//
// Atlas state in HBM: texture, gradient, first and second moments, each [H][W][3] fp32 (the
// reference's layout), 16-byte aligned so the dense Adam pass moves float4s.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr int kPhotoThreads = 256;

// texture_refiner.cpp:228-242: target RGB, mask = clamp(external mask) on covered pixels.
__global__ void prepare_view_kernel(const float* __restrict__ image, uint32_t C, const float* __restrict__ ext_mask,
                                    const float4* __restrict__ raster, size_t P, float* __restrict__ target,
                                    float* __restrict__ mask) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    target[p * 3] = image[p * C];
    target[p * 3 + 1] = image[p * C + 1];
    target[p * 3 + 2] = image[p * C + 2];
    float m = 0.0f;
    if (raster[p].w != 0.0f) {
        m = 1.0f;
        if (ext_mask) {
            const float e = ext_mask[p];
            m = e < 0.0f ? 0.0f : (1.0f < e ? 1.0f : e);  // std::clamp
        }
    }
    mask[p] = m;
}

struct ClampTaps {
    uint32_t o[4];
    float w[4];
};

// atlas_photometric_gradient.hlsl:56-74 / atlas_seam_gradient.hlsl:31-48
__device__ __forceinline__ ClampTaps clamp_taps(float u, float v, uint32_t tw, uint32_t th) {
    const float px = u * (float)tw - 0.5f, py = v * (float)th - 0.5f;
    const int32_t bx = f2i_sat(floorf(px)), by = f2i_sat(floorf(py));
    const float fx = px - floorf(px), fy = py - floorf(py);
    const uint32_t x0 = (uint32_t)clampi(bx, 0, (int32_t)tw - 1), x1 = (uint32_t)clampi(add1(bx), 0, (int32_t)tw - 1);
    const uint32_t y0 = (uint32_t)clampi(by, 0, (int32_t)th - 1), y1 = (uint32_t)clampi(add1(by), 0, (int32_t)th - 1);
    ClampTaps t;
    t.o[0] = y0 * tw + x0;
    t.o[1] = y0 * tw + x1;
    t.o[2] = y1 * tw + x0;
    t.o[3] = y1 * tw + x1;
    t.w[0] = (1.0f - fx) * (1.0f - fy);
    t.w[1] = fx * (1.0f - fy);
    t.w[2] = (1.0f - fx) * fy;
    t.w[3] = fx * fy;
    return t;
}

// The refiner's gradient is [texels][4] (RGB and one unused float), so a bilinear tap adds its three
// channel values with one 16-byte vector reduction instead of three scalar atomics.
__device__ __forceinline__ void red_rgb(float* grad, uint32_t texel, float r, float g, float b) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(grad + (size_t)texel * 4), "f"(r), "f"(g),
                 "f"(b), "f"(0.0f)
                 : "memory");
}

__device__ __forceinline__ float block_sum(float v) {
    __shared__ float warp_sums[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_sums[warp] = v;
    __syncthreads();
    float s = 0.0f;
    if (warp == 0) {
        s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    return s;
}

// One launch covers the batch views of one step (blockIdx.y = batch slot); view choice follows
// texture_refiner.cpp:318-340: view = (step * batch + slot) % view_count.
__global__ void __launch_bounds__(kPhotoThreads, 8)  // 32 registers: full occupancy
photometric_kernel(const float* __restrict__ tex, uint32_t tw, uint32_t th, const pdr_refine_view* __restrict__ views,
                   uint32_t nviews, uint32_t step, uint32_t batch, float eps, float norm, float* __restrict__ grad,
                   float* __restrict__ loss) {
    const pdr_refine_view v = views[((size_t)step * batch + blockIdx.y) % nviews];
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float local = 0.0f;
    if (p < v.pixel_count) {
        const float m = v.mask[p];
        if (m > 0.0f) {
            const float2 uv = reinterpret_cast<const float2*>(v.uv)[p];
            const ClampTaps t = clamp_taps(uv.x, uv.y, tw, th);
            float og[3];
#pragma unroll
            for (uint32_t c = 0; c < 3; ++c) {
                float rendered = 0.0f;
#pragma unroll
                for (int k = 0; k < 4; ++k) rendered += __ldg(tex + (size_t)t.o[k] * 3 + c) * t.w[k];
                const float d = rendered - v.target[p * 3 + c];
                const float robust = sqrtf(d * d + eps * eps);
                og[c] = d / robust * m * norm;
                local += robust * m * norm;
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) red_rgb(grad, t.o[k], og[0] * t.w[k], og[1] * t.w[k], og[2] * t.w[k]);
        }
    }
    const float s = block_sum(local);
    if (threadIdx.x == 0 && s != 0.0f) atomicAdd(loss + step, s);
}

// atlas_seam_gradient.hlsl:50-100
__global__ void seam_kernel(const float* __restrict__ tex, uint32_t tw, uint32_t th, const float4* __restrict__ pairs,
                            uint32_t npairs, float eps, float norm, float* __restrict__ grad, float* __restrict__ loss,
                            uint32_t loss_index) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float local = 0.0f;
    if (i < npairs) {
        const float4 pr = pairs[i];
        const ClampTaps a = clamp_taps(pr.x, pr.y, tw, th);
        const ClampTaps b = clamp_taps(pr.z, pr.w, tw, th);
        float g[3];
#pragma unroll
        for (uint32_t c = 0; c < 3; ++c) {
            float c0 = 0.0f, c1 = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                c0 += __ldg(tex + (size_t)a.o[k] * 3 + c) * a.w[k];
                c1 += __ldg(tex + (size_t)b.o[k] * 3 + c) * b.w[k];
            }
            const float d = c0 - c1;
            const float robust = sqrtf(d * d + eps * eps);
            g[c] = d / robust * norm;
            local += robust * norm;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            red_rgb(grad, a.o[k], g[0] * a.w[k], g[1] * a.w[k], g[2] * a.w[k]);
            red_rgb(grad, b.o[k], -g[0] * b.w[k], -g[1] * b.w[k], -g[2] * b.w[k]);
        }
    }
    const float s = block_sum(local);
    if (threadIdx.x == 0 && s != 0.0f) atomicAdd(loss + loss_index, s);
}

// One pair term of the chart-aware TV gradient, d / sqrt(d^2 + eps^2) * scale, with the reciprocal
// square root (about 2 ulp) in place of a square root and an IEEE division: the TV gradient is held to
// a tolerance (atlas.py's autograd, 1e-6 relative), and the exact form made the fused TV + Adam pass
// instruction-bound (12 square roots and divisions per texel).
__device__ __forceinline__ float tv_term(float d, float eps, float scale) { return d * rsqrtf(d * d + eps * eps) * scale; }

// Chart-aware robust total variation of atlas.py:84-115 added into the gradient: each valid
// same-chart neighbour pair (right and down) contributes d / sqrt(d^2 + eps^2) * scale.
__global__ void tv_kernel(const float* __restrict__ tex, uint32_t tw, uint32_t th, const uint8_t* __restrict__ valid,
                          const int32_t* __restrict__ chart, float eps, float scale, float* __restrict__ grad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tw * th) return;
    const uint32_t x = i % tw, y = i / tw;
    if (!valid[i]) return;
    float g[3] = {0.0f, 0.0f, 0.0f};
    const int32_t ci = chart ? chart[i] : 0;
    // pairs (i, right), (i, down) subtract; pairs (left, i), (up, i) add
    const int64_t nb[4] = {x + 1 < tw ? (int64_t)i + 1 : -1, y + 1 < th ? (int64_t)i + tw : -1,
                           x > 0 ? (int64_t)i - 1 : -1, y > 0 ? (int64_t)i - tw : -1};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (nb[k] < 0) continue;
        const size_t j = (size_t)nb[k];
        if (!valid[j] || (chart && chart[j] != ci)) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float d = k < 2 ? tex[j * 3 + c] - tex[(size_t)i * 3 + c] : tex[(size_t)i * 3 + c] - tex[j * 3 + c];
            const float gg = tv_term(d, eps, scale);
            g[c] += k < 2 ? -gg : gg;
        }
    }
    float4* gp = reinterpret_cast<float4*>(grad) + i;
    float4 cur = *gp;
    cur.x += g[0];
    cur.y += g[1];
    cur.z += g[2];
    *gp = cur;
}

// atlas_adam_update.hlsl:20-43 for one value (the update, then the gradient cleared).
__device__ __forceinline__ void adam_one(float& x, float& g, float& m, float& v, float lr, float b1, float b2, float eps,
                                         float bc1, float bc2, float cmin, float cmax) {
    const float m1 = b1 * m + (1.0f - b1) * g;
    const float m2 = b2 * v + (1.0f - b2) * g * g;
    m = m1;
    v = m2;
    const float c1 = m1 / bc1, c2 = m2 / bc2;
    x = clamp_hlsl(x - lr * c1 / (sqrtf(c2) + eps), cmin, cmax);
    g = 0.0f;
}

__global__ void adam_kernel(float* __restrict__ tex, float* __restrict__ grad, float* __restrict__ m1,
                            float* __restrict__ m2, size_t texels, float lr, float b1, float b2, float eps, float bc1,
                            float bc2, float cmin, float cmax) {
    // one texel per thread: texture and moments [texels][3], gradient [texels][4] read and cleared as one
    // float4 (measured against four texels per thread, 0.38 ms, and four values per thread with the
    // gradient gathered, 0.36-0.41 ms: 0.33 ms for 16.8 M texels)
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < texels; t += stride) {
        const float4 d = reinterpret_cast<const float4*>(grad)[t];
        float g[3] = {d.x, d.y, d.z};
#pragma unroll
        for (int c = 0; c < 3; ++c)
            adam_one(tex[t * 3 + c], g[c], m1[t * 3 + c], m2[t * 3 + c], lr, b1, b2, eps, bc1, bc2, cmin, cmax);
        reinterpret_cast<float4*>(grad)[t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// The TV gradient of texel i (tv_kernel's arithmetic on tex_in) added to its photometric gradient, then
// the Adam update of adam_kernel into tex_out: one pass over the atlas for a step with total variation.
// tex_in and tex_out are different buffers, so every texel reads its neighbours' values from before the
// step, as the separate TV pass does. Bit-identical to tv_kernel followed by adam_kernel.
__global__ void __launch_bounds__(256, 8)  // 32 registers: full occupancy for the streaming pass
adam_tv_kernel(const float* __restrict__ tex_in, float* __restrict__ tex_out,
                               float* __restrict__ grad, float* __restrict__ m1, float* __restrict__ m2,
                               uint32_t tw, uint32_t th, const uint8_t* __restrict__ valid,
                               const int32_t* __restrict__ chart, float tv_eps, float tv_scale, float lr, float b1,
                               float b2, float eps, float bc1, float bc2, float cmin, float cmax) {
    const size_t texels = (size_t)tw * th;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < texels; t += stride) {
        float4 d = reinterpret_cast<const float4*>(grad)[t];
        if (valid[t]) {
            const uint32_t i = (uint32_t)t, x = i % tw, y = i / tw;
            float g[3] = {0.0f, 0.0f, 0.0f};
            const int32_t ci = chart ? chart[i] : 0;
            const int64_t nb[4] = {x + 1 < tw ? (int64_t)i + 1 : -1, y + 1 < th ? (int64_t)i + tw : -1,
                                   x > 0 ? (int64_t)i - 1 : -1, y > 0 ? (int64_t)i - tw : -1};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (nb[k] < 0) continue;
                const size_t j = (size_t)nb[k];
                if (!valid[j] || (chart && chart[j] != ci)) continue;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float dd = k < 2 ? tex_in[j * 3 + c] - tex_in[t * 3 + c] : tex_in[t * 3 + c] - tex_in[j * 3 + c];
                    const float gg = tv_term(dd, tv_eps, tv_scale);
                    g[c] += k < 2 ? -gg : gg;
                }
            }
            d.x += g[0];
            d.y += g[1];
            d.z += g[2];
        }
        float gv[3] = {d.x, d.y, d.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float x = tex_in[t * 3 + c];
            adam_one(x, gv[c], m1[t * 3 + c], m2[t * 3 + c], lr, b1, b2, eps, bc1, bc2, cmin, cmax);
            tex_out[t * 3 + c] = x;
        }
        reinterpret_cast<float4*>(grad)[t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

}  // namespace

cudaError_t launch_adam_tv(const float* tex_in, float* tex_out, float* grad, float* m, float* v, uint32_t tw,
                           uint32_t th, const uint8_t* valid, const int32_t* chart, float tv_eps, float tv_scale,
                           float lr, float b1, float b2, float eps, float bc1, float bc2, float cmin, float cmax,
                           cudaStream_t stream) {
    const size_t texels = (size_t)tw * th;
    size_t blocks = (texels + 255) / 256;
    if (blocks > 0x7FFFFFFFu) blocks = 0x7FFFFFFFu;
    if (blocks == 0) blocks = 1;
    adam_tv_kernel<<<(unsigned)blocks, 256, 0, stream>>>(tex_in, tex_out, grad, m, v, tw, th, valid, chart, tv_eps,
                                                         tv_scale, lr, b1, b2, eps, bc1, bc2, cmin, cmax);
    return cudaGetLastError();
}

cudaError_t launch_prepare_view(const float* image, uint32_t C, const float* ext_mask, const float* raster, size_t P,
                                float* target, float* mask, cudaStream_t stream) {
    prepare_view_kernel<<<(unsigned)((P + 255) / 256), 256, 0, stream>>>(image, C, ext_mask,
                                                                         reinterpret_cast<const float4*>(raster), P,
                                                                         target, mask);
    return cudaGetLastError();
}

cudaError_t launch_photometric(const float* tex, uint32_t tw, uint32_t th, const pdr_refine_view* views,
                               uint32_t nviews, uint64_t max_pixels, uint32_t step, uint32_t batch, float eps,
                               float norm, float* grad, float* loss, cudaStream_t stream) {
    const dim3 grid((unsigned)((max_pixels + kPhotoThreads - 1) / kPhotoThreads), batch);
    photometric_kernel<<<grid, kPhotoThreads, 0, stream>>>(tex, tw, th, views, nviews, step, batch, eps, norm, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_seam(const float* tex, uint32_t tw, uint32_t th, const float* pairs, uint32_t npairs, float eps,
                        float norm, float* grad, float* loss, uint32_t loss_index, cudaStream_t stream) {
    seam_kernel<<<(npairs + 255) / 256, 256, 0, stream>>>(tex, tw, th, reinterpret_cast<const float4*>(pairs), npairs,
                                                          eps, norm, grad, loss, loss_index);
    return cudaGetLastError();
}

cudaError_t launch_tv(const float* tex, uint32_t tw, uint32_t th, const uint8_t* valid, const int32_t* chart, float eps,
                      float scale, float* grad, cudaStream_t stream) {
    tv_kernel<<<(tw * th + 255) / 256, 256, 0, stream>>>(tex, tw, th, valid, chart, eps, scale, grad);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* tex, float* grad, float* m, float* v, size_t n, float lr, float b1, float b2, float eps,
                        float bc1, float bc2, float cmin, float cmax, cudaStream_t stream) {
    // n = texels * 3 values. One texel per thread (the loop strides only past 2^31 blocks): a grid capped at
    // eight CTAs per SM that looped over the arrays kept fewer loads in flight
    const size_t texels = n / 3;
    size_t blocks = (texels + 255) / 256;
    if (blocks > 0x7FFFFFFFu) blocks = 0x7FFFFFFFu;
    if (blocks == 0) blocks = 1;
    adam_kernel<<<(unsigned)blocks, 256, 0, stream>>>(tex, grad, m, v, texels, lr, b1, b2, eps, bc1, bc2, cmin, cmax);
    return cudaGetLastError();
}

// texture_refiner.cpp:316-415: the per-step scalars in the reference's float arithmetic.
void refine_schedule(const pdr_refine_options* o, uint32_t step, float* lr, float* bc1, float* bc2) {
    const float pi = std::acos(-1.0F);
    const float phase = static_cast<float>(step) / static_cast<float>(o->steps);
    *lr = o->minimum_learning_rate +
          0.5F * (o->learning_rate - o->minimum_learning_rate) * (1.0F + std::cos(pi * phase));
    *bc1 = 1.0F - std::pow(o->adam_beta1, static_cast<float>(step + 1));
    *bc2 = 1.0F - std::pow(o->adam_beta2, static_cast<float>(step + 1));
}

}  // namespace pdr

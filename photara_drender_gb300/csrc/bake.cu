// Texture projection (bake) for all views in one launch, plus the small per-view transforms the
// bake and refine hosts need.
//
// Reference path: src/texture_baker.cpp:156-361 and shaders/project_texture.hlsl. The reference
// dispatches project_texture once per view and keeps the per-texel accumulators in device
// buffers between dispatches; here one thread owns one atlas texel, walks the views in order
// with the accumulators in registers, and writes the host-side normalisation of
// texture_baker.cpp:334-358 directly (colour / weight, valid mask, confidence, source view,
// coverage and face ids). Per-texel results equal the reference's view-by-view sequence.
#include <cuda_runtime.h>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"
#include "projection.cuh"

namespace pdr {
namespace {

__device__ __forceinline__ float lerp_hlsl(float x, float y, float s) { return x * (1.0f - s) + y * s; }

// project_texture.hlsl:46-56: the bilinear photo sample with clamped taps, for channels 0..2 (and 3 when
// the image has four). The tap positions and weights are the same for every channel, so they are
// computed once and each tap's channels are read together.
struct PhotoSample {
    float c0, c1, c2, alpha;
};

__device__ __forceinline__ PhotoSample sample_photo_rgba(const pdr_projection_view& v, float ppx, float ppy) {
    const float tx = ppx - 0.5f, ty = ppy - 0.5f;
    const int32_t bx = f2i_sat(floorf(tx)), by = f2i_sat(floorf(ty));
    const float fx = tx - floorf(tx), fy = ty - floorf(ty);
    const int32_t w = (int32_t)v.width - 1, h = (int32_t)v.height - 1;
    const uint32_t x0 = (uint32_t)clampi(bx, 0, w), x1 = (uint32_t)clampi(add1(bx), 0, w);
    const uint32_t y0 = (uint32_t)clampi(by, 0, h), y1 = (uint32_t)clampi(add1(by), 0, h);
    const uint32_t C = v.channel_count;
    const float* img = v.image;
    const size_t t00 = ((size_t)y0 * v.width + x0) * C, t10 = ((size_t)y0 * v.width + x1) * C;
    const size_t t01 = ((size_t)y1 * v.width + x0) * C, t11 = ((size_t)y1 * v.width + x1) * C;
    float r[4];
#pragma unroll
    for (uint32_t ch = 0; ch < 4; ++ch) {
        if (ch == 3 && C != 4) {
            r[3] = 1.0f;
            break;
        }
        const float v00 = __ldg(img + t00 + ch), v10 = __ldg(img + t10 + ch);
        const float v01 = __ldg(img + t01 + ch), v11 = __ldg(img + t11 + ch);
        r[ch] = lerp_hlsl(lerp_hlsl(v00, v10, fx), lerp_hlsl(v01, v11, fx), fy);
    }
    return {r[0], r[1], r[2], r[3]};
}

// project_texture.hlsl:58-74, with the host-side mask floor of texture_baker.cpp:283-292
// (std::max(mask, floor) on every mask texel) applied to the four taps.
__device__ __forceinline__ float mask_tap(const pdr_projection_view& v, int32_t x, int32_t y, float floor_value) {
    const float m = __ldg(v.visibility_mask + (size_t)y * v.width + x);
    return floor_value > 0.0f && m < floor_value ? floor_value : m;
}

__device__ __forceinline__ float sample_mask(const pdr_projection_view& v, float ppx, float ppy, float floor_value) {
    const int32_t w = (int32_t)v.width, h = (int32_t)v.height;
    const float tx = ppx - 0.5f, ty = ppy - 0.5f;
    const int32_t bx = f2i_sat(floorf(tx)), by = f2i_sat(floorf(ty));
    const float fx = tx - floorf(tx), fy = ty - floorf(ty);
    const int32_t x0 = clampi(bx, 0, w - 1), x1 = clampi(add1(bx), 0, w - 1);
    const int32_t y0 = clampi(by, 0, h - 1), y1 = clampi(add1(by), 0, h - 1);
    const float v00 = mask_tap(v, x0, y0, floor_value), v10 = mask_tap(v, x1, y0, floor_value);
    const float v01 = mask_tap(v, x0, y1, floor_value), v11 = mask_tap(v, x1, y1, floor_value);
    return lerp_hlsl(lerp_hlsl(v00, v10, fx), lerp_hlsl(v01, v11, fx), fy);
}

// project_texture.hlsl:76-101
__device__ __forceinline__ float shadow_visibility(const pdr_projection_view& v, float ppx, float ppy, float depth,
                                                   int32_t r) {
    const int32_t w = (int32_t)v.width, h = (int32_t)v.height;
    const int32_t cx = f2i_sat(floorf(ppx)), cy = f2i_sat(floorf(ppy));
    float visible = 0.0f, count = 0.0f;
    const float4* shadow = reinterpret_cast<const float4*>(v.shadow_raster);
    for (int32_t y = -r; y <= r; ++y) {
        for (int32_t x = -r; x <= r; ++x) {
            const int32_t X = cx + x, Y = cy + y;
            if (X < 0 || Y < 0 || X >= w || Y >= h) continue;
            const float4 s = __ldg(shadow + (size_t)Y * v.width + (size_t)X);
            if (raster_id(s.w) != 0) {
                visible += depth <= s.z + v.depth_bias ? 1.0f : 0.0f;
                count += 1.0f;
            }
        }
    }
    return count > 0.0f ? visible / count : 0.0f;
}

constexpr uint32_t kViewChunk = 32;
static_assert(sizeof(pdr_projection_view) % sizeof(uint4) == 0, "view records are copied as 16-byte words");

__global__ void __launch_bounds__(128, 12)  // 40 registers: 48 warps per SM for the gathers
project_views_kernel(const float* __restrict__ apos, const float* __restrict__ anrm,
                                     const float4* __restrict__ araster, uint32_t N,
                                     const pdr_projection_view* __restrict__ views, uint32_t nviews,
                                     uint32_t blend_mode, uint32_t pcf_radius, uint32_t visibility_mode,
                                     float* __restrict__ color4, float* __restrict__ confidence,
                                     uint32_t* __restrict__ source_view, float* __restrict__ valid_mask,
                                     float* __restrict__ coverage_mask, uint32_t* __restrict__ face_ids,
                                     const uint32_t* __restrict__ vis_bits, uint32_t vis_words) {
    // The view records are staged in shared memory kViewChunk at a time: every texel reads every field of
    // every view, and shared-memory loads are shorter than L1 hits on the global table.
    __shared__ __align__(16) pdr_projection_view sv[kViewChunk];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const float rw = i < N ? araster[i].w : 0.0f;
    const bool active = raster_id(rw) != 0;
    float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f, accw = 0.0f, best = 0.0f;
    uint32_t src = 0xffffffffu;
    float px = 0.0f, py = 0.0f, pz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f;
    if (active) {
        px = apos[(size_t)i * 3];
        py = apos[(size_t)i * 3 + 1];
        pz = apos[(size_t)i * 3 + 2];
        const float nx0 = anrm[(size_t)i * 3], ny0 = anrm[(size_t)i * 3 + 1], nz0 = anrm[(size_t)i * 3 + 2];
        const float nl = sqrtf(nx0 * nx0 + ny0 * ny0 + nz0 * nz0);
        nx = nx0 / nl;
        ny = ny0 / nl;
        nz = nz0 / nl;
    }
    const bool any_active = __syncthreads_or(active) != 0;
    for (uint32_t k0 = 0; any_active && k0 < nviews; k0 += kViewChunk) {
        const uint32_t cnt = min(kViewChunk, nviews - k0);
        __syncthreads();
        constexpr uint32_t kWords = sizeof(pdr_projection_view) / sizeof(uint4);
        for (uint32_t q = threadIdx.x; q < cnt * kWords; q += blockDim.x)
            reinterpret_cast<uint4*>(sv)[q] = __ldg(reinterpret_cast<const uint4*>(views + k0) + q);
        __syncthreads();
        if (!active) continue;
        for (uint32_t kk = 0; kk < cnt; ++kk) {
            const uint32_t k = k0 + kk;
            const pdr_projection_view& v = sv[kk];
            ProjectedTexel pt;
            if (!project_texel(v, px, py, pz, nx, ny, nz, pt)) continue;
            const float ppx = pt.ppx, ppy = pt.ppy, ndz = pt.ndz, vl = pt.vl, cosv = pt.cosv;
            // ray visibility: one bit per (texel, view) from the BVH ray caster, or a per-view array
            float vis = vis_bits ? (float)((__ldg(vis_bits + (size_t)i * vis_words + (k >> 5)) >> (k & 31u)) & 1u)
                                 : (v.ray_visibility ? __ldg(v.ray_visibility + i) : 1.0f);
            if (visibility_mode == 0) vis = shadow_visibility(v, ppx, ppy, ndz, (int32_t)pcf_radius);
            else if (visibility_mode == 1) vis *= shadow_visibility(v, ppx, ppy, ndz, (int32_t)pcf_radius);
            if (v.has_mask) vis *= clamp_hlsl(sample_mask(v, ppx, ppy, v.mask_floor), 0.0f, 1.0f);
            if (vis <= 0.0f) continue;
            const PhotoSample ps = sample_photo_rgba(v, ppx, ppy);
            const float c0 = ps.c0, c1 = ps.c1, c2 = ps.c2, alpha = ps.alpha;
            if (blend_mode == 2) {
                const float dist = fmaxf(vl, 1e-6f);
                const float footprint = cosv / (dist * dist);
                const float ex = clamp_hlsl(vis * alpha * footprint * v.weight, 0.0f, 64.0f);
                const float prev = best;
                const float cur = fmaxf(prev, ex);
                if (cur > prev) {
                    const float rs = expf(prev - cur);
                    acc0 *= rs;
                    acc1 *= rs;
                    acc2 *= rs;
                    accw *= rs;
                    best = cur;
                }
                if (ex >= prev) src = k;
                const float sw = expf(ex - cur);
                if (sw <= 0.0f) continue;
                acc0 += c0 * sw;
                acc1 += c1 * sw;
                acc2 += c2 * sw;
                accw += sw;
                continue;
            }
            const float conf = vis * alpha * cosv * v.weight;
            if (conf <= 0.0f) continue;
            if (conf > best) {
                best = conf;
                src = k;
            }
            if (blend_mode == 0) {
                if (conf >= accw) {
                    acc0 = c0;
                    acc1 = c1;
                    acc2 = c2;
                    accw = conf;
                }
            } else {
                acc0 += c0 * conf;
                acc1 += c1 * conf;
                acc2 += c2 * conf;
                accw += conf;
            }
        }
    }
    if (i >= N) return;
    // texture_baker.cpp:192-204 and 347-358
    const float valid = accw > 0.0f ? 1.0f : 0.0f;
    const float div = blend_mode != 0 && accw > 0.0f ? accw : 1.0f;
    reinterpret_cast<float4*>(color4)[i] = make_float4(acc0 / div, acc1 / div, acc2 / div, valid);
    confidence[i] = accw;
    source_view[i] = src;
    valid_mask[i] = valid;
    const float r = roundf(rw);
    const float cov = r != 0.0f ? 1.0f : 0.0f;
    if (coverage_mask) coverage_mask[i] = cov;
    if (face_ids) face_ids[i] = cov > 0.5f ? (uint32_t)r - 1u : 0xffffffffu;
}

// texture_baker.cpp:92-106 / texture_refiner.cpp:36-50 for every view: [views][V][4].
__global__ void transform_positions_kernel(const float* __restrict__ pos3, uint32_t V,
                                           const float* __restrict__ mats, float4* __restrict__ clip) {
    const uint32_t view = blockIdx.y;
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const float* m = mats + (size_t)view * 16;
    const float x = pos3[(size_t)v * 3], y = pos3[(size_t)v * 3 + 1], z = pos3[(size_t)v * 3 + 2];
    float4 o;
    o.x = m[0] * x + m[1] * y + m[2] * z + m[3];
    o.y = m[4] * x + m[5] * y + m[6] * z + m[7];
    o.z = m[8] * x + m[9] * y + m[10] * z + m[11];
    o.w = m[12] * x + m[13] * y + m[14] * z + m[15];
    clip[(size_t)view * V + v] = o;
}

// texture_baker.cpp:81-90
__global__ void atlas_clip_kernel(const float2* __restrict__ uv, uint32_t V, float4* __restrict__ clip) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const float2 t = uv[v];
    clip[v] = make_float4(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, 0.0f, 1.0f);
}

}  // namespace

cudaError_t launch_project_views(const float* apos, const float* anrm, const float* araster, uint32_t N,
                                 const pdr_projection_view* views, uint32_t nviews, uint32_t blend_mode,
                                 uint32_t pcf_radius, uint32_t visibility_mode, float* color4, float* confidence,
                                 uint32_t* source_view, float* valid_mask, float* coverage_mask, uint32_t* face_ids,
                                 cudaStream_t stream, const uint32_t* vis_bits, uint32_t vis_words) {
    project_views_kernel<<<(N + 127) / 128, 128, 0, stream>>>(
        apos, anrm, reinterpret_cast<const float4*>(araster), N, views, nviews, blend_mode, pcf_radius,
        visibility_mode, color4, confidence, source_view, valid_mask, coverage_mask, face_ids, vis_bits, vis_words);
    return cudaGetLastError();
}

cudaError_t launch_transform_positions(const float* pos3, uint32_t V, const float* mats, uint32_t views, float* clip,
                                       cudaStream_t stream) {
    const dim3 grid((V + 255) / 256, views);
    transform_positions_kernel<<<grid, 256, 0, stream>>>(pos3, V, mats, reinterpret_cast<float4*>(clip));
    return cudaGetLastError();
}

cudaError_t launch_atlas_clip(const float* uv, uint32_t V, float* clip, cudaStream_t stream) {
    atlas_clip_kernel<<<(V + 255) / 256, 256, 0, stream>>>(reinterpret_cast<const float2*>(uv), V,
                                                           reinterpret_cast<float4*>(clip));
    return cudaGetLastError();
}

}  // namespace pdr

// Homogeneous clipping across the near plane, which the reference does not implement (README.md:140,
// docs/architecture.md:62: triangles with a vertex at w <= 1e-8 are skipped, others are rasterized
// unclipped). Opt-in; the default path stays the reference's.
//
// * Clip: every triangle k of a view is clipped against the plane z + w = 0 (OpenGL-style clip space) into
//   at most two triangles. The clipped mesh has a fixed topology shared by all views, so the ordinary
//   multi-view binning and raster launches take it unchanged: four vertex slots per triangle and view
//   (4k .. 4k+3) and the index list slot 2k = (4k, 4k+1, 4k+2), slot 2k+1 = (4k, 4k+2, 4k+3). Per view the
//   slots hold the triangle itself (4th slot unused), the clipped triangle, or the clipped quad; an unused
//   slot is a vertex with w = 0, which binning skips, so a slot triangle touching it covers nothing. An
//   edge's intersection is computed from its lower-indexed vertex, so two triangles sharing the edge get
//   the same point (no cracks). Clipping keeps the winding, so culling is unchanged, and slot order keeps
//   the reference's depth tie rule (lower original triangle first).
// * The clipped mesh is binned and rasterized by the ordinary kernels, which decide coverage and depth.
// * Remap: each covered pixel's triangle id becomes the original k + 1 and its barycentrics, depth and
//   derivatives are recomputed from the original triangle with the rasterizer's homogeneous formulas
//   (winner_barycentrics), which hold for vertices behind the eye too. A triangle that needed no clipping
//   gets bit-identical outputs.
// * Backward: the raster adjoint with its per-triangle visit rule lifted for triangles with a vertex at
//   w <= 1e-8 (such triangles only own pixels after clipping); see raster.cu.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"
#include "raster_tile.cuh"

namespace pdr {
namespace {

// intersection of edge (a, b) with z + w = 0, computed from the lower-indexed vertex
__device__ __forceinline__ float4 near_point(uint32_t ia, float4 pa, uint32_t ib, float4 pb) {
    if (ib < ia) {
        const float4 t = pa;
        pa = pb;
        pb = t;
    }
    const float da = pa.z + pa.w, db = pb.z + pb.w;
    const float t = da / (da - db);
    return make_float4(pa.x + t * (pb.x - pa.x), pa.y + t * (pb.y - pa.y), pa.z + t * (pb.z - pa.z),
                       pa.w + t * (pb.w - pa.w));
}

// One thread per (triangle, view): writes the four vertex slots of the triangle; view 0 also writes the
// shared index list.
__global__ void clip_near_kernel(const float4* __restrict__ clip_all, uint32_t V, const uint3* __restrict__ idx,
                                 uint32_t T, float4* __restrict__ out_pos_all, uint3* __restrict__ out_idx,
                                 uint32_t* __restrict__ status) {
    const uint32_t view = blockIdx.y;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= T) return;
    float4* out = out_pos_all + ((size_t)view * T + k) * 4;
    if (view == 0) {
        out_idx[2 * k] = make_uint3(4 * k, 4 * k + 1, 4 * k + 2);
        out_idx[2 * k + 1] = make_uint3(4 * k, 4 * k + 2, 4 * k + 3);
    }
    const float4 none = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint3 vi = idx[k];
    if (vi.x >= V || vi.y >= V || vi.z >= V) {
        if (status) status[PDR_STATUS_INDEX_ERROR] = 1u;
        out[0] = none;
        out[1] = none;
        out[2] = none;
        out[3] = none;
        return;
    }
    const float4* clip = clip_all + (size_t)view * V;
    const uint32_t iv[3] = {vi.x, vi.y, vi.z};
    const float4 p[3] = {__ldg(clip + vi.x), __ldg(clip + vi.y), __ldg(clip + vi.z)};
    bool in[3];
    int n_in = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        in[c] = p[c].z + p[c].w >= 0.0f;
        n_in += in[c];
    }
    if (n_in == 3) {
        out[0] = p[0];
        out[1] = p[1];
        out[2] = p[2];
        out[3] = none;
        return;
    }
    if (n_in == 0) {
        out[0] = none;
        out[1] = none;
        out[2] = none;
        out[3] = none;
        return;
    }
    if (n_in == 1) {
        // the inside vertex i with the points on its two edges, in the triangle's cyclic order
        const int i = in[0] ? 0 : (in[1] ? 1 : 2);
        const int j = (i + 1) % 3, l = (i + 2) % 3;
        out[0] = p[i];
        out[1] = near_point(iv[i], p[i], iv[j], p[j]);  // on edge i -> j
        out[2] = near_point(iv[l], p[l], iv[i], p[i]);  // on edge l -> i
        out[3] = none;
        return;
    }
    // one outside vertex o: the quad (edge o -> a, a, b, edge b -> o) as slots (0, 1, 2) and (0, 2, 3)
    const int o = !in[0] ? 0 : (!in[1] ? 1 : 2);
    const int a = (o + 1) % 3, b = (o + 2) % 3;
    out[0] = near_point(iv[o], p[o], iv[a], p[a]);
    out[1] = p[a];
    out[2] = p[b];
    out[3] = near_point(iv[b], p[b], iv[o], p[o]);
}

__global__ void remap_near_kernel(const float4* __restrict__ clip_all, uint32_t V, const uint3* __restrict__ idx,
                                  uint32_t T, uint32_t W, uint32_t H, const float4* __restrict__ viewports,
                                  float4* __restrict__ raster, float4* __restrict__ deriv) {
    const uint32_t view = blockIdx.y;
    const size_t P = (size_t)W * H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const uint32_t id = raster_id(raster[pix].w);
    if (id == 0 || id > 2 * T) return;
    const uint32_t k = (id - 1) >> 1;
    const uint3 vi = idx[k];
    if (vi.x >= V || vi.y >= V || vi.z >= V) return;
    const float4* clip = clip_all + (size_t)view * V;
    const float4 p0 = __ldg(clip + vi.x), p1 = __ldg(clip + vi.y), p2 = __ldg(clip + vi.z);
    const float4 vp = viewports[view];
    const uint32_t x = (uint32_t)(p % W), y = (uint32_t)(p / W);
    const WinnerBary wb = winner_barycentrics(p0, p1, p2, sample_ndc(x, vp.x, vp.z), sample_ndc(y, vp.y, vp.w));
    raster[pix] = make_float4(wb.b0, wb.b1, wb.depth, (float)(k + 1));
    if (deriv) deriv[pix] = winner_derivatives(p0, p1, p2, wb, vp);
}

bool near_args_ok(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T) {
    return clip && idx && views > 0 && views <= 65535u && V > 0 && T > 0;
}

}  // namespace
}  // namespace pdr

using namespace pdr;

extern "C" {

pdr_status pdr_clip_near(const float* clip_positions, uint32_t views, uint32_t vertex_count, const uint32_t* indices,
                         uint32_t triangle_count, float* clipped_positions, uint32_t* clipped_indices,
                         uint32_t* status, void* stream) {
    if (!near_args_ok(clip_positions, views, vertex_count, indices, triangle_count) || !clipped_positions ||
        !clipped_indices)
        return set_error(PDR_INVALID_ARGUMENT, "near clipping needs positions, indices and the clipped buffers");
    if (triangle_count > PDR_NEAR_MAX_TRIANGLES)
        return set_error(PDR_OVERFLOW, "near-plane clipping supports at most 8388608 triangles");
    if (((uintptr_t)clip_positions | (uintptr_t)clipped_positions) & 15u)
        return set_error(PDR_INVALID_ARGUMENT, "positions must be 16-byte aligned");
    const dim3 grid((triangle_count + 255) / 256, views);
    clip_near_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4*>(clip_positions), vertex_count, reinterpret_cast<const uint3*>(indices),
        triangle_count, reinterpret_cast<float4*>(clipped_positions), reinterpret_cast<uint3*>(clipped_indices),
        status);
    return set_cuda_error(cudaGetLastError(), "clip_near");
}

pdr_status pdr_remap_near(const float* clip_positions, uint32_t views, uint32_t vertex_count, const uint32_t* indices,
                          uint32_t triangle_count, uint32_t width, uint32_t height, const float* viewports,
                          float* raster, float* barycentric_derivatives, void* stream) {
    const pdr_status st = check_raster_args(clip_positions, views, vertex_count, indices, triangle_count, width,
                                            height, viewports);
    if (st) return st;
    if (!raster) return set_error(PDR_INVALID_ARGUMENT, "near remap needs positions, indices, viewports and the raster");
    if (triangle_count > PDR_NEAR_MAX_TRIANGLES)
        return set_error(PDR_OVERFLOW, "near-plane clipping supports at most 8388608 triangles");
    if (((uintptr_t)clip_positions | (uintptr_t)raster | (uintptr_t)barycentric_derivatives) & 15u)
        return set_error(PDR_INVALID_ARGUMENT, "positions and raster buffers must be 16-byte aligned");
    const size_t P = (size_t)width * height;
    const dim3 grid((uint32_t)((P + 255) / 256), views);
    remap_near_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4*>(clip_positions), vertex_count, reinterpret_cast<const uint3*>(indices),
        triangle_count, width, height, reinterpret_cast<const float4*>(viewports), reinterpret_cast<float4*>(raster),
        reinterpret_cast<float4*>(barycentric_derivatives));
    return set_cuda_error(cudaGetLastError(), "remap_near");
}

pdr_status pdr_rasterize_backward_near(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                       const uint32_t* indices, uint32_t triangle_count, uint32_t width,
                                       uint32_t height, const float* viewports, const float* raster,
                                       const float* grad_raster, const float* grad_barycentric_derivatives,
                                       float* grad_clip_positions, void* stream) {
    const pdr_status st = check_raster_args(clip_positions, views, vertex_count, indices, triangle_count, width,
                                            height, viewports);
    if (st) return st;
    if (!raster || !grad_clip_positions)
        return set_error(PDR_INVALID_ARGUMENT, "raster, grad_raster and grad_clip_positions are required");
    if (((uintptr_t)clip_positions | (uintptr_t)raster | (uintptr_t)grad_raster |
         (uintptr_t)grad_barycentric_derivatives) & 15u)
        return set_error(PDR_INVALID_ARGUMENT, "raster buffers must be 16-byte aligned");
    return set_cuda_error(launch_raster_backward(clip_positions, views, vertex_count, indices, triangle_count, width,
                                                 height, viewports, raster, grad_raster, grad_clip_positions,
                                                 (cudaStream_t)stream, grad_barycentric_derivatives, true),
                          "rasterize_backward_near");
}

}  // extern "C"

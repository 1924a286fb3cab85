// Fused forward and backward of rasterize -> interpolate(attributes), interpolate(uv) -> texture for
// many views (the chain python/photara_drender/atlas.py:36-62 render_textured_mesh runs as three
// autograd functions, each a separate synchronous call in the reference).
//
// Forward: tile binning + one raster launch whose epilogue interpolates and samples for the winner.
// Backward: one thread per pixel runs, in the reference's order and arithmetic, texture_grad_texture
// (double-exact weights, vector atomics), texture_grad_uv, interpolate_grad_attributes /
// interpolate_grad_raster for both attribute sets, and rasterize_backward for the summed raster
// gradient. Per-vertex gradients are summed over each run of adjacent pixels of a warp that hit the
// same triangle (warp shuffles), then the run's last lane adds them to global memory with vector
// reductions. Intermediate grad_uv / grad_raster never leave registers. With sample_differences the
// forward keeps the texel differences of each covered pixel's sample, so the backward reads 32 bytes
// per pixel instead of gathering four texels again.
#include <cuda_runtime.h>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"
#include "render_bwd_tile.cuh"

namespace pdr {
namespace {

// The adjoint runs 16x8 tiles of 128 threads, 12 CTAs per SM (40 registers, a few spills): 2.42 ms on
// 64 views against 2.50 ms for 16x16 tiles of 256 threads at 6 CTAs per SM.
constexpr int kBwdTileH = 8;
constexpr int kBwdThreads = 16 * kBwdTileH;

template <int kA, int kTexAgg>
__global__ void __launch_bounds__(kBwdThreads, 12)
render_backward_kernel(const float4* __restrict__ clip_all, uint32_t V, const uint3* __restrict__ idx, uint32_t T,
                       uint32_t W, uint32_t H, const float4* __restrict__ viewports, uint32_t tcx,
                       const float* __restrict__ attrs, const float2* __restrict__ uv_attrs,
                       const float4* __restrict__ tex, uint32_t tw, uint32_t th, uint32_t mode,
                       const float4* __restrict__ raster, const float2* __restrict__ uv,
                       const float* __restrict__ grad_attr_out, const float4* __restrict__ grad_sampled,
                       float* __restrict__ g_clip_all, float* __restrict__ g_attr, float* __restrict__ g_uv,
                       float* __restrict__ g_tex, const float4* __restrict__ sdiff, uint32_t* __restrict__ status,
                       float* __restrict__ g_vtx_all) {
    const uint32_t view = blockIdx.y;
    const uint32_t tile = blockIdx.x;
    const size_t P = (size_t)W * H;
    BackwardView v;
    v.clip = clip_all + (size_t)view * V;
    v.V = V;
    v.idx = idx;
    v.T = T;
    v.W = W;
    v.H = H;
    v.vp = viewports[view];
    v.attrs = attrs;
    v.uv_attrs = uv_attrs;
    v.tex = tex;
    v.tw = tw;
    v.th = th;
    v.mode = mode;
    v.raster = raster + view * P;
    v.uv = uv ? uv + view * P : nullptr;
    v.grad_attr_out = grad_attr_out ? grad_attr_out + view * P * kA : nullptr;
    v.grad_sampled = grad_sampled ? grad_sampled + view * P : nullptr;
    v.g_clip = g_clip_all + (size_t)view * V * 4;
    v.g_attr = g_attr;
    v.g_uv = g_uv;
    v.g_tex = g_tex;
    v.sdiff = sdiff ? sdiff + view * P * 2 : nullptr;
    v.status = status;
    v.g_vtx = g_vtx_all ? g_vtx_all + (size_t)view * V * vertex_record_floats(kA) : nullptr;
    render_backward_tile<kA, kTexAgg, kBwdTileH>(v, tile % tcx, tile / tcx);
}

// The vertex-gradient records of all views into the outputs: each view's clip gradient (x, y, 0, w), and
// the uv and attribute gradients summed over the views in view order. One thread per vertex; every
// output element is written, so none needs clearing first.
template <int kA>
__global__ void __launch_bounds__(256)
vertex_grad_finish_kernel(const float* __restrict__ rec_all, uint32_t views, uint32_t V, float* __restrict__ g_clip_all,
                          float* __restrict__ g_attr, float* __restrict__ g_uv) {
    constexpr uint32_t kR = vertex_record_floats(kA);
    constexpr uint32_t kNV = 2 + kA + 3;
    const uint32_t vtx = blockIdx.x * blockDim.x + threadIdx.x;
    if (vtx >= V) return;
    float acc[2 + kA];
#pragma unroll
    for (int j = 0; j < 2 + kA; ++j) acc[j] = 0.0f;
    for (uint32_t view = 0; view < views; ++view) {
        const float4* rec = reinterpret_cast<const float4*>(rec_all + ((size_t)view * V + vtx) * kR);
        float r[kR];
#pragma unroll
        for (uint32_t c = 0; c < kR / 4; ++c) {
            const float4 q = __ldcs(rec + c);
            r[4 * c] = q.x;
            r[4 * c + 1] = q.y;
            r[4 * c + 2] = q.z;
            r[4 * c + 3] = q.w;
        }
#pragma unroll
        for (int j = 0; j < 2 + kA; ++j) acc[j] += r[j];
        reinterpret_cast<float4*>(g_clip_all)[(size_t)view * V + vtx] =
            make_float4(r[kNV - 3], r[kNV - 2], 0.0f, r[kNV - 1]);
    }
    if (g_uv) {
        g_uv[(size_t)vtx * 2] = acc[0];
        g_uv[(size_t)vtx * 2 + 1] = acc[1];
    }
    if (g_attr) {
#pragma unroll
        for (int a = 0; a < kA; ++a) g_attr[(size_t)vtx * kA + a] = acc[2 + a];
    }
}

}  // namespace

}  // namespace pdr

using namespace pdr;

extern "C" {

size_t pdr_render_backward_workspace_bytes(uint32_t views, uint32_t vertex_count, uint32_t attribute_count) {
    if (attribute_count > 8) return 0;
    return (size_t)views * vertex_count * vertex_record_floats((int)attribute_count) * sizeof(float);
}

size_t pdr_render_workspace_bytes(uint32_t views, uint32_t triangle_count, uint32_t width, uint32_t height,
                                  uint64_t capacity) {
    return bins_workspace_bytes(views, triangle_count, width, height, capacity);
}

size_t pdr_render_workspace_bytes_tiled(uint32_t views, uint32_t triangle_count, uint32_t width, uint32_t height,
                                        uint64_t capacity, uint32_t tile_width, uint32_t tile_height) {
    if (tile_width == 0 || tile_height == 0) return 0;
    return bins_workspace_bytes(views, triangle_count, width, height, capacity, tile_width, tile_height);
}

namespace {

struct TileConfig {
    uint32_t w, h, k;
};

TileConfig tile_config(const pdr_render_args* a) {
    if (a->tile_width == 0 && a->tile_height == 0 && a->stage_triangles == 0) return {16, 16, 256};
    return {a->tile_width, a->tile_height, a->stage_triangles};
}

pdr_status check_render_forward(const pdr_render_args* a) {
    if (!a || !a->clip_positions || !a->indices || !a->viewports || !a->raster || !a->tile_offsets ||
        !a->tile_triangles || !a->workspace || !a->status)
        return set_error(PDR_INVALID_ARGUMENT, "render arguments are incomplete");
    if (a->views == 0 || a->vertex_count == 0 || a->triangle_count == 0 || a->width == 0 || a->height == 0)
        return set_error(PDR_INVALID_ARGUMENT, "render dimensions must be positive");
    if (a->attributes && (a->attribute_count == 0 || a->attribute_count > 8 || !a->interpolated))
        return set_error(PDR_INVALID_ARGUMENT, "fused rendering supports 1..8 attributes with an output buffer");
    if (a->texture && (!a->uv_attributes || !a->uv || !a->sampled || a->texture_width == 0 || a->texture_height == 0 ||
                       a->address_mode > 2))
        return set_error(PDR_INVALID_ARGUMENT, "texture sampling needs uv attributes and uv/sampled outputs");
    const TileConfig tc = tile_config(a);
    if (!raster_config_supported(tc.w, tc.h, tc.k))
        return set_error(PDR_INVALID_ARGUMENT, "tile shape and stage depth must be 16x16/256, 16x16/128 or 16x8/128");
    const uint64_t tiles = (uint64_t)((a->width + tc.w - 1) / tc.w) * ((a->height + tc.h - 1) / tc.h);
    if (tiles * a->views >= 0x7fffffffull || (uint64_t)a->triangle_count * a->views >= 0x7fffffffull)
        return set_error(PDR_OVERFLOW, "Rasterization output size overflow");
    if (a->capacity > 0xffffffffull) return set_error(PDR_OVERFLOW, "tile list capacity exceeds the u32 tile offsets");
    if (a->workspace_bytes <
        bins_workspace_bytes(a->views, a->triangle_count, a->width, a->height, a->capacity, tc.w, tc.h))
        return set_error(PDR_INVALID_ARGUMENT, "workspace is smaller than pdr_render_workspace_bytes()");
    return PDR_OK;
}

}  // namespace

pdr_status pdr_render_bin(const pdr_render_args* a, void* stream) {
    const pdr_status st = check_render_forward(a);
    if (st) return st;
    const TileConfig tc = tile_config(a);
    const cudaError_t err = launch_bin_tiles(a->clip_positions, a->views, a->vertex_count, a->indices,
                                             a->triangle_count, a->width, a->height, a->viewports, a->tile_offsets,
                                             a->tile_triangles, a->capacity, a->workspace, a->status,
                                             (cudaStream_t)stream, /*sorted=*/false, tc.w, tc.h);
    return set_cuda_error(err, "render_bin");
}

pdr_status pdr_render_raster(const pdr_render_args* a, void* stream) {
    const pdr_status st = check_render_forward(a);
    if (st) return st;
    if (a->sample_differences && ((uintptr_t)a->sample_differences & 15u))
        return set_error(PDR_INVALID_ARGUMENT, "sample_differences must be 16-byte aligned");
    RasterShade shade{a->attributes, a->attribute_count, a->interpolated, a->uv_attributes, a->uv, a->texture,
                      a->texture_width, a->texture_height, a->address_mode, a->sampled,
                      a->texture ? a->sample_differences : nullptr};
    const cudaError_t err = launch_raster_forward(
        a->clip_positions, a->views, a->vertex_count, a->indices, a->triangle_count, a->width, a->height,
        a->viewports, a->cull_mode, a->tile_offsets, a->tile_triangles, a->capacity, a->raster,
        a->barycentric_derivatives, (cudaStream_t)stream, (a->attributes || a->uv_attributes) ? &shade : nullptr,
        a->status, tile_config(a).w, tile_config(a).h, tile_config(a).k);
    return set_cuda_error(err, "render_raster");
}

pdr_status pdr_render_forward(const pdr_render_args* a, void* stream) {
    const pdr_status st = pdr_render_bin(a, stream);
    return st ? st : pdr_render_raster(a, stream);
}

pdr_status pdr_render_backward(const pdr_render_args* a, void* stream) {
    if (!a || !a->clip_positions || !a->indices || !a->viewports || !a->raster || !a->grad_clip_positions || !a->status)
        return set_error(PDR_INVALID_ARGUMENT, "render arguments are incomplete");
    if (a->attributes && (!a->grad_interpolated || !a->grad_attributes || a->attribute_count == 0 ||
                          a->attribute_count > 8))
        return set_error(PDR_INVALID_ARGUMENT, "attribute gradients need grad_interpolated and grad_attributes");
    if (a->texture && (!a->uv || !a->grad_sampled || !a->grad_texture || !a->grad_uv_attributes || !a->uv_attributes))
        return set_error(PDR_INVALID_ARGUMENT, "texture gradients need uv, grad_sampled and gradient outputs");
    // the adjoint adds vertex gradients with vector reductions: clip gradients as float4, uv as float2
    if (((uintptr_t)a->grad_clip_positions & 15u) || ((uintptr_t)a->grad_uv_attributes & 7u) ||
        ((uintptr_t)a->grad_texture & 15u) || ((uintptr_t)a->grad_attributes & 15u) ||
        ((uintptr_t)a->sample_differences & 15u))
        return set_error(PDR_INVALID_ARGUMENT, "gradient outputs must be 16-byte (clip, texture, attributes) / 8-byte (uv) aligned");
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t A = a->attributes ? a->attribute_count : 0;
    // with a workspace of pdr_render_backward_workspace_bytes(): per-view vertex-gradient records, summed
    // into the outputs afterwards; without one, reductions straight into the outputs
    const size_t rec_bytes = pdr_render_backward_workspace_bytes(a->views, a->vertex_count, A);
    float* g_vtx = (a->workspace && a->workspace_bytes >= rec_bytes && !((uintptr_t)a->workspace & 15u))
                       ? static_cast<float*>(a->workspace)
                       : nullptr;
    cudaError_t err = cudaSuccess;
    if (g_vtx) {
        err = cudaMemsetAsync(g_vtx, 0, rec_bytes, s);
    } else {
        err = cudaMemsetAsync(a->grad_clip_positions, 0, (size_t)a->views * a->vertex_count * 4 * sizeof(float), s);
        if (err == cudaSuccess && a->grad_attributes)
            err = cudaMemsetAsync(a->grad_attributes, 0, (size_t)a->vertex_count * a->attribute_count * sizeof(float), s);
        if (err == cudaSuccess && a->grad_uv_attributes)
            err = cudaMemsetAsync(a->grad_uv_attributes, 0, (size_t)a->vertex_count * 2 * sizeof(float), s);
    }
    if (err == cudaSuccess && a->grad_texture)
        err = cudaMemsetAsync(a->grad_texture, 0, (size_t)a->texture_width * a->texture_height * 4 * sizeof(float), s);
    if (err != cudaSuccess) return set_cuda_error(err, "render_backward(memset)");
    const uint32_t tcx = (a->width + kTile - 1) / kTile, tcy = (a->height + kBwdTileH - 1) / kBwdTileH;
    const dim3 grid(tcx * tcy, a->views);
    // warp-aggregated texture-gradient taps for magnified textures (see red_add_v4_texel)
    const bool magnified = (uint64_t)a->texture_width * a->texture_height < (uint64_t)a->width * a->height;
#define PDR_RENDER_BWD_AGG(KA, AGG)                                                                                  \
    render_backward_kernel<KA, AGG><<<grid, kBwdThreads, 0, s>>>(                                                 \
        reinterpret_cast<const float4*>(a->clip_positions), a->vertex_count, reinterpret_cast<const uint3*>(a->indices), \
        a->triangle_count, a->width, a->height, reinterpret_cast<const float4*>(a->viewports), tcx, a->attributes,   \
        reinterpret_cast<const float2*>(a->uv_attributes), reinterpret_cast<const float4*>(a->texture),            \
        a->texture_width, a->texture_height, a->address_mode, reinterpret_cast<const float4*>(a->raster),           \
        reinterpret_cast<const float2*>(a->uv), a->grad_interpolated, reinterpret_cast<const float4*>(a->grad_sampled), \
        a->grad_clip_positions, a->grad_attributes, a->grad_uv_attributes, a->grad_texture,                     \
        reinterpret_cast<const float4*>(a->texture ? a->sample_differences : nullptr), a->status, g_vtx)
#define PDR_RENDER_BWD(KA)                  \
    if (magnified) {                        \
        PDR_RENDER_BWD_AGG(KA, 1);          \
    } else {                                \
        PDR_RENDER_BWD_AGG(KA, 0);          \
    }
    switch (A) {
        case 0: PDR_RENDER_BWD(0); break;
        case 1: PDR_RENDER_BWD(1); break;
        case 2: PDR_RENDER_BWD(2); break;
        case 3: PDR_RENDER_BWD(3); break;
        case 4: PDR_RENDER_BWD(4); break;
        case 5: PDR_RENDER_BWD(5); break;
        case 6: PDR_RENDER_BWD(6); break;
        case 7: PDR_RENDER_BWD(7); break;
        default: PDR_RENDER_BWD(8); break;
    }
#undef PDR_RENDER_BWD
#undef PDR_RENDER_BWD_AGG
    if (g_vtx) {
        const unsigned blocks = (a->vertex_count + 255) / 256;
        float* gc = a->grad_clip_positions;
        float* ga = a->grad_attributes;
        float* gu = a->grad_uv_attributes;
        switch (A) {
            case 0: vertex_grad_finish_kernel<0><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
            case 1: vertex_grad_finish_kernel<1><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
            case 2: vertex_grad_finish_kernel<2><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
            case 3: vertex_grad_finish_kernel<3><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
            case 4: vertex_grad_finish_kernel<4><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
            case 5: vertex_grad_finish_kernel<5><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
            case 6: vertex_grad_finish_kernel<6><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
            case 7: vertex_grad_finish_kernel<7><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
            default: vertex_grad_finish_kernel<8><<<blocks, 256, 0, s>>>(g_vtx, a->views, a->vertex_count, gc, ga, gu); break;
        }
    }
    return set_cuda_error(cudaGetLastError(), "render_backward");
}

}  // extern "C"

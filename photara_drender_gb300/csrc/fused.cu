// Fused forward and backward of rasterize -> interpolate(attributes), interpolate(uv) -> texture for
// many views (the chain python/photara_drender/atlas.py:36-62 render_textured_mesh runs as three
// autograd functions, each a separate synchronous call in the reference).
//
// Forward: tile binning + one raster launch whose epilogue interpolates and samples for the winner.
// Backward: one thread per pixel runs, in the reference's order and arithmetic, texture_grad_texture
// (double-exact weights, vector atomics), texture_grad_uv, interpolate_grad_attributes /
// interpolate_grad_raster for both attribute sets, and rasterize_backward for the summed raster
// gradient. Per-vertex gradients are summed in three stages: over each run of adjacent pixels of a
// warp that hit the same triangle (warp shuffles), then per 16x16 tile in a shared-memory hash table
// written only by each run's last lane, then flushed with one global atomic per (vertex, component).
// Intermediate grad_uv / grad_raster never leave registers.
#include <cuda_runtime.h>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr int kFusedThreads = 256;
constexpr uint32_t kSlots = 512;         // hash slots per CTA
constexpr uint32_t kMaxVals = 2 + 8 + 3; // uv attributes, up to 8 attributes, clip x/y/w
constexpr uint32_t kEmpty = 0xffffffffu;

__device__ __forceinline__ void red_v4(float* addr, float4 v) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

struct VertexTable {
    uint32_t key[kSlots];
    float val[kSlots * kMaxVals];
};

// Finds or claims the slot of vertex v; returns kSlots when the table is full.
__device__ __forceinline__ uint32_t table_slot(VertexTable& tb, uint32_t v) {
    uint32_t s = (v * 2654435761u) >> 23;  // top 9 bits
    for (uint32_t probe = 0; probe < kSlots; ++probe) {
        const uint32_t prev = atomicCAS(&tb.key[s], kEmpty, v);
        if (prev == kEmpty || prev == v) return s;
        s = (s + 1) & (kSlots - 1);
    }
    return kSlots;
}

// Segmented inclusive sums over runs of equal keys in a warp (Hillis-Steele with head flags). The
// add predicates depend only on the keys, so they are computed once and reused for every value.
// Step s adds the value 2^s lanes up; a run of length L needs the steps with 2^s < L, so the scan
// stops after the warp's longest run (usually 2 to 4 pixels of a tile row) instead of after 5 steps.
struct RunScan {
    bool add[5];
    bool tail;
    uint32_t steps;  // warp-uniform
    __device__ __forceinline__ explicit RunScan(uint32_t key) {
        const uint32_t lane = threadIdx.x & 31u;
        const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
        const uint32_t next = __shfl_down_sync(0xffffffffu, key, 1);
        bool f = lane == 0 || prev != key;
        tail = lane == 31 || next != key;
        // distance to the run's head: lane minus the highest head at or below this lane
        const uint32_t heads = __ballot_sync(0xffffffffu, f) & (0xffffffffu >> (31u - lane));
        const uint32_t dist = lane - (31u - (uint32_t)__clz(heads));
        const uint32_t longest = __reduce_max_sync(0xffffffffu, dist);
        steps = 32u - (uint32_t)__clz(longest);  // bit length: 2^steps > longest
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            add[s] = false;
            if ((uint32_t)s >= steps) continue;
            const uint32_t o = 1u << s;
            const bool fy = __shfl_up_sync(0xffffffffu, f, o);
            add[s] = lane >= o && !f;
            f = f || (lane >= o && fy);
        }
    }
    __device__ __forceinline__ float sum(float x) const {
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            if ((uint32_t)s >= steps) break;
            const float y = __shfl_up_sync(0xffffffffu, x, 1u << s);
            if (add[s]) x += y;
        }
        return x;
    }
};

template <int kA>
__global__ void __launch_bounds__(kFusedThreads, 4)
render_backward_kernel(const float4* __restrict__ clip_all, uint32_t V, const uint3* __restrict__ idx, uint32_t T,
                       uint32_t W, uint32_t H, const float4* __restrict__ viewports, uint32_t tcx,
                       const float* __restrict__ attrs, const float2* __restrict__ uv_attrs,
                       const float4* __restrict__ tex, uint32_t tw, uint32_t th, uint32_t mode,
                       const float4* __restrict__ raster, const float2* __restrict__ uv,
                       const float* __restrict__ grad_attr_out, const float4* __restrict__ grad_sampled,
                       float* __restrict__ g_clip_all, float* __restrict__ g_attr, float* __restrict__ g_uv,
                       float* __restrict__ g_tex, uint32_t* __restrict__ status) {
    constexpr uint32_t kNV = 2 + kA + 3;  // per vertex: uv attributes, attributes, clip x/y/w
    __shared__ VertexTable tb;
    const uint32_t view = blockIdx.y;
    const uint32_t tile = blockIdx.x;
    for (uint32_t i = threadIdx.x; i < kSlots; i += kFusedThreads) tb.key[i] = kEmpty;
    for (uint32_t i = threadIdx.x; i < kSlots * kNV; i += kFusedThreads) tb.val[i] = 0.0f;
    __syncthreads();
    float* g_clip = g_clip_all + (size_t)view * V * 4;
    const uint32_t lane = threadIdx.x & 31u;

    const uint32_t px = (tile % tcx) * kTile + (threadIdx.x & 15u);
    const uint32_t py = (tile / tcx) * kTile + (threadIdx.x >> 4);
    bool valid = false;           // pixel contributes vertex gradients (id in [1, T])
    uint3 vi = make_uint3(0, 0, 0);
    float cv[3][kNV];             // per corner contributions
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (uint32_t j = 0; j < kNV; ++j) cv[k][j] = 0.0f;
    uint32_t id = 0;

    if (px < W && py < H) {
        const size_t pix = ((size_t)view * H + py) * W + px;
        const float4 r = raster[pix];
        id = raster_id(r.w);
        const float2 u = uv ? uv[pix] : make_float2(0.0f, 0.0f);
        float gux = 0.0f, guy = 0.0f;
        if (tex) {
            const float4 gs = grad_sampled[pix];
            // texture_grad_texture: pixels with raster.w != 0, double-exact weights (rasterizer.cpp:198-229)
            if (r.w != 0.0f) {
                int32_t bx, by;
                float fx, fy;
                const int ex = exact_texel_coordinate(u.x, tw, &bx, &fx);
                const int ey = exact_texel_coordinate(u.y, th, &by, &fy);
                if (ex | ey) {
                    atomicMax(status + kStatusTexelError, ((ex | ey) & kTexelNonFinite) ? (uint32_t)kTexelNonFinite
                                                                                       : (uint32_t)kTexelRange);
                } else {
                    const int32_t xs0 = address_coordinate(bx, tw, mode), xs1 = address_coordinate(bx + 1, tw, mode);
                    const int32_t ys0 = address_coordinate(by, th, mode), ys1 = address_coordinate(by + 1, th, mode);
                    const float w0 = (1.0f - fx) * (1.0f - fy), w1 = fx * (1.0f - fy), w2 = (1.0f - fx) * fy,
                                w3 = fx * fy;
                    red_v4(g_tex + ((size_t)(uint32_t)ys0 * tw + (uint32_t)xs0) * 4, make_float4(w0 * gs.x, w0 * gs.y, w0 * gs.z, w0 * gs.w));
                    red_v4(g_tex + ((size_t)(uint32_t)ys0 * tw + (uint32_t)xs1) * 4, make_float4(w1 * gs.x, w1 * gs.y, w1 * gs.z, w1 * gs.w));
                    red_v4(g_tex + ((size_t)(uint32_t)ys1 * tw + (uint32_t)xs0) * 4, make_float4(w2 * gs.x, w2 * gs.y, w2 * gs.z, w2 * gs.w));
                    red_v4(g_tex + ((size_t)(uint32_t)ys1 * tw + (uint32_t)xs1) * 4, make_float4(w3 * gs.x, w3 * gs.y, w3 * gs.z, w3 * gs.w));
                }
            }
            // texture_grad_uv (fp32)
            if (id != 0) {
                const float tx = u.x * (float)tw - 0.5f, ty = u.y * (float)th - 0.5f;
                const int32_t bx = f2i_sat(floorf(tx)), by = f2i_sat(floorf(ty));
                const float fx = tx - floorf(tx), fy = ty - floorf(ty);
                const int32_t x0 = address_coordinate(bx, tw, mode), x1 = address_coordinate(add1(bx), tw, mode);
                const int32_t y0 = address_coordinate(by, th, mode), y1 = address_coordinate(add1(by), th, mode);
                const float4 c00 = __ldg(tex + (size_t)(uint32_t)y0 * tw + (uint32_t)x0);
                const float4 c10 = __ldg(tex + (size_t)(uint32_t)y0 * tw + (uint32_t)x1);
                const float4 c01 = __ldg(tex + (size_t)(uint32_t)y1 * tw + (uint32_t)x0);
                const float4 c11 = __ldg(tex + (size_t)(uint32_t)y1 * tw + (uint32_t)x1);
                const float cs00[4] = {c00.x, c00.y, c00.z, c00.w}, cs10[4] = {c10.x, c10.y, c10.z, c10.w};
                const float cs01[4] = {c01.x, c01.y, c01.z, c01.w}, cs11[4] = {c11.x, c11.y, c11.z, c11.w};
                const float g4[4] = {gs.x, gs.y, gs.z, gs.w};
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const float dx = (1.0f - fy) * (cs10[c] - cs00[c]) + fy * (cs11[c] - cs01[c]);
                    const float dy = (1.0f - fx) * (cs01[c] - cs00[c]) + fx * (cs11[c] - cs10[c]);
                    gux += g4[c] * (dx * (float)tw);
                    guy += g4[c] * (dy * (float)th);
                }
            }
        }
        if (id != 0 && id <= T) {
            valid = true;
            vi = idx[id - 1];
            const float bu = r.x, bv = r.y;
            const uint32_t vs[3] = {vi.x, vi.y, vi.z};
            const bool inside = vi.x < V && vi.y < V && vi.z < V;
            float ga[kA > 0 ? kA : 1];
#pragma unroll
            for (int a = 0; a < kA; ++a) ga[a] = grad_attr_out[pix * kA + a];
            // interpolate_grad_attributes for uv and attributes: each distinct vertex once, with the
            // weight accumulated as interpolate_grad_attributes.hlsl:42-54 does
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t vx = vs[k];
                bool first = true;
#pragma unroll
                for (int j = 0; j < k; ++j) first = first && vs[j] != vx;
                if (!first || vx >= V) continue;
                float wgt = 0.0f;
                if (vi.x == vx) wgt += bu;
                if (vi.y == vx) wgt += bv;
                if (vi.z == vx) wgt += 1.0f - bu - bv;
                if (uv_attrs) {
                    cv[k][0] = wgt * gux;
                    cv[k][1] = wgt * guy;
                }
#pragma unroll
                for (int a = 0; a < kA; ++a) cv[k][2 + a] = wgt * ga[a];
            }
            // interpolate_grad_raster: uv attributes first, attributes accumulated on top
            float grx = 0.0f, gry = 0.0f;
            if (inside) {
                if (uv_attrs) {
                    const float2 t0 = __ldg(uv_attrs + vi.x), t1 = __ldg(uv_attrs + vi.y), t2 = __ldg(uv_attrs + vi.z);
                    grx += gux * (t0.x - t2.x);
                    gry += gux * (t1.x - t2.x);
                    grx += guy * (t0.y - t2.y);
                    gry += guy * (t1.y - t2.y);
                }
                if (kA > 0) {
                    float ax = 0.0f, ay = 0.0f;
#pragma unroll
                    for (int a = 0; a < kA; ++a) {
                        const float a0 = __ldg(attrs + (size_t)vi.x * kA + a), a1 = __ldg(attrs + (size_t)vi.y * kA + a);
                        const float a2 = __ldg(attrs + (size_t)vi.z * kA + a);
                        ax += ga[a] * (a0 - a2);
                        ay += ga[a] * (a1 - a2);
                    }
                    grx = grx + ax;
                    gry = gry + ay;
                }
            }
            // rasterize_backward for this pixel (same visit rule as the per-triangle loop)
            if (inside && !(grx == 0.0f && gry == 0.0f)) {
                const float4* __restrict__ clip = clip_all + (size_t)view * V;
                const float4 p0 = clip[vi.x], p1 = clip[vi.y], p2 = clip[vi.z];
                const float4 vp = viewports[view];
                bool visit = !(p0.w <= 1e-8f || p1.w <= 1e-8f || p2.w <= 1e-8f);
                if (visit) {
                    const float s0x = p0.x / p0.w, s0y = p0.y / p0.w;
                    const float s1x = p1.x / p1.w, s1y = p1.y / p1.w;
                    const float s2x = p2.x / p2.w, s2y = p2.y / p2.w;
                    const float mnx = fminf(s0x, fminf(s1x, s2x)), mny = fminf(s0y, fminf(s1y, s2y));
                    const float mxx = fmaxf(s0x, fmaxf(s1x, s2x)), mxy = fmaxf(s0y, fmaxf(s1y, s2y));
                    const int32_t x0 = clampi(f2i_sat(floorf((mnx * 0.5f + 0.5f) * vp.z + vp.x)), 0, (int32_t)W);
                    const int32_t x1 = clampi(f2i_sat(ceilf((mxx * 0.5f + 0.5f) * vp.z + vp.x)), 0, (int32_t)W);
                    const int32_t y0 = clampi(f2i_sat(floorf((mny * 0.5f + 0.5f) * vp.w + vp.y)), 0, (int32_t)H);
                    const int32_t y1 = clampi(f2i_sat(ceilf((mxy * 0.5f + 0.5f) * vp.w + vp.y)), 0, (int32_t)H);
                    visit = (int32_t)px >= x0 && (int32_t)px < x1 && (int32_t)py >= y0 && (int32_t)py < y1;
                }
                if (visit) {
                    const float sx = sample_ndc(px, vp.x, vp.z);
                    const float sy = sample_ndc(py, vp.y, vp.w);
                    const float q0x = p0.x - sx * p0.w, q0y = p0.y - sy * p0.w;
                    const float q1x = p1.x - sx * p1.w, q1y = p1.y - sy * p1.w;
                    const float q2x = p2.x - sx * p2.w, q2y = p2.y - sy * p2.w;
                    const float area = cross2(q1x, q1y, q2x, q2y) + cross2(q2x, q2y, q0x, q0y) + cross2(q0x, q0y, q1x, q1y);
                    if (!(fabsf(area) <= 1e-12f)) {
                        const float eps = area >= 0.0f ? 1e-6f : -1e-6f;
                        const float inv = 1.0f / (area + eps);
                        const float a0 = cross2(q1x, q1y, q2x, q2y);
                        const float a1 = cross2(q2x, q2y, q0x, q0y);
                        const float b0 = a0 * inv, b1 = a1 * inv;
                        const float gb0 = grx * inv, gb1 = gry * inv;
                        const float gc = gb0 * b0 + gb1 * b1;
                        const float g0x = gc * (q2y - q1y) - gb1 * q2y;
                        const float g1x = gc * (q0y - q2y) + gb0 * q2y;
                        const float g2x = gc * (q1y - q0y) - gb0 * q1y + gb1 * q0y;
                        const float g0y = gc * (q1x - q2x) + gb1 * q2x;
                        const float g1y = gc * (q2x - q0x) - gb0 * q2x;
                        const float g2y = gc * (q0x - q1x) + gb0 * q1x - gb1 * q0x;
                        cv[0][2 + kA] = g0x; cv[0][3 + kA] = g0y; cv[0][4 + kA] = -sx * g0x - sy * g0y;
                        cv[1][2 + kA] = g1x; cv[1][3 + kA] = g1y; cv[1][4 + kA] = -sx * g1x - sy * g1y;
                        cv[2][2 + kA] = g2x; cv[2][3 + kA] = g2y; cv[2][4 + kA] = -sx * g2x - sy * g2y;
                    }
                }
            }
        }
    }
    // Runs of pixels on the same triangle are contiguous along the tile row a warp covers: sum each
    // run in registers, then only the run's last lane touches the shared table.
    const uint32_t key = valid ? id : (0x80000000u | lane);
    const RunScan scan(key);
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (uint32_t j = 0; j < kNV; ++j) cv[k][j] = scan.sum(cv[k][j]);
    if (valid && scan.tail) {
        const uint32_t corners[3] = {vi.x, vi.y, vi.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint32_t v = corners[k];
            if (v >= V) continue;
            const uint32_t slot = table_slot(tb, v);
            if (slot < kSlots) {
                float* dst = tb.val + (size_t)slot * kNV;
#pragma unroll
                for (uint32_t j = 0; j < kNV; ++j)
                    if (cv[k][j] != 0.0f) atomicAdd(dst + j, cv[k][j]);
            } else {  // table full: straight to global memory
                if (g_uv) {
                    atomicAdd(g_uv + (size_t)v * 2, cv[k][0]);
                    atomicAdd(g_uv + (size_t)v * 2 + 1, cv[k][1]);
                }
#pragma unroll
                for (int a = 0; a < kA; ++a) atomicAdd(g_attr + (size_t)v * kA + a, cv[k][2 + a]);
                atomicAdd(g_clip + (size_t)v * 4 + 0, cv[k][2 + kA]);
                atomicAdd(g_clip + (size_t)v * 4 + 1, cv[k][3 + kA]);
                atomicAdd(g_clip + (size_t)v * 4 + 3, cv[k][4 + kA]);
            }
        }
    }
    __syncthreads();
    // flush: one atomic per non-zero (vertex, component)
    for (uint32_t sl = threadIdx.x; sl < kSlots; sl += kFusedThreads) {
        const uint32_t v = tb.key[sl];
        if (v == kEmpty) continue;
        const float* src = tb.val + (size_t)sl * kNV;
        if (g_uv) {
            if (src[0] != 0.0f) atomicAdd(g_uv + (size_t)v * 2, src[0]);
            if (src[1] != 0.0f) atomicAdd(g_uv + (size_t)v * 2 + 1, src[1]);
        }
#pragma unroll
        for (int a = 0; a < kA; ++a)
            if (src[2 + a] != 0.0f) atomicAdd(g_attr + (size_t)v * kA + a, src[2 + a]);
        const float* pc = src + 2 + kA;
        if (pc[0] != 0.0f) atomicAdd(g_clip + (size_t)v * 4 + 0, pc[0]);
        if (pc[1] != 0.0f) atomicAdd(g_clip + (size_t)v * 4 + 1, pc[1]);
        if (pc[2] != 0.0f) atomicAdd(g_clip + (size_t)v * 4 + 3, pc[2]);
    }
}

}  // namespace

}  // namespace pdr

using namespace pdr;

extern "C" {

size_t pdr_render_workspace_bytes(uint32_t views, uint32_t triangle_count, uint32_t width, uint32_t height,
                                  uint64_t capacity) {
    return bins_workspace_bytes(views, triangle_count, width, height, capacity);
}

pdr_status pdr_render_forward(const pdr_render_args* a, void* stream) {
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
    if (a->workspace_bytes < bins_workspace_bytes(a->views, a->triangle_count, a->width, a->height, a->capacity))
        return set_error(PDR_INVALID_ARGUMENT, "workspace is smaller than pdr_render_workspace_bytes()");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = launch_bin_tiles(a->clip_positions, a->views, a->vertex_count, a->indices, a->triangle_count,
                                       a->width, a->height, a->viewports, a->tile_offsets, a->tile_triangles,
                                       a->capacity, a->workspace, a->status, s, /*sorted=*/false);
    if (err != cudaSuccess) return set_cuda_error(err, "render_forward(bins)");
    RasterShade shade{a->attributes, a->attribute_count, a->interpolated, a->uv_attributes, a->uv, a->texture,
                      a->texture_width, a->texture_height, a->address_mode, a->sampled};
    err = launch_raster_forward(a->clip_positions, a->views, a->vertex_count, a->indices, a->triangle_count, a->width,
                                a->height, a->viewports, a->cull_mode, a->tile_offsets, a->tile_triangles, a->capacity,
                                a->raster, a->barycentric_derivatives, s,
                                (a->attributes || a->uv_attributes) ? &shade : nullptr);
    return set_cuda_error(err, "render_forward");
}

pdr_status pdr_render_backward(const pdr_render_args* a, void* stream) {
    if (!a || !a->clip_positions || !a->indices || !a->viewports || !a->raster || !a->grad_clip_positions || !a->status)
        return set_error(PDR_INVALID_ARGUMENT, "render arguments are incomplete");
    if (a->attributes && (!a->grad_interpolated || !a->grad_attributes || a->attribute_count == 0 ||
                          a->attribute_count > 8))
        return set_error(PDR_INVALID_ARGUMENT, "attribute gradients need grad_interpolated and grad_attributes");
    if (a->texture && (!a->uv || !a->grad_sampled || !a->grad_texture || !a->grad_uv_attributes || !a->uv_attributes))
        return set_error(PDR_INVALID_ARGUMENT, "texture gradients need uv, grad_sampled and gradient outputs");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t err = cudaMemsetAsync(a->grad_clip_positions, 0, (size_t)a->views * a->vertex_count * 4 * sizeof(float), s);
    if (err == cudaSuccess && a->grad_attributes)
        err = cudaMemsetAsync(a->grad_attributes, 0, (size_t)a->vertex_count * a->attribute_count * sizeof(float), s);
    if (err == cudaSuccess && a->grad_uv_attributes)
        err = cudaMemsetAsync(a->grad_uv_attributes, 0, (size_t)a->vertex_count * 2 * sizeof(float), s);
    if (err == cudaSuccess && a->grad_texture)
        err = cudaMemsetAsync(a->grad_texture, 0, (size_t)a->texture_width * a->texture_height * 4 * sizeof(float), s);
    if (err != cudaSuccess) return set_cuda_error(err, "render_backward(memset)");
    const uint32_t tcx = (a->width + kTile - 1) / kTile, tcy = (a->height + kTile - 1) / kTile;
    const dim3 grid(tcx * tcy, a->views);
    const uint32_t A = a->attributes ? a->attribute_count : 0;
#define PDR_RENDER_BWD(KA)                                                                                          \
    render_backward_kernel<KA><<<grid, kFusedThreads, 0, s>>>(                                                      \
        reinterpret_cast<const float4*>(a->clip_positions), a->vertex_count, reinterpret_cast<const uint3*>(a->indices), \
        a->triangle_count, a->width, a->height, reinterpret_cast<const float4*>(a->viewports), tcx, a->attributes,   \
        reinterpret_cast<const float2*>(a->uv_attributes), reinterpret_cast<const float4*>(a->texture),            \
        a->texture_width, a->texture_height, a->address_mode, reinterpret_cast<const float4*>(a->raster),           \
        reinterpret_cast<const float2*>(a->uv), a->grad_interpolated, reinterpret_cast<const float4*>(a->grad_sampled), \
        a->grad_clip_positions, a->grad_attributes, a->grad_uv_attributes, a->grad_texture, a->status)
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
    return set_cuda_error(cudaGetLastError(), "render_backward");
}

}  // extern "C"

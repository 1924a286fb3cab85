// The fused adjoint of rasterize -> interpolate(attributes), interpolate(uv) -> texture for the
// pixels of one 16 x kTH tile of one view; shared by the per-mesh launch (fused.cu, 16x8 tiles) and the
// uneven multi-mesh batch (batch.cu, 16x16). The kernel that calls render_backward_tile runs 16 * kTH
// threads, each warp on two tile rows.
//
// One thread per pixel runs, in the reference's order and arithmetic, texture_grad_texture
// (double-exact weights, vector atomics, warp-aggregated for magnified textures), texture_grad_uv,
// interpolate_grad_attributes / interpolate_grad_raster for both attribute sets, and
// rasterize_backward for the summed raster gradient. Per-vertex gradients are summed over each run of adjacent pixels of a warp that hit the
// same triangle (warp shuffles); the run's last lane then adds them to global memory with vector
// reductions (clip x/y/0/w as one v4, uv as one v2). A per-tile shared-memory table that merged the
// runs' vertices before one flush was measured slower: its hash probes and shared float atomics cost
// more than the extra global reductions they saved (5.24 vs 4.00 ms for 64 views at 1024x1024).
// Intermediate grad_uv / grad_raster never leave registers.
#pragma once

#include <cuda_runtime.h>

#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {

constexpr int kFusedThreads = 256;
constexpr uint32_t kMaxVals = 2 + 8 + 3; // uv attributes, up to 8 attributes, clip x/y/w

__device__ __forceinline__ void red_v4(float* addr, float4 v) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

__device__ __forceinline__ void red_v2(float* addr, float x, float y) {
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(addr), "f"(x), "f"(y) : "memory");
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

// One view of one mesh as the adjoint sees it (pixel images are this view's; the attribute, uv and
// texture gradients are shared by all views of the mesh).
struct BackwardView {
    const float4* clip;           // [V] clip positions of this view
    uint32_t V;
    const uint3* idx;             // [T]
    uint32_t T, W, H;
    float4 vp;
    const float* attrs;           // [V][A], or nullptr
    const float2* uv_attrs;       // [V][2], or nullptr
    const float4* tex;            // [th][tw][4], or nullptr
    uint32_t tw, th, mode;
    const float4* raster;         // [H][W]
    const float2* uv;             // [H][W], or nullptr
    const float* grad_attr_out;   // [H][W][A]
    const float4* grad_sampled;   // [H][W]
    float* g_clip;                // [V][4] of this view
    float* g_attr;                // [V][A]
    float* g_uv;                  // [V][2]
    float* g_tex;                 // [th][tw][4]
    const float4* sdiff;          // [H][W][2] texel differences of the forward's sample, or nullptr
    uint32_t* status;
    // When set: this view's vertex-gradient records [V][vertex_record_floats(kA)] (uv, attributes,
    // clip x/y/w, zero padding), added with 16-byte reductions and summed over the views afterwards
    // (vertex_grad_finish_kernel); g_clip, g_attr and g_uv are then not touched here.
    float* g_vtx;
};

// Floats per vertex-gradient record: uv 2 + attributes kA + clip x/y/w 3, rounded up to 16 bytes.
__host__ __device__ constexpr uint32_t vertex_record_floats(int kA) { return (uint32_t)((5 + kA + 3) / 4 * 4); }

// kTexAgg: texture-gradient taps warp-aggregated (1), plain (0), or decided from the texture and image
// sizes (-1: aggregated when the texture has fewer texels than the view has pixels).
template <int kA, int kTexAgg = -1, int kTH = kTile>
__device__ __forceinline__ void render_backward_tile(const BackwardView& v, uint32_t tile_x, uint32_t tile_y) {
    const float4* __restrict__ clip_view = v.clip;
    const uint32_t V = v.V, T = v.T, W = v.W, H = v.H;
    const uint3* __restrict__ idx = v.idx;
    const float* __restrict__ attrs = v.attrs;
    const float2* __restrict__ uv_attrs = v.uv_attrs;
    const float4* __restrict__ tex = v.tex;
    const uint32_t tw = v.tw, th = v.th, mode = v.mode;
    const float4* __restrict__ raster = v.raster;
    const float2* __restrict__ uv = v.uv;
    const float* __restrict__ grad_attr_out = v.grad_attr_out;
    const float4* __restrict__ grad_sampled = v.grad_sampled;
    float* __restrict__ g_clip_view = v.g_clip;
    float* __restrict__ g_attr = v.g_attr;
    float* __restrict__ g_uv = v.g_uv;
    float* __restrict__ g_tex = v.g_tex;
    uint32_t* __restrict__ status = v.status;

    constexpr uint32_t kNV = 2 + kA + 3;  // per vertex: uv attributes, attributes, clip x/y/w
    const bool magnified = kTexAgg >= 0 ? kTexAgg == 1 : (uint64_t)tw * th < (uint64_t)W * H;
    float* g_clip = g_clip_view;
    const uint32_t lane = threadIdx.x & 31u;

    const uint32_t px = tile_x * kTile + (threadIdx.x & 15u);
    const uint32_t py = tile_y * (uint32_t)kTH + (threadIdx.x >> 4);
    bool valid = false;           // pixel contributes vertex gradients (id in [1, T])
    uint3 vi = make_uint3(0, 0, 0);
    float cv[3][kNV];             // per corner contributions
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (uint32_t j = 0; j < kNV; ++j) cv[k][j] = 0.0f;
    uint32_t id = 0;

    if (px < W && py < H) {
        const size_t pix = (size_t)py * W + px;
        // per-pixel inputs are read exactly once: loaded with the streaming (evict-first) hint so that L2
        // keeps the texture and the gradient texels the scatter below adds into (-0.24 ms on 64 views)
        const float4 r = __ldcs(raster + pix);
        id = raster_id(r.w);
        const float2 u = uv ? __ldcs(uv + pix) : make_float2(0.0f, 0.0f);
        float gux = 0.0f, guy = 0.0f;
        if (tex) {
            const float4 gs = __ldcs(grad_sampled + pix);
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
                    red_add_v4_texel(g_tex + ((size_t)(uint32_t)ys0 * tw + (uint32_t)xs0) * 4, make_float4(w0 * gs.x, w0 * gs.y, w0 * gs.z, w0 * gs.w), magnified);
                    red_add_v4_texel(g_tex + ((size_t)(uint32_t)ys0 * tw + (uint32_t)xs1) * 4, make_float4(w1 * gs.x, w1 * gs.y, w1 * gs.z, w1 * gs.w), magnified);
                    red_add_v4_texel(g_tex + ((size_t)(uint32_t)ys1 * tw + (uint32_t)xs0) * 4, make_float4(w2 * gs.x, w2 * gs.y, w2 * gs.z, w2 * gs.w), magnified);
                    red_add_v4_texel(g_tex + ((size_t)(uint32_t)ys1 * tw + (uint32_t)xs1) * 4, make_float4(w3 * gs.x, w3 * gs.y, w3 * gs.z, w3 * gs.w), magnified);
                }
            }
            // texture_grad_uv (fp32)
            if (id != 0) {
                float dxs[4], dys[4];
                if (v.sdiff) {
                    // the forward's texel differences: the same values the gathers below compute
                    const float4 du = __ldcs(v.sdiff + pix * 2), dv = __ldcs(v.sdiff + pix * 2 + 1);
                    dxs[0] = du.x; dxs[1] = du.y; dxs[2] = du.z; dxs[3] = du.w;
                    dys[0] = dv.x; dys[1] = dv.y; dys[2] = dv.z; dys[3] = dv.w;
                } else {
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
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        dxs[c] = (1.0f - fy) * (cs10[c] - cs00[c]) + fy * (cs11[c] - cs01[c]);
                        dys[c] = (1.0f - fx) * (cs01[c] - cs00[c]) + fx * (cs11[c] - cs10[c]);
                    }
                }
                const float g4[4] = {gs.x, gs.y, gs.z, gs.w};
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    gux += g4[c] * (dxs[c] * (float)tw);
                    guy += g4[c] * (dys[c] * (float)th);
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
            for (int a = 0; a < kA; ++a) ga[a] = __ldcs(grad_attr_out + pix * kA + a);
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
                const float4* __restrict__ clip = clip_view;
                const float4 p0 = clip[vi.x], p1 = clip[vi.y], p2 = clip[vi.z];
                const float4 vp = v.vp;
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
    // run in registers, then only the run's last lane adds to global memory.
    const uint32_t key = valid ? id : (0x80000000u | lane);
    const RunScan scan(key);
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (uint32_t j = 0; j < kNV; ++j) cv[k][j] = scan.sum(cv[k][j]);
    if (v.g_vtx) {
        // A warp covers two tile rows, so a triangle usually ends a run in each: the second run's sums move
        // to the first run's tail (one shuffle per value) and one tail adds them.
        const bool tail = valid && scan.tail;
        const unsigned same = __match_any_sync(0xffffffffu, tail ? id : (0x80000000u | lane));
        const bool pair = tail && __popc(same) == 2;
        const uint32_t partner = pair ? (uint32_t)(__ffs(same & ~(1u << lane)) - 1) : lane;
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (uint32_t j = 0; j < kNV; ++j) {
                const float o = __shfl_sync(0xffffffffu, cv[k][j], partner);
                if (pair && partner > lane) cv[k][j] += o;
            }
        if (pair && partner < lane) valid = false;  // its sums went to the first tail
    }
    if (valid && scan.tail && v.g_vtx) {
        // one record per vertex and view: kNV values in 16-byte reductions (two for up to three attributes,
        // against five reductions into the shared uv / attribute rows and the clip row otherwise)
        constexpr uint32_t kR = vertex_record_floats(kA);
        const uint32_t corners[3] = {vi.x, vi.y, vi.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (corners[k] >= V) continue;
            float* rec = v.g_vtx + (size_t)corners[k] * kR;
#pragma unroll
            for (uint32_t c = 0; c < kR; c += 4)
                red_v4(rec + c, make_float4(c < kNV ? cv[k][c] : 0.0f, c + 1 < kNV ? cv[k][c + 1] : 0.0f,
                                            c + 2 < kNV ? cv[k][c + 2] : 0.0f, c + 3 < kNV ? cv[k][c + 3] : 0.0f));
        }
    } else if (valid && scan.tail) {
        const uint32_t corners[3] = {vi.x, vi.y, vi.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint32_t v = corners[k];
            if (v >= V) continue;
            if (g_uv) red_v2(g_uv + (size_t)v * 2, cv[k][0], cv[k][1]);
            float* ga = g_attr + (size_t)v * kA;
            if (kA % 4 == 0) {  // rows of 4k floats: 16-byte aligned
#pragma unroll
                for (int a = 0; a < kA; a += 4)
                    red_v4(ga + a, make_float4(cv[k][2 + a], cv[k][3 + a], cv[k][4 + a], cv[k][5 + a]));
            } else if (kA % 2 == 0) {
#pragma unroll
                for (int a = 0; a < kA; a += 2) red_v2(ga + a, cv[k][2 + a], cv[k][3 + a]);
            } else {
#pragma unroll
                for (int a = 0; a < kA; ++a) atomicAdd(ga + a, cv[k][2 + a]);
            }
            // z of the clip gradient stays 0 (rasterize_backward.hlsl writes no depth gradient)
            red_v4(g_clip + (size_t)v * 4, make_float4(cv[k][2 + kA], cv[k][3 + kA], 0.0f, cv[k][4 + kA]));
        }
    }
}

}  // namespace pdr

// One raster tile (shaders/rasterize_forward.hlsl:45-175 for the pixels of a TW x TH tile) with the
// optional shading epilogue; shared by the per-mesh launch (raster.cu) and the uneven multi-mesh
// batch (batch.cu). The kernel that calls raster_tile must run TW * TH threads.
//
// Per tile: the tile's triangles are staged in shared memory (structure of arrays) CHUNK at a time,
// each with the rectangle of tile pixels whose samples can pass its edge tests (pixel_rect, a rigorous
// bound including the reference's 1e-7 tolerance and fp32 rounding); on 16x8 tiles, rectangles of more
// than kSpanMin pixels are cut to per-row spans (span_coefficients, row_span, another rigorous bound).
// The candidates, the (triangle, pixel) pairs of those rectangles or spans, are then spread over the
// lanes one pair per lane: each warp owns a
// share of the staged triangles, numbers their candidates with a prefix sum and works through them 32 at
// a time. A lane runs the reference's edge tests at its candidate's sample and, when they pass, computes
// the depth with the reference's arithmetic and folds (depth, triangle) into the pixel's winner key with
// a shared-memory atomicMin. Small triangles have a handful of candidates, so lanes stay busy where a
// warp-per-region coverage pass would test 32 pixels to find a few. Afterwards each pixel recomputes the
// winner's barycentrics once. The result does not depend on the order of the tile's triangles: the
// minimum (depth, id) key is what the reference's sequential depth test keeps. Which triangles a tile
// lists follows the reference's 16x16 binning for every tile shape (bin_rect.cuh triangle_tile_rect), so
// the (triangle, pixel) pairs tested are the reference's.
#pragma once

#include <cuda_runtime.h>

#include "bin_rect.cuh"
#include "pdr_common.cuh"

namespace pdr {

// Shading epilogue of one view: output pointers are the view's own images ([H][W][...]).
struct ShadeArgs {
    const float* attrs;     // [V][A], or nullptr
    uint32_t A;
    float* attr_out;        // [H][W][A]
    const float2* uv_attrs; // [V][2], or nullptr
    float2* uv_out;         // [H][W][2]
    const float4* tex;      // [th][tw][4], or nullptr
    uint32_t tw, th, mode;
    float4* sampled;        // [H][W][4]
    float4* sdiff;          // [H][W][2]: texel differences along u and v per channel, or nullptr
};

// One view of one mesh as the tile routine sees it.
struct RasterView {
    const float4* clip;  // [V] clip positions of this view
    const uint3* idx;    // [T]
    uint32_t V, T, W, H, cull;
    float4 vp;
    float4* raster;      // [H][W]
    float4* deriv;       // [H][W], or nullptr
    ShadeArgs shade;
};

template <int CHUNK>
struct TileStage {
    float4 edge_a[CHUNK];  // screen positions s0x, s0y, s1x, s1y
    float4 edge_b[CHUNK];  // s2x, s2y, orientation sign, triangle index (bits)
    uint32_t rect[CHUNK];  // candidate rectangle (x0 | x1 << 8 | y0 << 16 | y1 << 24, tile-local), or below
    float4 p0[CHUNK], p1[CHUNK], p2[CHUNK];
};

constexpr uint32_t kRectNone = 0xFFFFFFFEu;   // no pixel of the tile can pass: nothing to do
constexpr uint32_t kRectLarge = 0xFFFFFFFFu;  // the bound does not apply: every pixel of the tile

// The pixels of tile [x_org, x_org + TW) x [y_org, y_org + TH) (clipped to the image) whose samples can pass
// all three of the reference's edge tests fl(e) * sign >= -1e-7, as a rectangle, or kRectLarge when the
// bound below does not apply, or kRectNone when it is empty.
// Bound: let L bound |a - s| over vertices a and the tile's samples s. The fp32 edge value differs from the
// exact one by at most 4u(|AB| + |CD|) <= 8u L^2 (u = 2^-24), so a sample passing the fp32 test satisfies
// the exact test e * sign >= -tau, tau = 1e-7 + 2e-6 L^2; such samples lie in the triangle with every edge
// moved out by tau / |edge|, whose vertices move by at most tau (|e_a| + |e_b|) / |cross| <= tau P / |area|
// (P the perimeter, area = the cross product the reference computes). D = 2 tau P / |area| bounds that
// with room for the rounding of P and of area (at most 0.6% when |area| >= 1e-4 ext^2, required), so
// every passing sample lies in the vertex bounding box grown by D. Pixel indices come from inverting
// sample_ndc with 0.05 pixel (plus 1e-6 of the viewport size) of slack for its rounding.
// `err` receives 2e-6 L^2, the bound on |fl(e) - e| at any sample of the tile that the row spans use.
__device__ __forceinline__ uint32_t pixel_rect(float s0x, float s0y, float s1x, float s1y, float s2x, float s2y,
                                               float area, float4 vp, uint32_t x_org, uint32_t y_org, uint32_t x_end,
                                               uint32_t y_end, float tsx_lo, float tsx_hi, float tsy_lo,
                                               float tsy_hi, float& err) {
    const float mnx = fminf(s0x, fminf(s1x, s2x)), mxx = fmaxf(s0x, fmaxf(s1x, s2x));
    const float mny = fminf(s0y, fminf(s1y, s2y)), mxy = fmaxf(s0y, fmaxf(s1y, s2y));
    const float pxw = 2.0f / vp.z, pyw = 2.0f / vp.w;  // one pixel in NDC
    const float ext = fmaxf(mxx - mnx, mxy - mny);
    // |a - s| over vertices and tile samples (tile sample ranges [tsx_lo, tsx_hi] x [tsy_lo, tsy_hi]), 1% up
    const float L = 1.01f * fmaxf(fmaxf(fabsf(mxx - tsx_lo), fabsf(tsx_hi - mnx)),
                                  fmaxf(fabsf(mxy - tsy_lo), fabsf(tsy_hi - mny)));
    const float perim = fabsf(s1x - s0x) + fabsf(s1y - s0y) + fabsf(s2x - s1x) + fabsf(s2y - s1y) +
                        fabsf(s0x - s2x) + fabsf(s0y - s2y);
    err = 2e-6f * L * L;
    const float tau = 1e-7f + err;
    const float D = 2.0f * tau * perim / fabsf(area);
    // NaN-safe: every comparison with a NaN fails and sends the triangle to the warp path
    if (!(D <= fminf(pxw, pyw)) || !(fabsf(area) >= 1e-4f * ext * ext)) return kRectLarge;
    const float slx = 0.05f + 1e-6f * (vp.z + fabsf(vp.x)), sly = 0.05f + 1e-6f * (vp.w + fabsf(vp.y));
    // p = (s + 1) * size / 2 + origin - 0.5 inverts sample_ndc
    const float fx0 = ceilf(((mnx - D) + 1.0f) * 0.5f * vp.z + vp.x - 0.5f - slx);
    const float fx1 = floorf(((mxx + D) + 1.0f) * 0.5f * vp.z + vp.x - 0.5f + slx);
    const float fy0 = ceilf(((mny - D) + 1.0f) * 0.5f * vp.w + vp.y - 0.5f - sly);
    const float fy1 = floorf(((mxy + D) + 1.0f) * 0.5f * vp.w + vp.y - 0.5f + sly);
    const float cx0 = fmaxf(fx0, (float)x_org), cx1 = fminf(fx1, (float)(x_end - 1u));
    const float cy0 = fmaxf(fy0, (float)y_org), cy1 = fminf(fy1, (float)(y_end - 1u));
    if (!(cx0 <= cx1) || !(cy0 <= cy1)) return kRectNone;
    const uint32_t x0 = (uint32_t)cx0 - x_org, x1 = (uint32_t)cx1 - x_org;
    const uint32_t y0 = (uint32_t)cy0 - y_org, y1 = (uint32_t)cy1 - y_org;
    return x0 | (x1 << 8) | (y0 << 16) | (y1 << 24);
}

// Row spans of a candidate rectangle [x0, x1] x [y0, y1] (tile-local, at most 8 rows of at most 16
// columns): for each row, the columns whose samples can pass the three edge tests fl(e) * sign >= -1e-7.
// Bound: the exact edge value e(s) = cross(a - s, b - s) is affine in the sample s (the s x s terms
// cancel), so over the rectangle's samples it is the plane through its values at three corners of the
// sample box, s = (sx(t), sy(v)) with t, v in [0, 1] the sample's place between the box's first and last
// column and row. The fp32 values E00, E10, E01 at those corners (the reference's formula) each differ
// from the exact ones by at most `err` (pixel_rect's 2e-6 L^2 >= 8u L^2), so the exact value at any
// sample of the box is at most the plane through the fp32 corner values plus 3 err
// (|1 - t - v| + t + v <= 3), and a sample passing the fp32 test has exact e * sign >= -1e-7 - err.
// Every passing sample therefore satisfies alpha + beta t + gamma v >= 0 with alpha =
// sign E00 + 1e-7 + 4 err, beta = sign (E10 - E00), gamma = sign (E01 - E00); alpha also carries
// 4e-6 (|E00| + |E10| + |E01|) for the rounding of this arithmetic. Per row this bounds t from one side
// per edge; t maps to columns (nearly uniform sample spacing) with pixel_rect's 0.05 + 1e-6 viewport
// slack. NaN or infinite terms leave the row unconstrained.
// span_coefficients computes, once per (tile, triangle), A = (alpha per edge, -1 / beta of edge 0),
// G = (gamma per edge, -1 / beta of edge 1) and -1 / beta of edge 2 (0 where beta is 0).
__device__ __forceinline__ void span_coefficients(float4 ea, float4 eb, float err, uint32_t x0, uint32_t x1, uint32_t y0,
                                                  uint32_t y1, const float* tile_sx, const float* tile_sy, float4& A,
                                                  float4& G, float& nb2) {
    const float sgn = eb.z;
    const float sxa = tile_sx[x0], sxb = tile_sx[x1], sya = tile_sy[y0], syc = tile_sy[y1];
    const float vx[3] = {ea.x, ea.z, eb.x}, vy[3] = {ea.y, ea.w, eb.y};
    const uint32_t nx = x1 - x0;
    float al[3], ga[3], nb[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int ia = e == 0 ? 1 : (e == 1 ? 2 : 0), ib = e == 0 ? 2 : (e == 1 ? 0 : 1);
        const float ax = vx[ia], ay = vy[ia], bx = vx[ib], by = vy[ib];
        const float e00 = cross2(ax - sxa, ay - sya, bx - sxa, by - sya);
        const float e10 = cross2(ax - sxb, ay - sya, bx - sxb, by - sya);
        const float e01 = cross2(ax - sxa, ay - syc, bx - sxa, by - syc);
        const float mag = fabsf(e00) + fabsf(e10) + fabsf(e01);
        const float beta = nx ? sgn * (e10 - e00) : 0.0f;
        ga[e] = y1 > y0 ? sgn * (e01 - e00) : 0.0f;
        al[e] = sgn * e00 + ((1e-7f + 4.0f * err) + 4e-6f * mag);
        nb[e] = beta != 0.0f ? -1.0f / beta : 0.0f;
    }
    A = make_float4(al[0], al[1], al[2], nb[0]);
    G = make_float4(ga[0], ga[1], ga[2], nb[1]);
    nb2 = nb[2];
}

// The span of row y0 + i of rectangle [x0, x1] x [y0, y1]: (first column) | (width << 8), width 0 when no
// column of the row can pass.
__device__ __forceinline__ uint32_t row_span(float4 A, float4 G, float nb2, uint32_t x0, uint32_t x1, uint32_t y0,
                                             uint32_t y1, uint32_t i, const float* tile_sy, float slx) {
    const float sya = tile_sy[y0];
    const float inv_dy = y1 > y0 ? 1.0f / (tile_sy[y1] - sya) : 0.0f;
    const float v = (tile_sy[y0 + i] - sya) * inv_dy;
    const float fnx = (float)(x1 - x0);
    const float al[3] = {A.x, A.y, A.z}, ga[3] = {G.x, G.y, G.z}, nb[3] = {A.w, G.w, nb2};
    float lo = 0.0f, hi = 1.0f;
    bool empty = false;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const float a = al[e] + ga[e] * v;
        if (nb[e] < 0.0f) lo = fmaxf(lo, a * nb[e]);       // beta > 0: t >= -a / beta
        else if (nb[e] > 0.0f) hi = fminf(hi, a * nb[e]);  // beta < 0: t <= -a / beta
        else if (a < 0.0f) empty = true;                   // beta = 0: the whole row or none of it
    }
    if (empty || !(lo <= hi)) return 0u;
    const float cl = fmaxf(ceilf(lo * fnx - slx), 0.0f), ch = fminf(floorf(hi * fnx + slx), fnx);
    if (!(cl <= ch)) return 0u;
    const uint32_t c0 = (uint32_t)cl;
    return (x0 + c0) | (((uint32_t)ch - c0 + 1u) << 8);
}

// Four nibbles from the low nibbles of four bytes (byte j -> bits 4j .. 4j + 3).
__device__ __forceinline__ uint32_t pack_nibbles(uint32_t v) {
    v = (v | (v >> 4)) & 0x00FF00FFu;
    return (v | (v >> 8)) & 0xFFFFu;
}

// The winner's outputs at sample (sx, sy), rasterize_forward.hlsl's arithmetic: clamped barycentrics,
// 1 / area and clamped depth; and its pixel derivatives [du/dx, du/dy, dv/dx, dv/dy]. Shared with the
// near-plane remap, which evaluates them for the original triangle of a clipped one.
struct WinnerBary {
    float b0, b1, binv, depth;
};

__device__ __forceinline__ WinnerBary winner_barycentrics(float4 p0, float4 p1, float4 p2, float sx, float sy) {
    const float q0x = p0.x - sx * p0.w, q0y = p0.y - sy * p0.w;
    const float q1x = p1.x - sx * p1.w, q1y = p1.y - sy * p1.w;
    const float q2x = p2.x - sx * p2.w, q2y = p2.y - sy * p2.w;
    const float a0 = cross2(q1x, q1y, q2x, q2y);
    const float a1 = cross2(q2x, q2y, q0x, q0y);
    const float a2 = cross2(q0x, q0y, q1x, q1y);
    const float ha = a0 + a1 + a2;
    WinnerBary r;
    r.binv = 1.0f / ha;
    const float iz = p0.z * a0 + p1.z * a1 + p2.z * a2;
    const float iw = p0.w * a0 + p1.w * a1 + p2.w * a2;
    r.depth = clamp_hlsl(iz / iw, -1.0f, 1.0f);
    r.b0 = clamp_hlsl(a0 * r.binv, 0.0f, 1.0f);
    r.b1 = clamp_hlsl(a1 * r.binv, 0.0f, 1.0f);
    return r;
}

__device__ __forceinline__ float4 winner_derivatives(float4 p0, float4 p1, float4 p2, const WinnerBary& w, float4 vp) {
    const float da0_dx = -p1.w * p2.y + p2.w * p1.y;
    const float da0_dy = -p1.x * p2.w + p1.w * p2.x;
    const float da1_dx = -p2.w * p0.y + p2.y * p0.w;
    const float da1_dy = -p2.x * p0.w + p2.w * p0.x;
    const float da2_dx = -p0.w * p1.y + p0.y * p1.w;
    const float da2_dy = -p0.x * p1.w + p0.w * p1.x;
    const float dadx = da0_dx + da1_dx + da2_dx;
    const float dady = da0_dy + da1_dy + da2_dy;
    return make_float4((da0_dx - w.b0 * dadx) * w.binv * 2.0f / vp.z, (da0_dy - w.b0 * dady) * w.binv * 2.0f / vp.w,
                       (da1_dx - w.b1 * dadx) * w.binv * 2.0f / vp.z, (da1_dy - w.b1 * dady) * w.binv * 2.0f / vp.w);
}

// Orders (depth, triangle) pairs as the reference's depth test does: nearest depth first (-0 and
// +0 equal), then the lowest triangle index.
__device__ __forceinline__ unsigned long long depth_key(float depth, uint32_t t) {
    uint32_t b = __float_as_uint(depth);
    if ((b << 1) == 0u) b = 0u;
    const uint32_t o = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    return ((unsigned long long)o << 32) | t;
}

// The outputs of pixel (px, py) of a view whose winner is triangle best_tri - 1 (0: no triangle): the
// winner's barycentrics and depth recomputed with the reference's arithmetic (rasterize_forward.hlsl),
// its pixel derivatives, and the shading (interpolate_forward.hlsl, texture_forward.hlsl): the tile
// routine's epilogue.
template <bool kDeriv, bool kShade>
__device__ __forceinline__ void shade_pixel(const RasterView& v, uint32_t px, uint32_t py, size_t pix,
                                            uint32_t best_tri) {
    const ShadeArgs& shade = v.shade;
    if (best_tri == 0u) {
        v.raster[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (kDeriv) v.deriv[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (kShade) {
            if (shade.attr_out)
                for (uint32_t a = 0; a < shade.A; ++a) shade.attr_out[pix * shade.A + a] = 0.0f;
            if (shade.uv_out) shade.uv_out[pix] = make_float2(0.0f, 0.0f);
            if (shade.sampled) shade.sampled[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        return;
    }
    const float4 vp = v.vp;
    const float sx = sample_ndc(px, vp.x, vp.z);
    const float sy = sample_ndc(py, vp.y, vp.w);
    const uint3 vi = v.idx[best_tri - 1];
    const float4 p0 = v.clip[vi.x], p1 = v.clip[vi.y], p2 = v.clip[vi.z];
    const WinnerBary wb = winner_barycentrics(p0, p1, p2, sx, sy);
    const float bb0 = wb.b0, bb1 = wb.b1;
    v.raster[pix] = make_float4(bb0, bb1, wb.depth, (float)best_tri);
    if (kDeriv) v.deriv[pix] = winner_derivatives(p0, p1, p2, wb, vp);
    if (kShade) {
        // interpolate_forward.hlsl for the winner (id <= T and indices < V hold here), then
        // texture_forward.hlsl at the interpolated uv: the same arithmetic as the separate kernels.
        const float u = bb0, vv = bb1, w = 1.0f - u - vv;
        if (shade.attr_out) {
            const float* at = shade.attrs;
            const uint32_t A = shade.A;
            for (uint32_t a = 0; a < A; ++a)
                shade.attr_out[pix * A + a] = u * __ldg(at + (size_t)vi.x * A + a) + vv * __ldg(at + (size_t)vi.y * A + a) +
                                              w * __ldg(at + (size_t)vi.z * A + a);
        }
        if (shade.uv_out) {
            const float2 t0 = __ldg(shade.uv_attrs + vi.x), t1 = __ldg(shade.uv_attrs + vi.y), t2 = __ldg(shade.uv_attrs + vi.z);
            const float2 uvp = make_float2(u * t0.x + vv * t1.x + w * t2.x, u * t0.y + vv * t1.y + w * t2.y);
            shade.uv_out[pix] = uvp;
            if (shade.sampled) {
                const float tx_ = uvp.x * (float)shade.tw - 0.5f, ty_ = uvp.y * (float)shade.th - 0.5f;
                const int32_t bx = f2i_sat(floorf(tx_)), by = f2i_sat(floorf(ty_));
                const float fx = tx_ - floorf(tx_), fy = ty_ - floorf(ty_);
                const int32_t x0 = address_coordinate(bx, shade.tw, shade.mode), x1 = address_coordinate(add1(bx), shade.tw, shade.mode);
                const int32_t y0 = address_coordinate(by, shade.th, shade.mode), y1 = address_coordinate(add1(by), shade.th, shade.mode);
                const float w0 = (1.0f - fx) * (1.0f - fy), w1 = fx * (1.0f - fy), w2 = (1.0f - fx) * fy, w3 = fx * fy;
                const float4 c0 = __ldg(shade.tex + (size_t)(uint32_t)y0 * shade.tw + (uint32_t)x0);
                const float4 c1 = __ldg(shade.tex + (size_t)(uint32_t)y0 * shade.tw + (uint32_t)x1);
                const float4 c2 = __ldg(shade.tex + (size_t)(uint32_t)y1 * shade.tw + (uint32_t)x0);
                const float4 c3 = __ldg(shade.tex + (size_t)(uint32_t)y1 * shade.tw + (uint32_t)x1);
                float4 r;
                r.x = c0.x * w0 + c1.x * w1 + c2.x * w2 + c3.x * w3;
                r.y = c0.y * w0 + c1.y * w1 + c2.y * w2 + c3.y * w3;
                r.z = c0.z * w0 + c1.z * w1 + c2.z * w2 + c3.z * w3;
                r.w = c0.w * w0 + c1.w * w1 + c2.w * w2 + c3.w * w3;
                shade.sampled[pix] = r;
                if (shade.sdiff) {
                    // texture_grad_uv.hlsl's texel differences (c0 = c00, c1 = c10, c2 = c01, c3 = c11),
                    // kept for the backward so it does not gather the texels again
                    float4 du, dv;
                    du.x = (1.0f - fy) * (c1.x - c0.x) + fy * (c3.x - c2.x);
                    du.y = (1.0f - fy) * (c1.y - c0.y) + fy * (c3.y - c2.y);
                    du.z = (1.0f - fy) * (c1.z - c0.z) + fy * (c3.z - c2.z);
                    du.w = (1.0f - fy) * (c1.w - c0.w) + fy * (c3.w - c2.w);
                    dv.x = (1.0f - fx) * (c2.x - c0.x) + fx * (c3.x - c1.x);
                    dv.y = (1.0f - fx) * (c2.y - c0.y) + fx * (c3.y - c1.y);
                    dv.z = (1.0f - fx) * (c2.z - c0.z) + fx * (c3.z - c1.z);
                    dv.w = (1.0f - fx) * (c2.w - c0.w) + fx * (c3.w - c1.w);
                    shade.sdiff[pix * 2] = du;
                    shade.sdiff[pix * 2 + 1] = dv;
                }
            }
        }
    }
}


// Rasterizes tile (tx, ty) of view `v` from the triangle ids list[b..e). With kAll the tile visits the
// triangles [b, e) themselves (list unused) and keeps those the binning would have listed for it (the
// tile rectangle of src/rasterizer.cpp:73-125, as bin_count_kernel computes it): the path for a tile
// whose list did not fit the tile-list capacity, with the same result.
template <bool kDeriv, bool kShade, int TW, int TH, int CHUNK, bool kAll = false>
__device__ __forceinline__ void raster_tile(const RasterView& v, uint32_t tx, uint32_t ty,
                                            const uint32_t* __restrict__ list, uint32_t b, uint32_t e) {
    constexpr int kThreads = TW * TH;
    constexpr int kWarps = kThreads / 32;
    static_assert(TW <= 64 && TH <= 64 && kThreads <= 512 && kThreads % 32 == 0,
                  "candidate rectangles pack tile-local coordinates; li * width < 2^16");
    static_assert(CHUNK % 32 == 0 && CHUNK <= kThreads, "a stage holds at most one triangle per thread");
    // tiles of at most 16 x 8 pixels enumerate per-row spans of their rectangles of more than kSpanMin pixels
    // (span_coefficients, row_span; 8 measured fastest), larger tiles the rectangles themselves
    constexpr bool kRowSpans = TW <= 16 && TH <= 8;
    constexpr uint32_t kSpanMin = 8;
    __shared__ TileStage<CHUNK> tri;
    // Winner per pixel (row-major in the tile) as a 64-bit key (ordered depth bits << 32 | triangle
    // index): the minimum key is the nearest depth, ties to the lowest id, exactly the reference's
    // sequential test.
    __shared__ unsigned long long best_key[kThreads];
    __shared__ float tile_sx[TW], tile_sy[TH];  // sample positions of the tile's columns and rows
    __shared__ uint4 owners[kWarps][32];  // per warp: the triangles with candidates, in lane order
    // row-span bound per staged triangle (span_coefficients) and the spans of its rectangle's rows
    __shared__ float4 span_a[kRowSpans ? CHUNK : 1], span_g[kRowSpans ? CHUNK : 1];
    __shared__ float span_n[kRowSpans ? CHUNK : 1];
    __shared__ __align__(16) uint16_t spans[kRowSpans ? CHUNK : 1][8];
    __shared__ uint8_t span_list[kRowSpans ? CHUNK : 1];  // stage slots whose rectangles take row spans
    __shared__ uint32_t span_count;

    const float4* __restrict__ clip = v.clip;
    const uint3* __restrict__ idx = v.idx;
    const float4 vp = v.vp;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t x_org = tx * TW, y_org = ty * TH;
    const uint32_t px = x_org + threadIdx.x % (uint32_t)TW, py = y_org + threadIdx.x / (uint32_t)TW;
    best_key[threadIdx.x] = ~0ull;
    const bool in_image = px < v.W && py < v.H;
    const uint32_t x_end = min(x_org + (uint32_t)TW, v.W), y_end = min(y_org + (uint32_t)TH, v.H);
    const float slx = 0.05f + 1e-6f * (vp.z + fabsf(vp.x));  // column slack of the row spans (pixel_rect's)
    if (threadIdx.x < (uint32_t)TW) tile_sx[threadIdx.x] = sample_ndc(x_org + threadIdx.x, vp.x, vp.z);
    if (threadIdx.x < (uint32_t)TH) tile_sy[threadIdx.x] = sample_ndc(y_org + threadIdx.x, vp.y, vp.w);
    if (kRowSpans && threadIdx.x == 0) span_count = 0;
    for (uint32_t chunk = b; chunk < e; chunk += CHUNK) {
        __syncthreads();
        const uint32_t i = chunk + threadIdx.x;
        if (threadIdx.x < (uint32_t)CHUNK && i < e) {
            const uint32_t t = kAll ? i : list[i];
            float sgn = 0.0f;
            uint32_t rect = kRectNone;
            float err = 0.0f;
            float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f), p1 = p0, p2 = p0;
            float s0x = 0.f, s0y = 0.f, s1x = 0.f, s1y = 0.f, s2x = 0.f, s2y = 0.f;
            const uint3 vi = idx[t];
            bool binned = vi.x < v.V && vi.y < v.V && vi.z < v.V;
            if (kAll && binned) {
                const TriRect tr = triangle_tile_rect(clip, vi, v.W, v.H, vp, TW, TH);
                binned = tr.x != kNoRect && tx >= (tr.x & 0xffffu) && tx <= (tr.x >> 16) && ty >= (tr.y & 0xffffu) &&
                         ty <= (tr.y >> 16);
            }
            if (binned) {
                p0 = clip[vi.x];
                p1 = clip[vi.y];
                p2 = clip[vi.z];
            }
            tri.p0[threadIdx.x] = p0; tri.p1[threadIdx.x] = p1; tri.p2[threadIdx.x] = p2;
            if (binned) {
                if (!(p0.w <= 1e-8f || p1.w <= 1e-8f || p2.w <= 1e-8f)) {
                    s0x = p0.x / p0.w; s0y = p0.y / p0.w;
                    s1x = p1.x / p1.w; s1y = p1.y / p1.w;
                    s2x = p2.x / p2.w; s2y = p2.y / p2.w;
                    const float area = cross2(s1x - s0x, s1y - s0y, s2x - s0x, s2y - s0y);
                    const bool skip = fabsf(area) <= 1e-12f || (v.cull == 1 && area <= 0.0f) ||
                                      (v.cull == 2 && area >= 0.0f);
                    if (!skip) {
                        sgn = area > 0.0f ? 1.0f : -1.0f;
                        rect = pixel_rect(s0x, s0y, s1x, s1y, s2x, s2y, area, vp, x_org, y_org, x_end, y_end,
                                          tile_sx[0], tile_sx[x_end - x_org - 1u], tile_sy[0],
                                          tile_sy[y_end - y_org - 1u], err);
                    }
                }
            }
            tri.edge_a[threadIdx.x] = make_float4(s0x, s0y, s1x, s1y);
            tri.edge_b[threadIdx.x] = make_float4(s2x, s2y, sgn, __uint_as_float(t));
            tri.rect[threadIdx.x] = rect;
            if constexpr (kRowSpans) {
                // rectangles of more than kSpanMin pixels (the whole tile where the bound declines) are cut to
                // row spans; smaller ones are enumerated whole
                uint32_t x0 = 0, x1 = x_end - x_org - 1u, y0 = 0, y1 = y_end - y_org - 1u;
                if (rect < kRectNone) {
                    x0 = rect & 0xFFu;
                    x1 = (rect >> 8) & 0xFFu;
                    y0 = (rect >> 16) & 0xFFu;
                    y1 = rect >> 24;
                }
                if (rect != kRectNone && (x1 - x0 + 1u) * (y1 - y0 + 1u) > kSpanMin) {
                    span_coefficients(make_float4(s0x, s0y, s1x, s1y), make_float4(s2x, s2y, sgn, 0.0f), err, x0, x1,
                                      y0, y1, tile_sx, tile_sy, span_a[threadIdx.x], span_g[threadIdx.x],
                                      span_n[threadIdx.x]);
                    span_list[atomicAdd(&span_count, 1u)] = (uint8_t)threadIdx.x;
                }
            }
        }
        __syncthreads();
        const uint32_t n = min(e - chunk, (uint32_t)CHUNK);
        if constexpr (kRowSpans) {
            // the rows of the listed rectangles, eight threads per triangle (thread j takes row j & 7)
            const uint32_t listed = span_count;
            for (uint32_t q = threadIdx.x >> 3; q < listed; q += (uint32_t)kThreads / 8u) {
                const uint32_t kk = span_list[q], i = threadIdx.x & 7u, rc = tri.rect[kk];
                uint32_t x0 = 0, x1 = x_end - x_org - 1u, y0 = 0, y1 = y_end - y_org - 1u;
                if (rc < kRectNone) {
                    x0 = rc & 0xFFu;
                    x1 = (rc >> 8) & 0xFFu;
                    y0 = (rc >> 16) & 0xFFu;
                    y1 = rc >> 24;
                }
                spans[kk][i] = (uint16_t)(i <= y1 - y0 ? row_span(span_a[kk], span_g[kk], span_n[kk], x0, x1, y0, y1, i,
                                                                  tile_sy, slx)
                                                       : 0u);
            }
            __syncthreads();
            if (threadIdx.x == 0) span_count = 0;  // read by every thread above; rewritten after the next barrier
        }
        // Candidate expansion: lane j of warp w owns staged triangle k = w + kWarps * j and its candidate
        // pixels, the tile pixels of its rectangle (the whole tile for kRectLarge). The warp numbers its
        // triangles' candidates with a prefix sum, lists the triangles that have any (in that order) in
        // a per-warp table, and works through the candidates 32 at a time, one per lane: a lane finds its
        // candidate's triangle from the triangles whose last candidate precedes it, runs the reference's
        // edge tests at the candidate's sample and, when they pass, folds (depth, triangle) into the
        // pixel's winner key. Lanes stay busy whatever the triangles' sizes.
        const uint32_t k_own = warp + (uint32_t)kWarps * lane;
        uint32_t cnt = 0;
        uint4 entry = make_uint4(0u, 0u, 0u, 0u);
        if (k_own < n) {
            const uint32_t rc = tri.rect[k_own];
            uint32_t x0 = 0, x1 = x_end - x_org - 1u, y0 = 0, y1 = y_end - y_org - 1u;
            if (rc < kRectNone) {
                x0 = rc & 0xFFu;
                x1 = (rc >> 8) & 0xFFu;
                y0 = (rc >> 16) & 0xFFu;
                y1 = rc >> 24;
            }
            if (rc != kRectNone) {
                if constexpr (kRowSpans) {
                    // (first candidate, slot, first row) | first candidate index of rows 0-3 (bytes) | of rows
                    // 4-7 | first column of each row (nibbles). Rows past the rectangle have width 0.
                    uint32_t w_lo, w_hi, c_lo, c_hi;
                    if ((x1 - x0 + 1u) * (y1 - y0 + 1u) > kSpanMin) {
                        const uint4 sp = *reinterpret_cast<const uint4*>(spans[k_own]);
                        w_lo = __byte_perm(sp.x, sp.y, 0x7531);
                        w_hi = __byte_perm(sp.z, sp.w, 0x7531);
                        c_lo = __byte_perm(sp.x, sp.y, 0x6420);
                        c_hi = __byte_perm(sp.z, sp.w, 0x6420);
                    } else {
                        // every row of the rectangle whole
                        const uint32_t rows = y1 - y0 + 1u;  // 1..8
                        const uint32_t w = (x1 - x0 + 1u) * 0x01010101u;
                        w_lo = rows >= 4u ? w : w & ((1u << (8u * rows)) - 1u);
                        w_hi = rows <= 4u ? 0u : (rows == 8u ? w : w & ((1u << (8u * (rows - 4u))) - 1u));
                        c_lo = c_hi = x0 * 0x01010101u;
                    }
                    // bytewise inclusive prefix sums (every partial sum <= 128: no carries between bytes)
                    const uint32_t inc_lo = w_lo * 0x01010101u, inc_hi = w_hi * 0x01010101u;
                    const uint32_t tot_lo = inc_lo >> 24;
                    cnt = tot_lo + (inc_hi >> 24);
                    entry = make_uint4((k_own << 16) | (y0 << 24), inc_lo - w_lo, inc_hi - w_hi + tot_lo * 0x01010101u,
                                       pack_nibbles(c_lo) | (pack_nibbles(c_hi) << 16));
                } else {
                    // (first candidate, rectangle origin x | y << 8 | width << 16, row divisor, slot); the row of
                    // candidate li is li * m >> 16 with m = ceil(2^16 / width), exact for li * width < 2^16
                    const uint32_t w = x1 - x0 + 1u;
                    cnt = w * (y1 - y0 + 1u);
                    entry = make_uint4(0u, x0 | (y0 << 8) | (w << 16), (65536u + w - 1u) / w, k_own);
                }
            }
        }
        uint32_t incl = cnt;  // inclusive prefix sum over the warp's lanes
#pragma unroll
        for (uint32_t d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        const unsigned nonzero = __ballot_sync(0xffffffffu, cnt > 0);
        if (cnt > 0) {
            entry.x |= incl - cnt;
            owners[warp][__popc(nonzero & ((1u << lane) - 1u))] = entry;
        }
        __syncwarp();
        uint32_t ended = 0;  // triangles (with candidates) whose last candidate precedes this batch
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t c = base + lane;
            const uint32_t last = incl - 1u;  // this lane's triangle's last candidate
            const uint32_t mark = (cnt > 0 && last >= base && last - base < 32u) ? 1u << (last - base) : 0u;
            const uint32_t ends = __reduce_or_sync(0xffffffffu, mark);
            const uint32_t r = ended + __popc(ends & ((1u << lane) - 1u));
            ended += __popc(ends);
            if (c >= total) continue;
            const uint4 ow = owners[warp][r];
            uint32_t lx, ly, k;
            if constexpr (kRowSpans) {
                const uint32_t li = c - (ow.x & 0xFFFFu);  // candidate index within the triangle's spans
                // its row: the last row whose first candidate index is <= li (empty rows share the next
                // row's index and are passed over)
                const uint32_t rep = li * 0x01010101u;
                const uint32_t i = ((__popc(__vcmpleu4(ow.y, rep)) + __popc(__vcmpleu4(ow.z, rep))) >> 3) - 1u;
                const uint32_t pre = ((i < 4u ? ow.y : ow.z) >> ((i & 3u) * 8u)) & 0xFFu;
                lx = ((ow.w >> (i * 4u)) & 0xFu) + (li - pre);
                ly = (ow.x >> 24) + i;
                k = (ow.x >> 16) & 0xFFu;
            } else {
                const uint32_t li = c - ow.x;  // candidate index within the rectangle
                const uint32_t w = ow.y >> 16, qy = (li * ow.z) >> 16;
                lx = (ow.y & 0xFFu) + (li - qy * w);
                ly = ((ow.y >> 8) & 0xFFu) + qy;
                k = ow.w;
            }
            const float psx = tile_sx[lx], psy = tile_sy[ly];
            // coverage: rasterize_forward.hlsl's edge tests at the candidate's sample
            const float4 ea = tri.edge_a[k], eb = tri.edge_b[k];
            const float s0x = ea.x, s0y = ea.y, s1x = ea.z, s1y = ea.w, s2x = eb.x, s2y = eb.y, sgn = eb.z;
            const float e0 = cross2(s1x - psx, s1y - psy, s2x - psx, s2y - psy);
            const float e1 = cross2(s2x - psx, s2y - psy, s0x - psx, s0y - psy);
            const float e2 = cross2(s0x - psx, s0y - psy, s1x - psx, s1y - psy);
            const float ceps = -1e-7f;
            if (e0 * sgn < ceps || e1 * sgn < ceps || e2 * sgn < ceps) continue;
            // depth with the reference's arithmetic at the pair's sample, folded into the winner key
            const float4 p0 = tri.p0[k], p1 = tri.p1[k], p2 = tri.p2[k];
            const float q0x = p0.x - psx * p0.w, q0y = p0.y - psy * p0.w;
            const float q1x = p1.x - psx * p1.w, q1y = p1.y - psy * p1.w;
            const float q2x = p2.x - psx * p2.w, q2y = p2.y - psy * p2.w;
            const float a0 = cross2(q1x, q1y, q2x, q2y);
            const float a1 = cross2(q2x, q2y, q0x, q0y);
            const float a2 = cross2(q0x, q0y, q1x, q1y);
            const float ha = a0 + a1 + a2;
            if (fabsf(ha) <= 1e-12f) continue;
            const float iz = p0.z * a0 + p1.z * a1 + p2.z * a2;
            const float iw = p0.w * a0 + p1.w * a1 + p2.w * a2;
            if (fabsf(iw) <= 1e-12f) continue;
            const unsigned long long key = depth_key(clamp_hlsl(iz / iw, -1.0f, 1.0f), __float_as_uint(eb.w));
            unsigned long long* slot = &best_key[ly * (uint32_t)TW + lx];
            if (key < *slot) atomicMin(slot, key);  // keys only decrease: a stale read only adds an atomic
        }
        __syncwarp();  // the owner table is rewritten by the next stage
    }
    // candidates of any warp may land on any pixel of the tile
    __syncthreads();
    if (!in_image) return;
    const size_t pix = (size_t)py * v.W + px;
    const unsigned long long key = best_key[threadIdx.x];
    shade_pixel<kDeriv, kShade>(v, px, py, pix, key == ~0ull ? 0u : (uint32_t)key + 1u);
}

}  // namespace pdr

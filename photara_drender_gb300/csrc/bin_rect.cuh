// Tile rectangle of one triangle (src/rasterizer.cpp:73-125): shared by the per-mesh binning
// (raster.cu) and the multi-mesh batch binning (batch.cu).
#pragma once

#include <cuda_runtime.h>
#include <float.h>

#include "pdr_common.cuh"

namespace pdr {

constexpr uint32_t kNoRect = 0xffffffffu;

struct TriRect {
    uint32_t x;  // tx0 | tx1 << 16, or kNoRect
    uint32_t y;  // ty0 | ty1 << 16
};

// src/rasterizer.cpp:73-125 for one triangle: pixel bounding box of the NDC bounds, clamped, in the
// reference's 16 x 16 tiles. Which tiles list a triangle decides which pixels it can cover (a sample that
// passes the edge tests inside their 1e-7 tolerance may lie outside the triangle's pixel box, and the
// reference tests it when its 16 x 16 tile lists the triangle), so smaller tiles (tile_w, tile_h dividing
// 16) list a triangle in every sub-tile of the 16 x 16 tiles the reference lists it in: the set of
// (triangle, pixel) pairs tested is the reference's for every tile shape.
__device__ __forceinline__ TriRect triangle_tile_rect(const float4* __restrict__ pos, const uint3 vi,
                                                      uint32_t W, uint32_t H, float4 vp, uint32_t tile_w = kTile,
                                                      uint32_t tile_h = kTile) {
    TriRect r{kNoRect, 0};
    float min_x = INFINITY, min_y = INFINITY, max_x = -INFINITY, max_y = -INFINITY;
    const uint32_t v[3] = {vi.x, vi.y, vi.z};
    float sx_[3], sy_[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float4 p = pos[v[c]];
        if (!(p.w > 1e-8f) || !isfinite(p.w)) return r;
        const float x = p.x / p.w;
        const float y = p.y / p.w;
        if (!isfinite(x) || !isfinite(y)) return r;
        sx_[c] = x;
        sy_[c] = y;
        min_x = x < min_x ? x : min_x;
        min_y = y < min_y ? y : min_y;
        max_x = max_x < x ? x : max_x;
        max_y = max_y < y ? y : max_y;
    }
    if (max_x < -1.0f || min_x > 1.0f || max_y < -1.0f || min_y > 1.0f) return r;
    const int64_t px0 = f2i_sat(floorf((min_x * 0.5f + 0.5f) * vp.z + vp.x));
    const int64_t px1 = (int64_t)f2i_sat(ceilf((max_x * 0.5f + 0.5f) * vp.z + vp.x)) - 1;
    const int64_t py0 = f2i_sat(floorf((min_y * 0.5f + 0.5f) * vp.w + vp.y));
    const int64_t py1 = (int64_t)f2i_sat(ceilf((max_y * 0.5f + 0.5f) * vp.w + vp.y)) - 1;
    const int64_t wm = (int64_t)W - 1, hm = (int64_t)H - 1;
    const uint32_t x0 = (uint32_t)(px0 < 0 ? 0 : (px0 > wm ? wm : px0));
    const uint32_t x1 = (uint32_t)(px1 < 0 ? 0 : (px1 > wm ? wm : px1));
    const uint32_t y0 = (uint32_t)(py0 < 0 ? 0 : (py0 > hm ? hm : py0));
    const uint32_t y1 = (uint32_t)(py1 < 0 ? 0 : (py1 > hm ? hm : py1));
    const uint32_t sx = kTile / tile_w, sy = kTile / tile_h;  // sub-tiles per reference tile
    const uint32_t tx_last = (W + tile_w - 1) / tile_w - 1, ty_last = (H + tile_h - 1) / tile_h - 1;
    uint32_t rx0 = x0 / kTile * sx, rx1 = min((x1 / kTile + 1) * sx - 1, tx_last);
    uint32_t ry0 = y0 / kTile * sy, ry1 = min((y1 / kTile + 1) * sy - 1, ty_last);
    if (sx > 1 || sy > 1) {
        // Sub-tiles that no sample passing the edge tests can reach are left out. The raster's candidate
        // rectangle (raster_tile.cuh pixel_rect) reaches from its first row ceil(c - D' - 0.5 - s) to its
        // last floor(c' + D' - 0.5 + s) (c, c' the box's edges in pixels, D' its bound D in pixels, s its
        // slack 0.05 + 1e-6 S, S the viewport size plus offset), each within 4e-7 S of exact, against the
        // pixel box's floor(c) .. ceil(c') - 1: with D' <= 1 it stays within the box grown by one pixel
        // while 0.05 + 1.8e-6 S < 0.5 (S <= 1e5), by two pixels while S <= 5e5. D grows with the largest
        // distance L between a vertex and a sample of the tile, so D computed here with L over the whole
        // reference-tile rectangle bounds D in every sub-tile of it.
        const float s0x = sx_[0], s0y = sy_[0], s1x = sx_[1], s1y = sy_[1], s2x = sx_[2], s2y = sy_[2];
        const float area = (s1x - s0x) * (s2y - s0y) - (s1y - s0y) * (s2x - s0x);
        // sample positions of the reference-tile rectangle's first and last column and row, from one
        // reciprocal per axis instead of sample_ndc's division, widened by 1e-5 (far more than the few
        // roundings by which they can differ) so that the range holds every sample the raster uses
        const float ix = 2.0f / vp.z, iy = 2.0f / vp.w;
        const float tsx_lo = ((float)(x0 / kTile * kTile) - vp.x + 0.5f) * ix - 1.0f - 1e-5f;
        const float tsx_hi = ((float)min(x1 / kTile * kTile + kTile - 1, W - 1) - vp.x + 0.5f) * ix - 1.0f + 1e-5f;
        const float tsy_lo = ((float)(y0 / kTile * kTile) - vp.y + 0.5f) * iy - 1.0f - 1e-5f;
        const float tsy_hi = ((float)min(y1 / kTile * kTile + kTile - 1, H - 1) - vp.y + 0.5f) * iy - 1.0f + 1e-5f;
        const float L = 1.01f * fmaxf(fmaxf(fabsf(max_x - tsx_lo), fabsf(tsx_hi - min_x)),
                                      fmaxf(fabsf(max_y - tsy_lo), fabsf(tsy_hi - min_y)));
        const float perim = fabsf(s1x - s0x) + fabsf(s1y - s0y) + fabsf(s2x - s1x) + fabsf(s2y - s1y) +
                            fabsf(s0x - s2x) + fabsf(s0y - s2y);
        const float D = 2.0f * (1e-7f + 2e-6f * L * L) * perim / fabsf(area);
        const float ext = fmaxf(max_x - min_x, max_y - min_y);
        const float S = fmaxf(vp.z + fabsf(vp.x), vp.w + fabsf(vp.y));
        const bool bounded = D <= fminf(ix, iy) && fabsf(area) >= 1e-4f * ext * ext && S <= 5e5f;
        if (bounded) {
            const uint32_t m = S <= 1e5f ? 1u : 2u;
            rx0 = max(rx0, (x0 < m ? 0u : x0 - m) / tile_w);
            rx1 = min(rx1, min(x1 + m, (uint32_t)wm) / tile_w);
            ry0 = max(ry0, (y0 < m ? 0u : y0 - m) / tile_h);
            ry1 = min(ry1, min(y1 + m, (uint32_t)hm) / tile_h);
        }
    }
    r.x = rx0 | (rx1 << 16);
    r.y = ry0 | (ry1 << 16);
    return r;
}

}  // namespace pdr

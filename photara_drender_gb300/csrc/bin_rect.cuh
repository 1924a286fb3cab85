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
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float4 p = pos[v[c]];
        if (!(p.w > 1e-8f) || !isfinite(p.w)) return r;
        const float x = p.x / p.w;
        const float y = p.y / p.w;
        if (!isfinite(x) || !isfinite(y)) return r;
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
    r.x = (x0 / kTile * sx) | (min((x1 / kTile + 1) * sx - 1, tx_last) << 16);
    r.y = (y0 / kTile * sy) | (min((y1 / kTile + 1) * sy - 1, ty_last) << 16);
    return r;
}

}  // namespace pdr

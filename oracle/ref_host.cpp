// Host driver for the reference's own CPU routines of the raster path (src/rasterizer.cpp):
// build_tile_bins (:61-138), build_vertex_adjacency (:145-162) and build_texture_sample_adjacency
// (:187-258), with the helpers they call. oracle/build.py cuts those definitions out of the reference
// source by name (brace-matched) into oracle/_ref/gen/rasterizer_host.inc; the rest of that file needs
// the absent Vulkan wrapper and is not compiled.
// TEST INFRASTRUCTURE ONLY: it exists to check oracle/pdr_oracle.c against the reference's code.
#include <photara_drender/types.hpp>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <span>
#include <stdexcept>
#include <vector>

namespace photara_drender {
namespace {
#include "rasterizer_host.inc"
}  // namespace
}  // namespace photara_drender

using namespace photara_drender;

extern "C" {

// Tile bins of one view: returns the entry count (offsets get tiles+1 values, list up to capacity
// entries), or -1 when the reference throws.
int64_t ref_build_tile_bins(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T, uint32_t width,
                            uint32_t height, const float* vp, uint32_t* offsets, uint32_t* list, uint64_t capacity) {
    try {
        const Viewport viewport{vp[0], vp[1], vp[2], vp[3]};
        const TileBins bins = build_tile_bins(std::span<const float>(pos, (size_t)V * 4),
                                              std::span<const uint32_t>(idx, (size_t)T * 3), width, height, viewport);
        std::memcpy(offsets, bins.offsets.data(), bins.offsets.size() * sizeof(uint32_t));
        const size_t n = std::min<size_t>(bins.triangle_indices.size(), capacity);
        if (n) std::memcpy(list, bins.triangle_indices.data(), n * sizeof(uint32_t));
        return (int64_t)bins.triangle_indices.size();
    } catch (...) {
        return -1;
    }
}

// Vertex -> corner CSR: offsets [V+1], corners [3T].
void ref_build_vertex_adjacency(const uint32_t* idx, uint32_t T, uint32_t V, uint32_t* offsets, uint32_t* corners) {
    const VertexAdjacency a = build_vertex_adjacency(std::span<const uint32_t>(idx, (size_t)T * 3), V);
    std::memcpy(offsets, a.offsets.data(), a.offsets.size() * sizeof(uint32_t));
    std::memcpy(corners, a.corners.data(), a.corners.size() * sizeof(uint32_t));
}

// Texel -> sample CSR with the double-precision weights: texel_offsets [tw*th+1], entries up to
// capacity, weights [P*4]. Returns the entry count, -1 (invalid_argument), -2 (out_of_range).
int64_t ref_build_texture_sample_adjacency(const float* uv, const float* raster, uint32_t width, uint32_t height,
                                           uint32_t tw, uint32_t th, uint32_t mode, uint32_t* texel_offsets,
                                           uint32_t* entries, uint64_t capacity, float* weights) {
    const size_t P = (size_t)width * height;
    RasterizeOutput r;
    r.width = width;
    r.height = height;
    r.raster.assign(raster, raster + P * 4);
    TextureDesc d;
    d.width = tw;
    d.height = th;
    d.channel_count = 4;
    d.address_mode = static_cast<AddressMode>(mode);
    try {
        const TextureSampleAdjacency a = build_texture_sample_adjacency(std::span<const float>(uv, P * 2), r, d);
        std::memcpy(texel_offsets, a.texel_offsets.data(), a.texel_offsets.size() * sizeof(uint32_t));
        const size_t n = std::min<size_t>(a.sample_entries.size(), capacity);
        if (n) std::memcpy(entries, a.sample_entries.data(), n * sizeof(uint32_t));
        std::memcpy(weights, a.sample_weights.data(), a.sample_weights.size() * sizeof(float));
        return (int64_t)a.sample_entries.size();
    } catch (const std::invalid_argument&) {
        return -1;
    } catch (const std::out_of_range&) {
        return -2;
    }
}

}  // extern "C"

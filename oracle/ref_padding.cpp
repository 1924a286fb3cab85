// C entry points over the reference's CPU texture_padding.cpp (compiled from its own source by
// oracle/build.py into oracle/_ref). TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <span>
#include <vector>

#include "photara_drender/texture_padding.hpp"

extern "C" float ref_suggest_softmax_scale(const float* pos, std::uint32_t V, const float* cams, std::uint32_t ncam) {
    return photara_drender::suggest_softmax_scale(std::span<const float>(pos, V * 3u),
                                                  std::span<const float>(cams, ncam * 3u));
}

namespace {
int invalid(const std::exception& e, char* message, std::size_t capacity) {
    if (message && capacity) {
        std::snprintf(message, capacity, "%s", e.what());
    }
    return -1;
}
}  // namespace

// pad_texture_atlas over caller buffers; filled may hold a previous filled_mask (or zeros).
// stats: valid, gutter, unobserved, remaining_unobserved, filled.
extern "C" int ref_pad_texture_atlas(float* color, std::uint32_t channels, const float* valid, const float* coverage,
                                     float* filled, std::uint32_t width, std::uint32_t height, std::uint32_t margin,
                                     int fill_unobserved, std::uint32_t maximum_fill_distance, float threshold,
                                     std::uint64_t* stats, char* message, std::size_t capacity) {
    const std::size_t n = static_cast<std::size_t>(width) * height;
    photara_drender::TextureBakeOutput out;
    out.width = width;
    out.height = height;
    out.color.assign(color, color + n * channels);
    out.valid_mask.assign(valid, valid + n);
    if (coverage) out.coverage_mask.assign(coverage, coverage + n);
    out.filled_mask.assign(filled, filled + n);
    photara_drender::TexturePaddingOptions options;
    options.margin = margin;
    options.fill_unobserved = fill_unobserved != 0;
    options.maximum_fill_distance = maximum_fill_distance;
    options.valid_threshold = threshold;
    try {
        const auto s = photara_drender::pad_texture_atlas(out, options);
        stats[0] = s.valid_texels;
        stats[1] = s.gutter_texels;
        stats[2] = s.unobserved_texels;
        stats[3] = s.remaining_unobserved;
        stats[4] = s.filled_texels;
    } catch (const std::invalid_argument& e) {
        return invalid(e, message, capacity);
    }
    std::copy(out.color.begin(), out.color.end(), color);
    std::copy(out.filled_mask.begin(), out.filled_mask.end(), filled);
    return 0;
}

// fill_texture_on_surface over caller buffers. stats: filled, remaining, measured faces, propagated faces.
extern "C" int ref_fill_texture_on_surface(float* color, std::uint32_t channels, const float* valid,
                                           const std::uint32_t* face_ids, float* filled, std::uint32_t width,
                                           std::uint32_t height, const std::uint32_t* indices,
                                           std::uint32_t triangle_count, std::uint64_t* stats, char* message,
                                           std::size_t capacity) {
    const std::size_t n = static_cast<std::size_t>(width) * height;
    photara_drender::TextureBakeOutput out;
    out.width = width;
    out.height = height;
    out.color.assign(color, color + n * channels);
    out.valid_mask.assign(valid, valid + n);
    out.face_ids.assign(face_ids, face_ids + n);
    out.filled_mask.assign(filled, filled + n);
    try {
        const auto s = photara_drender::fill_texture_on_surface(
            out, std::span<const std::uint32_t>(indices, static_cast<std::size_t>(triangle_count) * 3));
        stats[0] = s.filled_texels;
        stats[1] = s.remaining_texels;
        stats[2] = s.measured_faces;
        stats[3] = s.propagated_faces;
    } catch (const std::invalid_argument& e) {
        return invalid(e, message, capacity);
    }
    std::copy(out.color.begin(), out.color.end(), color);
    std::copy(out.filled_mask.begin(), out.filled_mask.end(), filled);
    return 0;
}

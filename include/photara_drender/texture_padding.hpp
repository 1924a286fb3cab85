// The reference's include/photara_drender/texture_padding.hpp: atlas padding, surface fill and the
// softmax scale heuristic. Padding and surface fill run on the current CUDA device.
#pragma once

#include <cstdint>
#include <span>

#include "photara_drender/types.hpp"

namespace photara_drender {

struct SurfaceFillStats {
    std::uint64_t filled_texels = 0;
    std::uint64_t remaining_texels = 0;
    std::uint64_t measured_faces = 0;
    std::uint64_t propagated_faces = 0;
};

// Keeps measured texels; fills covered texels without a sample with the measured mean colour of their
// face, or of the nearest measured face over shared mesh edges. triangle_indices are the original mesh's
// (before UV seam duplication). Components without any measurement stay empty.
[[nodiscard]] SurfaceFillStats fill_texture_on_surface(TextureBakeOutput& output,
                                                       std::span<const std::uint32_t> triangle_indices);

struct TexturePaddingOptions {
    // Guard band in texels copied outwards from valid texels (0 keeps only the in-chart fill).
    std::uint32_t margin = 4;
    // Fill covered chart texels that hold no projection sample.
    bool fill_unobserved = true;
    // Cap on the in-chart fill distance in texels (0 = unlimited).
    std::uint32_t maximum_fill_distance = 0;
    // A texel is a colour source when valid_mask >= valid_threshold.
    float valid_threshold = 0.5F;
};

struct TexturePaddingStats {
    std::uint64_t valid_texels = 0;
    std::uint64_t gutter_texels = 0;
    std::uint64_t unobserved_texels = 0;
    std::uint64_t remaining_unobserved = 0;
    std::uint64_t filled_texels = 0;
    double seconds = 0.0;
};

// Extends output.color in place and records extrapolated texels in output.filled_mask; valid_mask
// keeps its projection-valid meaning. Earlier covered fills (fill_texture_on_surface) seed gutters.
[[nodiscard]] TexturePaddingStats pad_texture_atlas(TextureBakeOutput& output,
                                                    const TexturePaddingOptions& options = {});

// 20 * (minimum squared distance between a (subsampled) mesh vertex and any camera), the softmax
// bake's scene-relative exponent scale; 0 when the input is degenerate.
[[nodiscard]] float suggest_softmax_scale(std::span<const float> positions, std::span<const float> camera_positions);

} // namespace photara_drender

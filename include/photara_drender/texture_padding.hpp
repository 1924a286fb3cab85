// The part of the reference's include/photara_drender/texture_padding.hpp this build provides.
#pragma once

#include <span>

namespace photara_drender {

// 20 * (minimum squared distance between a (subsampled) mesh vertex and any camera), the softmax
// bake's scene-relative exponent scale; 0 when the input is degenerate.
[[nodiscard]] float suggest_softmax_scale(std::span<const float> positions, std::span<const float> camera_positions);

} // namespace photara_drender

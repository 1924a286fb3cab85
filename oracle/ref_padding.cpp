// C entry points over the reference's CPU texture_padding.cpp (compiled from its own source by
// oracle/build.py into oracle/_ref). TEST INFRASTRUCTURE ONLY.
#include <cstdint>
#include <span>
#include <vector>

#include "photara_drender/texture_padding.hpp"

extern "C" float ref_suggest_softmax_scale(const float* pos, std::uint32_t V, const float* cams, std::uint32_t ncam) {
    return photara_drender::suggest_softmax_scale(std::span<const float>(pos, V * 3u),
                                                  std::span<const float>(cams, ncam * 3u));
}

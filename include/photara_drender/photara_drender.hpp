// Umbrella header of the photara_drender GB300 C++ API.
#pragma once

#include "photara_drender/context.hpp"
#include "photara_drender/rasterizer.hpp"
#include "photara_drender/texture_baker.hpp"
#include "photara_drender/texture_padding.hpp"
#include "photara_drender/texture_refiner.hpp"
#include "photara_drender/types.hpp"

// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
//
// An RGBA float colour and pack_sRGB: each of r, g, b is encoded with the
// IEC 61966-2-1 sRGB transfer function (evaluated in double), scaled by 255,
// rounded half up and clamped to [0, 255]; alpha is 255.  Red is the low byte.
#pragma once

#include <cmath>
#include <cstdint>
#include "../core/Globals.h"

namespace cg
{

struct Color
{
    float r, g, b, a = 1.0f;
};

HOST DEVICE inline uint32_t pack_sRGB_channel(float c)
{
    const double x = c <= 0.0031308f ? 12.92 * c : 1.055 * std::pow(double(c), 1.0 / 2.4) - 0.055;
    const int v = int(x * 255.0 + 0.5);
    return uint32_t(v < 0 ? 0 : (v > 255 ? 255 : v));
}

HOST DEVICE inline uint32_t pack_sRGB(float r, float g, float b)
{
    return pack_sRGB_channel(r) | (pack_sRGB_channel(g) << 8) | (pack_sRGB_channel(b) << 16) | 0xFF000000u;
}

} // namespace cg

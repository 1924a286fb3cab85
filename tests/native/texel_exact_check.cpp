// Checks pdr::exact_texel_coordinate (integer arithmetic) against the double-precision
// formula of src/rasterizer.cpp:207-215 on seeded random and edge-case inputs.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "pdr_common.cuh"

static int check(float u, uint32_t size, long long* fails) {
    const double t = (double)u * size - 0.5;
    int32_t b = 0;
    float f = 0.0f;
    const int rc = pdr::exact_texel_coordinate(u, size, &b, &f);
    if (!std::isfinite(u)) {
        if (rc != pdr::kTexelNonFinite) ++*fails;
        return 0;
    }
    if (std::fabs(t) > 1.0e9) {
        if (rc != pdr::kTexelRange) { ++*fails; if (*fails < 10) std::printf("range u=%a size=%u\n", u, size); }
        return 0;
    }
    const int32_t rb = (int32_t)std::floor(t);
    const float rf = (float)(t - std::floor(t));
    uint32_t a, c;
    std::memcpy(&a, &f, 4);
    std::memcpy(&c, &rf, 4);
    if (rc != 0 || b != rb || a != c) {
        ++*fails;
        if (*fails < 10) std::printf("u=%a size=%u got (%d,%a) want (%d,%a) rc=%d\n", u, size, b, f, rb, rf, rc);
    }
    return 1;
}

int main() {
    std::mt19937_64 rng(1234);
    long long fails = 0, n = 0;
    const uint32_t sizes[] = {1, 2, 3, 4, 7, 16, 1000, 1024, 4095, 4096, 8192, 16384, 65535, 1u << 20, (1u << 28) + 3};
    for (uint32_t size : sizes) {
        for (int i = 0; i < 200000; ++i) {
            float u;
            switch (i % 5) {
                case 0: u = std::uniform_real_distribution<float>(-0.5f, 1.5f)(rng); break;
                case 1: u = std::ldexp(std::uniform_real_distribution<float>(-1.f, 1.f)(rng),
                                       -(int)(rng() % 140)); break;
                case 2: u = ((float)(rng() % (4ull * size + 1)) + 0.5f) / (float)size - 1.0f; break;
                case 3: { uint32_t bits = (uint32_t)rng(); std::memcpy(&u, &bits, 4); break; }
                default: u = std::nextafter(((float)(rng() % (2ull * size + 1)) + 0.5f) / (float)size,
                                            (rng() & 1) ? 10.f : -10.f);
            }
            n += check(u, size, &fails);
        }
        const float specials[] = {0.0f, -0.0f, 1.0f, -1.0f, 0.5f, 1e-45f, -1e-45f, 1e-30f, -1e-30f, INFINITY, NAN};
        for (float u : specials) n += check(u, size, &fails);
    }
    std::printf("checked=%lld fails=%lld\n", n, fails);
    return fails == 0 ? 0 : 1;
}

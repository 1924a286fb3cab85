// Shared device helpers for the photara_drender GB300 kernels.
//
// Numerics follow the reference's HLSL shaders operation by operation; the library is compiled
// with -fmad=false so no multiply-add is contracted, and with IEEE division and square root.
// Conventions where the shaders leave behaviour to the platform (same as the CPU oracle):
//  - float -> int conversions saturate, NaN -> 0;
//  - clamp/min/max are IEEE minNum/maxNum (fminf/fmaxf);
//  - round() is round-half-to-even (rintf).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PDR_HD __host__ __device__ __forceinline__
#else
#define PDR_HD inline
#include <cmath>
#endif

namespace pdr {

constexpr uint32_t kTile = 16;  // src/rasterizer.cpp:19 RASTER_TILE_SIZE

PDR_HD int32_t f2i_sat(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f < -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}

PDR_HD uint32_t f2u_sat(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return UINT32_MAX;
    return (uint32_t)f;
}

// (uint)round(raster.w): the shaders' triangle-id decode.
PDR_HD uint32_t raster_id(float w) { return f2u_sat(rintf(w)); }

PDR_HD float clamp_hlsl(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

PDR_HD int32_t clampi(int32_t x, int32_t lo, int32_t hi) { return x < lo ? lo : (x > hi ? hi : x); }

PDR_HD int32_t add1(int32_t x) { return (int32_t)((uint32_t)x + 1u); }

PDR_HD float cross2(float ax, float ay, float bx, float by) { return ax * by - ay * bx; }

// rasterize_forward.hlsl:55-57 pixel-centre NDC
PDR_HD float sample_ndc(uint32_t p, float v0, float vsize) {
    return ((float)p - v0 + 0.5f) * 2.0f / vsize - 1.0f;
}

// texture_forward.hlsl:16-35 / src/rasterizer.cpp:164-179
PDR_HD int32_t address_coordinate(int32_t c, uint32_t size, uint32_t mode) {
    if (mode == 0) return clampi(c, 0, (int32_t)size - 1);
    if (mode == 1) {
        const int32_t r = c % (int32_t)size;
        return r < 0 ? r + (int32_t)size : r;
    }
    const int32_t period = (int32_t)size * 2;
    int32_t m = c % period;
    if (m < 0) m += period;
    return m < (int32_t)size ? m : period - 1 - m;
}

// Correctly rounded unsigned 64-bit -> float.
PDR_HD float u64_to_float_rn(uint64_t n) {
#if defined(__CUDA_ARCH__)
    return __ull2float_rn(n);
#else
    return (float)n;
#endif
}

PDR_HD float ldexp_exact(float x, int e) {
#if defined(__CUDA_ARCH__)
    return ldexpf(x, e);
#else
    return std::ldexp(x, e);
#endif
}

// The texel->sample table of src/rasterizer.cpp:207-215 computes
//   t = (double)u * size - 0.5;  base = (int)floor(t);  fraction = (float)(t - floor(t))
// in double precision. For size < 2^29 and |t| <= 1e9 every double step there is exact, so the
// fraction is the correctly rounded float of frac(u*size - 0.5). This routine computes the same
// two values with 64-bit integer arithmetic from the bits of u (no FP64 instructions).
// Returns 0, or kTexelNonFinite for a non-finite u (the reference throws std::invalid_argument),
// or kTexelRange when |t| > 1e9 (the reference throws std::out_of_range).
constexpr int kTexelNonFinite = 1;
constexpr int kTexelRange = 2;

PDR_HD int exact_texel_coordinate(float u, uint32_t size, int32_t* base, float* fraction) {
    uint32_t bits;
#if defined(__CUDA_ARCH__)
    bits = __float_as_uint(u);
#else
    __builtin_memcpy(&bits, &u, 4);
#endif
    const uint32_t exp_field = (bits >> 23) & 0xffu;
    if (exp_field == 0xffu) return kTexelNonFinite;
    const bool negative = (bits >> 31) != 0;
    uint64_t m = bits & 0x7fffffu;
    int e2;
    if (exp_field == 0) {
        e2 = -149;
    } else {
        m |= 0x800000u;
        e2 = (int)exp_field - 150;
    }
    if (m == 0) {  // u = +-0: t = -0.5
        *base = -1;
        *fraction = 0.5f;
        return 0;
    }
    const uint64_t P = m * (uint64_t)size;  // < 2^54, exact
    if (e2 >= 0) {
        // integer x = +-P * 2^e2; t = x - 0.5
        if (e2 > 31 || P > ((1ull << 31) >> e2)) return kTexelRange;
        const int64_t x = (int64_t)(P << e2);
        const int64_t xs = negative ? -x : x;
        if (xs > 1000000000ll || xs < -999999999ll) return kTexelRange;  // |x - 0.5| > 1e9
        *base = (int32_t)(xs - 1);
        *fraction = 0.5f;
        return 0;
    }
    const int k = -e2;  // x = +-P / 2^k
    if (k >= 64) {
        // |x| < 2^-10: t lies in (-0.51, -0.49), base -1, fraction = 0.5 + x rounded to float.
        if (!negative) {
            // grid 2^-24 above 0.5: q = RN(x * 2^24)
            const int s = k - 24;  // >= 40
            uint64_t q = s >= 64 ? 0 : (P >> s);
            const uint64_t rem_mask = s >= 64 ? ~0ull : ((1ull << s) - 1);
            const uint64_t rem = s >= 64 ? P : (P & rem_mask);
            const uint64_t half = s >= 65 ? 0 : (1ull << (s - 1));
            if (s < 65 && (rem > half || (rem == half && (q & 1)))) q += 1;
            *base = -1;
            *fraction = 0.5f + ldexp_exact((float)q, -24);
        } else {
            // grid 2^-25 below 0.5: q = RN(|x| * 2^25)
            const int s = k - 25;  // >= 39
            uint64_t q = s >= 64 ? 0 : (P >> s);
            const uint64_t rem = s >= 64 ? P : (P & ((1ull << s) - 1));
            const uint64_t half = s >= 65 ? 0 : (1ull << (s - 1));
            if (s < 65 && (rem > half || (rem == half && (q & 1)))) q += 1;
            *base = -1;
            *fraction = 0.5f - ldexp_exact((float)q, -25);
        }
        return 0;
    }
    const uint64_t ip = P >> k;
    const uint64_t fp = P & ((1ull << k) - 1);
    int64_t I;
    uint64_t F;
    if (!negative) {
        I = (int64_t)ip;
        F = fp;
    } else if (fp == 0) {
        I = -(int64_t)ip;
        F = 0;
    } else {
        I = -(int64_t)ip - 1;
        F = (1ull << k) - fp;
    }
    const uint64_t half = 1ull << (k - 1);
    int64_t b;
    uint64_t N;
    if (F >= half) {
        b = I;
        N = F - half;
    } else {
        b = I - 1;
        N = F + half;
    }
    // t = b + N / 2^k ; reject |t| > 1e9
    if (b > 1000000000ll || b < -1000000000ll || (b == 1000000000ll && N != 0)) return kTexelRange;
    *base = (int32_t)b;
    *fraction = N == 0 ? 0.0f : ldexp_exact(u64_to_float_rn(N), -k);
    return 0;
}

#if defined(__CUDACC__)
// Warp-aggregated vector reduction: adds v to the four floats at addr (16-byte aligned). Lanes of the
// calling warp that target the same address first sum their values with shuffles (in lane order) and
// the lowest of them issues one red.global.add.v4.f32; a lane alone issues its own. Call it from
// converged code or through the same branch: the lanes reported by __activemask() all take part.
__device__ __forceinline__ void red_add_v4_aggregated(float* addr, float4 v) {
    const uint32_t active = __activemask();
    const uint32_t peers = __match_any_sync(active, (unsigned long long)addr);
    const uint32_t lane = threadIdx.x & 31u;
    if (peers != (1u << lane)) {
        const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
        uint32_t rest = peers & (peers - 1u);  // every peer but the leader, in lane order
        while (rest) {
            const int src = __ffs(rest) - 1;
            rest &= rest - 1u;
            const float x = __shfl_sync(peers, v.x, src), y = __shfl_sync(peers, v.y, src);
            const float z = __shfl_sync(peers, v.z, src), w = __shfl_sync(peers, v.w, src);
            if (lane == leader) {
                v.x += x;
                v.y += y;
                v.z += z;
                v.w += w;
            }
        }
        if (lane != leader) return;
    }
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

// A texture-gradient tap: warp-aggregated when the texture is magnified (fewer texels than pixels per
// view, so neighbouring pixels share texels), a plain vector reduction otherwise (mostly distinct texels:
// the address match costs more than it saves). Measured on the fused adjoint of 64 views at 1024x1024:
// a 256x256 atlas 4.27 -> 3.93 ms with aggregation, a 4096x4096 atlas 3.73 -> 4.22 ms.
__device__ __forceinline__ void red_add_v4_texel(float* addr, float4 v, bool aggregate) {
    if (aggregate) {
        red_add_v4_aggregated(addr, v);
        return;
    }
    // evict-last priority in L2: a texel's gradient line is hit again by the next views' pixels
    unsigned long long pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    asm volatile("red.global.add.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(addr), "f"(v.x), "f"(v.y),
                 "f"(v.z), "f"(v.w), "l"(pol)
                 : "memory");
}
#endif

}  // namespace pdr

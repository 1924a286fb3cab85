// Minimal HLSL-compute-to-C++ shim used only to compile the reference's own shader sources
// on the CPU as the checker (oracle/_ref). TEST INFRASTRUCTURE ONLY.
//
// The same platform conventions as oracle/pdr_oracle.c apply:
//  - float -> int casts saturate (NaN -> 0); float -> uint casts clamp negatives to 0;
//  - min/max/clamp follow IEEE maxNum/minNum (fminf/fmaxf);
//  - round() is round-half-to-even; lerp(x, y, s) = x*(1-s) + y*s;
//  - normalize(v) = v / sqrt(dot(v, v)).
// Group barriers run the 64 invocations of a group in lane order between barriers, so the
// shared-memory reductions and compare-exchange loops execute deterministically.
#pragma once

#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <mutex>

namespace hlsl {

typedef unsigned int uint;

struct hfloat {
    float v;
    operator float() const { return v; }
    explicit operator int() const {
        if (v != v) return 0;
        if (v >= 2147483648.0f) return 2147483647;
        if (v < -2147483648.0f) return (-2147483647 - 1);
        return (int)v;
    }
    explicit operator unsigned int() const {
        if (!(v > 0.0f)) return 0u;
        if (v >= 4294967296.0f) return 4294967295u;
        return (unsigned int)v;
    }
};

struct bool2 { bool x, y; };
struct bool3 { bool x, y, z; };
inline bool all(bool2 b) { return b.x && b.y; }
inline bool any(bool2 b) { return b.x || b.y; }

inline int sat_i(float v) { return (int)hfloat{v}; }

struct int2;
struct uint2 {
    uint x, y;
    uint2() = default;
    uint2(uint a, uint b) : x(a), y(b) {}
};
struct float2 {
    float x, y;
    float2() = default;
    float2(float s) : x(s), y(s) {}
    float2(float a, float b) : x(a), y(b) {}
    float2(uint a, uint b) : x((float)a), y((float)b) {}
    float2& operator+=(const float2& o) { x = x + o.x; y = y + o.y; return *this; }
};
// Read-only swizzle views; they share storage with the vector in an anonymous union.
template <int N> struct SwzXY3 { float v[N]; operator float2() const { return float2(v[0], v[1]); } };
struct float3 {
    union {
        struct { float x, y, z; };
        SwzXY3<3> xy;
    };
    float3() : x(0), y(0), z(0) {}
    float3(float s) : x(s), y(s), z(s) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
};
struct SwzZW4 { float v[4]; operator float2() const { return float2(v[2], v[3]); } };
struct SwzXYZ4 { float v[4]; operator float3() const { return float3(v[0], v[1], v[2]); } };
struct SwzUXY3 { uint v[3]; operator uint2() const { return uint2(v[0], v[1]); } };

struct uint3 {
    union {
        struct { uint x, y, z; };
        SwzUXY3 xy;
    };
    uint3() : x(0), y(0), z(0) {}
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};
struct uint4 { uint x, y, z, w; };

struct int2 {
    int x, y;
    int2() = default;
    int2(int a, int b) : x(a), y(b) {}
    explicit int2(const float2& f) : x(sat_i(f.x)), y(sat_i(f.y)) {}
};
inline int2 operator+(int2 a, int2 b) { return int2((int)((unsigned)a.x + (unsigned)b.x), (int)((unsigned)a.y + (unsigned)b.y)); }
inline int2 clamp(int2 v, int2 lo, int2 hi) {
    return int2(v.x < lo.x ? lo.x : (v.x > hi.x ? hi.x : v.x), v.y < lo.y ? lo.y : (v.y > hi.y ? hi.y : v.y));
}

struct float4 {
    union {
        struct { float x, y, z, w; };
        SwzXY3<4> xy;
        SwzZW4 zw;
        SwzXYZ4 xyz;
    };
    float4() : x(0), y(0), z(0), w(0) {}
    float4(float s) : x(s), y(s), z(s), w(s) {}
    float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    float4(const float3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float4(const float2& v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    float4& operator+=(const float4& o) { x = x + o.x; y = y + o.y; z = z + o.z; w = w + o.w; return *this; }
};

#define HLSL_V2OP(OP)                                                                  \
    inline float2 operator OP(float2 a, float2 b) { return float2(a.x OP b.x, a.y OP b.y); } \
    inline float2 operator OP(float2 a, float b) { return float2(a.x OP b, a.y OP b); }      \
    inline float2 operator OP(float a, float2 b) { return float2(a OP b.x, a OP b.y); }      \
    inline float3 operator OP(float3 a, float3 b) { return float3(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
    inline float3 operator OP(float3 a, float b) { return float3(a.x OP b, a.y OP b, a.z OP b); }        \
    inline float4 operator OP(float4 a, float4 b) { return float4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); }
HLSL_V2OP(+)
HLSL_V2OP(-)
HLSL_V2OP(*)
HLSL_V2OP(/)
#undef HLSL_V2OP
inline float2 operator-(float2 a) { return float2(-a.x, -a.y); }

inline bool2 operator==(float2 a, float b) { return bool2{a.x == b, a.y == b}; }
inline bool2 operator<(float2 a, float b) { return bool2{a.x < b, a.y < b}; }
inline bool2 operator>(float2 a, float b) { return bool2{a.x > b, a.y > b}; }
inline bool2 operator<(float2 a, float2 b) { return bool2{a.x < b.x, a.y < b.y}; }
inline bool2 operator>=(float2 a, float2 b) { return bool2{a.x >= b.x, a.y >= b.y}; }

inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }
inline float2 min(float2 a, float2 b) { return float2(fminf(a.x, b.x), fminf(a.y, b.y)); }
inline float2 max(float2 a, float2 b) { return float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
inline float clamp(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
inline int clamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline float2 clamp(float2 v, float lo, float hi) { return float2(clamp(v.x, lo, hi), clamp(v.y, lo, hi)); }
inline float saturate(float v) { return clamp(v, 0.0f, 1.0f); }
inline hfloat floor(float v) { return hfloat{floorf(v)}; }
inline float2 floor(float2 v) { return float2(floorf(v.x), floorf(v.y)); }
inline hfloat ceil(float v) { return hfloat{ceilf(v)}; }
inline hfloat round(float v) { return hfloat{rintf(v)}; }
inline float abs(float v) { return fabsf(v); }
inline float sqrt(float v) { return sqrtf(v); }
inline float exp(float v) { return expf(v); }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float length(float3 v) { return sqrtf(dot(v, v)); }
inline float3 normalize(float3 v) { return v / sqrtf(dot(v, v)); }
inline float lerp(float a, float b, float s) { return a * (1.0f - s) + b * s; }
inline uint asuint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline float asfloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }

template <class T>
struct StructuredBuffer {
    const T* data = nullptr;
    const T& operator[](uint i) const { return data[i]; }
};
template <class T>
struct RWStructuredBuffer {
    T* data = nullptr;
    T& operator[](uint i) const { return data[i]; }
};
template <class T>
using ConstantBuffer = T;

// Lane-ordered group scheduler: invocation `lane` runs only while it holds the turn.
struct GroupScheduler {
    std::mutex mu;
    std::condition_variable cv;
    uint lanes = 1;
    uint turn = 0;
    void wait_turn(uint lane) {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return turn == lane; });
    }
    void pass(uint lane) {
        std::lock_guard<std::mutex> lk(mu);
        turn = (lane + 1) % lanes;
        cv.notify_all();
    }
};
extern thread_local GroupScheduler* tls_group;
extern thread_local uint tls_lane;
inline void GroupMemoryBarrierWithGroupSync() {
    if (!tls_group) return;
    tls_group->pass(tls_lane);
    tls_group->wait_turn(tls_lane);
}
inline void InterlockedCompareExchange(uint& dest, uint compare, uint value, uint& original) {
    original = dest;
    if (dest == compare) dest = value;
}

} // namespace hlsl

// Atlas padding and surface fill on the device: src/texture_padding.cpp:37-351.
//
// pad_texture_atlas (texture_padding.cpp:226-351) extends valid texels into the chart gutter and into
// covered texels that received no sample, each taking the colour of its nearest source texel under the
// reference's Danielsson 8SSEDT field (texture_padding.cpp:37-95). That field is the result of two
// sequential raster sweeps; it is not the exact Euclidean transform, and the colour a texel receives
// depends on the sweeps' tie-breaking, so it is reproduced exactly:
//
// * a texel's forward-sweep value depends only on the forward values of (x-1,y), (x,y-1), (x-1,y-1) and
//   (x+1,y-1); the reverse sweep mirrors this. A warp therefore sweeps 32 rows at once on a skewed
//   wavefront: lane r handles row 32*band + r and reaches column i at step i + 2r, so the three upper
//   neighbours are the values lane r-1 produced one, two and three steps earlier (one shuffle a step)
//   and the left neighbour is the lane's own previous value. Each relaxation then runs in the
//   reference's order with its strict comparison and clamp, so every texel takes the same value.
// * bands are warps ordered by a ticket; a band's first row reads the row above from the previous
//   band's boundary buffer. Entries start as a marker that no offset can equal (|offset| <= 16384), so
//   a value is ready exactly when it differs from the marker: no fences. Every wait is bounded.
// * the fill is per texel. A source texel is never written, so copies from it are race-free; the only
//   other case (an offset inherited from a texel with no source that lands inside the atlas, possible
//   only when both sides exceed 12000) is resolved in the reference's raster order from a snapshot.
//
// fill_texture_on_surface (texture_padding.cpp:100-184): per-face means summed in double in pixel order
// (a stable radix sort of (face, pixel) keeps that order), the shared-edge face graph (radix-sorted edge
// keys), and a multi-source breadth-first search that assigns each face the source of the first face
// in the reference's FIFO order that reaches it (one CTA, level by level; queue order inside a level is
// the (parent position, neighbour slot) order, kept by an ordered compaction).
#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr int32_t kFar = 12000;      // texture_padding.cpp:20: offset of texels with no source yet
constexpr int32_t kMaxSide = 16384;  // texture_padding.cpp:18: offsets are clamped to +-kMaxSide
constexpr uint32_t kMarker = 0x80808080u;  // int16 halves -32640: never a stored offset
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kRing = 4;             // sweep steps of prefetch
constexpr int kLead = 8;             // columns a waiting band lets the previous band get ahead
constexpr int kL2Ahead = 64;         // steps the reverse sweep prefetches the forward field into L2
constexpr long long kWaitCycles = 1ll << 32;  // about two seconds at GB300 clocks
constexpr int kStatThreads = 256;

enum : uint32_t { kErrTimeout = 1, kErrFaceRange = 2, kErrDegenerate = 4, kErrManifold = 8 };

__device__ __forceinline__ uint32_t pack(int32_t x, int32_t y) {
    return (uint32_t)(uint16_t)(int16_t)x | ((uint32_t)(uint16_t)(int16_t)y << 16);
}
__device__ __forceinline__ int32_t unpack_x(uint32_t v) { return (int32_t)(int16_t)(v & 0xFFFFu); }
__device__ __forceinline__ int32_t unpack_y(uint32_t v) { return (int32_t)(int16_t)(v >> 16); }

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// texture_padding.cpp:54-78: adopt the candidate when its squared length is strictly smaller; the stored
// offset is clamped. |candidate| <= 16385 per component, so squared lengths fit in int32.
__device__ __forceinline__ void relax(int32_t& hx, int32_t& hy, int32_t& hk, int32_t cx, int32_t cy) {
    const int32_t ck = cx * cx + cy * cy;
    if (ck < hk) {
        hx = min(max(cx, -kMaxSide), kMaxSide);
        hy = min(max(cy, -kMaxSide), kMaxSide);
        hk = hx * hx + hy * hy;
    }
}

template <typename T>
__device__ __forceinline__ T block_sum(T v, T* shared) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) shared[warp] = v;
    __syncthreads();
    T total = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) total += shared[w];
    return total;  // valid in thread 0
}

// texture_padding.cpp:253-270: source texels (valid, or earlier covered fills), the cleared filled_mask
// of everything else, and the valid / carried-over counts. One warp per 32-texel word of a row.
__global__ void __launch_bounds__(kStatThreads) pad_classify_kernel(
    const float* __restrict__ valid, const float* __restrict__ coverage, float* __restrict__ filled,
    uint32_t* __restrict__ src_bits, uint32_t words_per_row, uint32_t W, uint32_t H, float threshold,
    unsigned long long* __restrict__ stats) {
    __shared__ unsigned long long red[kStatThreads / 32];
    const uint64_t words = (uint64_t)words_per_row * H;
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long nvalid = 0, ncarried = 0;
    for (uint64_t wd = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; wd < words;
         wd += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
        const uint32_t y = (uint32_t)(wd / words_per_row), word = (uint32_t)(wd % words_per_row);
        const uint32_t x = word * 32 + lane;
        bool v = false, src = false, carried = false;
        if (x < W) {
            const uint64_t p = (uint64_t)y * W + x;
            v = valid[p] >= threshold;
            src = v;
            if (!v) {
                if (filled[p] > 0.5f && coverage && coverage[p] > 0.5f) {
                    src = carried = true;
                } else {
                    filled[p] = 0.0f;
                }
            }
        }
        const uint32_t bits = __ballot_sync(0xFFFFFFFFu, src);
        if (lane == 0) src_bits[wd] = bits;
        nvalid += v;
        ncarried += carried;
    }
    const unsigned long long a = block_sum(nvalid, red);
    if (threadIdx.x == 0 && a) atomicAdd(&stats[0], a);
    const unsigned long long b = block_sum(ncarried, red);
    if (threadIdx.x == 0 && b) {
        atomicAdd(&stats[2], b);
        atomicAdd(&stats[4], b);
    }
}

// Waits for a boundary value of the previous band; kMarker when the wait gave up or another band failed.
__device__ uint32_t wait_boundary(const uint32_t* p, uint32_t* control) {
    const long long start = clock64();
    for (;;) {
        const uint32_t v = ld_relaxed(p);
        if (v != kMarker) return v;
        if (ld_relaxed(control + 2) != 0) return kMarker;
        if (clock64() - start > kWaitCycles) {
            atomicExch(control + 2, 1u);
            return kMarker;
        }
        __nanosleep(64);
    }
}

// Field layout: band-major, [band][step][lane] with W + 62 steps per band, so each sweep step stores one
// 128-byte line. Forward band b, lane r is row 32b + r and reaches column x at step x + 2r. The reverse
// sweep mirrors it: its band b' takes the rows of forward band B = bands - 1 - b' bottom-up (lane r' is
// row 32B + 31 - r') and its step t' is column W - 1 - (t' - 2r'), which the forward band stored at step
// W + 61 - t' for every lane: one coalesced line per step again.
__device__ __forceinline__ uint32_t field_index(uint32_t band, uint32_t steps, uint32_t t, uint32_t lane) {
    return (band * steps + t) * 32u + lane;
}

// The reverse-sweep (final) offset of texel (x, y).
__device__ __forceinline__ uint32_t final_index(uint32_t x, uint32_t y, uint32_t W, uint32_t bands) {
    const uint32_t r = 31u - (y & 31u);
    return field_index(bands - 1u - (y >> 5), W + 62u, (W - 1u - x) + 2u * r, r);
}

// One 8SSEDT sweep (texture_padding.cpp:80-94): the forward sweep writes `out` from the source bits, the
// reverse sweep (kBack) reads the forward field `in` and writes the final field `out`. control: [0]
// forward ticket, [1] reverse ticket, [2] failure flag.
//
// kExact keeps the reference's relaxations one by one, with their clamp of offsets to +-16384. Without
// it (atlas sides <= 4384) no offset component can exceed +-16383 (a real source is closer than the atlas
// side, an offset inherited from a texel without source is at most 12000 + side - 1), so no candidate is
// ever clamped, and the sequential relaxations equal "the first of [own, left, up, up-left, up-right] with
// the smallest squared length": everything but the left neighbour is reduced off the step's critical path.
template <bool kBack, bool kExact>
__global__ void __launch_bounds__(32) pad_sweep_kernel(const uint32_t* __restrict__ src_bits, uint32_t words_per_row,
                                                       const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                       uint32_t* __restrict__ boundary, uint32_t* control,
                                                       uint32_t* status, int32_t W, int32_t H) {
    const int lane = threadIdx.x;
    uint32_t band = 0;
    if (lane == 0) band = atomicAdd(&control[kBack ? 1 : 0], 1u);
    band = __shfl_sync(0xFFFFFFFFu, band, 0);
    const uint32_t bands = ((uint32_t)H + 31u) / 32u;
    const uint32_t steps = (uint32_t)W + 62u;
    // this lane's row and whether the row processed before it (above / below) exists
    const int32_t y = kBack ? (int32_t)((bands - 1u - band) * 32u + 31u) - lane : (int32_t)(band * 32u) + lane;
    const bool row_ok = y < H;
    const bool has_prev_row = kBack ? y + 1 < H : y >= 1;
    const int32_t dx = kBack ? -1 : 1, dy = kBack ? -1 : 1;
    const uint32_t* prev_boundary = boundary + (size_t)(band ? band - 1 : 0) * (uint32_t)W;
    uint32_t* my_boundary = boundary + (size_t)band * (uint32_t)W;
    const bool publish = lane == 31 && band + 1 < bands;
    // lane 0 reads the previous band's last row; in the reverse sweep's first band (a partial forward band)
    // lane 0 may have no row, and then neither it nor its band has a row below
    const bool reads_boundary = lane == 0 && band > 0 && row_ok;
    const uint32_t yc = row_ok ? (uint32_t)y : 0u;
    const uint32_t mirror = bands - 1u - band;

    // initial value of this lane's texel at step t (forward: source bit; reverse: the forward field)
    auto init_at = [&](int32_t t) -> uint32_t {
        if (kBack) {
            const int32_t tf = min(max((int32_t)steps - 1 - t, 0), (int32_t)steps - 1);
            return in[field_index(mirror, steps, (uint32_t)tf, 31u - lane)];
        }
        const int32_t x = min(max(t - 2 * lane, 0), W - 1);
        const uint32_t w = src_bits[yc * words_per_row + ((uint32_t)x >> 5)];
        return ((w >> (x & 31)) & 1u) ? 0u : pack(kFar, kFar);
    };
    // lane 0: the previous band's last row at sweep index t + 1 (may still be the marker)
    auto boundary_at = [&](int32_t t) -> uint32_t {
        const int32_t j = t + 1;
        if (!reads_boundary || j >= W) return kMarker;
        return ld_relaxed(prev_boundary + j);
    };

    // ring: this lane's initial values for the next kRing steps. cur / nxt: lane 0's boundary values
    // (row above, sweep index t + 1) for this chunk and the next one, loaded a chunk ahead.
    uint32_t ring[kRing], cur[kRing], nxt[kRing];
#pragma unroll
    for (int k = 0; k < kRing; ++k) {
        ring[k] = init_at(k);
        nxt[k] = boundary_at(k);
    }
    int32_t mx = 0, my = 0;                       // this lane's value at the previous step (index i - 1)
    int32_t nrx = 0, nry = 0, rx = 0, ry = 0, prx = 0, pry = 0;  // row above at i + 1, i, i - 1
    bool failed = false;
    if (reads_boundary) {
        // column 0 of the row above: lanes r > 0 receive it from lane r - 1 the step before they start
        const uint32_t v = wait_boundary(prev_boundary, control);
        failed = v == kMarker;
        nrx = unpack_x(v);
        nry = unpack_y(v);
    }
    for (int32_t t0 = 0; t0 < (int32_t)steps; t0 += kRing) {
        if (reads_boundary) {
            bool ready = true;
#pragma unroll
            for (int k = 0; k < kRing; ++k) {
                cur[k] = nxt[k];
                ready &= t0 + k + 1 >= W || cur[k] != kMarker;
            }
            if (!ready && !failed) {
                // The previous band has not reached this chunk: wait until it is kLead columns further
                // on, so the chunks after this one find their values written, then reload this chunk.
                // Stores of another SM may become visible out of order, so every value is re-checked.
                const int32_t far = min(t0 + kRing + kLead, W - 1);
                failed = wait_boundary(prev_boundary + far, control) == kMarker;
#pragma unroll
                for (int k = 0; k < kRing; ++k) {
                    const int32_t j = t0 + k + 1;
                    if (j < W) cur[k] = ld_relaxed(prev_boundary + j);
                }
#pragma unroll
                for (int k = 0; k < kRing; ++k) {
                    const int32_t j = t0 + k + 1;
                    if (j < W && cur[k] == kMarker && !failed) {
                        cur[k] = wait_boundary(prev_boundary + j, control);
                        failed |= cur[k] == kMarker;
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kRing; ++k) nxt[k] = boundary_at(t0 + kRing + k);
        }
#pragma unroll
        for (int k = 0; k < kRing; ++k) {
            const int32_t t = t0 + k;
            int32_t ux = __shfl_up_sync(0xFFFFFFFFu, mx, 1);
            int32_t uy = __shfl_up_sync(0xFFFFFFFFu, my, 1);
            if (reads_boundary) {
                ux = unpack_x(cur[k]);
                uy = unpack_y(cur[k]);
            }
            prx = rx; pry = ry;
            rx = nrx; ry = nry;
            nrx = ux; nry = uy;
            const uint32_t init = ring[k];
            ring[k] = init_at(t + kRing);
            if (kBack && lane == 0 && t + kL2Ahead < (int32_t)steps) {
                // the forward field line kL2Ahead steps ahead (all 32 lanes' values of that step): into L2
                // now, so the ring's load a few steps before its use finds it there instead of in DRAM
                const uint32_t* line = in + field_index(mirror, steps, steps - 1u - (uint32_t)(t + kL2Ahead), 0u);
                asm volatile("prefetch.global.L2 [%0];" ::"l"(line));
            }
            const int32_t i = t - 2 * lane;
            const bool active = row_ok && i >= 0 && i < W;
            const bool up = has_prev_row, left = i >= 1, right = i + 1 < W;
            const int32_t ix = unpack_x(init), iy = unpack_y(init);
            const int32_t lcx = mx - dx, lcy = my;                     // left (previous texel of the row)
            const int32_t rcx = rx, rcy = ry - dy;                     // up
            const int32_t pcx = prx - dx, pcy = pry - dy;              // up-left
            const int32_t ncx = nrx + dx, ncy = nry - dy;              // up-right
            int32_t hx, hy;
            if (kExact) {
                hx = ix;
                hy = iy;
                int32_t hk = ix * ix + iy * iy;
                if (left) relax(hx, hy, hk, lcx, lcy);
                if (up) {
                    relax(hx, hy, hk, rcx, rcy);
                    if (left) relax(hx, hy, hk, pcx, pcy);
                    if (right) relax(hx, hy, hk, ncx, ncy);
                }
            } else {
                constexpr int32_t kInf = 0x7FFFFFFF;
                const int32_t ki = ix * ix + iy * iy;
                const int32_t kr = up ? rcx * rcx + rcy * rcy : kInf;
                const int32_t kp = up && left ? pcx * pcx + pcy * pcy : kInf;
                const int32_t kn = up && right ? ncx * ncx + ncy * ncy : kInf;
                // first minimum of the up candidates, then of [own, that]: own wins ties
                int32_t ax = rcx, ay = rcy, ka = kr;
                if (kp < ka) { ax = pcx; ay = pcy; ka = kp; }
                if (kn < ka) { ax = ncx; ay = ncy; ka = kn; }
                const bool own = ki <= ka;
                const int32_t bx = own ? ix : ax, by = own ? iy : ay;
                // the left candidate comes after own (must be strictly shorter) and before the up ones
                const int32_t thr = own ? ki : ka + 1;
                const int32_t kl = left ? lcx * lcx + lcy * lcy : kInf;
                hx = kl < thr ? lcx : bx;
                hy = kl < thr ? lcy : by;
            }
            mx = active ? hx : mx;
            my = active ? hy : my;
            const uint32_t packed = pack(hx, hy);
            if (active) out[field_index(band, steps, (uint32_t)t, (uint32_t)lane)] = packed;
            if (active && publish) st_relaxed(my_boundary + i, packed);
        }
        if (__any_sync(0xFFFFFFFFu, failed)) {
            if (lane == 0) atomicOr(status + PDR_STATUS_PAD_ERROR, kErrTimeout);
            return;
        }
    }
}

struct FillParams {
    float* color;
    const float* snapshot;   // original colours; only when both sides exceed 12000
    const float* coverage;
    float* filled;
    const uint32_t* src_bits;
    const uint32_t* field;  // final offsets, band-major (final_index)
    uint32_t channels, words_per_row, margin, fill_unobserved, bands;
    int32_t W, H;
    unsigned long long margin2, limit2;
};

__device__ __forceinline__ bool is_source(const FillParams& P, uint32_t x, uint32_t y) {
    return (P.src_bits[(uint64_t)y * P.words_per_row + (x >> 5)] >> (x & 31)) & 1u;
}

// texture_padding.cpp:292-330 for one non-source texel: 0 skip, 1 fill, 2 covered but left unfilled.
__device__ __forceinline__ int fill_decision(const FillParams& P, uint32_t x, uint32_t y, uint64_t& src,
                                             bool& covered) {
    const uint64_t p = (uint64_t)y * (uint32_t)P.W + x;
    const uint32_t f = P.field[final_index(x, y, (uint32_t)P.W, P.bands)];
    const int32_t ox = unpack_x(f), oy = unpack_y(f);
    const int32_t d2 = ox * ox + oy * oy;
    if (d2 >= 2 * kFar * kFar) return 0;
    const int32_t sx = (int32_t)x + ox, sy = (int32_t)y + oy;
    if (sx < 0 || sy < 0 || sx >= P.W || sy >= P.H) return 0;
    src = (uint64_t)sy * (uint32_t)P.W + (uint32_t)sx;
    covered = P.coverage && P.coverage[p] > 0.5f;
    bool fill;
    if (!covered) fill = P.margin > 0 && (unsigned long long)d2 <= P.margin2;
    else fill = P.fill_unobserved && (unsigned long long)d2 <= P.limit2;
    return fill ? 1 : (covered ? 2 : 0);
}

// texture_padding.cpp:281-343. counters: [0] gutter, [1] unobserved, [2] remaining.
__global__ void __launch_bounds__(kStatThreads) pad_fill_kernel(FillParams P, const unsigned long long* stats,
                                                                const uint32_t* control,
                                                                unsigned long long* counters) {
    __shared__ unsigned long long red[kStatThreads / 32];
    if (control[2] != 0 || (stats[0] == 0 && stats[4] == 0)) return;
    const uint64_t n = (uint64_t)(uint32_t)P.W * (uint32_t)P.H;
    unsigned long long gutter = 0, unobserved = 0, remaining = 0;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t y = (uint32_t)(p / (uint32_t)P.W), x = (uint32_t)(p % (uint32_t)P.W);
        if (is_source(P, x, y)) continue;
        uint64_t s = 0;
        bool covered = false;
        const int d = fill_decision(P, x, y, s, covered);
        if (d == 0) continue;
        if (d == 2) {
            ++remaining;
            continue;
        }
        const float* from = P.color;
        uint32_t sx = (uint32_t)(s % (uint32_t)P.W), sy = (uint32_t)(s / (uint32_t)P.W);
        if (!is_source(P, sx, sy) && P.snapshot) {
            // The reference fills in raster order in place: a texel earlier than `limit` that it filled
            // holds its own fill colour, anything else still holds its original colour.
            uint64_t limit = p;
            for (uint64_t guard = 0; guard < n; ++guard) {
                if (is_source(P, sx, sy) || s >= limit) break;
                uint64_t next = 0;
                bool cov2 = false;
                if (fill_decision(P, sx, sy, next, cov2) != 1) break;
                limit = s;
                s = next;
                sx = (uint32_t)(s % (uint32_t)P.W);
                sy = (uint32_t)(s / (uint32_t)P.W);
            }
            from = is_source(P, sx, sy) ? P.color : P.snapshot;
        }
        for (uint32_t c = 0; c < P.channels; ++c) P.color[p * P.channels + c] = from[s * P.channels + c];
        if (P.channels == 4) P.color[p * 4 + 3] = 1.0f;
        P.filled[p] = 1.0f;
        if (covered) ++unobserved;
        else ++gutter;
    }
    const unsigned long long g = block_sum(gutter, red);
    if (threadIdx.x == 0 && g) atomicAdd(&counters[0], g);
    const unsigned long long u = block_sum(unobserved, red);
    if (threadIdx.x == 0 && u) atomicAdd(&counters[1], u);
    const unsigned long long r = block_sum(remaining, red);
    if (threadIdx.x == 0 && r) atomicAdd(&counters[2], r);
}

__global__ void pad_finish_kernel(unsigned long long* stats, const unsigned long long* counters) {
    stats[1] = counters[0];
    stats[2] += counters[1];
    stats[3] = counters[2];
    stats[4] += counters[0] + counters[1];
}

// ---- surface fill -----------------------------------------------------------------------------------

// (face, pixel) keys of measured texels; other texels get key T and sort last. Face ids beyond the mesh
// on covered texels are an error (texture_padding.cpp:117-119).
__global__ void surf_keys_kernel(const uint32_t* __restrict__ face_ids, const float* __restrict__ valid, uint64_t n,
                                 uint32_t T, uint32_t* __restrict__ keys, uint32_t* __restrict__ pixels,
                                 uint32_t* status) {
    bool bad = false;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t f = face_ids[p];
        uint32_t key = T;
        if (f != kNone) {
            if (f >= T) bad = true;
            else if (valid[p] >= 0.5f) key = f;
        }
        keys[p] = key;
        pixels[p] = (uint32_t)p;
    }
    if (__any_sync(0xFFFFFFFFu, bad) && (threadIdx.x & 31) == 0) atomicOr(status + PDR_STATUS_PAD_ERROR, kErrFaceRange);
}

__device__ __forceinline__ uint64_t lower_bound(const uint32_t* keys, uint64_t n, uint32_t v) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (keys[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// texture_padding.cpp:114-124,153-160: per-face sums in double in pixel order, then the mean.
__global__ void surf_means_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ pixels, uint64_t n,
                                  const float* __restrict__ color, uint32_t channels, uint32_t T,
                                  double* __restrict__ means, uint32_t* __restrict__ measured) {
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < T; f += gridDim.x * blockDim.x) {
        const uint64_t b = lower_bound(keys, n, f), e = lower_bound(keys, n, f + 1);
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (uint64_t k = b; k < e; ++k) {
            const uint64_t p = pixels[k];
            s0 += (double)color[p * channels];
            s1 += (double)color[p * channels + 1];
            s2 += (double)color[p * channels + 2];
        }
        const uint32_t count = (uint32_t)(e - b);
        if (count) {
            s0 /= count;
            s1 /= count;
            s2 /= count;
        }
        means[(uint64_t)f * 3] = s0;
        means[(uint64_t)f * 3 + 1] = s1;
        means[(uint64_t)f * 3 + 2] = s2;
        measured[f] = count != 0;
    }
}

// texture_padding.cpp:125-136: undirected edge keys, (face, slot) values.
__global__ void surf_edges_kernel(const uint32_t* __restrict__ idx, uint32_t T, unsigned long long* __restrict__ keys,
                                  uint32_t* __restrict__ slots, uint32_t* status) {
    bool bad = false;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < (uint64_t)T * 3;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t f = k / 3;
        const uint32_t e = (uint32_t)(k % 3);
        const uint32_t a = idx[f * 3 + e], b = idx[f * 3 + (e + 1) % 3];
        bad |= a == b;
        keys[k] = ((unsigned long long)min(a, b) << 32) | max(a, b);
        slots[k] = (uint32_t)k;
    }
    if (__any_sync(0xFFFFFFFFu, bad) && (threadIdx.x & 31) == 0) atomicOr(status + PDR_STATUS_PAD_ERROR, kErrDegenerate);
}

// texture_padding.cpp:140-151: pairs of equal keys are neighbours; more than two is non-manifold.
__global__ void surf_adjacency_kernel(const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ slots,
                                      uint64_t m, uint32_t* __restrict__ neighbours, uint32_t* status) {
    bool bad = false;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
        if (k > 0 && keys[k - 1] == keys[k]) continue;
        uint64_t e = k + 1;
        while (e < m && keys[e] == keys[k] && e - k <= 2) ++e;
        if (e - k > 2) {
            bad = true;
        } else if (e - k == 2) {
            neighbours[slots[k]] = slots[k + 1] / 3;
            neighbours[slots[k + 1]] = slots[k] / 3;
        }
    }
    if (__any_sync(0xFFFFFFFFu, bad) && (threadIdx.x & 31) == 0) atomicOr(status + PDR_STATUS_PAD_ERROR, kErrManifold);
}

constexpr int kBfsThreads = 1024;

// Ordered compaction of the kept values of [0, count) into out; returns the total (all threads).
template <typename Pred>
__device__ uint32_t block_compact(uint32_t count, Pred pred, uint32_t* out, uint32_t* warp_sums) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t total = 0;
    for (uint32_t base = 0; base < count; base += kBfsThreads) {
        const uint32_t k = base + threadIdx.x;
        uint32_t v = kNone;
        if (k < count) v = pred(k);
        const bool keep = v != kNone;
        const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, keep);
        const uint32_t before = __popc(ballot & ((1u << lane) - 1u));
        __syncthreads();
        if (lane == 0) warp_sums[warp] = __popc(ballot);
        __syncthreads();
        uint32_t offset = 0, chunk = 0;
        for (int w = 0; w < kBfsThreads / 32; ++w) {
            const uint32_t c = warp_sums[w];
            offset += w < warp ? c : 0;
            chunk += c;
        }
        if (keep) out[total + offset + before] = v;
        total += chunk;
    }
    __syncthreads();
    return total;
}

// texture_padding.cpp:152-171: multi-source BFS in the reference's FIFO order. stats[2] measured faces,
// stats[3] propagated faces.
__global__ void __launch_bounds__(kBfsThreads) surf_bfs_kernel(const uint32_t* __restrict__ neighbours,
                                                               const uint32_t* __restrict__ measured, uint32_t T,
                                                               uint32_t* sources, uint32_t* front_a, uint32_t* front_b,
                                                               uint32_t* best, const uint32_t* status,
                                                               unsigned long long* stats) {
    __shared__ uint32_t warp_sums[kBfsThreads / 32];
    if (status[PDR_STATUS_PAD_ERROR] & (kErrFaceRange | kErrDegenerate | kErrManifold)) return;
    uint32_t n = block_compact(
        T,
        [&](uint32_t f) {
            const bool m = measured[f] != 0;
            sources[f] = m ? f : kNone;
            return m ? f : kNone;
        },
        front_a, warp_sums);
    if (threadIdx.x == 0) stats[2] = n;
    unsigned long long propagated = 0;
    uint32_t* front = front_a;
    uint32_t* next = front_b;
    while (n > 0) {
        // the first (parent position, slot) reaching each unvisited face
        for (uint32_t k = threadIdx.x; k < 3 * n; k += kBfsThreads) {
            const uint32_t g = neighbours[(uint64_t)front[k / 3] * 3 + k % 3];
            if (g != kNone && sources[g] == kNone) atomicMin(&best[g], k);
        }
        __syncthreads();
        const uint32_t m = block_compact(
            3 * n,
            [&](uint32_t k) {
                const uint32_t parent = front[k / 3];
                const uint32_t g = neighbours[(uint64_t)parent * 3 + k % 3];
                if (g == kNone || sources[g] != kNone || best[g] != k) return kNone;
                sources[g] = sources[parent];
                return g;
            },
            next, warp_sums);
        propagated += m;
        n = m;
        uint32_t* tmp = front;
        front = next;
        next = tmp;
    }
    if (threadIdx.x == 0) stats[3] = propagated;
}

// texture_padding.cpp:172-183. stats[0] filled, stats[1] remaining.
__global__ void __launch_bounds__(kStatThreads) surf_fill_kernel(
    float* __restrict__ color, uint32_t channels, const float* __restrict__ valid,
    const uint32_t* __restrict__ face_ids, float* __restrict__ filled, uint64_t n, const uint32_t* __restrict__ sources,
    const double* __restrict__ means, const uint32_t* status, unsigned long long* stats) {
    __shared__ unsigned long long red[kStatThreads / 32];
    if (status[PDR_STATUS_PAD_ERROR] & (kErrFaceRange | kErrDegenerate | kErrManifold)) return;
    unsigned long long nfilled = 0, nremaining = 0;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t f = face_ids[p];
        if (f == kNone || valid[p] >= 0.5f) continue;
        const uint32_t s = sources[f];
        if (s == kNone) {
            ++nremaining;
            continue;
        }
        for (uint32_t c = 0; c < 3; ++c) color[p * channels + c] = (float)means[(uint64_t)s * 3 + c];
        if (channels == 4) color[p * 4 + 3] = 1.0f;
        filled[p] = 1.0f;
        ++nfilled;
    }
    const unsigned long long a = block_sum(nfilled, red);
    if (threadIdx.x == 0 && a) atomicAdd(&stats[0], a);
    const unsigned long long b = block_sum(nremaining, red);
    if (threadIdx.x == 0 && b) atomicAdd(&stats[1], b);
}

uint32_t stat_blocks(uint64_t work) {
    const uint64_t b = (work + kStatThreads - 1) / kStatThreads;
    return (uint32_t)(b < 152ull * 8 ? (b ? b : 1) : 152ull * 8);
}

struct PadLayout {
    size_t control, counters, bits, field, field2, boundary, snapshot, total;
};

PadLayout pad_layout(uint32_t W, uint32_t H, uint32_t C) {
    PadLayout L{};
    const size_t words = (size_t)((W + 31) / 32) * H, bands = (H + 31) / 32;
    size_t o = 0;
    L.control = o;
    o += align_up(4 * sizeof(uint32_t));
    L.counters = o;
    o += align_up(4 * sizeof(unsigned long long));
    L.bits = o;
    o += align_up(words * sizeof(uint32_t));
    const size_t field_words = bands * ((size_t)W + 62) * 32;
    L.field = o;
    o += align_up(field_words * sizeof(uint32_t));
    L.field2 = o;
    o += align_up(field_words * sizeof(uint32_t));
    L.boundary = o;
    o += align_up(2 * bands * W * sizeof(uint32_t));
    L.snapshot = o;
    if (W > (uint32_t)kFar && H > (uint32_t)kFar) o += align_up((size_t)W * H * C * sizeof(float));
    L.total = o;
    return L;
}

struct SurfLayout {
    size_t keys, pixels, keys_sorted, pixels_sorted, edge_keys, edge_keys_sorted, edge_slots, edge_slots_sorted,
        neighbours, means, measured, sources, front_a, front_b, best, cub, cub_bytes, total;
};

uint32_t key_bits(uint32_t v) {
    uint32_t b = 0;
    while (b < 32 && (v >> b) != 0) ++b;
    return b ? b : 1;
}

SurfLayout surf_layout(uint64_t n, uint32_t T) {
    SurfLayout L{};
    size_t a = 0, b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, (int64_t)n, 0, (int)key_bits(T));
    cub::DeviceRadixSort::SortPairs(nullptr, b, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (uint32_t*)nullptr, (uint32_t*)nullptr, (int64_t)T * 3, 0, 64);
    L.cub_bytes = a > b ? a : b;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t r = o;
        o += align_up(bytes);
        return r;
    };
    L.keys = take(n * 4);
    L.pixels = take(n * 4);
    L.keys_sorted = take(n * 4);
    L.pixels_sorted = take(n * 4);
    L.edge_keys = take((size_t)T * 3 * 8);
    L.edge_keys_sorted = take((size_t)T * 3 * 8);
    L.edge_slots = take((size_t)T * 3 * 4);
    L.edge_slots_sorted = take((size_t)T * 3 * 4);
    L.neighbours = take((size_t)T * 3 * 4);
    L.means = take((size_t)T * 3 * 8);
    L.measured = take((size_t)T * 4);
    L.sources = take((size_t)T * 4);
    L.front_a = take((size_t)T * 4);
    L.front_b = take((size_t)T * 4);
    L.best = take((size_t)T * 4);
    L.cub = take(L.cub_bytes);
    L.total = o;
    return L;
}

pdr_status check_pad_args(uint32_t width, uint32_t height, uint32_t channels, float threshold) {
    if (width == 0 || height == 0) return set_error(PDR_INVALID_ARGUMENT, "cannot pad an empty atlas");
    if (width > (uint32_t)kMaxSide || height > (uint32_t)kMaxSide)
        return set_error(PDR_INVALID_ARGUMENT, "atlas dimensions exceed the supported maximum");
    if (channels != 3 && channels != 4) return set_error(PDR_INVALID_ARGUMENT, "atlas color must have 3 or 4 channels");
    if (!(threshold > 0.0f) || threshold > 1.0f)
        return set_error(PDR_INVALID_ARGUMENT, "valid_threshold must be within (0, 1]");
    return PDR_OK;
}

}  // namespace
}  // namespace pdr

using namespace pdr;

extern "C" {

pdr_status pdr_pad_workspace_bytes(uint32_t width, uint32_t height, uint32_t channels, size_t* bytes) {
    if (!bytes) return set_error(PDR_INVALID_ARGUMENT, "pad workspace query needs an output");
    pdr_status st = check_pad_args(width, height, channels, 0.5f);
    if (st) return st;
    *bytes = pad_layout(width, height, channels).total;
    return PDR_OK;
}

pdr_status pdr_pad_texture_atlas(float* color, uint32_t channels, const float* valid_mask, const float* coverage_mask,
                                 float* filled_mask, uint32_t width, uint32_t height, uint32_t margin,
                                 uint32_t fill_unobserved, uint32_t maximum_fill_distance, float valid_threshold,
                                 void* workspace, size_t workspace_bytes, uint64_t* stats, uint32_t* status,
                                 void* stream) {
    pdr_status st = check_pad_args(width, height, channels, valid_threshold);
    if (st) return st;
    if (!color || !valid_mask || !filled_mask || !workspace || !stats || !status)
        return set_error(PDR_INVALID_ARGUMENT, "padding needs colour, masks, workspace, stats and status");
    const PadLayout L = pad_layout(width, height, channels);
    if (workspace_bytes < L.total) return set_error(PDR_INVALID_ARGUMENT, "pad workspace is smaller than required");
    const cudaStream_t s = (cudaStream_t)stream;
    char* ws = static_cast<char*>(workspace);
    uint32_t* control = reinterpret_cast<uint32_t*>(ws + L.control);
    unsigned long long* counters = reinterpret_cast<unsigned long long*>(ws + L.counters);
    uint32_t* bits = reinterpret_cast<uint32_t*>(ws + L.bits);
    uint32_t* field = reinterpret_cast<uint32_t*>(ws + L.field);
    uint32_t* boundary = reinterpret_cast<uint32_t*>(ws + L.boundary);
    const bool snapshot = width > (uint32_t)kFar && height > (uint32_t)kFar;
    const uint32_t wpr = (width + 31) / 32, bands = (height + 31) / 32;
    unsigned long long* st64 = reinterpret_cast<unsigned long long*>(stats);
    cudaError_t e = cudaMemsetAsync(stats, 0, 5 * sizeof(uint64_t), s);
    if (!e) e = cudaMemsetAsync(ws, 0, L.bits, s);  // control + counters
    if (!e) e = cudaMemsetAsync(boundary, 0x80, 2ull * bands * width * sizeof(uint32_t), s);
    if (e) return set_cuda_error(e, "pdr_pad_texture_atlas");
    const uint64_t words = (uint64_t)wpr * height;
    pad_classify_kernel<<<stat_blocks(words * 32), kStatThreads, 0, s>>>(valid_mask, coverage_mask, filled_mask, bits,
                                                                         wpr, width, height, valid_threshold, st64);
    uint32_t* field2 = reinterpret_cast<uint32_t*>(ws + L.field2);
    if (width > 4384 || height > 4384) {
        pad_sweep_kernel<false, true><<<bands, 32, 0, s>>>(bits, wpr, nullptr, field, boundary, control, status,
                                                           (int32_t)width, (int32_t)height);
        pad_sweep_kernel<true, true><<<bands, 32, 0, s>>>(bits, wpr, field, field2, boundary + (size_t)bands * width,
                                                          control, status, (int32_t)width, (int32_t)height);
    } else {
        pad_sweep_kernel<false, false><<<bands, 32, 0, s>>>(bits, wpr, nullptr, field, boundary, control, status,
                                                            (int32_t)width, (int32_t)height);
        pad_sweep_kernel<true, false><<<bands, 32, 0, s>>>(bits, wpr, field, field2, boundary + (size_t)bands * width,
                                                           control, status, (int32_t)width, (int32_t)height);
    }
    if (snapshot) {
        e = cudaMemcpyAsync(ws + L.snapshot, color, (size_t)width * height * channels * sizeof(float),
                            cudaMemcpyDeviceToDevice, s);
        if (e) return set_cuda_error(e, "pdr_pad_texture_atlas");
    }
    FillParams P{};
    P.color = color;
    P.snapshot = snapshot ? reinterpret_cast<const float*>(ws + L.snapshot) : nullptr;
    P.coverage = coverage_mask;
    P.filled = filled_mask;
    P.src_bits = bits;
    P.field = field2;
    P.bands = bands;
    P.channels = channels;
    P.words_per_row = wpr;
    P.margin = margin;
    P.fill_unobserved = fill_unobserved != 0;
    P.W = (int32_t)width;
    P.H = (int32_t)height;
    P.margin2 = (unsigned long long)margin * margin;
    P.limit2 = maximum_fill_distance == 0 ? ~0ull : (unsigned long long)maximum_fill_distance * maximum_fill_distance;
    pad_fill_kernel<<<stat_blocks((uint64_t)width * height), kStatThreads, 0, s>>>(P, st64, control, counters);
    pad_finish_kernel<<<1, 1, 0, s>>>(st64, counters);
    e = cudaGetLastError();
    return e ? set_cuda_error(e, "pdr_pad_texture_atlas") : PDR_OK;
}

pdr_status pdr_surface_fill_workspace_bytes(uint32_t width, uint32_t height, uint32_t triangle_count, size_t* bytes) {
    if (!bytes) return set_error(PDR_INVALID_ARGUMENT, "surface fill workspace query needs an output");
    if (width == 0 || height == 0 || triangle_count == 0)
        return set_error(PDR_INVALID_ARGUMENT, "surface fill requires mesh face IDs and a valid atlas");
    if (triangle_count >= kNone / 3) return set_error(PDR_INVALID_ARGUMENT, "surface fill has too many faces");
    if ((uint64_t)width * height > 0xFFFFFFFFull)
        return set_error(PDR_OVERFLOW, "surface fill atlas exceeds backend limits");
    *bytes = surf_layout((uint64_t)width * height, triangle_count).total;
    return PDR_OK;
}

pdr_status pdr_fill_texture_on_surface(float* color, uint32_t channels, const float* valid_mask,
                                       const uint32_t* face_ids, float* filled_mask, uint32_t width, uint32_t height,
                                       const uint32_t* indices, uint32_t triangle_count, void* workspace,
                                       size_t workspace_bytes, uint64_t* stats, uint32_t* status, void* stream) {
    size_t need = 0;
    pdr_status st = pdr_surface_fill_workspace_bytes(width, height, triangle_count, &need);
    if (st) return st;
    if (channels != 3 && channels != 4)
        return set_error(PDR_INVALID_ARGUMENT, "surface fill requires RGB or RGBA colours");
    if (!color || !valid_mask || !face_ids || !filled_mask || !indices || !workspace || !stats || !status)
        return set_error(PDR_INVALID_ARGUMENT, "surface fill needs colour, masks, face ids, indices and buffers");
    if (workspace_bytes < need) return set_error(PDR_INVALID_ARGUMENT, "surface fill workspace is smaller than required");
    const uint64_t n = (uint64_t)width * height;
    const uint32_t T = triangle_count;
    const SurfLayout L = surf_layout(n, T);
    const cudaStream_t s = (cudaStream_t)stream;
    char* ws = static_cast<char*>(workspace);
    auto u32 = [&](size_t off) { return reinterpret_cast<uint32_t*>(ws + off); };
    auto u64 = [&](size_t off) { return reinterpret_cast<unsigned long long*>(ws + off); };
    unsigned long long* st64 = reinterpret_cast<unsigned long long*>(stats);
    cudaError_t e = cudaMemsetAsync(stats, 0, 4 * sizeof(uint64_t), s);
    if (!e) e = cudaMemsetAsync(u32(L.neighbours), 0xFF, (size_t)T * 3 * 4, s);
    if (!e) e = cudaMemsetAsync(u32(L.best), 0xFF, (size_t)T * 4, s);
    if (e) return set_cuda_error(e, "pdr_fill_texture_on_surface");
    surf_keys_kernel<<<stat_blocks(n), kStatThreads, 0, s>>>(face_ids, valid_mask, n, T, u32(L.keys), u32(L.pixels),
                                                            status);
    size_t cub_bytes = L.cub_bytes;
    e = cub::DeviceRadixSort::SortPairs(ws + L.cub, cub_bytes, u32(L.keys), u32(L.keys_sorted), u32(L.pixels),
                                        u32(L.pixels_sorted), (int64_t)n, 0, (int)key_bits(T), s);
    if (e) return set_cuda_error(e, "pdr_fill_texture_on_surface");
    surf_means_kernel<<<(T + 255) / 256, 256, 0, s>>>(u32(L.keys_sorted), u32(L.pixels_sorted), n, color, channels, T,
                                                      reinterpret_cast<double*>(ws + L.means), u32(L.measured));
    surf_edges_kernel<<<stat_blocks((uint64_t)T * 3), kStatThreads, 0, s>>>(indices, T, u64(L.edge_keys),
                                                                           u32(L.edge_slots), status);
    cub_bytes = L.cub_bytes;
    e = cub::DeviceRadixSort::SortPairs(ws + L.cub, cub_bytes, u64(L.edge_keys), u64(L.edge_keys_sorted),
                                        u32(L.edge_slots), u32(L.edge_slots_sorted), (int64_t)T * 3, 0, 64, s);
    if (e) return set_cuda_error(e, "pdr_fill_texture_on_surface");
    surf_adjacency_kernel<<<stat_blocks((uint64_t)T * 3), kStatThreads, 0, s>>>(
        u64(L.edge_keys_sorted), u32(L.edge_slots_sorted), (uint64_t)T * 3, u32(L.neighbours), status);
    surf_bfs_kernel<<<1, kBfsThreads, 0, s>>>(u32(L.neighbours), u32(L.measured), T, u32(L.sources), u32(L.front_a),
                                              u32(L.front_b), u32(L.best), status, st64);
    surf_fill_kernel<<<stat_blocks(n), kStatThreads, 0, s>>>(color, channels, valid_mask, face_ids, filled_mask, n,
                                                            u32(L.sources), reinterpret_cast<double*>(ws + L.means),
                                                            status, st64);
    e = cudaGetLastError();
    return e ? set_cuda_error(e, "pdr_fill_texture_on_surface") : PDR_OK;
}

}  // extern "C"

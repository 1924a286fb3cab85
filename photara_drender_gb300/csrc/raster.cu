// Tile binning and rasterization (forward and backward) for many views in one launch.
//
// Reference path: src/rasterizer.cpp:61-138 (CPU tile binning), shaders/rasterize_forward.hlsl,
// shaders/rasterize_backward.hlsl + reduce_vertex_gradients.hlsl.
//
// Layout in HBM: clip positions [views][V][4] fp32, indices [T][3] u32 (shared by all views),
// viewports [views][4], tile bins as one CSR over (view, tile) keys: offsets [views*tiles+1]
// and triangle ids sorted ascending inside every tile, raster/derivatives [views][H][W][4].
#include <cuda_runtime.h>
#include <float.h>

#include <algorithm>

#include "pdr_common.cuh"
#include "pdr_internal.h"
#include "bin_rect.cuh"
#include "raster_tile.cuh"

namespace pdr {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr uint32_t kScanBlock = kScanThreads * kScanItems;
constexpr uint32_t kSmallSort = 1024;   // tiles up to this many entries sort in one warp
constexpr uint32_t kWindowBits = 8192 * 32;  // id window of the large-tile bitmap sort (32 KB)

// Pass 1: per (view, triangle) tile rectangle and per-tile counts (warp-aggregated when the
// lanes of a warp land in the same single tile).
__global__ void __launch_bounds__(256, 6)  // 40 registers: 48 warps per SM for the gathers and atomics
bin_count_kernel(const float4* __restrict__ clip, uint32_t V, const uint3* __restrict__ idx,
                                 uint32_t T, uint32_t W, uint32_t H, const float4* __restrict__ viewports,
                                 uint32_t tcx, uint32_t tiles, TriRect* __restrict__ rects,
                                 uint32_t* __restrict__ counts, uint32_t tile_w, uint32_t tile_h) {
    const uint32_t view = blockIdx.y;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = t < T;
    TriRect r{kNoRect, 0};
    if (live) {
        const uint3 vi = idx[t];
        if (vi.x < V && vi.y < V && vi.z < V)
            r = triangle_tile_rect(clip + (size_t)view * V, vi, W, H, viewports[view], tile_w, tile_h);
        rects[(size_t)view * T + t] = r;
    }
    uint32_t* cnt = counts + (size_t)view * tiles;
    const bool has = live && r.x != kNoRect;
    const uint32_t tx0 = r.x & 0xffffu, tx1 = r.x >> 16, ty0 = r.y & 0xffffu, ty1 = r.y >> 16;
    const bool single = has && tx0 == tx1 && ty0 == ty1;
    const uint32_t key = single ? ty0 * tcx + tx0 : 0xffffffffu - (threadIdx.x & 31u);
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (single && (__ffs(peers) - 1) == (int)(threadIdx.x & 31u)) atomicAdd(cnt + key, (uint32_t)__popc(peers));
    if (has && !single) {
        for (uint32_t ty = ty0; ty <= ty1; ++ty)
            for (uint32_t tx = tx0; tx <= tx1; ++tx) atomicAdd(cnt + ty * tcx + tx, 1u);
    }
}

// Exclusive scan over the (view, tile) counts in three phases.
// Block-wide exclusive scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ unsigned long long block_exclusive_u64(unsigned long long v, unsigned long long* total) {
    __shared__ unsigned long long warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long n = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += n;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        unsigned long long s = lane < nw ? warp_sums[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long n = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += n;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    const unsigned long long warp_prefix = warp > 0 ? warp_sums[warp - 1] : 0ull;
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + inc - v;
}

__global__ void scan_local_kernel(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ out,
                                  unsigned long long* __restrict__ block_sums) {
    const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    unsigned long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? in[base + i] : 0u;
        s += v[i];
    }
    unsigned long long total;
    unsigned long long pre = block_exclusive_u64(s, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = (uint32_t)pre;
        pre += v[i];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void scan_blocks_kernel(unsigned long long* __restrict__ block_sums, uint32_t nblocks,
                                   uint32_t* __restrict__ out, uint32_t n, uint32_t* __restrict__ status,
                                   unsigned long long capacity) {
    // single block: exclusive scan of the block totals, chunk by chunk
    unsigned long long carry = 0;
    for (uint32_t c = 0; c < nblocks; c += blockDim.x) {
        const uint32_t i = c + threadIdx.x;
        const unsigned long long v = i < nblocks ? block_sums[i] : 0ull;
        unsigned long long total;
        const unsigned long long pre = block_exclusive_u64(v, &total);
        if (i < nblocks) block_sums[i] = carry + pre;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const bool overflow = carry > 0xffffffffull;
        out[n] = overflow ? 0xffffffffu : (uint32_t)carry;
        status[kStatusTotal] = overflow ? 0xffffffffu : (uint32_t)carry;
        status[kStatusTotalHi] = (uint32_t)(carry >> 32);
        status[kStatusOverflow] = (overflow || carry > capacity) ? 1u : 0u;
        status[kStatusLargeTiles] = 0u;
    }
}

__global__ void scan_add_kernel(uint32_t* __restrict__ out, uint32_t n, const unsigned long long* __restrict__ block_sums,
                                uint32_t* __restrict__ cursor) {
    const size_t base = (size_t)blockIdx.x * kScanBlock;
    const uint32_t add = (uint32_t)block_sums[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < kScanBlock; i += blockDim.x) {
        const size_t k = base + i;
        if (k < n) {
            const uint32_t v = out[k] + add;
            out[k] = v;
            cursor[k] = v;
        }
    }
}

// Pass 2: scatter triangle ids into their tiles (unordered inside a tile).
__global__ void bin_fill_kernel(const TriRect* __restrict__ rects, uint32_t T, uint32_t tcx, uint32_t tiles,
                                uint32_t* __restrict__ cursor, uint32_t* __restrict__ unsorted,
                                unsigned long long capacity) {
    const uint32_t view = blockIdx.y;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = t < T;
    TriRect r{kNoRect, 0};
    if (live) r = rects[(size_t)view * T + t];
    uint32_t* cur = cursor + (size_t)view * tiles;
    const bool has = live && r.x != kNoRect;
    const uint32_t tx0 = r.x & 0xffffu, tx1 = r.x >> 16, ty0 = r.y & 0xffffu, ty1 = r.y >> 16;
    const bool single = has && tx0 == tx1 && ty0 == ty1;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t key = single ? ty0 * tcx + tx0 : 0xffffffffu - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (single) {
        const int leader = __ffs(peers) - 1;
        uint32_t slot = 0;
        if ((int)lane == leader) slot = atomicAdd(cur + key, (uint32_t)__popc(peers));
        slot = __shfl_sync(peers, slot, leader);
        slot += __popc(peers & ((1u << lane) - 1u));
        if (slot < capacity) unsorted[slot] = t;
    }
    if (has && !single) {
        for (uint32_t ty = ty0; ty <= ty1; ++ty)
            for (uint32_t tx = tx0; tx <= tx1; ++tx) {
                const uint32_t slot = atomicAdd(cur + ty * tcx + tx, 1u);
                if (slot < capacity) unsorted[slot] = t;
            }
    }
}

// Pass 3a: sort every tile with at most kSmallSort entries inside one warp (bitonic in shared
// memory); larger tiles are queued for pass 3b.
__global__ void bin_sort_small_kernel(const uint32_t* __restrict__ offsets, uint32_t segments,
                                      const uint32_t* __restrict__ unsorted, uint32_t* __restrict__ sorted,
                                      uint32_t* __restrict__ large_queue, uint32_t* __restrict__ status,
                                      unsigned long long capacity) {
    __shared__ uint32_t buf[8][kSmallSort];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t seg = blockIdx.x * 8 + warp;
    if (seg >= segments) return;
    const uint32_t b = offsets[seg];
    uint32_t e = offsets[seg + 1];
    if (e > capacity) e = (uint32_t)capacity;
    if (b >= e) return;
    const uint32_t n = e - b;
    if (n > kSmallSort) {
        if (lane == 0) {
            const uint32_t q = atomicAdd(status + kStatusLargeTiles, 1u);
            large_queue[q] = seg;
        }
        return;
    }
    if (n <= 32) {
        const uint32_t v = lane < n ? unsorted[b + lane] : 0xffffffffu;
        uint32_t rank = 0;
        for (uint32_t j = 0; j < 32; ++j) {
            const uint32_t o = __shfl_sync(0xffffffffu, v, j);
            rank += (o < v) ? 1u : 0u;
        }
        if (lane < n) sorted[b + rank] = v;
        return;
    }
    uint32_t m = 64;
    while (m < n) m <<= 1;
    uint32_t* s = buf[warp];
    for (uint32_t i = lane; i < m; i += 32) s[i] = i < n ? unsorted[b + i] : 0xffffffffu;
    __syncwarp();
    for (uint32_t k = 2; k <= m; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < m; i += 32) {
                const uint32_t l = i ^ j;
                if (l > i) {
                    const uint32_t a = s[i], c = s[l];
                    const bool up = (i & k) == 0;
                    if ((a > c) == up) {
                        s[i] = c;
                        s[l] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
    for (uint32_t i = lane; i < n; i += 32) sorted[b + i] = s[i];
}

// Pass 3b: tiles with more than kSmallSort entries. Triangle ids inside a tile are distinct, so a
// bitmap over an id window orders them; windows ascend over [min id, max id] of the tile.
__global__ void bin_sort_large_kernel(const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ unsorted,
                                      uint32_t* __restrict__ sorted, const uint32_t* __restrict__ large_queue,
                                      const uint32_t* __restrict__ status, unsigned long long capacity) {
    __shared__ uint32_t bitmap[kWindowBits / 32];
    __shared__ unsigned int lo_s, hi_s;
    const uint32_t count = status[kStatusLargeTiles];
    for (uint32_t q = blockIdx.x; q < count; q += gridDim.x) {
        const uint32_t seg = large_queue[q];
        const uint32_t b = offsets[seg];
        uint32_t e = offsets[seg + 1];
        if (e > capacity) e = (uint32_t)capacity;
        if (threadIdx.x == 0) {
            lo_s = 0xffffffffu;
            hi_s = 0u;
        }
        __syncthreads();
        uint32_t lo = 0xffffffffu, hi = 0u;
        for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
            const uint32_t v = unsorted[i];
            lo = v < lo ? v : lo;
            hi = v > hi ? v : hi;
        }
        atomicMin(&lo_s, lo);
        atomicMax(&hi_s, hi);
        __syncthreads();
        const uint32_t first = lo_s, last = hi_s;
        uint32_t written = 0;
        for (unsigned long long w0 = first; w0 <= last; w0 += kWindowBits) {
            for (uint32_t i = threadIdx.x; i < kWindowBits / 32; i += blockDim.x) bitmap[i] = 0u;
            __syncthreads();
            for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
                const unsigned long long v = unsorted[i];
                if (v >= w0 && v < w0 + kWindowBits) {
                    const uint32_t o = (uint32_t)(v - w0);
                    atomicOr(&bitmap[o >> 5], 1u << (o & 31u));
                }
            }
            __syncthreads();
            // each thread owns a contiguous run of words
            const uint32_t words = kWindowBits / 32;
            const uint32_t per = (words + blockDim.x - 1) / blockDim.x;
            const uint32_t w_begin = threadIdx.x * per;
            uint32_t cnt = 0;
            for (uint32_t w = w_begin; w < w_begin + per && w < words; ++w) cnt += __popc(bitmap[w]);
            unsigned long long total;
            const uint32_t pre = (uint32_t)block_exclusive_u64(cnt, &total);
            uint32_t outp = b + written + pre;
            for (uint32_t w = w_begin; w < w_begin + per && w < words; ++w) {
                uint32_t bits = bitmap[w];
                while (bits) {
                    const int bit = __ffs(bits) - 1;
                    bits &= bits - 1;
                    sorted[outp++] = (uint32_t)(w0 + w * 32u + (uint32_t)bit);
                }
            }
            written += (uint32_t)total;
            __syncthreads();
        }
        __syncthreads();
    }
}

// ---- rasterize forward: shaders/rasterize_forward.hlsl:45-175 ----------------------------
//
// One CTA per (view, TW x TH tile) running raster_tile (raster_tile.cuh) over the tile's bin, CHUNK
// triangles staged at a time. pdr_bin_tiles' bins are the reference's 16x16 tiles; the fused render
// may bin with another tile shape and stage depth (the result is the same: a pixel's candidates are
// the triangles whose bounding box holds it, whatever the tiles).

constexpr int kRasterThreads = 256;  // the default: one 16x16 tile per CTA

// true when tile list [b, e) lost entries to the capacity, or the list offsets overflowed u32
__device__ __forceinline__ bool tile_list_cut(uint32_t b, uint32_t e, unsigned long long capacity,
                                              const uint32_t* __restrict__ status) {
    return e > capacity || b > e || (status && status[kStatusTotalHi] != 0u);
}

template <bool kDeriv, bool kShade, int TW = kTile, int TH = kTile, int CHUNK = kRasterThreads>
__global__ void __launch_bounds__(TW * TH, 1280 / (TW * TH))  // 48 registers: 40 warps per SM
raster_forward_kernel(const float4* __restrict__ clip_all, uint32_t V, const uint3* __restrict__ idx,
                      uint32_t T, uint32_t W, uint32_t H, const float4* __restrict__ viewports, uint32_t cull,
                      uint32_t tcx, uint32_t tiles, const uint32_t* __restrict__ offsets,
                      const uint32_t* __restrict__ list, unsigned long long capacity, float4* __restrict__ raster,
                      float4* __restrict__ deriv, ShadeArgs shade, const uint32_t* __restrict__ status) {
    const uint32_t view = blockIdx.y;
    const uint32_t tile = blockIdx.x;
    const size_t P = (size_t)W * H;
    RasterView v;
    v.clip = clip_all + (size_t)view * V;
    v.idx = idx;
    v.V = V;
    v.T = T;
    v.W = W;
    v.H = H;
    v.cull = cull;
    v.vp = viewports[view];
    v.raster = raster + view * P;
    v.deriv = kDeriv ? deriv + view * P : nullptr;
    v.shade = shade;
    if (kShade) {
        if (shade.attr_out) v.shade.attr_out = shade.attr_out + view * P * shade.A;
        if (shade.uv_out) v.shade.uv_out = shade.uv_out + view * P;
        if (shade.sampled) v.shade.sampled = shade.sampled + view * P;
        if (shade.sdiff) v.shade.sdiff = shade.sdiff + view * P * 2;
    }
    const uint32_t seg = view * tiles + tile;
    const uint32_t b = offsets[seg];
    const uint32_t e = offsets[seg + 1];
    // a tile whose list did not fit the capacity is left to raster_overflow_kernel
    if (tile_list_cut(b, e, capacity, status)) return;
    raster_tile<kDeriv, kShade, TW, TH, CHUNK>(v, tile % tcx, tile / tcx, list, b, e);
}

// One tile whose list was cut, rasterized from all triangles with the binning rule.
template <bool kDeriv, bool kShade, int TW, int TH, int CHUNK>
__device__ __forceinline__ void raster_cut_tile(const float4* __restrict__ clip_all, uint32_t V,
                                                const uint3* __restrict__ idx, uint32_t T, uint32_t W, uint32_t H,
                                                const float4* __restrict__ viewports, uint32_t cull, uint32_t tcx,
                                                uint32_t tiles, uint32_t seg, size_t P, float4* __restrict__ raster,
                                                float4* __restrict__ deriv, const ShadeArgs& shade) {
    {
        const uint32_t view = seg / tiles, tile = seg % tiles;
        RasterView v;
        v.clip = clip_all + (size_t)view * V;
        v.idx = idx;
        v.V = V;
        v.T = T;
        v.W = W;
        v.H = H;
        v.cull = cull;
        v.vp = viewports[view];
        v.raster = raster + view * P;
        v.deriv = kDeriv ? deriv + view * P : nullptr;
        v.shade = shade;
        if (kShade) {
            if (shade.attr_out) v.shade.attr_out = shade.attr_out + view * P * shade.A;
            if (shade.uv_out) v.shade.uv_out = shade.uv_out + view * P;
            if (shade.sampled) v.shade.sampled = shade.sampled + view * P;
            if (shade.sdiff) v.shade.sdiff = shade.sdiff + view * P * 2;
        }
        raster_tile<kDeriv, kShade, TW, TH, CHUNK, true>(v, tile % tcx, tile / tcx, nullptr, 0u, T);
    }
}

// The tiles whose lists did not fit the tile-list capacity (or whose offsets overflowed u32), each
// rasterized from all triangles with the binning rule: the result is the one a sufficient list gives,
// only slower, so no caller has to wait for the entry count before rasterizing. Launched after
// raster_forward_kernel with a few CTAs per SM that walk all tiles; when nothing overflowed every CTA
// only reads offsets.
template <bool kDeriv, bool kShade, int TW = kTile, int TH = kTile, int CHUNK = kRasterThreads>
__global__ void __launch_bounds__(TW * TH)
raster_overflow_kernel(const float4* __restrict__ clip_all, uint32_t V, const uint3* __restrict__ idx, uint32_t T,
                       uint32_t W, uint32_t H, const float4* __restrict__ viewports, uint32_t cull, uint32_t tcx,
                       uint32_t tiles, uint32_t views, const uint32_t* __restrict__ offsets,
                       unsigned long long capacity, float4* __restrict__ raster, float4* __restrict__ deriv,
                       ShadeArgs shade, const uint32_t* __restrict__ status) {
    const size_t P = (size_t)W * H;
    constexpr uint32_t kThreads = TW * TH;
    __shared__ uint32_t cut_tiles[kThreads];
    __shared__ uint32_t cut_count;
    const uint32_t total = tiles * views;
    // each pass checks kThreads tiles at once (one per thread) and rasterizes the cut ones
    for (uint32_t base = blockIdx.x * kThreads; base < total; base += gridDim.x * kThreads) {
        if (threadIdx.x == 0) cut_count = 0;
        __syncthreads();
        const uint32_t mine = base + threadIdx.x;
        const bool cut = mine < total && tile_list_cut(offsets[mine], offsets[mine + 1], capacity, status);
        if (cut) cut_tiles[atomicAdd(&cut_count, 1u)] = mine;
        __syncthreads();
        const uint32_t n = cut_count;
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t seg = cut_tiles[i];
            raster_cut_tile<kDeriv, kShade, TW, TH, CHUNK>(clip_all, V, idx, T, W, H, viewports, cull, tcx, tiles,
                                                           seg, P, raster, deriv, shade);
            __syncthreads();  // the tile routine's shared memory is reused by the next tile
        }
    }
}


// ---- rasterize backward: shaders/rasterize_backward.hlsl:36-158 -------------------------
// One thread per pixel. A pixel contributes to triangle t exactly when the reference's
// per-triangle loop would visit it: raster id == t+1, inside t's clamped pixel bounds
// (rasterize_backward.hlsl:78-90) and a non-zero (u, v) gradient. Corner sums use atomics.
// With near-plane clipping (near != 0) a triangle with a vertex at w <= 1e-8, which the reference
// never visits, owns the pixels the clipped raster gave it and is visited on all of them (its
// projected bounds do not exist); every other triangle keeps the reference's rule.
__global__ void raster_backward_kernel(const float4* __restrict__ clip_all, uint32_t V, const uint3* __restrict__ idx,
                                       uint32_t T, uint32_t W, uint32_t H, const float4* __restrict__ viewports,
                                       const float4* __restrict__ raster, const float4* __restrict__ grad_raster,
                                       float* __restrict__ grad_clip, uint32_t near) {
    const uint32_t view = blockIdx.y;
    const size_t P = (size_t)W * H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const float rw = raster[pix].w;
    const uint32_t id = raster_id(rw);
    if (id == 0 || id > T) return;
    const float4 g = grad_raster[pix];
    if (g.x == 0.0f && g.y == 0.0f) return;
    const uint3 vi = idx[id - 1];
    if (vi.x >= V || vi.y >= V || vi.z >= V) return;
    const float4* __restrict__ clip = clip_all + (size_t)view * V;
    const float4 p0 = clip[vi.x], p1 = clip[vi.y], p2 = clip[vi.z];
    const bool behind = p0.w <= 1e-8f || p1.w <= 1e-8f || p2.w <= 1e-8f;
    if (behind && !near) return;
    const float4 vp = viewports[view];
    const uint32_t x = (uint32_t)(p % W), y = (uint32_t)(p / W);
    if (!behind) {
        const float s0x = p0.x / p0.w, s0y = p0.y / p0.w;
        const float s1x = p1.x / p1.w, s1y = p1.y / p1.w;
        const float s2x = p2.x / p2.w, s2y = p2.y / p2.w;
        const float mnx = fminf(s0x, fminf(s1x, s2x)), mny = fminf(s0y, fminf(s1y, s2y));
        const float mxx = fmaxf(s0x, fmaxf(s1x, s2x)), mxy = fmaxf(s0y, fmaxf(s1y, s2y));
        const int32_t x0 = clampi(f2i_sat(floorf((mnx * 0.5f + 0.5f) * vp.z + vp.x)), 0, (int32_t)W);
        const int32_t x1 = clampi(f2i_sat(ceilf((mxx * 0.5f + 0.5f) * vp.z + vp.x)), 0, (int32_t)W);
        const int32_t y0 = clampi(f2i_sat(floorf((mny * 0.5f + 0.5f) * vp.w + vp.y)), 0, (int32_t)H);
        const int32_t y1 = clampi(f2i_sat(ceilf((mxy * 0.5f + 0.5f) * vp.w + vp.y)), 0, (int32_t)H);
        if ((int32_t)x < x0 || (int32_t)x >= x1 || (int32_t)y < y0 || (int32_t)y >= y1) return;
    }
    const float sx = sample_ndc(x, vp.x, vp.z);
    const float sy = sample_ndc(y, vp.y, vp.w);
    const float q0x = p0.x - sx * p0.w, q0y = p0.y - sy * p0.w;
    const float q1x = p1.x - sx * p1.w, q1y = p1.y - sy * p1.w;
    const float q2x = p2.x - sx * p2.w, q2y = p2.y - sy * p2.w;
    const float area = cross2(q1x, q1y, q2x, q2y) + cross2(q2x, q2y, q0x, q0y) + cross2(q0x, q0y, q1x, q1y);
    if (fabsf(area) <= 1e-12f) return;
    const float eps = area >= 0.0f ? 1e-6f : -1e-6f;
    const float inv = 1.0f / (area + eps);
    const float a0 = cross2(q1x, q1y, q2x, q2y);
    const float a1 = cross2(q2x, q2y, q0x, q0y);
    const float b0 = a0 * inv, b1 = a1 * inv;
    const float gb0 = g.x * inv, gb1 = g.y * inv;
    const float gc = gb0 * b0 + gb1 * b1;
    const float g0x = gc * (q2y - q1y) - gb1 * q2y;
    const float g1x = gc * (q0y - q2y) + gb0 * q2y;
    const float g2x = gc * (q1y - q0y) - gb0 * q1y + gb1 * q0y;
    const float g0y = gc * (q1x - q2x) + gb1 * q2x;
    const float g1y = gc * (q2x - q0x) - gb0 * q2x;
    const float g2y = gc * (q0x - q1x) + gb0 * q1x - gb1 * q0x;
    float* gv = grad_clip + (size_t)view * V * 4;
    atomicAdd(gv + (size_t)vi.x * 4 + 0, g0x);
    atomicAdd(gv + (size_t)vi.x * 4 + 1, g0y);
    atomicAdd(gv + (size_t)vi.x * 4 + 3, -sx * g0x - sy * g0y);
    atomicAdd(gv + (size_t)vi.y * 4 + 0, g1x);
    atomicAdd(gv + (size_t)vi.y * 4 + 1, g1y);
    atomicAdd(gv + (size_t)vi.y * 4 + 3, -sx * g1x - sy * g1y);
    atomicAdd(gv + (size_t)vi.z * 4 + 0, g2x);
    atomicAdd(gv + (size_t)vi.z * 4 + 1, g2y);
    atomicAdd(gv + (size_t)vi.z * 4 + 3, -sx * g2x - sy * g2y);
}

}  // namespace

// ---- host launchers -----------------------------------------------------------------------

size_t bins_workspace_bytes(uint32_t views, uint32_t T, uint32_t W, uint32_t H, unsigned long long capacity,
                            uint32_t tile_w, uint32_t tile_h) {
    const size_t tiles = (size_t)((W + tile_w - 1) / tile_w) * ((H + tile_h - 1) / tile_h);
    const size_t segs = tiles * views;
    const size_t nblocks = (segs + 1 + kScanBlock - 1) / kScanBlock;
    size_t bytes = 0;
    bytes += align_up((size_t)views * T * sizeof(TriRect));  // rects
    bytes += align_up((segs + 1) * sizeof(uint32_t));          // counts
    bytes += align_up((segs + 1) * sizeof(uint32_t));          // cursor
    bytes += align_up(nblocks * sizeof(unsigned long long));   // scan block sums
    bytes += align_up(segs * sizeof(uint32_t));                // large-tile queue
    bytes += align_up((size_t)capacity * sizeof(uint32_t));    // unsorted list
    return bytes;
}

cudaError_t launch_scan_counts(const uint32_t* counts, size_t segs, uint32_t* offsets, unsigned long long* block_sums,
                               uint32_t* cursor, uint32_t* status, unsigned long long capacity, cudaStream_t stream) {
    const uint32_t nblocks = (uint32_t)((segs + 1 + kScanBlock - 1) / kScanBlock);
    scan_local_kernel<<<nblocks, kScanThreads, 0, stream>>>(counts, (uint32_t)segs, offsets, block_sums);
    scan_blocks_kernel<<<1, kScanThreads, 0, stream>>>(block_sums, nblocks, offsets, (uint32_t)segs, status, capacity);
    scan_add_kernel<<<nblocks, kScanThreads, 0, stream>>>(offsets, (uint32_t)segs, block_sums, cursor);
    return cudaGetLastError();
}

size_t scan_block_count(size_t segs) { return (segs + 1 + kScanBlock - 1) / kScanBlock; }

cudaError_t launch_bin_tiles(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                             uint32_t W, uint32_t H, const float* viewports, uint32_t* offsets, uint32_t* list,
                             unsigned long long capacity, void* workspace, uint32_t* status, cudaStream_t stream,
                             bool sorted, uint32_t tile_w, uint32_t tile_h) {
    const uint32_t tcx = (W + tile_w - 1) / tile_w, tcy = (H + tile_h - 1) / tile_h;
    const uint32_t tiles = tcx * tcy;
    const size_t segs = (size_t)tiles * views;
    const uint32_t nblocks = (uint32_t)((segs + 1 + kScanBlock - 1) / kScanBlock);
    char* ws = static_cast<char*>(workspace);
    TriRect* rects = reinterpret_cast<TriRect*>(ws);
    ws += align_up((size_t)views * T * sizeof(TriRect));
    uint32_t* counts = reinterpret_cast<uint32_t*>(ws);
    ws += align_up((segs + 1) * sizeof(uint32_t));
    uint32_t* cursor = reinterpret_cast<uint32_t*>(ws);
    ws += align_up((segs + 1) * sizeof(uint32_t));
    unsigned long long* block_sums = reinterpret_cast<unsigned long long*>(ws);
    ws += align_up((size_t)nblocks * sizeof(unsigned long long));
    uint32_t* large_queue = reinterpret_cast<uint32_t*>(ws);
    ws += align_up(segs * sizeof(uint32_t));
    uint32_t* unsorted = reinterpret_cast<uint32_t*>(ws);

    cudaError_t err = cudaMemsetAsync(counts, 0, (segs + 1) * sizeof(uint32_t), stream);
    if (err != cudaSuccess) return err;
    const dim3 tgrid((T + 255) / 256, views);
    bin_count_kernel<<<tgrid, 256, 0, stream>>>(reinterpret_cast<const float4*>(clip), V,
                                                reinterpret_cast<const uint3*>(idx), T, W, H,
                                                reinterpret_cast<const float4*>(viewports), tcx, tiles, rects, counts,
                                                tile_w, tile_h);
    scan_local_kernel<<<nblocks, kScanThreads, 0, stream>>>(counts, (uint32_t)segs, offsets, block_sums);
    scan_blocks_kernel<<<1, kScanThreads, 0, stream>>>(block_sums, nblocks, offsets, (uint32_t)segs, status, capacity);
    scan_add_kernel<<<nblocks, kScanThreads, 0, stream>>>(offsets, (uint32_t)segs, block_sums, cursor);
    bin_fill_kernel<<<tgrid, 256, 0, stream>>>(rects, T, tcx, tiles, cursor, sorted ? unsorted : list, capacity);
    if (!sorted) return cudaGetLastError();  // each tile's triangles stay in arrival order
    bin_sort_small_kernel<<<(uint32_t)((segs + 7) / 8), 256, 0, stream>>>(offsets, (uint32_t)segs, unsorted, list,
                                                                           large_queue, status, capacity);
    bin_sort_large_kernel<<<num_sms() * 2, 512, 0, stream>>>(offsets, unsorted, list, large_queue, status, capacity);
    return cudaGetLastError();
}

namespace {

template <int TW, int TH, int CHUNK>
cudaError_t launch_raster_config(const float4* c4, uint32_t views, uint32_t V, const uint3* i3, uint32_t T, uint32_t W,
                                 uint32_t H, const float4* v4, uint32_t cull, const uint32_t* offsets,
                                 const uint32_t* list, unsigned long long capacity, float4* r4, float4* d4,
                                 const ShadeArgs& sa, bool shade, const uint32_t* status, cudaStream_t stream) {
    const uint32_t tcx = (W + TW - 1) / TW, tcy = (H + TH - 1) / TH;
    const uint32_t tiles = tcx * tcy;
    const dim3 grid(tiles, views);
    constexpr int kThreads = TW * TH;
#define PDR_RASTER_MAIN(D, S, DP)                                                                                  \
    raster_forward_kernel<D, S, TW, TH, CHUNK><<<grid, kThreads, 0, stream>>>(c4, V, i3, T, W, H, v4, cull, tcx,   \
                                                                              tiles, offsets, list, capacity, r4,  \
                                                                              DP, sa, status)
    if (shade) {
        if (d4) PDR_RASTER_MAIN(true, true, d4); else PDR_RASTER_MAIN(false, true, nullptr);
    } else {
        if (d4) PDR_RASTER_MAIN(true, false, d4); else PDR_RASTER_MAIN(false, false, nullptr);
    }
#undef PDR_RASTER_MAIN
    // after the main launch: the tiles it skipped because their lists were cut
    const unsigned overflow_blocks = (unsigned)std::min<uint64_t>((uint64_t)tiles * views, (uint64_t)num_sms() * 4u);
#define PDR_RASTER_OVERFLOW(D, S, DP)                                                                              \
    raster_overflow_kernel<D, S, TW, TH, CHUNK><<<overflow_blocks, kThreads, 0, stream>>>(                         \
        c4, V, i3, T, W, H, v4, cull, tcx, tiles, views, offsets, capacity, r4, DP, sa, status)
    if (shade) {
        if (d4) PDR_RASTER_OVERFLOW(true, true, d4); else PDR_RASTER_OVERFLOW(false, true, nullptr);
    } else {
        if (d4) PDR_RASTER_OVERFLOW(true, false, d4); else PDR_RASTER_OVERFLOW(false, false, nullptr);
    }
#undef PDR_RASTER_OVERFLOW
    return cudaGetLastError();
}

}  // namespace

bool raster_config_supported(uint32_t tile_w, uint32_t tile_h, uint32_t chunk) {
    return (tile_w == 16 && tile_h == 16 && (chunk == 256 || chunk == 128)) || (tile_w == 16 && tile_h == 8 && chunk == 128);
}

cudaError_t launch_raster_forward(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                  uint32_t W, uint32_t H, const float* viewports, uint32_t cull,
                                  const uint32_t* offsets, const uint32_t* list, unsigned long long capacity,
                                  float* raster, float* deriv, cudaStream_t stream, const RasterShade* shade,
                                  const uint32_t* status, uint32_t tile_w, uint32_t tile_h, uint32_t chunk) {
    ShadeArgs sa{};
    if (shade) {
        sa.attrs = shade->attrs;
        sa.A = shade->attribute_count;
        sa.attr_out = shade->attr_out;
        sa.uv_attrs = reinterpret_cast<const float2*>(shade->uv_attrs);
        sa.uv_out = reinterpret_cast<float2*>(shade->uv_out);
        sa.tex = reinterpret_cast<const float4*>(shade->texture);
        sa.tw = shade->texture_width;
        sa.th = shade->texture_height;
        sa.mode = shade->address_mode;
        sa.sampled = reinterpret_cast<float4*>(shade->sampled);
        sa.sdiff = reinterpret_cast<float4*>(shade->sample_differences);
    }
    const float4* c4 = reinterpret_cast<const float4*>(clip);
    const uint3* i3 = reinterpret_cast<const uint3*>(idx);
    const float4* v4 = reinterpret_cast<const float4*>(viewports);
    float4* r4 = reinterpret_cast<float4*>(raster);
    float4* d4 = reinterpret_cast<float4*>(deriv);
    const bool sh = shade != nullptr;
    if (tile_w == 16 && tile_h == 16 && chunk == 256)
        return launch_raster_config<16, 16, 256>(c4, views, V, i3, T, W, H, v4, cull, offsets, list, capacity, r4, d4,
                                                 sa, sh, status, stream);
    if (tile_w == 16 && tile_h == 16 && chunk == 128)
        return launch_raster_config<16, 16, 128>(c4, views, V, i3, T, W, H, v4, cull, offsets, list, capacity, r4, d4,
                                                 sa, sh, status, stream);
    if (tile_w == 16 && tile_h == 8 && chunk == 128)
        return launch_raster_config<16, 8, 128>(c4, views, V, i3, T, W, H, v4, cull, offsets, list, capacity, r4, d4,
                                                sa, sh, status, stream);
    return cudaErrorInvalidValue;
}

// Gradient through the barycentric pixel derivatives (a capability the reference rejects,
// src/rasterizer.cpp:459-462): the adjoint of rasterize_forward.hlsl's derivative output for the pixel's
// winning triangle,
//   D = ((da0/dx - b0 dA/dx) / A * 2/vp.z, (da0/dy - b0 dA/dy) / A * 2/vp.w,
//        (da1/dx - b1 dA/dx) / A * 2/vp.z, (da1/dy - b1 dA/dy) / A * 2/vp.w),
// with a_i = cross(q_j, q_k) of the sample-relative positions q = p.xy - s p.w, A = a0 + a1 + a2,
// b_i = clamp(a_i / A, 0, 1) (no gradient through a clamped b_i) and da_i/dx, da_i/dy the products of
// clip coordinates. Added to grad_clip (x, y, w; z has no influence) after the barycentric adjoint.
__global__ void raster_deriv_backward_kernel(const float4* __restrict__ clip_all, uint32_t V,
                                             const uint3* __restrict__ idx, uint32_t T, uint32_t W, uint32_t H,
                                             const float4* __restrict__ viewports, const float4* __restrict__ raster,
                                             const float4* __restrict__ grad_deriv, float* __restrict__ grad_clip) {
    const uint32_t view = blockIdx.y;
    const size_t P = (size_t)W * H;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const size_t pix = (size_t)view * P + p;
    const uint32_t id = raster_id(raster[pix].w);
    if (id == 0 || id > T) return;
    const float4 g = grad_deriv[pix];
    if (g.x == 0.0f && g.y == 0.0f && g.z == 0.0f && g.w == 0.0f) return;
    const uint3 vi = idx[id - 1];
    if (vi.x >= V || vi.y >= V || vi.z >= V) return;
    const float4* __restrict__ clip = clip_all + (size_t)view * V;
    const float4 p0 = clip[vi.x], p1 = clip[vi.y], p2 = clip[vi.z];
    const float4 vp = viewports[view];
    const uint32_t x = (uint32_t)(p % W), y = (uint32_t)(p / W);
    const float sx = sample_ndc(x, vp.x, vp.z);
    const float sy = sample_ndc(y, vp.y, vp.w);
    // forward quantities
    const float q0x = p0.x - sx * p0.w, q0y = p0.y - sy * p0.w;
    const float q1x = p1.x - sx * p1.w, q1y = p1.y - sy * p1.w;
    const float q2x = p2.x - sx * p2.w, q2y = p2.y - sy * p2.w;
    const float a0 = cross2(q1x, q1y, q2x, q2y);
    const float a1 = cross2(q2x, q2y, q0x, q0y);
    const float a2 = cross2(q0x, q0y, q1x, q1y);
    const float ha = a0 + a1 + a2;
    if (fabsf(ha) <= 1e-12f) return;
    const float binv = 1.0f / ha;
    const float r0 = a0 * binv, r1 = a1 * binv;
    const float b0 = clamp_hlsl(r0, 0.0f, 1.0f), b1 = clamp_hlsl(r1, 0.0f, 1.0f);
    const float d0x = -p1.w * p2.y + p2.w * p1.y, d0y = -p1.x * p2.w + p1.w * p2.x;
    const float d1x = -p2.w * p0.y + p2.y * p0.w, d1y = -p2.x * p0.w + p2.w * p0.x;
    const float d2x = -p0.w * p1.y + p0.y * p1.w, d2y = -p0.x * p1.w + p0.w * p1.x;
    const float dAx = d0x + d1x + d2x, dAy = d0y + d1y + d2y;
    const float kx = 2.0f / vp.z, ky = 2.0f / vp.w;
    // adjoints of D's inputs
    const float gdAx = -(g.x * b0 + g.z * b1) * binv * kx;
    const float gdAy = -(g.y * b0 + g.w * b1) * binv * ky;
    const float G0x = g.x * binv * kx + gdAx, G1x = g.z * binv * kx + gdAx, G2x = gdAx;
    const float G0y = g.y * binv * ky + gdAy, G1y = g.w * binv * ky + gdAy, G2y = gdAy;
    float gb0 = -(g.x * dAx * kx + g.y * dAy * ky) * binv;
    float gb1 = -(g.z * dAx * kx + g.w * dAy * ky) * binv;
    float gbinv = g.x * (d0x - b0 * dAx) * kx + g.y * (d0y - b0 * dAy) * ky + g.z * (d1x - b1 * dAx) * kx +
                  g.w * (d1y - b1 * dAy) * ky;
    if (!(r0 > 0.0f && r0 < 1.0f)) gb0 = 0.0f;
    if (!(r1 > 0.0f && r1 < 1.0f)) gb1 = 0.0f;
    float A0 = gb0 * binv, A1 = gb1 * binv;
    gbinv += gb0 * a0 + gb1 * a1;
    const float gha = -gbinv * binv * binv;
    A0 += gha;
    A1 += gha;
    const float A2 = gha;
    // a_i -> q
    float gq0x = 0.f, gq0y = 0.f, gq1x = 0.f, gq1y = 0.f, gq2x = 0.f, gq2y = 0.f;
    gq1x += A0 * q2y; gq2y += A0 * q1x; gq1y -= A0 * q2x; gq2x -= A0 * q1y;
    gq2x += A1 * q0y; gq0y += A1 * q2x; gq2y -= A1 * q0x; gq0x -= A1 * q2y;
    gq0x += A2 * q1y; gq1y += A2 * q0x; gq0y -= A2 * q1x; gq1x -= A2 * q0y;
    // q -> p, then the da products -> p
    float g0[3] = {gq0x, gq0y, -sx * gq0x - sy * gq0y};  // x, y, w of vertex 0
    float g1[3] = {gq1x, gq1y, -sx * gq1x - sy * gq1y};
    float g2[3] = {gq2x, gq2y, -sx * gq2x - sy * gq2y};
    // d0x = -p1.w p2.y + p2.w p1.y ; d0y = -p1.x p2.w + p1.w p2.x
    g1[2] += -G0x * p2.y + G0y * p2.x; g2[1] += -G0x * p1.w; g2[2] += G0x * p1.y - G0y * p1.x; g1[1] += G0x * p2.w;
    g1[0] += -G0y * p2.w; g2[0] += G0y * p1.w;
    // d1x = -p2.w p0.y + p2.y p0.w ; d1y = -p2.x p0.w + p2.w p0.x
    g2[2] += -G1x * p0.y + G1y * p0.x; g0[1] += -G1x * p2.w; g2[1] += G1x * p0.w; g0[2] += G1x * p2.y - G1y * p2.x;
    g2[0] += -G1y * p0.w; g0[0] += G1y * p2.w;
    // d2x = -p0.w p1.y + p0.y p1.w ; d2y = -p0.x p1.w + p0.w p1.x
    g0[2] += -G2x * p1.y + G2y * p1.x; g1[1] += -G2x * p0.w; g0[1] += G2x * p1.w; g1[2] += G2x * p0.y - G2y * p0.x;
    g0[0] += -G2y * p1.w; g1[0] += G2y * p0.w;
    float* gv = grad_clip + (size_t)view * V * 4;
    const uint32_t vs[3] = {vi.x, vi.y, vi.z};
    const float* gs[3] = {g0, g1, g2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        atomicAdd(gv + (size_t)vs[k] * 4 + 0, gs[k][0]);
        atomicAdd(gv + (size_t)vs[k] * 4 + 1, gs[k][1]);
        atomicAdd(gv + (size_t)vs[k] * 4 + 3, gs[k][2]);
    }
}

cudaError_t launch_raster_backward(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                   uint32_t W, uint32_t H, const float* viewports, const float* raster,
                                   const float* grad_raster, float* grad_clip, cudaStream_t stream,
                                   const float* grad_derivatives, bool near) {
    cudaError_t err = cudaMemsetAsync(grad_clip, 0, (size_t)views * V * 4 * sizeof(float), stream);
    if (err != cudaSuccess) return err;
    const size_t P = (size_t)W * H;
    const dim3 grid((uint32_t)((P + 255) / 256), views);
    if (grad_raster)
        raster_backward_kernel<<<grid, 256, 0, stream>>>(
        reinterpret_cast<const float4*>(clip), V, reinterpret_cast<const uint3*>(idx), T, W, H,
        reinterpret_cast<const float4*>(viewports), reinterpret_cast<const float4*>(raster),
        reinterpret_cast<const float4*>(grad_raster), grad_clip, near ? 1u : 0u);
    if (grad_derivatives)
        raster_deriv_backward_kernel<<<grid, 256, 0, stream>>>(
            reinterpret_cast<const float4*>(clip), V, reinterpret_cast<const uint3*>(idx), T, W, H,
            reinterpret_cast<const float4*>(viewports), reinterpret_cast<const float4*>(raster),
            reinterpret_cast<const float4*>(grad_derivatives), grad_clip);
    return cudaGetLastError();
}

}  // namespace pdr

// Ray-query visibility for the bake: the visibility test of shaders/project_ray_visibility.hlsl:14-55
// against a bounding-volume hierarchy of the mesh, built on the device (the reference builds a Vulkan
// acceleration structure, src/context.cpp:446-453 create_ray_query_scene, and traces with RayQuery).
//
// Build (linear BVH): triangle centroids -> 30-bit Morton codes in the centroid bounds -> stable
// radix sort of (code, triangle) -> binary radix tree over the sorted codes (node i splits where the
// common prefix of its key range changes; equal codes are told apart by their index) -> boxes bottom
// up, the second child to arrive at a node writing its box. Internal nodes keep both children's boxes
// (64 bytes), leaves are single triangles stored in tree order (three float4 vertices).
//
// Traversal: one thread per (texel, view) ray, any hit ends the search (RAY_FLAG_ACCEPT_FIRST_HIT_AND_
// END_SEARCH), both triangle faces count (RAY_FLAG_NONE), hits with t in [t_min, t_max]. Ray set-up
// follows the shader operation by operation; the box test is a slab test on boxes widened by a
// relative 1e-6 of the scene size, the triangle test is Moller-Trumbore in fp32. Hardware ray-triangle
// tests are watertight and this one is not, so rays that graze an edge or a vertex may be classified
// differently than on the reference's GPU; everything else agrees.
#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"
#include "projection.cuh"

namespace pdr {
namespace {

struct BvhNode {     // children: >= 0 internal node, < 0 leaf ~index
    float4 a;        // lmin.x lmin.y lmin.z lmax.x
    float4 b;        // lmax.y lmax.z rmin.x rmin.y
    float4 c;        // rmin.z rmax.x rmax.y rmax.z
    int4 d;          // left, right, -, -
};

struct BvhHeader {
    uint32_t triangles;
    int32_t root;    // 0 (internal) or ~0 (a single leaf)
    float pad[2];
};

constexpr size_t kHeaderBytes = 256;

struct BvhView {
    const BvhHeader* header;
    const BvhNode* nodes;   // [T - 1]
    const float4* tris;     // [T][3] in leaf order
};

size_t nodes_bytes(uint32_t T) { return align_up((size_t)(T > 1 ? T - 1 : 1) * sizeof(BvhNode)); }
size_t tris_bytes(uint32_t T) { return align_up((size_t)T * 3 * sizeof(float4)); }

BvhView bvh_view(const void* buf, uint32_t T) {
    const char* c = static_cast<const char*>(buf);
    BvhView v;
    v.header = reinterpret_cast<const BvhHeader*>(c);
    v.nodes = reinterpret_cast<const BvhNode*>(c + kHeaderBytes);
    v.tris = reinterpret_cast<const float4*>(c + kHeaderBytes + nodes_bytes(T));
    return v;
}

// ---- build --------------------------------------------------------------------------------------

__device__ __forceinline__ uint32_t ordered(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

__device__ __forceinline__ bool tri_vertices(const float* __restrict__ pos, uint32_t V, const uint3* __restrict__ idx,
                                             uint32_t t, float3& p0, float3& p1, float3& p2) {
    const uint3 vi = idx[t];
    if (vi.x >= V || vi.y >= V || vi.z >= V) return false;
    p0 = make_float3(pos[vi.x * 3], pos[vi.x * 3 + 1], pos[vi.x * 3 + 2]);
    p1 = make_float3(pos[vi.y * 3], pos[vi.y * 3 + 1], pos[vi.y * 3 + 2]);
    p2 = make_float3(pos[vi.z * 3], pos[vi.z * 3 + 1], pos[vi.z * 3 + 2]);
    return isfinite(p0.x + p0.y + p0.z + p1.x + p1.y + p1.z + p2.x + p2.y + p2.z);
}

// Centroid bounds (ordered-int min/max in bounds[0..5]) and, per triangle, its centroid.
__global__ void centroid_bounds_kernel(const float* __restrict__ pos, uint32_t V, const uint3* __restrict__ idx,
                                       uint32_t T, float4* __restrict__ centroid, uint32_t* __restrict__ bounds) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    float3 p0, p1, p2;
    bool ok = false;
    float3 c = make_float3(0.f, 0.f, 0.f);
    if (t < T && tri_vertices(pos, V, idx, t, p0, p1, p2)) {
        ok = true;
        c = make_float3((p0.x + p1.x + p2.x) * (1.0f / 3.0f), (p0.y + p1.y + p2.y) * (1.0f / 3.0f),
                        (p0.z + p1.z + p2.z) * (1.0f / 3.0f));
    }
    if (t < T) centroid[t] = make_float4(c.x, c.y, c.z, ok ? 1.0f : 0.0f);
    uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
    if (ok) {
        const float cc[3] = {c.x, c.y, c.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) lo[k] = hi[k] = ordered(cc[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    if ((threadIdx.x & 31u) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(bounds + k, lo[k]);
            atomicMax(bounds + 3 + k, hi[k]);
        }
    }
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {  // 10 bits -> every third bit of 30
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void morton_kernel(const float4* __restrict__ centroid, uint32_t T, const uint32_t* __restrict__ bounds,
                              uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const float4 c = centroid[t];
    uint32_t code = 0x3fffffffu;  // unusable triangles sort last
    if (c.w > 0.0f) {
        const float cc[3] = {c.x, c.y, c.z};
        uint32_t q[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float lo = unordered(bounds[k]), hi = unordered(bounds[3 + k]);
            const float ext = hi - lo;
            const float u = ext > 0.0f ? (cc[k] - lo) / ext : 0.5f;
            q[k] = (uint32_t)fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f);
        }
        code = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    }
    keys[t] = code;
    vals[t] = t;
}

__device__ __forceinline__ int delta(const uint32_t* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = k[i], b = k[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

// Binary radix tree over the sorted codes: children and parents of internal node i.
__global__ void radix_tree_kernel(const uint32_t* __restrict__ keys, int n, int2* __restrict__ children,
                                  int* __restrict__ node_parent, int* __restrict__ leaf_parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
        const int t = (l + div - 1) / div;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int left = (min(i, j) == gamma) ? ~gamma : gamma;
    const int right = (max(i, j) == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    children[i] = make_int2(left, right);
    if (left < 0) leaf_parent[~left] = i;
    else node_parent[left] = i;
    if (right < 0) leaf_parent[~right] = i;
    else node_parent[right] = i;
    if (i == 0) node_parent[0] = -1;
}

struct Box {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box load_box(const float* __restrict__ boxes, int k) {
    Box b;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        b.lo[c] = __ldcg(boxes + (size_t)k * 6 + c);
        b.hi[c] = __ldcg(boxes + (size_t)k * 6 + 3 + c);
    }
    return b;
}

// Leaves: vertices in tree order and their boxes; then each thread climbs while it is the second child
// to arrive, so every internal node gets its box (and the packed node) exactly once.
__global__ void bottom_up_kernel(const float* __restrict__ pos, uint32_t V, const uint3* __restrict__ idx, int n,
                                 const uint32_t* __restrict__ order, const int2* __restrict__ children,
                                 const int* __restrict__ node_parent, const int* __restrict__ leaf_parent,
                                 float* __restrict__ leaf_boxes, float* __restrict__ node_boxes,
                                 uint32_t* __restrict__ arrivals, float pad, BvhNode* __restrict__ nodes,
                                 float4* __restrict__ tris) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n) return;
    const uint32_t t = order[l];
    float3 p0, p1, p2;
    Box b;
    if (tri_vertices(pos, V, idx, t, p0, p1, p2)) {
        b.lo[0] = fminf(p0.x, fminf(p1.x, p2.x)) - pad;
        b.lo[1] = fminf(p0.y, fminf(p1.y, p2.y)) - pad;
        b.lo[2] = fminf(p0.z, fminf(p1.z, p2.z)) - pad;
        b.hi[0] = fmaxf(p0.x, fmaxf(p1.x, p2.x)) + pad;
        b.hi[1] = fmaxf(p0.y, fmaxf(p1.y, p2.y)) + pad;
        b.hi[2] = fmaxf(p0.z, fmaxf(p1.z, p2.z)) + pad;
        tris[(size_t)l * 3] = make_float4(p0.x, p0.y, p0.z, 1.0f);
        tris[(size_t)l * 3 + 1] = make_float4(p1.x, p1.y, p1.z, 0.0f);
        tris[(size_t)l * 3 + 2] = make_float4(p2.x, p2.y, p2.z, 0.0f);
    } else {  // an empty box no ray enters, and a triangle no ray hits
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            b.lo[c] = INFINITY;
            b.hi[c] = -INFINITY;
        }
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        tris[(size_t)l * 3] = z;
        tris[(size_t)l * 3 + 1] = z;
        tris[(size_t)l * 3 + 2] = z;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        leaf_boxes[(size_t)l * 6 + c] = b.lo[c];
        leaf_boxes[(size_t)l * 6 + 3 + c] = b.hi[c];
    }
    if (n == 1) return;
    int node = leaf_parent[l];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(arrivals + node, 1u) == 0u) return;  // the other child is not done yet
        __threadfence();
        const int2 ch = children[node];
        const Box L = ch.x < 0 ? load_box(leaf_boxes, ~ch.x) : load_box(node_boxes, ch.x);
        const Box R = ch.y < 0 ? load_box(leaf_boxes, ~ch.y) : load_box(node_boxes, ch.y);
        BvhNode out;
        out.a = make_float4(L.lo[0], L.lo[1], L.lo[2], L.hi[0]);
        out.b = make_float4(L.hi[1], L.hi[2], R.lo[0], R.lo[1]);
        out.c = make_float4(R.lo[2], R.hi[0], R.hi[1], R.hi[2]);
        out.d = make_int4(ch.x, ch.y, 0, 0);
        nodes[node] = out;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            node_boxes[(size_t)node * 6 + c] = fminf(L.lo[c], R.lo[c]);
            node_boxes[(size_t)node * 6 + 3 + c] = fmaxf(L.hi[c], R.hi[c]);
        }
        node = node_parent[node];
    }
}

__global__ void header_kernel(BvhHeader* h, uint32_t T) {
    h->triangles = T;
    h->root = T > 1 ? 0 : ~0;
}

// ---- traversal ----------------------------------------------------------------------------------

// Moller-Trumbore: any hit with t in [t0, t1], either face.
__device__ __forceinline__ bool hits_triangle(const float4* __restrict__ tri, float ox, float oy, float oz, float dx,
                                              float dy, float dz, float t0, float t1) {
    const float4 v0 = tri[0], v1 = tri[1], v2 = tri[2];
    const float e1x = v1.x - v0.x, e1y = v1.y - v0.y, e1z = v1.z - v0.z;
    const float e2x = v2.x - v0.x, e2y = v2.y - v0.y, e2z = v2.z - v0.z;
    const float px = dy * e2z - dz * e2y, py = dz * e2x - dx * e2z, pz = dx * e2y - dy * e2x;
    const float det = e1x * px + e1y * py + e1z * pz;
    if (!(fabsf(det) > 1e-20f)) return false;
    const float inv = 1.0f / det;
    const float sx = ox - v0.x, sy = oy - v0.y, sz = oz - v0.z;
    const float u = (sx * px + sy * py + sz * pz) * inv;
    if (u < 0.0f || u > 1.0f) return false;
    const float qx = sy * e1z - sz * e1y, qy = sz * e1x - sx * e1z, qz = sx * e1y - sy * e1x;
    const float v = (dx * qx + dy * qy + dz * qz) * inv;
    if (v < 0.0f || u + v > 1.0f) return false;
    const float t = (e2x * qx + e2y * qy + e2z * qz) * inv;
    return t >= t0 && t <= t1;
}

constexpr int kStack = 64;

__device__ __forceinline__ bool load_texel(const float* __restrict__ apos, const float* __restrict__ anrm,
                                           const float4* __restrict__ araster, uint32_t i, float& px, float& py,
                                           float& pz, float& nx, float& ny, float& nz) {
    if (raster_id(araster[i].w) == 0) return false;
    px = apos[(size_t)i * 3];
    py = apos[(size_t)i * 3 + 1];
    pz = apos[(size_t)i * 3 + 2];
    const float nx0 = anrm[(size_t)i * 3], ny0 = anrm[(size_t)i * 3 + 1], nz0 = anrm[(size_t)i * 3 + 2];
    const float nl = sqrtf(nx0 * nx0 + ny0 * ny0 + nz0 * nz0);
    nx = nx0 / nl;
    ny = ny0 / nl;
    nz = nz0 / nl;
    return true;
}

// Slab test with each plane distance formed by one FMA: t = lo * (1/d) + (-o/d). Leaf boxes are padded
// by 1e-6, more than the rounding difference to (lo - o) / d, so no box holding a hit is pruned.
__device__ __forceinline__ bool slab_fma(float lox, float loy, float loz, float hix, float hiy, float hiz, float ix,
                                         float iy, float iz, float bx, float by, float bz, float t0, float t1) {
    const float tx0 = __fmaf_rn(lox, ix, bx), tx1 = __fmaf_rn(hix, ix, bx);
    const float ty0 = __fmaf_rn(loy, iy, by), ty1 = __fmaf_rn(hiy, iy, by);
    const float tz0 = __fmaf_rn(loz, iz, bz), tz1 = __fmaf_rn(hiz, iz, bz);
    const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), t0));
    const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), t1));
    return tn <= tf;
}

__device__ __forceinline__ float safe_inverse(float d) { return 1.0f / (fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d)); }

// Any hit with t in [t0, t1] below the root (an inner node); complete traversal, so the answer does not
// depend on the visiting order.
__device__ bool occluded(const BvhView& bvh, int root, float ox, float oy, float oz, float dx, float dy, float dz,
                         float t0, float t1) {
    const float ix = safe_inverse(dx), iy = safe_inverse(dy), iz = safe_inverse(dz);
    const float bx = -ox * ix, by = -oy * iy, bz = -oz * iz;
    int stack[kStack];
    int sp = 0;
    int node = root;
    for (;;) {
        const BvhNode nd = bvh.nodes[node];
        const bool hl = slab_fma(nd.a.x, nd.a.y, nd.a.z, nd.a.w, nd.b.x, nd.b.y, ix, iy, iz, bx, by, bz, t0, t1);
        const bool hr = slab_fma(nd.b.z, nd.b.w, nd.c.x, nd.c.y, nd.c.z, nd.c.w, ix, iy, iz, bx, by, bz, t0, t1);
        const int cl = nd.d.x, cr = nd.d.y;
        int next = -1;
        if (hl) {
            if (cl < 0) {
                if (hits_triangle(bvh.tris + (size_t)(~cl) * 3, ox, oy, oz, dx, dy, dz, t0, t1)) return true;
            } else {
                next = cl;
            }
        }
        if (hr) {
            if (cr < 0) {
                if (hits_triangle(bvh.tris + (size_t)(~cr) * 3, ox, oy, oz, dx, dy, dz, t0, t1)) return true;
            } else if (next < 0) {
                next = cr;
            } else if (sp < kStack) {
                stack[sp++] = cr;
            }
        }
        if (next >= 0) node = next;
        else if (sp > 0) node = stack[--sp];
        else return false;
    }
}

// project_ray_visibility.hlsl:35-54 for surface point p with unit normal n and one camera.
__device__ __forceinline__ bool camera_visible(const BvhView& bvh, int root, float4 p, float4 n, float cx, float cy,
                                               float cz, float bias) {
    const float vx = cx - p.x, vy = cy - p.y, vz = cz - p.z;
    const float dist = sqrtf(vx * vx + vy * vy + vz * vz);
    if (dist <= bias * 2.0f) return true;
    const float dx = vx / dist, dy = vy / dist, dz = vz / dist;
    const float sgn = (n.x * dx + n.y * dy + n.z * dz) >= 0.0f ? 1.0f : -1.0f;
    const float ox = p.x + n.x * (bias * sgn), oy = p.y + n.y * (bias * sgn), oz = p.z + n.z * (bias * sgn);
    const float t0 = bias;
    const float t1 = fmaxf(t0, dist - bias * 2.0f);
    if (root < 0) return !hits_triangle(bvh.tris + (size_t)(~root) * 3, ox, oy, oz, dx, dy, dz, t0, t1);
    return !occluded(bvh, root, ox, oy, oz, dx, dy, dz, t0, t1);
}

// shaders/project_ray_visibility.hlsl:14-55 for texel i and the 32 views of word blockIdx.y: bit
// (view & 31) of word i * words + view / 32 is set when the camera is visible. One thread builds the
// whole word in a register (no atomics; uncovered texels get 0, as the shader writes). kGated traces
// only the texel-views the projection reads (project_texel passes); the others report 0. The lanes of
// a warp are neighbouring texels tracing toward the same camera, so their node fetches coincide.
template <bool kGated>
__global__ void __launch_bounds__(128) trace_words_kernel(BvhView bvh, const float* __restrict__ apos,
                                                          const float* __restrict__ anrm,
                                                          const float4* __restrict__ araster, uint32_t N,
                                                          const float4* __restrict__ cameras,
                                                          const pdr_projection_view* __restrict__ views,
                                                          uint32_t nviews, float bias, uint32_t words,
                                                          uint32_t* __restrict__ bits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t w = blockIdx.y;
    if (i >= N) return;
    uint32_t word = 0;
    float px, py, pz, nx, ny, nz;
    if (load_texel(apos, anrm, araster, i, px, py, pz, nx, ny, nz)) {
        const float4 p = make_float4(px, py, pz, 1.0f), n = make_float4(nx, ny, nz, 0.0f);
        const int root = bvh.header->root;
        const uint32_t end = min(nviews, (w + 1) * 32);
        for (uint32_t k = w * 32; k < end; ++k) {
            float cx, cy, cz;
            if (kGated) {
                const pdr_projection_view& v = views[k];
                ProjectedTexel pt;
                if (!project_texel(v, px, py, pz, nx, ny, nz, pt)) continue;
                cx = v.camera_position[0];
                cy = v.camera_position[1];
                cz = v.camera_position[2];
            } else {
                const float4 c = cameras[k];
                cx = c.x;
                cy = c.y;
                cz = c.z;
            }
            if (camera_visible(bvh, root, p, n, cx, cy, cz, bias)) word |= 1u << (k & 31u);
        }
    }
    bits[(size_t)i * words + w] = word;
}

}  // namespace
}  // namespace pdr

using namespace pdr;

extern "C" {

pdr_status pdr_bvh_sizes(uint32_t triangle_count, size_t* bvh_bytes, size_t* build_bytes) {
    if (!bvh_bytes || !build_bytes || triangle_count == 0)
        return set_error(PDR_INVALID_ARGUMENT, "BVH sizes need a positive triangle count and outputs");
    if (triangle_count > 0x3fffffffu) return set_error(PDR_OVERFLOW, "BVH triangle count exceeds backend limits");
    const uint32_t T = triangle_count;
    *bvh_bytes = kHeaderBytes + nodes_bytes(T) + tris_bytes(T);
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, (int)T, 0, 30);
    size_t b = 0;
    b += align_up((size_t)T * sizeof(float4));     // centroids
    b += align_up(6 * sizeof(uint32_t));           // bounds
    b += 4 * align_up((size_t)T * sizeof(uint32_t));  // keys, sorted keys, values, sorted values
    b += align_up(cub_bytes);
    b += align_up((size_t)T * sizeof(int2));       // children
    b += align_up((size_t)T * sizeof(int)) * 2;    // node / leaf parents
    b += align_up((size_t)T * 6 * sizeof(float)) * 2;  // leaf / node boxes
    b += align_up((size_t)T * sizeof(uint32_t));   // arrival counters
    *build_bytes = b;
    return PDR_OK;
}

pdr_status pdr_bvh_build(const float* positions, uint32_t vertex_count, const uint32_t* indices,
                         uint32_t triangle_count, void* bvh, size_t bvh_bytes, void* scratch, size_t scratch_bytes,
                         void* stream) {
    if (!positions || !indices || !bvh || !scratch || vertex_count == 0 || triangle_count == 0)
        return set_error(PDR_INVALID_ARGUMENT, "BVH build needs positions, indices and buffers");
    size_t need_bvh = 0, need_build = 0;
    pdr_status st = pdr_bvh_sizes(triangle_count, &need_bvh, &need_build);
    if (st) return st;
    if (bvh_bytes < need_bvh || scratch_bytes < need_build)
        return set_error(PDR_INVALID_ARGUMENT, "BVH buffers are smaller than pdr_bvh_sizes()");
    const uint32_t T = triangle_count;
    const cudaStream_t s = (cudaStream_t)stream;
    char* c = static_cast<char*>(scratch);
    auto take = [&](size_t bytes) {
        char* r = c;
        c += align_up(bytes);
        return r;
    };
    float4* centroid = reinterpret_cast<float4*>(take((size_t)T * sizeof(float4)));
    uint32_t* bounds = reinterpret_cast<uint32_t*>(take(6 * sizeof(uint32_t)));
    uint32_t* keys = reinterpret_cast<uint32_t*>(take((size_t)T * 4));
    uint32_t* keys_sorted = reinterpret_cast<uint32_t*>(take((size_t)T * 4));
    uint32_t* vals = reinterpret_cast<uint32_t*>(take((size_t)T * 4));
    uint32_t* vals_sorted = reinterpret_cast<uint32_t*>(take((size_t)T * 4));
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, keys, keys_sorted, vals, vals_sorted, (int)T, 0, 30, s);
    void* cub_tmp = take(cub_bytes);
    int2* children = reinterpret_cast<int2*>(take((size_t)T * sizeof(int2)));
    int* node_parent = reinterpret_cast<int*>(take((size_t)T * sizeof(int)));
    int* leaf_parent = reinterpret_cast<int*>(take((size_t)T * sizeof(int)));
    float* leaf_boxes = reinterpret_cast<float*>(take((size_t)T * 6 * sizeof(float)));
    float* node_boxes = reinterpret_cast<float*>(take((size_t)T * 6 * sizeof(float)));
    uint32_t* arrivals = reinterpret_cast<uint32_t*>(take((size_t)T * sizeof(uint32_t)));
    const uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    cudaError_t e = cudaMemcpyAsync(bounds, init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(arrivals, 0, (size_t)T * sizeof(uint32_t), s);
    if (e != cudaSuccess) return set_cuda_error(e, "bvh_build(set-up)");
    const unsigned blocks = (T + 255) / 256;
    centroid_bounds_kernel<<<blocks, 256, 0, s>>>(positions, vertex_count, reinterpret_cast<const uint3*>(indices), T,
                                                  centroid, bounds);
    morton_kernel<<<blocks, 256, 0, s>>>(centroid, T, bounds, keys, vals);
    e = cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, keys, keys_sorted, vals, vals_sorted, (int)T, 0, 30, s);
    if (e != cudaSuccess) return set_cuda_error(e, "bvh_build(sort)");
    if (T > 1)
        radix_tree_kernel<<<(T - 1 + 255) / 256, 256, 0, s>>>(keys_sorted, (int)T, children, node_parent, leaf_parent);
    const BvhView v = bvh_view(bvh, T);
    // widen every box by a relative 1e-6 of the scene (positions up to |x| ~ 1e3 keep fp32 slab tests safe)
    bottom_up_kernel<<<blocks, 256, 0, s>>>(positions, vertex_count, reinterpret_cast<const uint3*>(indices), (int)T,
                                            vals_sorted, children, node_parent, leaf_parent, leaf_boxes, node_boxes,
                                            arrivals, 1e-6f, const_cast<BvhNode*>(v.nodes),
                                            const_cast<float4*>(v.tris));
    header_kernel<<<1, 1, 0, s>>>(const_cast<BvhHeader*>(v.header), T);
    // the host-side initial bounds must have been read before this function returns
    e = cudaStreamSynchronize(s);
    return set_cuda_error(e == cudaSuccess ? cudaGetLastError() : e, "bvh_build");
}

pdr_status pdr_ray_visibility(const void* bvh, uint32_t triangle_count, const float* atlas_positions,
                              const float* atlas_normals, const float* atlas_raster, uint32_t atlas_texels,
                              const float* cameras, uint32_t view_count, float ray_origin_bias, uint32_t* visibility,
                              void* stream) {
    if (!bvh || !atlas_positions || !atlas_normals || !atlas_raster || !cameras || !visibility || triangle_count == 0)
        return set_error(PDR_INVALID_ARGUMENT, "ray visibility needs the BVH, the atlas G-buffer and an output");
    if (view_count == 0 || view_count > 65535u) return set_error(PDR_INVALID_ARGUMENT, "view count must be 1..65535");
    if (!(ray_origin_bias > 0.0f) || !isfinite(ray_origin_bias))
        return set_error(PDR_INVALID_ARGUMENT, "ray_origin_bias must be positive and finite");
    if (atlas_texels == 0) return PDR_OK;
    const uint32_t words = (view_count + 31) / 32;
    const dim3 grid((atlas_texels + 127) / 128, words);
    trace_words_kernel<false><<<grid, 128, 0, (cudaStream_t)stream>>>(
        bvh_view(bvh, triangle_count), atlas_positions, atlas_normals, reinterpret_cast<const float4*>(atlas_raster),
        atlas_texels, reinterpret_cast<const float4*>(cameras), nullptr, view_count, ray_origin_bias, words,
        visibility);
    return set_cuda_error(cudaGetLastError(), "ray_visibility");
}

pdr_status pdr_ray_visibility_views(const void* bvh, uint32_t triangle_count, const float* atlas_positions,
                                    const float* atlas_normals, const float* atlas_raster, uint32_t atlas_texels,
                                    const pdr_projection_view* views, uint32_t view_count, float ray_origin_bias,
                                    uint32_t* visibility, void* stream) {
    if (!bvh || !atlas_positions || !atlas_normals || !atlas_raster || !views || !visibility || triangle_count == 0)
        return set_error(PDR_INVALID_ARGUMENT, "ray visibility needs the BVH, the atlas G-buffer and an output");
    if (view_count == 0 || view_count > 65535u) return set_error(PDR_INVALID_ARGUMENT, "view count must be 1..65535");
    if (!(ray_origin_bias > 0.0f) || !isfinite(ray_origin_bias))
        return set_error(PDR_INVALID_ARGUMENT, "ray_origin_bias must be positive and finite");
    if (atlas_texels == 0) return PDR_OK;
    const uint32_t words = (view_count + 31) / 32;
    const dim3 grid((atlas_texels + 127) / 128, words);
    trace_words_kernel<true><<<grid, 128, 0, (cudaStream_t)stream>>>(
        bvh_view(bvh, triangle_count), atlas_positions, atlas_normals, reinterpret_cast<const float4*>(atlas_raster),
        atlas_texels, nullptr, views, view_count, ray_origin_bias, words, visibility);
    return set_cuda_error(cudaGetLastError(), "ray_visibility_views");
}

pdr_status pdr_project_views_bits(const float* apos, const float* anrm, const float* araster, uint32_t N,
                                  const pdr_projection_view* views, uint32_t nviews, uint32_t blend_mode,
                                  uint32_t pcf_radius, uint32_t visibility_mode, const uint32_t* visibility,
                                  float* color, float* confidence, uint32_t* source_view, float* valid_mask,
                                  float* coverage_mask, uint32_t* face_ids, void* stream) {
    if (!apos || !anrm || !araster || !views || !color || !confidence || !source_view || !valid_mask || !visibility)
        return set_error(PDR_INVALID_ARGUMENT, "projection buffers are required");
    if (N == 0 || nviews == 0 || pcf_radius > 4 || blend_mode > 2 || visibility_mode < 1 || visibility_mode > 2)
        return set_error(PDR_INVALID_ARGUMENT, "ray-visibility projection needs visibility mode 1 or 2");
    if (((uintptr_t)araster | (uintptr_t)color | (uintptr_t)views) & 15u)
        return set_error(PDR_INVALID_ARGUMENT, "projection buffers must be 16-byte aligned");
    return set_cuda_error(launch_project_views(apos, anrm, araster, N, views, nviews, blend_mode, pcf_radius,
                                               visibility_mode, color, confidence, source_view, valid_mask,
                                               coverage_mask, face_ids, (cudaStream_t)stream, visibility,
                                               (nviews + 31) / 32),
                          "project_views_bits");
}

}  // extern "C"

// Uneven multi-mesh batches: every (mesh, view) of a batch is one job, and a batch runs as one
// binning pass, one raster launch over the tiles of all jobs and one adjoint launch, however the
// meshes differ in triangle count, view count, resolution and texture size. No counterpart in the
// reference (it renders one mesh per call).
//
// The host writes a job table into the workspace: per job the view's clip positions, viewport and
// image pointers, and three prefix sums (triangles, forward tiles, backward 16x16 tiles). A CTA or
// thread finds its job by binary search over the matching prefix. Forward tiles have the batch's tile
// shape (TW x TH pixels) and stage CHUNK triangles per pass; both come from the autotuner and change
// only the work distribution: outputs are bit-identical for every shape (the tile routine does not
// depend on the order or grouping of a tile's triangles).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/pdr_capi.h"
#include "bin_rect.cuh"
#include "pdr_common.cuh"
#include "pdr_internal.h"
#include "raster_tile.cuh"
#include "render_bwd_tile.cuh"

static_assert(sizeof(pdr_render_mesh) == 6 * 8 + 8 * 4 + 11 * 8, "pdr_render_mesh layout");
static_assert(sizeof(pdr_batch_config) == 12, "pdr_batch_config layout");

namespace pdr {
namespace {

struct BatchJob {
    const float4* clip;  // [V] of this view
    const uint3* idx;
    const float4* vp;    // this view's viewport
    uint32_t V, T, W, H;
    uint32_t tcx, btcx;  // forward tiles per row (batch tile shape), backward 16x16 tiles per row
    const float* attrs;
    const float2* uv_attrs;
    const float4* tex;
    uint32_t tw, th;
    float4* raster;      // [H][W] of this view
    float4* deriv;
    float* interp;
    float2* uv;
    float4* sampled;
    const float* grad_interp;
    const float4* grad_sampled;
    float* g_clip;       // [V][4] of this view
    float* g_attr;       // [V][A] of the mesh
    float* g_uv;         // [V][2] of the mesh
    float* g_tex;        // [th][tw][4] of the mesh
};

// The last job j with base[j] <= x (base[0] == 0, non-decreasing).
__device__ __forceinline__ uint32_t find_job(const unsigned long long* __restrict__ base, uint32_t njobs,
                                             unsigned long long x) {
    uint32_t lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (base[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Pass 1 over all (job, triangle) pairs: tile rectangle and per-tile counts, warp-aggregated when the
// lanes of a warp land in the same single tile.
__global__ void batch_bin_count_kernel(const BatchJob* __restrict__ jobs, const unsigned long long* __restrict__ tri_base,
                                       const unsigned long long* __restrict__ tile_base, uint32_t njobs,
                                       unsigned long long total, uint32_t tile_w, uint32_t tile_h,
                                       TriRect* __restrict__ rects, uint32_t* __restrict__ counts) {
    const unsigned long long gid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = gid < total;
    TriRect r{kNoRect, 0};
    unsigned long long seg0 = 0;
    uint32_t tcx = 1;
    if (live) {
        const uint32_t j = find_job(tri_base, njobs, gid);
        const BatchJob& b = jobs[j];
        const uint32_t t = (uint32_t)(gid - tri_base[j]);
        const uint3 vi = b.idx[t];
        if (vi.x < b.V && vi.y < b.V && vi.z < b.V) r = triangle_tile_rect(b.clip, vi, b.W, b.H, *b.vp, tile_w, tile_h);
        rects[gid] = r;
        seg0 = tile_base[j];
        tcx = b.tcx;
    }
    const bool has = live && r.x != kNoRect;
    const uint32_t tx0 = r.x & 0xffffu, tx1 = r.x >> 16, ty0 = r.y & 0xffffu, ty1 = r.y >> 16;
    const bool single = has && tx0 == tx1 && ty0 == ty1;
    const unsigned long long key = single ? seg0 + ty0 * tcx + tx0 : ~0ull - (threadIdx.x & 31u);
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (single && (__ffs(peers) - 1) == (int)(threadIdx.x & 31u)) atomicAdd(counts + key, (uint32_t)__popc(peers));
    if (has && !single) {
        for (uint32_t ty = ty0; ty <= ty1; ++ty)
            for (uint32_t tx = tx0; tx <= tx1; ++tx) atomicAdd(counts + seg0 + ty * tcx + tx, 1u);
    }
}

// Pass 2: every triangle id (the mesh's own index) into its tiles, in arrival order.
__global__ void batch_bin_fill_kernel(const BatchJob* __restrict__ jobs, const unsigned long long* __restrict__ tri_base,
                                      const unsigned long long* __restrict__ tile_base, uint32_t njobs,
                                      unsigned long long total, const TriRect* __restrict__ rects,
                                      uint32_t* __restrict__ cursor, uint32_t* __restrict__ list,
                                      unsigned long long capacity) {
    const unsigned long long gid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = gid < total;
    TriRect r{kNoRect, 0};
    unsigned long long seg0 = 0;
    uint32_t tcx = 1, t = 0;
    if (live) {
        const uint32_t j = find_job(tri_base, njobs, gid);
        r = rects[gid];
        t = (uint32_t)(gid - tri_base[j]);
        seg0 = tile_base[j];
        tcx = jobs[j].tcx;
    }
    const bool has = live && r.x != kNoRect;
    const uint32_t tx0 = r.x & 0xffffu, tx1 = r.x >> 16, ty0 = r.y & 0xffffu, ty1 = r.y >> 16;
    const bool single = has && tx0 == tx1 && ty0 == ty1;
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long key = single ? seg0 + ty0 * tcx + tx0 : ~0ull - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (single) {
        const int leader = __ffs(peers) - 1;
        uint32_t slot = 0;
        if ((int)lane == leader) slot = atomicAdd(cursor + key, (uint32_t)__popc(peers));
        slot = __shfl_sync(peers, slot, leader);
        slot += __popc(peers & ((1u << lane) - 1u));
        if (slot < capacity) list[slot] = t;
    }
    if (has && !single) {
        for (uint32_t ty = ty0; ty <= ty1; ++ty)
            for (uint32_t tx = tx0; tx <= tx1; ++tx) {
                const uint32_t slot = atomicAdd(cursor + seg0 + ty * tcx + tx, 1u);
                if (slot < capacity) list[slot] = t;
            }
    }
}

// One CTA per forward tile of any job.
template <int TW, int TH, int CHUNK>
__global__ void __launch_bounds__(TW * TH)
batch_raster_kernel(const BatchJob* __restrict__ jobs, const unsigned long long* __restrict__ tile_base, uint32_t njobs,
                    const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ list,
                    unsigned long long capacity, uint32_t A, uint32_t cull, uint32_t mode) {
    const unsigned long long tg = blockIdx.x;
    const uint32_t j = find_job(tile_base, njobs, tg);
    const BatchJob& b = jobs[j];
    const uint32_t tile = (uint32_t)(tg - tile_base[j]);
    RasterView v;
    v.clip = b.clip;
    v.idx = b.idx;
    v.V = b.V;
    v.T = b.T;
    v.W = b.W;
    v.H = b.H;
    v.cull = cull;
    v.vp = *b.vp;
    v.raster = b.raster;
    v.deriv = b.deriv;
    v.shade.attrs = b.attrs;
    v.shade.A = A;
    v.shade.attr_out = b.attrs ? b.interp : nullptr;
    v.shade.uv_attrs = b.uv_attrs;
    v.shade.uv_out = b.uv_attrs ? b.uv : nullptr;
    v.shade.tex = b.tex;
    v.shade.tw = b.tw;
    v.shade.th = b.th;
    v.shade.mode = mode;
    v.shade.sampled = b.tex ? b.sampled : nullptr;
    v.shade.sdiff = nullptr;
    const uint32_t s = offsets[tg];
    uint32_t e = offsets[tg + 1];
    if (e > capacity) e = (uint32_t)capacity;
    if (s > e) e = s;
    raster_tile<true, true, TW, TH, CHUNK>(v, tile % b.tcx, tile / b.tcx, list, s, e);
}

// One CTA per 16x16 backward tile of any job.
template <int kA>
__global__ void __launch_bounds__(kFusedThreads, 4)
batch_backward_kernel(const BatchJob* __restrict__ jobs, const unsigned long long* __restrict__ btile_base,
                      uint32_t njobs, uint32_t mode, uint32_t* __restrict__ status) {
    const unsigned long long tg = blockIdx.x;
    const uint32_t j = find_job(btile_base, njobs, tg);
    const BatchJob& b = jobs[j];
    const uint32_t tile = (uint32_t)(tg - btile_base[j]);
    BackwardView v;
    v.g_vtx = nullptr;
    v.clip = b.clip;
    v.V = b.V;
    v.idx = b.idx;
    v.T = b.T;
    v.W = b.W;
    v.H = b.H;
    v.vp = *b.vp;
    v.attrs = b.attrs;
    v.uv_attrs = b.uv_attrs;
    v.tex = b.tex;
    v.tw = b.tw;
    v.th = b.th;
    v.mode = mode;
    v.raster = b.raster;
    v.uv = b.uv_attrs ? b.uv : nullptr;
    v.grad_attr_out = b.grad_interp;
    v.grad_sampled = b.grad_sampled;
    v.g_clip = b.g_clip;
    v.g_attr = b.g_attr;
    v.g_uv = b.g_uv;
    v.g_tex = b.g_tex;
    v.sdiff = nullptr;
    v.status = status;
    render_backward_tile<kA>(v, tile % b.btcx, tile / b.btcx);
}

struct BatchPlan {
    std::vector<BatchJob> jobs;
    std::vector<unsigned long long> tri_base, tile_base, btile_base;  // njobs + 1 each
    unsigned long long total_tris = 0, segs = 0, btiles = 0;
};

bool config_supported(const pdr_batch_config* c) {
    if (!c) return false;
    const uint32_t w = c->tile_width, h = c->tile_height, k = c->stage_triangles;
    return (w == 16 && h == 8 && k == 128) || (w == 16 && h == 16 && (k == 128 || k == 256));
}

pdr_status plan_batch(const pdr_render_mesh* meshes, uint32_t n, const pdr_batch_config* cfg, uint32_t A,
                      bool need_grads, BatchPlan* plan) {
    if (!meshes || n == 0) return set_error(PDR_INVALID_ARGUMENT, "a batch needs at least one mesh");
    if (!config_supported(cfg))
        return set_error(PDR_INVALID_ARGUMENT, "batch tile shape must be 16x8 (stage 128) or 16x16 (stage 128 or 256)");
    if (A > 8) return set_error(PDR_INVALID_ARGUMENT, "batches support 0..8 attributes");
    plan->tri_base.assign(1, 0);
    plan->tile_base.assign(1, 0);
    plan->btile_base.assign(1, 0);
    for (uint32_t m = 0; m < n; ++m) {
        const pdr_render_mesh& M = meshes[m];
        if (!M.clip_positions || !M.indices || !M.viewports || !M.raster || !M.barycentric_derivatives ||
            M.views == 0 || M.vertex_count == 0 || M.triangle_count == 0 || M.width == 0 || M.height == 0)
            return set_error(PDR_INVALID_ARGUMENT, "every batch mesh needs positions, indices, viewports, raster and "
                                                   "derivative buffers and positive sizes");
        if ((A > 0) != (M.attributes != nullptr) || (A > 0 && !M.interpolated))
            return set_error(PDR_INVALID_ARGUMENT, "with attribute_count > 0 every mesh has attributes and an output");
        if (M.uv_attributes && !M.uv) return set_error(PDR_INVALID_ARGUMENT, "uv attributes need a uv output");
        if (M.texture && (!M.uv_attributes || !M.sampled || M.texture_width == 0 || M.texture_height == 0))
            return set_error(PDR_INVALID_ARGUMENT, "a texture needs uv attributes, a sampled output and positive sizes");
        if (M.width > 65535u * 8 || M.height > 65535u * 8)
            return set_error(PDR_OVERFLOW, "Rasterization output size overflow");
        if (need_grads) {
            if (!M.grad_clip_positions || (A > 0 && (!M.grad_interpolated || !M.grad_attributes)) ||
                (M.texture && (!M.grad_sampled || !M.grad_texture || !M.grad_uv_attributes)))
                return set_error(PDR_INVALID_ARGUMENT, "batch backward needs the gradient buffers of every mesh");
            // vertex gradients are added with vector reductions: clip as float4, uv as float2
            if (((uintptr_t)M.grad_clip_positions & 15u) || ((uintptr_t)M.grad_uv_attributes & 7u) ||
                ((uintptr_t)M.grad_texture & 15u) || ((uintptr_t)M.grad_attributes & 15u))
                return set_error(PDR_INVALID_ARGUMENT,
                                 "gradient outputs must be 16-byte (clip, texture, attributes) / 8-byte (uv) aligned");
        }
        const size_t P = (size_t)M.width * M.height;
        const uint32_t tcx = (M.width + cfg->tile_width - 1) / cfg->tile_width;
        const uint32_t tcy = (M.height + cfg->tile_height - 1) / cfg->tile_height;
        const uint32_t btcx = (M.width + kTile - 1) / kTile, btcy = (M.height + kTile - 1) / kTile;
        for (uint32_t k = 0; k < M.views; ++k) {
            BatchJob j{};
            j.clip = reinterpret_cast<const float4*>(M.clip_positions) + (size_t)k * M.vertex_count;
            j.idx = reinterpret_cast<const uint3*>(M.indices);
            j.vp = reinterpret_cast<const float4*>(M.viewports) + k;
            j.V = M.vertex_count;
            j.T = M.triangle_count;
            j.W = M.width;
            j.H = M.height;
            j.tcx = tcx;
            j.btcx = btcx;
            j.attrs = M.attributes;
            j.uv_attrs = reinterpret_cast<const float2*>(M.uv_attributes);
            j.tex = reinterpret_cast<const float4*>(M.texture);
            j.tw = M.texture_width;
            j.th = M.texture_height;
            j.raster = reinterpret_cast<float4*>(M.raster) + k * P;
            j.deriv = reinterpret_cast<float4*>(M.barycentric_derivatives) + k * P;
            j.interp = M.interpolated ? M.interpolated + k * P * A : nullptr;
            j.uv = M.uv ? reinterpret_cast<float2*>(M.uv) + k * P : nullptr;
            j.sampled = M.sampled ? reinterpret_cast<float4*>(M.sampled) + k * P : nullptr;
            j.grad_interp = M.grad_interpolated ? M.grad_interpolated + k * P * A : nullptr;
            j.grad_sampled = M.grad_sampled ? reinterpret_cast<const float4*>(M.grad_sampled) + k * P : nullptr;
            j.g_clip = M.grad_clip_positions ? M.grad_clip_positions + (size_t)k * M.vertex_count * 4 : nullptr;
            j.g_attr = M.grad_attributes;
            j.g_uv = M.grad_uv_attributes;
            j.g_tex = M.grad_texture;
            plan->jobs.push_back(j);
            plan->tri_base.push_back(plan->tri_base.back() + M.triangle_count);
            plan->tile_base.push_back(plan->tile_base.back() + (unsigned long long)tcx * tcy);
            plan->btile_base.push_back(plan->btile_base.back() + (unsigned long long)btcx * btcy);
        }
    }
    plan->total_tris = plan->tri_base.back();
    plan->segs = plan->tile_base.back();
    plan->btiles = plan->btile_base.back();
    if (plan->jobs.size() > 0xffffffffull || plan->segs >= 0x7fffffffull || plan->btiles >= 0x7fffffffull)
        return set_error(PDR_OVERFLOW, "batch exceeds the launch limits");
    return PDR_OK;
}

struct BatchWorkspace {
    BatchJob* jobs;
    unsigned long long *tri_base, *tile_base, *btile_base;
    TriRect* rects;
    uint32_t *counts, *cursor;
    unsigned long long* block_sums;
    size_t bytes;
};

BatchWorkspace layout(void* base, const BatchPlan& p) {
    BatchWorkspace w{};
    char* c = static_cast<char*>(base);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* r = c ? c + off : nullptr;
        off += align_up(bytes);
        return r;
    };
    const size_t nj = p.jobs.size();
    w.jobs = reinterpret_cast<BatchJob*>(take(nj * sizeof(BatchJob)));
    w.tri_base = reinterpret_cast<unsigned long long*>(take((nj + 1) * 8));
    w.tile_base = reinterpret_cast<unsigned long long*>(take((nj + 1) * 8));
    w.btile_base = reinterpret_cast<unsigned long long*>(take((nj + 1) * 8));
    w.rects = reinterpret_cast<TriRect*>(take(p.total_tris * sizeof(TriRect)));
    w.counts = reinterpret_cast<uint32_t*>(take((p.segs + 1) * 4));
    w.cursor = reinterpret_cast<uint32_t*>(take((p.segs + 1) * 4));
    w.block_sums = reinterpret_cast<unsigned long long*>(take(scan_block_count(p.segs) * 8));
    w.bytes = off;
    return w;
}

cudaError_t upload_plan(const BatchWorkspace& w, const BatchPlan& p, cudaStream_t s) {
    const size_t nj = p.jobs.size();
    cudaError_t e = cudaMemcpyAsync(w.jobs, p.jobs.data(), nj * sizeof(BatchJob), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.tri_base, p.tri_base.data(), (nj + 1) * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.tile_base, p.tile_base.data(), (nj + 1) * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.btile_base, p.btile_base.data(), (nj + 1) * 8, cudaMemcpyHostToDevice, s);
    // the host vectors die on return: make sure the copies have read them
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

template <int TW, int TH, int CHUNK>
cudaError_t launch_batch_raster(const BatchWorkspace& w, const BatchPlan& p, const uint32_t* offsets,
                                const uint32_t* list, unsigned long long capacity, uint32_t A, uint32_t cull,
                                uint32_t mode, cudaStream_t s) {
    batch_raster_kernel<TW, TH, CHUNK><<<(unsigned)p.segs, TW * TH, 0, s>>>(
        w.jobs, w.tile_base, (uint32_t)p.jobs.size(), offsets, list, capacity, A, cull, mode);
    return cudaGetLastError();
}

}  // namespace
}  // namespace pdr

using namespace pdr;

extern "C" {

pdr_status pdr_render_batch_sizes(const pdr_render_mesh* meshes, uint32_t mesh_count, const pdr_batch_config* config,
                                  uint32_t attribute_count, uint64_t* tile_segments, size_t* workspace_bytes) {
    if (!tile_segments || !workspace_bytes) return set_error(PDR_INVALID_ARGUMENT, "size outputs are required");
    BatchPlan plan;
    const pdr_status st = plan_batch(meshes, mesh_count, config, attribute_count, false, &plan);
    if (st) return st;
    *tile_segments = plan.segs;
    *workspace_bytes = layout(nullptr, plan).bytes;
    return PDR_OK;
}

pdr_status pdr_render_batch_forward(const pdr_render_mesh* meshes, uint32_t mesh_count, uint32_t attribute_count,
                                    uint32_t cull_mode, uint32_t address_mode, const pdr_batch_config* config,
                                    uint32_t* tile_offsets, uint32_t* tile_triangles, uint64_t capacity,
                                    void* workspace, size_t workspace_bytes, uint32_t* status, void* stream) {
    if (!tile_offsets || !workspace || !status || (capacity && !tile_triangles))
        return set_error(PDR_INVALID_ARGUMENT, "tile bins, workspace and status are required");
    if (cull_mode > 2 || address_mode > 2) return set_error(PDR_INVALID_ARGUMENT, "cull or address mode out of range");
    BatchPlan plan;
    pdr_status st = plan_batch(meshes, mesh_count, config, attribute_count, false, &plan);
    if (st) return st;
    const BatchWorkspace w = layout(workspace, plan);
    if (workspace_bytes < w.bytes) return set_error(PDR_INVALID_ARGUMENT, "workspace is smaller than the batch needs");
    const cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = upload_plan(w, plan, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.counts, 0, (plan.segs + 1) * 4, s);
    if (e != cudaSuccess) return set_cuda_error(e, "render_batch_forward(set-up)");
    const unsigned blocks = (unsigned)((plan.total_tris + 255) / 256);
    const uint32_t nj = (uint32_t)plan.jobs.size();
    batch_bin_count_kernel<<<blocks, 256, 0, s>>>(w.jobs, w.tri_base, w.tile_base, nj, plan.total_tris,
                                                  config->tile_width, config->tile_height, w.rects, w.counts);
    e = launch_scan_counts(w.counts, plan.segs, tile_offsets, w.block_sums, w.cursor, status, capacity, s);
    if (e != cudaSuccess) return set_cuda_error(e, "render_batch_forward(scan)");
    batch_bin_fill_kernel<<<blocks, 256, 0, s>>>(w.jobs, w.tri_base, w.tile_base, nj, plan.total_tris, w.rects,
                                                 w.cursor, tile_triangles, capacity);
    const uint32_t tw = config->tile_width, th = config->tile_height, k = config->stage_triangles;
    if (tw == 16 && th == 8) e = launch_batch_raster<16, 8, 128>(w, plan, tile_offsets, tile_triangles, capacity,
                                                                 attribute_count, cull_mode, address_mode, s);
    else if (tw == 16 && k == 128) e = launch_batch_raster<16, 16, 128>(w, plan, tile_offsets, tile_triangles, capacity,
                                                                       attribute_count, cull_mode, address_mode, s);
    else e = launch_batch_raster<16, 16, 256>(w, plan, tile_offsets, tile_triangles, capacity, attribute_count,
                                              cull_mode, address_mode, s);
    return set_cuda_error(e, "render_batch_forward");
}

pdr_status pdr_render_batch_backward(const pdr_render_mesh* meshes, uint32_t mesh_count, uint32_t attribute_count,
                                     uint32_t address_mode, const pdr_batch_config* config, void* workspace,
                                     size_t workspace_bytes, uint32_t* status, void* stream) {
    if (!workspace || !status) return set_error(PDR_INVALID_ARGUMENT, "workspace and status are required");
    if (address_mode > 2) return set_error(PDR_INVALID_ARGUMENT, "address mode out of range");
    BatchPlan plan;
    pdr_status st = plan_batch(meshes, mesh_count, config, attribute_count, true, &plan);
    if (st) return st;
    const BatchWorkspace w = layout(workspace, plan);
    if (workspace_bytes < w.bytes) return set_error(PDR_INVALID_ARGUMENT, "workspace is smaller than the batch needs");
    const cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = upload_plan(w, plan, s);
    for (uint32_t m = 0; m < mesh_count && e == cudaSuccess; ++m) {
        const pdr_render_mesh& M = meshes[m];
        e = cudaMemsetAsync(M.grad_clip_positions, 0, (size_t)M.views * M.vertex_count * 4 * sizeof(float), s);
        if (e == cudaSuccess && M.grad_attributes)
            e = cudaMemsetAsync(M.grad_attributes, 0, (size_t)M.vertex_count * attribute_count * sizeof(float), s);
        if (e == cudaSuccess && M.grad_uv_attributes)
            e = cudaMemsetAsync(M.grad_uv_attributes, 0, (size_t)M.vertex_count * 2 * sizeof(float), s);
        if (e == cudaSuccess && M.grad_texture)
            e = cudaMemsetAsync(M.grad_texture, 0, (size_t)M.texture_width * M.texture_height * 4 * sizeof(float), s);
    }
    if (e != cudaSuccess) return set_cuda_error(e, "render_batch_backward(set-up)");
    const uint32_t nj = (uint32_t)plan.jobs.size();
    const unsigned grid = (unsigned)plan.btiles;
#define PDR_BATCH_BWD(KA) batch_backward_kernel<KA><<<grid, kFusedThreads, 0, s>>>(w.jobs, w.btile_base, nj, address_mode, status)
    switch (attribute_count) {
        case 0: PDR_BATCH_BWD(0); break;
        case 1: PDR_BATCH_BWD(1); break;
        case 2: PDR_BATCH_BWD(2); break;
        case 3: PDR_BATCH_BWD(3); break;
        case 4: PDR_BATCH_BWD(4); break;
        case 5: PDR_BATCH_BWD(5); break;
        case 6: PDR_BATCH_BWD(6); break;
        case 7: PDR_BATCH_BWD(7); break;
        default: PDR_BATCH_BWD(8); break;
    }
#undef PDR_BATCH_BWD
    return set_cuda_error(cudaGetLastError(), "render_batch_backward");
}

}  // extern "C"

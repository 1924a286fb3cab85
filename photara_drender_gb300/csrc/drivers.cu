// C ABI for the bake and refine paths, and the native refinement driver (one CUDA graph for the
// whole TextureRefiner::refine loop, src/texture_refiner.cpp:304-426).
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

thread_local std::string g_driver_error;

pdr_status fail(pdr_status code, const char* msg);
pdr_status cuda_status(cudaError_t err, const char* what);

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

pdr_status check_refine_options(const pdr_refine_options* o) {
    if (!o) return fail(PDR_INVALID_ARGUMENT, "texture refinement options are invalid");
    const bool ok = o->width && o->height && o->steps && o->batch_size && std::isfinite(o->learning_rate) &&
                    o->learning_rate > 0.0f && std::isfinite(o->minimum_learning_rate) &&
                    o->minimum_learning_rate >= 0.0f && o->minimum_learning_rate <= o->learning_rate &&
                    std::isfinite(o->photometric_epsilon) && o->photometric_epsilon > 0.0f &&
                    o->adam_beta1 > 0.0f && o->adam_beta1 < 1.0f && o->adam_beta2 > 0.0f && o->adam_beta2 < 1.0f &&
                    o->clamp_min < o->clamp_max && std::isfinite(o->seam_learning_rate) &&
                    o->seam_learning_rate > 0.0f && std::isfinite(o->seam_epsilon) && o->seam_epsilon > 0.0f &&
                    std::isfinite(o->tv_scale) && o->tv_scale >= 0.0f;
    if (!ok) return fail(PDR_INVALID_ARGUMENT, "texture refinement options are invalid");
    if ((uint64_t)o->width * o->height * 3 > 0xffffffffull)
        return fail(PDR_OVERFLOW, "texture refinement atlas exceeds the shader element limit");
    return PDR_OK;
}

// Enqueues the whole optimisation on `stream` (capturable: kernels and memsets only).
pdr_status enqueue_refine(const pdr_refine_options* o, const pdr_refine_view* views, uint32_t nviews,
                          const double* valid_weights, uint64_t max_pixels, const float* pairs, uint32_t npairs,
                          const uint8_t* tv_valid, const int32_t* tv_chart, float* tex, float* grad, float* m1,
                          float* m2, float* loss, cudaStream_t stream) {
    const size_t n = (size_t)o->width * o->height * 3;
    const uint32_t seam_steps = npairs == 0 ? 0u : o->seam_polish_steps;
    cudaError_t err = cudaSuccess;
    auto chk = [&](cudaError_t e) {
        if (err == cudaSuccess && e != cudaSuccess) err = e;
    };
    chk(cudaMemsetAsync(loss, 0, (size_t)(o->steps + seam_steps) * sizeof(float), stream));
    chk(cudaMemsetAsync(grad, 0, n * sizeof(float), stream));
    chk(cudaMemsetAsync(m1, 0, n * sizeof(float), stream));
    chk(cudaMemsetAsync(m2, 0, n * sizeof(float), stream));
    for (uint32_t step = 0; step < o->steps && err == cudaSuccess; ++step) {
        // texture_refiner.cpp:317-324
        double bvw = 0.0;
        for (uint32_t b = 0; b < o->batch_size; ++b) bvw += valid_weights[((size_t)step * o->batch_size + b) % nviews];
        const float norm = bvw > 0.0 ? static_cast<float>(1.0 / (bvw * 3.0)) : 0.0f;
        chk(launch_photometric(tex, o->width, o->height, views, nviews, max_pixels, step, o->batch_size,
                               o->photometric_epsilon, norm, grad, loss, stream));
        if (o->tv_scale > 0.0f && tv_valid)
            chk(launch_tv(tex, o->width, o->height, tv_valid, tv_chart, o->tv_epsilon, o->tv_scale, grad, stream));
        float lr, bc1, bc2;
        refine_schedule(o, step, &lr, &bc1, &bc2);
        chk(launch_adam(tex, grad, m1, m2, n, lr, o->adam_beta1, o->adam_beta2, o->adam_epsilon, bc1, bc2, o->clamp_min,
                        o->clamp_max, stream));
    }
    if (seam_steps) {
        // texture_refiner.cpp:371-415: reset gradient and moments, then seam + Adam steps
        chk(cudaMemsetAsync(grad, 0, n * sizeof(float), stream));
        chk(cudaMemsetAsync(m1, 0, n * sizeof(float), stream));
        chk(cudaMemsetAsync(m2, 0, n * sizeof(float), stream));
        const float norm = 1.0F / static_cast<float>(npairs * 3u);
        for (uint32_t s = 0; s < seam_steps && err == cudaSuccess; ++s) {
            chk(launch_seam(tex, o->width, o->height, pairs, npairs, o->seam_epsilon, norm, grad, loss, o->steps + s,
                            stream));
            const float bc1 = 1.0F - std::pow(o->adam_beta1, static_cast<float>(s + 1));
            const float bc2 = 1.0F - std::pow(o->adam_beta2, static_cast<float>(s + 1));
            chk(launch_adam(tex, grad, m1, m2, n, o->seam_learning_rate, o->adam_beta1, o->adam_beta2, o->adam_epsilon,
                            bc1, bc2, o->clamp_min, o->clamp_max, stream));
        }
    }
    return cuda_status(err, "refine");
}

pdr_status check_refine_run(const pdr_refine_options* o, const pdr_refine_view* views, uint32_t nviews,
                            const double* valid_weights, uint64_t max_pixels, const float* pairs, uint32_t npairs,
                            float* tex, float* grad, float* m1, float* m2, float* loss) {
    pdr_status st = check_refine_options(o);
    if (st) return st;
    if (!views || nviews == 0 || !valid_weights || max_pixels == 0)
        return fail(PDR_INVALID_ARGUMENT, "texture refinement needs at least one view");
    if (max_pixels > 0xffffffffull) return fail(PDR_INVALID_ARGUMENT, "texture refinement image or mask has an invalid shape");
    if (!tex || !grad || !m1 || !m2 || !loss) return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers are required");
    if (!aligned(tex, 16) || !aligned(grad, 16) || !aligned(m1, 16) || !aligned(m2, 16))
        return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers must be 16-byte aligned");
    if (npairs && (!pairs || !aligned(pairs, 16))) return fail(PDR_INVALID_ARGUMENT, "seam_uv_pairs must be 16-byte aligned");
    return PDR_OK;
}

}  // namespace

// error helpers shared with capi.cu through the thread-local message there
pdr_status set_error(pdr_status code, const char* msg);
pdr_status set_cuda_error(cudaError_t err, const char* what);

namespace {
pdr_status fail(pdr_status code, const char* msg) { return set_error(code, msg); }
pdr_status cuda_status(cudaError_t err, const char* what) { return set_cuda_error(err, what); }
}  // namespace

}  // namespace pdr

using namespace pdr;

struct pdr_refine_graph_t {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" {

pdr_status pdr_transform_positions(const float* pos, uint32_t V, const float* mats, uint32_t views, float* clip,
                                   void* stream) {
    if (!pos || !mats || !clip || V == 0 || views == 0) return fail(PDR_INVALID_ARGUMENT, "positions must have shape [vertex_count, 3]");
    if (!aligned(clip, 16)) return fail(PDR_INVALID_ARGUMENT, "clip_positions must be 16-byte aligned");
    return cuda_status(launch_transform_positions(pos, V, mats, views, clip, (cudaStream_t)stream), "transform_positions");
}

pdr_status pdr_atlas_clip_positions(const float* uv, uint32_t V, float* clip, void* stream) {
    if (!uv || !clip || V == 0) return fail(PDR_INVALID_ARGUMENT, "uv must have shape [vertex_count, 2]");
    if (!aligned(uv, 8) || !aligned(clip, 16)) return fail(PDR_INVALID_ARGUMENT, "uv/clip buffers are misaligned");
    return cuda_status(launch_atlas_clip(uv, V, clip, (cudaStream_t)stream), "atlas_clip_positions");
}

pdr_status pdr_project_views(const float* apos, const float* anrm, const float* araster, uint32_t N,
                             const pdr_projection_view* views, uint32_t nviews, uint32_t blend_mode, uint32_t pcf_radius,
                             uint32_t visibility_mode, float* color, float* confidence, uint32_t* source_view,
                             float* valid_mask, float* coverage_mask, uint32_t* face_ids, void* stream) {
    if (!apos || !anrm || !araster || !views || !color || !confidence || !source_view || !valid_mask)
        return fail(PDR_INVALID_ARGUMENT, "projection buffers are required");
    if (N == 0) return fail(PDR_INVALID_ARGUMENT, "atlas dimensions are invalid or pcf_radius exceeds 4");
    if (nviews == 0) return fail(PDR_INVALID_ARGUMENT, "at least one projection view is required");
    if (pcf_radius > 4 || blend_mode > 2 || visibility_mode > 2)
        return fail(PDR_INVALID_ARGUMENT, "atlas dimensions are invalid or pcf_radius exceeds 4");
    if (!aligned(araster, 16) || !aligned(color, 16) || !aligned(views, 16))
        return fail(PDR_INVALID_ARGUMENT, "projection buffers must be 16-byte aligned");
    return cuda_status(launch_project_views(apos, anrm, araster, N, views, nviews, blend_mode, pcf_radius,
                                            visibility_mode, color, confidence, source_view, valid_mask, coverage_mask,
                                            face_ids, (cudaStream_t)stream),
                       "project_views");
}

pdr_status pdr_refine_prepare_view(const float* image, uint32_t C, const float* mask, const float* raster, uint64_t P,
                                   float* target, float* out_mask, void* stream) {
    if (!image || !raster || !target || !out_mask || P == 0 || (C != 3 && C != 4))
        return fail(PDR_INVALID_ARGUMENT, "texture refinement images must contain RGB or RGBA data");
    if (!aligned(raster, 16)) return fail(PDR_INVALID_ARGUMENT, "raster must be 16-byte aligned");
    return cuda_status(launch_prepare_view(image, C, mask, raster, P, target, out_mask, (cudaStream_t)stream),
                       "refine_prepare_view");
}

pdr_status pdr_refine_photometric(const float* tex, uint32_t W, uint32_t H, const pdr_refine_view* views, uint32_t nviews,
                                  uint64_t max_pixels, uint32_t step, uint32_t batch, float eps, float norm, float* grad,
                                  float* loss, void* stream) {
    if (!tex || !views || !grad || !loss || nviews == 0 || batch == 0 || W == 0 || H == 0)
        return fail(PDR_INVALID_ARGUMENT, "texture refinement options are invalid");
    return cuda_status(launch_photometric(tex, W, H, views, nviews, max_pixels, step, batch, eps, norm, grad, loss,
                                          (cudaStream_t)stream),
                       "refine_photometric");
}

pdr_status pdr_refine_seam(const float* tex, uint32_t W, uint32_t H, const float* pairs, uint32_t npairs, float eps,
                           float norm, float* grad, float* loss, uint32_t loss_index, void* stream) {
    if (!tex || !grad || !loss || W == 0 || H == 0 || (npairs && (!pairs || !aligned(pairs, 16))))
        return fail(PDR_INVALID_ARGUMENT, "seam_uv_pairs must have shape [pair_count, 2, 2]");
    if (npairs == 0) return PDR_OK;
    return cuda_status(launch_seam(tex, W, H, pairs, npairs, eps, norm, grad, loss, loss_index, (cudaStream_t)stream),
                       "refine_seam");
}

pdr_status pdr_refine_total_variation(const float* tex, uint32_t W, uint32_t H, const uint8_t* valid, const int32_t* chart,
                                      float eps, float scale, float* grad, void* stream) {
    if (!tex || !valid || !grad || W == 0 || H == 0) return fail(PDR_INVALID_ARGUMENT, "valid_mask must have shape [texture_height, texture_width]");
    return cuda_status(launch_tv(tex, W, H, valid, chart, eps, scale, grad, (cudaStream_t)stream), "refine_total_variation");
}

pdr_status pdr_refine_adam(float* tex, float* grad, float* m1, float* m2, uint64_t n, float lr, float b1, float b2,
                           float eps, float bc1, float bc2, float cmin, float cmax, void* stream) {
    if (!tex || !grad || !m1 || !m2) return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers are required");
    if (!aligned(tex, 16) || !aligned(grad, 16) || !aligned(m1, 16) || !aligned(m2, 16))
        return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers must be 16-byte aligned");
    if (n == 0) return PDR_OK;
    return cuda_status(launch_adam(tex, grad, m1, m2, n, lr, b1, b2, eps, bc1, bc2, cmin, cmax, (cudaStream_t)stream),
                       "refine_adam");
}

pdr_status pdr_refine_schedule(const pdr_refine_options* o, uint32_t step, float* lr, float* bc1, float* bc2) {
    if (!o || !lr || !bc1 || !bc2 || o->steps == 0) return fail(PDR_INVALID_ARGUMENT, "texture refinement options are invalid");
    refine_schedule(o, step, lr, bc1, bc2);
    return PDR_OK;
}

pdr_status pdr_refine_run(const pdr_refine_options* o, const pdr_refine_view* views, uint32_t nviews,
                          const double* valid_weights, uint64_t max_pixels, const float* pairs, uint32_t npairs,
                          const uint8_t* tv_valid, const int32_t* tv_chart, float* tex, float* grad, float* m1, float* m2,
                          float* loss, int32_t use_graph, void* stream) {
    pdr_status st = check_refine_run(o, views, nviews, valid_weights, max_pixels, pairs, npairs, tex, grad, m1, m2, loss);
    if (st) return st;
    if (!use_graph)
        return enqueue_refine(o, views, nviews, valid_weights, max_pixels, pairs, npairs, tv_valid, tv_chart, tex, grad,
                              m1, m2, loss, (cudaStream_t)stream);
    pdr_refine_graph g = nullptr;
    st = pdr_refine_graph_create(&g, o, views, nviews, valid_weights, max_pixels, pairs, npairs, tv_valid, tv_chart, tex,
                                 grad, m1, m2, loss, stream);
    if (st) return st;
    st = pdr_refine_graph_launch(g, stream);
    pdr_refine_graph_destroy(g);
    return st;
}

pdr_status pdr_refine_graph_create(pdr_refine_graph* out, const pdr_refine_options* o, const pdr_refine_view* views,
                                   uint32_t nviews, const double* valid_weights, uint64_t max_pixels, const float* pairs,
                                   uint32_t npairs, const uint8_t* tv_valid, const int32_t* tv_chart, float* tex,
                                   float* grad, float* m1, float* m2, float* loss, void* stream) {
    if (!out) return fail(PDR_INVALID_ARGUMENT, "graph handle is required");
    *out = nullptr;
    pdr_status st = check_refine_run(o, views, nviews, valid_weights, max_pixels, pairs, npairs, tex, grad, m1, m2, loss);
    if (st) return st;
    // record on a private stream so the caller's stream is never left in capture mode
    cudaStream_t cap = nullptr;
    cudaError_t err = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (err != cudaSuccess) return cuda_status(err, "cudaStreamCreate");
    auto* g = new pdr_refine_graph_t();
    err = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) {
        st = enqueue_refine(o, views, nviews, valid_weights, max_pixels, pairs, npairs, tv_valid, tv_chart, tex, grad, m1,
                            m2, loss, cap);
        const cudaError_t end = cudaStreamEndCapture(cap, &g->graph);
        if (st == PDR_OK && end != cudaSuccess) st = cuda_status(end, "cudaStreamEndCapture");
    } else {
        st = cuda_status(err, "cudaStreamBeginCapture");
    }
    if (st == PDR_OK) {
        err = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (err != cudaSuccess) st = cuda_status(err, "cudaGraphInstantiate");
    }
    cudaStreamDestroy(cap);
    (void)stream;
    if (st != PDR_OK) {
        pdr_refine_graph_destroy(g);
        return st;
    }
    *out = g;
    return PDR_OK;
}

pdr_status pdr_refine_graph_launch(pdr_refine_graph g, void* stream) {
    if (!g || !g->exec) return fail(PDR_INVALID_ARGUMENT, "graph handle is invalid");
    return cuda_status(cudaGraphLaunch(g->exec, (cudaStream_t)stream), "cudaGraphLaunch");
}

pdr_status pdr_refine_graph_destroy(pdr_refine_graph g) {
    if (!g) return PDR_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return PDR_OK;
}

}  // extern "C"

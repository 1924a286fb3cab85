// C ABI for the bake and refine paths, and the native refinement driver (one CUDA graph for the
// whole TextureRefiner::refine loop, src/texture_refiner.cpp:304-426).
#include <cuda_runtime.h>

#include <cmath>

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
                          float* m2, float* loss, cudaStream_t stream, const pdr_precond_run* pc = nullptr) {
    const size_t n = (size_t)o->width * o->height * 3;
    const uint32_t seam_steps = npairs == 0 ? 0u : o->seam_polish_steps;
    cudaError_t err = cudaSuccess;
    auto chk = [&](cudaError_t e) {
        if (err == cudaSuccess && e != cudaSuccess) err = e;
    };
    chk(cudaMemsetAsync(loss, 0, (size_t)(o->steps + seam_steps) * sizeof(float), stream));
    const uint64_t texels = (uint64_t)o->width * o->height;
    chk(cudaMemsetAsync(grad, 0, texels * 4 * sizeof(float), stream));  // [texels][4]
    chk(cudaMemsetAsync(m1, 0, n * sizeof(float), stream));
    chk(cudaMemsetAsync(m2, 0, n * sizeof(float), stream));
    if (pc) chk(cudaMemsetAsync(pc->fallback, 0, sizeof(uint32_t), stream));
    // plain refinement with TV and a second atlas buffer: TV + Adam in one pass, the texture alternating
    // between the two buffers (the one read this step, the one written)
    const bool fused_tv = !pc && o->tv_scale > 0.0f && tv_valid && o->texture_scratch;
    float* cur = tex;
    float* other = fused_tv ? o->texture_scratch : nullptr;
    for (uint32_t step = 0; fused_tv && step < o->steps && err == cudaSuccess; ++step) {
        double bvw = 0.0;
        for (uint32_t b = 0; b < o->batch_size; ++b) bvw += valid_weights[((size_t)step * o->batch_size + b) % nviews];
        const float norm = bvw > 0.0 ? static_cast<float>(1.0 / (bvw * 3.0)) : 0.0f;
        chk(launch_photometric(cur, o->width, o->height, views, nviews, max_pixels, step, o->batch_size,
                               o->photometric_epsilon, norm, grad, loss, stream));
        float lr, bc1, bc2;
        refine_schedule(o, step, &lr, &bc1, &bc2);
        chk(launch_adam_tv(cur, other, grad, m1, m2, o->width, o->height, tv_valid, tv_chart, o->tv_epsilon,
                           o->tv_scale, lr, o->adam_beta1, o->adam_beta2, o->adam_epsilon, bc1, bc2, o->clamp_min,
                           o->clamp_max, stream));
        float* t = cur;
        cur = other;
        other = t;
    }
    if (fused_tv && cur != tex) chk(cudaMemcpyAsync(tex, cur, n * sizeof(float), cudaMemcpyDeviceToDevice, stream));
    for (uint32_t step = 0; !fused_tv && step < o->steps && err == cudaSuccess; ++step) {
        if (pc && step % pc->refresh_interval == 0) {
            // learned multipliers from the state after `step` updates (moments corrected for that count)
            const uint32_t K = pc->refresh_interval;
            if (step >= 2 * K) chk(launch_fallback_check(loss, step - 2 * K, K, pc->fallback_tolerance, pc->fallback, stream));
            float lr_prev = 0.0f, bc1 = 1.0f, bc2 = 1.0f;
            if (step > 0) refine_schedule(o, step - 1, &lr_prev, &bc1, &bc2);
            chk(launch_precond_features(tex, m1, m2, bc1, bc2, o->adam_epsilon, pc->observation, pc->view_counts,
                                        pc->edge_distance, (float)step / (float)o->steps, texels, pc->features, stream));
            chk(launch_precond_forward(pc->params, pc->params_bf16, pc->features, texels, pc->multipliers, pc->status,
                                       stream));
        }
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
        if (pc)
            chk(launch_adam_scaled(tex, grad, m1, m2, texels, pc->multipliers, pc->fallback, lr, o->adam_beta1,
                                   o->adam_beta2, o->adam_epsilon, bc1, bc2, o->clamp_min, o->clamp_max, stream));
        else
            chk(launch_adam(tex, grad, m1, m2, n, lr, o->adam_beta1, o->adam_beta2, o->adam_epsilon, bc1, bc2,
                            o->clamp_min, o->clamp_max, stream));
    }
    if (seam_steps) {
        // texture_refiner.cpp:371-415: reset gradient and moments, then seam + Adam steps
        chk(cudaMemsetAsync(grad, 0, texels * 4 * sizeof(float), stream));
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
    if (!aligned(tex, 16) || !aligned(grad, 16) || !aligned(m1, 16) || !aligned(m2, 16) ||
        !aligned(o->texture_scratch, 16))
        return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers must be 16-byte aligned");
    if (o->texture_scratch && (o->texture_scratch == tex || o->texture_scratch == m1 || o->texture_scratch == m2))
        return fail(PDR_INVALID_ARGUMENT, "texture_scratch must be a buffer of its own");
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

namespace {

// Records `enqueue(stream)` on a private stream (the caller's stream is never left in capture mode)
// and instantiates the graph.
template <class Enqueue>
pdr_status capture_graph(pdr_refine_graph* out, Enqueue&& enqueue) {
    cudaStream_t cap = nullptr;
    cudaError_t err = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (err != cudaSuccess) return cuda_status(err, "cudaStreamCreate");
    auto* g = new pdr_refine_graph_t();
    pdr_status st = PDR_OK;
    err = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) {
        st = enqueue(cap);
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
    if (st != PDR_OK) {
        pdr_refine_graph_destroy(g);
        return st;
    }
    *out = g;
    return PDR_OK;
}

bool precond_params_ok(const float* params, const uint16_t* wbf) {
    return params && wbf && aligned(wbf, 16) && aligned(params, 4);
}

}  // namespace

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
    if (!aligned(grad, 16)) return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers must be 16-byte aligned");
    return cuda_status(launch_photometric(tex, W, H, views, nviews, max_pixels, step, batch, eps, norm, grad, loss,
                                          (cudaStream_t)stream),
                       "refine_photometric");
}

pdr_status pdr_refine_seam(const float* tex, uint32_t W, uint32_t H, const float* pairs, uint32_t npairs, float eps,
                           float norm, float* grad, float* loss, uint32_t loss_index, void* stream) {
    if (!tex || !grad || !loss || W == 0 || H == 0 || (npairs && (!pairs || !aligned(pairs, 16))))
        return fail(PDR_INVALID_ARGUMENT, "seam_uv_pairs must have shape [pair_count, 2, 2]");
    if (!aligned(grad, 16)) return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers must be 16-byte aligned");
    if (npairs == 0) return PDR_OK;
    return cuda_status(launch_seam(tex, W, H, pairs, npairs, eps, norm, grad, loss, loss_index, (cudaStream_t)stream),
                       "refine_seam");
}

pdr_status pdr_refine_total_variation(const float* tex, uint32_t W, uint32_t H, const uint8_t* valid, const int32_t* chart,
                                      float eps, float scale, float* grad, void* stream) {
    if (!tex || !valid || !grad || W == 0 || H == 0) return fail(PDR_INVALID_ARGUMENT, "valid_mask must have shape [texture_height, texture_width]");
    if (!aligned(grad, 16)) return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers must be 16-byte aligned");
    return cuda_status(launch_tv(tex, W, H, valid, chart, eps, scale, grad, (cudaStream_t)stream), "refine_total_variation");
}

pdr_status pdr_refine_adam(float* tex, float* grad, float* m1, float* m2, uint64_t n, float lr, float b1, float b2,
                           float eps, float bc1, float bc2, float cmin, float cmax, void* stream) {
    if (!tex || !grad || !m1 || !m2) return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers are required");
    if (!aligned(tex, 16) || !aligned(grad, 16) || !aligned(m1, 16) || !aligned(m2, 16))
        return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers must be 16-byte aligned");
    if (n % 3) return fail(PDR_INVALID_ARGUMENT, "texture refinement values must be RGB texels (a multiple of 3)");
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
    (void)stream;
    return capture_graph(out, [&](cudaStream_t cap) {
        return enqueue_refine(o, views, nviews, valid_weights, max_pixels, pairs, npairs, tv_valid, tv_chart, tex, grad,
                              m1, m2, loss, cap);
    });
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


pdr_status pdr_precond_forward(const float* params, const uint16_t* wbf, const uint16_t* features, uint64_t count,
                               float* out, uint32_t* status, void* stream) {
    if (!precond_params_ok(params, wbf) || !features || !out || !status)
        return fail(PDR_INVALID_ARGUMENT, "preconditioner buffers are required (BF16 buffers 16-byte aligned)");
    if (!aligned(features, 16) || !aligned(out, 16)) return fail(PDR_INVALID_ARGUMENT, "features/out must be 16-byte aligned");
    if (count == 0) return PDR_OK;
    return cuda_status(launch_precond_forward(params, wbf, features, count, out, status, (cudaStream_t)stream),
                       "precond_forward");
}

pdr_status pdr_precond_train_step(const float* params, const uint16_t* wbf, const uint16_t* features,
                                  const float* targets, const float* weights, uint64_t count, float inv_norm,
                                  float* grads, float* loss, uint32_t* status, void* stream) {
    if (!precond_params_ok(params, wbf) || !features || !targets || !weights || !grads || !loss || !status)
        return fail(PDR_INVALID_ARGUMENT, "preconditioner buffers are required (BF16 buffers 16-byte aligned)");
    if (!aligned(features, 16) || !aligned(targets, 16) || !aligned(weights, 16))
        return fail(PDR_INVALID_ARGUMENT, "features/targets/weights must be 16-byte aligned");
    if (count == 0 || !std::isfinite(inv_norm)) return fail(PDR_INVALID_ARGUMENT, "training batch is empty");
    return cuda_status(launch_precond_train(params, wbf, features, targets, weights, count, inv_norm, grads, loss, status,
                                            (cudaStream_t)stream),
                       "precond_train_step");
}

pdr_status pdr_precond_adam(float* params, const float* grads, float* m, float* v, uint32_t step, float lr, float b1,
                            float b2, float eps, uint16_t* wbf, void* stream) {
    if (!params || !grads || !m || !v || !wbf) return fail(PDR_INVALID_ARGUMENT, "preconditioner buffers are required");
    if (!(lr > 0.0f) || !(b1 > 0.0f && b1 < 1.0f) || !(b2 > 0.0f && b2 < 1.0f) || !(eps > 0.0f))
        return fail(PDR_INVALID_ARGUMENT, "preconditioner optimiser options are invalid");
    const float bc1 = 1.0f - std::pow(b1, (float)(step + 1)), bc2 = 1.0f - std::pow(b2, (float)(step + 1));
    return cuda_status(launch_precond_adam(params, grads, m, v, lr, b1, b2, eps, bc1, bc2, wbf, (cudaStream_t)stream),
                       "precond_adam");
}

pdr_status pdr_precond_texel_stats(const pdr_refine_view* views_host, uint32_t nviews, uint32_t W, uint32_t H,
                                   const uint8_t* valid, const int32_t* chart, float* obs, float* view_counts,
                                   float* edge, uint8_t* scratch, void* stream) {
    if (!views_host || nviews == 0 || W == 0 || H == 0 || !valid || !obs || !view_counts || !edge || !scratch)
        return fail(PDR_INVALID_ARGUMENT, "texel statistics need views, the valid mask and output buffers");
    const cudaStream_t s = (cudaStream_t)stream;
    const size_t N = (size_t)W * H;
    cudaError_t err = cudaMemsetAsync(obs, 0, N * sizeof(float), s);
    if (err == cudaSuccess) err = cudaMemsetAsync(view_counts, 0, N * sizeof(float), s);
    if (err == cudaSuccess) err = cudaMemsetAsync(scratch, 0, N, s);
    for (uint32_t k = 0; k < nviews && err == cudaSuccess; ++k) {
        const pdr_refine_view& v = views_host[k];
        if (!v.uv || !v.mask) return fail(PDR_INVALID_ARGUMENT, "a cached view has no uv or mask buffer");
        err = launch_observe_view(v.uv, v.mask, v.pixel_count, W, H, obs, scratch, view_counts, s);
    }
    if (err == cudaSuccess) err = launch_edge_distance(valid, chart, W, H, edge, s);
    return cuda_status(err, "precond_texel_stats");
}

pdr_status pdr_precond_features(const float* tex, const float* m1, const float* m2, float bc1, float bc2, float eps,
                                const float* obs, const float* view_counts, const float* edge, float progress,
                                uint64_t N, uint16_t* feat, void* stream) {
    if (!tex || !m1 || !m2 || !obs || !view_counts || !edge || !feat)
        return fail(PDR_INVALID_ARGUMENT, "feature inputs are required");
    if (!aligned(feat, 16)) return fail(PDR_INVALID_ARGUMENT, "features must be 16-byte aligned");
    if (!(bc1 > 0.0f) || !(bc2 > 0.0f)) return fail(PDR_INVALID_ARGUMENT, "bias corrections must be positive");
    if (N == 0) return PDR_OK;
    return cuda_status(launch_precond_features(tex, m1, m2, bc1, bc2, eps, obs, view_counts, edge, progress, N, feat,
                                               (cudaStream_t)stream),
                       "precond_features");
}

pdr_status pdr_refine_adam_scaled(float* tex, float* grad, float* m1, float* m2, uint64_t N, const float* mult,
                                  const uint32_t* fallback, float lr, float b1, float b2, float eps, float bc1, float bc2,
                                  float cmin, float cmax, void* stream) {
    if (!tex || !grad || !m1 || !m2 || !mult || !fallback)
        return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers are required");
    if (!aligned(mult, 16) || !aligned(tex, 16) || !aligned(grad, 16) || !aligned(m1, 16) || !aligned(m2, 16))
        return fail(PDR_INVALID_ARGUMENT, "texture refinement buffers and multipliers must be 16-byte aligned");
    if (N == 0) return PDR_OK;
    return cuda_status(launch_adam_scaled(tex, grad, m1, m2, N, mult, fallback, lr, b1, b2, eps, bc1, bc2, cmin, cmax,
                                          (cudaStream_t)stream),
                       "refine_adam_scaled");
}

pdr_status pdr_precond_fallback_check(const float* loss, uint32_t begin, uint32_t window, float tolerance,
                                      uint32_t* fallback, void* stream) {
    if (!loss || !fallback || window == 0 || !(tolerance >= 0.0f))
        return fail(PDR_INVALID_ARGUMENT, "fallback check needs a loss history, a window and a flag");
    return cuda_status(launch_fallback_check(loss, begin, window, tolerance, fallback, (cudaStream_t)stream),
                       "precond_fallback_check");
}

pdr_status pdr_refine_run_learned(const pdr_refine_options* o, const pdr_refine_view* views, uint32_t nviews,
                                  const double* valid_weights, uint64_t max_pixels, const float* pairs, uint32_t npairs,
                                  const uint8_t* tv_valid, const int32_t* tv_chart, float* tex, float* grad, float* m1,
                                  float* m2, float* loss, const pdr_precond_run* pc, int32_t use_graph, void* stream) {
    pdr_status st = check_refine_run(o, views, nviews, valid_weights, max_pixels, pairs, npairs, tex, grad, m1, m2, loss);
    if (st) return st;
    if (!pc || !precond_params_ok(pc->params, pc->params_bf16) || !pc->observation || !pc->view_counts ||
        !pc->edge_distance || !pc->features || !pc->multipliers || !pc->fallback || !pc->status ||
        pc->refresh_interval == 0 || !(pc->fallback_tolerance >= 0.0f))
        return fail(PDR_INVALID_ARGUMENT, "the learned refinement state is incomplete");
    if (!aligned(pc->features, 16) || !aligned(pc->multipliers, 16))
        return fail(PDR_INVALID_ARGUMENT, "features/multipliers must be 16-byte aligned");
    // kernel attributes are set before any capture begins
    const cudaError_t init = precond_prepare();
    if (init != cudaSuccess) return cuda_status(init, "precond_prepare");
    if (!use_graph)
        return enqueue_refine(o, views, nviews, valid_weights, max_pixels, pairs, npairs, tv_valid, tv_chart, tex, grad,
                              m1, m2, loss, (cudaStream_t)stream, pc);
    pdr_refine_graph g = nullptr;
    st = capture_graph(&g, [&](cudaStream_t cap) {
        return enqueue_refine(o, views, nviews, valid_weights, max_pixels, pairs, npairs, tv_valid, tv_chart, tex, grad,
                              m1, m2, loss, cap, pc);
    });
    if (st) return st;
    st = pdr_refine_graph_launch(g, stream);
    pdr_refine_graph_destroy(g);
    return st;
}

}  // extern "C"

// Internal declarations shared by the CUDA translation units of libphotara_drender_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace pdr {

// Words of the device status block every pipeline call may write.
enum StatusWord : uint32_t {
    kStatusTotal = 0,        // tile-list entries of the last binning (low 32 bits)
    kStatusTotalHi = 1,      // high bits (non-zero means the u32 CSR overflowed)
    kStatusOverflow = 2,     // 1 when the tile list did not fit its capacity
    kStatusLargeTiles = 3,   // tiles sorted by the large-tile pass
    kStatusTexelError = 4,   // 1 = non-finite uv in a covered pixel, 2 = |texel| > 1e9
    kStatusWords = 8,
};

inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

int num_sms();

size_t bins_workspace_bytes(uint32_t views, uint32_t T, uint32_t W, uint32_t H, unsigned long long capacity,
                            uint32_t tile_w = 16, uint32_t tile_h = 16);

// Exclusive scan of per-segment counts into CSR offsets (offsets[segs] = total) and the fill cursors;
// status gets the total and the overflow flag against capacity. block_sums holds scan_block_count(segs).
cudaError_t launch_scan_counts(const uint32_t* counts, size_t segs, uint32_t* offsets, unsigned long long* block_sums,
                               uint32_t* cursor, uint32_t* status, unsigned long long capacity, cudaStream_t stream);
size_t scan_block_count(size_t segs);
cudaError_t launch_bin_tiles(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                             uint32_t W, uint32_t H, const float* viewports, uint32_t* offsets, uint32_t* list,
                             unsigned long long capacity, void* workspace, uint32_t* status, cudaStream_t stream,
                             bool sorted = true, uint32_t tile_w = 16, uint32_t tile_h = 16);

// Optional fused forward epilogue: interpolate attributes and uv for the winning triangle and sample
// a 4-channel texture at that uv, with the same arithmetic as the separate kernels.
struct RasterShade {
    const float* attrs;
    uint32_t attribute_count;
    float* attr_out;
    const float* uv_attrs;
    float* uv_out;
    const float* texture;
    uint32_t texture_width, texture_height, address_mode;
    float* sampled;
    float* sample_differences;  // optional [views][H][W][8] (pdr_render_args.sample_differences)
};

cudaError_t launch_raster_forward(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                  uint32_t W, uint32_t H, const float* viewports, uint32_t cull,
                                  const uint32_t* offsets, const uint32_t* list, unsigned long long capacity,
                                  float* raster, float* deriv, cudaStream_t stream,
                                  const RasterShade* shade = nullptr, const uint32_t* status = nullptr,
                                  uint32_t tile_w = 16, uint32_t tile_h = 16, uint32_t chunk = 256);
// Tile shapes and stage depths the raster kernels are compiled for: 16x16 with 256 or 128 staged
// triangles, 16x8 with 128 (shapes that divide the reference's 16x16 tile: triangle_tile_rect).
bool raster_config_supported(uint32_t tile_w, uint32_t tile_h, uint32_t chunk);

cudaError_t launch_raster_backward(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                   uint32_t W, uint32_t H, const float* viewports, const float* raster,
                                   const float* grad_raster, float* grad_clip, cudaStream_t stream,
                                   const float* grad_derivatives = nullptr, bool near = false);

cudaError_t launch_interpolate_forward(const float* attr, size_t attr_view_stride, uint32_t V, uint32_t A,
                                       const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                       size_t P, float* out, cudaStream_t stream);

cudaError_t launch_interpolate_backward(const float* attr, size_t attr_view_stride, uint32_t V, uint32_t A,
                                        const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                        size_t P, const float* grad_out, float* grad_attr, float* grad_raster,
                                        cudaStream_t stream, bool accumulate_raster = false);

cudaError_t launch_texture_forward(const float* tex, size_t tex_view_stride, uint32_t tw, uint32_t th, uint32_t C,
                                   uint32_t mode, const float* uv, const float* raster, uint32_t views, size_t P,
                                   float* out, cudaStream_t stream);

cudaError_t launch_texture_backward(const float* tex, size_t tex_view_stride, uint32_t tw, uint32_t th, uint32_t C,
                                    uint32_t mode, const float* uv, const float* raster, uint32_t views, size_t P,
                                    const float* grad, float* grad_tex, float* grad_uv, uint32_t* status,
                                    cudaStream_t stream);


}  // namespace pdr

#include "../../include/pdr_capi.h"

namespace pdr {

pdr_status set_error(pdr_status code, const char* msg);
pdr_status set_cuda_error(cudaError_t err, const char* what);
// The shape, size and alignment checks every raster entry point makes (the reference's messages).
pdr_status check_raster_args(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                             uint32_t W, uint32_t H, const float* viewports);

cudaError_t launch_project_views(const float* apos, const float* anrm, const float* araster, uint32_t N,
                                 const pdr_projection_view* views, uint32_t nviews, uint32_t blend_mode,
                                 uint32_t pcf_radius, uint32_t visibility_mode, float* color4, float* confidence,
                                 uint32_t* source_view, float* valid_mask, float* coverage_mask, uint32_t* face_ids,
                                 cudaStream_t stream, const uint32_t* vis_bits = nullptr,
                                 uint32_t vis_words = 0);
cudaError_t launch_transform_positions(const float* pos3, uint32_t V, const float* mats, uint32_t views, float* clip,
                                       cudaStream_t stream);
cudaError_t launch_atlas_clip(const float* uv, uint32_t V, float* clip, cudaStream_t stream);
cudaError_t launch_prepare_view(const float* image, uint32_t C, const float* ext_mask, const float* raster, size_t P,
                                float* target, float* mask, cudaStream_t stream);
cudaError_t launch_photometric(const float* tex, uint32_t tw, uint32_t th, const pdr_refine_view* views,
                               uint32_t nviews, uint64_t max_pixels, uint32_t step, uint32_t batch, float eps,
                               float norm, float* grad, float* loss, cudaStream_t stream);
cudaError_t launch_seam(const float* tex, uint32_t tw, uint32_t th, const float* pairs, uint32_t npairs, float eps,
                        float norm, float* grad, float* loss, uint32_t loss_index, cudaStream_t stream);
cudaError_t launch_tv(const float* tex, uint32_t tw, uint32_t th, const uint8_t* valid, const int32_t* chart, float eps,
                      float scale, float* grad, cudaStream_t stream);
cudaError_t launch_adam(float* tex, float* grad, float* m, float* v, size_t n, float lr, float b1, float b2, float eps,
                        float bc1, float bc2, float cmin, float cmax, cudaStream_t stream);
// launch_tv followed by launch_adam in one pass, reading tex_in and writing tex_out (different buffers)
cudaError_t launch_adam_tv(const float* tex_in, float* tex_out, float* grad, float* m, float* v, uint32_t tw,
                           uint32_t th, const uint8_t* valid, const int32_t* chart, float tv_eps, float tv_scale,
                           float lr, float b1, float b2, float eps, float bc1, float bc2, float cmin, float cmax,
                           cudaStream_t stream);
cudaError_t precond_prepare();  // sets the kernels' shared-memory limits (once; before any capture)
cudaError_t launch_precond_forward(const float* params, const uint16_t* wbf, const uint16_t* feat, uint64_t n,
                                   float* out, uint32_t* status, cudaStream_t stream);
cudaError_t launch_precond_train(const float* params, const uint16_t* wbf, const uint16_t* feat, const float* target,
                                 const float* weight, uint64_t n, float inv_norm, float* grads, float* loss,
                                 uint32_t* status, cudaStream_t stream);
cudaError_t launch_precond_adam(float* params, const float* grads, float* m, float* v, float lr, float b1, float b2,
                                float eps, float bc1, float bc2, uint16_t* wbf, cudaStream_t stream);
cudaError_t launch_observe_view(const float* uv, const float* mask, uint64_t P, uint32_t tw, uint32_t th, float* obs,
                                uint8_t* seen, float* views, cudaStream_t stream);
cudaError_t launch_edge_distance(const uint8_t* valid, const int32_t* chart, uint32_t tw, uint32_t th, float* edge,
                                 cudaStream_t stream);
cudaError_t launch_precond_features(const float* tex, const float* m1, const float* m2, float bc1, float bc2,
                                    float eps, const float* obs, const float* views, const float* edge, float progress,
                                    uint64_t N, uint16_t* feat, cudaStream_t stream);
cudaError_t launch_adam_scaled(float* tex, float* grad, float* m1, float* m2, uint64_t N, const float* mult,
                               const uint32_t* fallback, float lr, float b1, float b2, float eps, float bc1, float bc2,
                               float cmin, float cmax, cudaStream_t stream);
cudaError_t launch_fallback_check(const float* loss, uint32_t begin, uint32_t window, float tolerance,
                                  uint32_t* fallback, cudaStream_t stream);
void refine_schedule(const pdr_refine_options* o, uint32_t step, float* lr, float* bc1, float* bc2);

}  // namespace pdr

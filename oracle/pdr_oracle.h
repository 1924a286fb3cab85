/*
 * CPU oracle for the photara_drender raster / texture / bake / refine path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path is
 * compared against; nothing in the product package links, loads or calls it.
 *
 * Every function restates one routine of the reference (fenghuayumo/photara_drender
 * v0.4.0) in plain C with the same fp32 operation order, compiled with
 * -ffp-contract=off so no multiply-add is fused. The "_f64" functions are FP64
 * twins used only to state the error of fp32 results; with abs_terms they accumulate |term|
 * instead (the sum of absolute terms that bounds summation-order error).
 *
 * Return codes mirror the reference's exception types:
 *   0 ok, -1 std::invalid_argument, -2 std::out_of_range, -3 std::overflow_error.
 */
#ifndef PDR_ORACLE_H
#define PDR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Host threads of the parallel loops (0: all processors). Every result is independent of the
 * thread count: sums are partitioned by owner, never split. */
void ora_set_threads(int threads);
int ora_get_threads(void);

#define ORA_OK 0
#define ORA_INVALID (-1)
#define ORA_RANGE (-2)
#define ORA_OVERFLOW (-3)

/* src/rasterizer.cpp:61-138 build_tile_bins. offsets has tiles+1 entries.
 * list may be NULL (count only). Returns the entry count, or <0 on error. */
int64_t ora_bin_tiles(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                      uint32_t width, uint32_t height, const float viewport[4],
                      uint32_t* offsets, uint32_t* list, int64_t list_capacity);

/* shaders/rasterize_forward.hlsl:45-175 over the tile bins of build_tile_bins. */
int ora_rasterize_forward(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                          uint32_t width, uint32_t height, uint32_t cull_mode,
                          int output_derivatives, const float viewport[4],
                          float* raster, float* derivatives);

/* ora_rasterize_forward (no derivatives) that also flags, per pixel, how the winner was decided:
 * ORA_TIE_DEPTH when another covering triangle had the same depth (the lowest-id rule decided),
 * ORA_TIE_EDGE when the winner's sample lies on one of its edges or inside the 1e-7 tolerance. */
#define ORA_TIE_DEPTH 1
#define ORA_TIE_EDGE 2
int ora_rasterize_forward_ties(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                               uint32_t width, uint32_t height, uint32_t cull_mode, const float viewport[4],
                               float* raster, uint8_t* ties);

/* FP64 twin of the barycentric/derivative arithmetic for the fp32 winners in raster. */
int ora_rasterize_forward_f64(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                              uint32_t width, uint32_t height, const float viewport[4],
                              const float* raster, double* raster64, double* deriv64);

/* shaders/rasterize_backward.hlsl + reduce_vertex_gradients.hlsl + rasterizer.cpp:145-162. */
int ora_rasterize_backward(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                           uint32_t width, uint32_t height, const float viewport[4],
                           const float* raster, const float* grad_raster, float* grad_pos);
int ora_rasterize_backward_f64(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                               uint32_t width, uint32_t height, const float viewport[4],
                               const float* raster, const float* grad_raster, double* grad_pos, int abs_terms);

/* shaders/interpolate_forward.hlsl */
int ora_interpolate_forward(const float* attr, uint32_t V, uint32_t A, const uint32_t* idx,
                            uint32_t T, const float* raster, uint64_t P, float* out);
/* shaders/interpolate_grad_attributes.hlsl + interpolate_grad_raster.hlsl */
int ora_interpolate_backward(const float* attr, uint32_t V, uint32_t A, const uint32_t* idx,
                             uint32_t T, const float* raster, uint64_t P, const float* grad_out,
                             float* grad_attr, float* grad_raster);
int ora_interpolate_backward_f64(const float* attr, uint32_t V, uint32_t A, const uint32_t* idx,
                                 uint32_t T, const float* raster, uint64_t P, const float* grad_out,
                                 double* grad_attr, double* grad_raster, int abs_terms);

/* shaders/texture_forward.hlsl */
int ora_texture_forward(const float* tex, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                        const float* uv, const float* raster, uint64_t P, float* out);
/* rasterizer.cpp:187-258 (double weights) + texture_grad_texture.hlsl + texture_grad_uv.hlsl.
 * grad_uv may be NULL. */
int ora_texture_backward(const float* tex, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                         const float* uv, const float* raster, uint64_t P, const float* grad,
                         float* grad_tex, float* grad_uv);
int ora_texture_backward_f64(const float* tex, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                             const float* uv, const float* raster, uint64_t P, const float* grad,
                             double* grad_tex, double* grad_uv, int abs_terms);

/* texture_baker.cpp:92-106 / texture_refiner.cpp:36-50 */
void ora_transform_positions(const float* pos3, uint32_t V, const float m[16], float* clip4);

/* src/texture_padding.cpp:187-224 */
float ora_suggest_softmax_scale(const float* pos3, uint32_t V, const float* cams, uint32_t ncam);

/* One shaders/project_texture.hlsl dispatch for one view; state arrays are read-modify-write. */
typedef struct {
    float world_to_clip[16];
    float camera_position[3];
    float view_weight;          /* weight, or weight*softmax_scale for softmax */
    float viewport[4];
    uint32_t atlas_width, atlas_height, image_width, image_height;
    float depth_bias, min_view_cosine;
    uint32_t channel_count, blend_mode, pcf_radius, has_mask, visibility_mode, view_index;
} ora_project_params;

void ora_project_texture(const ora_project_params* pp, const float* atlas_pos, const float* atlas_nrm,
                         const float* atlas_raster, const float* shadow_raster, const float* photo,
                         const float* mask, const float* ray_visibility, float* acc_color,
                         float* acc_weight, float* best_conf, uint32_t* source_view);

/* texture_baker.cpp:156-361 with shadow-map visibility (the only mode without ray queries). */
typedef struct {
    uint32_t width, height, channel_count;
    const float* image;
    const float* visibility_mask; /* NULL = none */
    float world_to_clip[16];
    float camera_position[3];
    int has_viewport;
    float viewport[4];
    float weight, depth_bias, min_view_cosine;
} ora_view;

int ora_bake(const float* pos3, const float* nrm3, const float* uv2, uint32_t V, const uint32_t* idx,
             uint32_t T, const ora_view* views, uint32_t nviews, uint32_t atlas_w, uint32_t atlas_h,
             uint32_t blend_mode, uint32_t pcf_radius, float mask_floor, float softmax_scale,
             float* color4, float* confidence, uint32_t* source_view, float* valid_mask,
             float* coverage_mask, uint32_t* face_ids);

/* ora_bake with ray visibility: visibility_mode 1 (ray x shadow map) or 2 (ray) taking the camera
 * visibility of texel i and view k from bit k % 32 of ray_bits[i * ceil(nviews / 32) + k / 32]. */
int ora_bake_ex(const float* pos3, const float* nrm3, const float* uv2, uint32_t V, const uint32_t* idx,
                uint32_t T, const ora_view* views, uint32_t nviews, uint32_t atlas_w, uint32_t atlas_h,
                uint32_t blend_mode, uint32_t pcf_radius, float mask_floor, float softmax_scale,
                uint32_t visibility_mode, const uint32_t* ray_bits,
                float* color4, float* confidence, uint32_t* source_view, float* valid_mask,
                float* coverage_mask, uint32_t* face_ids);
/* shaders/project_ray_visibility.hlsl:14-55, triangles tested in double: 1 visible, 0 occluded (or
 * texel not covered), -1 undecided (a triangle within 1e-5 of the ray without a clear hit). */
int ora_ray_visibility(const float* pos3, uint32_t V, const uint32_t* idx, uint32_t T, const float* apos,
                       const float* anrm, const float* araster, uint64_t N, const float camera[3], float bias,
                       int8_t* state);

/* atlas_photometric_gradient.hlsl for one view; grad is accumulated; returns loss added. */
float ora_photometric_gradient(const float* tex3, uint32_t tw, uint32_t th, const float* uv,
                               const float* target3, const float* mask, uint32_t P, float eps,
                               float normalization, float* grad);
/* atlas_seam_gradient.hlsl */
float ora_seam_gradient(const float* tex3, uint32_t tw, uint32_t th, const float* pairs,
                        uint32_t npairs, float eps, float normalization, float* grad);
/* FP64 twins of the two gradients above (abs_terms: accumulate |term|); return the loss. */
double ora_photometric_gradient_f64(const float* tex3, uint32_t tw, uint32_t th, const float* uv,
                                    const float* target3, const float* mask, uint32_t P, float eps,
                                    float normalization, double* grad, int abs_terms);
double ora_seam_gradient_f64(const float* tex3, uint32_t tw, uint32_t th, const float* pairs,
                             uint32_t npairs, float eps, float normalization, double* grad, int abs_terms);
/* Visit pixels and seam pairs in reverse order in the two functions above (and in ora_refine): a
 * second accumulation order of the reference's atomics, for stating order noise. Process-wide. */
void ora_set_reverse_order(int reverse);
/* atlas_adam_update.hlsl */
void ora_adam_update(float* tex, float* grad, float* m, float* v, uint64_t n, float lr, float b1,
                     float b2, float eps, float bc1, float bc2, float cmin, float cmax);

/* texture_refiner.cpp:174-454 */
typedef struct {
    uint32_t width, height, steps, batch_size;
    float learning_rate, minimum_learning_rate, photometric_epsilon;
    float adam_beta1, adam_beta2, adam_epsilon, clamp_min, clamp_max;
    uint32_t seam_polish_steps;
    float seam_learning_rate, seam_epsilon;
} ora_refine_options;

int ora_refine(const float* initial_tex3, const float* pos3, const float* uv2, uint32_t V,
               const uint32_t* idx, uint32_t T, const ora_view* views, uint32_t nviews,
               const float* seam_pairs, uint32_t npairs, const ora_refine_options* o,
               float* out_tex3, float* loss_history, float* seam_loss_history);

/* Refine precompute for one view (texture_refiner.cpp:219-242): uv [P,2], target [P,3],
 * mask [P]; returns the valid weight through *valid_weight. */
int ora_refine_view_cache(const float* pos3, const float* uv2, uint32_t V, const uint32_t* idx,
                          uint32_t T, const ora_view* view, float* uv_out, float* target_out,
                          float* mask_out, double* valid_weight);

/* Chart-aware robust total variation gradient (python/photara_drender/atlas.py:84-115),
 * added into grad with the given weight; returns the weighted loss. */
double ora_tv_gradient(const float* tex, uint32_t tw, uint32_t th, uint32_t C,
                       const uint8_t* valid, const int32_t* chart, float eps, float weight,
                       float* grad);

/* FP64 twin of ora_tv_gradient (abs_terms: accumulate |term|); returns the weighted loss. */
double ora_tv_gradient_f64(const float* tex, uint32_t tw, uint32_t th, uint32_t C,
                           const uint8_t* valid, const int32_t* chart, float eps, float weight,
                           double* grad, int abs_terms);

/* src/texture_padding.cpp:37-95: the 8SSEDT nearest-source offsets (sources: mask >= threshold). */
int ora_nearest_field_offsets(const float* source_mask, uint32_t width, uint32_t height, float threshold,
                              int16_t* offset_x, int16_t* offset_y);
/* src/texture_padding.cpp:226-351 pad_texture_atlas, in place on color [H][W][channels] and filled
 * [H][W] (pass zeros for an absent filled_mask). coverage may be NULL. stats: valid, gutter,
 * unobserved, remaining_unobserved, filled. reason (on ORA_INVALID): 1 empty atlas, 2 too large,
 * 4 channel count, 6 threshold. */
int ora_pad_texture_atlas(float* color, uint32_t channels, const float* valid, const float* coverage, float* filled,
                          uint32_t width, uint32_t height, uint32_t margin, int fill_unobserved,
                          uint32_t maximum_fill_distance, float threshold, uint64_t stats[5], int* reason);
/* src/texture_padding.cpp:100-184 fill_texture_on_surface. stats: filled, remaining, measured faces,
 * propagated faces. reason: 1 empty atlas or mesh, 2 channel count, 3 too many faces, 4 face id out
 * of range, 5 degenerate edge, 6 non-manifold edge. */
int ora_fill_texture_on_surface(float* color, uint32_t channels, const float* valid, const uint32_t* face_ids,
                                float* filled, uint32_t width, uint32_t height, const uint32_t* indices,
                                uint32_t triangle_count, uint64_t stats[4], int* reason);

#ifdef __cplusplus
}
#endif
#endif

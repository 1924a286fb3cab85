/*
 * photara_drender GB300 C ABI.
 *
 * Plain C entry points over the sm_103a CUDA kernels that replace the reference's Vulkan
 * compute dispatches (reference: fenghuayumo/photara_drender v0.4.0). Every call takes device
 * pointers, plain sizes and a CUDA stream (cudaStream_t passed as void*, NULL = legacy default
 * stream), enqueues its kernels and returns without synchronising. No call allocates device
 * memory: scratch space is passed in by the caller, sized by the matching *_workspace_bytes query.
 * Memory layouts are those of the reference's Python bindings, with a leading view axis:
 *   clip positions [views][V][4] f32, triangle indices [T][3] u32 (shared by all views),
 *   viewports [views][4] f32 (x, y, width, height), raster and barycentric derivatives
 *   [views][H][W][4] f32, attributes [V][A] f32, textures [H][W][C] f32, uv [views][H][W][2] f32.
 * Buffers read or written as float4/float2 must be 16-/8-byte aligned.
 *
 * Status codes mirror the reference's exception types: PDR_INVALID_ARGUMENT is
 * std::invalid_argument, PDR_OUT_OF_RANGE std::out_of_range, PDR_OVERFLOW std::overflow_error,
 * PDR_CUDA_ERROR std::runtime_error. pdr_last_error() returns the calling thread's last message.
 */
#ifndef PDR_CAPI_H
#define PDR_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define PDR_API __declspec(dllexport)
#else
#define PDR_API __attribute__((visibility("default")))
#endif

typedef int32_t pdr_status;

#define PDR_OK 0
#define PDR_INVALID_ARGUMENT (-1)
#define PDR_OUT_OF_RANGE (-2)
#define PDR_OVERFLOW (-3)
#define PDR_CUDA_ERROR (-4)
#define PDR_NOT_SUPPORTED (-5)

/* Device status block written by pipeline calls (8 u32 words in device memory). */
#define PDR_STATUS_WORDS 8
#define PDR_STATUS_TILE_ENTRIES 0  /* entries of the last tile binning */
#define PDR_STATUS_TILE_ENTRIES_HI 1
#define PDR_STATUS_TILE_OVERFLOW 2 /* 1 when the tile list exceeded its capacity */
#define PDR_STATUS_LARGE_TILES 3
#define PDR_STATUS_TEXEL_ERROR 4   /* 1 non-finite uv on a covered pixel, 2 texel position beyond 1e9 */
#define PDR_STATUS_INDEX_ERROR 5   /* 1 when a triangle index is >= the vertex count */
#define PDR_STATUS_PRECOND_TIMEOUT 6 /* 1 when a tensor-core wait of the preconditioner MLP gave up */
#define PDR_STATUS_PAD_ERROR 7     /* padding / surface fill: 1 a sweep wait gave up, 2 face id out of range,
                                      4 degenerate edge, 8 non-manifold edge */

PDR_API const char* pdr_last_error(void);
PDR_API int32_t pdr_version(void);

/* Context: replaces Context::Impl::Impl / enumerate_devices (src/context.cpp:248-382, 625-655). */
PDR_API int32_t pdr_device_count(void);
PDR_API pdr_status pdr_device_info(int32_t device, char* name, size_t name_capacity, uint32_t* vendor_id,
                                   uint32_t* device_id, uint32_t* api_version, int32_t* sm_count);

/* Index validation (src/rasterizer.cpp:29-40 validate_mesh): sets PDR_STATUS_INDEX_ERROR when any of
 * the n indices is >= vertex_count. */
PDR_API pdr_status pdr_validate_indices(const uint32_t* indices, uint64_t n, uint32_t vertex_count,
                                        uint32_t* status, void* stream);

/* Tile binning (src/rasterizer.cpp:61-138 build_tile_bins) for all views at once: CSR over
 * (view, 16x16 tile) with triangle ids ascending in every tile, bit-identical to the reference's
 * lists. tile_offsets has views*tiles+1 entries; tile_triangles holds `capacity` entries; the
 * entry count lands in status[PDR_STATUS_TILE_ENTRIES] and status[PDR_STATUS_TILE_OVERFLOW] is
 * set when it exceeds capacity (the caller then grows the list and calls again). A capacity above
 * UINT32_MAX is refused with PDR_OVERFLOW (the offsets are u32). */
PDR_API size_t pdr_bin_tiles_workspace_bytes(uint32_t views, uint32_t triangle_count, uint32_t width,
                                             uint32_t height, uint64_t capacity);
PDR_API pdr_status pdr_bin_tiles(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                 const uint32_t* indices, uint32_t triangle_count, uint32_t width, uint32_t height,
                                 const float* viewports, uint32_t* tile_offsets, uint32_t* tile_triangles,
                                 uint64_t capacity, void* workspace, size_t workspace_bytes, uint32_t* status,
                                 void* stream);

/* Rasterizer::forward (src/rasterizer.cpp:373-442 + shaders/rasterize_forward.hlsl) over bins
 * made by pdr_bin_tiles. barycentric_derivatives may be NULL (output_barycentric_derivatives off). */
PDR_API pdr_status pdr_rasterize_forward(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                         const uint32_t* indices, uint32_t triangle_count, uint32_t width,
                                         uint32_t height, const float* viewports, uint32_t cull_mode,
                                         const uint32_t* tile_offsets, const uint32_t* tile_triangles,
                                         uint64_t capacity, float* raster, float* barycentric_derivatives,
                                         void* stream);

/* Rasterizer::backward (src/rasterizer.cpp:444-537 + shaders/rasterize_backward.hlsl +
 * reduce_vertex_gradients.hlsl): grad_clip_positions [views][V][4] is overwritten. */
PDR_API pdr_status pdr_rasterize_backward(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                          const uint32_t* indices, uint32_t triangle_count, uint32_t width,
                                          uint32_t height, const float* viewports, const float* raster,
                                          const float* grad_raster, float* grad_clip_positions, void* stream);
/* pdr_rasterize_backward plus the gradient through the barycentric pixel derivatives
 * (grad_barycentric_derivatives [views][H][W][4], d/d of [du/dx, du/dy, dv/dx, dv/dy]), which the
 * reference rejects (src/rasterizer.cpp:459-462). Either gradient may be NULL (then it is zero). */
PDR_API pdr_status pdr_rasterize_backward_derivatives(const float* clip_positions, uint32_t views,
                                                      uint32_t vertex_count, const uint32_t* indices,
                                                      uint32_t triangle_count, uint32_t width, uint32_t height,
                                                      const float* viewports, const float* raster,
                                                      const float* grad_raster,
                                                      const float* grad_barycentric_derivatives,
                                                      float* grad_clip_positions, void* stream);

/* ---- near-plane clipping ------------------------------------------------------------------------
 * The reference has none: it skips every triangle with a vertex at w <= 1e-8 and rasterizes the others
 * unclipped (README.md:140, docs/architecture.md:62; Rasterizer::forward, src/rasterizer.cpp:373-442).
 * Opt-in sequence: pdr_clip_near -> pdr_bin_tiles + pdr_rasterize_forward on the clipped mesh (vertex
 * count 4 * T, triangle count 2 * T) -> pdr_remap_near; gradients with pdr_rasterize_backward_near. */
#define PDR_NEAR_MAX_TRIANGLES 8388608u /* ids of the clipped mesh (up to 2 * T) stay exact in fp32 */
/* Clips every triangle of every view against z + w = 0 into clipped_positions [views][4 * T][4] and the
 * view-independent clipped_indices [2 * T][3] (slots 2k and 2k + 1 hold what is left of triangle k; a slot
 * with nothing left touches a vertex with w = 0 and covers nothing). An index >= vertex_count leaves
 * the triangle empty and sets status[PDR_STATUS_INDEX_ERROR] (status may be NULL). */
PDR_API pdr_status pdr_clip_near(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                 const uint32_t* indices, uint32_t triangle_count, float* clipped_positions,
                                 uint32_t* clipped_indices, uint32_t* status, void* stream);
/* In place on the raster (and derivatives, may be NULL) of the clipped mesh: ids become the original
 * triangle's, and barycentrics, depth and derivatives are those of the original triangle at the pixel
 * (rasterize_forward.hlsl's formulas); identical to pdr_rasterize_forward where no clipping happened. */
PDR_API pdr_status pdr_remap_near(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                  const uint32_t* indices, uint32_t triangle_count, uint32_t width, uint32_t height,
                                  const float* viewports, float* raster, float* barycentric_derivatives,
                                  void* stream);
/* pdr_rasterize_backward_derivatives for a remapped raster: triangles with a vertex at w <= 1e-8 (never
 * visited by the reference's adjoint) are visited on every pixel they own; others as the reference. */
PDR_API pdr_status pdr_rasterize_backward_near(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                               const uint32_t* indices, uint32_t triangle_count, uint32_t width,
                                               uint32_t height, const float* viewports, const float* raster,
                                               const float* grad_raster, const float* grad_barycentric_derivatives,
                                               float* grad_clip_positions, void* stream);

/* Rasterizer::interpolate_forward (src/rasterizer.cpp:539-601 + shaders/interpolate_forward.hlsl).
 * attribute_view_stride = 0 shares one [V][A] table across views, else floats between views. */
PDR_API pdr_status pdr_interpolate_forward(const float* attributes, uint64_t attribute_view_stride,
                                           uint32_t vertex_count, uint32_t attribute_count, const uint32_t* indices,
                                           uint32_t triangle_count, const float* raster, uint32_t views,
                                           uint64_t pixels_per_view, float* interpolated, void* stream);

/* Rasterizer::interpolate_backward (src/rasterizer.cpp:603-683 + interpolate_grad_attributes.hlsl +
 * interpolate_grad_raster.hlsl). grad_attributes (summed over views when shared) and grad_raster are
 * overwritten; either may be NULL. */
PDR_API pdr_status pdr_interpolate_backward(const float* attributes, uint64_t attribute_view_stride,
                                            uint32_t vertex_count, uint32_t attribute_count,
                                            const uint32_t* indices, uint32_t triangle_count, const float* raster,
                                            uint32_t views, uint64_t pixels_per_view, const float* grad_interpolated,
                                            float* grad_attributes, float* grad_raster, void* stream);

/* As pdr_interpolate_backward, but grad_raster is accumulated into (+=) instead of overwritten, so the
 * raster gradients of several interpolations of one raster sum in place (what autograd does when
 * one raster feeds several interpolate() calls, python/photara_drender/torch.py:121-123). */
PDR_API pdr_status pdr_interpolate_backward_accumulate(const float* attributes, uint64_t attribute_view_stride,
                                                       uint32_t vertex_count, uint32_t attribute_count,
                                                       const uint32_t* indices, uint32_t triangle_count,
                                                       const float* raster, uint32_t views, uint64_t pixels_per_view,
                                                       const float* grad_interpolated, float* grad_attributes,
                                                       float* grad_raster, void* stream);

/* Rasterizer::texture_forward (src/rasterizer.cpp:685-735 + shaders/texture_forward.hlsl).
 * address_mode: 0 clamp, 1 wrap, 2 mirror (types.hpp AddressMode). */
PDR_API pdr_status pdr_texture_forward(const float* texture, uint64_t texture_view_stride, uint32_t texture_width,
                                       uint32_t texture_height, uint32_t channel_count, uint32_t address_mode,
                                       const float* uv, const float* raster, uint32_t views,
                                       uint64_t pixels_per_view, float* sampled, void* stream);

/* Rasterizer::texture_backward (src/rasterizer.cpp:737-829 + texture_grad_texture.hlsl +
 * texture_grad_uv.hlsl). grad_texture (summed over views when shared) is overwritten; grad_uv may be
 * NULL (compute_uv_gradient off). A non-finite uv on a covered pixel or a texel position beyond 1e9
 * sets status[PDR_STATUS_TEXEL_ERROR] (the reference throws before dispatching). */
PDR_API pdr_status pdr_texture_backward(const float* texture, uint64_t texture_view_stride, uint32_t texture_width,
                                        uint32_t texture_height, uint32_t channel_count, uint32_t address_mode,
                                        const float* uv, const float* raster, uint32_t views,
                                        uint64_t pixels_per_view, const float* grad_sampled, float* grad_texture,
                                        float* grad_uv, uint32_t* status, void* stream);


/* ---- bake: src/texture_baker.cpp + shaders/project_texture.hlsl ------------------------------ */

/* One projection view (types.hpp ProjectionView plus the device buffers the projection reads).
 * 160 bytes; the array passed to pdr_project_views lives in device memory. */
typedef struct {
    float world_to_clip[16];     /* row-major, clip = M [p, 1] */
    float camera_position[3];
    float weight;                /* ProjectionView::weight (times the softmax scale when blending softmax) */
    float viewport[4];           /* x, y, width, height in image pixels */
    uint32_t width, height, channel_count, has_mask;
    float depth_bias, min_view_cosine, mask_floor, reserved;
    const float* image;          /* [height][width][channel_count] */
    const float* visibility_mask;/* [height][width] when has_mask */
    const float* shadow_raster;  /* [height][width][4] raster of this view (visibility modes 0 and 1) */
    const float* ray_visibility; /* [atlas texels] visibility for modes 1 and 2, or NULL for 1.0 */
} pdr_projection_view;

/* texture_baker.cpp:92-106: clip [views][V][4] = world_to_clip[views] (row-major 4x4) * [p, 1]. */
PDR_API pdr_status pdr_transform_positions(const float* positions, uint32_t vertex_count, const float* world_to_clip,
                                           uint32_t views, float* clip_positions, void* stream);
/* texture_baker.cpp:81-90: clip [V][4] = (2u - 1, 2v - 1, 0, 1). */
PDR_API pdr_status pdr_atlas_clip_positions(const float* uv, uint32_t vertex_count, float* clip_positions,
                                            void* stream);
/* All views of a bake in one launch (project_texture.hlsl per view, in view order, per atlas texel)
 * with the host normalisation of texture_baker.cpp:334-358 fused: color [N][4] (rgb, valid),
 * confidence [N], source_view [N] (UINT32_MAX when unseen), valid_mask [N], coverage_mask [N] and
 * face_ids [N] (the last two may be NULL). blend_mode: 0 best_view, 1 weighted_average, 2 softmax;
 * visibility_mode: 0 shadow map, 1 ray visibility times shadow map, 2 ray visibility. */
PDR_API pdr_status pdr_project_views(const float* atlas_positions, const float* atlas_normals, const float* atlas_raster,
                                     uint32_t atlas_texels, const pdr_projection_view* views, uint32_t view_count,
                                     uint32_t blend_mode, uint32_t pcf_radius, uint32_t visibility_mode, float* color,
                                     float* confidence, uint32_t* source_view, float* valid_mask, float* coverage_mask,
                                     uint32_t* face_ids, void* stream);

/* ---- refine: src/texture_refiner.cpp + atlas_* shaders ---------------------------------------- *
 * Layouts: texture and Adam moments [height][width][3]; the gradient is [height][width][4] (RGB and
 * one unused float per texel, 16-byte aligned), so a bilinear tap adds its three channels with one
 * vector reduction. The gradient is scratch: zero before the first accumulation, zero after Adam. */

/* Cached per-view refinement inputs (texture_refiner.cpp:79-85), device pointers; 32 bytes. */
typedef struct {
    const float* uv;      /* [P][2] interpolated atlas uv */
    const float* target;  /* [P][3] */
    const float* mask;    /* [P] */
    uint64_t pixel_count;
} pdr_refine_view;

/* types.hpp TextureRefineOptions plus the optional chart-aware total variation term
 * (python/photara_drender/atlas.py:84-115): tv_scale = weight / (valid pairs * 3), 0 disables. */
typedef struct {
    uint32_t width, height, steps, batch_size;
    float learning_rate, minimum_learning_rate, photometric_epsilon;
    float adam_beta1, adam_beta2, adam_epsilon, clamp_min, clamp_max;
    uint32_t seam_polish_steps;
    float seam_learning_rate, seam_epsilon;
    float tv_scale, tv_epsilon;
    /* Optional second atlas [height][width][3], 16-byte aligned. With the total variation on, plain
     * refinement then alternates the texture between `texture` and this buffer, so each step's TV
     * gradient (which needs the neighbours' values from before the step) and its Adam update run as one
     * pass over the atlas instead of two. Results are bit-identical and end in `texture`. Null keeps the
     * separate TV pass. */
    float* texture_scratch;
} pdr_refine_options;

/* texture_refiner.cpp:228-242 for one view: target [P][3] and mask [P] from the image and raster. */
PDR_API pdr_status pdr_refine_prepare_view(const float* image, uint32_t channel_count, const float* visibility_mask,
                                           const float* raster, uint64_t pixel_count, float* target, float* mask,
                                           void* stream);
/* One photometric dispatch set (all batch views of `step`) accumulating into gradient and loss[step]. */
PDR_API pdr_status pdr_refine_photometric(const float* texture, uint32_t width, uint32_t height,
                                          const pdr_refine_view* views, uint32_t view_count,
                                          uint64_t max_view_pixels, uint32_t step, uint32_t batch_size,
                                          float epsilon, float normalization, float* gradient, float* loss_history,
                                          void* stream);
PDR_API pdr_status pdr_refine_seam(const float* texture, uint32_t width, uint32_t height, const float* seam_uv_pairs,
                                   uint32_t pair_count, float epsilon, float normalization, float* gradient,
                                   float* loss_history, uint32_t loss_index, void* stream);
PDR_API pdr_status pdr_refine_total_variation(const float* texture, uint32_t width, uint32_t height,
                                              const uint8_t* valid, const int32_t* chart_ids, float epsilon,
                                              float scale, float* gradient, void* stream);
/* count = texels * 3 values of texture and moments; gradient [texels][4]. */
PDR_API pdr_status pdr_refine_adam(float* texture, float* gradient, float* moment1, float* moment2, uint64_t count,
                                   float learning_rate, float beta1, float beta2, float epsilon,
                                   float bias_correction1, float bias_correction2, float clamp_min, float clamp_max,
                                   void* stream);
/* The per-step learning rate and bias corrections of texture_refiner.cpp:343-353, in float. */
PDR_API pdr_status pdr_refine_schedule(const pdr_refine_options* options, uint32_t step, float* learning_rate,
                                       float* bias_correction1, float* bias_correction2);

/* The whole TextureRefiner::refine optimisation (texture_refiner.cpp:256-415): `steps` photometric
 * + Adam steps with the cosine learning rate, then (when pair_count > 0) the seam polish with reset
 * moments. view_valid_weights is a host array of the views' valid weights (double, as the reference
 * keeps them); texture is updated in place; gradient/moment buffers are overwritten;
 * loss_history has steps + seam steps floats. With use_graph != 0 the sequence is recorded once
 * into a CUDA graph and launched as a single unit. */
PDR_API pdr_status pdr_refine_run(const pdr_refine_options* options, const pdr_refine_view* views, uint32_t view_count,
                                  const double* view_valid_weights, uint64_t max_view_pixels,
                                  const float* seam_uv_pairs, uint32_t pair_count, const uint8_t* tv_valid,
                                  const int32_t* tv_chart_ids, float* texture, float* gradient, float* moment1,
                                  float* moment2, float* loss_history, int32_t use_graph, void* stream);

/* A recorded refinement (same arguments as pdr_refine_run) that can be launched many times. */
typedef struct pdr_refine_graph_t* pdr_refine_graph;
PDR_API pdr_status pdr_refine_graph_create(pdr_refine_graph* graph, const pdr_refine_options* options,
                                           const pdr_refine_view* views, uint32_t view_count,
                                           const double* view_valid_weights, uint64_t max_view_pixels,
                                           const float* seam_uv_pairs, uint32_t pair_count, const uint8_t* tv_valid,
                                           const int32_t* tv_chart_ids, float* texture, float* gradient,
                                           float* moment1, float* moment2, float* loss_history, void* stream);
PDR_API pdr_status pdr_refine_graph_launch(pdr_refine_graph graph, void* stream);
PDR_API pdr_status pdr_refine_graph_destroy(pdr_refine_graph graph);


/* ---- fused many-view rendering: rasterize -> interpolate -> texture forward and backward ------- */

/* Arguments of pdr_render_forward / pdr_render_backward (device pointers). Attributes, uv attributes
 * and the texture are optional (NULL); the texture needs uv attributes and has 4 channels. */
typedef struct {
    const float* clip_positions;  /* [views][V][4] */
    uint32_t views, vertex_count;
    const uint32_t* indices;      /* [T][3] */
    uint32_t triangle_count, width, height;
    const float* viewports;       /* [views][4] */
    uint32_t cull_mode;
    const float* attributes;      /* [V][A], A <= 8, shared by all views */
    uint32_t attribute_count;
    const float* uv_attributes;   /* [V][2] */
    const float* texture;         /* [texture_height][texture_width][4] */
    uint32_t texture_width, texture_height, address_mode;
    uint32_t* tile_offsets;       /* [views*tiles + 1] */
    uint32_t* tile_triangles;     /* [capacity] */
    uint64_t capacity;
    void* workspace;              /* forward: pdr_render_workspace_bytes() bytes; backward: optional,
                                   * see pdr_render_backward_workspace_bytes() */
    size_t workspace_bytes;
    uint32_t* status;             /* PDR_STATUS_WORDS words */
    float* raster;                /* [views][H][W][4] */
    float* barycentric_derivatives; /* [views][H][W][4] or NULL */
    float* interpolated;          /* [views][H][W][A] */
    float* uv;                    /* [views][H][W][2] */
    float* sampled;               /* [views][H][W][4] */
    const float* grad_interpolated; /* [views][H][W][A] */
    const float* grad_sampled;    /* [views][H][W][4] */
    float* grad_clip_positions;   /* [views][V][4] */
    float* grad_attributes;       /* [V][A] summed over views */
    float* grad_uv_attributes;    /* [V][2] summed over views */
    float* grad_texture;          /* [texture_height][texture_width][4] summed over views */
    /* Optional [views][H][W][8], 16-byte aligned: the texel differences of the bilinear sample along u
     * and v per channel ((1-fy)(c10-c00) + fy(c11-c01), then the same along v), written by the forward
     * for covered pixels and read by the backward for texture_grad_uv instead of gathering the four
     * texels again. Null: the backward gathers them. Results are identical either way. */
    float* sample_differences;
    /* Tile shape and triangles staged per pass of the fused render's binning and raster; zeros mean
     * 16 x 16 and 256 (the reference's tile). Supported: 16x16 with 256 or 128, 16x8 with 128 (shapes
     * dividing the reference's tile: a triangle is listed in every sub-tile of the 16 x 16 tiles the
     * reference lists it in, so the (triangle, pixel) pairs tested are the reference's). Outputs are
     * bit-identical for every shape; tile_offsets then has
     * views * ceil(W / tile_width) * ceil(H / tile_height) + 1 entries. */
    uint32_t tile_width, tile_height, stage_triangles;
} pdr_render_args;

PDR_API size_t pdr_render_workspace_bytes(uint32_t views, uint32_t triangle_count, uint32_t width, uint32_t height,
                                          uint64_t capacity);
/* pdr_render_workspace_bytes for a tile shape other than 16 x 16. */
PDR_API size_t pdr_render_workspace_bytes_tiled(uint32_t views, uint32_t triangle_count, uint32_t width,
                                                uint32_t height, uint64_t capacity, uint32_t tile_width,
                                                uint32_t tile_height);
/* Tile binning and one raster launch whose epilogue interpolates both attribute sets and samples the
 * texture for every pixel: the outputs of Rasterizer::forward + interpolate_forward (x2) +
 * texture_forward, bit-identical to the separate calls. The raster does not depend on the order of
 * a tile's triangles, so tile_triangles holds each tile's triangles unsorted (pdr_bin_tiles sorts). */
PDR_API pdr_status pdr_render_forward(const pdr_render_args* args, void* stream);
/* pdr_render_forward in two parts: the tile binning alone (tile_offsets, tile_triangles, status), and the
 * raster launch with its epilogue over bins already made. A caller whose clip positions do not change
 * between calls (texture or attribute optimisation) bins once and rasterizes many times. */
PDR_API pdr_status pdr_render_bin(const pdr_render_args* args, void* stream);
PDR_API pdr_status pdr_render_raster(const pdr_render_args* args, void* stream);
/* The adjoints of the forward in one pixel pass: texture_backward, interpolate_backward for both
 * attribute sets (raster gradients summed) and rasterize_backward. With a 16-byte aligned workspace of
 * at least pdr_render_backward_workspace_bytes() bytes, the per-vertex gradients of each view are
 * gathered in records of the workspace (16-byte reductions, uv + attributes + clip together) and summed
 * into grad_uv_attributes / grad_attributes over the views in view order by a second pass; without
 * one they are added into the outputs directly. The gradients agree to float rounding either way. */
PDR_API pdr_status pdr_render_backward(const pdr_render_args* args, void* stream);
/* Workspace bytes for pdr_render_backward's per-view vertex-gradient records:
 * views * vertex_count * 4 * ceil((attribute_count + 5) / 4) * sizeof(float); 0 for attribute_count > 8. */
PDR_API size_t pdr_render_backward_workspace_bytes(uint32_t views, uint32_t vertex_count, uint32_t attribute_count);


/* ---- calibration --------------------------------------------------------------------------------
 * No counterpart in the reference. `reductions` red.global.add.v4.f32 operations (1.0 into each of
 * four floats) to pseudo-random 16-byte slots of buffer [slots][4], from a grid of 8 CTAs per SM:
 * timed by the caller, the rate of scattered vector reductions the GPU sustains, against which the
 * gradient scatters of the refiner and the fused adjoint are reported. */
PDR_API pdr_status pdr_calibrate_reductions(float* buffer, uint64_t slots, uint64_t reductions, uint32_t seed,
                                            void* stream);


/* ---- allocation-free binning ------------------------------------------------------------------ */

/* Size of the fixed scratch array behind pdr_bin_tiles_no_alloc (16 MiB). */
#define PDR_BIN_TILES_NO_ALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)

/* pdr_bin_tiles without a caller workspace; no counterpart in the reference. For callers that cannot
 * allocate device memory: code running inside another component's CUDA-graph capture, real-time
 * loops that must avoid cudaMalloc's synchronisation, plugin hosts that hand out buffers but no
 * allocator. Inputs, outputs and status are the caller's, exactly as for pdr_bin_tiles; the scratch
 * is a 16 MiB array compiled into the library and held on every GPU that loads it until the process
 * exits. Bins needing more scratch than that (pdr_bin_tiles_workspace_bytes() > 16 MiB) are rejected
 * with PDR_INVALID_ARGUMENT. The first call on a device looks the array's device address up
 * (cudaGetSymbolAddress); make it before any stream capture. The address is kept for the life of the
 * process, so the entry point must not be used across a device reset. Every call shares the array:
 * calls that overlap on the GPU race and must be serialised by the caller. Argument checks are those
 * of pdr_bin_tiles (16-byte aligned clip positions and viewports; capacity at most UINT32_MAX, else
 * PDR_OVERFLOW). */
PDR_API pdr_status pdr_bin_tiles_no_alloc(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                          const uint32_t* indices, uint32_t triangle_count, uint32_t width,
                                          uint32_t height, const float* viewports, uint32_t* tile_offsets,
                                          uint32_t* tile_triangles, uint64_t capacity, uint32_t* status,
                                          void* stream);


/* ---- learned refine preconditioner --------------------------------------------------------------
 * No counterpart in the reference. A 16 -> 64 -> 64 -> 4 MLP (ReLU, BF16 weights and operands, FP32
 * accumulation on the tensor cores) maps per-texel refine features to per-channel log step
 * multipliers for the Adam update. Parameters are one FP32 vector of PDR_PRECOND_PARAMS values,
 * [W1 64x16 | b1 64 | W2 64x64 | b2 64 | W3 4x64 | b3 4] with weights row-major [out][in], plus its
 * BF16 copy (same layout, 16-byte aligned) that the matrix multiplies read. */
#define PDR_PRECOND_IN 16
#define PDR_PRECOND_HIDDEN 64
#define PDR_PRECOND_OUT 4
#define PDR_PRECOND_PARAMS 5508

/* out [count][4] = MLP(features [count][16] BF16). */
PDR_API pdr_status pdr_precond_forward(const float* params, const uint16_t* params_bf16, const uint16_t* features,
                                       uint64_t count, float* out, uint32_t* status, void* stream);
/* One training pass over count samples: loss = inv_norm * sum weight * (MLP(x) - target)^2 (targets and
 * weights [count][4] FP32); grads [PDR_PRECOND_PARAMS] and loss [1] are overwritten with its gradient
 * and value. */
PDR_API pdr_status pdr_precond_train_step(const float* params, const uint16_t* params_bf16, const uint16_t* features,
                                          const float* targets, const float* target_weights, uint64_t count,
                                          float inv_norm, float* grads, float* loss, uint32_t* status, void* stream);
/* Adam step `step` (0-based) on the FP32 parameters; refreshes params_bf16. */
PDR_API pdr_status pdr_precond_adam(float* params, const float* grads, float* moment1, float* moment2, uint32_t step,
                                    float learning_rate, float beta1, float beta2, float epsilon,
                                    uint16_t* params_bf16, void* stream);
/* Static per-texel inputs of the features: observation weight (sum of masked bilinear tap weights over
 * all views), the number of views that see the texel, and a chart-edge distance proxy (the smallest
 * r in 1, 2, 4 .. 32 with an invalid or other-chart texel at offset r, 64 when none). views_host is a
 * HOST array of the cached views (device buffers); scratch holds width*height bytes. */
PDR_API pdr_status pdr_precond_texel_stats(const pdr_refine_view* views_host, uint32_t view_count, uint32_t width,
                                           uint32_t height, const uint8_t* valid, const int32_t* chart_ids,
                                           float* observation, float* view_counts, float* edge_distance,
                                           uint8_t* scratch, void* stream);
/* features [texel_count][16] BF16 from the refine state (texture, Adam moments with their bias
 * corrections) and the static inputs; progress is the fraction of the schedule done. */
PDR_API pdr_status pdr_precond_features(const float* texture, const float* moment1, const float* moment2,
                                        float bias_correction1, float bias_correction2, float epsilon,
                                        const float* observation, const float* view_counts,
                                        const float* edge_distance, float progress, uint64_t texel_count,
                                        uint16_t* features, void* stream);
/* The Adam update of pdr_refine_adam with each texel's step scaled per channel by
 * exp(clamp(multipliers[t][c], log 1/8, log 16)); plain Adam when *fallback != 0. */
PDR_API pdr_status pdr_refine_adam_scaled(float* texture, float* gradient, float* moment1, float* moment2,
                                          uint64_t texel_count, const float* multipliers, const uint32_t* fallback,
                                          float learning_rate, float beta1, float beta2, float epsilon,
                                          float bias_correction1, float bias_correction2, float clamp_min,
                                          float clamp_max, void* stream);

/* The plain-Adam fallback test of pdr_refine_run_learned on its own: sets *fallback to 1 when
 * sum(loss[begin + window .. begin + 2 window)) > (1 + tolerance) * sum(loss[begin .. begin + window)). */
PDR_API pdr_status pdr_precond_fallback_check(const float* loss_history, uint32_t begin, uint32_t window,
                                              float tolerance, uint32_t* fallback, void* stream);

/* State of a learned refinement (device pointers). */
typedef struct {
    const float* params;
    const uint16_t* params_bf16;
    const float* observation;     /* [texels] from pdr_precond_texel_stats */
    const float* view_counts;     /* [texels] */
    const float* edge_distance;   /* [texels] */
    uint16_t* features;           /* [texels][16] scratch */
    float* multipliers;           /* [texels][4] */
    uint32_t* fallback;           /* one word; cleared at the start, set when plain Adam takes over */
    uint32_t* status;             /* PDR_STATUS_WORDS words */
    uint32_t refresh_interval;    /* steps between MLP evaluations */
    float fallback_tolerance;     /* relative rise of the windowed batch loss that switches to plain Adam */
} pdr_precond_run;

/* pdr_refine_run with the learned preconditioner: every refresh_interval steps the features and the
 * MLP give new multipliers; from the second window on, a rise of the mean batch loss of the last
 * window over the one before by more than fallback_tolerance switches to plain Adam for the rest of
 * the run (decided on the device, so the whole run can be one CUDA graph). The seam polish is plain. */
PDR_API pdr_status pdr_refine_run_learned(const pdr_refine_options* options, const pdr_refine_view* views,
                                          uint32_t view_count, const double* view_valid_weights,
                                          uint64_t max_view_pixels, const float* seam_uv_pairs, uint32_t pair_count,
                                          const uint8_t* tv_valid, const int32_t* tv_chart_ids, float* texture,
                                          float* gradient, float* moment1, float* moment2, float* loss_history,
                                          const pdr_precond_run* precond, int32_t use_graph, void* stream);


/* ---- uneven multi-mesh batches in one launch ------------------------------------------------------
 * No counterpart in the reference, which renders one mesh per call. Every (mesh, view) of a batch is
 * one job. A batch runs as one binning pass, one raster launch over the tiles of all jobs (with the
 * shading epilogue of pdr_render_forward) and one adjoint launch (pdr_render_backward per job), for
 * meshes of any mix of triangle counts, view counts, resolutions and texture sizes. The mesh array is
 * a HOST array of structs holding device pointers; all meshes share one attribute count. */
typedef struct {
    const float* clip_positions;      /* [views][V][4] */
    const uint32_t* indices;          /* [T][3] */
    const float* viewports;           /* [views][4] */
    const float* attributes;          /* [V][A], or NULL when the batch's attribute_count is 0 */
    const float* uv_attributes;       /* [V][2], or NULL */
    const float* texture;             /* [texture_height][texture_width][4], or NULL (needs uv_attributes) */
    uint32_t views, vertex_count, triangle_count, width, height, texture_width, texture_height;
    float* raster;                    /* [views][H][W][4] */
    float* barycentric_derivatives;   /* [views][H][W][4] */
    float* interpolated;              /* [views][H][W][A] */
    float* uv;                        /* [views][H][W][2] */
    float* sampled;                   /* [views][H][W][4] */
    const float* grad_interpolated;   /* [views][H][W][A] (backward) */
    const float* grad_sampled;        /* [views][H][W][4] (backward) */
    float* grad_clip_positions;       /* [views][V][4] (backward) */
    float* grad_attributes;           /* [V][A] (backward) */
    float* grad_uv_attributes;        /* [V][2] (backward) */
    float* grad_texture;              /* [texture_height][texture_width][4] (backward) */
} pdr_render_mesh;

/* Forward tile shape and the triangles staged in shared memory per pass (the bin depth): 16x8/128,
 * 16x16/128 or 16x16/256 (sub-tiles of the reference's 16x16 tile). The outputs do not depend on the
 * choice. */
typedef struct {
    uint32_t tile_width, tile_height, stage_triangles;
} pdr_batch_config;

/* Number of tile segments (tile_offsets holds segments + 1 words) and workspace bytes of a batch. */
PDR_API pdr_status pdr_render_batch_sizes(const pdr_render_mesh* meshes, uint32_t mesh_count,
                                          const pdr_batch_config* config, uint32_t attribute_count,
                                          uint64_t* tile_segments, size_t* workspace_bytes);
/* Bins and rasterizes every view of every mesh, writing raster, derivatives, interpolated attributes,
 * uv and texture samples; status as pdr_bin_tiles (re-run with a larger capacity on overflow). */
PDR_API pdr_status pdr_render_batch_forward(const pdr_render_mesh* meshes, uint32_t mesh_count,
                                            uint32_t attribute_count, uint32_t cull_mode, uint32_t address_mode,
                                            const pdr_batch_config* config, uint32_t* tile_offsets,
                                            uint32_t* tile_triangles, uint64_t capacity, void* workspace,
                                            size_t workspace_bytes, uint32_t* status, void* stream);
/* The adjoints of the forward for every mesh (gradient outputs are overwritten). */
PDR_API pdr_status pdr_render_batch_backward(const pdr_render_mesh* meshes, uint32_t mesh_count,
                                             uint32_t attribute_count, uint32_t address_mode,
                                             const pdr_batch_config* config, void* workspace,
                                             size_t workspace_bytes, uint32_t* status, void* stream);


/* ---- ray-query visibility (shaders/project_ray_visibility.hlsl:14-55, src/context.cpp:446-453) ----
 * A bounding-volume hierarchy of the world-space mesh built on the device, traced with one any-hit ray
 * per (atlas texel, view). */
/* Bytes of the BVH buffer and of the scratch its build uses. */
PDR_API pdr_status pdr_bvh_sizes(uint32_t triangle_count, size_t* bvh_bytes, size_t* build_bytes);
/* Builds the BVH of positions [V][3] / indices [T][3] into bvh (synchronises the stream once). */
PDR_API pdr_status pdr_bvh_build(const float* positions, uint32_t vertex_count, const uint32_t* indices,
                                 uint32_t triangle_count, void* bvh, size_t bvh_bytes, void* scratch,
                                 size_t scratch_bytes, void* stream);
/* project_ray_visibility.hlsl for every covered texel and view: bit (v & 31) of visibility
 * [texel][ceil(views / 32)] is set when camera v (cameras [views][4], xyz used) is visible. */
PDR_API pdr_status pdr_ray_visibility(const void* bvh, uint32_t triangle_count, const float* atlas_positions,
                                      const float* atlas_normals, const float* atlas_raster, uint32_t atlas_texels,
                                      const float* cameras, uint32_t view_count, float ray_origin_bias,
                                      uint32_t* visibility, void* stream);
/* pdr_ray_visibility for the texel-views the projection reads: views (device memory, the projection's
 * table) whose camera the texel faces by min_view_cosine and whose clip volume and viewport contain it.
 * The other bits are 0; pdr_project_views_bits never reads them, so the bake is unchanged. */
PDR_API pdr_status pdr_ray_visibility_views(const void* bvh, uint32_t triangle_count, const float* atlas_positions,
                                            const float* atlas_normals, const float* atlas_raster,
                                            uint32_t atlas_texels, const pdr_projection_view* views,
                                            uint32_t view_count, float ray_origin_bias, uint32_t* visibility,
                                            void* stream);
/* pdr_project_views for visibility modes 1 (ray x shadow map) and 2 (ray) with the visibility bits of
 * pdr_ray_visibility instead of per-view arrays. */
PDR_API pdr_status pdr_project_views_bits(const float* atlas_positions, const float* atlas_normals,
                                          const float* atlas_raster, uint32_t atlas_texels,
                                          const pdr_projection_view* views, uint32_t view_count, uint32_t blend_mode,
                                          uint32_t pcf_radius, uint32_t visibility_mode, const uint32_t* visibility,
                                          float* color, float* confidence, uint32_t* source_view, float* valid_mask,
                                          float* coverage_mask, uint32_t* face_ids, void* stream);

/* ---- atlas padding and surface fill (src/texture_padding.cpp) --------------------------------------- */

/* Workspace of pdr_pad_texture_atlas for a width x height atlas of `channels` channels. */
PDR_API pdr_status pdr_pad_workspace_bytes(uint32_t width, uint32_t height, uint32_t channels, size_t* bytes);
/* Replaces pad_texture_atlas (texture_padding.cpp:226-351; include/photara_drender/texture_padding.hpp:62-67)
 * on the device, in place on color [height][width][channels] and filled_mask [height][width] (its
 * previous contents are the output's earlier filled_mask, zeros when there was none). coverage_mask may
 * be NULL. stats (5 device uint64): valid, gutter, unobserved, remaining_unobserved, filled texels. Sets
 * status[PDR_STATUS_PAD_ERROR] bit 1 if a sweep wait gave up. Enqueues only; no host synchronisation. */
PDR_API pdr_status pdr_pad_texture_atlas(float* color, uint32_t channels, const float* valid_mask,
                                         const float* coverage_mask, float* filled_mask, uint32_t width,
                                         uint32_t height, uint32_t margin, uint32_t fill_unobserved,
                                         uint32_t maximum_fill_distance, float valid_threshold, void* workspace,
                                         size_t workspace_bytes, uint64_t* stats, uint32_t* status, void* stream);
/* Workspace of pdr_fill_texture_on_surface. */
PDR_API pdr_status pdr_surface_fill_workspace_bytes(uint32_t width, uint32_t height, uint32_t triangle_count,
                                                    size_t* bytes);
/* Replaces fill_texture_on_surface (texture_padding.cpp:100-184; texture_padding.hpp:17-23) on the
 * device. face_ids [height][width] (0xFFFFFFFF outside the mesh), indices [triangle_count][3] of the
 * original (seam-free) mesh. stats (4 device uint64): filled texels, remaining texels, measured faces,
 * propagated faces. Data errors set status[PDR_STATUS_PAD_ERROR] bits 2 (face id out of range), 4
 * (degenerate edge), 8 (non-manifold edge) and then leave colour and filled_mask untouched; the
 * reference raises them in that order of precedence. */
PDR_API pdr_status pdr_fill_texture_on_surface(float* color, uint32_t channels, const float* valid_mask,
                                               const uint32_t* face_ids, float* filled_mask, uint32_t width,
                                               uint32_t height, const uint32_t* indices, uint32_t triangle_count,
                                               void* workspace, size_t workspace_bytes, uint64_t* stats,
                                               uint32_t* status, void* stream);

/* ---- mipmapped (trilinear) texture sampling: planned in the reference (README.md:141) ---------------- */

/* Levels of the box-filtered pyramid of a width x height texture (at most max_level levels above level 0)
 * and the texels of levels 1.. (level 0 is the caller's texture). */
PDR_API pdr_status pdr_mip_pyramid_size(uint32_t width, uint32_t height, uint32_t max_level, uint32_t* levels,
                                        uint64_t* pyramid_texels);
/* Builds levels 1.. of texture [height][width][channels] into pyramid (pyramid_texels * channels floats). */
PDR_API pdr_status pdr_mip_build(const float* texture, uint32_t width, uint32_t height, uint32_t channels,
                                 uint32_t max_level, float* pyramid, void* stream);
/* Trilinear sampling at uv [views][P][2] with uv_da [views][P][4] = (du/dx, du/dy, dv/dx, dv/dy): level of
 * detail 0.5 log2 of the larger squared texel-space derivative, texture_forward.hlsl's bilinear per level;
 * equal to pdr_texture_forward where the level of detail is <= 0. */
PDR_API pdr_status pdr_texture_forward_mip(const float* texture, const float* pyramid, uint32_t width,
                                           uint32_t height, uint32_t channels, uint32_t max_level,
                                           uint32_t address_mode, const float* uv, const float* uv_da,
                                           const float* raster, uint32_t views, uint64_t pixels_per_view,
                                           float* sampled, void* stream);
/* Adjoint of pdr_texture_forward_mip: grad_texture (level 0, overwritten) includes the folded gradient of the
 * pyramid levels (grad_pyramid is scratch of the pyramid's size); grad_uv [views][P][2] may be NULL. The
 * level of detail is a constant: uv_da receives no gradient. */
PDR_API pdr_status pdr_texture_backward_mip(const float* texture, const float* pyramid, uint32_t width,
                                            uint32_t height, uint32_t channels, uint32_t max_level,
                                            uint32_t address_mode, const float* uv, const float* uv_da,
                                            const float* raster, uint32_t views, uint64_t pixels_per_view,
                                            const float* grad_sampled, float* grad_texture, float* grad_pyramid,
                                            float* grad_uv, void* stream);
/* Pixel derivatives of interpolated attributes from the raster's barycentric derivatives:
 * attribute_derivatives [views][P][A][2] = (d/dx, d/dy) per attribute; zeros on uncovered pixels. */
PDR_API pdr_status pdr_interpolate_derivatives(const float* attributes, uint32_t vertex_count,
                                               uint32_t attribute_count, const uint32_t* indices,
                                               uint32_t triangle_count, const float* raster,
                                               const float* barycentric_derivatives, uint32_t views,
                                               uint64_t pixels_per_view, float* attribute_derivatives, void* stream);

#ifdef __cplusplus
}
#endif
#endif

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
 * set when it exceeds capacity (the caller then grows the list and calls again). */
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

#ifdef __cplusplus
}
#endif
#endif

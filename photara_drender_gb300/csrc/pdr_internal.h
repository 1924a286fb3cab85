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

size_t bins_workspace_bytes(uint32_t views, uint32_t T, uint32_t W, uint32_t H, unsigned long long capacity);

cudaError_t launch_bin_tiles(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                             uint32_t W, uint32_t H, const float* viewports, uint32_t* offsets, uint32_t* list,
                             unsigned long long capacity, void* workspace, uint32_t* status, cudaStream_t stream);

cudaError_t launch_raster_forward(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                  uint32_t W, uint32_t H, const float* viewports, uint32_t cull,
                                  const uint32_t* offsets, const uint32_t* list, unsigned long long capacity,
                                  float* raster, float* deriv, cudaStream_t stream);

cudaError_t launch_raster_backward(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                   uint32_t W, uint32_t H, const float* viewports, const float* raster,
                                   const float* grad_raster, float* grad_clip, cudaStream_t stream);

cudaError_t launch_interpolate_forward(const float* attr, size_t attr_view_stride, uint32_t V, uint32_t A,
                                       const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                       size_t P, float* out, cudaStream_t stream);

cudaError_t launch_interpolate_backward(const float* attr, size_t attr_view_stride, uint32_t V, uint32_t A,
                                        const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                        size_t P, const float* grad_out, float* grad_attr, float* grad_raster,
                                        cudaStream_t stream);

cudaError_t launch_texture_forward(const float* tex, size_t tex_view_stride, uint32_t tw, uint32_t th, uint32_t C,
                                   uint32_t mode, const float* uv, const float* raster, uint32_t views, size_t P,
                                   float* out, cudaStream_t stream);

cudaError_t launch_texture_backward(const float* tex, size_t tex_view_stride, uint32_t tw, uint32_t th, uint32_t C,
                                    uint32_t mode, const float* uv, const float* raster, uint32_t views, size_t P,
                                    const float* grad, float* grad_tex, float* grad_uv, uint32_t* status,
                                    cudaStream_t stream);

}  // namespace pdr

// C ABI entry points (include/pdr_capi.h): argument checks, status mapping and kernel launches.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {

namespace {
thread_local std::string g_last_error;

pdr_status fail(pdr_status code, const char* msg) {
    g_last_error = msg;
    return code;
}

pdr_status cuda_status(cudaError_t err, const char* what) {
    if (err == cudaSuccess) return PDR_OK;
    g_last_error = std::string(what) + ": " + cudaGetErrorString(err);
    return PDR_CUDA_ERROR;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

__global__ void validate_indices_kernel(const uint32_t* __restrict__ idx, uint64_t n, uint32_t V,
                                        uint32_t* __restrict__ status) {
    bool bad = false;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        bad = bad || idx[i] >= V;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicMax(status + 5, 1u);
}
}  // namespace

pdr_status set_error(pdr_status code, const char* msg) { return fail(code, msg); }
pdr_status set_cuda_error(cudaError_t err, const char* what) { return cuda_status(err, what); }

int num_sms() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    }
    return sms;
}

pdr_status check_raster_args(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                    uint32_t W, uint32_t H, const float* viewports) {
    if (!clip || !idx || !viewports) return fail(PDR_INVALID_ARGUMENT, "clip_positions, indices and viewports are required");
    if (views == 0 || V == 0) return fail(PDR_INVALID_ARGUMENT, "clip_positions must have shape [vertex_count, 4]");
    if (T == 0) return fail(PDR_INVALID_ARGUMENT, "triangle_indices must have shape [triangle_count, 3]");
    if (W == 0 || H == 0) return fail(PDR_INVALID_ARGUMENT, "Rasterization width and height must be positive");
    if (W > 65535u * kTile || H > 65535u * kTile) return fail(PDR_OVERFLOW, "Rasterization output size overflow");
    const uint64_t tiles = (uint64_t)((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile);
    if (tiles * views >= 0x7fffffffull || (uint64_t)T * views >= 0x7fffffffull)
        return fail(PDR_OVERFLOW, "Rasterization output size overflow");
    if (!aligned(clip, 16) || !aligned(viewports, 16)) return fail(PDR_INVALID_ARGUMENT, "clip_positions and viewports must be 16-byte aligned");
    return PDR_OK;
}

}  // namespace pdr

using namespace pdr;

extern "C" {

const char* pdr_last_error(void) { return g_last_error.c_str(); }

int32_t pdr_version(void) { return 100; }

int32_t pdr_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

pdr_status pdr_device_info(int32_t device, char* name, size_t name_capacity, uint32_t* vendor_id, uint32_t* device_id,
                           uint32_t* api_version, int32_t* sm_count) {
    cudaDeviceProp prop;
    cudaError_t err = cudaGetDeviceProperties(&prop, device);
    if (err == cudaErrorInvalidDevice) return fail(PDR_OUT_OF_RANGE, "device_index is out of range");
    if (err != cudaSuccess) return cuda_status(err, "cudaGetDeviceProperties");
    if (name && name_capacity) {
        std::strncpy(name, prop.name, name_capacity - 1);
        name[name_capacity - 1] = 0;
    }
    if (vendor_id) *vendor_id = 0x10deu;  // PCI vendor id of NVIDIA
    if (device_id) *device_id = (uint32_t)prop.pciDeviceID;
    if (api_version) *api_version = (uint32_t)(prop.major * 10 + prop.minor);
    if (sm_count) *sm_count = prop.multiProcessorCount;
    return PDR_OK;
}

pdr_status pdr_validate_indices(const uint32_t* indices, uint64_t n, uint32_t vertex_count, uint32_t* status,
                                void* stream) {
    if (!status || (n && !indices)) return fail(PDR_INVALID_ARGUMENT, "indices and status are required");
    if (n == 0) return PDR_OK;
    const uint64_t blocks = (n + 255) / 256;
    validate_indices_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, (cudaStream_t)stream>>>(
        indices, n, vertex_count, status);
    return cuda_status(cudaGetLastError(), "validate_indices");
}

size_t pdr_bin_tiles_workspace_bytes(uint32_t views, uint32_t triangle_count, uint32_t width, uint32_t height,
                                     uint64_t capacity) {
    return bins_workspace_bytes(views, triangle_count, width, height, capacity);
}

pdr_status pdr_bin_tiles(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T, uint32_t W,
                         uint32_t H, const float* viewports, uint32_t* offsets, uint32_t* list, uint64_t capacity,
                         void* workspace, size_t workspace_bytes, uint32_t* status, void* stream) {
    pdr_status st = check_raster_args(clip, views, V, idx, T, W, H, viewports);
    if (st) return st;
    if (!offsets || !status || (capacity && !list)) return fail(PDR_INVALID_ARGUMENT, "tile_offsets, tile_triangles and status are required");
    // tile offsets are u32: a larger capacity means nothing and would wrap the workspace size
    if (capacity > 0xffffffffull) return fail(PDR_OVERFLOW, "tile list capacity exceeds the u32 tile offsets");
    if (workspace_bytes < bins_workspace_bytes(views, T, W, H, capacity) || !workspace)
        return fail(PDR_INVALID_ARGUMENT, "workspace is smaller than pdr_bin_tiles_workspace_bytes()");
    return cuda_status(launch_bin_tiles(clip, views, V, idx, T, W, H, viewports, offsets, list, capacity, workspace,
                                        status, (cudaStream_t)stream),
                       "bin_tiles");
}

pdr_status pdr_rasterize_forward(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                 uint32_t W, uint32_t H, const float* viewports, uint32_t cull_mode,
                                 const uint32_t* offsets, const uint32_t* list, uint64_t capacity, float* raster,
                                 float* deriv, void* stream) {
    pdr_status st = check_raster_args(clip, views, V, idx, T, W, H, viewports);
    if (st) return st;
    if (cull_mode > 2) return fail(PDR_INVALID_ARGUMENT, "cull_mode must be 'none', 'back', or 'front'");
    if (!offsets || !raster || (capacity && !list)) return fail(PDR_INVALID_ARGUMENT, "tile bins and raster are required");
    if (!aligned(raster, 16) || (deriv && !aligned(deriv, 16))) return fail(PDR_INVALID_ARGUMENT, "raster outputs must be 16-byte aligned");
    return cuda_status(launch_raster_forward(clip, views, V, idx, T, W, H, viewports, cull_mode, offsets, list, capacity,
                                             raster, deriv, (cudaStream_t)stream),
                       "rasterize_forward");
}

pdr_status pdr_rasterize_backward(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx, uint32_t T,
                                  uint32_t W, uint32_t H, const float* viewports, const float* raster,
                                  const float* grad_raster, float* grad_clip, void* stream) {
    pdr_status st = check_raster_args(clip, views, V, idx, T, W, H, viewports);
    if (st) return st;
    if (!raster || !grad_raster || !grad_clip) return fail(PDR_INVALID_ARGUMENT, "raster, grad_raster and grad_clip_positions are required");
    if (!aligned(raster, 16) || !aligned(grad_raster, 16)) return fail(PDR_INVALID_ARGUMENT, "raster buffers must be 16-byte aligned");
    return cuda_status(launch_raster_backward(clip, views, V, idx, T, W, H, viewports, raster, grad_raster, grad_clip,
                                              (cudaStream_t)stream),
                       "rasterize_backward");
}

pdr_status pdr_rasterize_backward_derivatives(const float* clip, uint32_t views, uint32_t V, const uint32_t* idx,
                                              uint32_t T, uint32_t W, uint32_t H, const float* viewports,
                                              const float* raster, const float* grad_raster, const float* grad_deriv,
                                              float* grad_clip, void* stream) {
    pdr_status st = check_raster_args(clip, views, V, idx, T, W, H, viewports);
    if (st) return st;
    if (!raster || !grad_clip) return fail(PDR_INVALID_ARGUMENT, "raster and grad_clip_positions are required");
    if (!aligned(raster, 16) || (grad_raster && !aligned(grad_raster, 16)) || (grad_deriv && !aligned(grad_deriv, 16)))
        return fail(PDR_INVALID_ARGUMENT, "raster buffers must be 16-byte aligned");
    return cuda_status(launch_raster_backward(clip, views, V, idx, T, W, H, viewports, raster, grad_raster, grad_clip,
                                              (cudaStream_t)stream, grad_deriv),
                       "rasterize_backward_derivatives");
}

pdr_status pdr_interpolate_forward(const float* attr, uint64_t stride, uint32_t V, uint32_t A, const uint32_t* idx,
                                   uint32_t T, const float* raster, uint32_t views, uint64_t P, float* out,
                                   void* stream) {
    if (!attr || !idx || !raster || !out) return fail(PDR_INVALID_ARGUMENT, "attributes, indices, raster and output are required");
    if (A == 0 || V == 0) return fail(PDR_INVALID_ARGUMENT, "vertex_attributes must have shape [vertex_count, attribute_count]");
    if (T == 0) return fail(PDR_INVALID_ARGUMENT, "triangle_indices must have shape [triangle_count, 3]");
    if (P == 0 || views == 0) return fail(PDR_INVALID_ARGUMENT, "raster_output has inconsistent dimensions");
    if (P > 0xffffffffull) return fail(PDR_OVERFLOW, "Interpolation pixel count exceeds backend limits");
    if (!aligned(raster, 16)) return fail(PDR_INVALID_ARGUMENT, "raster must be 16-byte aligned");
    return cuda_status(launch_interpolate_forward(attr, stride, V, A, idx, T, raster, views, P, out, (cudaStream_t)stream),
                       "interpolate_forward");
}

static pdr_status interpolate_backward_impl(const float* attr, uint64_t stride, uint32_t V, uint32_t A,
                                            const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                            uint64_t P, const float* grad_out, float* grad_attr, float* grad_raster,
                                            void* stream, bool accumulate);

pdr_status pdr_interpolate_backward(const float* attr, uint64_t stride, uint32_t V, uint32_t A, const uint32_t* idx,
                                    uint32_t T, const float* raster, uint32_t views, uint64_t P, const float* grad_out,
                                    float* grad_attr, float* grad_raster, void* stream) {
    return interpolate_backward_impl(attr, stride, V, A, idx, T, raster, views, P, grad_out, grad_attr, grad_raster,
                                     stream, false);
}

pdr_status pdr_interpolate_backward_accumulate(const float* attr, uint64_t stride, uint32_t V, uint32_t A,
                                               const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                               uint64_t P, const float* grad_out, float* grad_attr, float* grad_raster,
                                               void* stream) {
    return interpolate_backward_impl(attr, stride, V, A, idx, T, raster, views, P, grad_out, grad_attr, grad_raster,
                                     stream, true);
}

static pdr_status interpolate_backward_impl(const float* attr, uint64_t stride, uint32_t V, uint32_t A,
                                            const uint32_t* idx, uint32_t T, const float* raster, uint32_t views,
                                            uint64_t P, const float* grad_out, float* grad_attr, float* grad_raster,
                                            void* stream, bool accumulate) {
    if (!attr || !idx || !raster || !grad_out) return fail(PDR_INVALID_ARGUMENT, "attributes, indices, raster and grad_interpolated are required");
    if (A == 0 || V == 0) return fail(PDR_INVALID_ARGUMENT, "vertex_attributes must have shape [vertex_count, attribute_count]");
    if (T == 0) return fail(PDR_INVALID_ARGUMENT, "triangle_indices is incompatible with vertex_attributes");
    if (P == 0 || views == 0) return fail(PDR_INVALID_ARGUMENT, "raster_output has inconsistent dimensions");
    if (P > 0xffffffffull) return fail(PDR_OVERFLOW, "Interpolation pixel count exceeds backend limits");
    if (!aligned(raster, 16) || (grad_raster && !aligned(grad_raster, 16))) return fail(PDR_INVALID_ARGUMENT, "raster buffers must be 16-byte aligned");
    return cuda_status(launch_interpolate_backward(attr, stride, V, A, idx, T, raster, views, P, grad_out, grad_attr,
                                                   grad_raster, (cudaStream_t)stream, accumulate),
                       "interpolate_backward");
}

static pdr_status check_texture(const float* tex, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                                const float* uv, const float* raster, uint32_t views, uint64_t P) {
    if (!tex || !uv || !raster) return fail(PDR_INVALID_ARGUMENT, "texture, uv and raster are required");
    if (tw == 0 || th == 0 || C == 0) return fail(PDR_INVALID_ARGUMENT, "Texture width, height, and channel_count must be positive");
    if (tw > 1073741823u || th > 1073741823u) return fail(PDR_OUT_OF_RANGE, "Texture dimensions exceed portable addressing limits");
    if (mode > 2) return fail(PDR_INVALID_ARGUMENT, "address_mode must be 'clamp', 'wrap', or 'mirror'");
    if (P == 0 || views == 0) return fail(PDR_INVALID_ARGUMENT, "raster_output has inconsistent dimensions");
    if (P > 0xffffffffull || (uint64_t)tw * th > 0xffffffffull) return fail(PDR_OVERFLOW, "Texture operation exceeds backend element limits");
    if (!aligned(raster, 16) || !aligned(uv, 8) || (C == 4 && !aligned(tex, 16))) return fail(PDR_INVALID_ARGUMENT, "texture buffers are misaligned");
    return PDR_OK;
}

pdr_status pdr_texture_forward(const float* tex, uint64_t stride, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                               const float* uv, const float* raster, uint32_t views, uint64_t P, float* out,
                               void* stream) {
    pdr_status st = check_texture(tex, tw, th, C, mode, uv, raster, views, P);
    if (st) return st;
    if (!out || (C == 4 && !aligned(out, 16))) return fail(PDR_INVALID_ARGUMENT, "sampled output is missing or misaligned");
    if (P * C > 0xffffffffull) return fail(PDR_OVERFLOW, "Sampled texture output exceeds backend element limits");
    return cuda_status(launch_texture_forward(tex, stride, tw, th, C, mode, uv, raster, views, P, out, (cudaStream_t)stream),
                       "texture_forward");
}

pdr_status pdr_texture_backward(const float* tex, uint64_t stride, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                                const float* uv, const float* raster, uint32_t views, uint64_t P, const float* grad,
                                float* grad_tex, float* grad_uv, uint32_t* status, void* stream) {
    pdr_status st = check_texture(tex, tw, th, C, mode, uv, raster, views, P);
    if (st) return st;
    if (!grad || !status || (C == 4 && (!aligned(grad, 16) || (grad_tex && !aligned(grad_tex, 16)))))
        return fail(PDR_INVALID_ARGUMENT, "grad_sampled and status are required and must be aligned");
    if (P * C > 0xffffffffull || (uint64_t)tw * th * C > 0xffffffffull || P > 0xffffffffull / 4)
        return fail(PDR_OVERFLOW, "Texture gradient operation exceeds backend element limits");
    return cuda_status(launch_texture_backward(tex, stride, tw, th, C, mode, uv, raster, views, P, grad, grad_tex,
                                               grad_uv, status, (cudaStream_t)stream),
                       "texture_backward");
}

}  // extern "C"

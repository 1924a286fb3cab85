// Calibration kernel for the atomic roofline: vector reductions at the rate the memory system
// sustains. The refiner's photometric and seam gradients and the fused adjoint's texture gradient add
// their bilinear taps with red.global.add.v4.f32 to scattered texels; timing this kernel on buffers
// that fit in L2 and on buffers that do not gives the peak those kernels are measured against.
// No counterpart in the reference.
#include <cuda_runtime.h>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

// Each thread adds to pseudo-random 16-byte slots (a 64-bit mix of the reduction index), so
// consecutive reductions of a warp land on unrelated lines, as bilinear taps of minified textures do.
__global__ void reduction_rate_kernel(float* __restrict__ buffer, uint64_t slots, uint64_t reductions,
                                      uint32_t seed) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < reductions; i += stride) {
        uint64_t h = (i + 1) * 0x9E3779B97F4A7C15ull ^ ((uint64_t)seed << 32);
        h ^= h >> 31;
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 29;
        float* p = buffer + (h % slots) * 4;
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(1.0f), "f"(1.0f), "f"(1.0f),
                     "f"(1.0f)
                     : "memory");
    }
}

}  // namespace
}  // namespace pdr

using namespace pdr;

extern "C" {

pdr_status pdr_calibrate_reductions(float* buffer, uint64_t slots, uint64_t reductions, uint32_t seed, void* stream) {
    if (!buffer || slots == 0) return set_error(PDR_INVALID_ARGUMENT, "buffer and a positive slot count are required");
    if ((uintptr_t)buffer & 15u) return set_error(PDR_INVALID_ARGUMENT, "buffer must be 16-byte aligned");
    if (reductions == 0) return PDR_OK;
    const unsigned blocks = (unsigned)num_sms() * 8u;
    reduction_rate_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(buffer, slots, reductions, seed);
    return set_cuda_error(cudaGetLastError(), "calibrate_reductions");
}

}  // extern "C"

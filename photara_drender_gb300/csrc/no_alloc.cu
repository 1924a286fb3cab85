// pdr_bin_tiles_no_alloc: tile binning whose scratch memory is a fixed array compiled into the
// library, for callers that cannot allocate device memory themselves.
//
// Such callers include code that runs while someone else is capturing a CUDA graph (an allocation
// call there would break the capture), real-time loops that must not take the synchronising path of
// cudaMalloc, and plugin hosts that hand out input and output buffers but no allocator. They still
// pass inputs and outputs; only the scratch space comes from here.
//
// The array lives in device memory of every GPU that loads this library, for the life of the
// process. Its address is looked up once per device (cudaGetSymbolAddress, with that device
// current) on the first call made on that device; make that first call before any stream capture.
// The looked-up address is kept for the life of the process: do not use this entry point across a
// device reset (cudaDeviceReset, or a primary context released and created again), after which the
// array may sit at another address.
// All calls share the one array, so calls that overlap on the GPU (different streams, or different
// host threads without ordering) race with each other: serialise them.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr size_t kStaticScratchBytes = (size_t)PDR_BIN_TILES_NO_ALLOC_SCRATCH_BYTES;

// The scratch space. Device code could name it directly; host code only ever uses the device
// address obtained below (the host-side symbol is a stand-in, not a device pointer).
static __device__ __align__(256) unsigned char g_bin_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_address[kMaxDevices] = {};

// Device address of g_bin_scratch on the current device, looked up on first use.
pdr_status scratch_address(void** out) {
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) return set_cuda_error(err, "cudaGetDevice");
    if (device < 0 || device >= kMaxDevices) return set_error(PDR_OUT_OF_RANGE, "device index beyond 64");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_address[device]) {
        void* ptr = nullptr;
        err = cudaGetSymbolAddress(&ptr, g_bin_scratch);
        if (err != cudaSuccess) return set_cuda_error(err, "cudaGetSymbolAddress(g_bin_scratch)");
        if (!ptr) return set_error(PDR_CUDA_ERROR, "cudaGetSymbolAddress returned a null scratch address");
        g_scratch_address[device] = ptr;
    }
    *out = g_scratch_address[device];
    return PDR_OK;
}

}  // namespace
}  // namespace pdr

using namespace pdr;

extern "C" {

pdr_status pdr_bin_tiles_no_alloc(const float* clip_positions, uint32_t views, uint32_t vertex_count,
                                  const uint32_t* indices, uint32_t triangle_count, uint32_t width, uint32_t height,
                                  const float* viewports, uint32_t* tile_offsets, uint32_t* tile_triangles,
                                  uint64_t capacity, uint32_t* status, void* stream) {
    // the same shape, size and alignment checks as pdr_bin_tiles: the count kernel reads clip
    // positions and viewports as float4, so a misaligned pointer is refused here, before any launch
    pdr_status st = check_raster_args(clip_positions, views, vertex_count, indices, triangle_count, width, height,
                                      viewports);
    if (st != PDR_OK) return st;
    if (!tile_offsets || !status || (capacity && !tile_triangles))
        return set_error(PDR_INVALID_ARGUMENT, "tile_offsets, tile_triangles and status are required");
    // tile offsets are u32: a larger capacity means nothing and would wrap the size computation below
    if (capacity > 0xffffffffull) return set_error(PDR_OVERFLOW, "tile list capacity exceeds the u32 tile offsets");
    const size_t need = bins_workspace_bytes(views, triangle_count, width, height, capacity);
    if (need > kStaticScratchBytes)
        return set_error(PDR_INVALID_ARGUMENT,
                         "pdr_bin_tiles_no_alloc: this binning needs more scratch than the library's fixed "
                         "PDR_BIN_TILES_NO_ALLOC_SCRATCH_BYTES array; use pdr_bin_tiles with a caller workspace");
    void* scratch = nullptr;
    st = scratch_address(&scratch);
    if (st != PDR_OK) return st;
    // launch_bin_tiles clears the per-tile counters itself (cudaMemsetAsync); every other scratch
    // word is written before it is read, so leftovers of the previous call do not matter.
    return set_cuda_error(launch_bin_tiles(clip_positions, views, vertex_count, indices, triangle_count, width, height,
                                           viewports, tile_offsets, tile_triangles, capacity, scratch, status,
                                           (cudaStream_t)stream),
                          "bin_tiles_no_alloc");
}

}  // extern "C"

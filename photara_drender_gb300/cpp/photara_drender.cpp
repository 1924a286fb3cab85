// The photara_drender C++ API (include/photara_drender/*.hpp) implemented over the C ABI of
// include/pdr_capi.h. Inputs are host spans and outputs host vectors, as in the reference
// (src/context.cpp, src/rasterizer.cpp, src/texture_baker.cpp, src/texture_refiner.cpp); each call
// uploads its inputs, runs the CUDA kernels on the context's stream and downloads the results.
// Validation and exception types/messages follow the reference routines cited per method.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pdr_capi.h"
#include "photara_drender/photara_drender.hpp"

namespace photara_drender {
namespace {

constexpr std::uint32_t kTile = 16;

void check(pdr_status st) {
    if (st == PDR_OK) return;
    const std::string msg = pdr_last_error();
    switch (st) {
        case PDR_INVALID_ARGUMENT: throw std::invalid_argument(msg);
        case PDR_OUT_OF_RANGE: throw std::out_of_range(msg);
        case PDR_OVERFLOW: throw std::overflow_error(msg);
        default: throw std::runtime_error(msg);
    }
}

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + " failed: " + cudaGetErrorString(e));
}

template <class T>
class DeviceArray {
public:
    DeviceArray() = default;
    explicit DeviceArray(std::size_t n) : count_(n) {
        if (n) check_cuda(cudaMalloc(reinterpret_cast<void**>(&ptr_), n * sizeof(T)), "cudaMalloc");
    }
    DeviceArray(const T* host, std::size_t n, cudaStream_t s) : DeviceArray(n) {
        if (n) check_cuda(cudaMemcpyAsync(ptr_, host, n * sizeof(T), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    }
    ~DeviceArray() {
        if (ptr_) cudaFree(ptr_);
    }
    DeviceArray(DeviceArray&& o) noexcept : ptr_(std::exchange(o.ptr_, nullptr)), count_(std::exchange(o.count_, 0)) {}
    DeviceArray& operator=(DeviceArray&& o) noexcept {
        if (this != &o) {
            if (ptr_) cudaFree(ptr_);
            ptr_ = std::exchange(o.ptr_, nullptr);
            count_ = std::exchange(o.count_, 0);
        }
        return *this;
    }
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;

    T* get() const { return ptr_; }
    std::size_t size() const { return count_; }
    void zero(cudaStream_t s) {
        if (count_) check_cuda(cudaMemsetAsync(ptr_, 0, count_ * sizeof(T), s), "cudaMemsetAsync");
    }
    std::vector<T> download(cudaStream_t s, std::size_t n = ~std::size_t{0}) const {
        n = std::min(n, count_);
        std::vector<T> out(n);
        if (n) check_cuda(cudaMemcpyAsync(out.data(), ptr_, n * sizeof(T), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        return out;
    }

private:
    T* ptr_ = nullptr;
    std::size_t count_ = 0;
};

template <class T>
DeviceArray<T> upload(std::span<const T> v, cudaStream_t s) {
    return DeviceArray<T>(v.data(), v.size(), s);
}

DeviceInfo query_device(std::uint32_t index) {
    char name[256] = {};
    std::uint32_t vendor = 0, device = 0, api = 0;
    std::int32_t sms = 0;
    check(pdr_device_info(static_cast<std::int32_t>(index), name, sizeof(name), &vendor, &device, &api, &sms));
    DeviceInfo info;
    info.name = name;
    info.vendor_id = vendor;
    info.device_id = device;
    info.api_version = api;
    info.supports_ray_query = true;  // the library's BVH ray caster (csrc/bvh.cu)
    return info;
}

// src/rasterizer.cpp:48-59
Viewport resolve_viewport(std::uint32_t w, std::uint32_t h, const std::optional<Viewport>& requested) {
    const Viewport vp = requested.value_or(Viewport{0.0F, 0.0F, static_cast<float>(w), static_cast<float>(h)});
    if (!std::isfinite(vp.x) || !std::isfinite(vp.y) || !std::isfinite(vp.width) || !std::isfinite(vp.height) ||
        vp.width <= 0.0F || vp.height <= 0.0F) {
        throw std::invalid_argument("viewport must contain finite values and positive dimensions");
    }
    return vp;
}

// src/rasterizer.cpp:29-40
void validate_mesh(std::span<const float> positions, std::span<const std::uint32_t> indices) {
    if (positions.empty() || positions.size() % 4 != 0)
        throw std::invalid_argument("clip_positions must have shape [vertex_count, 4]");
    if (indices.empty() || indices.size() % 3 != 0)
        throw std::invalid_argument("triangle_indices must have shape [triangle_count, 3]");
    const auto vertex_count = positions.size() / 4;
    if (std::any_of(indices.begin(), indices.end(), [vertex_count](std::uint32_t i) { return i >= vertex_count; }))
        throw std::out_of_range("triangle_indices contains an invalid vertex index");
}

}  // namespace

// ---- Context ----------------------------------------------------------------------------------

class Context::Impl {
public:
    explicit Impl(const ContextOptions& options) {
        const int count = pdr_device_count();
        if (count <= 0) throw std::runtime_error("No CUDA devices were found");
        if (options.device_index >= static_cast<std::uint32_t>(count))
            throw std::out_of_range("device_index is out of range");
        device = static_cast<int>(options.device_index);
        check_cuda(cudaSetDevice(device), "cudaSetDevice");
        check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        info = query_device(options.device_index);
    }
    ~Impl() {
        if (stream) cudaStreamDestroy(stream);
    }
    void activate() const { check_cuda(cudaSetDevice(device), "cudaSetDevice"); }

    int device = 0;
    cudaStream_t stream = nullptr;
    DeviceInfo info;
    std::mutex mutex;  // one dispatch at a time per context, as src/context_internal.hpp:101
    std::uint64_t tile_capacity = 0;
};

Context::Context(const ContextOptions& options) : impl_(std::make_unique<Impl>(options)) {}
Context::~Context() = default;
Context::Context(Context&&) noexcept = default;
Context& Context::operator=(Context&&) noexcept = default;

const DeviceInfo& Context::device_info() const noexcept { return impl_->info; }

std::vector<DeviceInfo> Context::enumerate_devices() {
    std::vector<DeviceInfo> out;
    const int count = pdr_device_count();
    for (int i = 0; i < count; ++i) out.push_back(query_device(static_cast<std::uint32_t>(i)));
    return out;
}

// ---- shared raster helper -----------------------------------------------------------------------

namespace {

// Bins and rasterizes `views` views of equal size; raster (and derivatives) stay on the device.
void rasterize_device(Context::Impl& ctx, const float* d_clip, std::uint32_t views, std::uint32_t V,
                      const std::uint32_t* d_idx, std::uint32_t T, std::uint32_t W, std::uint32_t H,
                      const float* d_viewports, std::uint32_t cull, float* d_raster, float* d_deriv) {
    const std::uint64_t tiles = static_cast<std::uint64_t>((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile);
    DeviceArray<std::uint32_t> offsets(tiles * views + 1);
    DeviceArray<std::uint32_t> status(PDR_STATUS_WORDS);
    std::uint64_t capacity = std::max<std::uint64_t>(ctx.tile_capacity, 2ull * T * views + 1024);
    for (int attempt = 0; attempt < 3; ++attempt) {
        DeviceArray<std::uint32_t> list(capacity);
        const std::size_t ws_bytes = pdr_bin_tiles_workspace_bytes(views, T, W, H, capacity);
        DeviceArray<unsigned char> ws(std::max<std::size_t>(ws_bytes, 1));
        status.zero(ctx.stream);
        check(pdr_bin_tiles(d_clip, views, V, d_idx, T, W, H, d_viewports, offsets.get(), list.get(), capacity,
                            ws.get(), ws_bytes, status.get(), ctx.stream));
        const auto st = status.download(ctx.stream);
        if (st[PDR_STATUS_TILE_ENTRIES_HI] != 0) throw std::overflow_error("Tile triangle list exceeds backend limits");
        if (!st[PDR_STATUS_TILE_OVERFLOW]) {
            ctx.tile_capacity = std::max(ctx.tile_capacity, capacity);
            check(pdr_rasterize_forward(d_clip, views, V, d_idx, T, W, H, d_viewports, cull, offsets.get(), list.get(),
                                        capacity, d_raster, d_deriv, ctx.stream));
            return;
        }
        capacity = st[PDR_STATUS_TILE_ENTRIES] + st[PDR_STATUS_TILE_ENTRIES] / 8 + 1024;
    }
    throw std::runtime_error("tile binning did not converge");
}

}  // namespace

// ---- Rasterizer ---------------------------------------------------------------------------------

class Rasterizer::Impl {
public:
    explicit Impl(Context::Impl& c) : ctx(c) {}
    Context::Impl& ctx;
};

Rasterizer::Rasterizer(Context& context) : impl_(std::make_unique<Impl>(*context.impl_)) {}
Rasterizer::~Rasterizer() = default;
Rasterizer::Rasterizer(Rasterizer&&) noexcept = default;
Rasterizer& Rasterizer::operator=(Rasterizer&&) noexcept = default;

// src/rasterizer.cpp:373-442
RasterizeOutput Rasterizer::forward(std::span<const float> clip_positions, std::span<const std::uint32_t> triangle_indices,
                                    const RasterizeOptions& options) {
    validate_mesh(clip_positions, triangle_indices);
    if (options.width == 0 || options.height == 0)
        throw std::invalid_argument("Rasterization width and height must be positive");
    const Viewport vp = resolve_viewport(options.width, options.height, options.viewport);
    Context::Impl& ctx = impl_->ctx;
    std::lock_guard<std::mutex> lock(ctx.mutex);
    ctx.activate();
    const std::size_t P = static_cast<std::size_t>(options.width) * options.height;
    auto d_clip = upload(clip_positions, ctx.stream);
    auto d_idx = upload(triangle_indices, ctx.stream);
    const float vps[4] = {vp.x, vp.y, vp.width, vp.height};
    DeviceArray<float> d_vp(vps, 4, ctx.stream);
    DeviceArray<float> d_raster(P * 4);
    DeviceArray<float> d_deriv(options.output_barycentric_derivatives ? P * 4 : 0);
    rasterize_device(ctx, d_clip.get(), 1, static_cast<std::uint32_t>(clip_positions.size() / 4), d_idx.get(),
                     static_cast<std::uint32_t>(triangle_indices.size() / 3), options.width, options.height, d_vp.get(),
                     static_cast<std::uint32_t>(options.cull_mode), d_raster.get(), d_deriv.get());
    RasterizeOutput out;
    out.width = options.width;
    out.height = options.height;
    out.raster = d_raster.download(ctx.stream);
    if (options.output_barycentric_derivatives) out.barycentric_derivatives = d_deriv.download(ctx.stream);
    out.viewport = vp;
    return out;
}

// src/rasterizer.cpp:444-537
std::vector<float> Rasterizer::backward(std::span<const float> clip_positions,
                                        std::span<const std::uint32_t> triangle_indices,
                                        const RasterizeOutput& forward_output, std::span<const float> grad_raster,
                                        std::span<const float> grad_barycentric_derivatives) {
    validate_mesh(clip_positions, triangle_indices);
    const std::size_t P = static_cast<std::size_t>(forward_output.width) * forward_output.height;
    if (forward_output.width == 0 || forward_output.height == 0 || forward_output.raster.size() != P * 4)
        throw std::invalid_argument("forward_output has inconsistent dimensions");
    if (grad_raster.size() != P * 4) throw std::invalid_argument("grad_raster must have shape [height, width, 4]");
    // the reference rejects a derivative gradient (rasterizer.cpp:459-462); this build propagates it
    if (!grad_barycentric_derivatives.empty() && grad_barycentric_derivatives.size() != P * 4)
        throw std::invalid_argument("grad_barycentric_derivatives must have shape [height, width, 4]");
    const Viewport vp = resolve_viewport(
        forward_output.width, forward_output.height,
        forward_output.viewport.width > 0.0F ? std::optional<Viewport>(forward_output.viewport) : std::nullopt);
    Context::Impl& ctx = impl_->ctx;
    std::lock_guard<std::mutex> lock(ctx.mutex);
    ctx.activate();
    const auto V = static_cast<std::uint32_t>(clip_positions.size() / 4);
    auto d_clip = upload(clip_positions, ctx.stream);
    auto d_idx = upload(triangle_indices, ctx.stream);
    auto d_raster = upload(std::span<const float>(forward_output.raster), ctx.stream);
    auto d_grad = upload(grad_raster, ctx.stream);
    const float vps[4] = {vp.x, vp.y, vp.width, vp.height};
    DeviceArray<float> d_vp(vps, 4, ctx.stream);
    DeviceArray<float> d_out(static_cast<std::size_t>(V) * 4);
    DeviceArray<float> d_gdb;
    if (!grad_barycentric_derivatives.empty()) d_gdb = upload(grad_barycentric_derivatives, ctx.stream);
    check(pdr_rasterize_backward_derivatives(
        d_clip.get(), 1, V, d_idx.get(), static_cast<std::uint32_t>(triangle_indices.size() / 3), forward_output.width,
        forward_output.height, d_vp.get(), d_raster.get(), d_grad.get(), d_gdb.get(), d_out.get(), ctx.stream));
    return d_out.download(ctx.stream);
}

// src/rasterizer.cpp:539-601
InterpolateOutput Rasterizer::interpolate_forward(std::span<const float> vertex_attributes, std::uint32_t attribute_count,
                                                  std::span<const std::uint32_t> triangle_indices,
                                                  const RasterizeOutput& raster_output) {
    if (attribute_count == 0 || vertex_attributes.empty() || vertex_attributes.size() % attribute_count != 0)
        throw std::invalid_argument("vertex_attributes must have shape [vertex_count, attribute_count]");
    if (triangle_indices.empty() || triangle_indices.size() % 3 != 0)
        throw std::invalid_argument("triangle_indices must have shape [triangle_count, 3]");
    const auto V = static_cast<std::uint32_t>(vertex_attributes.size() / attribute_count);
    if (std::any_of(triangle_indices.begin(), triangle_indices.end(), [V](std::uint32_t i) { return i >= V; }))
        throw std::out_of_range("triangle_indices contains an invalid attribute vertex index");
    const std::size_t P = static_cast<std::size_t>(raster_output.width) * raster_output.height;
    if (raster_output.width == 0 || raster_output.height == 0 || raster_output.raster.size() != P * 4)
        throw std::invalid_argument("raster_output has inconsistent dimensions");
    if (P > std::numeric_limits<std::uint32_t>::max())
        throw std::overflow_error("Interpolation pixel count exceeds backend limits");
    Context::Impl& ctx = impl_->ctx;
    std::lock_guard<std::mutex> lock(ctx.mutex);
    ctx.activate();
    auto d_attr = upload(vertex_attributes, ctx.stream);
    auto d_idx = upload(triangle_indices, ctx.stream);
    auto d_raster = upload(std::span<const float>(raster_output.raster), ctx.stream);
    DeviceArray<float> d_out(P * attribute_count);
    check(pdr_interpolate_forward(d_attr.get(), 0, V, attribute_count, d_idx.get(),
                                  static_cast<std::uint32_t>(triangle_indices.size() / 3), d_raster.get(), 1, P,
                                  d_out.get(), ctx.stream));
    InterpolateOutput out;
    out.width = raster_output.width;
    out.height = raster_output.height;
    out.attribute_count = attribute_count;
    out.values = d_out.download(ctx.stream);
    return out;
}

// src/rasterizer.cpp:603-683
InterpolateGradients Rasterizer::interpolate_backward(std::span<const float> vertex_attributes,
                                                      std::uint32_t attribute_count,
                                                      std::span<const std::uint32_t> triangle_indices,
                                                      const RasterizeOutput& raster_output,
                                                      std::span<const float> grad_interpolated) {
    if (attribute_count == 0 || vertex_attributes.empty() || vertex_attributes.size() % attribute_count != 0)
        throw std::invalid_argument("vertex_attributes must have shape [vertex_count, attribute_count]");
    const auto V = static_cast<std::uint32_t>(vertex_attributes.size() / attribute_count);
    if (triangle_indices.empty() || triangle_indices.size() % 3 != 0 ||
        std::any_of(triangle_indices.begin(), triangle_indices.end(), [V](std::uint32_t i) { return i >= V; }))
        throw std::invalid_argument("triangle_indices is incompatible with vertex_attributes");
    const std::size_t P = static_cast<std::size_t>(raster_output.width) * raster_output.height;
    if (raster_output.width == 0 || raster_output.height == 0 || raster_output.raster.size() != P * 4)
        throw std::invalid_argument("raster_output has inconsistent dimensions");
    if (grad_interpolated.size() != P * attribute_count)
        throw std::invalid_argument("grad_interpolated must have shape [height, width, attribute_count]");
    if (P > std::numeric_limits<std::uint32_t>::max())
        throw std::overflow_error("Interpolation pixel count exceeds backend limits");
    Context::Impl& ctx = impl_->ctx;
    std::lock_guard<std::mutex> lock(ctx.mutex);
    ctx.activate();
    auto d_attr = upload(vertex_attributes, ctx.stream);
    auto d_idx = upload(triangle_indices, ctx.stream);
    auto d_raster = upload(std::span<const float>(raster_output.raster), ctx.stream);
    auto d_grad = upload(grad_interpolated, ctx.stream);
    DeviceArray<float> d_ga(vertex_attributes.size()), d_gr(P * 4);
    check(pdr_interpolate_backward(d_attr.get(), 0, V, attribute_count, d_idx.get(),
                                   static_cast<std::uint32_t>(triangle_indices.size() / 3), d_raster.get(), 1, P,
                                   d_grad.get(), d_ga.get(), d_gr.get(), ctx.stream));
    InterpolateGradients out;
    out.attributes = d_ga.download(ctx.stream);
    out.raster = d_gr.download(ctx.stream);
    return out;
}

namespace {
// src/rasterizer.cpp:260-289
void validate_texture_inputs(std::span<const float> texture, const TextureDesc& d, std::span<const float> uv,
                             const RasterizeOutput& raster_output) {
    if (d.width == 0 || d.height == 0 || d.channel_count == 0)
        throw std::invalid_argument("Texture width, height, and channel_count must be positive");
    if (d.width > static_cast<std::uint32_t>(std::numeric_limits<std::int32_t>::max() / 2) ||
        d.height > static_cast<std::uint32_t>(std::numeric_limits<std::int32_t>::max() / 2))
        throw std::out_of_range("Texture dimensions exceed portable addressing limits");
    if (texture.size() != static_cast<std::size_t>(d.width) * d.height * d.channel_count)
        throw std::invalid_argument("texture must have shape [texture_height, texture_width, channel_count]");
    const std::size_t P = static_cast<std::size_t>(raster_output.width) * raster_output.height;
    if (raster_output.width == 0 || raster_output.height == 0 || raster_output.raster.size() != P * 4)
        throw std::invalid_argument("raster_output has inconsistent dimensions");
    if (uv.size() != P * 2) throw std::invalid_argument("uv must have shape [image_height, image_width, 2]");
    if (P > std::numeric_limits<std::uint32_t>::max() ||
        static_cast<std::size_t>(d.width) * d.height > std::numeric_limits<std::uint32_t>::max())
        throw std::overflow_error("Texture operation exceeds backend element limits");
}
}  // namespace

// src/rasterizer.cpp:685-735
TextureOutput Rasterizer::texture_forward(std::span<const float> texture, const TextureDesc& texture_desc,
                                          std::span<const float> uv, const RasterizeOutput& raster_output) {
    validate_texture_inputs(texture, texture_desc, uv, raster_output);
    const std::size_t P = static_cast<std::size_t>(raster_output.width) * raster_output.height;
    Context::Impl& ctx = impl_->ctx;
    std::lock_guard<std::mutex> lock(ctx.mutex);
    ctx.activate();
    auto d_tex = upload(texture, ctx.stream);
    auto d_uv = upload(uv, ctx.stream);
    auto d_raster = upload(std::span<const float>(raster_output.raster), ctx.stream);
    DeviceArray<float> d_out(P * texture_desc.channel_count);
    check(pdr_texture_forward(d_tex.get(), 0, texture_desc.width, texture_desc.height, texture_desc.channel_count,
                              static_cast<std::uint32_t>(texture_desc.address_mode), d_uv.get(), d_raster.get(), 1, P,
                              d_out.get(), ctx.stream));
    TextureOutput out;
    out.width = raster_output.width;
    out.height = raster_output.height;
    out.channel_count = texture_desc.channel_count;
    out.values = d_out.download(ctx.stream);
    return out;
}

// src/rasterizer.cpp:737-829
TextureGradients Rasterizer::texture_backward(std::span<const float> texture, const TextureDesc& texture_desc,
                                              std::span<const float> uv, const RasterizeOutput& raster_output,
                                              std::span<const float> grad_sampled, bool compute_uv_gradient) {
    validate_texture_inputs(texture, texture_desc, uv, raster_output);
    const std::size_t P = static_cast<std::size_t>(raster_output.width) * raster_output.height;
    if (grad_sampled.size() != P * texture_desc.channel_count)
        throw std::invalid_argument("grad_sampled must have shape [image_height, image_width, channel_count]");
    Context::Impl& ctx = impl_->ctx;
    std::lock_guard<std::mutex> lock(ctx.mutex);
    ctx.activate();
    auto d_tex = upload(texture, ctx.stream);
    auto d_uv = upload(uv, ctx.stream);
    auto d_raster = upload(std::span<const float>(raster_output.raster), ctx.stream);
    auto d_grad = upload(grad_sampled, ctx.stream);
    DeviceArray<float> d_gt(texture.size()), d_gu(compute_uv_gradient ? P * 2 : 0);
    DeviceArray<std::uint32_t> status(PDR_STATUS_WORDS);
    status.zero(ctx.stream);
    check(pdr_texture_backward(d_tex.get(), 0, texture_desc.width, texture_desc.height, texture_desc.channel_count,
                               static_cast<std::uint32_t>(texture_desc.address_mode), d_uv.get(), d_raster.get(), 1, P,
                               d_grad.get(), d_gt.get(), d_gu.get(), status.get(), ctx.stream));
    const auto st = status.download(ctx.stream);
    if (st[PDR_STATUS_TEXEL_ERROR] == 1) throw std::invalid_argument("uv contains a non-finite value in a covered pixel");
    if (st[PDR_STATUS_TEXEL_ERROR] == 2) throw std::out_of_range("uv is too large for portable texture addressing");
    TextureGradients out;
    out.texture = d_gt.download(ctx.stream);
    if (compute_uv_gradient) out.uv = d_gu.download(ctx.stream);
    return out;
}

// ---- atlas padding and surface fill (src/texture_padding.cpp:100-184,226-351) -----------------

namespace {

// A stream on the current device for the free padding functions, which take no Context.
struct ScopedStream {
    cudaStream_t s = nullptr;
    ScopedStream() { check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate"); }
    ~ScopedStream() {
        if (s) cudaStreamDestroy(s);
    }
    ScopedStream(const ScopedStream&) = delete;
    ScopedStream& operator=(const ScopedStream&) = delete;
};

std::uint32_t pad_status(const DeviceArray<std::uint32_t>& status, cudaStream_t s) {
    return status.download(s)[PDR_STATUS_PAD_ERROR];
}

}  // namespace

SurfaceFillStats fill_texture_on_surface(TextureBakeOutput& output, std::span<const std::uint32_t> triangle_indices) {
    const std::size_t pixels = static_cast<std::size_t>(output.width) * output.height;
    if (pixels == 0 || triangle_indices.empty() || triangle_indices.size() % 3 != 0 ||
        output.face_ids.size() != pixels || output.valid_mask.size() != pixels || output.color.size() % pixels != 0)
        throw std::invalid_argument("surface fill requires mesh face IDs and a valid atlas");
    const std::size_t channels = output.color.size() / pixels;
    if (channels != 3 && channels != 4) throw std::invalid_argument("surface fill requires RGB or RGBA colours");
    const std::size_t faces = triangle_indices.size() / 3;
    if (faces >= UINT32_MAX / 3) throw std::invalid_argument("surface fill has too many faces");
    ScopedStream stream;
    const cudaStream_t s = stream.s;
    std::vector<float> filled = output.filled_mask.size() == pixels ? output.filled_mask
                                                                   : std::vector<float>(pixels, 0.0F);
    DeviceArray<float> d_color(output.color.data(), output.color.size(), s);
    DeviceArray<float> d_valid(output.valid_mask.data(), pixels, s);
    DeviceArray<std::uint32_t> d_faces(output.face_ids.data(), pixels, s);
    DeviceArray<float> d_filled(filled.data(), pixels, s);
    DeviceArray<std::uint32_t> d_idx(triangle_indices.data(), triangle_indices.size(), s);
    std::size_t bytes = 0;
    check(pdr_surface_fill_workspace_bytes(output.width, output.height, static_cast<std::uint32_t>(faces), &bytes));
    DeviceArray<unsigned char> ws(bytes);
    DeviceArray<std::uint64_t> d_stats(4);
    DeviceArray<std::uint32_t> status(PDR_STATUS_WORDS);
    status.zero(s);
    check(pdr_fill_texture_on_surface(d_color.get(), static_cast<std::uint32_t>(channels), d_valid.get(),
                                      d_faces.get(), d_filled.get(), output.width, output.height, d_idx.get(),
                                      static_cast<std::uint32_t>(faces), ws.get(), bytes, d_stats.get(),
                                      status.get(), s));
    const std::uint32_t err = pad_status(status, s);
    if (err & 2u) throw std::invalid_argument("atlas face ID is out of range");
    if (err & 4u) throw std::invalid_argument("surface fill mesh has a degenerate edge");
    if (err & 8u) throw std::invalid_argument("surface fill requires manifold edges");
    const auto st = d_stats.download(s);
    output.color = d_color.download(s);
    output.filled_mask = d_filled.download(s);
    SurfaceFillStats out;
    out.filled_texels = st[0];
    out.remaining_texels = st[1];
    out.measured_faces = st[2];
    out.propagated_faces = st[3];
    return out;
}

TexturePaddingStats pad_texture_atlas(TextureBakeOutput& output, const TexturePaddingOptions& options) {
    const auto start = std::chrono::steady_clock::now();
    const std::uint32_t width = output.width, height = output.height;
    if (width == 0 || height == 0) throw std::invalid_argument("cannot pad an empty atlas");
    if (width > 16384 || height > 16384) throw std::invalid_argument("atlas dimensions exceed the supported maximum");
    const std::size_t pixels = static_cast<std::size_t>(width) * height;
    if (output.color.size() % pixels != 0)
        throw std::invalid_argument("atlas color size does not match its dimensions");
    const std::size_t channels = output.color.size() / pixels;
    if (channels != 3 && channels != 4) throw std::invalid_argument("atlas color must have 3 or 4 channels");
    if (output.valid_mask.size() != pixels)
        throw std::invalid_argument("atlas valid_mask must match the atlas dimensions");
    if (!std::isfinite(options.valid_threshold) || options.valid_threshold <= 0.0F || options.valid_threshold > 1.0F)
        throw std::invalid_argument("valid_threshold must be within (0, 1]");
    if (output.filled_mask.size() != pixels) output.filled_mask.assign(pixels, 0.0F);
    const bool has_coverage = output.coverage_mask.size() == pixels;
    ScopedStream stream;
    const cudaStream_t s = stream.s;
    DeviceArray<float> d_color(output.color.data(), output.color.size(), s);
    DeviceArray<float> d_valid(output.valid_mask.data(), pixels, s);
    DeviceArray<float> d_cov = has_coverage ? DeviceArray<float>(output.coverage_mask.data(), pixels, s)
                                            : DeviceArray<float>();
    DeviceArray<float> d_filled(output.filled_mask.data(), pixels, s);
    std::size_t bytes = 0;
    check(pdr_pad_workspace_bytes(width, height, static_cast<std::uint32_t>(channels), &bytes));
    DeviceArray<unsigned char> ws(bytes);
    DeviceArray<std::uint64_t> d_stats(5);
    DeviceArray<std::uint32_t> status(PDR_STATUS_WORDS);
    status.zero(s);
    check(pdr_pad_texture_atlas(d_color.get(), static_cast<std::uint32_t>(channels), d_valid.get(),
                                has_coverage ? d_cov.get() : nullptr, d_filled.get(), width, height, options.margin,
                                options.fill_unobserved ? 1u : 0u, options.maximum_fill_distance,
                                options.valid_threshold, ws.get(), bytes, d_stats.get(), status.get(), s));
    if (pad_status(status, s) & 1u) throw std::runtime_error("atlas padding sweep did not complete");
    const auto st = d_stats.download(s);
    output.color = d_color.download(s);
    output.filled_mask = d_filled.download(s);
    TexturePaddingStats out;
    out.valid_texels = st[0];
    out.gutter_texels = st[1];
    out.unobserved_texels = st[2];
    out.remaining_unobserved = st[3];
    out.filled_texels = st[4];
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    return out;
}

// ---- softmax scale (src/texture_padding.cpp:187-224) ------------------------------------------

float suggest_softmax_scale(std::span<const float> positions, std::span<const float> camera_positions) {
    if (positions.size() < 3 || positions.size() % 3 != 0)
        throw std::invalid_argument("positions must have shape [vertex_count, 3]");
    if (camera_positions.size() < 3 || camera_positions.size() % 3 != 0)
        throw std::invalid_argument("camera_positions must have shape [camera_count, 3]");
    const std::size_t n = positions.size() / 3, cams = camera_positions.size() / 3;
    const std::size_t stride = std::max<std::size_t>(1, n / 10000);
    double best = std::numeric_limits<double>::infinity();
    for (std::size_t v = 0; v < n; v += stride) {
        const double x = positions[v * 3], y = positions[v * 3 + 1], z = positions[v * 3 + 2];
        if (!std::isfinite(x) || !std::isfinite(y) || !std::isfinite(z)) continue;
        for (std::size_t c = 0; c < cams; ++c) {
            const double dx = camera_positions[c * 3] - x, dy = camera_positions[c * 3 + 1] - y;
            const double dz = camera_positions[c * 3 + 2] - z;
            best = std::min(best, dx * dx + dy * dy + dz * dz);
        }
    }
    if (!std::isfinite(best) || best <= 0.0) return 0.0F;
    return static_cast<float>(20.0 * best);
}

// ---- TextureBaker (src/texture_baker.cpp:156-361) -----------------------------------------------

class TextureBaker::Impl {
public:
    explicit Impl(Context::Impl& c) : ctx(c) {}
    Context::Impl& ctx;
};

TextureBaker::TextureBaker(Context& context) : impl_(std::make_unique<Impl>(*context.impl_)) {}
TextureBaker::~TextureBaker() = default;
TextureBaker::TextureBaker(TextureBaker&&) noexcept = default;
TextureBaker& TextureBaker::operator=(TextureBaker&&) noexcept = default;

namespace {
Viewport view_viewport(const ProjectionView& v) {
    const Viewport vp = v.viewport.value_or(Viewport{0.0F, 0.0F, static_cast<float>(v.width), static_cast<float>(v.height)});
    if (!std::isfinite(vp.x) || !std::isfinite(vp.y) || !std::isfinite(vp.width) || !std::isfinite(vp.height) ||
        vp.width <= 0.0F || vp.height <= 0.0F)
        throw std::invalid_argument("projection viewport must contain finite values and positive dimensions");
    return vp;
}
}  // namespace

TextureBakeOutput TextureBaker::bake(std::span<const float> positions, std::span<const float> normals,
                                     std::span<const float> uv, std::span<const std::uint32_t> triangle_indices,
                                     std::span<const ProjectionView> views, const TextureBakeOptions& options) {
    // texture_baker.cpp:39-60 / 163-180
    if (positions.empty() || positions.size() % 3 != 0)
        throw std::invalid_argument("positions must have shape [vertex_count, 3]");
    const std::size_t V = positions.size() / 3;
    if (normals.size() != positions.size()) throw std::invalid_argument("normals must have shape [vertex_count, 3]");
    if (uv.size() != V * 2) throw std::invalid_argument("uv must have shape [vertex_count, 2]");
    if (triangle_indices.empty() || triangle_indices.size() % 3 != 0)
        throw std::invalid_argument("triangle_indices must have shape [triangle_count, 3]");
    if (std::any_of(triangle_indices.begin(), triangle_indices.end(), [V](std::uint32_t i) { return i >= V; }))
        throw std::out_of_range("triangle_indices contains an invalid vertex index");
    if (views.empty()) throw std::invalid_argument("at least one projection view is required");
    if (options.width == 0 || options.height == 0 || options.pcf_radius > 4 || !std::isfinite(options.ray_origin_bias) ||
        options.ray_origin_bias <= 0.0F || !std::isfinite(options.mask_floor) || options.mask_floor < 0.0F ||
        options.mask_floor > 1.0F)
        throw std::invalid_argument("atlas dimensions are invalid or pcf_radius exceeds 4");
    Context::Impl& ctx = impl_->ctx;
    const bool ray_requested = options.visibility_mode != VisibilityMode::shadow_map;
    if (ray_requested && !ctx.info.supports_ray_query && !options.allow_visibility_fallback)
        throw std::runtime_error("ray-query visibility was requested but the selected device does not support it");
    std::vector<Viewport> vps;
    for (const auto& v : views) {
        if (v.width == 0 || v.height == 0 || (v.channel_count != 3 && v.channel_count != 4))
            throw std::invalid_argument("projection image must have nonzero dimensions and 3 or 4 channels");
        const std::size_t P = static_cast<std::size_t>(v.width) * v.height;
        if (v.image.size() != P * v.channel_count)
            throw std::invalid_argument("projection image data size does not match its descriptor");
        if (!v.visibility_mask.empty() && v.visibility_mask.size() != P)
            throw std::invalid_argument("projection visibility_mask must have shape [height, width]");
        if (!std::isfinite(v.weight) || v.weight < 0.0F || !std::isfinite(v.depth_bias) || v.depth_bias < 0.0F ||
            !std::isfinite(v.min_view_cosine) || v.min_view_cosine < -1.0F || v.min_view_cosine > 1.0F)
            throw std::invalid_argument("projection confidence parameters are invalid");
        vps.push_back(view_viewport(v));
    }
    std::lock_guard<std::mutex> lock(ctx.mutex);
    ctx.activate();
    cudaStream_t s = ctx.stream;
    const auto Vu = static_cast<std::uint32_t>(V);
    const auto T = static_cast<std::uint32_t>(triangle_indices.size() / 3);
    const std::uint32_t AW = options.width, AH = options.height;
    const std::size_t N = static_cast<std::size_t>(AW) * AH;
    auto d_pos = upload(positions, s);
    auto d_nrm = upload(normals, s);
    auto d_uv = upload(uv, s);
    auto d_idx = upload(triangle_indices, s);
    // atlas G-buffer
    DeviceArray<float> d_aclip(V * 4), d_araster(N * 4), d_apos(N * 3), d_anrm(N * 3);
    check(pdr_atlas_clip_positions(d_uv.get(), Vu, d_aclip.get(), s));
    const float avp[4] = {0.0F, 0.0F, static_cast<float>(AW), static_cast<float>(AH)};
    DeviceArray<float> d_avp(avp, 4, s);
    rasterize_device(ctx, d_aclip.get(), 1, Vu, d_idx.get(), T, AW, AH, d_avp.get(), 0, d_araster.get(), nullptr);
    check(pdr_interpolate_forward(d_pos.get(), 0, Vu, 3, d_idx.get(), T, d_araster.get(), 1, N, d_apos.get(), s));
    check(pdr_interpolate_forward(d_nrm.get(), 0, Vu, 3, d_idx.get(), T, d_araster.get(), 1, N, d_anrm.get(), s));
    float scale = options.softmax_scale;
    if (options.blend_mode == ProjectionBlendMode::softmax && (!(scale > 0.0F) || !std::isfinite(scale))) {
        std::vector<float> cams(views.size() * 3);
        for (std::size_t i = 0; i < views.size(); ++i) std::copy_n(views[i].camera_position.begin(), 3, cams.begin() + i * 3);
        scale = suggest_softmax_scale(positions, cams);
        if (!(scale > 0.0F) || !std::isfinite(scale)) scale = 1.0F;
    }
    const std::uint32_t vis_mode = static_cast<std::uint32_t>(options.visibility_mode);
    // shadow rasters, one per view (not needed for ray-only visibility)
    std::vector<DeviceArray<float>> images, masks, shadows;
    std::vector<pdr_projection_view> table(views.size());
    DeviceArray<float> d_clip(V * 4);
    for (std::size_t k = 0; k < views.size(); ++k) {
        const auto& v = views[k];
        const std::size_t P = static_cast<std::size_t>(v.width) * v.height;
        DeviceArray<float> d_m(v.world_to_clip.data(), 16, s);
        check(pdr_transform_positions(d_pos.get(), Vu, d_m.get(), 1, d_clip.get(), s));
        const float vp4[4] = {vps[k].x, vps[k].y, vps[k].width, vps[k].height};
        DeviceArray<float> d_vvp(vp4, 4, s);
        DeviceArray<float> shadow(vis_mode == 2 ? 0 : P * 4);
        if (vis_mode != 2)
            rasterize_device(ctx, d_clip.get(), 1, Vu, d_idx.get(), T, v.width, v.height, d_vvp.get(), 0,
                             shadow.get(), nullptr);
        images.push_back(upload(std::span<const float>(v.image), s));
        masks.push_back(upload(std::span<const float>(v.visibility_mask), s));
        pdr_projection_view& t = table[k];
        std::memcpy(t.world_to_clip, v.world_to_clip.data(), sizeof(t.world_to_clip));
        std::memcpy(t.camera_position, v.camera_position.data(), sizeof(t.camera_position));
        t.weight = options.blend_mode == ProjectionBlendMode::softmax ? v.weight * scale : v.weight;
        t.viewport[0] = vps[k].x;
        t.viewport[1] = vps[k].y;
        t.viewport[2] = vps[k].width;
        t.viewport[3] = vps[k].height;
        t.width = v.width;
        t.height = v.height;
        t.channel_count = v.channel_count;
        t.has_mask = v.visibility_mask.empty() ? 0u : 1u;
        t.depth_bias = v.depth_bias;
        t.min_view_cosine = v.min_view_cosine;
        t.mask_floor = v.visibility_mask.empty() ? 0.0F : options.mask_floor;
        t.reserved = 0.0F;
        t.image = images.back().get();
        t.visibility_mask = masks.back().get();
        t.shadow_raster = shadow.get();
        t.ray_visibility = nullptr;
        shadows.push_back(std::move(shadow));
    }
    DeviceArray<unsigned char> d_table(reinterpret_cast<const unsigned char*>(table.data()),
                                       table.size() * sizeof(pdr_projection_view), s);
    // ray visibility bits (visibility modes 1 and 2): BVH of the world-space mesh, one ray per texel and
    // view that the projection reads
    DeviceArray<std::uint32_t> ray_bits;
    if (vis_mode != 0) {
        std::size_t bvh_bytes = 0, build_bytes = 0;
        check(pdr_bvh_sizes(T, &bvh_bytes, &build_bytes));
        DeviceArray<unsigned char> bvh(bvh_bytes), scratch(build_bytes);
        check(pdr_bvh_build(d_pos.get(), Vu, d_idx.get(), T, bvh.get(), bvh_bytes, scratch.get(), build_bytes, s));
        ray_bits = DeviceArray<std::uint32_t>(N * ((views.size() + 31) / 32));
        check(pdr_ray_visibility_views(bvh.get(), T, d_apos.get(), d_anrm.get(), d_araster.get(),
                                       static_cast<std::uint32_t>(N),
                                       reinterpret_cast<const pdr_projection_view*>(d_table.get()),
                                       static_cast<std::uint32_t>(views.size()), options.ray_origin_bias,
                                       ray_bits.get(), s));
        check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    }
    DeviceArray<float> d_color(N * 4), d_conf(N), d_valid(N), d_cov(N);
    DeviceArray<std::uint32_t> d_src(N), d_faces(N);
    if (vis_mode == 0)
        check(pdr_project_views(d_apos.get(), d_anrm.get(), d_araster.get(), static_cast<std::uint32_t>(N),
                                reinterpret_cast<const pdr_projection_view*>(d_table.get()),
                                static_cast<std::uint32_t>(views.size()), static_cast<std::uint32_t>(options.blend_mode),
                                options.pcf_radius, 0, d_color.get(), d_conf.get(), d_src.get(), d_valid.get(),
                                d_cov.get(), d_faces.get(), s));
    else
        check(pdr_project_views_bits(d_apos.get(), d_anrm.get(), d_araster.get(), static_cast<std::uint32_t>(N),
                                     reinterpret_cast<const pdr_projection_view*>(d_table.get()),
                                     static_cast<std::uint32_t>(views.size()),
                                     static_cast<std::uint32_t>(options.blend_mode), options.pcf_radius, vis_mode,
                                     ray_bits.get(), d_color.get(), d_conf.get(), d_src.get(), d_valid.get(),
                                     d_cov.get(), d_faces.get(), s));
    TextureBakeOutput out;
    out.width = AW;
    out.height = AH;
    out.color = d_color.download(s);
    out.confidence = d_conf.download(s);
    out.source_view = d_src.download(s);
    out.valid_mask = d_valid.download(s);
    out.coverage_mask = d_cov.download(s);
    out.face_ids = d_faces.download(s);
    out.used_ray_query = vis_mode != 0;
    return out;
}

// ---- TextureRefiner (src/texture_refiner.cpp:174-454) -------------------------------------------

class TextureRefiner::Impl {
public:
    explicit Impl(Context::Impl& c) : ctx(c) {}
    Context::Impl& ctx;
};

TextureRefiner::TextureRefiner(Context& context) : impl_(std::make_unique<Impl>(*context.impl_)) {}
TextureRefiner::~TextureRefiner() = default;
TextureRefiner::TextureRefiner(TextureRefiner&&) noexcept = default;
TextureRefiner& TextureRefiner::operator=(TextureRefiner&&) noexcept = default;

TextureRefineOutput TextureRefiner::refine(std::span<const float> initial_texture, std::span<const float> positions,
                                           std::span<const float> uv, std::span<const std::uint32_t> triangle_indices,
                                           std::span<const ProjectionView> views, std::span<const float> seam_uv_pairs,
                                           const TextureRefineOptions& o) {
    const std::size_t V = positions.size() / 3;
    if (positions.empty() || positions.size() % 3 != 0 || uv.size() != V * 2 || triangle_indices.empty() ||
        triangle_indices.size() % 3 != 0 ||
        std::any_of(triangle_indices.begin(), triangle_indices.end(), [V](std::uint32_t i) { return i >= V; }))
        throw std::invalid_argument("texture refinement mesh arrays have inconsistent shapes");
    const std::size_t n = static_cast<std::size_t>(o.width) * o.height * 3;
    if (o.width == 0 || o.height == 0 || initial_texture.size() != n || views.empty() || o.steps == 0 ||
        o.batch_size == 0 || !std::isfinite(o.learning_rate) || o.learning_rate <= 0.0F ||
        !std::isfinite(o.minimum_learning_rate) || o.minimum_learning_rate < 0.0F ||
        o.minimum_learning_rate > o.learning_rate || !std::isfinite(o.photometric_epsilon) ||
        o.photometric_epsilon <= 0.0F || !(o.adam_beta1 > 0.0F && o.adam_beta1 < 1.0F) ||
        !(o.adam_beta2 > 0.0F && o.adam_beta2 < 1.0F) || !(o.clamp_min < o.clamp_max) || seam_uv_pairs.size() % 4 != 0 ||
        !std::isfinite(o.seam_learning_rate) || o.seam_learning_rate <= 0.0F || !std::isfinite(o.seam_epsilon) ||
        o.seam_epsilon <= 0.0F)
        throw std::invalid_argument("texture refinement options are invalid");
    if (n > std::numeric_limits<std::uint32_t>::max())
        throw std::overflow_error("texture refinement atlas exceeds the shader element limit");
    Context::Impl& ctx = impl_->ctx;
    std::lock_guard<std::mutex> lock(ctx.mutex);
    ctx.activate();
    cudaStream_t s = ctx.stream;
    const auto t0 = std::chrono::steady_clock::now();
    const auto Vu = static_cast<std::uint32_t>(V);
    const auto T = static_cast<std::uint32_t>(triangle_indices.size() / 3);
    auto d_pos = upload(positions, s);
    auto d_uv = upload(uv, s);
    auto d_idx = upload(triangle_indices, s);
    DeviceArray<float> d_clip(V * 4);
    std::vector<DeviceArray<float>> keep;
    std::vector<pdr_refine_view> table(views.size());
    std::vector<double> weights(views.size());
    std::uint64_t max_pixels = 0;
    for (std::size_t k = 0; k < views.size(); ++k) {
        const auto& v = views[k];
        if (v.width == 0 || v.height == 0 || (v.channel_count != 3 && v.channel_count != 4))
            throw std::invalid_argument("texture refinement images must contain RGB or RGBA data");
        const std::size_t P = static_cast<std::size_t>(v.width) * v.height;
        if (v.image.size() != P * v.channel_count || (!v.visibility_mask.empty() && v.visibility_mask.size() != P) ||
            P > std::numeric_limits<std::uint32_t>::max())
            throw std::invalid_argument("texture refinement image or mask has an invalid shape");
        DeviceArray<float> d_m(v.world_to_clip.data(), 16, s);
        check(pdr_transform_positions(d_pos.get(), Vu, d_m.get(), 1, d_clip.get(), s));
        const Viewport vp = resolve_viewport(v.width, v.height, v.viewport);
        const float vp4[4] = {vp.x, vp.y, vp.width, vp.height};
        DeviceArray<float> d_vvp(vp4, 4, s);
        DeviceArray<float> raster(P * 4);
        rasterize_device(ctx, d_clip.get(), 1, Vu, d_idx.get(), T, v.width, v.height, d_vvp.get(), 0, raster.get(), nullptr);
        DeviceArray<float> uvk(P * 2), target(P * 3), mask(P);
        check(pdr_interpolate_forward(d_uv.get(), 0, Vu, 2, d_idx.get(), T, raster.get(), 1, P, uvk.get(), s));
        auto image = upload(std::span<const float>(v.image), s);
        auto ext = upload(std::span<const float>(v.visibility_mask), s);
        check(pdr_refine_prepare_view(image.get(), v.channel_count, v.visibility_mask.empty() ? nullptr : ext.get(),
                                      raster.get(), P, target.get(), mask.get(), s));
        const auto host_mask = mask.download(s);
        double vw = 0.0;
        for (float m : host_mask) vw += m;  // texture_refiner.cpp:240 sums in double, in pixel order
        weights[k] = vw;
        table[k] = pdr_refine_view{uvk.get(), target.get(), mask.get(), P};
        max_pixels = std::max<std::uint64_t>(max_pixels, P);
        keep.push_back(std::move(uvk));
        keep.push_back(std::move(target));
        keep.push_back(std::move(mask));
    }
    DeviceArray<unsigned char> d_table(reinterpret_cast<const unsigned char*>(table.data()),
                                       table.size() * sizeof(pdr_refine_view), s);
    check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    const auto t1 = std::chrono::steady_clock::now();
    auto d_tex = upload(initial_texture, s);
    DeviceArray<float> g(n / 3 * 4), m1(n), m2(n);  // the gradient is [texels][4]
    const std::uint32_t pairs = static_cast<std::uint32_t>(seam_uv_pairs.size() / 4);
    auto d_pairs = upload(seam_uv_pairs, s);
    const std::uint32_t seam_steps = pairs == 0 ? 0u : o.seam_polish_steps;
    DeviceArray<float> loss(o.steps + seam_steps);
    pdr_refine_options ro{o.width, o.height, o.steps, o.batch_size, o.learning_rate, o.minimum_learning_rate,
                          o.photometric_epsilon, o.adam_beta1, o.adam_beta2, o.adam_epsilon, o.clamp_min, o.clamp_max,
                          o.seam_polish_steps, o.seam_learning_rate, o.seam_epsilon, 0.0F, 1e-4F};
    check(pdr_refine_run(&ro, reinterpret_cast<const pdr_refine_view*>(d_table.get()),
                         static_cast<std::uint32_t>(views.size()), weights.data(), max_pixels, d_pairs.get(), pairs,
                         nullptr, nullptr, d_tex.get(), g.get(), m1.get(), m2.get(), loss.get(), 1, s));
    check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    const auto t2 = std::chrono::steady_clock::now();
    TextureRefineOutput out;
    out.width = o.width;
    out.height = o.height;
    out.color = d_tex.download(s);
    const auto hist = loss.download(s);
    out.loss_history.assign(hist.begin(), hist.begin() + o.steps);
    out.seam_loss_history.assign(hist.begin() + o.steps, hist.end());
    out.precompute_seconds = std::chrono::duration<double>(t1 - t0).count();
    out.optimization_seconds = std::chrono::duration<double>(t2 - t1).count();
    return out;
}

}  // namespace photara_drender

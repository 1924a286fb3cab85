// Host driver that runs the reference's own HLSL compute shaders on the CPU, one invocation
// at a time, after oracle/build.py has stripped the two HLSL-only annotations
// ("[numthreads(...)]" and ": SV_*" semantics) into oracle/_ref/gen/*.inc.
// TEST INFRASTRUCTURE ONLY: it exists to check oracle/pdr_oracle.c against the reference's code.
#include "ref_shim.hpp"

#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace hlsl {
thread_local GroupScheduler* tls_group = nullptr;
thread_local uint tls_lane = 0;
}

#define groupshared static
#define main shader_main

namespace sh_rasterize_forward { using namespace hlsl;
#include "rasterize_forward.hlsl.inc"
}
namespace sh_rasterize_backward { using namespace hlsl;
#include "rasterize_backward.hlsl.inc"
}
namespace sh_reduce_vertex_gradients { using namespace hlsl;
#include "reduce_vertex_gradients.hlsl.inc"
}
namespace sh_interpolate_forward { using namespace hlsl;
#include "interpolate_forward.hlsl.inc"
}
namespace sh_interpolate_grad_attributes { using namespace hlsl;
#include "interpolate_grad_attributes.hlsl.inc"
}
namespace sh_interpolate_grad_raster { using namespace hlsl;
#include "interpolate_grad_raster.hlsl.inc"
}
namespace sh_texture_forward { using namespace hlsl;
#include "texture_forward.hlsl.inc"
}
namespace sh_texture_grad_texture { using namespace hlsl;
#include "texture_grad_texture.hlsl.inc"
}
namespace sh_texture_grad_uv { using namespace hlsl;
#include "texture_grad_uv.hlsl.inc"
}
namespace sh_project_texture { using namespace hlsl;
#include "project_texture.hlsl.inc"
}
namespace sh_atlas_photometric_gradient { using namespace hlsl;
#include "atlas_photometric_gradient.hlsl.inc"
}
#define out
namespace sh_atlas_seam_gradient { using namespace hlsl;
#include "atlas_seam_gradient.hlsl.inc"
}
#undef out
namespace sh_atlas_adam_update { using namespace hlsl;
#include "atlas_adam_update.hlsl.inc"
}
#undef main
#undef groupshared

using hlsl::uint;
using hlsl::uint3;

namespace {

template <class F>
void dispatch_1d(uint count, F&& f) {
    const uint groups = (count + 63) / 64;
    for (uint g = 0; g < groups; ++g)
        for (uint l = 0; l < 64; ++l) f(uint3(g * 64 + l, 0, 0));
}

// Runs each 64-invocation group with lane-ordered barriers.
template <class F>
void dispatch_groups(uint count, F&& f) {
    const uint groups = (count + 63) / 64;
    for (uint g = 0; g < groups; ++g) {
        hlsl::GroupScheduler sched;
        sched.lanes = 64;
        sched.turn = 0;
        std::vector<std::thread> threads;
        threads.reserve(64);
        for (uint l = 0; l < 64; ++l) {
            threads.emplace_back([&, l] {
                hlsl::tls_group = &sched;
                hlsl::tls_lane = l;
                sched.wait_turn(l);
                f(uint3(g * 64 + l, 0, 0), l);
                sched.pass(l);
            });
        }
        for (auto& t : threads) t.join();
    }
}

} // namespace

extern "C" {

void ref_rasterize_forward(const float* pos, uint V, const uint* idx, uint T, uint W, uint H, uint cull,
                           uint out_deriv, const float* vp, uint tile_count_x, const uint* tile_offsets,
                           const uint* tile_list, float* raster, float* deriv) {
    namespace S = sh_rasterize_forward;
    S::positions.data = reinterpret_cast<const hlsl::float4*>(pos);
    S::indices.data = idx;
    S::tile_offsets.data = tile_offsets;
    S::tile_triangle_indices.data = tile_list;
    S::raster.data = raster;
    S::barycentric_derivatives.data = deriv;
    S::push_constants.vertex_count = V;
    S::push_constants.triangle_count = T;
    S::push_constants.width = W;
    S::push_constants.height = H;
    S::push_constants.cull_mode = cull;
    S::push_constants.output_derivatives = out_deriv;
    S::push_constants.tile_count_x = tile_count_x;
    S::push_constants.tile_size = 16;
    S::push_constants.viewport = hlsl::float4(vp[0], vp[1], vp[2], vp[3]);
    const uint gx = (W + 7) / 8, gy = (H + 7) / 8;
    for (uint y = 0; y < gy * 8; ++y)
        for (uint x = 0; x < gx * 8; ++x) S::shader_main(uint3(x, y, 0));
}

void ref_rasterize_backward(const float* pos, uint V, const uint* idx, uint T, uint W, uint H, const float* vp,
                            const float* raster, const float* grad_raster, float* corner_grads) {
    namespace S = sh_rasterize_backward;
    static float dummy = 0.0f;
    S::positions.data = reinterpret_cast<const hlsl::float4*>(pos);
    S::indices.data = idx;
    S::raster.data = raster;
    S::grad_raster.data = grad_raster;
    S::grad_barycentric_derivatives.data = &dummy;
    S::corner_gradients.data = reinterpret_cast<hlsl::float4*>(corner_grads);
    S::push_constants.vertex_count = V;
    S::push_constants.triangle_count = T;
    S::push_constants.width = W;
    S::push_constants.height = H;
    S::push_constants.viewport = hlsl::float4(vp[0], vp[1], vp[2], vp[3]);
    dispatch_1d(T, [](uint3 id) { S::shader_main(id); });
}

void ref_reduce_vertex_gradients(const uint* offsets, const uint* corners, const float* corner_grads, uint V,
                                 float* vertex_grads) {
    namespace S = sh_reduce_vertex_gradients;
    S::vertex_offsets.data = offsets;
    S::vertex_corners.data = corners;
    S::corner_gradients.data = reinterpret_cast<const hlsl::float4*>(corner_grads);
    S::vertex_gradients.data = reinterpret_cast<hlsl::float4*>(vertex_grads);
    S::push_constants.vertex_count = V;
    dispatch_1d(V, [](uint3 id) { S::shader_main(id); });
}

void ref_interpolate_forward(const float* attr, uint V, uint A, const uint* idx, uint T, const float* raster,
                             uint P, float* out_values) {
    namespace S = sh_interpolate_forward;
    S::vertex_attributes.data = attr;
    S::indices.data = idx;
    S::raster.data = raster;
    S::interpolated.data = out_values;
    S::push_constants.vertex_count = V;
    S::push_constants.triangle_count = T;
    S::push_constants.pixel_count = P;
    S::push_constants.attribute_count = A;
    dispatch_1d(P * A, [](uint3 id) { S::shader_main(id); });
}

void ref_interpolate_grad_attributes(const uint* idx, uint V, uint A, uint T, const float* raster, uint P,
                                     const float* grad, float* grad_attr) {
    namespace S = sh_interpolate_grad_attributes;
    S::indices.data = idx;
    S::raster.data = raster;
    S::grad_interpolated.data = grad;
    S::grad_attributes.data = grad_attr;
    S::push_constants.vertex_count = V;
    S::push_constants.triangle_count = T;
    S::push_constants.pixel_count = P;
    S::push_constants.attribute_count = A;
    dispatch_1d(V * A, [](uint3 id) { S::shader_main(id); });
}

void ref_interpolate_grad_raster(const float* attr, uint V, uint A, const uint* idx, uint T, const float* raster,
                                 uint P, const float* grad, float* grad_raster) {
    namespace S = sh_interpolate_grad_raster;
    S::vertex_attributes.data = attr;
    S::indices.data = idx;
    S::raster.data = raster;
    S::grad_interpolated.data = grad;
    S::grad_raster.data = grad_raster;
    S::push_constants.vertex_count = V;
    S::push_constants.triangle_count = T;
    S::push_constants.pixel_count = P;
    S::push_constants.attribute_count = A;
    dispatch_1d(P, [](uint3 id) { S::shader_main(id); });
}

void ref_texture_forward(const float* tex, uint tw, uint th, uint C, uint mode, const float* uv,
                         const float* raster, uint P, float* sampled) {
    namespace S = sh_texture_forward;
    S::texture_values.data = tex;
    S::uv_values.data = uv;
    S::raster.data = raster;
    S::sampled_values.data = sampled;
    S::push_constants.pixel_count = P;
    S::push_constants.texture_width = tw;
    S::push_constants.texture_height = th;
    S::push_constants.channel_count = C;
    S::push_constants.address_mode = mode;
    dispatch_1d(P * C, [](uint3 id) { S::shader_main(id); });
}

void ref_texture_grad_texture(const float* grad, const uint* texel_offsets, const uint* entries,
                              const float* weights, uint texels, uint P, uint C, float* grad_tex) {
    namespace S = sh_texture_grad_texture;
    S::grad_sampled.data = grad;
    S::texel_offsets.data = texel_offsets;
    S::sample_entries.data = entries;
    S::sample_weights.data = weights;
    S::grad_texture.data = grad_tex;
    S::push_constants.texel_count = texels;
    S::push_constants.pixel_count = P;
    S::push_constants.channel_count = C;
    dispatch_1d(texels * C, [](uint3 id) { S::shader_main(id); });
}

void ref_texture_grad_uv(const float* tex, uint tw, uint th, uint C, uint mode, const float* uv,
                         const float* raster, uint P, const float* grad, float* grad_uv) {
    namespace S = sh_texture_grad_uv;
    S::texture_values.data = tex;
    S::uv_values.data = uv;
    S::raster.data = raster;
    S::grad_sampled.data = grad;
    S::grad_uv.data = reinterpret_cast<hlsl::float2*>(grad_uv);
    S::push_constants.pixel_count = P;
    S::push_constants.texture_width = tw;
    S::push_constants.texture_height = th;
    S::push_constants.channel_count = C;
    S::push_constants.address_mode = mode;
    dispatch_1d(P, [](uint3 id) { S::shader_main(id); });
}

// settings packing follows texture_baker.cpp:312-322.
void ref_project_texture(const float* m16, const float* cam_weight4, const float* vp4, const uint* dims4,
                         float depth_bias, float min_cos, uint packed, uint view_index,
                         const float* apos, const float* anrm, const float* araster, const float* shadow,
                         const float* photo, const float* mask, const float* rayvis, float* acc_color,
                         float* acc_weight, float* best_conf, uint* source_view) {
    namespace S = sh_project_texture;
    S::atlas_positions.data = apos;
    S::atlas_normals.data = anrm;
    S::atlas_raster.data = araster;
    S::shadow_raster.data = shadow;
    S::photo.data = photo;
    S::photo_mask.data = mask;
    S::ray_visibility.data = rayvis;
    S::accumulated_color.data = acc_color;
    S::accumulated_weight.data = acc_weight;
    S::best_confidence.data = best_conf;
    S::source_view.data = source_view;
    S::push_constants.matrix_row_0 = hlsl::float4(m16[0], m16[1], m16[2], m16[3]);
    S::push_constants.matrix_row_1 = hlsl::float4(m16[4], m16[5], m16[6], m16[7]);
    S::push_constants.matrix_row_2 = hlsl::float4(m16[8], m16[9], m16[10], m16[11]);
    S::push_constants.matrix_row_3 = hlsl::float4(m16[12], m16[13], m16[14], m16[15]);
    S::push_constants.camera_position_weight = hlsl::float4(cam_weight4[0], cam_weight4[1], cam_weight4[2], cam_weight4[3]);
    S::push_constants.viewport = hlsl::float4(vp4[0], vp4[1], vp4[2], vp4[3]);
    S::push_constants.dimensions = hlsl::uint4{dims4[0], dims4[1], dims4[2], dims4[3]};
    S::push_constants.settings = hlsl::float4(depth_bias, min_cos, hlsl::asfloat(packed), hlsl::asfloat(view_index));
    dispatch_1d(dims4[0] * dims4[1], [](uint3 id) { S::shader_main(id); });
}

void ref_atlas_photometric_gradient(const float* tex, const float* uv, const float* target, const float* mask,
                                    uint P, uint tw, uint th, uint loss_index, float eps, float norm,
                                    float* grad, float* loss_history) {
    namespace S = sh_atlas_photometric_gradient;
    S::texture_values.data = tex;
    S::uv_values.data = uv;
    S::target_rgb.data = target;
    S::valid_mask.data = mask;
    S::texture_gradient.data = reinterpret_cast<uint*>(grad);
    S::loss_history.data = reinterpret_cast<uint*>(loss_history);
    S::push_constants.pixel_count = P;
    S::push_constants.texture_width = tw;
    S::push_constants.texture_height = th;
    S::push_constants.loss_index = loss_index;
    S::push_constants.photometric_epsilon = eps;
    S::push_constants.normalization = norm;
    dispatch_groups(P, [](uint3 id, uint lane) { S::shader_main(id, lane); });
}

void ref_atlas_seam_gradient(const float* tex, const float* pairs, uint npairs, uint tw, uint th, uint loss_index,
                             float eps, float norm, float* grad, float* loss_history) {
    namespace S = sh_atlas_seam_gradient;
    S::texture_values.data = tex;
    S::seam_uv_pairs.data = pairs;
    S::texture_gradient.data = reinterpret_cast<uint*>(grad);
    S::loss_history.data = reinterpret_cast<uint*>(loss_history);
    S::push_constants.pair_count = npairs;
    S::push_constants.texture_width = tw;
    S::push_constants.texture_height = th;
    S::push_constants.loss_index = loss_index;
    S::push_constants.seam_epsilon = eps;
    S::push_constants.normalization = norm;
    dispatch_groups(npairs, [](uint3 id, uint lane) { S::shader_main(id, lane); });
}

void ref_atlas_adam_update(float* tex, float* grad, float* m, float* v, uint n, float lr, float b1, float b2,
                           float eps, float bc1, float bc2, float cmin, float cmax) {
    namespace S = sh_atlas_adam_update;
    S::texture_values.data = tex;
    S::texture_gradient.data = grad;
    S::first_moment.data = m;
    S::second_moment.data = v;
    S::push_constants.value_count = n;
    S::push_constants.learning_rate = lr;
    S::push_constants.beta1 = b1;
    S::push_constants.beta2 = b2;
    S::push_constants.adam_epsilon = eps;
    S::push_constants.bias_correction1 = bc1;
    S::push_constants.bias_correction2 = bc2;
    S::push_constants.clamp_min = cmin;
    S::push_constants.clamp_max = cmax;
    dispatch_1d(n, [](uint3 id) { S::shader_main(id); });
}

} // extern "C"

// Exercises the C++ API (include/photara_drender/*.hpp, libphotara_drender.so) on a GPU.
//
// Part 1 checks the properties the reference's tests/native_tests.cpp checks through the same API:
// output sizes, coverage, finite-difference agreement of the raster, uv and texture gradients,
// viewport clipping, the single-triangle bake (colour, face ids), the near view winning a softmax
// bake, a refinement whose loss falls, and the padding / surface-fill regressions of
// tests/native_tests.cpp and tests/texture_surface_fill_test.cpp. It also checks the exception types of invalid calls.
//
// Part 2 (when given an input directory) reads a mesh and gradients written by the pytest driver,
// runs forward, backward, interpolate and texture through the C++ API and writes the raw outputs
// back, so the driver can compare them with the oracle.
//
// Usage: cpp_api_test [in_dir out_dir]; exit status 0 when every check passed.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "photara_drender/photara_drender.hpp"

namespace pd = photara_drender;

namespace {

int g_checks = 0;

void expect(bool ok, const std::string& what) {
    ++g_checks;
    if (!ok) throw std::runtime_error("check failed: " + what);
}

template <class E, class F>
void expect_throws(F&& f, const std::string& what) {
    ++g_checks;
    try {
        f();
    } catch (const E&) {
        return;
    } catch (const std::exception& e) {
        throw std::runtime_error("wrong exception for " + what + ": " + e.what());
    }
    throw std::runtime_error("no exception for " + what);
}

double channel_sum(const std::vector<float>& v, std::size_t stride, std::size_t channel) {
    double s = 0.0;
    for (std::size_t i = channel; i < v.size(); i += stride) s += v[i];
    return s;
}

const std::vector<float> kTriClip{-0.75F, -0.75F, 0.0F, 1.0F, 0.75F, -0.75F, 0.0F, 1.0F, 0.0F, 0.75F, 0.0F, 1.0F};
const std::vector<std::uint32_t> kTri{0, 1, 2};

void raster_checks(pd::Rasterizer& r) {
    pd::RasterizeOptions opt;
    opt.width = 32;
    opt.height = 32;
    const auto out = r.forward(kTriClip, kTri, opt);
    expect(out.raster.size() == 32 * 32 * 4, "raster size");
    expect(out.barycentric_derivatives.size() == out.raster.size(), "derivative size");
    std::size_t covered = 0;
    for (std::size_t p = 0; p < 32 * 32; ++p) {
        const float id = out.raster[p * 4 + 3];
        if (id != 0.0F) {
            ++covered;
            expect(id == 1.0F, "triangle id of a covered pixel");
            const float u = out.raster[p * 4], v = out.raster[p * 4 + 1];
            expect(u >= -1e-6F && v >= -1e-6F && u + v <= 1.0F + 1e-5F, "barycentrics inside the triangle");
        }
    }
    // The triangle covers 1.5 x 1.5 / 2 of the 2 x 2 clip square: 0.28 of 1024 pixels.
    expect(covered > 250 && covered < 330, "coverage of the test triangle");

    // loss = sum of u over the image; d loss / d x0 against a central difference
    std::vector<float> g(out.raster.size(), 0.0F);
    for (std::size_t p = 0; p < 32 * 32; ++p) g[p * 4] = out.raster[p * 4 + 3] > 0.0F ? 1.0F : 0.0F;
    const auto gp = r.backward(kTriClip, kTri, out, g);
    expect(gp.size() == kTriClip.size(), "position gradient size");
    expect(std::all_of(gp.begin(), gp.end(), [](float x) { return std::isfinite(x); }), "finite position gradient");
    const float h = 1e-3F;
    auto plus = kTriClip, minus = kTriClip;
    plus[0] += h;
    minus[0] -= h;
    const double fd = (channel_sum(r.forward(plus, kTri, opt).raster, 4, 0) -
                       channel_sum(r.forward(minus, kTri, opt).raster, 4, 0)) / (2.0 * h);
    expect(std::abs(gp[0] - fd) < 0.2, "raster gradient vs finite difference");

    // interpolating the identity attributes returns (u, v, 1 - u - v)
    const std::vector<float> eye{1, 0, 0, 0, 1, 0, 0, 0, 1};
    const auto it = r.interpolate_forward(eye, 3, kTri, out);
    expect(it.values.size() == 32 * 32 * 3, "interpolation size");
    for (std::size_t p = 0; p < 32 * 32; ++p) {
        if (out.raster[p * 4 + 3] == 0.0F) continue;
        const float u = out.raster[p * 4], v = out.raster[p * 4 + 1];
        expect(std::abs(it.values[p * 3] - u) < 1e-6F && std::abs(it.values[p * 3 + 1] - v) < 1e-6F &&
                   std::abs(it.values[p * 3 + 2] - (1.0F - u - v)) < 1e-5F,
               "identity interpolation");
    }
    const std::vector<float> ones(it.values.size(), 1.0F);
    const auto ig = r.interpolate_backward(eye, 3, kTri, out, ones);
    expect(ig.attributes.size() == eye.size() && ig.raster.size() == out.raster.size(), "interpolation gradient sizes");
    // with unit upstream gradients each vertex attribute collects the sum of its barycentric weight
    double wsum = 0.0;
    for (int c = 0; c < 3; ++c) wsum += ig.attributes[c * 3 + c];
    expect(std::abs(wsum - static_cast<double>(covered)) < 1e-2 * covered, "attribute gradient mass");

    // texture: gradients against central differences at one covered pixel
    const std::vector<float> vuv{0.2F, 0.2F, 0.8F, 0.2F, 0.5F, 0.8F};
    const auto uv = r.interpolate_forward(vuv, 2, kTri, out).values;
    std::vector<float> tex(5 * 4 * 2);
    for (std::uint32_t y = 0; y < 4; ++y)
        for (std::uint32_t x = 0; x < 5; ++x) {
            tex[(y * 5 + x) * 2] = 0.5F * static_cast<float>(x) + 0.25F * static_cast<float>(y * y);
            tex[(y * 5 + x) * 2 + 1] = static_cast<float>(static_cast<int>(2 * x) - static_cast<int>(3 * y));
        }
    const pd::TextureDesc td{5, 4, 2, pd::AddressMode::clamp};
    const auto s = r.texture_forward(tex, td, uv, out);
    expect(s.values.size() == 32 * 32 * 2, "texture sample size");
    std::size_t px = 0;
    while (px < 32 * 32 && out.raster[px * 4 + 3] == 0.0F) ++px;
    expect(px < 32 * 32, "a covered pixel exists");
    std::vector<float> gs(s.values.size(), 0.0F);
    gs[px * 2] = 1.0F;
    const auto tg = r.texture_backward(tex, td, uv, out, gs);
    expect(tg.texture.size() == tex.size() && tg.uv.size() == uv.size(), "texture gradient sizes");
    auto up = uv, um = uv;
    up[px * 2] += h;
    um[px * 2] -= h;
    const double fdu = (r.texture_forward(tex, td, up, out).values[px * 2] -
                        r.texture_forward(tex, td, um, out).values[px * 2]) / (2.0 * h);
    expect(std::abs(tg.uv[px * 2] - fdu) < 1e-2 * std::max(1.0, std::abs(fdu)), "uv gradient vs finite difference");
    std::size_t texel = 0;
    while (texel < tg.texture.size() && std::abs(tg.texture[texel]) < 1e-8F) ++texel;
    expect(texel < tg.texture.size(), "a texel received gradient");
    auto tp = tex, tm = tex;
    tp[texel] += h;
    tm[texel] -= h;
    const double fdt = (r.texture_forward(tp, td, uv, out).values[px * 2] -
                        r.texture_forward(tm, td, uv, out).values[px * 2]) / (2.0 * h);
    expect(std::abs(tg.texture[texel] - fdt) < 1e-3, "texture gradient vs finite difference");

    // a viewport confines coverage to its rectangle
    auto vopt = opt;
    vopt.viewport = pd::Viewport{8.0F, 4.0F, 16.0F, 20.0F};
    const auto vo = r.forward(kTriClip, kTri, vopt);
    for (std::uint32_t y = 0; y < 32; ++y)
        for (std::uint32_t x = 0; x < 32; ++x)
            if (x < 8 || x >= 24 || y < 4 || y >= 24)
                expect(vo.raster[(y * 32 + x) * 4 + 3] == 0.0F, "no coverage outside the viewport");
    const auto vg = r.backward(kTriClip, kTri, vo, g);
    expect(std::all_of(vg.begin(), vg.end(), [](float x) { return std::isfinite(x); }), "finite viewport gradient");

    // invalid calls throw the reference's exception types
    const std::vector<std::uint32_t> bad{0, 1, 3};
    expect_throws<std::out_of_range>([&] { (void)r.forward(kTriClip, bad, opt); }, "an out-of-range index");
    auto zero = opt;
    zero.width = 0;
    expect_throws<std::invalid_argument>([&] { (void)r.forward(kTriClip, kTri, zero); }, "a zero width");
    auto badvp = opt;
    badvp.viewport = pd::Viewport{0.0F, 0.0F, -1.0F, 4.0F};
    expect_throws<std::invalid_argument>([&] { (void)r.forward(kTriClip, kTri, badvp); }, "a negative viewport");
    const std::vector<float> three(3, 0.0F);
    expect_throws<std::invalid_argument>([&] { (void)r.forward(three, kTri, opt); }, "a ragged position array");
    std::vector<float> nan_uv = uv;
    nan_uv[px * 2] = std::nanf("");
    expect_throws<std::invalid_argument>([&] { (void)r.texture_backward(tex, td, nan_uv, out, gs); },
                                         "a non-finite uv on a covered pixel");
}

pd::ProjectionView flat_view(float r, float g, float b, float cam_z) {
    pd::ProjectionView v;
    v.width = 16;
    v.height = 16;
    v.channel_count = 4;
    v.image.resize(16 * 16 * 4);
    for (std::size_t p = 0; p < 16 * 16; ++p) {
        v.image[p * 4] = r;
        v.image[p * 4 + 1] = g;
        v.image[p * 4 + 2] = b;
        v.image[p * 4 + 3] = 1.0F;
    }
    v.world_to_clip = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    v.camera_position = {0.0F, 0.0F, cam_z};
    return v;
}

void bake_checks(pd::Context& ctx) {
    const std::vector<float> pos{-0.75F, -0.75F, 0.0F, 0.75F, -0.75F, 0.0F, 0.0F, 0.75F, 0.0F};
    const std::vector<float> nrm{0, 0, 1, 0, 0, 1, 0, 0, 1};
    const std::vector<float> buv{0.125F, 0.125F, 0.875F, 0.125F, 0.5F, 0.875F};
    pd::TextureBaker baker(ctx);
    pd::TextureBakeOptions o;
    o.width = 16;
    o.height = 16;
    o.blend_mode = pd::ProjectionBlendMode::weighted_average;
    const auto near = flat_view(0.8F, 0.2F, 0.1F, 2.0F);
    const auto b = baker.bake(pos, nrm, buv, kTri, std::span<const pd::ProjectionView>(&near, 1), o);
    expect(b.color.size() == 16 * 16 * 4 && b.face_ids.size() == 16 * 16 && b.coverage_mask.size() == 16 * 16,
           "bake output sizes");
    for (std::size_t t = 0; t < 16 * 16; ++t)
        expect(b.face_ids[t] == (b.coverage_mask[t] > 0.5F ? 0u : 0xFFFFFFFFu), "face ids follow coverage");
    const auto it = std::find_if(b.valid_mask.begin(), b.valid_mask.end(), [](float x) { return x > 0.5F; });
    expect(it != b.valid_mask.end(), "some texels are valid");
    const auto t = static_cast<std::size_t>(it - b.valid_mask.begin());
    expect(std::abs(b.color[t * 4] - 0.8F) < 1e-4F, "baked colour of a valid texel");
    expect(b.used_ray_query == ctx.device_info().supports_ray_query, "ray queries in the default visibility mode");

    // softmax: the near view dominates where weighted averaging mixes the two
    const auto far = flat_view(0.1F, 0.2F, 0.8F, 6.0F);
    const std::array<pd::ProjectionView, 2> two{near, far};
    const auto avg = baker.bake(pos, nrm, buv, kTri, two, o);
    auto so = o;
    so.blend_mode = pd::ProjectionBlendMode::softmax;
    const auto soft = baker.bake(pos, nrm, buv, kTri, two, so);
    const auto sv = std::find_if(soft.valid_mask.begin(), soft.valid_mask.end(), [](float x) { return x > 0.5F; });
    expect(sv != soft.valid_mask.end(), "softmax bake has valid texels");
    const auto k = static_cast<std::size_t>(sv - soft.valid_mask.begin());
    expect(soft.coverage_mask[k] > 0.5F, "valid texels are covered");
    expect(soft.color[k * 4] > avg.color[k * 4] + 0.05F, "softmax favours the near view");
    expect(std::abs(soft.color[k * 4] - 0.8F) < 0.05F, "softmax colour is close to the near view");

    // a zero visibility mask rejects everything unless a mask floor keeps weak samples
    auto masked = near;
    masked.visibility_mask.assign(16 * 16, 0.0F);
    const auto mspan = std::span<const pd::ProjectionView>(&masked, 1);
    const auto strict = baker.bake(pos, nrm, buv, kTri, mspan, so);
    expect(std::none_of(strict.valid_mask.begin(), strict.valid_mask.end(), [](float x) { return x > 0.0F; }),
           "a strict zero mask rejects every texel");
    auto fo = so;
    fo.mask_floor = 0.1F;
    const auto floored = baker.bake(pos, nrm, buv, kTri, mspan, fo);
    const auto fv = std::find_if(floored.valid_mask.begin(), floored.valid_mask.end(), [](float x) { return x > 0.5F; });
    expect(fv != floored.valid_mask.end(), "a mask floor keeps masked texels");
    expect(std::abs(floored.color[static_cast<std::size_t>(fv - floored.valid_mask.begin()) * 4] - 0.8F) < 1e-3F,
           "mask-floor texels carry the image colour");

    std::vector<pd::ProjectionView> none;
    expect_throws<std::invalid_argument>([&] { (void)baker.bake(pos, nrm, buv, kTri, none, o); }, "a bake without views");
    auto big = o;
    big.pcf_radius = 5;
    expect_throws<std::invalid_argument>([&] { (void)baker.bake(pos, nrm, buv, kTri, two, big); }, "pcf radius 5");
}

void refine_checks(pd::Context& ctx) {
    const std::vector<float> pos{-0.75F, -0.75F, 0.0F, 0.75F, -0.75F, 0.0F, 0.0F, 0.75F, 0.0F};
    const std::vector<float> ruv{0.125F, 0.125F, 0.875F, 0.125F, 0.5F, 0.875F};
    const auto view = flat_view(0.9F, 0.4F, 0.1F, 2.0F);
    pd::TextureRefineOptions o;
    o.width = 16;
    o.height = 16;
    o.steps = 40;
    o.batch_size = 1;
    o.learning_rate = 5e-2F;
    o.minimum_learning_rate = 5e-3F;
    std::vector<float> init(16 * 16 * 3, 0.5F);
    pd::TextureRefiner refiner(ctx);
    const auto out = refiner.refine(init, pos, ruv, kTri, std::span<const pd::ProjectionView>(&view, 1), {}, o);
    expect(out.color.size() == init.size() && out.loss_history.size() == 40 && out.seam_loss_history.empty(),
           "refine output sizes");
    expect(out.loss_history.back() < 0.5F * out.loss_history.front(), "refinement lowers the photometric loss");
    expect(std::all_of(out.color.begin(), out.color.end(), [](float x) { return x >= 0.0F && x <= 1.0F; }),
           "refined colours stay in the clamp range");
    auto bad = o;
    bad.learning_rate = -1.0F;
    expect_throws<std::invalid_argument>(
        [&] { (void)refiner.refine(init, pos, ruv, kTri, std::span<const pd::ProjectionView>(&view, 1), {}, bad); },
        "a negative learning rate");
}

template <class T>
std::vector<T> read_file(const std::string& path, std::size_t n) {
    std::vector<T> v(n);
    std::ifstream f(path, std::ios::binary);
    if (!f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * sizeof(T))))
        throw std::runtime_error("cannot read " + path);
    return v;
}

template <class T>
void write_file(const std::string& path, const std::vector<T>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
    if (!f) throw std::runtime_error("cannot write " + path);
}

// in_dir/dims.u32 = V, T, W, H, A, TW, TH, TC; clip.f32 [V][4]; idx.u32 [T][3]; grad_raster.f32 [H][W][4];
// attr.f32 [V][A]; uv.f32 [H][W][2]; tex.f32 [TH][TW][TC]; grad_tex.f32 [H][W][TC]
void file_pass(const std::string& in, const std::string& out, pd::Rasterizer& r) {
    const auto d = read_file<std::uint32_t>(in + "/dims.u32", 8);
    const std::uint32_t V = d[0], T = d[1], W = d[2], H = d[3], A = d[4], TW = d[5], TH = d[6], TC = d[7];
    const std::size_t P = static_cast<std::size_t>(W) * H;
    const auto clip = read_file<float>(in + "/clip.f32", V * 4ull);
    const auto idx = read_file<std::uint32_t>(in + "/idx.u32", T * 3ull);
    const auto gr = read_file<float>(in + "/grad_raster.f32", P * 4);
    const auto attr = read_file<float>(in + "/attr.f32", static_cast<std::size_t>(V) * A);
    const auto uv = read_file<float>(in + "/uv.f32", P * 2);
    const auto tex = read_file<float>(in + "/tex.f32", static_cast<std::size_t>(TW) * TH * TC);
    const auto gt = read_file<float>(in + "/grad_tex.f32", P * TC);
    pd::RasterizeOptions opt;
    opt.width = W;
    opt.height = H;
    const auto fw = r.forward(clip, idx, opt);
    write_file(out + "/raster.f32", fw.raster);
    write_file(out + "/derivatives.f32", fw.barycentric_derivatives);
    write_file(out + "/grad_clip.f32", r.backward(clip, idx, fw, gr));
    write_file(out + "/interp.f32", r.interpolate_forward(attr, A, idx, fw).values);
    const pd::TextureDesc td{TW, TH, TC, pd::AddressMode::wrap};
    write_file(out + "/sampled.f32", r.texture_forward(tex, td, uv, fw).values);
    const auto tg = r.texture_backward(tex, td, uv, fw, gt);
    write_file(out + "/grad_texture.f32", tg.texture);
    write_file(out + "/grad_uv.f32", tg.uv);
}

}  // namespace

// tests/native_tests.cpp:34-117 (padding) and tests/texture_surface_fill_test.cpp through the C++ API.
void padding_checks() {
    constexpr std::uint32_t n = 24;
    const auto at = [](std::uint32_t x, std::uint32_t y) { return static_cast<std::size_t>(y) * n + x; };
    pd::TextureBakeOutput out;
    out.width = out.height = n;
    out.color.assign(n * n * 4, 0.0F);
    out.valid_mask.assign(n * n, 0.0F);
    out.coverage_mask.assign(n * n, 0.0F);
    const std::array<float, 4> src{0.25F, 0.5F, 0.75F, 1.0F};
    for (std::uint32_t y = 2; y < 6; ++y)
        for (std::uint32_t x = 2; x < 6; ++x) {
            out.valid_mask[at(x, y)] = out.coverage_mask[at(x, y)] = 1.0F;
            std::copy(src.begin(), src.end(), out.color.begin() + at(x, y) * 4);
        }
    for (std::uint32_t y = 10; y < 18; ++y)
        for (std::uint32_t x = 10; x < 18; ++x) out.coverage_mask[at(x, y)] = 1.0F;
    pd::TextureBakeOutput untouched = out;
    pd::TexturePaddingOptions opt;
    opt.margin = 3;
    const auto st = pd::pad_texture_atlas(out, opt);
    expect(st.valid_texels == 16 && st.unobserved_texels == 64 && st.remaining_unobserved == 0, "padding counts");
    expect(st.gutter_texels > 0 && st.filled_texels == st.gutter_texels + st.unobserved_texels, "padding totals");
    const auto is_src = [&](std::uint32_t x, std::uint32_t y) {
        const float* p = out.color.data() + at(x, y) * 4;
        return std::abs(p[0] - src[0]) < 1e-6F && std::abs(p[1] - src[1]) < 1e-6F &&
               std::abs(p[2] - src[2]) < 1e-6F && p[3] == 1.0F;
    };
    expect(is_src(2, 6) && is_src(10, 10), "gutter and unobserved texels take the source colour");
    expect(out.filled_mask[at(10, 10)] > 0.5F && out.filled_mask[at(2, 2)] < 0.5F, "filled_mask provenance");
    expect(out.valid_mask[at(10, 10)] < 0.5F && out.color[at(2, 12) * 4] == 0.0F, "padding stays in bounds");
    pd::TexturePaddingOptions off;
    off.margin = 0;
    off.fill_unobserved = false;
    const auto none = pd::pad_texture_atlas(untouched, off);
    expect(none.filled_texels == 0 && none.remaining_unobserved == 64, "disabled padding");
    pd::TextureBakeOutput empty;
    expect_throws<std::invalid_argument>([&] { (void)pd::pad_texture_atlas(empty); }, "padding an empty atlas");

    pd::TextureBakeOutput atlas;
    atlas.width = 7;
    atlas.height = 1;
    atlas.color.assign(7 * 4, 0.0F);
    atlas.valid_mask = {1, 0, 1, 0, 0, 0, 0};
    atlas.coverage_mask = {1, 1, 1, 1, 1, 0, 0};
    atlas.face_ids = {0, 0, 2, 1, 3, UINT32_MAX, UINT32_MAX};
    atlas.color[0] = 0.8F;
    atlas.color[3] = 1.0F;
    atlas.color[2 * 4 + 2] = 0.6F;
    atlas.color[2 * 4 + 3] = 1.0F;
    const std::uint32_t topology[] = {0, 1, 2, 2, 1, 3, 4, 5, 6, 7, 8, 9};
    const auto fs = pd::fill_texture_on_surface(atlas, topology);
    expect(fs.measured_faces == 2 && fs.propagated_faces == 1 && fs.filled_texels == 2 && fs.remaining_texels == 1,
           "surface fill statistics");
    expect(atlas.color[4] == 0.8F && atlas.color[3 * 4] == 0.8F && atlas.color[3 * 4 + 2] == 0.0F,
           "surface fill crosses the mesh edge, not the UV island");
    pd::TexturePaddingOptions guard;
    guard.margin = 2;
    guard.fill_unobserved = false;
    const auto padded = pd::pad_texture_atlas(atlas, guard);
    expect(padded.unobserved_texels == 2 && padded.remaining_unobserved == 1, "padding keeps surface fills");
    expect(atlas.color[5 * 4] == 0.8F && atlas.color[4 * 4] == 0.0F && atlas.filled_mask[3] == 1.0F, "gutter colour");
    auto bad = atlas;
    bad.face_ids[1] = 100;
    expect_throws<std::invalid_argument>([&] { (void)pd::fill_texture_on_surface(bad, topology); },
                                         "a face id beyond the mesh");
}

int main(int argc, char** argv) {
    try {
        expect_throws<std::out_of_range>([] { pd::Context bad(pd::ContextOptions{4096, false}); },
                                         "a device index beyond the device count");
        pd::Context ctx;
        expect(!ctx.device_info().name.empty(), "device name");
        expect(!pd::Context::enumerate_devices().empty(), "device enumeration");
        pd::Rasterizer r(ctx);
        raster_checks(r);
        bake_checks(ctx);
        refine_checks(ctx);
        padding_checks();
        if (argc == 3) file_pass(argv[1], argv[2], r);
        std::printf("cpp_api_test: %d checks passed\n", g_checks);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "cpp_api_test: %s (after %d checks)\n", e.what(), g_checks);
        return 1;
    }
}

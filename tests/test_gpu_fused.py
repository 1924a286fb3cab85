"""The fused many-view render path (pdr_render_forward / pdr_render_backward) against the separate
reference-shaped kernels and the oracle: forward bit-exact, gradients within the FP64 tolerance."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import api
from photara_drender_gb300 import synthetic as S
from tests.gpu_util import grad_check, same_bits

pytestmark = pytest.mark.gpu


def run(fused, clip, idx, attrs, uva, tex, g_attr, g_samp, H, W, mode=0, viewports=None):
    from photara_drender_gb300 import Rasterizer
    from photara_drender_gb300.pipeline import RenderFwdBwd

    r = Rasterizer(0)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    views, V = clip.shape[0], clip.shape[1]
    p = RenderFwdBwd(r, torch.tensor(idx.astype(np.int32)), V, views, H, W, attrs.shape[1], tex.shape,
                     viewports=viewports, address_mode=mode, fused=fused)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    args = [t(clip), t(attrs), t(uva), t(tex)]
    p.forward(*args, stream)
    p.backward(*args, t(g_attr), t(g_samp), stream)
    torch.cuda.synchronize()
    p.check_capacity()
    return {k: getattr(p, k).cpu().numpy() for k in ("raster", "deriv", "attr_out", "uv", "sampled", "grad_tex",
                                                     "grad_attr", "grad_uv_attr", "grad_clip")}


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_fused_matches_separate_kernels_and_oracle(mode):
    rng = np.random.default_rng(mode)
    pos3, idx = S.icosphere(4)
    mats, _ = S.orbit_cameras(3)
    clip = S.clip_positions(pos3, mats)
    uva = (S.spherical_uv(pos3) * 1.2 - 0.1).astype(np.float32)
    attrs = rng.uniform(size=(pos3.shape[0], 3)).astype(np.float32)
    tex = rng.uniform(size=(64, 48, 4)).astype(np.float32)
    H, W = 96, 80
    g_attr = rng.normal(size=(3, H, W, 3)).astype(np.float32)
    g_samp = rng.normal(size=(3, H, W, 4)).astype(np.float32)
    vps = [None, (3.0, -2.0, 70.0, 90.0), None]
    f = run(True, clip, idx, attrs, uva, tex, g_attr, g_samp, H, W, mode, vps)
    s = run(False, clip, idx, attrs, uva, tex, g_attr, g_samp, H, W, mode, vps)
    for k in ("raster", "deriv", "attr_out", "uv", "sampled"):
        assert same_bits(f[k], s[k]), k
    names = ["clamp", "wrap", "mirror"]
    # oracle chain (reference order) and FP64 twins, summed over the views
    o = {k: 0 for k in ("gt32", "gt64", "gtabs", "ga32", "ga64", "gaabs", "gu32", "gu64", "guabs")}
    for v in range(3):
        vp = vps[v]
        r, d = api.rasterize_forward(clip[v], idx, (H, W), viewport=vp)
        assert same_bits(f["raster"][v], r) and same_bits(f["deriv"][v], d)
        uv = api.interpolate_forward(uva, idx, r)
        gt, gu = api.texture_backward(tex, uv, r, g_samp[v], names[mode])
        o["gt32"] = o["gt32"] + gt.astype(np.float64)
        o["gt64"] = o["gt64"] + api.texture_backward(tex, uv, r, g_samp[v], names[mode], f64=True)[0]
        o["gtabs"] = o["gtabs"] + api.texture_backward(tex, uv, r, g_samp[v], names[mode], f64=True, abs_terms=True)[0]
        guv, gr1 = api.interpolate_backward(uva, idx, r, gu)
        ga, gr2 = api.interpolate_backward(attrs, idx, r, g_attr[v])
        o["gu32"] = o["gu32"] + guv.astype(np.float64)
        o["gu64"] = o["gu64"] + api.interpolate_backward(uva, idx, r, gu, f64=True)[0]
        o["guabs"] = o["guabs"] + api.interpolate_backward(uva, idx, r, gu, f64=True, abs_terms=True)[0]
        o["ga32"] = o["ga32"] + ga.astype(np.float64)
        o["ga64"] = o["ga64"] + api.interpolate_backward(attrs, idx, r, g_attr[v], f64=True)[0]
        o["gaabs"] = o["gaabs"] + api.interpolate_backward(attrs, idx, r, g_attr[v], f64=True, abs_terms=True)[0]
        grs = (gr1 + gr2).astype(np.float32)
        gp32 = api.rasterize_backward(clip[v], idx, r, grs, viewport=vp)
        gp64 = api.rasterize_backward(clip[v], idx, r, grs, viewport=vp, f64=True)
        gpab = api.rasterize_backward(clip[v], idx, r, grs, viewport=vp, f64=True, abs_terms=True)
        grad_check(f["grad_clip"][v], gp32, gp64, gpab, name=f"fused grad_clip view {v}")
        grad_check(s["grad_clip"][v], gp32, gp64, gpab, name=f"separate grad_clip view {v}")
    for key, a, b, c in (("grad_tex", "gt32", "gt64", "gtabs"), ("grad_attr", "ga32", "ga64", "gaabs"),
                         ("grad_uv_attr", "gu32", "gu64", "guabs")):
        grad_check(f[key], o[a], o[b], o[c], name=f"fused {key}")
        grad_check(s[key], o[a], o[b], o[c], name=f"separate {key}")


def test_bin_once_raster_many():
    """pdr_render_bin + pdr_render_raster equal pdr_render_forward, and bins made once serve later rasters
    with other attributes and textures (the geometry is unchanged)."""
    from photara_drender_gb300 import Rasterizer, _native
    from photara_drender_gb300.pipeline import RenderFwdBwd

    rng = np.random.default_rng(3)
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(2)
    clip = S.clip_positions(pos3, mats)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    uva = t(S.spherical_uv(pos3).astype(np.float32))
    H, W = 72, 88
    V = pos3.shape[0]
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    L = _native.lib()
    outs = []
    p = RenderFwdBwd(Rasterizer(0), torch.tensor(idx.astype(np.int32)), V, 2, H, W, 3, (32, 40, 4))
    tclip = t(clip)
    for k in range(3):
        attrs = t(rng.uniform(size=(V, 3)).astype(np.float32))
        tex = t(rng.uniform(size=(32, 40, 4)).astype(np.float32))
        a = p._args(tclip, attrs, uva, tex, None, None)  # the tensors above stay referenced while a is used
        if k == 0:
            _native.check(L.pdr_render_forward(C.addressof(a), stream))
        else:
            if k == 1:
                _native.check(L.pdr_render_bin(C.addressof(a), stream))
            _native.check(L.pdr_render_raster(C.addressof(a), stream))
        torch.cuda.synchronize()
        got = {n: getattr(p, n).cpu().numpy().copy() for n in ("raster", "attr_out", "sampled")}
        _native.check(L.pdr_render_forward(C.addressof(a), stream))
        torch.cuda.synchronize()
        want = {n: getattr(p, n).cpu().numpy() for n in ("raster", "attr_out", "sampled")}
        for n in got:
            assert same_bits(got[n], want[n]), (k, n)
        outs.append(want["sampled"])
    assert not np.array_equal(outs[1], outs[2])


@pytest.mark.parametrize("atlas", [4096, 256])
def test_gradient_sums_at_scale(atlas):
    """Size-independent properties of the fused adjoint at the benchmark's view size (4 views at
    1024x1024): bilinear and barycentric weights each sum to one, so the texture gradient summed over
    texels equals the sample gradient summed over covered pixels, and the attribute gradient summed over
    vertices equals the attribute gradient summed over covered pixels, within 1e-5 of the sum of
    |terms| (fp32 atomics in any order); a minified (4096^2) and a magnified (256^2) texture take the
    plain and the warp-aggregated reductions."""
    from photara_drender_gb300 import Rasterizer
    from photara_drender_gb300.pipeline import RenderFwdBwd

    dev = torch.device("cuda", 0)
    pos3, idx = S.icosphere(6)
    mats, _ = S.orbit_cameras(4)
    clip = torch.tensor(S.clip_positions(pos3, mats), device=dev)
    V, T, H, W = pos3.shape[0], idx.shape[0], 1024, 1024
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    attrs = torch.rand((V, 3), device=dev, generator=g)
    uva = torch.tensor(S.spherical_uv(pos3).astype(np.float32), device=dev)
    tex = torch.rand((atlas, atlas, 4), device=dev, generator=g)
    g_attr = torch.randn((4, H, W, 3), device=dev, generator=g)
    g_samp = torch.randn((4, H, W, 4), device=dev, generator=g)
    p = RenderFwdBwd(Rasterizer(0), torch.tensor(idx.astype(np.int32)), V, 4, H, W, 3, tuple(tex.shape))
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    p.forward(clip, attrs, uva, tex, stream)
    p.backward(clip, attrs, uva, tex, g_attr, g_samp, stream)
    torch.cuda.synchronize()
    p.check_capacity()
    ids = p.raster[..., 3]
    cov = (ids != 0).unsqueeze(-1).double()
    ref_t, abs_t = (g_samp.double() * cov).sum((0, 1, 2)), (g_samp.double().abs() * cov).sum((0, 1, 2))
    covv = ((ids >= 0.5) & (ids < T + 0.5)).unsqueeze(-1).double()
    ref_a, abs_a = (g_attr.double() * covv).sum((0, 1, 2)), (g_attr.double().abs() * covv).sum((0, 1, 2))
    err_t = ((p.grad_tex.double().sum((0, 1)) - ref_t).abs() / abs_t).max().item()
    err_a = ((p.grad_attr.double().sum(0) - ref_a).abs() / abs_a).max().item()
    assert cov.sum().item() > 1e6
    assert err_t <= 1e-5 and err_a <= 1e-5, (err_t, err_a)


def test_tile_configurations_give_identical_outputs():
    """The fused forward with every compiled tile shape and stage depth (pipeline.TILE_CONFIGS) gives the
    outputs of the default 16x16/256 bins bit for bit, also when a configuration's tile list overflows;
    the autotuner picks one of them and sizes its list."""
    from photara_drender_gb300 import Rasterizer
    from photara_drender_gb300.pipeline import TILE_CONFIGS, RenderFwdBwd

    rng = np.random.default_rng(12)
    pos3, idx = S.icosphere(5)
    mats, _ = S.orbit_cameras(3)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev)  # noqa: E731
    clip, V = t(S.clip_positions(pos3, mats)), pos3.shape[0]
    attrs, uva = t(rng.uniform(size=(V, 3))), t(S.spherical_uv(pos3))
    tex = t(rng.uniform(size=(128, 96, 4)))
    H, W = 150, 131  # ragged: partial tiles in both directions for every shape
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    r = Rasterizer(0)
    outs = {}
    for cfg in TILE_CONFIGS:
        for cap in (None, 2000):
            p = RenderFwdBwd(r, torch.tensor(idx.astype(np.int32)), V, 3, H, W, 3, tuple(tex.shape), capacity=cap,
                             tile_config=cfg, viewports=[None, (5.0, -3.0, 120.0, 140.0), None])
            p.forward(clip, attrs, uva, tex, stream)
            torch.cuda.synchronize()
            outs[(cfg, cap)] = [getattr(p, k).clone() for k in ("raster", "deriv", "attr_out", "uv", "sampled")]
            if cap:
                assert int(p.status[2]) == 1  # the small list overflowed
    ref = outs[((16, 16, 256), None)]
    for key, got in outs.items():
        for a, b in zip(got, ref):
            assert torch.equal(a.view(torch.int32), b.view(torch.int32)), key
    p = RenderFwdBwd(r, torch.tensor(idx.astype(np.int32)), V, 3, H, W, 3, tuple(tex.shape),
                     viewports=[None, (5.0, -3.0, 120.0, 140.0), None])
    times = p.autotune(clip, attrs, uva, tex, reps=2)
    assert set(times) == set(TILE_CONFIGS) and p.tile_config in TILE_CONFIGS
    p.forward(clip, attrs, uva, tex, stream)
    torch.cuda.synchronize()
    assert p.check_capacity() > 0 and torch.equal(p.raster.view(torch.int32), ref[0].view(torch.int32))


@pytest.mark.parametrize("attributes", [3, 8, 0])
def test_backward_with_and_without_vertex_records(attributes):
    """pdr_render_backward with a workspace of pdr_render_backward_workspace_bytes() (per-view vertex
    records, summed over the views by a second pass) and without one (reductions straight into the
    outputs): every gradient agrees to float rounding, the texture gradient (the same reductions both
    ways) included."""
    from photara_drender_gb300 import Rasterizer, _native
    from photara_drender_gb300.pipeline import RenderFwdBwd

    rng = np.random.default_rng(7)
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(3)
    clip = S.clip_positions(pos3, mats)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)  # noqa: E731
    V, H, W = pos3.shape[0], 96, 112
    A = max(attributes, 1)
    p = RenderFwdBwd(Rasterizer(0), torch.tensor(idx.astype(np.int32)), V, 3, H, W, A, (64, 48, 4))
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    args = [t(clip), t(rng.uniform(size=(V, A)).astype(np.float32)), t(S.spherical_uv(pos3).astype(np.float32)),
            t(rng.uniform(size=(64, 48, 4)).astype(np.float32))]
    g_attr = t(rng.standard_normal((3, H, W, A)).astype(np.float32))
    g_samp = t(rng.standard_normal((3, H, W, 4)).astype(np.float32))
    p.forward(*args, stream)
    L = _native.lib()
    res = []
    for records in (True, False):
        a = p._args(*args, g_attr, g_samp)
        if not attributes:
            a.attributes, a.attribute_count, a.grad_attributes, a.grad_interpolated = None, 0, None, None
        if not records:
            a.workspace, a.workspace_bytes = None, 0
        else:
            assert a.workspace_bytes >= L.pdr_render_backward_workspace_bytes(3, V, attributes)
        _native.check(L.pdr_render_backward(C.addressof(a), stream))
        torch.cuda.synchronize()
        res.append({k: getattr(p, k).cpu().numpy().copy() for k in ("grad_tex", "grad_uv_attr", "grad_clip")
                    + (("grad_attr",) if attributes else ())})
    for k, want in res[1].items():
        got = res[0][k]
        scale = np.abs(want).max()
        assert scale > 0, k
        assert np.allclose(got, want, rtol=1e-5, atol=1e-6 * scale), (k, np.abs(got - want).max(), scale)

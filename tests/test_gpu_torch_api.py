"""The reference's Python surface on the GPU: tests/python_smoke.py restated (shapes, finiteness,
autograd through rasterize -> interpolate -> texture, the atlas helpers, the native refiner) plus
autograd-vs-direct-adjoint equality."""
import numpy as np
import pytest
import torch

import photara_drender_gb300 as pdr
from oracle import api
from photara_drender_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

TRI = np.array([[-0.75, -0.75, 0.0, 1.0], [0.75, -0.75, 0.0, 1.0], [0.0, 0.75, 0.0, 1.0]], np.float32)
IDX = np.array([[0, 1, 2]], np.uint32)


@pytest.fixture(scope="module")
def rast():
    return pdr.Rasterizer()


def test_python_smoke_numpy_surface(rast):
    raster, derivatives = rast.forward(TRI, IDX, (16, 20))
    assert raster.shape == (16, 20, 4) and derivatives.shape == raster.shape
    assert np.count_nonzero(raster[..., 3]) > 0
    grad_raster = np.zeros_like(raster)
    grad_raster[..., 0] = 1.0
    gp = rast.backward(TRI, IDX, raster, grad_raster)
    assert gp.shape == TRI.shape and np.isfinite(gp).all()
    attributes = np.eye(3, dtype=np.float32)
    interp = rast.interpolate_forward(attributes, IDX, raster)
    assert interp.shape == (16, 20, 3)
    ga, gr = rast.interpolate_backward(attributes, IDX, raster, np.ones_like(interp))
    assert ga.shape == attributes.shape and gr.shape == raster.shape and np.isfinite(ga).all()
    uva = np.array([[0.2, 0.2], [0.8, 0.2], [0.5, 0.8]], np.float32)
    uv = rast.interpolate_forward(uva, IDX, raster)
    tex = np.arange(4 * 4 * 3, dtype=np.float32).reshape(4, 4, 3) / 48.0
    sampled = rast.texture_forward(tex, uv, raster)
    assert sampled.shape == (16, 20, 3)
    gt, gu = rast.texture_backward(tex, uv, raster, np.ones_like(sampled))
    assert gt.shape == tex.shape and gu.shape == uv.shape and np.isfinite(gt).all() and np.isfinite(gu).all()
    gt2, gu2 = rast.texture_backward(tex, uv, raster, np.ones_like(sampled), compute_uv_gradient=False)
    assert gu2 is None
    for mode in ("wrap", "mirror"):
        assert np.isfinite(rast.texture_forward(tex, uv + 1.25, raster, mode)).all()
    vr, _ = rast.forward(TRI, IDX, (20, 24), viewport=(4.0, 3.0, 16.0, 12.0))
    assert np.count_nonzero(vr[:3, ..., 3]) == 0 and np.count_nonzero(vr[15:, ..., 3]) == 0
    assert rast.device_info.name


def test_python_smoke_torch_surface(rast):
    dev = torch.device("cuda", 0)
    positions = torch.tensor(TRI, device=dev, requires_grad=True)
    indices = torch.tensor(IDX.astype(np.int64), device=dev)
    raster, _ = pdr.rasterize(positions, indices, (16, 20), rasterizer=rast)
    attrs = torch.eye(3, dtype=torch.float32, device=dev, requires_grad=True)
    image = pdr.interpolate(attrs, raster, indices, rasterizer=rast)
    uva = torch.tensor([[0.2, 0.2], [0.8, 0.2], [0.5, 0.8]], device=dev, requires_grad=True)
    uv = pdr.interpolate(uva, raster, indices, rasterizer=rast)
    tex = torch.tensor(np.arange(48, dtype=np.float32).reshape(4, 4, 3) / 48.0, device=dev, requires_grad=True)
    sampled = pdr.texture(tex, uv, raster, rasterizer=rast)
    (image[..., 0].sum() + sampled.square().sum()).backward()
    for t in (positions, attrs, uva, tex):
        assert t.grad is not None and torch.isfinite(t.grad).all()
    render = pdr.render_textured_mesh(positions.detach(), indices, uva.detach(), tex.detach(), (16, 20),
                                      rasterizer=rast)
    assert render.image.shape == (16, 20, 3)
    assert torch.isfinite(pdr.masked_charbonnier_loss(render.image, sampled.detach(), render.valid_mask))
    assert torch.isfinite(pdr.atlas_total_variation(tex.detach()))
    opts = pdr.AtlasOptimizationOptions(steps=2, learning_rate=1e-2, total_variation_weight=0.0, seam_weight=0.0,
                                        cache_view_rasters=True)
    out, hist = pdr.optimize_texture_atlas(tex.detach() * 0.9, positions.detach()[None], indices, uva.detach(),
                                           [sampled.detach()], rasterizer=rast, options=opts)
    assert out.shape == tex.shape and len(hist) == 2 and np.isfinite(hist).all()


def test_autograd_equals_direct_adjoints(rast):
    rng = np.random.default_rng(0)
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(2)
    clip = S.clip_positions(pos3, mats)
    dev = torch.device("cuda", 0)
    tclip = torch.tensor(clip, device=dev, requires_grad=True)
    tidx = torch.tensor(idx.astype(np.int64), device=dev)
    uva = torch.tensor(S.spherical_uv(pos3), device=dev, requires_grad=True)
    tex = torch.tensor(rng.uniform(size=(32, 32, 4)).astype(np.float32), device=dev, requires_grad=True)
    raster, _ = pdr.rasterize(tclip, tidx, (64, 64), rasterizer=rast, recompute_in_backward=True)
    uv = pdr.interpolate(uva, raster, tidx, rasterizer=rast)
    img = pdr.texture(tex, uv, raster, rasterizer=rast)
    g = torch.tensor(rng.normal(size=img.shape).astype(np.float32), device=dev)
    img.backward(g)
    gt, gu = rast.texture_backward(tex.detach(), uv.detach(), raster.detach(), g)
    ga, gr = rast.interpolate_backward(uva.detach(), tidx, raster.detach(), gu)
    gp = rast.backward(tclip.detach(), tidx, raster.detach(), gr)
    # Both sides sum with atomics in no fixed order: they agree to the summation-order error, a few
    # ulps of the sum of absolute terms (the same adjoints run on |upstream gradient|).
    gt_abs, _ = rast.texture_backward(tex.detach(), uv.detach(), raster.detach(), g.abs())
    assert bool(((tex.grad - gt).abs() <= 8e-6 * gt_abs + 1e-12).all())
    ga_abs, _ = rast.interpolate_backward(uva.detach(), tidx, raster.detach(), gu.abs())
    assert bool(((uva.grad - ga).abs() <= 8e-6 * ga_abs.abs() + 1e-12).all())
    assert torch.allclose(tclip.grad, gp, rtol=1e-4, atol=1e-5)


def test_native_refine_smoke(rast):
    # tests/python_smoke.py:83-100
    baker = pdr.TextureBaker()
    wp = TRI[:, :3].copy()
    buv = np.array([[0.125, 0.125], [0.875, 0.125], [0.5, 0.875]], np.float32)
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (3, 1))
    image = np.zeros((16, 16, 4), np.float32)
    image[..., 0], image[..., 1], image[..., 3] = 0.75, 0.25, 1.0
    mats = np.eye(4, dtype=np.float32)[None]
    baked = pdr.project_texture_atlas(pdr.UnwrappedMesh(wp, nrm, buv, IDX, np.arange(3), np.zeros(1), 1, 0.0),
                                      [image], mats, np.array([[0, 0, 2]], np.float32), resolution=(16, 16),
                                      baker=baker)
    assert baked.color.shape == (16, 16, 4) and baked.valid_mask.any()
    refined, hist, seam, pre, opt = baker.refine_texture(np.ascontiguousarray(baked.color[..., :3] * 0.5), wp, buv, IDX,
                                                         [image], mats, steps=3, batch_size=1, learning_rate=0.05,
                                                         minimum_learning_rate=0.01, seam_polish_steps=0)
    assert refined.shape == (16, 16, 3) and hist.shape == (3,) and np.isfinite(hist).all()
    assert hist[-1] < hist[0] and seam.shape == (0,) and pre >= 0 and opt >= 0
    o_ref, o_hist, _ = api.refine(baked.color[..., :3] * 0.5, wp, buv, IDX, [image], mats, steps=3, batch_size=1,
                                  learning_rate=0.05, minimum_learning_rate=0.01, seam_polish_steps=0)
    assert np.allclose(hist, o_hist, rtol=1e-5) and np.abs(refined - o_ref).max() < 1e-5


@pytest.mark.parametrize("batched", [True, False])
def test_fused_render_equals_separate_ops(rast, batched):
    """photara_drender_gb300.torch.render (one fused forward and one fused backward kernel) against
    rasterize -> interpolate x2 -> texture: outputs bit-identical; gradients equal up to the summation
    order of the atomics (here also with upstream gradients on the raster and uv outputs, which take
    the separate adjoint kernels)."""
    rng = np.random.default_rng(9)
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(3)
    clip = S.clip_positions(pos3, mats)
    if not batched:
        clip = clip[1]
    dev = torch.device("cuda", 0)
    V = pos3.shape[0]
    inputs = dict(clip=clip, attrs=rng.uniform(size=(V, 3)).astype(np.float32),
                  uv=S.spherical_uv(pos3) * 1.2 - 0.1, tex=rng.uniform(size=(32, 48, 4)).astype(np.float32))
    tidx = torch.tensor(idx.astype(np.int64), device=dev)
    res = (80, 96)
    lead = (3,) if batched else ()
    g = dict(a=rng.normal(size=lead + res + (3,)), u=rng.normal(size=lead + res + (2,)),
             s=rng.normal(size=lead + res + (4,)), r=rng.normal(size=lead + res + (4,)))
    g = {k: torch.tensor(v.astype(np.float32), device=dev) for k, v in g.items()}

    def leaves():
        return {k: torch.tensor(np.asarray(v, np.float32), device=dev, requires_grad=True) for k, v in inputs.items()}

    f = leaves()
    out = pdr.render(f["clip"], tidx, res, rasterizer=rast, vertex_attributes=f["attrs"], vertex_uv=f["uv"],
                     texture=f["tex"], address_mode="wrap")
    s_ = leaves()
    raster, deriv = pdr.rasterize(s_["clip"], tidx, res, rasterizer=rast)
    a = pdr.interpolate(s_["attrs"], raster, tidx, rasterizer=rast)
    u = pdr.interpolate(s_["uv"], raster, tidx, rasterizer=rast)
    smp = pdr.texture(s_["tex"], u, raster, rasterizer=rast, address_mode="wrap")
    for x, y in ((out.raster, raster), (out.derivatives, deriv), (out.interpolated, a), (out.uv, u), (out.sampled, smp)):
        assert x.shape == y.shape and torch.equal(x.view(torch.int32), y.view(torch.int32))
    loss_f = (out.interpolated * g["a"]).sum() + (out.sampled * g["s"]).sum() + (out.uv * g["u"]).sum() + \
        (out.raster * g["r"]).sum()
    loss_s = (a * g["a"]).sum() + (smp * g["s"]).sum() + (u * g["u"]).sum() + (raster * g["r"]).sum()
    loss_f.backward()
    loss_s.backward()
    for k in inputs:
        x, y = f[k].grad, s_[k].grad
        assert x.shape == y.shape
        scale = float(y.abs().max())
        assert float((x - y).abs().max()) <= 1e-4 * scale + 1e-7, k


def _render_case(seed=4, views=3, res=(96, 112)):
    rng = np.random.default_rng(seed)
    pos3, idx = S.icosphere(4)
    mats, _ = S.orbit_cameras(views)
    V = pos3.shape[0]
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev)  # noqa: E731
    inputs = dict(clip=t(S.clip_positions(pos3, mats)), attrs=t(rng.uniform(size=(V, 3))),
                  uv=t(S.spherical_uv(pos3)), tex=t(rng.uniform(size=(64, 48, 4))))
    grads = dict(a=t(rng.normal(size=(views,) + res + (3,))), s=t(rng.normal(size=(views,) + res + (4,))))
    return inputs, torch.tensor(idx.astype(np.int64), device=dev), res, grads


def test_render_without_host_waits_captures_in_a_cuda_graph():
    """torch.render with deferred_errors=True waits for nothing, so its forward and backward can be
    captured in a CUDA graph: replays give the forward outputs of an ordinary call bit for bit and its
    gradients up to the summation order of the atomics."""
    r = pdr.Rasterizer()
    inputs, tidx, res, grads = _render_case()
    static = {k: v.clone().requires_grad_(True) for k, v in inputs.items()}

    def step():
        out = pdr.render(static["clip"], tidx, res, rasterizer=r, vertex_attributes=static["attrs"],
                         vertex_uv=static["uv"], texture=static["tex"], deferred_errors=True)
        torch.autograd.backward([out.interpolated, out.sampled], [grads["a"], grads["s"]])
        return out

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):  # warm-up outside the capture sizes the tile-list capacity
        for _ in range(2):
            for v in static.values():
                v.grad = None
            step()
    torch.cuda.current_stream().wait_stream(side)
    pdr.check_deferred_errors(r)
    for v in static.values():
        v.grad = None
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        out = step()
    ref_leaves = {k: v.clone().requires_grad_(True) for k, v in inputs.items()}
    ref = pdr.render(ref_leaves["clip"], tidx, res, rasterizer=r, vertex_attributes=ref_leaves["attrs"],
                     vertex_uv=ref_leaves["uv"], texture=ref_leaves["tex"])
    torch.autograd.backward([ref.interpolated, ref.sampled], [grads["a"], grads["s"]])
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        for x, y in ((out.raster, ref.raster), (out.interpolated, ref.interpolated), (out.uv, ref.uv),
                     (out.sampled, ref.sampled)):
            assert torch.equal(x.view(torch.int32), y.view(torch.int32))
        for k in inputs:
            x, y = static[k].grad, ref_leaves[k].grad
            assert float((x - y).abs().max()) <= 1e-5 * float(y.abs().max()) + 1e-7, k
    pdr.check_deferred_errors(r)


def test_tile_list_overflow_keeps_results_exact():
    """A tile list far below the binning's need: the raster kernel rasterizes the tiles whose lists were
    cut from all triangles with the binning rule, so the fused forward (and the separate rasterize call)
    give exactly the outputs of a sufficient list, and the status reports the overflow."""
    import ctypes as C

    from photara_drender_gb300 import _native
    from photara_drender_gb300.pipeline import RenderFwdBwd

    inputs, tidx, res, grads = _render_case(seed=5, views=2, res=(80, 72))
    r = pdr.Rasterizer()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    V = inputs["clip"].shape[1]
    outs = []
    for cap in (None, 300):
        p = RenderFwdBwd(r, tidx, V, 2, res[0], res[1], 3, tuple(inputs["tex"].shape), capacity=cap)
        p.forward(inputs["clip"], inputs["attrs"], inputs["uv"], inputs["tex"], stream)
        torch.cuda.synchronize()
        overflow = int(p.status[_native.STATUS_TILE_OVERFLOW])
        outs.append(({k: getattr(p, k).clone() for k in ("raster", "deriv", "attr_out", "uv", "sampled")}, overflow))
    (full, ov0), (cut, ov1) = outs
    assert ov0 == 0 and ov1 == 1
    for k in full:
        assert torch.equal(full[k].view(torch.int32), cut[k].view(torch.int32)), k
    # the separate, reference-shaped path (sorted bins) with the same cut list
    sep = RenderFwdBwd(r, tidx, V, 2, res[0], res[1], 3, tuple(inputs["tex"].shape), capacity=300, fused=False)
    sep.forward(inputs["clip"], inputs["attrs"], inputs["uv"], inputs["tex"], stream)
    torch.cuda.synchronize()
    assert int(sep.status[_native.STATUS_TILE_OVERFLOW]) == 1
    assert torch.equal(sep.raster.view(torch.int32), full["raster"].view(torch.int32))


def test_deferred_errors_raise_later():
    """A non-finite uv in a covered pixel: the synchronous render raises in backward as the reference's
    texture adjoint does; with deferred_errors=True nothing waits and the error is raised by
    check_deferred_errors."""
    inputs, tidx, res, grads = _render_case(seed=6, views=1)
    uv = inputs["uv"].clone()
    uv[:] = float("nan")
    r = pdr.Rasterizer()

    def run(deferred):
        leaves = {k: v.clone().requires_grad_(True) for k, v in dict(inputs, uv=uv).items()}
        out = pdr.render(leaves["clip"][:1], tidx, res, rasterizer=r, vertex_attributes=leaves["attrs"],
                         vertex_uv=leaves["uv"], texture=leaves["tex"], deferred_errors=deferred)
        torch.autograd.backward([out.interpolated, out.sampled], [grads["a"][:1], grads["s"][:1]])

    with pytest.raises(ValueError, match="non-finite"):
        run(False)
    run(True)
    with pytest.raises(ValueError, match="non-finite"):
        pdr.check_deferred_errors(r)
    pdr.check_deferred_errors(r)  # reported once

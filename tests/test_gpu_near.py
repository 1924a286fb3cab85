"""Near-plane clipping on the GPU (the reference has none: README.md:140) through the C ABI: the clipped
mesh (pdr_clip_near), the clipped raster with its remap (pdr_remap_near) and the adjoint
(pdr_rasterize_backward_near) against the oracle's float32 restatement, bit for bit for positions, ids,
barycentrics, depth and derivatives, and tests/gpu_util.grad_check (1e-5 relative against float64) for
the gradient sums."""
import numpy as np
import pytest
import torch

from oracle import api
from photara_drender_gb300 import Rasterizer, _native
from photara_drender_gb300 import synthetic as S
from photara_drender_gb300 import torch as pdr_torch
from tests.gpu_util import grad_check, same_bits
from tests.near_scenes import cloud, ground

pytestmark = pytest.mark.gpu

CULL = {"none": 0, "back": 1, "front": 2}


@pytest.fixture(scope="module")
def r():
    return Rasterizer(0)


def test_clipped_mesh_bit_exact(r):
    clip, idx, _ = cloud(views=3)
    dev = torch.device("cuda", 0)
    c = torch.tensor(clip, device=dev)
    i = torch.tensor(idx.astype(np.int32), device=dev)
    views, V, T = clip.shape[0], clip.shape[1], idx.shape[0]
    cp = torch.full((views, 4 * T, 4), float("nan"), device=dev)
    ci = torch.full((2 * T, 3), -1, dtype=torch.int32, device=dev)
    status = torch.zeros(8, dtype=torch.int32, device=dev)
    _native.call("pdr_clip_near", c.data_ptr(), views, V, i.data_ptr(), T, cp.data_ptr(), ci.data_ptr(),
                 status.data_ptr(), None)
    torch.cuda.synchronize()
    for k in range(views):
        o_p, o_i = api.clip_near(clip[k], idx)
        assert same_bits(cp[k].cpu().numpy(), o_p), f"view {k} clipped positions"
        assert np.array_equal(ci.cpu().numpy().view(np.uint32), o_i)
    assert not status.any()


@pytest.mark.parametrize("scene", [ground, cloud])
@pytest.mark.parametrize("cull", ["none", "back", "front"])
def test_near_raster_bit_exact(r, scene, cull):
    clip, idx, res = scene()
    for vp in (None, (-3.0, 4.0, 70.0, 58.0)):
        raster, deriv = r.forward(clip, idx, res, cull_mode=cull, viewport=vp, clip_near_plane=True)
        o_r, o_d = api.rasterize_forward_near(clip, idx, res, CULL[cull], viewport=vp)
        assert same_bits(raster, o_r), f"raster cull={cull} vp={vp}"
        assert same_bits(deriv, o_d), f"derivatives cull={cull} vp={vp}"


def test_near_raster_many_views(r):
    clip, idx, res = cloud(views=4)
    raster, deriv = r.forward(clip, idx, res, clip_near_plane=True)
    for k in range(4):
        o_r, o_d = api.rasterize_forward_near(clip[k], idx, res)
        assert same_bits(raster[k], o_r) and same_bits(deriv[k], o_d), f"view {k}"


def test_nothing_clipped_equals_plain_path(r):
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(3)
    clip = S.clip_positions(pos3, mats)
    near = r.forward(clip, idx, (96, 80), clip_near_plane=True)
    plain = r.forward(clip, idx, (96, 80))
    assert same_bits(near[0], plain[0]) and same_bits(near[1], plain[1])
    g = np.random.default_rng(3).normal(size=plain[0].shape).astype(np.float32)
    a = r.backward(clip, idx, plain[0], g, clip_near_plane=True)
    b = r.backward(clip, idx, plain[0], g)
    assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()


@pytest.mark.parametrize("scene", [ground, cloud])
def test_near_backward_vs_oracle(r, scene):
    clip, idx, res = scene()
    o_r, _ = api.rasterize_forward_near(clip, idx, res)
    g = np.random.default_rng(7).normal(size=o_r.shape).astype(np.float32)
    got = r.backward(clip, idx, o_r, g, clip_near_plane=True)
    f32 = api.rasterize_backward_near(clip, idx, o_r, g, dtype=np.float32)
    f64 = api.rasterize_backward_near(clip, idx, o_r, g)
    fabs = api.rasterize_backward_near(clip, idx, o_r, g, abs_terms=True)
    grad_check(got, f32, f64, fabs, name="near grad_positions")
    behind = clip[:, 3] <= 1e-8
    assert np.abs(got[behind]).max() > 0, "vertices behind the eye receive gradient"


def test_torch_rasterize_near_autograd(r):
    clip, idx, res = ground()
    dev = torch.device("cuda", 0)
    pos = torch.tensor(clip, device=dev, requires_grad=True)
    tri = torch.tensor(idx.astype(np.int32), device=dev)
    g = torch.tensor(np.random.default_rng(8).normal(size=res + (4,)).astype(np.float32), device=dev)
    for recompute in (False, True):
        raster, _ = pdr_torch.rasterize(pos, tri, res, rasterizer=r, clip_near_plane=True,
                                        recompute_in_backward=recompute)
        (raster * g).sum().backward()
        want = r.backward(pos.detach(), tri, raster.detach(), g, clip_near_plane=True).cpu().numpy()
        got = pos.grad.detach().cpu().numpy()
        assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()
        pos.grad = None
    with pytest.raises(OverflowError):
        big = np.zeros((8388609, 3), np.uint32)
        r.forward(clip, big, res, clip_near_plane=True)


def test_near_derivatives_and_their_gradient(r):
    """With clipping, the derivative output and its gradient are those of the original triangle at the
    pixel, triangles behind the eye included: against the float64 derivative formula and its adjoint
    (oracle/api.py, checked by central differences in tests/test_oracle_derivative_grad.py)."""
    clip, idx, res = ground()
    raster, deriv = r.forward(clip, idx, res, clip_near_plane=True)
    ref = api.barycentric_derivatives_f64(clip, idx, raster)
    covered = raster[..., 3] > 0
    behind = (clip[idx.astype(np.int64)][..., 3] <= 1e-8).any(1)
    ids = np.rint(raster[..., 3]).astype(np.int64)
    assert behind[ids[covered] - 1].any()
    err = np.abs(deriv.astype(np.float64) - ref)[covered]
    assert err.max() <= 1e-4 * np.abs(ref).max(), err.max()
    gd = np.random.default_rng(9).normal(size=res + (4,)).astype(np.float32)
    got = r.backward(clip, idx, raster, np.zeros_like(raster), grad_barycentric_derivatives=gd, clip_near_plane=True)
    f64 = api.barycentric_derivatives_backward_f64(clip, idx, raster, gd)
    f32 = api.barycentric_derivatives_backward_f64(clip, idx, raster, gd, dtype=np.float32)
    fabs = api.barycentric_derivatives_backward_f64(clip, idx, raster, gd, abs_terms=True)
    bound = 4.0 * np.abs(f32 - f64) + 2e-6 * fabs + 1e-7 * np.abs(f64).max()
    assert np.all(np.abs(got.astype(np.float64) - f64) <= bound)
    assert np.abs(got[clip[:, 3] <= 1e-8]).max() > 0

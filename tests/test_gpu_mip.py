"""Mipmapped texture sampling on the GPU (csrc/mip.cu), a filtering mode the reference lists as planned
(README.md:141): the pyramid bit for bit against the host's fp32 box filter; sampling and its adjoint
against the float64 checker (oracle/api.py, itself checked by finite differences); bit-identical to
bilinear sampling where the level of detail is 0; the autograd path and attribute derivatives."""
import numpy as np
import pytest
import torch

from oracle import api
from photara_drender_gb300 import Rasterizer
from photara_drender_gb300 import mip as M
from photara_drender_gb300 import synthetic as S
from photara_drender_gb300 import torch as pdr_torch
from tests.gpu_util import same_bits
from tests.test_oracle_mip import case

pytestmark = pytest.mark.gpu
dev = torch.device("cuda", 0)


def t(a):
    return torch.tensor(np.ascontiguousarray(a), device=dev)


@pytest.fixture(scope="module")
def r():
    return Rasterizer(0)


@pytest.mark.parametrize("shape", [(37, 50, 3), (64, 64, 4), (1, 9, 2), (13, 1, 1)])
def test_pyramid_matches_host(shape):
    tex = np.random.default_rng(0).uniform(size=shape).astype(np.float32)
    levels = api.mip_pyramid(tex)
    pyr = M.mip_pyramid(t(tex)).cpu().numpy()
    flat = np.concatenate([lv.reshape(-1) for lv in levels[1:]]) if len(levels) > 1 else np.zeros(1, np.float32)
    assert same_bits(pyr[: flat.size], flat)


def masked(lod):
    # pixels whose level of detail sits within 1e-4 of an integer may pick the other level pair
    return np.abs(lod - np.rint(lod)) > 1e-4


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_sampling_and_adjoint_match_f64(mode):
    rng = np.random.default_rng(mode)
    tex, uv, da, raster = case(rng, h=48, w=64, th=70, tw=90, ch=4)
    ref, lod = api.texture_mip_forward(tex, uv, da, raster, mode)
    keep = masked(lod)
    addr = ["clamp", "wrap", "mirror"][mode]
    out = M.texture_mip(t(tex), t(uv), t(da), t(raster), address_mode=addr).cpu().numpy()
    assert np.abs(out - ref)[keep].max() < 1e-5
    g = rng.normal(size=uv.shape[:2] + (4,)).astype(np.float32) * keep[..., None]
    tt = t(tex).requires_grad_(True)
    tu = t(uv).requires_grad_(True)
    (M.texture_mip(tt, tu, t(da), t(raster), address_mode=addr) * t(g)).sum().backward()
    gt, gu = api.texture_mip_backward(tex, uv, da, raster, g, mode)
    gabs, _ = api.texture_mip_backward(tex, uv, da, raster, np.abs(g), mode)
    assert np.all(np.abs(tt.grad.cpu().numpy() - gt) <= 1e-5 * np.abs(gabs) + 1e-6)
    gu_got = tu.grad.cpu().numpy()
    assert np.all(np.abs(gu_got - gu) <= 2e-4 * np.maximum(np.abs(gu), 1.0))


def test_lod_zero_equals_bilinear(r):
    rng = np.random.default_rng(5)
    tex, uv, da, raster = case(rng)
    da[...] = 0.0
    lin = r.texture_forward(t(tex), t(uv), t(raster))
    mipped = M.texture_mip(t(tex), t(uv), t(da), t(raster))
    assert same_bits(lin.cpu().numpy(), mipped.cpu().numpy())


def test_render_chain_with_interpolated_derivatives(r):
    # rasterize -> interpolate uv -> uv_da from the barycentric derivatives -> trilinear texture
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(1)
    clip = t(S.clip_positions(pos3, mats)[0])
    uvv = S.spherical_uv(pos3).astype(np.float32)
    t_idx = t(idx.astype(np.int32))
    raster, deriv = pdr_torch.rasterize(clip, t_idx, (64, 80), rasterizer=r)
    uv = pdr_torch.interpolate(t(uvv), raster, t_idx, rasterizer=r)
    da = M.interpolate_derivatives(t(uvv), raster, deriv, t_idx, rasterizer=r)
    # the derivative of u along x equals the analytic expression from the barycentric derivatives
    rn, dn = raster.cpu().numpy(), deriv.cpu().numpy()
    ids = np.rint(rn[..., 3]).astype(np.int64)
    cov = ids > 0
    tri = idx[ids[cov] - 1]
    a0, a1, a2 = (uvv[tri[:, k]] for k in range(3))
    want_ux = dn[cov][:, 0] * (a0[:, 0] - a2[:, 0]) + dn[cov][:, 2] * (a1[:, 0] - a2[:, 0])
    assert np.allclose(da.cpu().numpy()[cov][:, 0], want_ux, rtol=1e-5, atol=1e-7)
    tex = t(np.random.default_rng(2).uniform(size=(256, 256, 4)).astype(np.float32)).requires_grad_(True)
    out = pdr_torch.texture(tex, uv, raster, rasterizer=r, filter_mode="linear-mipmap-linear", uv_da=da)
    out.sum().backward()
    assert tex.grad is not None and torch.isfinite(tex.grad).all()
    # a minified view: the sphere covers far fewer pixels than texels, so coarser levels are used
    lod = api.mip_lod32(da.cpu().numpy(), 256, 256, 9)
    assert lod[cov].max() > 1.0
    with pytest.raises(ValueError, match="uv_da"):
        pdr_torch.texture(tex, uv, raster, rasterizer=r, filter_mode="linear-mipmap-linear")

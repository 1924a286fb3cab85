"""Gradient through the barycentric pixel derivatives on the GPU (pdr_rasterize_backward_derivatives),
a capability the reference rejects (src/rasterizer.cpp:459-462): against the float64 adjoint of the
forward formula (oracle/api.py, itself checked by central differences), linear in the two upstream
gradients, and equal to the plain adjoint when the derivative gradient is zero."""
import numpy as np
import pytest
import torch

from oracle import api
from photara_drender_gb300 import Rasterizer
from photara_drender_gb300 import synthetic as S
from photara_drender_gb300 import torch as pdr_torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def r():
    return Rasterizer(0)


def scene(k=0, res=(72, 96)):
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(3)
    clip = S.clip_positions(pos3, mats)[k]
    return clip, idx, res


def within(gpu, f64, f32, fabs):
    """The adjoint subtracts nearly equal terms (d0x - b0 dA/dx, the 1/A^2 chain), so fp32 loses up to
    about 5e-5 of a component's magnitude against float64. Per component the GPU's error may be at most
    four times that of the same per-pixel arithmetic evaluated in fp32 on the host, plus 2e-6 of the
    sum of absolute contributions for the order of the atomic sums."""
    err = np.abs(gpu.astype(np.float64) - f64)
    bound = 4.0 * np.abs(f32 - f64) + 2e-6 * fabs + 1e-7 * np.abs(f64).max()
    return bool(np.all(err <= bound)), float((err / np.maximum(bound, 1e-30)).max())


@pytest.mark.parametrize("vp", [None, (4.0, -3.0, 80.0, 70.0)])
def test_derivative_gradient_matches_f64(r, vp):
    clip, idx, res = scene()
    rng = np.random.default_rng(1)
    raster, deriv = r.forward(clip, idx, res, viewport=vp)
    ref_deriv = api.barycentric_derivatives_f64(clip, idx, raster, vp)
    assert np.allclose(deriv, ref_deriv, rtol=1e-4, atol=1e-6 * np.abs(ref_deriv).max())
    gd = rng.normal(size=res + (4,)).astype(np.float32)
    zero = np.zeros_like(raster)
    got = r.backward(clip, idx, raster, zero, vp, grad_barycentric_derivatives=gd)
    f64 = api.barycentric_derivatives_backward_f64(clip, idx, raster, gd, vp)
    fabs = api.barycentric_derivatives_backward_f64(clip, idx, raster, gd, vp, abs_terms=True)
    f32 = api.barycentric_derivatives_backward_f64(clip, idx, raster, gd, vp, dtype=np.float32)
    ok, worst = within(got, f64, f32, fabs)
    assert ok, worst
    assert not got[:, 2].any()


def test_linear_and_plain_path_unchanged(r):
    clip, idx, res = scene(1)
    rng = np.random.default_rng(2)
    raster, _ = r.forward(clip, idx, res)
    gr = rng.normal(size=res + (4,)).astype(np.float32)
    gd = rng.normal(size=res + (4,)).astype(np.float32)
    plain = r.backward(clip, idx, raster, gr)
    # a zero derivative gradient adds nothing; the adjoint's atomic sums may round in another order
    zero_d = r.backward(clip, idx, raster, gr, grad_barycentric_derivatives=np.zeros_like(gd))
    assert np.abs(zero_d - plain).max() <= 1e-6 * np.abs(plain).max()
    only_d = r.backward(clip, idx, raster, np.zeros_like(gr), grad_barycentric_derivatives=gd)
    both = r.backward(clip, idx, raster, gr, grad_barycentric_derivatives=gd)
    scale = np.abs(plain).max() + np.abs(only_d).max()
    assert np.abs(both - (plain + only_d)).max() <= 1e-5 * scale
    with pytest.raises(ValueError, match="grad_barycentric_derivatives"):
        r.backward(clip, idx, raster, gr, grad_barycentric_derivatives=gd[:10])


def test_autograd_through_derivatives(r):
    clip, idx, res = scene(2)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(3)
    gd = torch.tensor(rng.normal(size=res + (4,)).astype(np.float32), device=dev)
    gu = torch.tensor(rng.normal(size=res + (4,)).astype(np.float32), device=dev)
    gu[..., 2:] = 0
    pos = torch.tensor(clip, device=dev, requires_grad=True)
    t_idx = torch.tensor(idx.astype(np.int32), device=dev)
    raster, deriv = pdr_torch.rasterize(pos, t_idx, res, rasterizer=r, differentiable_derivatives=True)
    ((raster * gu).sum() + (deriv * gd).sum()).backward()
    want = r.backward(pos.detach(), t_idx, raster.detach(), gu, grad_barycentric_derivatives=gd)
    assert torch.allclose(pos.grad, want, rtol=1e-5, atol=1e-6 * float(want.abs().max()))
    # by default the derivatives are constants, as in the reference
    pos2 = torch.tensor(clip, device=dev, requires_grad=True)
    _, deriv2 = pdr_torch.rasterize(pos2, t_idx, res, rasterizer=r)
    assert not deriv2.requires_grad

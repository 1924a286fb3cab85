"""Mipmapped (trilinear) texture sampling on the GPU (csrc/mip.cu): the filtering the reference lists
as planned (README.md:141). `texture(..., filter_mode="linear-mipmap-linear", uv_da=...)` in
photara_drender_gb300.torch uses it; `interpolate_derivatives` turns the raster's barycentric
derivatives into the pixel derivatives of interpolated attributes (uv_da for the uv attributes).

The pyramid is box filtered (level k+1 texel = mean of its 2x2 children, sides halved down to 1); the
level of detail is 0.5 log2 of the larger squared texel-space uv derivative; where it is <= 0 the result
equals bilinear sampling bit for bit. The level of detail is a constant of the adjoint: gradients reach
the texture (every level sampled, folded back to level 0) and uv, not uv_da.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import torch

from . import _native
from .rasterizer import ADDRESS_MODES, Rasterizer, _ptr

_NO_LIMIT = 0xFFFFFFFF


def _level_limit(max_mip_level: Optional[int]) -> int:
    if max_mip_level is None:
        return _NO_LIMIT
    if int(max_mip_level) < 0:
        raise ValueError("max_mip_level must be non-negative")
    return int(max_mip_level)


def pyramid_size(height: int, width: int, max_mip_level: Optional[int] = None) -> Tuple[int, int]:
    """(levels including level 0, texels of levels 1..)."""
    levels, texels = C.c_uint32(), C.c_uint64()
    _native.call("pdr_mip_pyramid_size", int(width), int(height), _level_limit(max_mip_level), C.byref(levels),
                 C.byref(texels))
    return levels.value, texels.value


def mip_pyramid(texture: torch.Tensor, max_mip_level: Optional[int] = None, stream=None) -> torch.Tensor:
    """Levels 1.. of texture [H, W, C] (CUDA, float32) as one flat buffer (level 0 stays the texture)."""
    h, w, ch = texture.shape
    _, texels = pyramid_size(h, w, max_mip_level)
    pyr = torch.empty(max(texels * ch, 1), dtype=torch.float32, device=texture.device)
    s = stream if stream is not None else C.c_void_p(torch.cuda.current_stream(texture.device).cuda_stream)
    _native.call("pdr_mip_build", _ptr(texture), w, h, ch, _level_limit(max_mip_level), _ptr(pyr), s)
    return pyr


def _check(texture, uv, uv_da, raster):
    if texture.dtype != torch.float32 or texture.ndim != 3:
        raise ValueError("texture_values must be float32 with shape [texture_height, texture_width, channels]")
    if uv.dtype != torch.float32 or uv.shape[-1] != 2 or uv.ndim not in (3, 4):
        raise ValueError("uv must be float32 with shape [image_height, image_width, 2]")
    if uv_da is None:
        raise ValueError("linear-mipmap-linear filtering needs uv_da (see interpolate_derivatives)")
    if uv_da.dtype != torch.float32 or uv_da.shape[:-1] != uv.shape[:-1] or uv_da.shape[-1] != 4:
        raise ValueError("uv_da must be float32 with shape [image_height, image_width, 4]")
    if raster.shape[:-1] != uv.shape[:-1] or raster.shape[-1] != 4:
        raise ValueError("uv and raster image dimensions must match")


class _TextureMipFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, texture, uv, uv_da, raster, address_mode, max_mip_level):
        _check(texture, uv, uv_da, raster)
        dev = texture.device
        tex = texture.detach().contiguous()
        uvc, dac, rc = (t.detach().to(dev).contiguous() for t in (uv, uv_da, raster))
        views = 1 if uvc.ndim == 3 else uvc.shape[0]
        P = uvc.shape[-3] * uvc.shape[-2]
        h, w, ch = tex.shape
        lim = _level_limit(max_mip_level)
        s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        pyr = mip_pyramid(tex, max_mip_level, s)
        out = torch.empty(uvc.shape[:-1] + (ch,), dtype=torch.float32, device=dev)
        _native.call("pdr_texture_forward_mip", _ptr(tex), _ptr(pyr), w, h, ch, lim, ADDRESS_MODES[address_mode],
                     _ptr(uvc), _ptr(dac), _ptr(rc), views, P, _ptr(out), s)
        ctx.save_for_backward(tex, pyr, uvc, dac, rc)
        ctx.meta = (w, h, ch, lim, ADDRESS_MODES[address_mode], views, P)
        return out

    @staticmethod
    def backward(ctx, grad_sampled):
        tex, pyr, uvc, dac, rc = ctx.saved_tensors
        w, h, ch, lim, mode, views, P = ctx.meta
        dev = tex.device
        g = grad_sampled.contiguous()
        grad_tex = torch.empty_like(tex)
        grad_pyr = torch.empty_like(pyr)
        grad_uv = torch.empty_like(uvc) if ctx.needs_input_grad[1] else None
        s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        _native.call("pdr_texture_backward_mip", _ptr(tex), _ptr(pyr), w, h, ch, lim, mode, _ptr(uvc), _ptr(dac),
                     _ptr(rc), views, P, _ptr(g), _ptr(grad_tex), _ptr(grad_pyr),
                     _ptr(grad_uv) if grad_uv is not None else None, s)
        return grad_tex, grad_uv, None, None, None, None


def texture_mip(texture: torch.Tensor, uv: torch.Tensor, uv_da: torch.Tensor, raster: torch.Tensor, *,
                address_mode: str = "clamp", max_mip_level: Optional[int] = None) -> torch.Tensor:
    """Trilinear sampling of texture [H, W, C] at uv [.., h, w, 2] with uv_da [.., h, w, 4]."""
    if address_mode not in ADDRESS_MODES:
        raise ValueError("address_mode must be 'clamp', 'wrap', or 'mirror'")
    return _TextureMipFunction.apply(texture, uv, uv_da, raster, address_mode, max_mip_level)


def interpolate_derivatives(vertex_attributes: torch.Tensor, raster: torch.Tensor,
                            barycentric_derivatives: torch.Tensor, indices: torch.Tensor, *,
                            rasterizer: Rasterizer) -> torch.Tensor:
    """Pixel derivatives of interpolated attributes, [.., h, w, 2A] = (da/dx, da/dy) per attribute (for uv:
    du/dx, du/dy, dv/dx, dv/dy), from the barycentric derivatives of `rasterize`. Not differentiable."""
    dev = rasterizer.context.device
    attrs = vertex_attributes.detach().to(dev, torch.float32).contiguous()
    if attrs.ndim != 2:
        raise ValueError("vertex_attributes must have shape [vertex_count, attribute_count]")
    r = raster.detach().to(dev).contiguous()
    d = barycentric_derivatives.detach().to(dev).contiguous()
    if d.shape != r.shape or r.shape[-1] != 4:
        raise ValueError("barycentric_derivatives must match the raster's shape")
    idx = indices.detach().to(dev, torch.int32).contiguous()
    views = 1 if r.ndim == 3 else r.shape[0]
    P = r.shape[-3] * r.shape[-2]
    A = attrs.shape[1]
    out = torch.empty(r.shape[:-1] + (2 * A,), dtype=torch.float32, device=dev)
    _native.call("pdr_interpolate_derivatives", _ptr(attrs), attrs.shape[0], A, _ptr(idx), idx.shape[0], _ptr(r),
                 _ptr(d), views, P, _ptr(out), rasterizer.context.stream())
    return out

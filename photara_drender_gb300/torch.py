"""PyTorch autograd adapter (python/photara_drender/torch.py:17-241) over the GB300 kernels.

CUDA tensors stay on the device end to end (the reference stages every call through host NumPy).
Every backward is the hand-written adjoint kernel of the matching forward. A leading view axis
is accepted: positions [B, V, 4] give rasters [B, H, W, 4].
"""
from __future__ import annotations

from typing import Optional, Sequence, Tuple

import torch

from .rasterizer import Rasterizer

_default_rasterizers: dict = {}


def _rasterizer_for(device_index: int, enable_validation: bool) -> Rasterizer:
    key = (device_index, enable_validation)
    if key not in _default_rasterizers:
        _default_rasterizers[key] = Rasterizer(device_index, enable_validation)
    return _default_rasterizers[key]


class _RasterizeFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, indices, resolution, rasterizer, cull_mode, output_barycentric_derivatives, viewport,
                recompute):
        if positions.dtype != torch.float32 or positions.ndim not in (2, 3) or positions.shape[-1] != 4:
            raise ValueError("positions must be a float32 tensor with shape [vertex_count, 4]")
        if indices.ndim != 2 or indices.shape[1] != 3:
            raise ValueError("indices must have shape [triangle_count, 3]")
        raster, derivatives = rasterizer.forward(positions.detach(), indices.detach(), resolution, cull_mode,
                                                 output_barycentric_derivatives, viewport)
        ctx.rasterizer = rasterizer
        ctx.viewport = viewport
        ctx.resolution = resolution
        ctx.cull_mode = cull_mode
        ctx.recompute = recompute
        if recompute:
            ctx.save_for_backward(positions.detach(), indices.detach())
        else:
            ctx.save_for_backward(positions.detach(), indices.detach(), raster.detach())
        ctx.mark_non_differentiable(derivatives)
        return raster, derivatives

    @staticmethod
    def backward(ctx, grad_raster, _grad_derivatives):
        if grad_raster is None:
            return (None,) * 8
        if ctx.recompute:
            positions, indices = ctx.saved_tensors
            raster, _ = ctx.rasterizer.forward(positions, indices, ctx.resolution, ctx.cull_mode, False, ctx.viewport)
        else:
            positions, indices, raster = ctx.saved_tensors
        grad_positions = ctx.rasterizer.backward(positions, indices, raster, grad_raster.contiguous(), ctx.viewport)
        return grad_positions, None, None, None, None, None, None, None


class _InterpolateFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vertex_attributes, raster, indices, rasterizer):
        if vertex_attributes.dtype != torch.float32 or vertex_attributes.ndim not in (2, 3):
            raise ValueError("vertex_attributes must be a float32 tensor with shape [vertex_count, attribute_count]")
        if raster.dtype != torch.float32 or raster.ndim not in (3, 4) or raster.shape[-1] != 4:
            raise ValueError("raster must be a float32 tensor with shape [height, width, 4]")
        if indices.ndim != 2 or indices.shape[1] != 3:
            raise ValueError("indices must have shape [triangle_count, 3]")
        if vertex_attributes.device != raster.device:
            raise ValueError("vertex_attributes and raster must be on the same device")
        out = rasterizer.interpolate_forward(vertex_attributes.detach(), indices.detach(), raster.detach())
        ctx.rasterizer = rasterizer
        ctx.save_for_backward(vertex_attributes.detach(), raster.detach(), indices.detach())
        return out

    @staticmethod
    def backward(ctx, grad_interpolated):
        attributes, raster, indices = ctx.saved_tensors
        grad_attributes, grad_raster = ctx.rasterizer.interpolate_backward(attributes, indices, raster,
                                                                           grad_interpolated.contiguous())
        return grad_attributes, grad_raster, None, None


class _TextureFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, texture_values, uv, raster, rasterizer, address_mode):
        if texture_values.dtype != torch.float32 or texture_values.ndim not in (3, 4):
            raise ValueError("texture_values must be float32 with shape [texture_height, texture_width, channels]")
        if uv.dtype != torch.float32 or uv.ndim not in (3, 4) or uv.shape[-1] != 2:
            raise ValueError("uv must be float32 with shape [image_height, image_width, 2]")
        if raster.dtype != torch.float32 or raster.ndim not in (3, 4) or raster.shape[-1] != 4:
            raise ValueError("raster must be float32 with shape [image_height, image_width, 4]")
        if uv.shape[:-1] != raster.shape[:-1]:
            raise ValueError("uv and raster image dimensions must match")
        if texture_values.device != uv.device or uv.device != raster.device:
            raise ValueError("texture_values, uv, and raster must be on the same device")
        out = rasterizer.texture_forward(texture_values.detach(), uv.detach(), raster.detach(), address_mode)
        ctx.rasterizer = rasterizer
        ctx.address_mode = address_mode
        ctx.save_for_backward(texture_values.detach(), uv.detach(), raster.detach())
        return out

    @staticmethod
    def backward(ctx, grad_sampled):
        texture_values, uv, raster = ctx.saved_tensors
        grad_texture, grad_uv = ctx.rasterizer.texture_backward(texture_values, uv, raster, grad_sampled.contiguous(),
                                                                ctx.address_mode, bool(ctx.needs_input_grad[1]))
        return grad_texture, grad_uv, None, None, None


def rasterize(positions: torch.Tensor, indices: torch.Tensor, resolution: Sequence[int], *,
              rasterizer: Optional[Rasterizer] = None, device_index: int = 0, enable_validation: bool = False,
              cull_mode: str = "none", output_barycentric_derivatives: bool = True,
              viewport: Optional[Sequence[float]] = None, recompute_in_backward: bool = False
              ) -> Tuple[torch.Tensor, torch.Tensor]:
    """Rasterize clip-space vertices and connect the output to autograd (torch.py:181-216).

    Resolution uses ``(height, width)`` order. ``recompute_in_backward`` keeps only positions and
    indices for the backward pass and rasterizes again there, instead of holding the raster."""
    if len(resolution) != 2 or int(resolution[0]) <= 0 or int(resolution[1]) <= 0:
        raise ValueError("resolution must be (height, width) with positive values")
    active = rasterizer or _rasterizer_for(device_index, enable_validation)
    normalized_viewport = None
    if viewport is not None:
        if len(viewport) == 4 and not isinstance(viewport[0], (list, tuple)):
            normalized_viewport = tuple(float(v) for v in viewport)
        else:
            normalized_viewport = [None if v is None else tuple(float(x) for x in v) for v in viewport]
    return _RasterizeFunction.apply(positions, indices, (int(resolution[0]), int(resolution[1])), active, cull_mode,
                                    output_barycentric_derivatives, normalized_viewport, recompute_in_backward)


def interpolate(vertex_attributes: torch.Tensor, raster: torch.Tensor, indices: torch.Tensor, *,
                rasterizer: Rasterizer) -> torch.Tensor:
    """Interpolate vertex attributes and propagate gradients to attributes and raster (torch.py:219-228)."""
    return _InterpolateFunction.apply(vertex_attributes, raster, indices, rasterizer)


def texture(texture_values: torch.Tensor, uv: torch.Tensor, raster: torch.Tensor, *, rasterizer: Rasterizer,
            address_mode: str = "clamp") -> torch.Tensor:
    """Sample a texture bilinearly and propagate gradients to texels and UV coordinates (torch.py:231-241)."""
    return _TextureFunction.apply(texture_values, uv, raster, rasterizer, address_mode)

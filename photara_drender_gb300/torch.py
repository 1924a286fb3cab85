"""PyTorch autograd adapter (python/photara_drender/torch.py:17-241) over the GB300 kernels.

CUDA tensors stay on the device end to end (the reference stages every call through host NumPy).
Every backward is the hand-written adjoint kernel of the matching forward. A leading view axis
is accepted: positions [B, V, 4] give rasters [B, H, W, 4].
"""
from __future__ import annotations

import ctypes as C
from typing import NamedTuple, Optional, Sequence, Tuple

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
                recompute, differentiable_derivatives=False, clip_near_plane=False):
        if positions.dtype != torch.float32 or positions.ndim not in (2, 3) or positions.shape[-1] != 4:
            raise ValueError("positions must be a float32 tensor with shape [vertex_count, 4]")
        if indices.ndim != 2 or indices.shape[1] != 3:
            raise ValueError("indices must have shape [triangle_count, 3]")
        raster, derivatives = rasterizer.forward(positions.detach(), indices.detach(), resolution, cull_mode,
                                                 output_barycentric_derivatives, viewport,
                                                 clip_near_plane=clip_near_plane)
        ctx.rasterizer = rasterizer
        ctx.clip_near_plane = clip_near_plane
        ctx.viewport = viewport
        ctx.resolution = resolution
        ctx.cull_mode = cull_mode
        ctx.recompute = recompute
        ctx.differentiable_derivatives = bool(differentiable_derivatives and output_barycentric_derivatives)
        if recompute:
            ctx.save_for_backward(positions.detach(), indices.detach())
        else:
            ctx.save_for_backward(positions.detach(), indices.detach(), raster.detach())
        if not ctx.differentiable_derivatives:
            ctx.mark_non_differentiable(derivatives)
        return raster, derivatives

    @staticmethod
    def backward(ctx, grad_raster, grad_derivatives):
        use_deriv = ctx.differentiable_derivatives and grad_derivatives is not None
        if grad_raster is None and not use_deriv:
            return (None,) * 10
        if ctx.recompute:
            positions, indices = ctx.saved_tensors
            raster, _ = ctx.rasterizer.forward(positions, indices, ctx.resolution, ctx.cull_mode, False, ctx.viewport,
                                               clip_near_plane=ctx.clip_near_plane)
        else:
            positions, indices, raster = ctx.saved_tensors
        if grad_raster is None:
            grad_raster = torch.zeros_like(raster)
        grad_positions = ctx.rasterizer.backward(
            positions, indices, raster, grad_raster.contiguous(), ctx.viewport,
            grad_barycentric_derivatives=grad_derivatives.contiguous() if use_deriv else None,
            clip_near_plane=ctx.clip_near_plane)
        return grad_positions, None, None, None, None, None, None, None, None, None


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
              viewport: Optional[Sequence[float]] = None, recompute_in_backward: bool = False,
              differentiable_derivatives: bool = False,
              clip_near_plane: bool = False) -> Tuple[torch.Tensor, torch.Tensor]:
    """Rasterize clip-space vertices and connect the output to autograd (torch.py:181-216).

    Resolution uses ``(height, width)`` order. ``recompute_in_backward`` keeps only positions and
    indices for the backward pass and rasterizes again there, instead of holding the raster.
    ``differentiable_derivatives`` makes the barycentric derivative output differentiable (its gradient
    reaches the positions); by default it is a constant, as in the reference. ``clip_near_plane`` clips
    triangles against the near plane before rasterizing (the reference drops triangles with a vertex at
    w <= 1e-8 instead); outputs and gradients refer to the original triangles."""
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
                                    output_barycentric_derivatives, normalized_viewport, recompute_in_backward,
                                    differentiable_derivatives, clip_near_plane)


def interpolate(vertex_attributes: torch.Tensor, raster: torch.Tensor, indices: torch.Tensor, *,
                rasterizer: Rasterizer) -> torch.Tensor:
    """Interpolate vertex attributes and propagate gradients to attributes and raster (torch.py:219-228)."""
    return _InterpolateFunction.apply(vertex_attributes, raster, indices, rasterizer)


def texture(texture_values: torch.Tensor, uv: torch.Tensor, raster: torch.Tensor, *, rasterizer: Rasterizer,
            address_mode: str = "clamp", filter_mode: str = "linear", uv_da: Optional[torch.Tensor] = None,
            max_mip_level: Optional[int] = None) -> torch.Tensor:
    """Sample a texture bilinearly and propagate gradients to texels and UV coordinates (torch.py:231-241).

    ``filter_mode="linear-mipmap-linear"`` samples a box-filtered mip pyramid trilinearly instead, with the
    level of detail from ``uv_da`` (du/dx, du/dy, dv/dx, dv/dy per pixel; ``mip.interpolate_derivatives``
    makes it from the raster's barycentric derivatives). The reference has only bilinear sampling."""
    if filter_mode == "linear":
        return _TextureFunction.apply(texture_values, uv, raster, rasterizer, address_mode)
    if filter_mode == "linear-mipmap-linear":
        from .mip import texture_mip

        return texture_mip(texture_values, uv, uv_da, raster, address_mode=address_mode, max_mip_level=max_mip_level)
    raise ValueError("filter_mode must be 'linear' or 'linear-mipmap-linear'")


# ---- fused rasterize -> interpolate -> texture ---------------------------------------------------------

class RenderOutput(NamedTuple):
    raster: torch.Tensor          # [B, H, W, 4] (or [H, W, 4] for unbatched positions)
    derivatives: torch.Tensor     # [B, H, W, 4]
    interpolated: Optional[torch.Tensor]  # [B, H, W, A] when vertex_attributes were given
    uv: Optional[torch.Tensor]    # [B, H, W, 2] when vertex_uv was given
    sampled: Optional[torch.Tensor]       # [B, H, W, 4] when a texture was given


_MODES = {"none": 0, "back": 1, "front": 2}
_ADDRESS = {"clamp": 0, "wrap": 1, "mirror": 2}


def _apply_status(r: Rasterizer, reports) -> None:
    """Acts on status blocks of earlier calls that did not wait for their work: grows the tile-list
    capacity to what the binning needed, raises the errors the device recorded."""
    from . import _native

    for kind, st in reports:
        if kind == "render_forward":
            if st[_native.STATUS_TILE_ENTRIES_HI] != 0:
                raise OverflowError("Tile triangle list exceeds backend limits")
            total = st[_native.STATUS_TILE_ENTRIES] & 0xFFFFFFFF
            r._render_capacity = max(getattr(r, "_render_capacity", 0), total + total // 8 + 1024)
        elif st[_native.STATUS_TEXEL_ERROR] == 1:
            raise ValueError("uv contains a non-finite value in a covered pixel")
        elif st[_native.STATUS_TEXEL_ERROR] == 2:
            raise IndexError("uv is too large for portable texture addressing")


def _cached_viewports(r: Rasterizer, viewport, views: int, w: int, h: int) -> torch.Tensor:
    """The device viewport rows of render calls, kept per (viewport, views, size) on the rasterizer: an
    upload from pageable host memory is not allowed inside a CUDA graph capture, so a captured call
    reuses the rows an earlier call made."""
    from .rasterizer import _viewports

    try:
        key = (views, w, h, None if viewport is None else tuple(
            tuple(float(x) for x in v) if isinstance(v, (list, tuple)) else float(v) for v in viewport))
    except TypeError:
        key = None
    cache = r.__dict__.setdefault("_render_viewports", {})
    if key is not None and key in cache:
        return cache[key]
    vps, _ = _viewports(viewport, views, w, h, r.context.device)
    if key is not None:
        cache[key] = vps
    return vps


def check_deferred_errors(rasterizer: Rasterizer) -> None:
    """Waits for every `render(..., deferred_errors=True)` call made on this rasterizer and raises the
    first error the device recorded for them (ValueError / IndexError / OverflowError, as the
    synchronous path raises at once)."""
    with rasterizer.context.lock:
        _apply_status(rasterizer, rasterizer.context.poll_status(wait=True, kinds=("render_forward",
                                                                                   "render_backward")))


def _render_forward(r: Rasterizer, clip, idx, h, w, attrs, uv_attrs, tex, vps, cull, mode, deferred=False):
    from . import _native
    from .pipeline import RenderArgsC
    from .rasterizer import TILE, _ptr

    ctx = r.context
    dev = ctx.device
    views, V = clip.shape[0], clip.shape[1]
    T = idx.shape[0]
    # tile shape and stage depth of the fused binning and raster (pipeline.TILE_CONFIGS; outputs do not
    # depend on it): the rasterizer's render_tile_config, e.g. one RenderFwdBwd.autotune picked
    tw_, th_, stage = getattr(r, "render_tile_config", (TILE, TILE, 256))
    tiles = ((w + tw_ - 1) // tw_) * ((h + th_ - 1) // th_)
    f = dict(dtype=torch.float32, device=dev)
    out = dict(raster=torch.empty((views, h, w, 4), **f), deriv=torch.empty((views, h, w, 4), **f),
               interp=torch.empty((views, h, w, attrs.shape[1]), **f) if attrs is not None else None,
               uv=torch.empty((views, h, w, 2), **f) if uv_attrs is not None else None,
               sampled=torch.empty((views, h, w, 4), **f) if tex is not None else None,
               # texel differences of each covered pixel's sample, kept for the backward (32 B per pixel)
               sdiff=torch.empty((views, h, w, 8), **f) if tex is not None else None)
    offsets = torch.empty(views * tiles + 1, dtype=torch.int32, device=dev)
    _apply_status(r, ctx.poll_status(kinds=("render_forward", "render_backward")))
    capacity = max(getattr(r, "_render_capacity", 0), 2 * T * views + 1024)
    L = _native.lib()
    for _ in range(1 if deferred else 3):
        lst = torch.empty(capacity, dtype=torch.int32, device=dev)
        ws_bytes = L.pdr_render_workspace_bytes_tiled(views, T, w, h, capacity, tw_, th_)
        ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
        ctx.status.zero_()
        a = RenderArgsC()
        a.clip_positions, a.views, a.vertex_count = clip.data_ptr(), views, V
        a.indices, a.triangle_count, a.width, a.height = idx.data_ptr(), T, w, h
        a.viewports, a.cull_mode = vps.data_ptr(), cull
        if attrs is not None:
            a.attributes, a.attribute_count, a.interpolated = attrs.data_ptr(), attrs.shape[1], out["interp"].data_ptr()
        if uv_attrs is not None:
            a.uv_attributes, a.uv = uv_attrs.data_ptr(), out["uv"].data_ptr()
        if tex is not None:
            a.texture, a.texture_width, a.texture_height = tex.data_ptr(), tex.shape[1], tex.shape[0]
            a.address_mode, a.sampled = mode, out["sampled"].data_ptr()
            a.sample_differences = out["sdiff"].data_ptr()
        a.tile_offsets, a.tile_triangles, a.capacity = offsets.data_ptr(), lst.data_ptr(), capacity
        a.workspace, a.workspace_bytes, a.status = ws.data_ptr(), ws_bytes, ctx.status.data_ptr()
        a.raster, a.barycentric_derivatives = out["raster"].data_ptr(), out["deriv"].data_ptr()
        a.tile_width, a.tile_height, a.stage_triangles = tw_, th_, stage
        _native.check(L.pdr_render_forward(C.addressof(a), ctx.stream()))
        if deferred:
            # No wait: a tile whose list overflowed the capacity is rasterized from all triangles with the
            # binning rule (same result, slower); the entry count reaches the host later and sizes the
            # capacity of the next calls.
            ctx.defer_status("render_forward")
            return out
        st = ctx.status.cpu()
        total = int(st[_native.STATUS_TILE_ENTRIES]) & 0xFFFFFFFF
        if int(st[_native.STATUS_TILE_ENTRIES_HI]) != 0:
            raise OverflowError("Tile triangle list exceeds backend limits")
        if not int(st[_native.STATUS_TILE_OVERFLOW]):
            r._render_capacity = max(getattr(r, "_render_capacity", 0), total + total // 8 + 1024)
            return out
        capacity = total + total // 8 + 1024
    raise RuntimeError("tile binning did not converge")


class _RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, vertex_attributes, vertex_uv, texture_values, indices, resolution, rasterizer,
                viewport, cull_mode, address_mode, deferred_errors):
        from .rasterizer import _viewports

        r = rasterizer
        deferred = bool(deferred_errors) or torch.cuda.is_current_stream_capturing()
        with r.context.lock:
            clip = positions.detach()
            batched = clip.ndim == 3
            clip = (clip if batched else clip.unsqueeze(0)).contiguous()
            idx = indices.detach().to(r.context.device, torch.int32).contiguous()
            h, w = int(resolution[0]), int(resolution[1])
            vps = _cached_viewports(r, viewport, clip.shape[0], w, h)
            attrs = vertex_attributes.detach().contiguous() if vertex_attributes is not None else None
            uva = vertex_uv.detach().contiguous() if vertex_uv is not None else None
            tex = texture_values.detach().contiguous() if texture_values is not None else None
            out = _render_forward(r, clip, idx, h, w, attrs, uva, tex, vps, _MODES[cull_mode], _ADDRESS[address_mode],
                                  deferred)
        ctx.r, ctx.vps, ctx.batched, ctx.viewport = r, vps, batched, viewport
        ctx.deferred = deferred
        ctx.mode = _ADDRESS[address_mode]
        # outputs the loss does not use get no gradient (None), not a zero tensor: a zero raster or uv
        # gradient would otherwise run the separate adjoints over every pixel for nothing
        ctx.set_materialize_grads(False)
        ctx.save_for_backward(clip, idx, attrs, uva, tex, out["raster"], out["uv"], out["sdiff"])
        squeeze = (lambda t: t) if batched else (lambda t: t[0] if t is not None else None)
        result = (squeeze(out["raster"]), squeeze(out["deriv"]), squeeze(out["interp"]), squeeze(out["uv"]),
                  squeeze(out["sampled"]))
        ctx.mark_non_differentiable(result[1])
        return result

    @staticmethod
    def backward(ctx, g_raster, _g_deriv, g_interp, g_uv, g_sampled):
        from . import _native
        from .pipeline import RenderArgsC

        clip, idx, attrs, uva, tex, raster, uv_out, sdiff = ctx.saved_tensors
        r = ctx.r
        unb = (lambda t: t) if ctx.batched else (lambda t: t.unsqueeze(0) if t is not None else None)
        g_raster, g_interp, g_uv, g_sampled = unb(g_raster), unb(g_interp), unb(g_uv), unb(g_sampled)
        views, V = clip.shape[0], clip.shape[1]
        dev = clip.device
        f = dict(dtype=torch.float32, device=dev)
        grad_clip = torch.empty((views, V, 4), **f)
        grad_attr = torch.empty_like(attrs) if attrs is not None else None
        grad_uv = torch.empty_like(uva) if uva is not None else None
        grad_tex = torch.empty_like(tex) if tex is not None else None
        with r.context.lock:
            a = RenderArgsC()
            a.clip_positions, a.views, a.vertex_count = clip.data_ptr(), views, V
            a.indices, a.triangle_count = idx.data_ptr(), idx.shape[0]
            a.width, a.height = raster.shape[2], raster.shape[1]
            a.viewports, a.raster = ctx.vps.data_ptr(), raster.data_ptr()
            keep = []
            if attrs is not None:
                gi = g_interp.contiguous() if g_interp is not None else torch.zeros(
                    (views,) + tuple(raster.shape[1:3]) + (attrs.shape[1],), **f)
                keep.append(gi)
                a.attributes, a.attribute_count = attrs.data_ptr(), attrs.shape[1]
                a.grad_interpolated, a.grad_attributes = gi.data_ptr(), grad_attr.data_ptr()
            if uva is not None:
                a.uv_attributes, a.uv, a.grad_uv_attributes = uva.data_ptr(), uv_out.data_ptr(), grad_uv.data_ptr()
            if tex is not None:
                gs = g_sampled.contiguous() if g_sampled is not None else torch.zeros_like(raster)
                keep.append(gs)
                a.texture, a.texture_width, a.texture_height, a.address_mode = (tex.data_ptr(), tex.shape[1],
                                                                                tex.shape[0], ctx.mode)
                a.grad_sampled, a.grad_texture = gs.data_ptr(), grad_tex.data_ptr()
                a.sample_differences = sdiff.data_ptr()
            a.grad_clip_positions, a.status = grad_clip.data_ptr(), r.context.status.data_ptr()
            # per-view vertex-gradient records for the adjoint (16-byte reductions, summed over the views after)
            ws_bytes = _native.lib().pdr_render_backward_workspace_bytes(
                views, V, attrs.shape[1] if attrs is not None else 0)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
            a.workspace, a.workspace_bytes = ws.data_ptr(), ws_bytes
            deferred = ctx.deferred or torch.cuda.is_current_stream_capturing()
            _apply_status(r, r.context.poll_status(kinds=("render_forward", "render_backward")))
            r.context.status.zero_()
            _native.check(_native.lib().pdr_render_backward(C.addressof(a), r.context.stream()))
            if deferred:
                r.context.defer_status("render_backward")
            else:
                st = r.context.status.cpu()
                if int(st[_native.STATUS_TEXEL_ERROR]) == 1:
                    raise ValueError("uv contains a non-finite value in a covered pixel")
                if int(st[_native.STATUS_TEXEL_ERROR]) == 2:
                    raise IndexError("uv is too large for portable texture addressing")
        # upstream gradients on the raster or uv outputs themselves go through the separate adjoints
        extra = g_raster.contiguous() if g_raster is not None else None
        if g_uv is not None and uva is not None:
            gua, gr = r.interpolate_backward(uva, idx, raster, g_uv.contiguous())
            grad_uv = grad_uv + gua
            extra = gr if extra is None else extra + gr
        if extra is not None:
            grad_clip = grad_clip + r.backward(clip, idx, raster, extra.contiguous(), ctx.viewport)
        if not ctx.batched:
            grad_clip = grad_clip[0]
        return grad_clip, grad_attr, grad_uv, grad_tex, None, None, None, None, None, None, None


def render(positions: torch.Tensor, indices: torch.Tensor, resolution: Sequence[int], *, rasterizer: Rasterizer,
           vertex_attributes: Optional[torch.Tensor] = None, vertex_uv: Optional[torch.Tensor] = None,
           texture: Optional[torch.Tensor] = None, viewport=None, cull_mode: str = "none",
           address_mode: str = "clamp", deferred_errors: bool = False) -> RenderOutput:
    """rasterize -> interpolate(vertex_attributes), interpolate(vertex_uv) -> texture in one fused forward
    kernel and one fused backward kernel: the outputs of `rasterize`, two `interpolate` calls and `texture`,
    bit-identical to them, with the same gradients. vertex_attributes [V, A] (A <= 8) and vertex_uv [V, 2]
    are shared by all views; the texture is [H, W, 4] and needs vertex_uv.

    By default each forward and backward waits for its kernels to check the device status (tile-list
    capacity, non-finite or out-of-range uv) and raises at once, as the separate calls do. With
    deferred_errors=True (and always inside a CUDA graph capture) neither waits: the host can run ahead
    of the GPU and the pass can be captured. A tile-list overflow then costs time, not correctness (the
    tiles concerned rasterize from all triangles with the binning rule), and errors the device records
    are raised by a later call on the same rasterizer, or by check_deferred_errors(rasterizer)."""
    if positions.dtype != torch.float32 or positions.ndim not in (2, 3) or positions.shape[-1] != 4:
        raise ValueError("positions must be a float32 tensor with shape [vertex_count, 4]")
    if indices.ndim != 2 or indices.shape[1] != 3:
        raise ValueError("indices must have shape [triangle_count, 3]")
    if cull_mode not in _MODES:
        raise ValueError("cull_mode must be 'none', 'back', or 'front'")
    if address_mode not in _ADDRESS:
        raise ValueError("address_mode must be 'clamp', 'wrap', or 'mirror'")
    V = positions.shape[-2]
    if vertex_attributes is not None and (vertex_attributes.ndim != 2 or vertex_attributes.shape[0] != V
                                          or not 1 <= vertex_attributes.shape[1] <= 8):
        raise ValueError("vertex_attributes must have shape [vertex_count, 1..8]")
    if vertex_uv is not None and tuple(vertex_uv.shape) != (V, 2):
        raise ValueError("vertex_uv must have shape [vertex_count, 2]")
    if texture is not None and (vertex_uv is None or texture.ndim != 3 or texture.shape[2] != 4):
        raise ValueError("texture must have shape [height, width, 4] and needs vertex_uv")
    return RenderOutput(*_RenderFunction.apply(positions, vertex_attributes, vertex_uv, texture, indices,
                                               tuple(resolution), rasterizer, viewport, cull_mode, address_mode,
                                               deferred_errors))

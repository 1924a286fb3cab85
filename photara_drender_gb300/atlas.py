"""Differentiable texture-atlas rendering and optimisation helpers
(python/photara_drender/atlas.py:36-257), on the GB300 rasterize/interpolate/texture kernels.

The losses are the reference's research objective. optimize_texture_atlas runs it on the native refiner
kernels when the atlas is RGB float32 with clamp addressing and no prior term: per step one view's masked
Charbonnier gradient (pdr_refine_photometric), the chart-aware TV (pdr_refine_total_variation) and the
seam term (pdr_refine_seam) into one gradient buffer, then the Adam update with the clamp
(pdr_refine_adam, torch.optim.Adam's arithmetic), with the loss history read back once at the end.
Other cases run the same objective as torch tensor ops over the CUDA renderer
(photara_drender_gb300.torch). For the reference's native refinement (one CUDA graph for the whole
optimisation) see TextureBaker.refine_texture.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, NamedTuple, Optional, Sequence, Tuple

import torch

from . import _native
from .rasterizer import Rasterizer, _ptr
from .torch import interpolate, rasterize, render, texture as sample_texture


class TexturedRender(NamedTuple):
    image: torch.Tensor
    valid_mask: torch.Tensor
    raster: torch.Tensor
    barycentric_derivatives: torch.Tensor
    uv: torch.Tensor


@dataclass(frozen=True)
class AtlasOptimizationOptions:
    """atlas.py:22-33"""

    steps: int = 150
    learning_rate: float = 1e-2
    photometric_epsilon: float = 1e-3
    total_variation_weight: float = 1e-4
    seam_weight: float = 1e-3
    initial_prior_weight: float = 0.0
    address_mode: str = "clamp"
    clamp_min: float = 0.0
    clamp_max: float = 1.0
    cache_view_rasters: bool = False


def render_textured_mesh(clip_positions: torch.Tensor, indices: torch.Tensor, vertex_uv: torch.Tensor,
                         texture_values: torch.Tensor, resolution: Sequence[int], *, rasterizer: Rasterizer,
                         viewport: Optional[Sequence[float]] = None, cull_mode: str = "none",
                         address_mode: str = "clamp") -> TexturedRender:
    """atlas.py:36-62: rasterize -> interpolate uv -> texture, keeping the intermediates. A 4-channel
    texture takes the fused forward / backward kernels (same outputs and gradients)."""
    if texture_values.ndim == 3 and texture_values.shape[2] == 4 and texture_values.dtype == torch.float32:
        out = render(clip_positions, indices, resolution, rasterizer=rasterizer, vertex_uv=vertex_uv,
                     texture=texture_values, viewport=viewport, cull_mode=cull_mode, address_mode=address_mode)
        valid_mask = (out.raster[..., 3:4] > 0).to(dtype=out.sampled.dtype)
        return TexturedRender(out.sampled, valid_mask, out.raster, out.derivatives, out.uv)
    raster, derivatives = rasterize(clip_positions, indices, resolution, rasterizer=rasterizer, viewport=viewport,
                                    cull_mode=cull_mode, output_barycentric_derivatives=True)
    uv = interpolate(vertex_uv, raster, indices, rasterizer=rasterizer)
    image = sample_texture(texture_values, uv, raster, rasterizer=rasterizer, address_mode=address_mode)
    valid_mask = (raster[..., 3:4] > 0).to(dtype=image.dtype)
    return TexturedRender(image, valid_mask, raster, derivatives, uv)


def masked_charbonnier_loss(rendered: torch.Tensor, target: torch.Tensor, valid_mask: torch.Tensor, *,
                            epsilon: float = 1e-3) -> torch.Tensor:
    """atlas.py:65-81: mean of sqrt(d^2 + eps^2) over valid pixels and channels."""
    if rendered.shape != target.shape:
        raise ValueError("rendered and target must have the same shape")
    if valid_mask.shape != rendered.shape[:-1] + (1,):
        raise ValueError("valid_mask must have shape [height, width, 1]")
    robust = torch.sqrt((rendered - target).square() + epsilon * epsilon)
    return (robust * valid_mask).sum() / (valid_mask.sum().clamp_min(1.0) * rendered.shape[-1])


def atlas_total_variation(texture_values: torch.Tensor, *, valid_mask: Optional[torch.Tensor] = None,
                          chart_ids: Optional[torch.Tensor] = None, epsilon: float = 1e-4) -> torch.Tensor:
    """atlas.py:84-115: robust total variation over valid neighbour pairs inside one chart."""
    if texture_values.ndim != 3:
        raise ValueError("texture_values must have shape [height, width, channels]")
    height, width = texture_values.shape[:2]
    if valid_mask is None:
        valid = torch.ones((height, width), dtype=torch.bool, device=texture_values.device)
    else:
        valid = valid_mask.to(device=texture_values.device, dtype=torch.bool)
    if valid.shape != (height, width):
        raise ValueError("valid_mask must have shape [texture_height, texture_width]")
    if chart_ids is not None and chart_ids.shape != (height, width):
        raise ValueError("chart_ids must have shape [texture_height, texture_width]")
    pair_h = valid[:, 1:] & valid[:, :-1]
    pair_v = valid[1:, :] & valid[:-1, :]
    if chart_ids is not None:
        ids = chart_ids.to(device=texture_values.device)
        pair_h = pair_h & (ids[:, 1:] == ids[:, :-1])
        pair_v = pair_v & (ids[1:, :] == ids[:-1, :])
    dh = torch.sqrt((texture_values[:, 1:] - texture_values[:, :-1]).square() + epsilon * epsilon)
    dv = torch.sqrt((texture_values[1:, :] - texture_values[:-1, :]).square() + epsilon * epsilon)
    total = (dh * pair_h[..., None]).sum() + (dv * pair_v[..., None]).sum()
    pairs = pair_h.sum() + pair_v.sum()
    return total / (pairs.clamp_min(1) * texture_values.shape[-1])


def seam_consistency_loss(texture_values: torch.Tensor, seam_uv_pairs: torch.Tensor, *, rasterizer: Rasterizer,
                          address_mode: str = "clamp", epsilon: float = 1e-4) -> torch.Tensor:
    """atlas.py:118-144: Charbonnier difference of the texture sampled at both sides of each seam pair."""
    if seam_uv_pairs.ndim != 3 or tuple(seam_uv_pairs.shape[1:]) != (2, 2):
        raise ValueError("seam_uv_pairs must have shape [seam_count, 2, 2]")
    count = seam_uv_pairs.shape[0]
    if count == 0:
        return texture_values.sum() * 0.0
    uv = seam_uv_pairs.reshape(1, count * 2, 2).contiguous()
    covered = torch.zeros((1, count * 2, 4), dtype=torch.float32, device=texture_values.device)
    covered[..., 3] = 1.0
    colors = sample_texture(texture_values, uv, covered, rasterizer=rasterizer, address_mode=address_mode)
    colors = colors.reshape(count, 2, texture_values.shape[-1])
    difference = colors[:, 0] - colors[:, 1]
    return torch.sqrt(difference.square() + epsilon * epsilon).mean()


def optimize_texture_atlas(initial_texture: torch.Tensor, clip_positions_by_view: torch.Tensor, indices: torch.Tensor,
                           vertex_uv: torch.Tensor, target_images: Sequence[torch.Tensor], *, rasterizer: Rasterizer,
                           viewports: Optional[Sequence[Optional[Sequence[float]]]] = None,
                           visibility_masks: Optional[Sequence[Optional[torch.Tensor]]] = None,
                           atlas_valid_mask: Optional[torch.Tensor] = None, chart_ids: Optional[torch.Tensor] = None,
                           seam_uv_pairs: Optional[torch.Tensor] = None,
                           options: AtlasOptimizationOptions = AtlasOptimizationOptions()
                           ) -> Tuple[torch.Tensor, List[float]]:
    """atlas.py:147-257: torch.optim.Adam over the atlas, one view per step in round-robin order.

    ``clip_positions_by_view`` has shape ``[view_count, vertex_count, 4]``."""
    if clip_positions_by_view.ndim != 3 or clip_positions_by_view.shape[2] != 4:
        raise ValueError("clip_positions_by_view must have shape [view_count, vertex_count, 4]")
    view_count = clip_positions_by_view.shape[0]
    if len(target_images) != view_count or view_count == 0:
        raise ValueError("target_images must contain one image per view")
    viewports = [None] * view_count if viewports is None else viewports
    visibility_masks = [None] * view_count if visibility_masks is None else visibility_masks
    if len(viewports) != view_count or len(visibility_masks) != view_count:
        raise ValueError("viewports and visibility_masks must match the view count")
    if options.steps <= 0 or options.learning_rate <= 0:
        raise ValueError("optimization steps and learning_rate must be positive")
    if _native_path_applies(initial_texture, target_images, options):
        return _optimize_native(initial_texture, clip_positions_by_view, indices, vertex_uv, target_images,
                                rasterizer, viewports, visibility_masks, atlas_valid_mask, chart_ids, seam_uv_pairs,
                                options)
    parameter = torch.nn.Parameter(initial_texture.detach().clone())
    initial = initial_texture.detach().clone()
    optimizer = torch.optim.Adam([parameter], lr=options.learning_rate)
    history: List[float] = []
    cache: dict = {}
    for step in range(options.steps):
        optimizer.zero_grad(set_to_none=True)
        k = step % view_count
        target = target_images[k]
        if k in cache:
            raster, uv, valid_mask = cache[k]
            image = sample_texture(parameter, uv, raster, rasterizer=rasterizer, address_mode=options.address_mode)
        else:
            render = render_textured_mesh(clip_positions_by_view[k], indices, vertex_uv, parameter, target.shape[:2],
                                          rasterizer=rasterizer, viewport=viewports[k],
                                          address_mode=options.address_mode)
            image, valid_mask = render.image, render.valid_mask
            if options.cache_view_rasters:
                cache[k] = (render.raster.detach(), render.uv.detach(), render.valid_mask.detach())
        external = visibility_masks[k]
        if external is not None:
            if external.ndim == 2:
                external = external[..., None]
            valid_mask = valid_mask * external.to(device=valid_mask.device, dtype=valid_mask.dtype)
        loss = masked_charbonnier_loss(image, target, valid_mask, epsilon=options.photometric_epsilon)
        if options.total_variation_weight != 0:
            loss = loss + options.total_variation_weight * atlas_total_variation(parameter, valid_mask=atlas_valid_mask,
                                                                                  chart_ids=chart_ids)
        if options.seam_weight != 0 and seam_uv_pairs is not None:
            loss = loss + options.seam_weight * seam_consistency_loss(parameter, seam_uv_pairs, rasterizer=rasterizer,
                                                                      address_mode=options.address_mode)
        if options.initial_prior_weight != 0:
            prior = (parameter - initial).square()
            if atlas_valid_mask is not None:
                prior = prior * atlas_valid_mask.to(device=prior.device, dtype=prior.dtype)[..., None]
            loss = loss + options.initial_prior_weight * prior.mean()
        loss.backward()
        optimizer.step()
        with torch.no_grad():
            parameter.clamp_(options.clamp_min, options.clamp_max)
        history.append(float(loss.detach().cpu()))
    return parameter.detach(), history


# optimize_texture_atlas takes the refiner kernels when they apply; False keeps the torch operations
# (the reference's own loop over the CUDA renderer) for every call.
USE_REFINER_KERNELS = True


def _native_path_applies(initial_texture, target_images, options) -> bool:
    """The native kernels hold an RGB atlas and sample with clamp addressing; the prior term and other
    channel counts or address modes take the torch path."""
    return (USE_REFINER_KERNELS and isinstance(initial_texture, torch.Tensor) and initial_texture.is_cuda
            and initial_texture.ndim == 3
            and initial_texture.shape[2] == 3 and initial_texture.dtype == torch.float32
            and options.address_mode == "clamp" and options.initial_prior_weight == 0
            and all(isinstance(t, torch.Tensor) and t.ndim == 3 and t.shape[2] == 3 for t in target_images))


def _optimize_native(initial_texture, clip_positions_by_view, indices, vertex_uv, target_images, rasterizer,
                     viewports, visibility_masks, atlas_valid_mask, chart_ids, seam_uv_pairs, options):
    """atlas.py:147-257 on the refiner kernels. Per step, as the reference's loop: the round-robin view's
    masked Charbonnier loss over valid_mask * visibility mask (mean over masked pixels and channels),
    plus total_variation_weight * the chart-aware TV, plus seam_weight * the seam Charbonnier mean;
    then Adam (torch.optim.Adam's update with its bias corrections, eps 1e-8) and the clamp."""
    from .baking import RefineViewC

    ctx = rasterizer.context
    dev = ctx.device
    tex = initial_texture.detach().to(dev).contiguous().clone()
    th, tw, _ = tex.shape
    grad = torch.zeros((th, tw, 4), dtype=torch.float32, device=dev)  # RGB + pad, cleared by the Adam pass
    m1, m2 = torch.zeros_like(tex), torch.zeros_like(tex)
    steps = int(options.steps)
    losses = torch.zeros((steps, 3), dtype=torch.float32, device=dev)  # photometric, seam, TV per step
    idx = indices.to(dev)
    uvv = vertex_uv.to(dev)
    pairs = None
    if options.seam_weight != 0 and seam_uv_pairs is not None and seam_uv_pairs.shape[0] > 0:
        pairs = seam_uv_pairs.to(dev, torch.float32).reshape(-1, 4).contiguous()
    tv_valid = tv_chart = None
    tv_scale = 0.0
    if options.total_variation_weight != 0:
        valid = (torch.ones((th, tw), dtype=torch.bool, device=dev) if atlas_valid_mask is None
                 else atlas_valid_mask.to(dev).bool())
        ph, pv = valid[:, 1:] & valid[:, :-1], valid[1:, :] & valid[:-1, :]
        if chart_ids is not None:
            ids = chart_ids.to(dev)
            ph, pv = ph & (ids[:, 1:] == ids[:, :-1]), pv & (ids[1:, :] == ids[:-1, :])
            tv_chart = ids.to(torch.int32).contiguous()
        pair_count = max(int(ph.sum().item() + pv.sum().item()), 1)
        tv_scale = float(options.total_variation_weight) / (pair_count * 3)
        tv_valid = valid.to(torch.uint8).contiguous()
    stream = ctx.stream()
    cache: dict = {}

    def view_inputs(k):
        if k in cache:
            return cache[k]
        target = target_images[k].to(dev, torch.float32).contiguous()
        h, w = target.shape[:2]
        raster, _ = rasterize(clip_positions_by_view[k].detach(), idx, (h, w), rasterizer=rasterizer,
                              viewport=viewports[k], output_barycentric_derivatives=False)
        uv = interpolate(uvv.detach(), raster, idx, rasterizer=rasterizer).contiguous()
        mask = (raster[..., 3] > 0).to(torch.float32)
        external = visibility_masks[k]
        if external is not None:
            mask = mask * (external[..., 0] if external.ndim == 3 else external).to(dev, torch.float32)
        mask = mask.contiguous()
        table = (RefineViewC * 1)()
        table[0].uv, table[0].target, table[0].mask, table[0].pixel_count = (uv.data_ptr(), target.data_ptr(),
                                                                             mask.data_ptr(), h * w)
        entry = (torch.frombuffer(bytearray(bytes(table)), dtype=torch.uint8).to(dev), uv, target, mask,
                 float(mask.double().sum().item()), h * w)
        # the geometry does not change during the optimisation, so a view's raster, uv and mask are the
        # same at every visit: kept after the first (the reference re-rasterizes unless
        # cache_view_rasters is set, with identical results)
        cache[k] = entry
        return entry

    lr, b1, b2, eps = float(options.learning_rate), 0.9, 0.999, 1e-8
    view_count = clip_positions_by_view.shape[0]
    with ctx.lock:
        for step in range(steps):
            table, _uv, _target, _mask, weight, pixels = view_inputs(step % view_count)
            norm = 1.0 / (max(weight, 1.0) * 3)
            row = losses[step]
            _native.call("pdr_refine_photometric", _ptr(tex), tw, th, _ptr(table), 1, pixels, 0, 1,
                         float(options.photometric_epsilon), norm, _ptr(grad), _ptr(row), stream)
            if pairs is not None:
                _native.call("pdr_refine_seam", _ptr(tex), tw, th, _ptr(pairs), pairs.shape[0], 1e-4,
                             float(options.seam_weight) / (pairs.shape[0] * 3), _ptr(grad), _ptr(row), 1, stream)
            if tv_valid is not None:
                with torch.no_grad():
                    row[2] = options.total_variation_weight * atlas_total_variation(
                        tex, valid_mask=tv_valid.bool(), chart_ids=tv_chart)
                _native.call("pdr_refine_total_variation", _ptr(tex), tw, th, _ptr(tv_valid), _ptr(tv_chart), 1e-4,
                             tv_scale, _ptr(grad), stream)
            t = step + 1
            _native.call("pdr_refine_adam", _ptr(tex), _ptr(grad), _ptr(m1), _ptr(m2), tex.numel(), lr, b1, b2, eps,
                         1.0 - b1 ** t, 1.0 - b2 ** t, float(options.clamp_min), float(options.clamp_max), stream)
        history = losses.sum(1).tolist()
    return tex, history

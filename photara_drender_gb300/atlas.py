"""Differentiable texture-atlas rendering and optimisation helpers
(python/photara_drender/atlas.py:36-257), on the GB300 rasterize/interpolate/texture kernels.

The losses are the reference's research objective written with torch tensor ops; the renderer under
them is the hand-written CUDA path (photara_drender_gb300.torch). For the fused native refinement
(one CUDA graph for the whole optimisation) see TextureBaker.refine_texture.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, NamedTuple, Optional, Sequence, Tuple

import torch

from .rasterizer import Rasterizer
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

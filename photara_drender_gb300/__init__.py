"""photara_drender for GB300: the differentiable raster / texture / bake / refine path of
fenghuayumo/photara_drender rebuilt as sm_103a CUDA kernels behind a C ABI
(include/pdr_capi.h, libphotara_drender_gb300.so), with the reference's Python surface on top.
"""
from .rasterizer import ADDRESS_MODES, CULL_MODES, Context, DeviceInfo, Rasterizer, enumerate_devices
from .baking import (BakedTexture, TextureBakeOutput, TextureBaker, UnwrappedMesh, project_texture_atlas,
                     suggest_softmax_scale)
from .padding import (SurfaceFillStats, TexturePaddingStats, fill_texture_on_surface, pad_texture_atlas,
                      pad_texture_atlas_native)
from . import formats
from .torch import RenderOutput, check_deferred_errors, interpolate, rasterize, render, texture
from .atlas import (AtlasOptimizationOptions, TexturedRender, atlas_total_variation, masked_charbonnier_loss,
                    optimize_texture_atlas, render_textured_mesh, seam_consistency_loss)

__version__ = "0.4.0+gb300"

__all__ = [
    "ADDRESS_MODES", "AtlasOptimizationOptions", "BakedTexture", "CULL_MODES", "Context", "DeviceInfo", "Rasterizer",
    "check_deferred_errors",
    "TextureBakeOutput", "TextureBaker", "TexturedRender", "UnwrappedMesh", "atlas_total_variation",
    "enumerate_devices", "fill_texture_on_surface", "formats", "interpolate", "pad_texture_atlas", "pad_texture_atlas_native",
    "SurfaceFillStats", "TexturePaddingStats", "masked_charbonnier_loss", "optimize_texture_atlas", "project_texture_atlas",
    "rasterize", "render", "RenderOutput", "render_textured_mesh", "seam_consistency_loss", "suggest_softmax_scale",
    "texture",
]

"""photara_drender for GB300: the differentiable raster / texture / bake / refine path of
fenghuayumo/photara_drender rebuilt as sm_103a CUDA kernels behind a C ABI
(include/pdr_capi.h, libphotara_drender_gb300.so), with the reference's Python surface on top.
"""
from .rasterizer import ADDRESS_MODES, CULL_MODES, Context, DeviceInfo, Rasterizer, enumerate_devices

__version__ = "0.4.0+gb300"

__all__ = ["ADDRESS_MODES", "CULL_MODES", "Context", "DeviceInfo", "Rasterizer", "enumerate_devices"]

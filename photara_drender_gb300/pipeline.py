"""Many-view rasterize -> interpolate -> texture forward + backward over preallocated device buffers.

The reference runs each stage as a synchronous call with host staging (python/photara_drender/
torch.py). This pipeline keeps everything resident, uses one tile-list capacity sized once (the
overflow flag is checked on demand, not per step) and enqueues the whole pass without host
synchronisation, so it can be timed on the device or captured in a CUDA graph.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import torch

from . import _native
from .rasterizer import Rasterizer, TILE, _ptr, _viewports


class RenderFwdBwd:
    """Batched fwd+bwd of rasterize (with derivatives) -> interpolate(attributes) and interpolate(uv)
    -> texture, for `views` views of one mesh at one resolution."""

    def __init__(self, rasterizer: Rasterizer, indices: torch.Tensor, vertex_count: int, views: int, height: int,
                 width: int, attribute_count: int, texture_shape, viewports=None, capacity: Optional[int] = None,
                 address_mode: int = 0):
        self.r = rasterizer
        ctx = rasterizer.context
        dev = ctx.device
        self.idx = indices.to(dev, torch.int32).contiguous()
        self.V, self.T = vertex_count, self.idx.shape[0]
        self.views, self.H, self.W, self.A = views, height, width, attribute_count
        self.th, self.tw, self.C = texture_shape
        self.mode = address_mode
        self.vps, _ = _viewports(viewports, views, width, height, dev)
        tiles = ((width + TILE - 1) // TILE) * ((height + TILE - 1) // TILE)
        self.offsets = torch.empty(views * tiles + 1, dtype=torch.int32, device=dev)
        self.capacity = int(capacity) if capacity else 4 * self.T * views + 1024
        self.list = torch.empty(self.capacity, dtype=torch.int32, device=dev)
        self.ws_bytes = _native.lib().pdr_bin_tiles_workspace_bytes(views, self.T, width, height, self.capacity)
        self.ws = torch.empty(max(self.ws_bytes, 1), dtype=torch.uint8, device=dev)
        self.status = torch.zeros(_native.STATUS_WORDS, dtype=torch.int32, device=dev)
        f = dict(dtype=torch.float32, device=dev)
        P = height * width
        self.P = P
        self.raster = torch.empty((views, height, width, 4), **f)
        self.deriv = torch.empty((views, height, width, 4), **f)
        self.attr_out = torch.empty((views, height, width, attribute_count), **f)
        self.uv = torch.empty((views, height, width, 2), **f)
        self.sampled = torch.empty((views, height, width, self.C), **f)
        self.grad_tex = torch.empty(texture_shape, **f)
        self.grad_uv = torch.empty((views, height, width, 2), **f)
        self.grad_attr = torch.empty((vertex_count, attribute_count), **f)
        self.grad_uv_attr = torch.empty((vertex_count, 2), **f)
        self.grad_raster = torch.empty((views, height, width, 4), **f)
        self.grad_clip = torch.empty((views, vertex_count, 4), **f)

    def check_capacity(self) -> int:
        """Entry count of the last binning; raises when the tile list overflowed its capacity."""
        st = self.status.cpu()
        if int(st[_native.STATUS_TILE_OVERFLOW]):
            raise OverflowError(f"tile list needs {int(st[0]) & 0xFFFFFFFF} entries, capacity {self.capacity}")
        return int(st[0]) & 0xFFFFFFFF

    def forward(self, clip: torch.Tensor, attrs: torch.Tensor, uv_attrs: torch.Tensor, texture: torch.Tensor,
                stream) -> None:
        L = _native.lib()
        v, V, T, W, H = self.views, self.V, self.T, self.W, self.H
        _native.check(L.pdr_bin_tiles(_ptr(clip), v, V, _ptr(self.idx), T, W, H, _ptr(self.vps), _ptr(self.offsets),
                                      _ptr(self.list), self.capacity, _ptr(self.ws), self.ws_bytes, _ptr(self.status),
                                      stream))
        _native.check(L.pdr_rasterize_forward(_ptr(clip), v, V, _ptr(self.idx), T, W, H, _ptr(self.vps), 0,
                                              _ptr(self.offsets), _ptr(self.list), self.capacity, _ptr(self.raster),
                                              _ptr(self.deriv), stream))
        _native.check(L.pdr_interpolate_forward(_ptr(attrs), 0, V, self.A, _ptr(self.idx), T, _ptr(self.raster), v,
                                                self.P, _ptr(self.attr_out), stream))
        _native.check(L.pdr_interpolate_forward(_ptr(uv_attrs), 0, V, 2, _ptr(self.idx), T, _ptr(self.raster), v,
                                                self.P, _ptr(self.uv), stream))
        _native.check(L.pdr_texture_forward(_ptr(texture), 0, self.tw, self.th, self.C, self.mode, _ptr(self.uv),
                                            _ptr(self.raster), v, self.P, _ptr(self.sampled), stream))

    def backward(self, clip: torch.Tensor, attrs: torch.Tensor, uv_attrs: torch.Tensor, texture: torch.Tensor,
                 grad_attr_out: torch.Tensor, grad_sampled: torch.Tensor, stream) -> None:
        L = _native.lib()
        v, V, T, W, H = self.views, self.V, self.T, self.W, self.H
        _native.check(L.pdr_texture_backward(_ptr(texture), 0, self.tw, self.th, self.C, self.mode, _ptr(self.uv),
                                             _ptr(self.raster), v, self.P, _ptr(grad_sampled), _ptr(self.grad_tex),
                                             _ptr(self.grad_uv), _ptr(self.status), stream))
        _native.check(L.pdr_interpolate_backward(_ptr(uv_attrs), 0, V, 2, _ptr(self.idx), T, _ptr(self.raster), v,
                                                 self.P, _ptr(self.grad_uv), _ptr(self.grad_uv_attr),
                                                 _ptr(self.grad_raster), stream))
        _native.check(L.pdr_interpolate_backward_accumulate(_ptr(attrs), 0, V, self.A, _ptr(self.idx), T,
                                                            _ptr(self.raster), v, self.P, _ptr(grad_attr_out),
                                                            _ptr(self.grad_attr), _ptr(self.grad_raster), stream))
        _native.check(L.pdr_rasterize_backward(_ptr(clip), v, V, _ptr(self.idx), T, W, H, _ptr(self.vps),
                                               _ptr(self.raster), _ptr(self.grad_raster), _ptr(self.grad_clip),
                                               stream))

    def step(self, clip, attrs, uv_attrs, texture, grad_attr_out, grad_sampled, stream=None) -> None:
        if stream is None:
            stream = C.c_void_p(torch.cuda.current_stream(self.r.context.device).cuda_stream)
        self.forward(clip, attrs, uv_attrs, texture, stream)
        self.backward(clip, attrs, uv_attrs, texture, grad_attr_out, grad_sampled, stream)

    # number of kernels one step launches (bin: count, 3 scan, fill, 2 sort; raster; 3 forward;
    # texture backward; 2 interpolate backward; raster backward) and the memsets it issues
    KERNELS_PER_STEP = 7 + 1 + 3 + 1 + 2 + 1

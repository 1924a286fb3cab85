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


class RenderArgsC(C.Structure):
    """include/pdr_capi.h pdr_render_args."""

    _fields_ = [
        ("clip_positions", C.c_void_p), ("views", C.c_uint32), ("vertex_count", C.c_uint32), ("indices", C.c_void_p),
        ("triangle_count", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("viewports", C.c_void_p),
        ("cull_mode", C.c_uint32), ("attributes", C.c_void_p), ("attribute_count", C.c_uint32),
        ("uv_attributes", C.c_void_p), ("texture", C.c_void_p), ("texture_width", C.c_uint32),
        ("texture_height", C.c_uint32), ("address_mode", C.c_uint32), ("tile_offsets", C.c_void_p),
        ("tile_triangles", C.c_void_p), ("capacity", C.c_uint64), ("workspace", C.c_void_p),
        ("workspace_bytes", C.c_size_t), ("status", C.c_void_p), ("raster", C.c_void_p),
        ("barycentric_derivatives", C.c_void_p), ("interpolated", C.c_void_p), ("uv", C.c_void_p),
        ("sampled", C.c_void_p), ("grad_interpolated", C.c_void_p), ("grad_sampled", C.c_void_p),
        ("grad_clip_positions", C.c_void_p), ("grad_attributes", C.c_void_p), ("grad_uv_attributes", C.c_void_p),
        ("grad_texture", C.c_void_p), ("sample_differences", C.c_void_p), ("tile_width", C.c_uint32),
        ("tile_height", C.c_uint32), ("stage_triangles", C.c_uint32),
    ]


# Tile shapes and stage depths of the fused render (pdr_render_args.tile_width / tile_height /
# stage_triangles): the raster kernels are compiled for these.
TILE_CONFIGS = ((16, 16, 256), (16, 16, 128), (16, 8, 128))


class RenderFwdBwd:
    """Batched fwd+bwd of rasterize (with derivatives) -> interpolate(attributes) and interpolate(uv)
    -> texture, for `views` views of one mesh at one resolution."""

    def __init__(self, rasterizer: Rasterizer, indices: torch.Tensor, vertex_count: int, views: int, height: int,
                 width: int, attribute_count: int, texture_shape, viewports=None, capacity: Optional[int] = None,
                 address_mode: int = 0, fused: bool = True, keep_sample_differences: bool = True,
                 tile_config=(16, 16, 256)):
        self.r = rasterizer
        self.fused = fused
        ctx = rasterizer.context
        dev = ctx.device
        self.idx = indices.to(dev, torch.int32).contiguous()
        self.V, self.T = vertex_count, self.idx.shape[0]
        self.views, self.H, self.W, self.A = views, height, width, attribute_count
        self.th, self.tw, self.C = texture_shape
        self.mode = address_mode
        self.vps, _ = _viewports(viewports, views, width, height, dev)
        self.status = torch.zeros(_native.STATUS_WORDS, dtype=torch.int32, device=dev)
        self.set_tile_config(tile_config if fused else (16, 16, 256), capacity)
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
        # the forward's texel differences per covered pixel, read by the fused backward instead of
        # gathering the texels again (32 bytes per pixel)
        self.sample_diff = torch.empty((views, height, width, 8), **f) if fused and keep_sample_differences else None

    def set_tile_config(self, config, capacity: Optional[int] = None) -> None:
        """Tile shape and stage depth of the fused binning and raster (one of TILE_CONFIGS), with the
        tile list, offsets and workspace they need."""
        config = tuple(int(x) for x in config)
        if config not in TILE_CONFIGS:
            raise ValueError(f"tile configuration must be one of {TILE_CONFIGS}")
        dev = self.r.context.device
        tw, th, _ = config
        self.tile_config = config
        tiles = ((self.W + tw - 1) // tw) * ((self.H + th - 1) // th)
        self.offsets = torch.empty(self.views * tiles + 1, dtype=torch.int32, device=dev)
        self.capacity = int(capacity) if capacity else 4 * self.T * self.views + 1024
        self.list = torch.empty(self.capacity, dtype=torch.int32, device=dev)
        # one workspace for the binning and for the backward's per-view vertex-gradient records
        L = _native.lib()
        self.ws_bytes = max(L.pdr_render_workspace_bytes_tiled(self.views, self.T, self.W, self.H, self.capacity, tw,
                                                               th),
                            L.pdr_render_backward_workspace_bytes(self.views, self.V, self.A))
        self.ws = torch.empty(max(self.ws_bytes, 1), dtype=torch.uint8, device=dev)

    def autotune(self, clip, attrs, uv_attrs, texture, reps: int = 5, configs=TILE_CONFIGS):
        """Times the fused forward (binning + raster) of these inputs for every tile configuration, keeps the
        fastest and sizes its tile list to the measured entry count (+25%). Returns {config: median ms}.
        Outputs are the same for every configuration."""
        if not self.fused:
            return {}
        dev = self.r.context.device
        stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        times, needs = {}, {}
        for cfg in configs:
            self.set_tile_config(cfg)
            self.forward(clip, attrs, uv_attrs, texture, stream)
            entries = self.check_capacity()
            needs[cfg] = int(entries * 1.25) + 1024
            self.set_tile_config(cfg, needs[cfg])
            samples = []
            for i in range(reps + 1):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                self.forward(clip, attrs, uv_attrs, texture, stream)
                e1.record()
                torch.cuda.synchronize(dev)
                if i:
                    samples.append(e0.elapsed_time(e1))
            times[cfg] = sorted(samples)[len(samples) // 2]
        best = min(times, key=times.get)
        self.set_tile_config(best, needs[best])
        return times

    def check_capacity(self) -> int:
        """Entry count of the last binning; raises when the tile list overflowed its capacity."""
        st = self.status.cpu()
        if int(st[_native.STATUS_TILE_OVERFLOW]):
            raise OverflowError(f"tile list needs {int(st[0]) & 0xFFFFFFFF} entries, capacity {self.capacity}")
        return int(st[0]) & 0xFFFFFFFF

    def _args(self, clip, attrs, uv_attrs, texture, grad_attr_out=None, grad_sampled=None) -> RenderArgsC:
        a = RenderArgsC()
        a.clip_positions, a.views, a.vertex_count = clip.data_ptr(), self.views, self.V
        a.indices, a.triangle_count, a.width, a.height = self.idx.data_ptr(), self.T, self.W, self.H
        a.viewports, a.cull_mode = self.vps.data_ptr(), 0
        a.attributes, a.attribute_count, a.uv_attributes = attrs.data_ptr(), self.A, uv_attrs.data_ptr()
        a.texture, a.texture_width, a.texture_height, a.address_mode = texture.data_ptr(), self.tw, self.th, self.mode
        a.tile_offsets, a.tile_triangles, a.capacity = self.offsets.data_ptr(), self.list.data_ptr(), self.capacity
        a.workspace, a.workspace_bytes, a.status = self.ws.data_ptr(), self.ws_bytes, self.status.data_ptr()
        a.raster, a.barycentric_derivatives = self.raster.data_ptr(), self.deriv.data_ptr()
        a.interpolated, a.uv, a.sampled = self.attr_out.data_ptr(), self.uv.data_ptr(), self.sampled.data_ptr()
        if grad_attr_out is not None:
            a.grad_interpolated, a.grad_sampled = grad_attr_out.data_ptr(), grad_sampled.data_ptr()
        a.grad_clip_positions, a.grad_attributes = self.grad_clip.data_ptr(), self.grad_attr.data_ptr()
        a.grad_uv_attributes, a.grad_texture = self.grad_uv_attr.data_ptr(), self.grad_tex.data_ptr()
        if self.sample_diff is not None:
            a.sample_differences = self.sample_diff.data_ptr()
        a.tile_width, a.tile_height, a.stage_triangles = self.tile_config
        return a

    def forward(self, clip: torch.Tensor, attrs: torch.Tensor, uv_attrs: torch.Tensor, texture: torch.Tensor,
                stream) -> None:
        L = _native.lib()
        if self.fused:
            a = self._args(clip, attrs, uv_attrs, texture)
            _native.check(L.pdr_render_forward(C.addressof(a), stream))
            return
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
        if self.fused:
            a = self._args(clip, attrs, uv_attrs, texture, grad_attr_out, grad_sampled)
            _native.check(L.pdr_render_backward(C.addressof(a), stream))
            return
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

    def kernels_per_step(self) -> int:
        """Kernels one step launches: binning (count, three scan phases, fill; the unfused path also
        sorts each tile, two passes), the raster (the main launch and the pass over tiles whose lists were
        cut), then fused: the shading is the raster's epilogue and the backward is the adjoint plus the pass
        that sums its per-view vertex records; unfused: three forwards, texture backward, two interpolate
        backwards, raster backward."""
        return 5 + 2 + 2 if self.fused else 5 + 2 + 2 + 3 + 1 + 2 + 1

    def capture(self, clip, attrs, uv_attrs, texture, grad_attr_out, grad_sampled) -> "torch.cuda.CUDAGraph":
        """Records one step into a CUDA graph (replay with .replay()); for small, launch-bound batches.
        The inputs must stay at the same addresses while the graph is in use."""
        dev = self.r.context.device
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):  # warm the argument paths outside the capture
            self.step(clip, attrs, uv_attrs, texture, grad_attr_out, grad_sampled)
        torch.cuda.current_stream(dev).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step(clip, attrs, uv_attrs, texture, grad_attr_out, grad_sampled)
        return g

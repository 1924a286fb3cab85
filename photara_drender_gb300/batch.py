"""Uneven multi-mesh batches in one launch (no counterpart in the reference, which renders one mesh per
call): many meshes, each with its own views, resolution and texture, run through one binning pass, one
raster launch with the shading epilogue and one adjoint launch (include/pdr_capi.h
pdr_render_batch_*). The forward tile shape and the triangles staged per pass (the bin depth) come
from `MeshBatch.autotune`, which times every compiled configuration on the batch itself; outputs are
bit-identical for every configuration.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _native
from .rasterizer import Rasterizer, _ptr, _viewports

CONFIGS: Tuple[Tuple[int, int, int], ...] = ((16, 8, 128), (16, 16, 128), (16, 16, 256))
_MODES = {"none": 0, "back": 1, "front": 2}
_ADDRESS = {"clamp": 0, "wrap": 1, "mirror": 2}


class RenderMeshC(C.Structure):
    """include/pdr_capi.h pdr_render_mesh."""
    _fields_ = [
        ("clip_positions", C.c_void_p), ("indices", C.c_void_p), ("viewports", C.c_void_p),
        ("attributes", C.c_void_p), ("uv_attributes", C.c_void_p), ("texture", C.c_void_p),
        ("views", C.c_uint32), ("vertex_count", C.c_uint32), ("triangle_count", C.c_uint32), ("width", C.c_uint32),
        ("height", C.c_uint32), ("texture_width", C.c_uint32), ("texture_height", C.c_uint32),
        ("raster", C.c_void_p), ("barycentric_derivatives", C.c_void_p), ("interpolated", C.c_void_p),
        ("uv", C.c_void_p), ("sampled", C.c_void_p), ("grad_interpolated", C.c_void_p),
        ("grad_sampled", C.c_void_p), ("grad_clip_positions", C.c_void_p), ("grad_attributes", C.c_void_p),
        ("grad_uv_attributes", C.c_void_p), ("grad_texture", C.c_void_p),
    ]


class BatchConfigC(C.Structure):
    _fields_ = [("tile_width", C.c_uint32), ("tile_height", C.c_uint32), ("stage_triangles", C.c_uint32)]


@dataclass
class BatchMesh:
    """One mesh of a batch: inputs (device tensors) and the output / gradient buffers the batch fills."""
    clip: torch.Tensor                      # [views, V, 4]
    indices: torch.Tensor                   # [T, 3] int32
    height: int
    width: int
    attributes: Optional[torch.Tensor] = None   # [V, A]
    uv_attributes: Optional[torch.Tensor] = None  # [V, 2]
    texture: Optional[torch.Tensor] = None  # [th, tw, 4]
    viewports: Optional[torch.Tensor] = None  # [views, 4]
    outputs: Dict[str, torch.Tensor] = field(default_factory=dict)
    grads: Dict[str, torch.Tensor] = field(default_factory=dict)


class MeshBatch:
    """A fixed set of meshes rendered forward and backward together."""

    def __init__(self, rasterizer: Rasterizer, meshes: Sequence[BatchMesh], cull_mode: str = "none",
                 address_mode: str = "clamp", config: Tuple[int, int, int] = (16, 16, 256)):
        self.r = rasterizer
        dev = rasterizer.context.device
        self.meshes = list(meshes)
        if not self.meshes:
            raise ValueError("a batch needs at least one mesh")
        A = {m.attributes.shape[1] if m.attributes is not None else 0 for m in self.meshes}
        if len(A) != 1:
            raise ValueError("all meshes of a batch share one attribute count")
        self.A = A.pop()
        self.cull, self.mode = _MODES[cull_mode], _ADDRESS[address_mode]
        f = dict(dtype=torch.float32, device=dev)
        for m in self.meshes:
            views = m.clip.shape[0]
            m.indices = m.indices.to(dev, torch.int32).contiguous()
            if m.viewports is None:
                m.viewports, _ = _viewports(None, views, m.width, m.height, dev)
            shape = (views, m.height, m.width)
            # outputs already attached to the mesh (e.g. by another batch holding it) are reused
            need = {"raster": 4, "deriv": 4}
            if m.attributes is not None:
                need["interp"] = self.A
            if m.uv_attributes is not None:
                need["uv"] = 2
            if m.texture is not None:
                need["sampled"] = 4
            for name, channels in need.items():
                if name not in m.outputs:
                    m.outputs[name] = torch.empty(shape + (channels,), **f)
        self.status = torch.zeros(_native.STATUS_WORDS, dtype=torch.int32, device=dev)
        self.capacity = 0
        self.set_config(config)

    # -- native structures -------------------------------------------------------------------------------
    def _table(self):
        arr = (RenderMeshC * len(self.meshes))()
        for k, m in enumerate(self.meshes):
            c = arr[k]
            c.clip_positions, c.indices, c.viewports = m.clip.data_ptr(), m.indices.data_ptr(), m.viewports.data_ptr()
            c.views, c.vertex_count, c.triangle_count = m.clip.shape[0], m.clip.shape[1], m.indices.shape[0]
            c.width, c.height = m.width, m.height
            if m.attributes is not None:
                c.attributes, c.interpolated = m.attributes.data_ptr(), m.outputs["interp"].data_ptr()
            if m.uv_attributes is not None:
                c.uv_attributes, c.uv = m.uv_attributes.data_ptr(), m.outputs["uv"].data_ptr()
            if m.texture is not None:
                c.texture, c.sampled = m.texture.data_ptr(), m.outputs["sampled"].data_ptr()
                c.texture_height, c.texture_width = m.texture.shape[0], m.texture.shape[1]
            c.raster, c.barycentric_derivatives = m.outputs["raster"].data_ptr(), m.outputs["deriv"].data_ptr()
            g = m.grads
            for name, attr in (("interp", "grad_interpolated"), ("sampled", "grad_sampled"),
                               ("clip", "grad_clip_positions"), ("attributes", "grad_attributes"),
                               ("uv_attributes", "grad_uv_attributes"), ("texture", "grad_texture")):
                if name in g:
                    setattr(c, attr, g[name].data_ptr())
        return arr

    def set_config(self, config: Tuple[int, int, int]) -> None:
        if tuple(config) not in CONFIGS:
            raise ValueError(f"batch configuration must be one of {CONFIGS}")
        self.config = BatchConfigC(*config)
        segs, ws = C.c_uint64(), C.c_size_t()
        _native.call("pdr_render_batch_sizes", self._table(), len(self.meshes), C.byref(self.config), self.A,
                     C.byref(segs), C.byref(ws))
        dev = self.r.context.device
        self.segments = segs.value
        self.offsets = torch.empty(self.segments + 1, dtype=torch.int32, device=dev)
        self.workspace = torch.empty(max(ws.value, 1), dtype=torch.uint8, device=dev)
        total_tris = sum(m.clip.shape[0] * m.indices.shape[0] for m in self.meshes)
        self._ensure_capacity(max(self.capacity, 2 * total_tris + 1024))

    def _ensure_capacity(self, capacity: int) -> None:
        if capacity > self.capacity or not hasattr(self, "list"):
            self.capacity = int(capacity)
            self.list = torch.empty(self.capacity, dtype=torch.int32, device=self.r.context.device)

    # -- passes --------------------------------------------------------------------------------------------
    def forward(self, stream=None) -> None:
        """Renders every view of every mesh (re-running with a larger tile list when it overflowed)."""
        ctx = self.r.context
        s = stream if stream is not None else ctx.stream()
        for _ in range(3):
            self.status.zero_()
            _native.call("pdr_render_batch_forward", self._table(), len(self.meshes), self.A, self.cull, self.mode,
                         C.byref(self.config), _ptr(self.offsets), _ptr(self.list), self.capacity,
                         _ptr(self.workspace), self.workspace.numel(), _ptr(self.status), s)
            st = self.status.cpu()
            if int(st[_native.STATUS_TILE_ENTRIES_HI]) != 0:
                raise OverflowError("Tile triangle list exceeds backend limits")
            if not int(st[_native.STATUS_TILE_OVERFLOW]):
                return
            total = int(st[_native.STATUS_TILE_ENTRIES]) & 0xFFFFFFFF
            self._ensure_capacity(total + total // 8 + 1024)
        raise RuntimeError("tile binning did not converge")

    def allocate_gradients(self) -> None:
        for m in self.meshes:
            f = dict(dtype=torch.float32, device=m.clip.device)
            for name, src in (("clip", m.clip), ("attributes", m.attributes), ("uv_attributes", m.uv_attributes),
                              ("texture", m.texture)):
                if src is not None and name not in m.grads:
                    m.grads[name] = torch.empty(src.shape, **f)

    def backward(self, stream=None) -> None:
        """Adjoints of the last forward; upstream gradients are m.grads['interp'] / m.grads['sampled']."""
        ctx = self.r.context
        s = stream if stream is not None else ctx.stream()
        self.allocate_gradients()
        self.status.zero_()
        _native.call("pdr_render_batch_backward", self._table(), len(self.meshes), self.A, self.mode,
                     C.byref(self.config), _ptr(self.workspace), self.workspace.numel(), _ptr(self.status), s)

    def autotune(self, configs: Sequence[Tuple[int, int, int]] = CONFIGS, reps: int = 3,
                 backward: bool = True) -> Dict[Tuple[int, int, int], float]:
        """Times forward (+ backward) of this batch for every configuration and keeps the fastest.
        Returns {config: median milliseconds}."""
        dev = self.r.context.device
        times = {}
        for cfg in configs:
            self.set_config(cfg)
            self.forward()
            if backward:
                self.backward()
            samples = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize(dev)
                e0.record()
                self.forward()
                if backward:
                    self.backward()
                e1.record()
                torch.cuda.synchronize(dev)
                samples.append(e0.elapsed_time(e1))
            times[tuple(cfg)] = sorted(samples)[len(samples) // 2]
        best = min(times, key=times.get)
        self.set_config(best)
        return times

"""Atlas padding and surface fill on the GPU (csrc/padding.cu through include/pdr_capi.h).

`pad_texture_atlas` mirrors python/photara_drender/baking.py:33-80 (the public helper, which returns a
padded copy of the colour); `pad_texture_atlas_native` mirrors the binding it wraps,
python/bindings.cpp:786-836 (`(color, filled_mask, gutter, unobserved, remaining)`), and
`fill_texture_on_surface` the C++ routine of include/photara_drender/texture_padding.hpp:17-23.
NumPy inputs are copied to the device and results copied back; CUDA tensors stay on the device.
Results equal the reference's CPU code bit for bit (the 8SSEDT field is reproduced sweep for sweep).
"""
from __future__ import annotations

import ctypes as C
import threading
from typing import Dict, NamedTuple, Optional

import numpy as np
import torch

from . import _native
from .rasterizer import Context, _ptr

_ERR_TIMEOUT, _ERR_FACE_RANGE, _ERR_DEGENERATE, _ERR_MANIFOLD = 1, 2, 4, 8


class TexturePaddingStats(NamedTuple):
    """include/photara_drender/texture_padding.hpp:46-57 (without the host timing)."""
    valid_texels: int
    gutter_texels: int
    unobserved_texels: int
    remaining_unobserved: int
    filled_texels: int


class SurfaceFillStats(NamedTuple):
    """include/photara_drender/texture_padding.hpp:10-15."""
    filled_texels: int
    remaining_texels: int
    measured_faces: int
    propagated_faces: int


_contexts: Dict[int, Context] = {}
_contexts_lock = threading.Lock()


def _context(device_index: int) -> Context:
    with _contexts_lock:
        if device_index not in _contexts:
            _contexts[device_index] = Context(device_index)
        return _contexts[device_index]


def _device_f32(x, dev, copy: bool) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x.detach().to(dev, torch.float32)
        return t.clone().contiguous() if copy or not t.is_contiguous() else t
    return torch.from_numpy(np.array(x, dtype=np.float32, copy=True, order="C")).to(dev)


def _is_host(*xs) -> bool:
    return any(not isinstance(x, torch.Tensor) for x in xs if x is not None)


def pad_texture_atlas_device(color: torch.Tensor, valid_mask: torch.Tensor, margin: int = 4,
                             coverage_mask: Optional[torch.Tensor] = None, fill_unobserved: bool = True,
                             maximum_fill_distance: int = 0, *, filled_mask: Optional[torch.Tensor] = None,
                             valid_threshold: float = 0.5, context: Optional[Context] = None) -> TexturePaddingStats:
    """texture_padding.cpp:226-351 in place on CUDA tensors: color [H, W, 3|4] and filled_mask [H, W]
    (created as zeros when None and then returned through the stats' caller). Returns the statistics."""
    ctx = context or _context(color.device.index or 0)
    if color.ndim != 3 or color.shape[2] not in (3, 4):
        raise ValueError("atlas color must have 3 or 4 channels")
    h, w, ch = color.shape
    for t in (color, valid_mask, coverage_mask, filled_mask):
        if t is not None and (t.dtype != torch.float32 or not t.is_contiguous() or t.device != ctx.device):
            raise ValueError("padding buffers must be contiguous float32 tensors on the context's device")
    if tuple(valid_mask.shape) != (h, w):
        raise ValueError("atlas valid_mask must match the atlas dimensions")
    if coverage_mask is not None and tuple(coverage_mask.shape) != (h, w):
        raise ValueError("coverage_mask must match the color dimensions")
    if filled_mask is None:
        raise ValueError("filled_mask is required")
    if margin < 0 or maximum_fill_distance < 0:
        raise ValueError("padding must be non-negative")
    with ctx.lock:
        need = C.c_size_t()
        _native.call("pdr_pad_workspace_bytes", w, h, ch, C.byref(need))
        ws = torch.empty(max(need.value, 1), dtype=torch.uint8, device=ctx.device)
        stats = torch.empty(5, dtype=torch.int64, device=ctx.device)
        ctx.status.zero_()
        _native.call("pdr_pad_texture_atlas", _ptr(color), ch, _ptr(valid_mask),
                     _ptr(coverage_mask) if coverage_mask is not None else None, _ptr(filled_mask), w, h, int(margin),
                     int(bool(fill_unobserved)), int(maximum_fill_distance), float(valid_threshold), _ptr(ws),
                     ws.numel(), _ptr(stats), _ptr(ctx.status), ctx.stream())
        err = int(ctx.status[_native.STATUS_PAD_ERROR])
        if err & _ERR_TIMEOUT:
            raise RuntimeError("atlas padding sweep did not complete")
        return TexturePaddingStats(*(int(v) for v in stats.cpu()))


def pad_texture_atlas_native(color, valid_mask, margin: int = 4, coverage_mask=None, fill_unobserved: bool = True,
                             maximum_fill_distance: int = 0, *, device_index: int = 0):
    """python/bindings.cpp:786-836: (padded color, filled_mask, gutter_texels, unobserved_texels,
    remaining_unobserved) on copies of the inputs."""
    shape = tuple(color.shape)
    if len(shape) != 3 or shape[0] <= 0 or shape[1] <= 0 or shape[2] not in (3, 4):
        raise ValueError("color must have shape [height, width, 3 or 4]")
    if tuple(valid_mask.shape) != shape[:2]:
        raise ValueError("valid_mask must match the color dimensions")
    if coverage_mask is not None and tuple(coverage_mask.shape) != shape[:2]:
        raise ValueError("coverage_mask must match the color dimensions")
    if margin < 0 or maximum_fill_distance < 0:
        raise TypeError("margin and maximum_fill_distance must be unsigned 32-bit integers")
    dev_index = color.device.index if isinstance(color, torch.Tensor) and color.is_cuda else device_index
    ctx = _context(dev_index or 0)
    col = _device_f32(color, ctx.device, copy=True)
    valid = _device_f32(valid_mask, ctx.device, copy=False)
    cov = None if coverage_mask is None else _device_f32(coverage_mask, ctx.device, copy=False)
    filled = torch.zeros(shape[:2], dtype=torch.float32, device=ctx.device)
    st = pad_texture_atlas_device(col, valid, margin, cov, fill_unobserved, maximum_fill_distance, filled_mask=filled,
                                  context=ctx)
    if _is_host(color, valid_mask, coverage_mask):
        col, filled = col.cpu().numpy(), filled.cpu().numpy()
    return col, filled, st.gutter_texels, st.unobserved_texels, st.remaining_unobserved


def pad_texture_atlas(color, valid_mask, padding: int, *, coverage_mask=None, fill_unobserved: bool = False,
                      maximum_fill_distance: int = 0):
    """python/photara_drender/baking.py:33-80: extends valid atlas texels into empty neighbours and returns
    a padded copy of the colour; valid_mask is not modified."""
    host = _is_host(color, valid_mask, coverage_mask)
    if host:
        color = np.asarray(color, dtype=np.float32)
        valid = np.asarray(valid_mask, dtype=bool)
        if color.ndim != 3 or color.shape[2] not in (3, 4):
            raise ValueError("color must have shape [height, width, 3 or 4]")
        if valid.shape != color.shape[:2]:
            raise ValueError("valid_mask must match the color dimensions")
    else:
        valid = valid_mask.to(torch.bool)
        if color.ndim != 3 or color.shape[2] not in (3, 4):
            raise ValueError("color must have shape [height, width, 3 or 4]")
        if tuple(valid.shape) != tuple(color.shape[:2]):
            raise ValueError("valid_mask must match the color dimensions")
    if padding < 0:
        raise ValueError("padding must be non-negative")

    def copy():
        return np.ascontiguousarray(color.copy()) if host else color.to(torch.float32).clone().contiguous()

    if padding == 0 and not fill_unobserved:
        return copy()
    if not bool(valid.any()):
        return copy()
    if coverage_mask is not None and tuple(coverage_mask.shape) != tuple(valid.shape):
        raise ValueError("coverage_mask must match the color dimensions")
    if maximum_fill_distance < 0:
        raise ValueError("maximum_fill_distance must be non-negative")
    valid_f = valid.astype(np.float32) if host else valid.to(torch.float32)
    padded, _filled, _gutter, _unobserved, _remaining = pad_texture_atlas_native(
        color, valid_f, int(padding), coverage_mask, bool(fill_unobserved), int(maximum_fill_distance))
    return padded


def fill_texture_on_surface(color, valid_mask, face_ids, triangle_indices, *, filled_mask=None, device_index: int = 0):
    """include/photara_drender/texture_padding.hpp:17-23 on copies: fills covered texels without a
    sample with the measured mean colour of their face, or of the nearest measured face over shared
    mesh edges. triangle_indices are the original (seam-free) mesh's. Returns (color, filled_mask,
    SurfaceFillStats)."""
    shape = tuple(color.shape)
    if len(shape) != 3 or shape[0] * shape[1] == 0 or tuple(valid_mask.shape) != shape[:2] \
            or tuple(face_ids.shape) != shape[:2]:
        raise ValueError("surface fill requires mesh face IDs and a valid atlas")
    if shape[2] not in (3, 4):
        raise ValueError("surface fill requires RGB or RGBA colours")
    host = _is_host(color, valid_mask, face_ids, triangle_indices)
    dev_index = color.device.index if isinstance(color, torch.Tensor) and color.is_cuda else device_index
    ctx = _context(dev_index or 0)
    h, w, ch = shape
    col = _device_f32(color, ctx.device, copy=True)
    valid = _device_f32(valid_mask, ctx.device, copy=False)
    if isinstance(face_ids, torch.Tensor):
        faces = face_ids.detach().to(ctx.device).to(torch.int64).to(torch.int32).contiguous()
    else:
        faces = torch.from_numpy(np.ascontiguousarray(np.asarray(face_ids, dtype=np.uint32)).view(np.int32)).to(
            ctx.device)
    if isinstance(triangle_indices, torch.Tensor):
        idx = triangle_indices.detach().to(ctx.device).to(torch.int64).to(torch.int32).reshape(-1).contiguous()
    else:
        idx = torch.from_numpy(np.ascontiguousarray(np.asarray(triangle_indices, dtype=np.uint32).reshape(-1))
                               .view(np.int32)).to(ctx.device)
    if idx.numel() == 0 or idx.numel() % 3 != 0:
        raise ValueError("surface fill requires mesh face IDs and a valid atlas")
    T = idx.numel() // 3
    filled = (torch.zeros((h, w), dtype=torch.float32, device=ctx.device) if filled_mask is None
              else _device_f32(filled_mask, ctx.device, copy=True))
    with ctx.lock:
        need = C.c_size_t()
        _native.call("pdr_surface_fill_workspace_bytes", w, h, T, C.byref(need))
        ws = torch.empty(max(need.value, 1), dtype=torch.uint8, device=ctx.device)
        stats = torch.empty(4, dtype=torch.int64, device=ctx.device)
        ctx.status.zero_()
        _native.call("pdr_fill_texture_on_surface", _ptr(col), ch, _ptr(valid), _ptr(faces), _ptr(filled), w, h,
                     _ptr(idx), T, _ptr(ws), ws.numel(), _ptr(stats), _ptr(ctx.status), ctx.stream())
        err = int(ctx.status[_native.STATUS_PAD_ERROR])
    if err & _ERR_FACE_RANGE:
        raise ValueError("atlas face ID is out of range")
    if err & _ERR_DEGENERATE:
        raise ValueError("surface fill mesh has a degenerate edge")
    if err & _ERR_MANIFOLD:
        raise ValueError("surface fill requires manifold edges")
    st = SurfaceFillStats(*(int(v) for v in stats.cpu()))
    if host:
        return col.cpu().numpy(), filled.cpu().numpy(), st
    return col, filled, st

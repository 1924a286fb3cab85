"""Rasterizer: the reference's `_photara_drender.Rasterizer` binding (python/bindings.cpp:414-711)
re-implemented over the GB300 C ABI.

Method names, keyword arguments, defaults, array shapes and exception types follow the
reference. Inputs may be NumPy arrays (results come back as NumPy arrays, with the host<->device
copies the reference's binding also performs) or torch tensors (results stay on the tensors'
device, zero-copy when they already live on the GPU). A leading view axis is accepted
everywhere: positions [B, V, 4] rasterize B views in one launch.
"""
from __future__ import annotations

import ctypes as C
import math
import threading
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native

CULL_MODES = {"none": 0, "back": 1, "front": 2}
ADDRESS_MODES = {"clamp": 0, "wrap": 1, "mirror": 2}
TILE = 16
NEAR_MAX_TRIANGLES = 8388608  # PDR_NEAR_MAX_TRIANGLES: ids of the clipped mesh (2 T) stay exact in fp32


def parse_cull_mode(value: str) -> int:
    if value not in CULL_MODES:
        raise ValueError("cull_mode must be 'none', 'back', or 'front'")
    return CULL_MODES[value]


def parse_address_mode(value: str) -> int:
    if value not in ADDRESS_MODES:
        raise ValueError("address_mode must be 'clamp', 'wrap', or 'mirror'")
    return ADDRESS_MODES[value]


@dataclass(frozen=True)
class DeviceInfo:
    """include/photara_drender/types.hpp DeviceInfo."""

    name: str
    vendor_id: int
    device_id: int
    api_version: int
    supports_ray_query: bool = False

    def __repr__(self) -> str:
        return f"DeviceInfo(name='{self.name}', vendor_id={self.vendor_id})"


def enumerate_devices():
    L = _native.lib()
    out = []
    for d in range(L.pdr_device_count()):
        out.append(_device_info(d))
    return out


def _device_info(index: int) -> DeviceInfo:
    name = C.create_string_buffer(256)
    vendor, dev, api = C.c_uint32(), C.c_uint32(), C.c_uint32()
    sms = C.c_int32()
    _native.call("pdr_device_info", index, name, 256, C.byref(vendor), C.byref(dev), C.byref(api), C.byref(sms))
    # ray queries run through the library's own BVH ray caster (csrc/bvh.cu) on every CUDA device
    return DeviceInfo(name.value.decode(), vendor.value, dev.value, api.value, True)


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else C.c_void_p(t.data_ptr())


class Context:
    """One CUDA device plus a lock that serialises calls, as the reference's per-context
    dispatch mutex does (src/context_internal.hpp:101)."""

    def __init__(self, device_index: int = 0, enable_validation: bool = False):
        if not torch.cuda.is_available():
            raise RuntimeError("photara_drender_gb300 needs a CUDA device")
        if device_index < 0 or device_index >= torch.cuda.device_count():
            raise IndexError("device_index is out of range")
        self.device = torch.device("cuda", device_index)
        self.enable_validation = enable_validation
        self.lock = threading.RLock()
        self.info = _device_info(device_index)
        self.status = torch.zeros(_native.STATUS_WORDS, dtype=torch.int32, device=self.device)
        self._pending = []  # (event, pinned copy of the status block, kind) of calls that did not wait
        self._spare = []    # pinned buffers ready for reuse

    def stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def defer_status(self, kind: str) -> None:
        """Queues a copy of the status block to pinned host memory behind the work just enqueued,
        without waiting for it; poll_status() hands it back once that work has finished. Inside a CUDA
        graph capture nothing is queued (the captured work's status is not observable per replay)."""
        if torch.cuda.is_current_stream_capturing():
            return
        if len(self._pending) >= 64:  # bound the queue: wait for the oldest copy
            self._pending[0][0].synchronize()
        buf = self._spare.pop() if self._spare else torch.empty(_native.STATUS_WORDS, dtype=torch.int32,
                                                                  pin_memory=True)
        buf.copy_(self.status, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self._pending.append((ev, buf, kind))

    def poll_status(self, wait: bool = False, kinds=None):
        """[(kind, status words)] of the queued copies whose work has finished (all of them when `wait`),
        oldest first; with `kinds`, only copies of those kinds are taken (the others stay queued)."""
        done = []
        if torch.cuda.is_current_stream_capturing():  # no event queries while a capture is recording
            return done
        keep = []
        for entry in self._pending:
            ev, buf, kind = entry
            if (kinds is None or kind in kinds) and (wait or ev.query()):
                ev.synchronize()
                done.append((kind, [int(x) for x in buf.tolist()]))
                self._spare.append(buf)
            else:
                keep.append(entry)
        self._pending = keep
        return done


class _Io:
    """Converts caller arrays to device tensors and results back to the caller's kind."""

    def __init__(self, ctx: Context, *inputs):
        self.ctx = ctx
        self.numpy = any(isinstance(x, np.ndarray) for x in inputs if x is not None)
        dev = [x.device for x in inputs if isinstance(x, torch.Tensor)]
        self.out_device = dev[0] if dev and not self.numpy else None

    def f32(self, x, name: str) -> torch.Tensor:
        if isinstance(x, torch.Tensor):
            if x.dtype != torch.float32:
                x = x.to(torch.float32)
            return x.detach().to(self.ctx.device, non_blocking=True).contiguous()
        arr = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
        return torch.from_numpy(arr).to(self.ctx.device, non_blocking=False)

    def indices(self, x, vertex_count: int, exc=IndexError,
                msg="triangle_indices contains an invalid vertex index") -> torch.Tensor:
        if isinstance(x, torch.Tensor):
            t = x.detach()
            if t.ndim != 2 or t.shape[1] != 3 or t.shape[0] <= 0:
                raise ValueError("indices must have shape [triangle_count, 3]")
            if t.dtype.is_floating_point:
                raise ValueError("indices must be an integer tensor")
            if t.numel() and bool(((t.to(torch.int64) < 0) | (t.to(torch.int64) >= vertex_count)).any()):
                raise exc(msg)
            return t.to(self.ctx.device, torch.int32).contiguous()
        a = np.asarray(x)
        if a.ndim != 2 or a.shape[1] != 3 or a.shape[0] <= 0:
            raise ValueError("indices must have shape [triangle_count, 3]")
        a64 = a.astype(np.int64, copy=False)
        if a64.size and (a64.min() < 0 or a64.max() >= vertex_count):
            raise exc(msg)
        return torch.from_numpy(np.ascontiguousarray(a64.astype(np.uint32).view(np.int32))).to(self.ctx.device)

    def out(self, t: Optional[torch.Tensor]):
        if t is None:
            return None
        if self.numpy:
            return t.cpu().numpy()
        if self.out_device is not None and self.out_device != t.device:
            return t.to(self.out_device)
        return t


def _single_viewport(vp) -> bool:
    """True for one (x, y, width, height) viewport, False for a per-view sequence of them."""
    if isinstance(vp, (list, tuple)) and any(v is None or hasattr(v, "__len__") for v in vp):
        return False
    try:
        a = np.asarray(vp, dtype=np.float64)
    except (TypeError, ValueError):
        return False
    return a.ndim == 1 and a.shape[0] == 4


def _viewports(viewport, views: int, width: int, height: int, device) -> Tuple[torch.Tensor, list]:
    """src/rasterizer.cpp:48-59 resolve_viewport, per view."""
    if viewport is None or _single_viewport(viewport):
        per = [viewport] * views
    else:
        per = list(viewport)
        if len(per) != views:
            raise ValueError("viewports must contain one entry per view")
    rows = []
    for vp in per:
        if vp is None:
            vp = (0.0, 0.0, float(width), float(height))
        if len(vp) != 4:
            raise ValueError("viewport must be (x, y, width, height)")
        vp = [float(np.float32(v)) for v in vp]
        if not all(math.isfinite(v) for v in vp) or vp[2] <= 0.0 or vp[3] <= 0.0:
            raise ValueError("viewport must contain finite values and positive dimensions")
        rows.append(vp)
    return torch.tensor(rows, dtype=torch.float32, device=device), rows


class Rasterizer:
    """Differentiable rasterizer (reference: include/photara_drender/rasterizer.hpp)."""

    def __init__(self, device_index: int = 0, enable_validation: bool = False):
        self.context = Context(device_index, enable_validation)
        self._capacity = 0

    @property
    def device_info(self) -> DeviceInfo:
        return self.context.info

    # -- tile binning -------------------------------------------------------------------------
    def _bin(self, clip: torch.Tensor, idx: torch.Tensor, width: int, height: int, vps: torch.Tensor):
        ctx = self.context
        views, V = clip.shape[0], clip.shape[1]
        T = idx.shape[0]
        tiles = ((width + TILE - 1) // TILE) * ((height + TILE - 1) // TILE)
        offsets = torch.empty(views * tiles + 1, dtype=torch.int32, device=ctx.device)
        capacity = max(self._capacity, 2 * T * views + 1024)
        for _ in range(2):
            lst = torch.empty(capacity, dtype=torch.int32, device=ctx.device)
            ws_bytes = _native.lib().pdr_bin_tiles_workspace_bytes(views, T, width, height, capacity)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=ctx.device)
            ctx.status.zero_()
            _native.call("pdr_bin_tiles", _ptr(clip), views, V, _ptr(idx), T, width, height, _ptr(vps), _ptr(offsets),
                         _ptr(lst), capacity, _ptr(ws), ws_bytes, _ptr(ctx.status), ctx.stream())
            st = ctx.status.cpu()
            total = int(st[_native.STATUS_TILE_ENTRIES]) & 0xFFFFFFFF
            if int(st[_native.STATUS_TILE_ENTRIES_HI]) != 0:
                raise OverflowError("Tile triangle list exceeds backend limits")
            if not int(st[_native.STATUS_TILE_OVERFLOW]):
                self._capacity = max(self._capacity, capacity)
                return offsets, lst, capacity, total
            capacity = total + total // 8 + 1024
        raise RuntimeError("tile binning did not converge")

    def bin_tiles(self, positions, indices, resolution, viewport=None):
        """Tile bins of src/rasterizer.cpp:61-138: (offsets [views*tiles+1], triangle ids)."""
        with self.context.lock:
            io = _Io(self.context, positions, indices)
            clip = self._clip(io, positions)
            idx = io.indices(indices, clip.shape[1])
            h, w = int(resolution[0]), int(resolution[1])
            vps, _ = _viewports(viewport, clip.shape[0], w, h, self.context.device)
            offsets, lst, _, total = self._bin(clip, idx, w, h, vps)
            return io.out(offsets.view(torch.int32)), io.out(lst[:total])

    def _clip(self, io: _Io, positions) -> torch.Tensor:
        clip = io.f32(positions, "positions")
        if clip.ndim == 2:
            clip = clip.unsqueeze(0)
        if clip.ndim != 3 or clip.shape[2] != 4 or clip.shape[1] <= 0:
            raise ValueError("positions must have shape [vertex_count, 4]")
        return clip

    # -- rasterize ----------------------------------------------------------------------------
    def forward(self, positions, indices, resolution, cull_mode: str = "none",
                output_barycentric_derivatives: bool = True, viewport=None, *, clip_near_plane: bool = False):
        """Rasterizer::forward (src/rasterizer.cpp:373-442). resolution is (height, width).
        clip_near_plane clips triangles against the near plane z = -w first (the reference has no
        clipping: it drops triangles with a vertex at w <= 1e-8, README.md:140); ids, barycentrics,
        depth and derivatives stay those of the original triangles."""
        with self.context.lock:
            ctx = self.context
            cull = parse_cull_mode(cull_mode)
            io = _Io(ctx, positions, indices)
            clip = self._clip(io, positions)
            batched = _is_batched(positions)
            views, V = clip.shape[0], clip.shape[1]
            idx = io.indices(indices, V)
            h, w = int(resolution[0]), int(resolution[1])
            if h <= 0 or w <= 0:
                raise ValueError("Rasterization width and height must be positive")
            vps, _ = _viewports(viewport, views, w, h, ctx.device)
            raster = torch.empty((views, h, w, 4), dtype=torch.float32, device=ctx.device)
            deriv = torch.empty((views, h, w, 4), dtype=torch.float32, device=ctx.device) \
                if output_barycentric_derivatives else None
            if clip_near_plane:
                T = idx.shape[0]
                if T > NEAR_MAX_TRIANGLES:
                    raise OverflowError("near-plane clipping supports at most 8388608 triangles")
                cpos = torch.empty((views, 4 * T, 4), dtype=torch.float32, device=ctx.device)
                cidx = torch.empty((2 * T, 3), dtype=torch.int32, device=ctx.device)
                _native.call("pdr_clip_near", _ptr(clip), views, V, _ptr(idx), T, _ptr(cpos), _ptr(cidx), None,
                             ctx.stream())
                offsets, lst, capacity, _ = self._bin(cpos, cidx, w, h, vps)
                _native.call("pdr_rasterize_forward", _ptr(cpos), views, 4 * T, _ptr(cidx), 2 * T, w, h, _ptr(vps),
                             cull, _ptr(offsets), _ptr(lst), capacity, _ptr(raster), _ptr(deriv), ctx.stream())
                _native.call("pdr_remap_near", _ptr(clip), views, V, _ptr(idx), T, w, h, _ptr(vps), _ptr(raster),
                             _ptr(deriv), ctx.stream())
            else:
                offsets, lst, capacity, _ = self._bin(clip, idx, w, h, vps)
                _native.call("pdr_rasterize_forward", _ptr(clip), views, V, _ptr(idx), idx.shape[0], w, h, _ptr(vps),
                             cull, _ptr(offsets), _ptr(lst), capacity, _ptr(raster), _ptr(deriv), ctx.stream())
            if deriv is None:
                deriv = torch.empty((views, 0, 0, 4), dtype=torch.float32, device=ctx.device)
            if not batched:
                raster, deriv = raster[0], deriv[0]
            return io.out(raster), io.out(deriv)

    def backward(self, positions, indices, raster, grad_raster, viewport=None, *, grad_barycentric_derivatives=None,
                 clip_near_plane: bool = False):
        """Rasterizer::backward (src/rasterizer.cpp:444-537); returns d loss / d clip positions.
        grad_barycentric_derivatives ([H, W, 4], like the forward's derivative output) adds the gradient
        through the pixel derivatives, which the reference rejects (src/rasterizer.cpp:459-462).
        clip_near_plane is the adjoint of forward(..., clip_near_plane=True): triangles with a vertex at
        w <= 1e-8 pass gradient on every pixel they own."""
        with self.context.lock:
            ctx = self.context
            io = _Io(ctx, positions, indices, raster, grad_raster)
            clip = self._clip(io, positions)
            batched = _is_batched(positions)
            views, V = clip.shape[0], clip.shape[1]
            idx = io.indices(indices, V)
            r = io.f32(raster, "raster")
            g = io.f32(grad_raster, "grad_raster")
            r = r.unsqueeze(0) if r.ndim == 3 else r
            g = g.unsqueeze(0) if g.ndim == 3 else g
            if r.ndim != 4 or r.shape[3] != 4 or r.shape[0] != views:
                raise ValueError("raster must have shape [height, width, 4]")
            if g.shape != r.shape:
                raise ValueError("grad_raster must have shape [height, width, 4]")
            h, w = r.shape[1], r.shape[2]
            vps, _ = _viewports(viewport, views, w, h, ctx.device)
            out = torch.empty((views, V, 4), dtype=torch.float32, device=ctx.device)
            gd = None
            if grad_barycentric_derivatives is not None:
                gd = io.f32(grad_barycentric_derivatives, "grad_barycentric_derivatives")
                gd = gd.unsqueeze(0) if gd.ndim == 3 else gd
                if gd.shape != r.shape:
                    raise ValueError("grad_barycentric_derivatives must have shape [height, width, 4]")
            if clip_near_plane:
                _native.call("pdr_rasterize_backward_near", _ptr(clip), views, V, _ptr(idx), idx.shape[0], w, h,
                             _ptr(vps), _ptr(r), _ptr(g), _ptr(gd), _ptr(out), ctx.stream())
            elif gd is None:
                _native.call("pdr_rasterize_backward", _ptr(clip), views, V, _ptr(idx), idx.shape[0], w, h,
                             _ptr(vps), _ptr(r), _ptr(g), _ptr(out), ctx.stream())
            else:
                _native.call("pdr_rasterize_backward_derivatives", _ptr(clip), views, V, _ptr(idx), idx.shape[0], w,
                             h, _ptr(vps), _ptr(r), _ptr(g), _ptr(gd), _ptr(out), ctx.stream())
            return io.out(out if batched else out[0])

    # -- interpolate --------------------------------------------------------------------------
    def _attr_raster(self, io, vertex_attributes, raster):
        attr = io.f32(vertex_attributes, "vertex_attributes")
        if attr.ndim not in (2, 3) or attr.shape[-2] <= 0 or attr.shape[-1] <= 0:
            raise ValueError("vertex_attributes must have shape [vertex_count, attribute_count]")
        r = io.f32(raster, "raster")
        batched = r.ndim == 4
        r = r.unsqueeze(0) if r.ndim == 3 else r
        if r.ndim != 4 or r.shape[3] != 4:
            raise ValueError("raster must have shape [height, width, 4]")
        views = r.shape[0]
        if attr.ndim == 3:
            if attr.shape[0] != views:
                raise ValueError("per-view vertex_attributes must match the raster's view count")
            stride = attr.shape[1] * attr.shape[2]
        else:
            stride = 0
        return attr, r, stride, batched

    def interpolate_forward(self, vertex_attributes, indices, raster):
        """Rasterizer::interpolate_forward (src/rasterizer.cpp:539-601)."""
        with self.context.lock:
            ctx = self.context
            io = _Io(ctx, vertex_attributes, indices, raster)
            attr, r, stride, batched = self._attr_raster(io, vertex_attributes, raster)
            V, A = attr.shape[-2], attr.shape[-1]
            idx = io.indices(indices, V, IndexError, "triangle_indices contains an invalid attribute vertex index")
            views, h, w = r.shape[0], r.shape[1], r.shape[2]
            out = torch.empty((views, h, w, A), dtype=torch.float32, device=ctx.device)
            _native.call("pdr_interpolate_forward", _ptr(attr), stride, V, A, _ptr(idx), idx.shape[0], _ptr(r), views,
                         h * w, _ptr(out), ctx.stream())
            return io.out(out if batched else out[0])

    def interpolate_backward(self, vertex_attributes, indices, raster, grad_interpolated):
        """Rasterizer::interpolate_backward (src/rasterizer.cpp:603-683): (grad_attributes, grad_raster)."""
        with self.context.lock:
            ctx = self.context
            io = _Io(ctx, vertex_attributes, indices, raster, grad_interpolated)
            attr, r, stride, batched = self._attr_raster(io, vertex_attributes, raster)
            V, A = attr.shape[-2], attr.shape[-1]
            idx = io.indices(indices, V, ValueError, "triangle_indices is incompatible with vertex_attributes")
            views, h, w = r.shape[0], r.shape[1], r.shape[2]
            g = io.f32(grad_interpolated, "grad_interpolated")
            g = g.unsqueeze(0) if g.ndim == 3 else g
            if tuple(g.shape) != (views, h, w, A):
                raise ValueError("grad_interpolated must have shape [height, width, attribute_count]")
            ga = torch.empty(attr.shape, dtype=torch.float32, device=ctx.device)
            gr = torch.empty((views, h, w, 4), dtype=torch.float32, device=ctx.device)
            _native.call("pdr_interpolate_backward", _ptr(attr), stride, V, A, _ptr(idx), idx.shape[0], _ptr(r), views,
                         h * w, _ptr(g), _ptr(ga), _ptr(gr), ctx.stream())
            return io.out(ga), io.out(gr if batched else gr[0])

    # -- texture ------------------------------------------------------------------------------
    def _texture_inputs(self, io, texture, uv, raster):
        tex = io.f32(texture, "texture")
        if tex.ndim not in (3, 4) or min(tex.shape[-3:]) <= 0:
            raise ValueError("texture must have shape [texture_height, texture_width, channel_count]")
        r = io.f32(raster, "raster")
        batched = r.ndim == 4
        r = r.unsqueeze(0) if r.ndim == 3 else r
        if r.ndim != 4 or r.shape[3] != 4:
            raise ValueError("raster must have shape [image_height, image_width, 4]")
        u = io.f32(uv, "uv")
        u = u.unsqueeze(0) if u.ndim == 3 else u
        if u.ndim != 4 or u.shape[:3] != r.shape[:3] or u.shape[3] != 2:
            raise ValueError("uv must have shape [image_height, image_width, 2]")
        views = r.shape[0]
        if tex.ndim == 4:
            if tex.shape[0] != views:
                raise ValueError("per-view textures must match the raster's view count")
            stride = tex.shape[1] * tex.shape[2] * tex.shape[3]
        else:
            stride = 0
        return tex, u, r, stride, batched

    def texture_forward(self, texture, uv, raster, address_mode: str = "clamp"):
        """Rasterizer::texture_forward (src/rasterizer.cpp:685-735)."""
        with self.context.lock:
            ctx = self.context
            mode = parse_address_mode(address_mode)
            io = _Io(ctx, texture, uv, raster)
            tex, u, r, stride, batched = self._texture_inputs(io, texture, uv, raster)
            th, tw, Cc = tex.shape[-3], tex.shape[-2], tex.shape[-1]
            views, h, w = r.shape[0], r.shape[1], r.shape[2]
            out = torch.empty((views, h, w, Cc), dtype=torch.float32, device=ctx.device)
            _native.call("pdr_texture_forward", _ptr(tex), stride, tw, th, Cc, mode, _ptr(u), _ptr(r), views, h * w,
                         _ptr(out), ctx.stream())
            return io.out(out if batched else out[0])

    def texture_backward(self, texture, uv, raster, grad_sampled, address_mode: str = "clamp",
                         compute_uv_gradient: bool = True):
        """Rasterizer::texture_backward (src/rasterizer.cpp:737-829): (grad_texture, grad_uv or None)."""
        with self.context.lock:
            ctx = self.context
            mode = parse_address_mode(address_mode)
            io = _Io(ctx, texture, uv, raster, grad_sampled)
            tex, u, r, stride, batched = self._texture_inputs(io, texture, uv, raster)
            th, tw, Cc = tex.shape[-3], tex.shape[-2], tex.shape[-1]
            views, h, w = r.shape[0], r.shape[1], r.shape[2]
            g = io.f32(grad_sampled, "grad_sampled")
            g = g.unsqueeze(0) if g.ndim == 3 else g
            if tuple(g.shape) != (views, h, w, Cc):
                raise ValueError("grad_sampled must have shape [image_height, image_width, channel_count]")
            gt = torch.empty(tex.shape, dtype=torch.float32, device=ctx.device)
            gu = torch.empty((views, h, w, 2), dtype=torch.float32, device=ctx.device) if compute_uv_gradient else None
            ctx.status.zero_()
            _native.call("pdr_texture_backward", _ptr(tex), stride, tw, th, Cc, mode, _ptr(u), _ptr(r), views, h * w,
                         _ptr(g), _ptr(gt), _ptr(gu), _ptr(ctx.status), ctx.stream())
            err = int(ctx.status[_native.STATUS_TEXEL_ERROR].item())
            if err == 1:
                raise ValueError("uv contains a non-finite value in a covered pixel")
            if err == 2:
                raise IndexError("uv is too large for portable texture addressing")
            if gu is not None and not batched:
                gu = gu[0]
            return io.out(gt), io.out(gu)


def _is_batched(positions) -> bool:
    if isinstance(positions, (np.ndarray, torch.Tensor)):
        return positions.ndim == 3
    return np.asarray(positions).ndim == 3

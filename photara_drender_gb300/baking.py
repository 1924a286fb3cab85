"""TextureBaker: the reference's `_photara_drender.TextureBaker` binding (python/bindings.cpp:156-412)
and `photara_drender.baking.project_texture_atlas` (python/photara_drender/baking.py:147-220) over the
GB300 C ABI.

bake(): atlas G-buffer raster, shadow rasters of every view in batched launches, and one projection
launch over all views (src/texture_baker.cpp:156-361). refine_texture(): per-view raster + uv caches,
then the whole Adam loop recorded as one CUDA graph (src/texture_refiner.cpp:174-454).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass
from typing import List, NamedTuple, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native
from .rasterizer import Context, DeviceInfo, Rasterizer, _Io, _ptr, _viewports

@dataclass
class _RefineState:
    """Validated refinement inputs and the per-view caches (device buffers kept alive in `keep`)."""
    io: object
    init: torch.Tensor
    options: "RefineOptionsC"
    table: object
    table_dev: torch.Tensor
    weights: list
    max_pixels: int
    pairs: Optional[torch.Tensor]
    npairs: int
    tv_valid: Optional[torch.Tensor]
    tv_chart: Optional[torch.Tensor]
    keep: list
    t0: float
    t1: float
    initial_is_tensor: bool


BLEND_MODES = {"best_view": 0, "weighted_average": 1, "softmax": 2}
VISIBILITY_MODES = {"shadow_map": 0, "hybrid_ray_query": 1, "ray_query": 2}


class ProjectionViewC(C.Structure):
    """include/pdr_capi.h pdr_projection_view (160 bytes)."""

    _fields_ = [
        ("world_to_clip", C.c_float * 16), ("camera_position", C.c_float * 3), ("weight", C.c_float),
        ("viewport", C.c_float * 4), ("width", C.c_uint32), ("height", C.c_uint32), ("channel_count", C.c_uint32),
        ("has_mask", C.c_uint32), ("depth_bias", C.c_float), ("min_view_cosine", C.c_float),
        ("mask_floor", C.c_float), ("reserved", C.c_float), ("image", C.c_void_p), ("visibility_mask", C.c_void_p),
        ("shadow_raster", C.c_void_p), ("ray_visibility", C.c_void_p),
    ]


class RefineViewC(C.Structure):
    """include/pdr_capi.h pdr_refine_view (32 bytes)."""

    _fields_ = [("uv", C.c_void_p), ("target", C.c_void_p), ("mask", C.c_void_p), ("pixel_count", C.c_uint64)]


class RefineOptionsC(C.Structure):
    """include/pdr_capi.h pdr_refine_options (types.hpp TextureRefineOptions + total variation)."""

    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("steps", C.c_uint32), ("batch_size", C.c_uint32),
        ("learning_rate", C.c_float), ("minimum_learning_rate", C.c_float), ("photometric_epsilon", C.c_float),
        ("adam_beta1", C.c_float), ("adam_beta2", C.c_float), ("adam_epsilon", C.c_float),
        ("clamp_min", C.c_float), ("clamp_max", C.c_float), ("seam_polish_steps", C.c_uint32),
        ("seam_learning_rate", C.c_float), ("seam_epsilon", C.c_float), ("tv_scale", C.c_float),
        ("tv_epsilon", C.c_float), ("texture_scratch", C.c_void_p),
    ]




@dataclass
class TextureBakeOutput:
    """include/photara_drender/types.hpp TextureBakeOutput."""

    width: int
    height: int
    color: np.ndarray
    confidence: np.ndarray
    source_view: np.ndarray
    valid_mask: np.ndarray
    coverage_mask: np.ndarray
    face_ids: np.ndarray
    used_ray_query: bool = False
    filled_mask: Optional[np.ndarray] = None  # texels extrapolated by padding / surface fill


class BakedTexture(NamedTuple):
    color: np.ndarray
    confidence: np.ndarray
    source_view: np.ndarray
    valid_mask: np.ndarray
    coverage_mask: np.ndarray
    used_ray_query: bool


class UnwrappedMesh(NamedTuple):
    positions: np.ndarray
    normals: np.ndarray
    uv: np.ndarray
    indices: np.ndarray
    vertex_remap: np.ndarray
    face_chart_ids: np.ndarray
    chart_count: int
    max_stretch: float
    partition_count: int = 1


def suggest_softmax_scale(positions, camera_positions) -> float:
    """src/texture_padding.cpp:187-224: 20 * min squared vertex-camera distance (double), vertices
    subsampled to at most ~10000."""
    pos = np.asarray(positions, dtype=np.float32).reshape(-1, 3)
    cams = np.asarray(camera_positions, dtype=np.float32).reshape(-1, 3)
    if pos.shape[0] < 1 or cams.shape[0] < 1:
        raise ValueError("positions must have shape [vertex_count, 3]")
    stride = max(1, pos.shape[0] // 10000)
    p = pos[::stride].astype(np.float64)
    p = p[np.isfinite(p).all(axis=1)]
    if p.shape[0] == 0:
        return 0.0
    c = cams.astype(np.float64)
    d = c[None, :, :] - p[:, None, :]
    sq = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    best = float(sq.min())
    if not math.isfinite(best) or best <= 0.0:
        return 0.0
    return float(np.float32(20.0 * best))


class TextureBaker:
    """Multi-view texture projection and atlas refinement (include/photara_drender/texture_baker.hpp,
    texture_refiner.hpp)."""

    def __init__(self, device_index: int = 0, enable_validation: bool = False):
        self.rasterizer = Rasterizer(device_index, enable_validation)
        self.context: Context = self.rasterizer.context

    @property
    def device_info(self) -> DeviceInfo:
        return self.context.info

    # -- helpers ---------------------------------------------------------------------------------
    def _rasters(self, clip: torch.Tensor, idx: torch.Tensor, sizes: List[Tuple[int, int]], viewports):
        """Rasterizes every view (no derivatives), batching views of equal size into one launch. The bins
        are the fused render's (unsorted: the raster does not depend on the order of a tile's triangles)
        and nothing waits for their entry count: tiles whose lists overflow the capacity are rasterized
        from all triangles with the binning rule, and the count sizes the capacity of later calls."""
        from .pipeline import RenderArgsC

        out: List[Optional[torch.Tensor]] = [None] * len(sizes)
        groups = {}
        for k, s in enumerate(sizes):
            groups.setdefault(s, []).append(k)
        ctx = self.context
        V, T = clip.shape[1], idx.shape[0]
        L = _native.lib()
        for kind, st in ctx.poll_status(kinds=("bake_raster",)):
            if kind == "bake_raster":
                self._raster_capacity = max(getattr(self, "_raster_capacity", 0),
                                            (st[_native.STATUS_TILE_ENTRIES] & 0xFFFFFFFF) * 9 // 8 + 1024)
        for (h, w), ks in groups.items():
            n = len(ks)
            sub = clip[ks].contiguous()
            vps, _ = _viewports([viewports[k] for k in ks], n, w, h, ctx.device)
            # 16x8 tiles with 128 staged triangles: the fused render's fastest shape on the bake's meshes and
            # views (the autotuner's pick for the 200k-triangle views); outputs are the same for every shape
            tw_, th_, stage = 16, 8, 128
            tiles = ((w + tw_ - 1) // tw_) * ((h + th_ - 1) // th_)
            # four tiles per triangle plus one entry per tile covers meshes of small triangles; a larger need
            # costs time on the first call only (the count then sizes later calls)
            capacity = max(getattr(self, "_raster_capacity", 0), 4 * T * n + tiles * n + 1024)
            offsets = torch.empty(n * tiles + 1, dtype=torch.int32, device=ctx.device)
            lst = torch.empty(capacity, dtype=torch.int32, device=ctx.device)
            ws_bytes = L.pdr_render_workspace_bytes_tiled(n, T, w, h, capacity, tw_, th_)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=ctx.device)
            raster = torch.empty((n, h, w, 4), dtype=torch.float32, device=ctx.device)
            a = RenderArgsC()
            a.clip_positions, a.views, a.vertex_count = sub.data_ptr(), n, V
            a.indices, a.triangle_count, a.width, a.height = idx.data_ptr(), T, w, h
            a.viewports, a.raster = vps.data_ptr(), raster.data_ptr()
            a.tile_offsets, a.tile_triangles, a.capacity = offsets.data_ptr(), lst.data_ptr(), capacity
            a.workspace, a.workspace_bytes, a.status = ws.data_ptr(), ws_bytes, ctx.status.data_ptr()
            a.tile_width, a.tile_height, a.stage_triangles = tw_, th_, stage
            ctx.status.zero_()
            _native.check(L.pdr_render_forward(C.addressof(a), ctx.stream()))
            ctx.defer_status("bake_raster")
            for j, k in enumerate(ks):
                out[k] = raster[j]
        return out

    def _transform(self, pos3: torch.Tensor, mats: torch.Tensor) -> torch.Tensor:
        views = mats.shape[0]
        clip = torch.empty((views, pos3.shape[0], 4), dtype=torch.float32, device=self.context.device)
        _native.call("pdr_transform_positions", _ptr(pos3), pos3.shape[0], _ptr(mats), views, _ptr(clip),
                     self.context.stream())
        return clip

    @staticmethod
    def _views_in(images, world_to_clip, visibility_masks, viewports, cameras=None):
        n = len(images)
        if n <= 0:
            raise ValueError("world_to_clip must have shape [view_count, 4, 4]")
        mats = np.asarray(world_to_clip.detach().cpu() if isinstance(world_to_clip, torch.Tensor) else world_to_clip,
                          dtype=np.float32)
        if mats.ndim != 3 or mats.shape != (n, 4, 4):
            raise ValueError("world_to_clip must have shape [view_count, 4, 4]")
        if cameras is not None:
            cams = np.asarray(cameras.detach().cpu() if isinstance(cameras, torch.Tensor) else cameras,
                              dtype=np.float32)
            if cams.ndim != 2 or cams.shape != (n, 3):
                raise ValueError("camera_positions must have shape [view_count, 3]")
        else:
            cams = None
        if visibility_masks is not None and len(visibility_masks) != n:
            raise ValueError("visibility_masks must contain one entry per view")
        if viewports is not None and len(viewports) != n:
            raise ValueError("viewports must contain one entry per view")
        return mats, cams

    # -- bake ------------------------------------------------------------------------------------
    def bake_output(self, positions, normals, uv, indices, images, world_to_clip, camera_positions,
                    visibility_masks=None, viewports=None, resolution=(1024, 1024), blend_mode="weighted_average",
                    visibility_mode="ray_query", pcf_radius=1, allow_visibility_fallback=True, softmax_scale=0.0,
                    mask_floor=0.0, weights=None, depth_bias=1e-3, min_view_cosine=0.05,
                    ray_origin_bias=1e-4) -> TextureBakeOutput:
        """TextureBaker::bake with every field of TextureBakeOutput (face_ids included)."""
        with self.context.lock:
            return self._bake(positions, normals, uv, indices, images, world_to_clip, camera_positions,
                              visibility_masks, viewports, resolution, blend_mode, visibility_mode, pcf_radius,
                              allow_visibility_fallback, softmax_scale, mask_floor, weights, depth_bias,
                              min_view_cosine, ray_origin_bias)

    def bake(self, positions, normals, uv, indices, images, world_to_clip, camera_positions, visibility_masks=None,
             viewports=None, resolution=(1024, 1024), blend_mode="weighted_average", visibility_mode="ray_query",
             pcf_radius=1, allow_visibility_fallback=True, softmax_scale=0.0, mask_floor=0.0):
        """python/bindings.cpp:161-287: (color, confidence, source_view, valid_mask, coverage_mask,
        used_ray_query)."""
        o = self.bake_output(positions, normals, uv, indices, images, world_to_clip, camera_positions,
                             visibility_masks, viewports, resolution, blend_mode, visibility_mode, pcf_radius,
                             allow_visibility_fallback, softmax_scale, mask_floor)
        return o.color, o.confidence, o.source_view, o.valid_mask, o.coverage_mask, o.used_ray_query

    def _bake(self, positions, normals, uv, indices, images, world_to_clip, camera_positions, visibility_masks,
              viewports, resolution, blend_mode, visibility_mode, pcf_radius, allow_visibility_fallback,
              softmax_scale, mask_floor, weights, depth_bias, min_view_cosine, ray_origin_bias):
        ctx = self.context
        if blend_mode not in BLEND_MODES:
            raise ValueError("blend_mode must be 'best_view', 'weighted_average', or 'softmax'")
        if visibility_mode not in VISIBILITY_MODES:
            raise ValueError("visibility_mode must be 'shadow_map', 'hybrid_ray_query', or 'ray_query'")
        io = _Io(ctx, positions, normals, uv, indices)
        pos = io.f32(positions, "positions")
        nrm = io.f32(normals, "normals")
        uvt = io.f32(uv, "uv")
        if pos.ndim != 2 or pos.shape[1] != 3 or pos.shape[0] <= 0:
            raise ValueError("positions must have shape [vertex_count, 3]")
        V = pos.shape[0]
        if tuple(nrm.shape) != (V, 3):
            raise ValueError("normals must have shape [vertex_count, 3]")
        if tuple(uvt.shape) != (V, 2):
            raise ValueError("uv must have shape [vertex_count, 2]")
        idx = io.indices(indices, V)
        mats, cams = self._views_in(images, world_to_clip, visibility_masks, viewports, camera_positions)
        n = len(images)
        h, w = int(resolution[0]), int(resolution[1])
        if (w <= 0 or h <= 0 or pcf_radius > 4 or pcf_radius < 0 or not math.isfinite(ray_origin_bias)
                or ray_origin_bias <= 0.0 or not math.isfinite(mask_floor) or mask_floor < 0.0 or mask_floor > 1.0):
            raise ValueError("atlas dimensions are invalid or pcf_radius exceeds 4")
        ray_requested = VISIBILITY_MODES[visibility_mode] != 0
        if ray_requested and not ctx.info.supports_ray_query and not allow_visibility_fallback:
            raise RuntimeError("ray-query visibility was requested but the selected device does not support it")
        effective_visibility = VISIBILITY_MODES[visibility_mode] if ctx.info.supports_ray_query else 0

        # per-view validation (texture_baker.cpp:62-79)
        imgs, masks, sizes, vps = [], [], [], []
        for k in range(n):
            img = io.f32(images[k], "image")
            if img.ndim != 3 or img.shape[0] <= 0 or img.shape[1] <= 0 or img.shape[2] not in (3, 4):
                raise ValueError("each image must have shape [height, width, 3 or 4]")
            m = None if visibility_masks is None else visibility_masks[k]
            if m is not None:
                m = io.f32(m, "mask")
                if tuple(m.shape) != tuple(img.shape[:2]):
                    raise ValueError("each visibility mask must have shape [image_height, image_width]")
            wt = 1.0 if weights is None else float(weights[k])
            if (not math.isfinite(wt) or wt < 0.0 or not math.isfinite(depth_bias) or depth_bias < 0.0
                    or not math.isfinite(min_view_cosine) or min_view_cosine < -1.0 or min_view_cosine > 1.0):
                raise ValueError("projection confidence parameters are invalid")
            vp = None if viewports is None else viewports[k]
            _, rows = _viewports(vp, 1, img.shape[1], img.shape[0], "cpu")
            imgs.append(img)
            masks.append(m)
            sizes.append((img.shape[0], img.shape[1]))
            vps.append(rows[0])

        # atlas G-buffer (texture_baker.cpp:182-204)
        aclip = torch.empty((1, V, 4), dtype=torch.float32, device=ctx.device)
        _native.call("pdr_atlas_clip_positions", _ptr(uvt), V, _ptr(aclip), ctx.stream())
        araster = self._rasters(aclip, idx, [(h, w)], [None])[0]
        apos = self.rasterizer.interpolate_forward(pos, idx, araster)
        anrm = self.rasterizer.interpolate_forward(nrm, idx, araster)

        scale = float(softmax_scale)
        if blend_mode == "softmax" and (not (scale > 0.0) or not math.isfinite(scale)):
            scale = suggest_softmax_scale(pos.cpu().numpy(), cams)
            if not (scale > 0.0) or not math.isfinite(scale):
                scale = 1.0

        shadows: List[Optional[torch.Tensor]] = [None] * n
        if effective_visibility != 2:
            clip = self._transform(pos, torch.from_numpy(mats).to(ctx.device))
            shadows = self._rasters(clip, idx, sizes, vps)
        table = (ProjectionViewC * n)()
        for k in range(n):
            v = table[k]
            v.world_to_clip[:] = [float(x) for x in mats[k].reshape(16)]
            v.camera_position[:] = [float(x) for x in cams[k]]
            wt = np.float32(1.0 if weights is None else weights[k])
            v.weight = float(np.float32(wt * np.float32(scale))) if blend_mode == "softmax" else float(wt)
            v.viewport[:] = vps[k]
            v.height, v.width, v.channel_count = imgs[k].shape
            v.has_mask = int(masks[k] is not None)
            v.depth_bias, v.min_view_cosine = depth_bias, min_view_cosine
            v.mask_floor = float(mask_floor) if masks[k] is not None else 0.0
            v.image = imgs[k].data_ptr()
            v.visibility_mask = masks[k].data_ptr() if masks[k] is not None else None
            v.shadow_raster = shadows[k].data_ptr() if shadows[k] is not None else None
            v.ray_visibility = None
        table_dev = torch.frombuffer(bytearray(bytes(table)), dtype=torch.uint8).to(ctx.device)
        ray_bits = None
        if effective_visibility != 0:
            ray_bits = self._ray_visibility(pos, idx, apos, anrm, araster, cams, ray_origin_bias, views=table_dev)

        N = h * w
        color = torch.empty((h, w, 4), dtype=torch.float32, device=ctx.device)
        conf = torch.empty((h, w), dtype=torch.float32, device=ctx.device)
        src = torch.empty((h, w), dtype=torch.int32, device=ctx.device)
        valid = torch.empty((h, w), dtype=torch.float32, device=ctx.device)
        cov = torch.empty((h, w), dtype=torch.float32, device=ctx.device)
        faces = torch.empty((h, w), dtype=torch.int32, device=ctx.device)
        if ray_bits is None:
            _native.call("pdr_project_views", _ptr(apos), _ptr(anrm), _ptr(araster), N, _ptr(table_dev), n,
                         BLEND_MODES[blend_mode], int(pcf_radius), effective_visibility, _ptr(color), _ptr(conf),
                         _ptr(src), _ptr(valid), _ptr(cov), _ptr(faces), ctx.stream())
        else:
            _native.call("pdr_project_views_bits", _ptr(apos), _ptr(anrm), _ptr(araster), N, _ptr(table_dev), n,
                         BLEND_MODES[blend_mode], int(pcf_radius), effective_visibility, _ptr(ray_bits), _ptr(color),
                         _ptr(conf), _ptr(src), _ptr(valid), _ptr(cov), _ptr(faces), ctx.stream())
        host = io.numpy or not isinstance(positions, torch.Tensor)

        def out(t, u32=False):
            if host:
                a = t.cpu().numpy()
                return a.view(np.uint32) if u32 else a
            return t

        return TextureBakeOutput(w, h, out(color), out(conf), out(src, True), out(valid), out(cov), out(faces, True),
                                 ray_bits is not None)

    def _ray_visibility(self, pos: torch.Tensor, idx: torch.Tensor, apos, anrm, araster, cams, bias: float,
                        views: Optional[torch.Tensor] = None):
        """project_ray_visibility.hlsl through a device BVH: camera-visibility bits [texels, ceil(views/32)].
        With `views` (the projection's device table) only the texel-views the projection reads are traced;
        the other bits are 0."""
        ctx = self.context
        V, T = pos.shape[0], idx.shape[0]
        bvh_bytes, build_bytes = C.c_size_t(), C.c_size_t()
        _native.call("pdr_bvh_sizes", T, C.byref(bvh_bytes), C.byref(build_bytes))
        bvh = torch.empty(bvh_bytes.value, dtype=torch.uint8, device=ctx.device)
        scratch = torch.empty(build_bytes.value, dtype=torch.uint8, device=ctx.device)
        _native.call("pdr_bvh_build", _ptr(pos), V, _ptr(idx), T, _ptr(bvh), bvh_bytes.value, _ptr(scratch),
                     build_bytes.value, ctx.stream())
        del scratch
        n = cams.shape[0]
        N = araster.numel() // 4
        bits = torch.empty((N, (n + 31) // 32), dtype=torch.int32, device=ctx.device)
        if views is not None:
            _native.call("pdr_ray_visibility_views", _ptr(bvh), T, _ptr(apos), _ptr(anrm), _ptr(araster), N,
                         _ptr(views), n, float(bias), _ptr(bits), ctx.stream())
            return bits
        cam4 = torch.zeros((n, 4), dtype=torch.float32, device=ctx.device)
        cam4[:, :3] = torch.from_numpy(np.ascontiguousarray(cams, dtype=np.float32)).to(ctx.device)
        _native.call("pdr_ray_visibility", _ptr(bvh), T, _ptr(apos), _ptr(anrm), _ptr(araster), N, _ptr(cam4), n,
                     float(bias), _ptr(bits), ctx.stream())
        return bits

    # -- refine ----------------------------------------------------------------------------------
    def refine_texture(self, initial_texture, positions, uv, indices, images, world_to_clip, visibility_masks=None,
                       viewports=None, seam_uv_pairs=None, steps=1000, batch_size=4, learning_rate=5e-3,
                       minimum_learning_rate=2.5e-4, photometric_epsilon=1e-3, seam_polish_steps=30,
                       seam_learning_rate=1e-3, *, adam_beta1=0.9, adam_beta2=0.999, adam_epsilon=1e-8,
                       clamp_min=0.0, clamp_max=1.0, seam_epsilon=1e-4, total_variation_weight=0.0,
                       atlas_valid_mask=None, chart_ids=None, total_variation_epsilon=1e-4, use_graph=True):
        """python/bindings.cpp:289-404 / TextureRefiner::refine: (color [H, W, 3], loss_history,
        seam_loss_history, precompute_seconds, optimization_seconds). The keyword-only total
        variation arguments add the chart-aware TV of atlas.py:84-115 (off by default)."""
        with self.context.lock:
            return self._refine(initial_texture, positions, uv, indices, images, world_to_clip, visibility_masks,
                                viewports, seam_uv_pairs, steps, batch_size, learning_rate, minimum_learning_rate,
                                photometric_epsilon, seam_polish_steps, seam_learning_rate, adam_beta1, adam_beta2,
                                adam_epsilon, clamp_min, clamp_max, seam_epsilon, total_variation_weight,
                                atlas_valid_mask, chart_ids, total_variation_epsilon, use_graph=use_graph)

    def _refine(self, *args, use_graph=True):
        st = self._refine_prepare(*args)
        return self._refine_finish(st, use_graph)

    def _refine_prepare(self, initial_texture, positions, uv, indices, images, world_to_clip, visibility_masks,
                        viewports, seam_uv_pairs, steps, batch_size, learning_rate, minimum_learning_rate,
                        photometric_epsilon, seam_polish_steps, seam_learning_rate, adam_beta1, adam_beta2,
                        adam_epsilon, clamp_min, clamp_max, seam_epsilon, tv_weight, atlas_valid_mask, chart_ids,
                        tv_epsilon) -> "_RefineState":
        """texture_refiner.cpp:174-253: validation, options and the per-view caches (uv, target, mask)."""
        ctx = self.context
        t0 = time.perf_counter()
        io = _Io(ctx, initial_texture, positions, uv, indices)
        init = io.f32(initial_texture, "initial_texture")
        if init.ndim != 3 or init.shape[0] <= 0 or init.shape[1] <= 0 or init.shape[2] != 3:
            raise ValueError("initial_texture must have shape [height, width, 3]")
        pos = io.f32(positions, "positions")
        uvt = io.f32(uv, "uv")
        if pos.ndim != 2 or pos.shape[0] <= 0 or pos.shape[1] != 3 or tuple(uvt.shape) != (pos.shape[0], 2):
            raise ValueError("positions and uv must have shapes [vertex_count, 3] and [vertex_count, 2]")
        V = pos.shape[0]
        idx = io.indices(indices, V, ValueError, "texture refinement mesh arrays have inconsistent shapes")
        mats, _ = self._views_in(images, world_to_clip, visibility_masks, viewports)
        n = len(images)
        H, W = init.shape[0], init.shape[1]
        o = RefineOptionsC()
        o.width, o.height, o.steps, o.batch_size = W, H, int(steps), int(batch_size)
        o.learning_rate, o.minimum_learning_rate = learning_rate, minimum_learning_rate
        o.photometric_epsilon, o.adam_beta1, o.adam_beta2 = photometric_epsilon, adam_beta1, adam_beta2
        o.adam_epsilon, o.clamp_min, o.clamp_max = adam_epsilon, clamp_min, clamp_max
        o.seam_polish_steps, o.seam_learning_rate, o.seam_epsilon = int(seam_polish_steps), seam_learning_rate, seam_epsilon
        o.tv_epsilon = tv_epsilon
        pairs = None
        if seam_uv_pairs is not None:
            pairs = io.f32(seam_uv_pairs, "seam_uv_pairs")
            if pairs.ndim != 3 or pairs.shape[1:] != (2, 2):
                raise ValueError("seam_uv_pairs must have shape [pair_count, 2, 2]")
        npairs = 0 if pairs is None else pairs.shape[0]
        tv_valid = tv_chart = None
        tv_scale = 0.0
        if tv_weight:
            valid = torch.ones((H, W), dtype=torch.bool, device=ctx.device) if atlas_valid_mask is None else \
                io.f32(atlas_valid_mask, "atlas_valid_mask").bool()
            chart = None if chart_ids is None else torch.as_tensor(np.asarray(chart_ids) if not isinstance(
                chart_ids, torch.Tensor) else chart_ids).to(ctx.device, torch.int32).contiguous()
            hm = valid[:, 1:] & valid[:, :-1]
            vm = valid[1:, :] & valid[:-1, :]
            if chart is not None:
                hm &= chart[:, 1:] == chart[:, :-1]
                vm &= chart[1:, :] == chart[:-1, :]
            count = int(hm.sum().item() + vm.sum().item())
            tv_scale = float(np.float32(tv_weight / (max(count, 1) * 3)))
            tv_valid = valid.to(torch.uint8).contiguous()
            tv_chart = chart
        o.tv_scale = tv_scale

        # texture_refiner.cpp:206-253: per-view caches
        imgs, masks, sizes, vps = [], [], [], []
        for k in range(n):
            img = io.f32(images[k], "image")
            if img.ndim != 3 or img.shape[0] <= 0 or img.shape[1] <= 0 or img.shape[2] not in (3, 4):
                raise ValueError("each image must have shape [height, width, 3 or 4]")
            m = None if visibility_masks is None else visibility_masks[k]
            if m is not None:
                m = io.f32(m, "mask")
                if tuple(m.shape) != tuple(img.shape[:2]):
                    raise ValueError("each visibility mask must match its image dimensions")
            vp = None if viewports is None else viewports[k]
            _, rows = _viewports(vp, 1, img.shape[1], img.shape[0], "cpu")
            imgs.append(img)
            masks.append(m)
            sizes.append((img.shape[0], img.shape[1]))
            vps.append(rows[0])
        clip = self._transform(pos, torch.from_numpy(mats).to(ctx.device))
        rasters = self._rasters(clip, idx, sizes, vps)
        table = (RefineViewC * n)()
        keep, weights = [], []
        for k in range(n):
            P = sizes[k][0] * sizes[k][1]
            uvk = self.rasterizer.interpolate_forward(uvt, idx, rasters[k])
            tgt = torch.empty((P, 3), dtype=torch.float32, device=ctx.device)
            msk = torch.empty((P,), dtype=torch.float32, device=ctx.device)
            _native.call("pdr_refine_prepare_view", _ptr(imgs[k]), imgs[k].shape[2], _ptr(masks[k]), _ptr(rasters[k]),
                         P, _ptr(tgt), _ptr(msk), ctx.stream())
            keep += [uvk, tgt, msk]
            weights.append(float(msk.double().sum().item()))
            table[k].uv, table[k].target, table[k].mask, table[k].pixel_count = (uvk.data_ptr(), tgt.data_ptr(),
                                                                                 msk.data_ptr(), P)
        table_dev = torch.frombuffer(bytearray(bytes(table)), dtype=torch.uint8).to(ctx.device)
        max_pixels = max(s[0] * s[1] for s in sizes)
        torch.cuda.synchronize(ctx.device)
        t1 = time.perf_counter()

        return _RefineState(io=io, init=init, options=o, table=table, table_dev=table_dev, weights=weights,
                            max_pixels=max_pixels, pairs=pairs, npairs=npairs, tv_valid=tv_valid, tv_chart=tv_chart,
                            keep=keep, t0=t0, t1=t1, initial_is_tensor=isinstance(initial_texture, torch.Tensor))

    def _refine_finish(self, st: "_RefineState", use_graph: bool, precond=None):
        """Runs the optimisation (plain, or learned when `precond` is a pdr_precond_run structure)."""
        ctx = self.context
        o = st.options
        init, pairs, npairs = st.init, st.pairs, st.npairs
        steps, seam_polish_steps = int(o.steps), int(o.seam_polish_steps)
        t1 = st.t1
        tex = init.clone().contiguous()
        grad = torch.empty((tex.shape[0], tex.shape[1], 4), dtype=torch.float32, device=tex.device)  # RGB + pad
        m1 = torch.empty_like(tex)
        m2 = torch.empty_like(tex)
        seam_steps = 0 if npairs == 0 else int(seam_polish_steps)
        loss = torch.empty(int(steps) + seam_steps, dtype=torch.float32, device=ctx.device)
        n = len(st.weights)
        vw = (C.c_double * n)(*st.weights)
        # a second atlas buffer lets the plain refinement run each step's TV gradient and Adam update as one
        # pass (bit-identical; the result ends in tex)
        scratch = torch.empty_like(tex) if precond is None and float(o.tv_scale) > 0.0 else None
        o.texture_scratch = scratch.data_ptr() if scratch is not None else None
        if precond is None:
            _native.call("pdr_refine_run", C.addressof(o), _ptr(st.table_dev), n, C.addressof(vw), st.max_pixels,
                         _ptr(pairs), npairs, _ptr(st.tv_valid), _ptr(st.tv_chart), _ptr(tex), _ptr(grad), _ptr(m1),
                         _ptr(m2), _ptr(loss), int(bool(use_graph)), ctx.stream())
        else:
            _native.call("pdr_refine_run_learned", C.addressof(o), _ptr(st.table_dev), n, C.addressof(vw),
                         st.max_pixels, _ptr(pairs), npairs, _ptr(st.tv_valid), _ptr(st.tv_chart), _ptr(tex),
                         _ptr(grad), _ptr(m1), _ptr(m2), _ptr(loss), C.addressof(precond), int(bool(use_graph)),
                         ctx.stream())
        torch.cuda.synchronize(ctx.device)
        t2 = time.perf_counter()
        color = tex
        hist = loss[: int(steps)]
        seam = loss[int(steps):]
        if st.io.numpy or not st.initial_is_tensor:
            color, hist, seam = color.cpu().numpy(), hist.cpu().numpy(), seam.cpu().numpy()
        return color, hist, seam, t1 - st.t0, t2 - t1


def project_texture_atlas(mesh: UnwrappedMesh, images: Sequence[np.ndarray], world_to_clip, camera_positions, *,
                          baker: Optional[TextureBaker] = None, device_index: int = 0, visibility_masks=None,
                          viewports=None, resolution=(1024, 1024), blend_mode="weighted_average",
                          visibility_mode="ray_query", pcf_radius=1, allow_visibility_fallback=True,
                          softmax_scale=0.0, mask_floor=0.0, padding=0, fill_unobserved=False,
                          maximum_fill_distance=0) -> BakedTexture:
    """python/photara_drender/baking.py:147-220."""
    if baker is None:
        baker = TextureBaker(device_index=device_index)
    out = baker.bake(mesh.positions, mesh.normals, mesh.uv, mesh.indices, list(images), world_to_clip,
                     camera_positions, visibility_masks=visibility_masks, viewports=viewports, resolution=resolution,
                     blend_mode=blend_mode, visibility_mode=visibility_mode, pcf_radius=pcf_radius,
                     allow_visibility_fallback=allow_visibility_fallback, softmax_scale=float(softmax_scale),
                     mask_floor=float(mask_floor))
    baked = BakedTexture(*out)
    if padding or fill_unobserved:
        from .padding import pad_texture_atlas

        baked = baked._replace(color=pad_texture_atlas(baked.color, baked.valid_mask, padding,
                                                       coverage_mask=baked.coverage_mask,
                                                       fill_unobserved=fill_unobserved,
                                                       maximum_fill_distance=maximum_fill_distance))
    return baked

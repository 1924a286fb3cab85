"""ctypes binding of libphotara_drender_gb300.so (the C ABI declared in include/pdr_capi.h).

The shared library is the only compute path: importing this module fails loudly when it is
missing, and every call raises the exception type the reference's bindings raise for the
matching C++ exception (ValueError, IndexError, OverflowError, RuntimeError).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libphotara_drender_gb300.so")

_lib = None
_lock = threading.Lock()

PDR_OK = 0
_ERRORS = {-1: ValueError, -2: IndexError, -3: OverflowError, -4: RuntimeError, -5: NotImplementedError}

STATUS_WORDS = 8
STATUS_TILE_ENTRIES = 0
STATUS_TILE_ENTRIES_HI = 1
STATUS_TILE_OVERFLOW = 2
STATUS_TEXEL_ERROR = 4
STATUS_INDEX_ERROR = 5
STATUS_PRECOND_TIMEOUT = 6
STATUS_PAD_ERROR = 7

_vp = C.c_void_p
_u32 = C.c_uint32
_u64 = C.c_uint64
_i32 = C.c_int32
_sz = C.c_size_t

_SIGNATURES = {
    "pdr_last_error": (C.c_char_p, []),
    "pdr_version": (_i32, []),
    "pdr_device_count": (_i32, []),
    "pdr_device_info": (_i32, [_i32, C.c_char_p, _sz, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32),
                               C.POINTER(_i32)]),
    "pdr_validate_indices": (_i32, [_vp, _u64, _u32, _vp, _vp]),
    "pdr_bin_tiles_workspace_bytes": (_sz, [_u32, _u32, _u32, _u32, _u64]),
    "pdr_bin_tiles": (_i32, [_vp, _u32, _u32, _vp, _u32, _u32, _u32, _vp, _vp, _vp, _u64, _vp, _sz, _vp, _vp]),
    "pdr_rasterize_forward": (_i32, [_vp, _u32, _u32, _vp, _u32, _u32, _u32, _vp, _u32, _vp, _vp, _u64, _vp, _vp,
                                     _vp]),
    "pdr_rasterize_backward": (_i32, [_vp, _u32, _u32, _vp, _u32, _u32, _u32, _vp, _vp, _vp, _vp, _vp]),
    "pdr_rasterize_backward_derivatives": (_i32, [_vp, _u32, _u32, _vp, _u32, _u32, _u32, _vp, _vp, _vp, _vp, _vp,
                                                  _vp]),
    "pdr_clip_near": (_i32, [_vp, _u32, _u32, _vp, _u32, _vp, _vp, _vp, _vp]),
    "pdr_remap_near": (_i32, [_vp, _u32, _u32, _vp, _u32, _u32, _u32, _vp, _vp, _vp, _vp]),
    "pdr_rasterize_backward_near": (_i32, [_vp, _u32, _u32, _vp, _u32, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp]),
    "pdr_interpolate_forward": (_i32, [_vp, _u64, _u32, _u32, _vp, _u32, _vp, _u32, _u64, _vp, _vp]),
    "pdr_interpolate_backward": (_i32, [_vp, _u64, _u32, _u32, _vp, _u32, _vp, _u32, _u64, _vp, _vp, _vp, _vp]),
    "pdr_interpolate_backward_accumulate": (_i32, [_vp, _u64, _u32, _u32, _vp, _u32, _vp, _u32, _u64, _vp, _vp,
                                                   _vp, _vp]),
    "pdr_texture_forward": (_i32, [_vp, _u64, _u32, _u32, _u32, _u32, _vp, _vp, _u32, _u64, _vp, _vp]),
    "pdr_texture_backward": (_i32, [_vp, _u64, _u32, _u32, _u32, _u32, _vp, _vp, _u32, _u64, _vp, _vp, _vp, _vp,
                                    _vp]),
    "pdr_render_workspace_bytes": (_sz, [_u32, _u32, _u32, _u32, _u64]),
    "pdr_render_forward": (_i32, [_vp, _vp]),
    "pdr_render_bin": (_i32, [_vp, _vp]),
    "pdr_render_raster": (_i32, [_vp, _vp]),
    "pdr_render_backward": (_i32, [_vp, _vp]),
    "pdr_transform_positions": (_i32, [_vp, _u32, _vp, _u32, _vp, _vp]),
    "pdr_atlas_clip_positions": (_i32, [_vp, _u32, _vp, _vp]),
    "pdr_project_views": (_i32, [_vp, _vp, _vp, _u32, _vp, _u32, _u32, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp,
                                 _vp]),
    "pdr_bvh_sizes": (_i32, [_u32, _vp, _vp]),
    "pdr_bvh_build": (_i32, [_vp, _u32, _vp, _u32, _vp, _sz, _vp, _sz, _vp]),
    "pdr_ray_visibility": (_i32, [_vp, _u32, _vp, _vp, _vp, _u32, _vp, _u32, C.c_float, _vp, _vp]),
    "pdr_ray_visibility_views": (_i32, [_vp, _u32, _vp, _vp, _vp, _u32, _vp, _u32, C.c_float, _vp, _vp]),
    "pdr_project_views_bits": (_i32, [_vp, _vp, _vp, _u32, _vp, _u32, _u32, _u32, _u32, _vp, _vp, _vp, _vp, _vp,
                                      _vp, _vp, _vp]),
    "pdr_pad_workspace_bytes": (_i32, [_u32, _u32, _u32, _vp]),
    "pdr_pad_texture_atlas": (_i32, [_vp, _u32, _vp, _vp, _vp, _u32, _u32, _u32, _u32, _u32, C.c_float, _vp, _sz, _vp,
                                     _vp, _vp]),
    "pdr_surface_fill_workspace_bytes": (_i32, [_u32, _u32, _u32, _vp]),
    "pdr_fill_texture_on_surface": (_i32, [_vp, _u32, _vp, _vp, _vp, _u32, _u32, _vp, _u32, _vp, _sz, _vp, _vp, _vp]),
    "pdr_mip_pyramid_size": (_i32, [_u32, _u32, _u32, _vp, _vp]),
    "pdr_mip_build": (_i32, [_vp, _u32, _u32, _u32, _u32, _vp, _vp]),
    "pdr_texture_forward_mip": (_i32, [_vp, _vp, _u32, _u32, _u32, _u32, _u32, _vp, _vp, _vp, _u32, _u64, _vp, _vp]),
    "pdr_texture_backward_mip": (_i32, [_vp, _vp, _u32, _u32, _u32, _u32, _u32, _vp, _vp, _vp, _u32, _u64, _vp, _vp,
                                        _vp, _vp, _vp]),
    "pdr_interpolate_derivatives": (_i32, [_vp, _u32, _u32, _vp, _u32, _vp, _vp, _u32, _u64, _vp, _vp]),
    "pdr_refine_prepare_view": (_i32, [_vp, _u32, _vp, _vp, _u64, _vp, _vp, _vp]),
    "pdr_refine_photometric": (_i32, [_vp, _u32, _u32, _vp, _u32, _u64, _u32, _u32, C.c_float, C.c_float, _vp, _vp,
                                      _vp]),
    "pdr_calibrate_reductions": (_i32, [_vp, _u64, _u64, _u32, _vp]),
    "pdr_render_workspace_bytes_tiled": (_sz, [_u32, _u32, _u32, _u32, _u64, _u32, _u32]),
    "pdr_render_backward_workspace_bytes": (_sz, [_u32, _u32, _u32]),
    "pdr_refine_seam": (_i32, [_vp, _u32, _u32, _vp, _u32, C.c_float, C.c_float, _vp, _vp, _u32, _vp]),
    "pdr_refine_total_variation": (_i32, [_vp, _u32, _u32, _vp, _vp, C.c_float, C.c_float, _vp, _vp]),
    "pdr_refine_adam": (_i32, [_vp, _vp, _vp, _vp, _u64] + [C.c_float] * 8 + [_vp]),
    "pdr_refine_schedule": (_i32, [_vp, _u32, _vp, _vp, _vp]),
    "pdr_refine_run": (_i32, [_vp, _vp, _u32, _vp, _u64, _vp, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp]),
    "pdr_refine_graph_create": (_i32, [_vp, _vp, _vp, _u32, _vp, _u64, _vp, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                       _vp]),
    "pdr_refine_graph_launch": (_i32, [_vp, _vp]),
    "pdr_refine_graph_destroy": (_i32, [_vp]),
    "pdr_precond_forward": (_i32, [_vp, _vp, _vp, _u64, _vp, _vp, _vp]),
    "pdr_precond_train_step": (_i32, [_vp, _vp, _vp, _vp, _vp, _u64, C.c_float, _vp, _vp, _vp, _vp]),
    "pdr_precond_adam": (_i32, [_vp, _vp, _vp, _vp, _u32, C.c_float, C.c_float, C.c_float, C.c_float, _vp, _vp]),
    "pdr_precond_texel_stats": (_i32, [_vp, _u32, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "pdr_precond_features": (_i32, [_vp, _vp, _vp, C.c_float, C.c_float, C.c_float, _vp, _vp, _vp, C.c_float, _u64,
                                    _vp, _vp]),
    "pdr_refine_adam_scaled": (_i32, [_vp, _vp, _vp, _vp, _u64, _vp, _vp] + [C.c_float] * 8 + [_vp]),
    "pdr_precond_fallback_check": (_i32, [_vp, _u32, _u32, C.c_float, _vp, _vp]),
    "pdr_refine_run_learned": (_i32, [_vp, _vp, _u32, _vp, _u64, _vp, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                      _i32, _vp]),
    "pdr_render_batch_sizes": (_i32, [_vp, _u32, _vp, _u32, _vp, _vp]),
    "pdr_render_batch_forward": (_i32, [_vp, _u32, _u32, _u32, _u32, _vp, _vp, _vp, _u64, _vp, _sz, _vp, _vp]),
    "pdr_render_batch_backward": (_i32, [_vp, _u32, _u32, _u32, _vp, _vp, _sz, _vp, _vp]),
}

OPTIONAL_SIGNATURES: dict = {}


def lib():
    """Loads the native library, raising ImportError with build instructions when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing; build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                    "or `python photara_drender_gb300/build.py` (needs nvcc for sm_103a)")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in {**_SIGNATURES, **OPTIONAL_SIGNATURES}.items():
                fn = getattr(L, name, None)
                if fn is None:
                    if name in _SIGNATURES:
                        raise ImportError(f"{LIB_PATH} does not export {name}")
                    continue
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status: int) -> None:
    if status != PDR_OK:
        msg = lib().pdr_last_error().decode("utf-8", "replace")
        raise _ERRORS.get(int(status), RuntimeError)(msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))

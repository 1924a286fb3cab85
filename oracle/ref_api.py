"""NumPy face of ``libpdr_ref.so``: the reference's own HLSL shaders (and its CPU
``texture_padding.cpp``) compiled for the CPU. TEST INFRASTRUCTURE ONLY.

The reference's host-side routines of the path come from its own source as well: tile binning
(src/rasterizer.cpp:61-138 build_tile_bins), the vertex->corner table (:145-162) and the
texel->sample table with double-precision weights (:187-258), cut out of ``src/rasterizer.cpp``
by ``oracle/build.py`` (the rest of that file needs the absent Vulkan wrapper).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import api

_f32p = C.POINTER(C.c_float)
_u32p = C.POINTER(C.c_uint32)


def available() -> bool:
    return api.ref() is not None


def _L():
    L = api.ref()
    if L is None:
        raise RuntimeError("reference sources are not available on this machine")
    L.ref_suggest_softmax_scale.restype = C.c_float
    L.ref_build_tile_bins.restype = C.c_int64
    L.ref_build_texture_sample_adjacency.restype = C.c_int64
    return L


def _p(a, t=_f32p):
    return a.ctypes.data_as(t) if a is not None else None


def bin_tiles(pos, idx, resolution, viewport=None):
    """src/rasterizer.cpp:61-138 build_tile_bins: (offsets [tiles+1], ascending triangle ids)."""
    pos, idx = api._f(pos), api._u(idx)
    h, w = resolution
    vp = api._vp(viewport, w, h)
    tiles = ((w + 15) // 16) * ((h + 15) // 16)
    offsets = np.zeros(tiles + 1, np.uint32)
    L = _L()
    n = L.ref_build_tile_bins(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, _p(vp),
                              _p(offsets, _u32p), None, C.c_uint64(0))
    if n < 0:
        raise OverflowError("Tile triangle list exceeds backend limits")
    lst = np.zeros(max(n, 1), np.uint32)
    L.ref_build_tile_bins(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, _p(vp), _p(offsets, _u32p),
                          _p(lst, _u32p), C.c_uint64(n))
    return offsets, lst[:n]


def rasterize_forward(pos, idx, resolution, cull_mode=0, output_derivatives=True, viewport=None):
    pos, idx = api._f(pos), api._u(idx)
    h, w = resolution
    vp = api._vp(viewport, w, h)
    offsets, lst = bin_tiles(pos, idx, resolution, vp)
    lst = np.ascontiguousarray(lst if lst.size else np.zeros(1, np.uint32))
    raster = np.zeros((h, w, 4), np.float32)
    deriv = np.zeros((h, w, 4), np.float32)
    _L().ref_rasterize_forward(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, cull_mode,
                               int(bool(output_derivatives)), _p(vp), (w + 15) // 16, _p(offsets, _u32p),
                               _p(lst, _u32p), _p(raster), _p(deriv))
    return raster, (deriv if output_derivatives else None)


def vertex_corner_table(idx, V):
    """src/rasterizer.cpp:145-162 build_vertex_adjacency: CSR of corners per vertex."""
    idx = api._u(idx)
    offsets = np.zeros(V + 1, np.uint32)
    corners = np.zeros(max(idx.size, 1), np.uint32)
    _L().ref_build_vertex_adjacency(_p(idx, _u32p), idx.shape[0], V, _p(offsets, _u32p), _p(corners, _u32p))
    return offsets, corners[:idx.size]


def rasterize_backward(pos, idx, raster, grad_raster, viewport=None):
    pos, idx, raster, grad_raster = api._f(pos), api._u(idx), api._f(raster), api._f(grad_raster)
    h, w = raster.shape[:2]
    vp = api._vp(viewport, w, h)
    T, V = idx.shape[0], pos.shape[0]
    corner = np.zeros((T * 3, 4), np.float32)
    L = _L()
    L.ref_rasterize_backward(_p(pos), V, _p(idx, _u32p), T, w, h, _p(vp), _p(raster), _p(grad_raster), _p(corner))
    off, corners = vertex_corner_table(idx, V)
    out = np.zeros((V, 4), np.float32)
    L.ref_reduce_vertex_gradients(_p(off, _u32p), _p(corners, _u32p), _p(corner), V, _p(out))
    return out


def interpolate_forward(attr, idx, raster):
    attr, idx, raster = api._f(attr), api._u(idx), api._f(raster)
    h, w = raster.shape[:2]
    V, A = attr.shape
    out = np.zeros((h, w, A), np.float32)
    _L().ref_interpolate_forward(_p(attr), V, A, _p(idx, _u32p), idx.shape[0], _p(raster), h * w, _p(out))
    return out


def interpolate_backward(attr, idx, raster, grad):
    attr, idx, raster, grad = api._f(attr), api._u(idx), api._f(raster), api._f(grad)
    h, w = raster.shape[:2]
    V, A = attr.shape
    ga = np.zeros((V, A), np.float32)
    gr = np.zeros((h, w, 4), np.float32)
    L = _L()
    L.ref_interpolate_grad_attributes(_p(idx, _u32p), V, A, idx.shape[0], _p(raster), h * w, _p(grad), _p(ga))
    L.ref_interpolate_grad_raster(_p(attr), V, A, _p(idx, _u32p), idx.shape[0], _p(raster), h * w, _p(grad), _p(gr))
    return ga, gr


def texture_forward(tex, uv, raster, address_mode="clamp"):
    tex, uv, raster = api._f(tex), api._f(uv), api._f(raster)
    th, tw, Cc = tex.shape
    h, w = raster.shape[:2]
    out = np.zeros((h, w, Cc), np.float32)
    _L().ref_texture_forward(_p(tex), tw, th, Cc, api.ADDRESS[address_mode], _p(uv), _p(raster), h * w, _p(out))
    return out


def texture_sample_table(uv, raster, tw, th, mode):
    """src/rasterizer.cpp:187-258 build_texture_sample_adjacency: texel CSR of sample entries and
    float weights from double-precision texel positions."""
    uv, raster = api._f(uv), api._f(raster)
    h, w = raster.shape[:2]
    P = h * w
    offsets = np.zeros(tw * th + 1, np.uint32)
    weights = np.zeros(P * 4, np.float32)
    L = _L()
    n = L.ref_build_texture_sample_adjacency(_p(uv), _p(raster), w, h, tw, th, mode, _p(offsets, _u32p), None,
                                             C.c_uint64(0), _p(weights))
    if n == -1:
        raise ValueError("uv contains a non-finite value in a covered pixel")
    if n == -2:
        raise IndexError("uv is too large for portable texture addressing")
    entries = np.zeros(max(n, 1), np.uint32)
    L.ref_build_texture_sample_adjacency(_p(uv), _p(raster), w, h, tw, th, mode, _p(offsets, _u32p),
                                         _p(entries, _u32p), C.c_uint64(n), _p(weights))
    return offsets, entries[:n], weights


def texture_backward(tex, uv, raster, grad, address_mode="clamp", compute_uv_gradient=True):
    tex, uv, raster, grad = api._f(tex), api._f(uv), api._f(raster), api._f(grad)
    th, tw, Cc = tex.shape
    h, w = raster.shape[:2]
    mode = api.ADDRESS[address_mode]
    off, ent, wts = texture_sample_table(uv, raster, tw, th, mode)
    ent = ent if ent.size else np.zeros(1, np.uint32)
    gt = np.zeros(tex.shape, np.float32)
    L = _L()
    L.ref_texture_grad_texture(_p(grad), _p(off, _u32p), _p(ent, _u32p), _p(wts), tw * th, h * w, Cc, _p(gt))
    gu = None
    if compute_uv_gradient:
        gu = np.zeros((h, w, 2), np.float32)
        L.ref_texture_grad_uv(_p(tex), tw, th, Cc, mode, _p(uv), _p(raster), h * w, _p(grad), _p(gu))
    return gt, gu


def project_texture(m16, cam_weight4, vp4, dims4, depth_bias, min_cos, packed, view_index, apos, anrm, araster,
                    shadow, photo, mask, rayvis, acc_color, acc_weight, best_conf, source_view):
    a = [api._f(x) for x in (m16, cam_weight4, vp4)]
    dims = np.ascontiguousarray(dims4, dtype=np.uint32)
    _L().ref_project_texture(_p(a[0]), _p(a[1]), _p(a[2]), _p(dims, _u32p), C.c_float(depth_bias),
                             C.c_float(min_cos), C.c_uint32(packed), C.c_uint32(view_index), _p(apos), _p(anrm),
                             _p(araster), _p(shadow), _p(photo), _p(mask), _p(rayvis), _p(acc_color), _p(acc_weight),
                             _p(best_conf), _p(source_view, _u32p))


def photometric_gradient(tex3, uv, target, mask, eps, normalization, grad=None):
    tex3, uv, target, mask = api._f(tex3), api._f(uv), api._f(target), api._f(mask)
    th, tw, _ = tex3.shape
    g = np.zeros_like(tex3) if grad is None else grad
    loss = np.zeros(1, np.float32)
    P = int(np.prod(mask.shape))
    _L().ref_atlas_photometric_gradient(_p(tex3), _p(uv), _p(target), _p(mask), P, tw, th, 0, C.c_float(eps),
                                        C.c_float(normalization), _p(g), _p(loss))
    return g, float(loss[0])


def seam_gradient(tex3, pairs, eps, normalization, grad=None):
    tex3, pairs = api._f(tex3), api._f(pairs)
    th, tw, _ = tex3.shape
    g = np.zeros_like(tex3) if grad is None else grad
    loss = np.zeros(1, np.float32)
    _L().ref_atlas_seam_gradient(_p(tex3), _p(pairs), pairs.shape[0], tw, th, 0, C.c_float(eps),
                                 C.c_float(normalization), _p(g), _p(loss))
    return g, float(loss[0])


def adam_update(tex, grad, m, v, lr, b1, b2, eps, bc1, bc2, cmin, cmax):
    _L().ref_atlas_adam_update(_p(tex), _p(grad), _p(m), _p(v), tex.size, C.c_float(lr), C.c_float(b1), C.c_float(b2),
                               C.c_float(eps), C.c_float(bc1), C.c_float(bc2), C.c_float(cmin), C.c_float(cmax))


def suggest_softmax_scale(positions, camera_positions):
    pos, cams = api._f(positions), api._f(camera_positions)
    return float(_L().ref_suggest_softmax_scale(_p(pos), pos.shape[0], _p(cams), cams.shape[0]))


def pad_texture_atlas(color, valid_mask, margin=4, *, coverage_mask=None, filled_mask=None, fill_unobserved=True,
                      maximum_fill_distance=0, valid_threshold=0.5):
    """The reference's pad_texture_atlas on copies: (color, filled_mask, stats) as oracle.api."""
    col = np.array(color, dtype=np.float32, copy=True, order="C")
    h, w, ch = col.shape
    valid = api._f(valid_mask)
    cov = None if coverage_mask is None else api._f(coverage_mask)
    filled = np.zeros((h, w), np.float32) if filled_mask is None else np.array(filled_mask, np.float32, copy=True)
    stats = np.zeros(5, np.uint64)
    msg = C.create_string_buffer(256)
    rc = _L().ref_pad_texture_atlas(_p(col), ch, _p(valid), _p(cov) if cov is not None else None, _p(filled), w, h,
                                    int(margin), int(bool(fill_unobserved)), int(maximum_fill_distance),
                                    C.c_float(valid_threshold), stats.ctypes.data_as(C.c_void_p), msg, 256)
    if rc < 0:
        raise ValueError(msg.value.decode())
    return col, filled, tuple(int(s) for s in stats)


def fill_texture_on_surface(color, valid_mask, face_ids, indices, *, filled_mask=None):
    """The reference's fill_texture_on_surface on copies: (color, filled_mask, stats) as oracle.api."""
    col = np.array(color, dtype=np.float32, copy=True, order="C")
    h, w, ch = col.shape
    valid = api._f(valid_mask)
    faces = np.ascontiguousarray(face_ids, dtype=np.uint32)
    idx = api._u(indices)
    filled = np.zeros((h, w), np.float32) if filled_mask is None else np.array(filled_mask, np.float32, copy=True)
    stats = np.zeros(4, np.uint64)
    msg = C.create_string_buffer(256)
    rc = _L().ref_fill_texture_on_surface(_p(col), ch, _p(valid), _p(faces, _u32p), _p(filled), w, h, _p(idx, _u32p),
                                          idx.size // 3, stats.ctypes.data_as(C.c_void_p), msg, 256)
    if rc < 0:
        raise ValueError(msg.value.decode())
    return col, filled, tuple(int(s) for s in stats)

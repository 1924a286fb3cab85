"""NumPy wrappers over the CPU oracle (``libpdr_oracle.so``) and the reference-built checker
(``libpdr_ref.so``). TEST INFRASTRUCTURE ONLY: imported by tests, ``smoke()`` and the
CPU-baseline leg of ``bench.py``; never by the product package.

Array conventions follow the reference's Python bindings (python/bindings.cpp): clip positions
``[V, 4]`` float32, indices ``[T, 3]`` uint32, raster ``[H, W, 4]``, textures ``[H, W, C]``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_i32p = C.POINTER(C.c_int32)

ERRORS = {-1: ValueError, -2: IndexError, -3: OverflowError}

_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build_oracle())
        _declare(_lib)
    return _lib


def ref():
    """The reference's own shaders/padding built for the CPU, or None when unavailable."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None or not os.path.exists(path):
            return None
        _ref = C.CDLL(path)
    return _ref


def _declare(L):
    L.ora_bin_tiles.restype = C.c_int64
    L.ora_suggest_softmax_scale.restype = C.c_float
    L.ora_photometric_gradient.restype = C.c_float
    L.ora_seam_gradient.restype = C.c_float
    L.ora_tv_gradient.restype = C.c_double
    L.ora_photometric_gradient_f64.restype = C.c_double
    L.ora_seam_gradient_f64.restype = C.c_double
    L.ora_tv_gradient_f64.restype = C.c_double


def _p(a, t=_f32p):
    return a.ctypes.data_as(t) if a is not None else None


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _u(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _check(rc):
    if rc < 0:
        raise ERRORS.get(int(rc), RuntimeError)(f"oracle error {rc}")
    return rc


def _vp(viewport, w, h):
    if viewport is None:
        return np.array([0.0, 0.0, float(w), float(h)], dtype=np.float32)
    return np.asarray(viewport, dtype=np.float32)


# ---- raster ------------------------------------------------------------------------------

def bin_tiles(pos, idx, resolution, viewport=None):
    pos, idx = _f(pos), _u(idx)
    h, w = resolution
    vp = _vp(viewport, w, h)
    tiles = ((w + 15) // 16) * ((h + 15) // 16)
    offsets = np.zeros(tiles + 1, dtype=np.uint32)
    n = _check(lib().ora_bin_tiles(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, _p(vp),
                                   _p(offsets, _u32p), None, C.c_int64(0)))
    lst = np.zeros(max(n, 1), dtype=np.uint32)
    lib().ora_bin_tiles(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, _p(vp),
                        _p(offsets, _u32p), _p(lst, _u32p), C.c_int64(n))
    return offsets, lst[:n]


def rasterize_forward(pos, idx, resolution, cull_mode=0, output_derivatives=True, viewport=None):
    pos, idx = _f(pos), _u(idx)
    h, w = resolution
    vp = _vp(viewport, w, h)
    raster = np.zeros((h, w, 4), dtype=np.float32)
    deriv = np.zeros((h, w, 4), dtype=np.float32) if output_derivatives else None
    _check(lib().ora_rasterize_forward(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, cull_mode,
                                       int(bool(output_derivatives)), _p(vp), _p(raster), _p(deriv)))
    return raster, deriv


def rasterize_tie_counts(pos, idx, resolution, cull_mode=0, viewport=None):
    """How the reference's rasterizer decided each covered pixel: returns (raster, ties [H, W] u8, counts)
    with counts = {"covered", "depth_ties", "edge_ties"}: pixels where another covering triangle had
    the winner's depth (the lowest-id rule decided) and pixels whose winner passed an edge test only on
    the edge or inside the 1e-7 tolerance."""
    pos, idx = _f(pos), _u(idx)
    h, w = resolution
    vp = _vp(viewport, w, h)
    raster = np.zeros((h, w, 4), dtype=np.float32)
    ties = np.zeros((h, w), dtype=np.uint8)
    _check(lib().ora_rasterize_forward_ties(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, cull_mode,
                                            _p(vp), _p(raster), _p(ties, _u8p)))
    counts = {"covered": int(np.count_nonzero(raster[..., 3])), "depth_ties": int(np.count_nonzero(ties & 1)),
              "edge_ties": int(np.count_nonzero(ties & 2))}
    return raster, ties, counts


def rasterize_forward_f64(pos, idx, raster, viewport=None):
    pos, idx, raster = _f(pos), _u(idx), _f(raster)
    h, w = raster.shape[:2]
    vp = _vp(viewport, w, h)
    r64 = np.zeros((h, w, 4)), np.zeros((h, w, 4))
    lib().ora_rasterize_forward_f64(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, _p(vp),
                                    _p(raster), _p(r64[0], _f64p), _p(r64[1], _f64p))
    return r64


def rasterize_backward(pos, idx, raster, grad_raster, viewport=None, f64=False, abs_terms=False):
    pos, idx, raster, grad_raster = _f(pos), _u(idx), _f(raster), _f(grad_raster)
    h, w = raster.shape[:2]
    vp = _vp(viewport, w, h)
    if f64:
        out = np.zeros((pos.shape[0], 4), dtype=np.float64)
        fn, t = lib().ora_rasterize_backward_f64, _f64p
    else:
        out = np.zeros((pos.shape[0], 4), dtype=np.float32)
        fn, t = lib().ora_rasterize_backward, _f32p
    extra = (int(abs_terms),) if f64 else ()
    _check(fn(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], w, h, _p(vp), _p(raster), _p(grad_raster),
              _p(out, t), *extra))
    return out


# ---- interpolation -------------------------------------------------------------------------

def interpolate_forward(attr, idx, raster):
    attr, idx, raster = _f(attr), _u(idx), _f(raster)
    h, w = raster.shape[:2]
    A = attr.shape[1]
    out = np.zeros((h, w, A), dtype=np.float32)
    _check(lib().ora_interpolate_forward(_p(attr), attr.shape[0], A, _p(idx, _u32p), idx.shape[0], _p(raster),
                                         C.c_uint64(h * w), _p(out)))
    return out


def interpolate_backward(attr, idx, raster, grad, f64=False, abs_terms=False):
    attr, idx, raster, grad = _f(attr), _u(idx), _f(raster), _f(grad)
    h, w = raster.shape[:2]
    V, A = attr.shape
    dt, t = (np.float64, _f64p) if f64 else (np.float32, _f32p)
    ga = np.zeros((V, A), dtype=dt)
    gr = np.zeros((h, w, 4), dtype=dt)
    fn = lib().ora_interpolate_backward_f64 if f64 else lib().ora_interpolate_backward
    extra = (int(abs_terms),) if f64 else ()
    _check(fn(_p(attr), V, A, _p(idx, _u32p), idx.shape[0], _p(raster), C.c_uint64(h * w), _p(grad), _p(ga, t),
              _p(gr, t), *extra))
    return ga, gr


# ---- texture -------------------------------------------------------------------------------

ADDRESS = {"clamp": 0, "wrap": 1, "mirror": 2}


def texture_forward(tex, uv, raster, address_mode="clamp"):
    tex, uv, raster = _f(tex), _f(uv), _f(raster)
    th, tw, Cc = tex.shape
    h, w = raster.shape[:2]
    out = np.zeros((h, w, Cc), dtype=np.float32)
    _check(lib().ora_texture_forward(_p(tex), tw, th, Cc, ADDRESS[address_mode], _p(uv), _p(raster),
                                     C.c_uint64(h * w), _p(out)))
    return out


def texture_backward(tex, uv, raster, grad, address_mode="clamp", compute_uv_gradient=True, f64=False,
                     abs_terms=False):
    tex, uv, raster, grad = _f(tex), _f(uv), _f(raster), _f(grad)
    th, tw, Cc = tex.shape
    h, w = raster.shape[:2]
    dt, t = (np.float64, _f64p) if f64 else (np.float32, _f32p)
    gt = np.zeros(tex.shape, dtype=dt)
    gu = np.zeros((h, w, 2), dtype=dt) if compute_uv_gradient else None
    fn = lib().ora_texture_backward_f64 if f64 else lib().ora_texture_backward
    extra = (int(abs_terms),) if f64 else ()
    _check(fn(_p(tex), tw, th, Cc, ADDRESS[address_mode], _p(uv), _p(raster), C.c_uint64(h * w), _p(grad),
              _p(gt, t), _p(gu, t), *extra))
    return gt, gu


# ---- bake / refine ---------------------------------------------------------------------------

class _View(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("channel_count", C.c_uint32),
        ("image", _f32p), ("visibility_mask", _f32p),
        ("world_to_clip", C.c_float * 16), ("camera_position", C.c_float * 3),
        ("has_viewport", C.c_int), ("viewport", C.c_float * 4),
        ("weight", C.c_float), ("depth_bias", C.c_float), ("min_view_cosine", C.c_float),
    ]


class _RefineOptions(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("steps", C.c_uint32), ("batch_size", C.c_uint32),
        ("learning_rate", C.c_float), ("minimum_learning_rate", C.c_float), ("photometric_epsilon", C.c_float),
        ("adam_beta1", C.c_float), ("adam_beta2", C.c_float), ("adam_epsilon", C.c_float),
        ("clamp_min", C.c_float), ("clamp_max", C.c_float), ("seam_polish_steps", C.c_uint32),
        ("seam_learning_rate", C.c_float), ("seam_epsilon", C.c_float),
    ]


def _views(images, world_to_clip, camera_positions=None, visibility_masks=None, viewports=None, weights=None,
           depth_bias=1e-3, min_view_cosine=0.05):
    keep = []
    arr = (_View * len(images))()
    for k, img in enumerate(images):
        img = _f(img)
        keep.append(img)
        v = arr[k]
        v.height, v.width, v.channel_count = img.shape
        v.image = _p(img)
        m = None if visibility_masks is None else visibility_masks[k]
        if m is not None:
            m = _f(m)
            keep.append(m)
            v.visibility_mask = _p(m)
        v.world_to_clip[:] = [float(x) for x in np.asarray(world_to_clip[k], dtype=np.float32).reshape(16)]
        if camera_positions is not None:
            v.camera_position[:] = [float(x) for x in np.asarray(camera_positions[k], dtype=np.float32)]
        vp = None if viewports is None else viewports[k]
        v.has_viewport = int(vp is not None)
        if vp is not None:
            v.viewport[:] = [float(x) for x in vp]
        v.weight = 1.0 if weights is None else float(weights[k])
        v.depth_bias = depth_bias
        v.min_view_cosine = min_view_cosine
    return arr, keep


BLEND = {"best_view": 0, "weighted_average": 1, "softmax": 2}


def bake(positions, normals, uv, indices, images, world_to_clip, camera_positions, *, visibility_masks=None,
         viewports=None, resolution=(1024, 1024), blend_mode="weighted_average", pcf_radius=1, softmax_scale=0.0,
         mask_floor=0.0, weights=None, depth_bias=1e-3, min_view_cosine=0.05, visibility_mode=0, ray_bits=None):
    """texture_baker.cpp:156-361. With ray_bits ([texels, ceil(views / 32)] uint32 camera-visibility bits)
    visibility_mode 1 multiplies them with the shadow map and 2 uses them alone."""
    pos, nrm, uvv, idx = _f(positions), _f(normals), _f(uv), _u(indices)
    h, w = resolution
    views, keep = _views(images, world_to_clip, camera_positions, visibility_masks, viewports, weights, depth_bias,
                         min_view_cosine)
    color = np.zeros((h, w, 4), dtype=np.float32)
    conf = np.zeros((h, w), dtype=np.float32)
    src = np.zeros((h, w), dtype=np.uint32)
    valid = np.zeros((h, w), dtype=np.float32)
    cov = np.zeros((h, w), dtype=np.float32)
    faces = np.zeros((h, w), dtype=np.uint32)
    bits = None if ray_bits is None else np.ascontiguousarray(ray_bits, dtype=np.uint32)
    _check(lib().ora_bake_ex(_p(pos), _p(nrm), _p(uvv), pos.shape[0], _p(idx, _u32p), idx.shape[0], views,
                             len(images), w, h, BLEND[blend_mode], pcf_radius, C.c_float(mask_floor),
                             C.c_float(softmax_scale), int(visibility_mode) if bits is not None else 0,
                             _p(bits, _u32p), _p(color), _p(conf), _p(src, _u32p), _p(valid), _p(cov),
                             _p(faces, _u32p)))
    del keep
    return color, conf, src, valid, cov, faces


def refine_options(width, height, steps=1000, batch_size=4, learning_rate=5e-3, minimum_learning_rate=2.5e-4,
                   photometric_epsilon=1e-3, adam_beta1=0.9, adam_beta2=0.999, adam_epsilon=1e-8, clamp_min=0.0,
                   clamp_max=1.0, seam_polish_steps=30, seam_learning_rate=1e-3, seam_epsilon=1e-4):
    o = _RefineOptions()
    o.width, o.height, o.steps, o.batch_size = width, height, steps, batch_size
    o.learning_rate, o.minimum_learning_rate, o.photometric_epsilon = learning_rate, minimum_learning_rate, photometric_epsilon
    o.adam_beta1, o.adam_beta2, o.adam_epsilon = adam_beta1, adam_beta2, adam_epsilon
    o.clamp_min, o.clamp_max, o.seam_polish_steps = clamp_min, clamp_max, seam_polish_steps
    o.seam_learning_rate, o.seam_epsilon = seam_learning_rate, seam_epsilon
    return o


def refine(initial_texture, positions, uv, indices, images, world_to_clip, *, visibility_masks=None, viewports=None,
           seam_uv_pairs=None, reverse_order=False, **kw):
    """TextureRefiner::refine (texture_refiner.cpp:256-415). reverse_order visits pixels and seam pairs
    in reverse: another order the reference's atomic additions may take on a GPU."""
    init = _f(initial_texture)
    h, w, _ = init.shape
    o = refine_options(w, h, **kw)
    pos, uvv, idx = _f(positions), _f(uv), _u(indices)
    views, keep = _views(images, world_to_clip, None, visibility_masks, viewports)
    pairs = _f(seam_uv_pairs) if seam_uv_pairs is not None else np.zeros((0, 2, 2), np.float32)
    npairs = pairs.shape[0]
    out = np.zeros_like(init)
    loss = np.zeros(o.steps, dtype=np.float32)
    seam_steps = 0 if npairs == 0 else o.seam_polish_steps
    seam = np.zeros(seam_steps, dtype=np.float32)
    lib().ora_set_reverse_order(int(bool(reverse_order)))
    try:
        _check(lib().ora_refine(_p(init), _p(pos), _p(uvv), pos.shape[0], _p(idx, _u32p), idx.shape[0], views,
                                len(images), _p(pairs), npairs, C.byref(o), _p(out), _p(loss), _p(seam)))
    finally:
        lib().ora_set_reverse_order(0)
    del keep
    return out, loss, seam


def refine_view_cache(positions, uv, indices, image, world_to_clip, visibility_mask=None, viewport=None):
    pos, uvv, idx = _f(positions), _f(uv), _u(indices)
    views, keep = _views([image], [world_to_clip], None, [visibility_mask], [viewport])
    h, w = image.shape[:2]
    uv_out = np.zeros((h, w, 2), np.float32)
    tgt = np.zeros((h, w, 3), np.float32)
    msk = np.zeros((h, w), np.float32)
    vw = C.c_double(0.0)
    _check(lib().ora_refine_view_cache(_p(pos), _p(uvv), pos.shape[0], _p(idx, _u32p), idx.shape[0], views,
                                       _p(uv_out), _p(tgt), _p(msk), C.byref(vw)))
    del keep
    return uv_out, tgt, msk, vw.value


def photometric_gradient(tex3, uv, target, mask, eps, normalization, grad=None, f64=False, abs_terms=False):
    """atlas_photometric_gradient.hlsl for one view: (gradient added into `grad`, loss). With f64 the
    FP64 twin (gradient float64; abs_terms accumulates |term|)."""
    tex3, uv, target, mask = _f(tex3), _f(uv), _f(target), _f(mask)
    th, tw, _ = tex3.shape
    P = int(np.prod(mask.shape))
    if f64:
        g = np.zeros(tex3.shape, np.float64) if grad is None else grad
        loss = lib().ora_photometric_gradient_f64(_p(tex3), tw, th, _p(uv), _p(target), _p(mask), P, C.c_float(eps),
                                                  C.c_float(normalization), g.ctypes.data_as(_f64p), int(abs_terms))
        return g, loss
    g = np.zeros_like(tex3) if grad is None else grad
    loss = lib().ora_photometric_gradient(_p(tex3), tw, th, _p(uv), _p(target), _p(mask), P, C.c_float(eps),
                                          C.c_float(normalization), _p(g))
    return g, loss


def seam_gradient(tex3, pairs, eps, normalization, grad=None, f64=False, abs_terms=False):
    """atlas_seam_gradient.hlsl: (gradient added into `grad`, loss); f64 / abs_terms as above."""
    tex3, pairs = _f(tex3), _f(pairs)
    th, tw, _ = tex3.shape
    if f64:
        g = np.zeros(tex3.shape, np.float64) if grad is None else grad
        loss = lib().ora_seam_gradient_f64(_p(tex3), tw, th, _p(pairs), pairs.shape[0], C.c_float(eps),
                                           C.c_float(normalization), g.ctypes.data_as(_f64p), int(abs_terms))
        return g, loss
    g = np.zeros_like(tex3) if grad is None else grad
    loss = lib().ora_seam_gradient(_p(tex3), tw, th, _p(pairs), pairs.shape[0], C.c_float(eps),
                                   C.c_float(normalization), _p(g))
    return g, loss


def adam_update(tex, grad, m, v, lr, b1, b2, eps, bc1, bc2, cmin, cmax):
    lib().ora_adam_update(_p(tex), _p(grad), _p(m), _p(v), C.c_uint64(tex.size), C.c_float(lr), C.c_float(b1),
                          C.c_float(b2), C.c_float(eps), C.c_float(bc1), C.c_float(bc2), C.c_float(cmin),
                          C.c_float(cmax))


def tv_gradient(tex, valid=None, chart=None, eps=1e-4, weight=1.0, grad=None, f64=False, abs_terms=False):
    tex = _f(tex)
    th, tw, Cc = tex.shape
    valid = np.ones((th, tw), np.uint8) if valid is None else np.ascontiguousarray(valid, dtype=np.uint8)
    chart = None if chart is None else np.ascontiguousarray(chart, dtype=np.int32)
    if f64:
        g = np.zeros(tex.shape, np.float64) if grad is None else grad
        loss = lib().ora_tv_gradient_f64(_p(tex), tw, th, Cc, _p(valid, _u8p), _p(chart, _i32p), C.c_float(eps),
                                         C.c_float(weight), g.ctypes.data_as(_f64p), int(abs_terms))
        return g, loss
    g = np.zeros_like(tex) if grad is None else grad
    loss = lib().ora_tv_gradient(_p(tex), tw, th, Cc, _p(valid, _u8p), _p(chart, _i32p), C.c_float(eps),
                                 C.c_float(weight), _p(g))
    return g, loss


def transform_positions(pos3, m):
    pos3 = _f(pos3)
    m = _f(np.asarray(m).reshape(16))
    out = np.zeros((pos3.shape[0], 4), np.float32)
    lib().ora_transform_positions(_p(pos3), pos3.shape[0], _p(m), _p(out))
    return out


def suggest_softmax_scale(positions, camera_positions):
    pos, cams = _f(positions), _f(camera_positions)
    return float(lib().ora_suggest_softmax_scale(_p(pos), pos.shape[0], _p(cams), cams.shape[0]))


class _ProjectParams(C.Structure):
    _fields_ = [
        ("world_to_clip", C.c_float * 16), ("camera_position", C.c_float * 3), ("view_weight", C.c_float),
        ("viewport", C.c_float * 4), ("atlas_width", C.c_uint32), ("atlas_height", C.c_uint32),
        ("image_width", C.c_uint32), ("image_height", C.c_uint32), ("depth_bias", C.c_float),
        ("min_view_cosine", C.c_float), ("channel_count", C.c_uint32), ("blend_mode", C.c_uint32),
        ("pcf_radius", C.c_uint32), ("has_mask", C.c_uint32), ("visibility_mode", C.c_uint32),
        ("view_index", C.c_uint32),
    ]


def project_texture_view(m16, camera, view_weight, viewport, atlas_wh, image_wh, depth_bias, min_cos, channels,
                         blend_mode, pcf_radius, has_mask, visibility_mode, view_index, apos, anrm, araster, shadow,
                         photo, mask, rayvis, acc_color, acc_weight, best_conf, source_view):
    """One shaders/project_texture.hlsl dispatch; accumulator arrays are updated in place."""
    pp = _ProjectParams()
    pp.world_to_clip[:] = [float(x) for x in np.asarray(m16, np.float32).reshape(16)]
    pp.camera_position[:] = [float(x) for x in camera]
    pp.view_weight = view_weight
    pp.viewport[:] = [float(x) for x in viewport]
    pp.atlas_width, pp.atlas_height = atlas_wh
    pp.image_width, pp.image_height = image_wh
    pp.depth_bias, pp.min_view_cosine = depth_bias, min_cos
    pp.channel_count, pp.blend_mode, pp.pcf_radius = channels, blend_mode, pcf_radius
    pp.has_mask, pp.visibility_mode, pp.view_index = int(has_mask), visibility_mode, view_index
    lib().ora_project_texture(C.byref(pp), _p(apos), _p(anrm), _p(araster), _p(shadow), _p(photo), _p(mask),
                              _p(rayvis), _p(acc_color), _p(acc_weight), _p(best_conf), _p(source_view, _u32p))


def ray_visibility(positions, indices, atlas_positions, atlas_normals, atlas_raster, camera, bias=1e-4):
    """project_ray_visibility.hlsl for one camera with triangles tested in double: int8 per texel,
    1 visible, 0 occluded or uncovered, -1 undecided (a near miss or near hit)."""
    pos, idx = _f(positions), _u(indices)
    ap, an, ar = _f(atlas_positions), _f(atlas_normals), _f(atlas_raster)
    N = ar.size // 4
    state = np.empty(N, dtype=np.int8)
    cam = _f(camera).reshape(3)
    _check(lib().ora_ray_visibility(_p(pos), pos.shape[0], _p(idx, _u32p), idx.shape[0], _p(ap), _p(an), _p(ar),
                                    C.c_uint64(N), _p(cam), C.c_float(bias), state.ctypes.data_as(C.POINTER(C.c_int8))))
    return state


# ---- atlas padding / surface fill (src/texture_padding.cpp) -------------------------------------

PAD_REASONS = {1: "cannot pad an empty atlas", 2: "atlas dimensions exceed the supported maximum",
               4: "atlas color must have 3 or 4 channels", 6: "valid_threshold must be within (0, 1]"}
FILL_REASONS = {1: "surface fill requires mesh face IDs and a valid atlas",
                2: "surface fill requires RGB or RGBA colours", 3: "surface fill has too many faces",
                4: "atlas face ID is out of range", 5: "surface fill mesh has a degenerate edge",
                6: "surface fill requires manifold edges"}


def nearest_field(source_mask, threshold=0.5):
    """texture_padding.cpp:37-95: int16 offsets (x, y) [H, W] from each texel to its nearest source."""
    m = _f(source_mask)
    h, w = m.shape
    ox = np.empty((h, w), np.int16)
    oy = np.empty((h, w), np.int16)
    _check(lib().ora_nearest_field_offsets(_p(m), w, h, C.c_float(threshold), ox.ctypes.data_as(C.c_void_p),
                                           oy.ctypes.data_as(C.c_void_p)))
    return ox, oy


def pad_texture_atlas(color, valid_mask, margin=4, *, coverage_mask=None, filled_mask=None, fill_unobserved=True,
                      maximum_fill_distance=0, valid_threshold=0.5):
    """texture_padding.cpp:226-351 on copies: (color, filled_mask, stats) with stats = (valid, gutter,
    unobserved, remaining_unobserved, filled)."""
    col = np.array(color, dtype=np.float32, copy=True, order="C")
    h, w, ch = col.shape
    valid = _f(valid_mask)
    cov = None if coverage_mask is None else _f(coverage_mask)
    filled = np.zeros((h, w), np.float32) if filled_mask is None else np.array(filled_mask, np.float32, copy=True)
    stats = np.zeros(5, np.uint64)
    reason = C.c_int(0)
    rc = lib().ora_pad_texture_atlas(_p(col), ch, _p(valid), _p(cov) if cov is not None else None, _p(filled), w, h,
                                     int(margin), int(bool(fill_unobserved)), int(maximum_fill_distance),
                                     C.c_float(valid_threshold), stats.ctypes.data_as(C.c_void_p), C.byref(reason))
    if rc < 0:
        raise ValueError(PAD_REASONS.get(reason.value, "invalid padding input"))
    return col, filled, tuple(int(s) for s in stats)


def fill_texture_on_surface(color, valid_mask, face_ids, indices, *, filled_mask=None):
    """texture_padding.cpp:100-184 on copies: (color, filled_mask, stats) with stats = (filled,
    remaining, measured faces, propagated faces)."""
    col = np.array(color, dtype=np.float32, copy=True, order="C")
    h, w, ch = col.shape
    valid = _f(valid_mask)
    faces = np.ascontiguousarray(face_ids, dtype=np.uint32)
    idx = _u(indices)
    filled = np.zeros((h, w), np.float32) if filled_mask is None else np.array(filled_mask, np.float32, copy=True)
    stats = np.zeros(4, np.uint64)
    reason = C.c_int(0)
    rc = lib().ora_fill_texture_on_surface(_p(col), ch, _p(valid), _p(faces, _u32p), _p(filled), w, h,
                                           _p(idx, _u32p), idx.size // 3, stats.ctypes.data_as(C.c_void_p),
                                           C.byref(reason))
    if rc < 0:
        raise ValueError(FILL_REASONS.get(reason.value, "invalid surface fill input"))
    return col, filled, tuple(int(s) for s in stats)


# ---- gradient through the barycentric pixel derivatives (no reference counterpart) ----------------------

def _deriv_setup(clip, idx, raster, viewport, dtype=np.float64):
    """Per covered pixel: vertex ids and sample position (rasterize_forward.hlsl's pixel centre), in
    float64, or in float32 with the kernels' sample_ndc order of operations."""
    idx = np.asarray(idx, np.int64).reshape(-1, 3)
    h, w = raster.shape[:2]
    ids = np.rint(raster[..., 3]).astype(np.int64).reshape(-1)
    pix = np.flatnonzero((ids > 0) & (ids <= idx.shape[0]))
    tri = idx[ids[pix] - 1]
    vp = np.asarray(_vp(viewport, w, h), dtype)
    x, y = (pix % w).astype(dtype), (pix // w).astype(dtype)
    one, half, two = dtype(1.0), dtype(0.5), dtype(2.0)
    sx = ((x - vp[0] + half) * two / vp[2] - one).astype(dtype)
    sy = ((y - vp[1] + half) * two / vp[3] - one).astype(dtype)
    return np.asarray(clip, dtype), tri, pix, sx, sy, vp


def barycentric_derivatives_f64(clip, idx, raster, viewport=None):
    """The derivative output of rasterize_forward.hlsl in float64 for the triangles `raster` assigns to
    its pixels, as a function of the clip positions: [H, W, 4] (zeros where uncovered)."""
    clip, tri, pix, sx, sy, vp = _deriv_setup(clip, idx, raster, viewport)
    p0, p1, p2 = (clip[tri[:, k]] for k in range(3))
    q = [(p[:, 0] - sx * p[:, 3], p[:, 1] - sy * p[:, 3]) for p in (p0, p1, p2)]
    cr = lambda a, b: a[0] * b[1] - a[1] * b[0]  # noqa: E731
    a0, a1, a2 = cr(q[1], q[2]), cr(q[2], q[0]), cr(q[0], q[1])
    binv = 1.0 / (a0 + a1 + a2)
    b0, b1 = np.clip(a0 * binv, 0, 1), np.clip(a1 * binv, 0, 1)
    d0x, d0y = -p1[:, 3] * p2[:, 1] + p2[:, 3] * p1[:, 1], -p1[:, 0] * p2[:, 3] + p1[:, 3] * p2[:, 0]
    d1x, d1y = -p2[:, 3] * p0[:, 1] + p2[:, 1] * p0[:, 3], -p2[:, 0] * p0[:, 3] + p2[:, 3] * p0[:, 0]
    d2x, d2y = -p0[:, 3] * p1[:, 1] + p0[:, 1] * p1[:, 3], -p0[:, 0] * p1[:, 3] + p0[:, 3] * p1[:, 0]
    dAx, dAy = d0x + d1x + d2x, d0y + d1y + d2y
    kx, ky = 2.0 / vp[2], 2.0 / vp[3]
    out = np.zeros((raster.shape[0] * raster.shape[1], 4))
    out[pix] = np.stack([(d0x - b0 * dAx) * binv * kx, (d0y - b0 * dAy) * binv * ky,
                         (d1x - b1 * dAx) * binv * kx, (d1y - b1 * dAy) * binv * ky], 1)
    return out.reshape(raster.shape)


def _clamp_gates32(clip, tri, pix, w, vp):
    """Whether b0 / b1 = a_i / A lie strictly inside (0, 1) when computed in fp32 in the kernel's order
    (sample_ndc, q = p.xy - s p.w, a_i = cross(q_j, q_k), A = a0 + a1 + a2, b = a_i * (1 / A)): the clamp
    decides whether a pixel's barycentric passes a gradient, and at a triangle edge fp32 and fp64 can
    decide differently."""
    f = np.float32
    c = np.asarray(clip, np.float32)
    x, y = (pix % w).astype(np.float32), (pix // w).astype(np.float32)
    v = np.asarray(vp, np.float32)
    sx = ((x - v[0] + f(0.5)) * f(2.0) / v[2] - f(1.0)).astype(np.float32)
    sy = ((y - v[1] + f(0.5)) * f(2.0) / v[3] - f(1.0)).astype(np.float32)
    q = [(c[tri[:, k], 0] - sx * c[tri[:, k], 3], c[tri[:, k], 1] - sy * c[tri[:, k], 3]) for k in range(3)]
    cr = lambda a, b: a[0] * b[1] - a[1] * b[0]  # noqa: E731
    a0, a1, a2 = cr(q[1], q[2]), cr(q[2], q[0]), cr(q[0], q[1])
    binv = f(1.0) / (a0 + a1 + a2)
    r0, r1 = a0 * binv, a1 * binv
    return (r0 > 0) & (r0 < 1), (r1 > 0) & (r1 < 1)


def barycentric_derivatives_backward_f64(clip, idx, raster, grad, viewport=None, abs_terms=False, dtype=np.float64):
    """d(sum grad * derivatives)/d clip [V, 4] in float64 (z stays 0). With abs_terms the per-pixel
    contributions are accumulated as absolute values (a bound for summation-order error). Whether a
    clamped barycentric passes gradient is decided in fp32 as the kernel decides it. dtype=np.float32
    evaluates the per-pixel adjoint in fp32 with the kernel's operations (an estimate of fp32 error)."""
    clip, tri, pix, sx, sy, vp = _deriv_setup(clip, idx, raster, viewport, dtype)
    gate0, gate1 = _clamp_gates32(clip, tri, pix, raster.shape[1], vp)
    g = np.asarray(grad, dtype).reshape(-1, 4)[pix]
    p0, p1, p2 = (clip[tri[:, k]] for k in range(3))
    q0 = (p0[:, 0] - sx * p0[:, 3], p0[:, 1] - sy * p0[:, 3])
    q1 = (p1[:, 0] - sx * p1[:, 3], p1[:, 1] - sy * p1[:, 3])
    q2 = (p2[:, 0] - sx * p2[:, 3], p2[:, 1] - sy * p2[:, 3])
    a0 = q1[0] * q2[1] - q1[1] * q2[0]
    a1 = q2[0] * q0[1] - q2[1] * q0[0]
    a2 = q0[0] * q1[1] - q0[1] * q1[0]
    binv = dtype(1.0) / (a0 + a1 + a2)
    r0, r1 = a0 * binv, a1 * binv
    b0, b1 = np.clip(r0, 0, 1).astype(dtype), np.clip(r1, 0, 1).astype(dtype)
    d0x, d0y = -p1[:, 3] * p2[:, 1] + p2[:, 3] * p1[:, 1], -p1[:, 0] * p2[:, 3] + p1[:, 3] * p2[:, 0]
    d1x, d1y = -p2[:, 3] * p0[:, 1] + p2[:, 1] * p0[:, 3], -p2[:, 0] * p0[:, 3] + p2[:, 3] * p0[:, 0]
    d2x, d2y = -p0[:, 3] * p1[:, 1] + p0[:, 1] * p1[:, 3], -p0[:, 0] * p1[:, 3] + p0[:, 3] * p1[:, 0]
    dAx, dAy = d0x + d1x + d2x, d0y + d1y + d2y
    kx, ky = dtype(2.0) / vp[2], dtype(2.0) / vp[3]
    gx, gy, gz, gw = g[:, 0], g[:, 1], g[:, 2], g[:, 3]
    gdAx = -(gx * b0 + gz * b1) * binv * kx
    gdAy = -(gy * b0 + gw * b1) * binv * ky
    G0x, G1x, G2x = gx * binv * kx + gdAx, gz * binv * kx + gdAx, gdAx
    G0y, G1y, G2y = gy * binv * ky + gdAy, gw * binv * ky + gdAy, gdAy
    gb0 = np.where(gate0, -(gx * dAx * kx + gy * dAy * ky) * binv, dtype(0.0))
    gb1 = np.where(gate1, -(gz * dAx * kx + gw * dAy * ky) * binv, dtype(0.0))
    gbinv = (gx * (d0x - b0 * dAx) * kx + gy * (d0y - b0 * dAy) * ky + gz * (d1x - b1 * dAx) * kx +
             gw * (d1y - b1 * dAy) * ky + gb0 * a0 + gb1 * a1)
    gha = -gbinv * binv * binv
    A0, A1, A2 = gb0 * binv + gha, gb1 * binv + gha, gha
    gq = {k: np.zeros_like(sx) for k in ("0x", "0y", "1x", "1y", "2x", "2y")}
    gq["1x"] += A0 * q2[1]; gq["2y"] += A0 * q1[0]; gq["1y"] -= A0 * q2[0]; gq["2x"] -= A0 * q1[1]  # noqa: E702
    gq["2x"] += A1 * q0[1]; gq["0y"] += A1 * q2[0]; gq["2y"] -= A1 * q0[0]; gq["0x"] -= A1 * q2[1]  # noqa: E702
    gq["0x"] += A2 * q1[1]; gq["1y"] += A2 * q0[0]; gq["0y"] -= A2 * q1[0]; gq["1x"] -= A2 * q0[1]  # noqa: E702
    gp = [np.stack([gq[f"{k}x"], gq[f"{k}y"], -sx * gq[f"{k}x"] - sy * gq[f"{k}y"]], 1) for k in range(3)]
    P = (p0, p1, p2)
    # d0x = -p1.w p2.y + p2.w p1.y ; d0y = -p1.x p2.w + p1.w p2.x
    gp[1][:, 2] += -G0x * P[2][:, 1] + G0y * P[2][:, 0]; gp[2][:, 1] += -G0x * P[1][:, 3]  # noqa: E702
    gp[2][:, 2] += G0x * P[1][:, 1] - G0y * P[1][:, 0]; gp[1][:, 1] += G0x * P[2][:, 3]  # noqa: E702
    gp[1][:, 0] += -G0y * P[2][:, 3]; gp[2][:, 0] += G0y * P[1][:, 3]  # noqa: E702
    # d1x = -p2.w p0.y + p2.y p0.w ; d1y = -p2.x p0.w + p2.w p0.x
    gp[2][:, 2] += -G1x * P[0][:, 1] + G1y * P[0][:, 0]; gp[0][:, 1] += -G1x * P[2][:, 3]  # noqa: E702
    gp[2][:, 1] += G1x * P[0][:, 3]; gp[0][:, 2] += G1x * P[2][:, 1] - G1y * P[2][:, 0]  # noqa: E702
    gp[2][:, 0] += -G1y * P[0][:, 3]; gp[0][:, 0] += G1y * P[2][:, 3]  # noqa: E702
    # d2x = -p0.w p1.y + p0.y p1.w ; d2y = -p0.x p1.w + p0.w p1.x
    gp[0][:, 2] += -G2x * P[1][:, 1] + G2y * P[1][:, 0]; gp[1][:, 1] += -G2x * P[0][:, 3]  # noqa: E702
    gp[0][:, 1] += G2x * P[1][:, 3]; gp[1][:, 2] += G2x * P[0][:, 1] - G2y * P[0][:, 0]  # noqa: E702
    gp[0][:, 0] += -G2y * P[1][:, 3]; gp[1][:, 0] += G2y * P[0][:, 3]  # noqa: E702
    out = np.zeros((clip.shape[0], 4))
    for k in range(3):
        vals = np.abs(gp[k]) if abs_terms else gp[k]
        for c, col in ((0, 0), (1, 1), (2, 3)):
            np.add.at(out[:, col], tri[:, k], vals[:, c])
    return out


# ---- mipmapped texture sampling (no reference counterpart; README.md:141 lists it as planned) ---------

def _address(c, size, mode):
    """src/rasterizer.cpp:164-179 addressing of integer texel coordinates (numpy arrays)."""
    c = np.asarray(c, np.int64)
    if mode == 0:
        return np.clip(c, 0, size - 1)
    if mode == 1:
        return np.mod(c, size)
    m = np.mod(c, 2 * size)
    return np.where(m < size, m, 2 * size - 1 - m)


def mip_pyramid(texture, max_level=None):
    """Levels 0.. of the box-filtered pyramid, each level summed as ((a + b) + (c + d)) * 0.25 in fp32
    over children {2x, min(2x + 1, w - 1)} x {2y, min(2y + 1, h - 1)}."""
    levels = [np.asarray(texture, np.float32)]
    while (levels[-1].shape[0] > 1 or levels[-1].shape[1] > 1) and (max_level is None or len(levels) - 1 < max_level):
        s = levels[-1]
        h, w = s.shape[:2]
        nh, nw = max(1, h >> 1), max(1, w >> 1)
        y0, x0 = 2 * np.arange(nh), 2 * np.arange(nw)
        y1, x1 = np.minimum(y0 + 1, h - 1), np.minimum(x0 + 1, w - 1)
        a, b = s[y0][:, x0], s[y0][:, x1]
        c, d = s[y1][:, x0], s[y1][:, x1]
        levels.append((((a + b) + (c + d)) * np.float32(0.25)).astype(np.float32))
    return levels


def mip_lod32(uv_da, w0, h0, nlevels):
    """The level of detail as the kernel computes it in fp32 (0.5 log2 of the larger squared texel-space
    derivative, clamped to [0, levels - 1], NaN -> 0)."""
    da = np.asarray(uv_da, np.float32)
    ux, uy = da[..., 0] * np.float32(w0), da[..., 1] * np.float32(w0)
    vx, vy = da[..., 2] * np.float32(h0), da[..., 3] * np.float32(h0)
    m = np.maximum(ux * ux + vx * vx, uy * uy + vy * vy)
    with np.errstate(divide="ignore", invalid="ignore"):
        lod = np.float32(0.5) * np.log2(m)
    return np.where(lod > 0, np.minimum(lod, np.float32(nlevels - 1)), np.float32(0)).astype(np.float32)


def _bilinear_level(level, uv, mode):
    h, w = level.shape[:2]
    tx = uv[:, 0].astype(np.float64) * w - 0.5
    ty = uv[:, 1].astype(np.float64) * h - 0.5
    bx, by = np.floor(tx).astype(np.int64), np.floor(ty).astype(np.int64)
    fx, fy = tx - np.floor(tx), ty - np.floor(ty)
    x0, x1 = _address(bx, w, mode), _address(bx + 1, w, mode)
    y0, y1 = _address(by, h, mode), _address(by + 1, h, mode)
    return (x0, x1, y0, y1), (fx, fy)


def texture_mip_forward(texture, uv, uv_da, raster, mode=0, max_level=None):
    """Trilinear sample per pixel in float64 from the fp32 pyramid, the level chosen in fp32: [.., C]."""
    lv = mip_pyramid(texture, max_level)
    shape = np.asarray(uv).shape[:-1]
    u = np.asarray(uv, np.float32).reshape(-1, 2)
    lod = mip_lod32(uv_da, lv[0].shape[1], lv[0].shape[0], len(lv)).reshape(-1)
    cov = np.rint(np.asarray(raster)[..., 3]).reshape(-1) != 0
    C_ = lv[0].shape[2]
    out = np.zeros((u.shape[0], C_))
    l0 = np.floor(lod).astype(np.int64)
    f = (lod - np.floor(lod)).astype(np.float64)
    for k in range(len(lv)):
        for which, wgt in ((l0 == k, np.where(f > 0, 1.0 - f, 1.0)), ((np.minimum(l0 + 1, len(lv) - 1) == k) & (f > 0), f)):
            sel = np.flatnonzero(which & cov)
            if sel.size == 0:
                continue
            (x0, x1, y0, y1), (fx, fy) = _bilinear_level(lv[k], u[sel], mode)
            L = lv[k].astype(np.float64)
            s = (L[y0, x0] * ((1 - fx) * (1 - fy))[:, None] + L[y0, x1] * (fx * (1 - fy))[:, None] +
                 L[y1, x0] * ((1 - fx) * fy)[:, None] + L[y1, x1] * (fx * fy)[:, None])
            out[sel] += wgt[sel][:, None] * s
    return out.reshape(shape + (C_,)), lod.reshape(shape)


def texture_mip_backward(texture, uv, uv_da, raster, grad, mode=0, max_level=None):
    """(grad_texture [H, W, C], grad_uv [.., 2]) in float64: scatter into every sampled level, then fold
    the pyramid gradient to level 0 (coarsest first); the level of detail is a constant."""
    lv = mip_pyramid(texture, max_level)
    shape = np.asarray(uv).shape[:-1]
    u = np.asarray(uv, np.float32).reshape(-1, 2)
    g = np.asarray(grad, np.float64).reshape(u.shape[0], -1)
    lod = mip_lod32(uv_da, lv[0].shape[1], lv[0].shape[0], len(lv)).reshape(-1)
    cov = np.rint(np.asarray(raster)[..., 3]).reshape(-1) != 0
    gl = [np.zeros(x.shape, np.float64) for x in lv]
    guv = np.zeros((u.shape[0], 2))
    l0 = np.floor(lod).astype(np.int64)
    f = (lod - np.floor(lod)).astype(np.float64)
    for k in range(len(lv)):
        for which, wgt in ((l0 == k, np.where(f > 0, 1.0 - f, 1.0)), ((np.minimum(l0 + 1, len(lv) - 1) == k) & (f > 0), f)):
            sel = np.flatnonzero(which & cov)
            if sel.size == 0:
                continue
            h, w = lv[k].shape[:2]
            (x0, x1, y0, y1), (fx, fy) = _bilinear_level(lv[k], u[sel], mode)
            gc = g[sel] * wgt[sel][:, None]
            for (yy, xx), ww in (((y0, x0), (1 - fx) * (1 - fy)), ((y0, x1), fx * (1 - fy)),
                                 ((y1, x0), (1 - fx) * fy), ((y1, x1), fx * fy)):
                np.add.at(gl[k], (yy, xx), gc * ww[:, None])
            L = lv[k].astype(np.float64)
            c00, c10, c01, c11 = L[y0, x0], L[y0, x1], L[y1, x0], L[y1, x1]
            guv[sel, 0] += (gc * (((1 - fy)[:, None] * (c10 - c00) + fy[:, None] * (c11 - c01)) * w)).sum(1)
            guv[sel, 1] += (gc * (((1 - fx)[:, None] * (c01 - c00) + fx[:, None] * (c11 - c10)) * h)).sum(1)
    for k in range(len(lv) - 1, 0, -1):
        ph, pw = lv[k].shape[:2]
        ch, cw = lv[k - 1].shape[:2]
        y0, x0 = 2 * np.arange(ph), 2 * np.arange(pw)
        y1, x1 = np.minimum(y0 + 1, ch - 1), np.minimum(x0 + 1, cw - 1)
        q = gl[k] * 0.25
        for yy in (y0, y1):
            for xx in (x0, x1):
                np.add.at(gl[k - 1], (yy[:, None], xx[None, :]), q)
    return gl[0], guv.reshape(shape + (2,))


# ---- near-plane clipping (no reference counterpart; README.md:140 and docs/architecture.md:62 say the
# reference drops every triangle with a vertex at w <= 1e-8 and rasterizes the rest unclipped) ----------
#
# clip_near / rasterize_forward_near restate the GPU design in float32, operation by operation, so that the
# GPU result can be checked bit for bit; near_truth_f64 and rasterize_backward_near (float64) are the
# independent checks: what a pixel should see, decided geometrically in float64, and the adjoint.

def _near_point(ia, pa, ib, pb):
    """Intersection of edges (a, b) with z + w = 0, from the lower-indexed vertex, in float32."""
    sw = (ib < ia)[:, None]
    a, b = np.where(sw, pb, pa), np.where(sw, pa, pb)
    da, db = a[:, 2] + a[:, 3], b[:, 2] + b[:, 3]
    t = (da / (da - db))[:, None]
    return (a + t * (b - a)).astype(np.float32)


def clip_near(clip, idx):
    """One view's clipped mesh: positions [4 T, 4] (slots 4k .. 4k+3) and indices [2 T, 3] with slot
    2k = (4k, 4k+1, 4k+2), 2k+1 = (4k, 4k+2, 4k+3). A triangle entirely in front (z + w >= 0) is copied
    into slots 0-2; with one vertex in front, slots 0-2 hold it and the points on its two edges; with one
    vertex behind, the quad (edge o->a, a, b, edge b->o); unused slots are zero (w = 0: never binned)."""
    c = _f(clip).reshape(-1, 4)
    I = np.asarray(idx, np.int64).reshape(-1, 3)
    T = I.shape[0]
    k4 = 4 * np.arange(T, dtype=np.uint32)[:, None]
    cidx = np.stack([k4 + np.array([0, 1, 2], np.uint32), k4 + np.array([0, 2, 3], np.uint32)], 1).reshape(-1, 3)
    out = np.zeros((T, 4, 4), np.float32)
    P = c[I]
    with np.errstate(all="ignore"):
        inside = (P[..., 2] + P[..., 3]) >= np.float32(0.0)
        n_in = inside.sum(1)
        all_in = np.flatnonzero(n_in == 3)
        out[all_in, :3] = P[all_in]
        one = np.flatnonzero(n_in == 1)
        if one.size:
            i = np.argmax(inside[one], 1)
            j, l = (i + 1) % 3, (i + 2) % 3
            pi, pj, pl = P[one, i], P[one, j], P[one, l]
            ii, ij, il = I[one, i], I[one, j], I[one, l]
            out[one, 0] = pi
            out[one, 1] = _near_point(ii, pi, ij, pj)
            out[one, 2] = _near_point(il, pl, ii, pi)
        two = np.flatnonzero(n_in == 2)
        if two.size:
            o = np.argmin(inside[two], 1)
            a, b = (o + 1) % 3, (o + 2) % 3
            po, pa, pb = P[two, o], P[two, a], P[two, b]
            io, ia, ib = I[two, o], I[two, a], I[two, b]
            out[two, 0] = _near_point(io, po, ia, pa)
            out[two, 1] = pa
            out[two, 2] = pb
            out[two, 3] = _near_point(ib, pb, io, po)
    return out.reshape(-1, 4), cidx


def _sample32(pix, w, vp):
    f = np.float32
    x, y = (pix % w).astype(np.float32), (pix // w).astype(np.float32)
    sx = ((x - vp[0] + f(0.5)) * f(2.0) / vp[2] - f(1.0)).astype(np.float32)
    sy = ((y - vp[1] + f(0.5)) * f(2.0) / vp[3] - f(1.0)).astype(np.float32)
    return sx, sy


def rasterize_forward_near(clip, idx, resolution, cull_mode=0, viewport=None):
    """Raster and derivatives of one view with near-plane clipping: the clipped mesh through the
    reference-order rasterizer (ora_rasterize_forward), then each covered pixel remapped to the original
    triangle k = (slot id - 1) // 2 with rasterize_forward.hlsl's float32 formulas evaluated on it."""
    c = _f(clip).reshape(-1, 4)
    I = np.asarray(idx, np.int64).reshape(-1, 3)
    h, w = int(resolution[0]), int(resolution[1])
    cp, ci = clip_near(c, I)
    raster, deriv = rasterize_forward(cp, ci, (h, w), cull_mode, True, viewport)
    vp = _vp(viewport, w, h)
    f = np.float32
    r = raster.reshape(-1, 4)
    d = deriv.reshape(-1, 4)
    ids = np.rint(r[:, 3]).astype(np.int64)
    pix = np.flatnonzero((ids > 0) & (ids <= 2 * I.shape[0]))
    k = (ids[pix] - 1) // 2
    tri = I[k]
    p0, p1, p2 = (c[tri[:, m]] for m in range(3))
    sx, sy = _sample32(pix, w, vp)
    with np.errstate(all="ignore"):
        q = [(p[:, 0] - sx * p[:, 3], p[:, 1] - sy * p[:, 3]) for p in (p0, p1, p2)]
        cr = lambda u, v: u[0] * v[1] - u[1] * v[0]  # noqa: E731
        a0, a1, a2 = cr(q[1], q[2]), cr(q[2], q[0]), cr(q[0], q[1])
        ha = (a0 + a1) + a2
        binv = f(1.0) / ha
        iz = (p0[:, 2] * a0 + p1[:, 2] * a1) + p2[:, 2] * a2
        iw = (p0[:, 3] * a0 + p1[:, 3] * a1) + p2[:, 3] * a2
        clamp = lambda x, lo, hi: np.fmin(np.fmax(x, f(lo)), f(hi))  # noqa: E731
        depth = clamp(iz / iw, -1.0, 1.0)
        b0, b1 = clamp(a0 * binv, 0.0, 1.0), clamp(a1 * binv, 0.0, 1.0)
        r[pix] = np.stack([b0, b1, depth, (k + 1).astype(np.float32)], 1)
        d0x = -p1[:, 3] * p2[:, 1] + p2[:, 3] * p1[:, 1]
        d0y = -p1[:, 0] * p2[:, 3] + p1[:, 3] * p2[:, 0]
        d1x = -p2[:, 3] * p0[:, 1] + p2[:, 1] * p0[:, 3]
        d1y = -p2[:, 0] * p0[:, 3] + p2[:, 3] * p0[:, 0]
        d2x = -p0[:, 3] * p1[:, 1] + p0[:, 1] * p1[:, 3]
        d2y = -p0[:, 0] * p1[:, 3] + p0[:, 3] * p1[:, 0]
        dAx, dAy = (d0x + d1x) + d2x, (d0y + d1y) + d2y
        two = f(2.0)
        d[pix] = np.stack([(d0x - b0 * dAx) * binv * two / vp[2], (d0y - b0 * dAy) * binv * two / vp[3],
                           (d1x - b1 * dAx) * binv * two / vp[2], (d1y - b1 * dAy) * binv * two / vp[3]], 1)
    return r.reshape(h, w, 4), d.reshape(h, w, 4)


def near_truth_f64(clip, idx, resolution, cull_mode=0, viewport=None, margin=1e-4, depth_gap=1e-5):
    """What each pixel sees with near-plane clipping, decided in float64 from the geometry alone: the ray
    through the pixel centre hits triangle t at the clip-space point sum(l_i p_i) with the homogeneous
    barycentrics l_i = a_i / A (a_i the 2D homogeneous edge functions, A their sum); t covers the pixel
    when every l_i >= 0 and the hit lies in front of the near plane (z + w >= 0, w > 0); culling uses the
    sign of det[x y w] of the vertices (A = det / w_hit, so it is the winding of the part in front of the
    eye); the nearest depth z / w wins. Pixels within `margin` of
    an edge or the near plane, or with two candidates closer than `depth_gap` in depth, are undecided.
    Returns (ids [H, W] int64: 0 empty, t + 1, or -1 undecided; barycentrics [H, W, 2]; depth [H, W])."""
    c = np.asarray(clip, np.float64).reshape(-1, 4)
    I = np.asarray(idx, np.int64).reshape(-1, 3)
    h, w = int(resolution[0]), int(resolution[1])
    vp = np.asarray(_vp(viewport, w, h), np.float64)
    pix = np.arange(h * w)
    sx = ((pix % w) - vp[0] + 0.5) * 2.0 / vp[2] - 1.0
    sy = ((pix // w) - vp[1] + 0.5) * 2.0 / vp[3] - 1.0
    best = np.full(h * w, np.inf)
    second = np.full(h * w, np.inf)
    best_id = np.zeros(h * w, np.int64)
    lam = np.zeros((h * w, 2))
    marginal = np.zeros(h * w, bool)
    for t in range(I.shape[0]):
        p = c[I[t]]
        qx = p[:, 0][:, None] - sx[None] * p[:, 3][:, None]
        qy = p[:, 1][:, None] - sy[None] * p[:, 3][:, None]
        a = np.stack([qx[1] * qy[2] - qy[1] * qx[2], qx[2] * qy[0] - qy[2] * qx[0], qx[0] * qy[1] - qy[0] * qx[1]])
        A = a.sum(0)
        D = np.linalg.det(p[:, [0, 1, 3]])  # A = D / w of the hit: the winding seen in front of the eye
        if not np.any(np.abs(A) > 1e-12) or D == 0:
            continue
        if (cull_mode == 1 and D <= 0) or (cull_mode == 2 and D >= 0):
            continue
        with np.errstate(all="ignore"):
            l = a / A
            pz, pw = l.T @ p[:, 2], l.T @ p[:, 3]
            front = (pz + pw) / np.abs(pw)
            depth = pz / pw
        lmin = l.min(0)
        inside = (lmin >= 0) & (front >= 0) & (pw > 0)
        near_edge = (np.abs(lmin) < margin) | ((np.abs(front) < margin) & (lmin > -margin))
        marginal |= near_edge
        cov = np.flatnonzero(inside & ~near_edge)
        d = depth[cov]
        closer = d < best[cov]
        second[cov] = np.where(closer, best[cov], np.minimum(second[cov], d))
        upd = cov[closer]
        best[upd] = d[closer]
        best_id[upd] = t + 1
        lam[upd] = l[:2, upd].T
    ids = best_id.copy()
    with np.errstate(invalid="ignore"):
        undecided = marginal | (second - best < depth_gap)
    ids[undecided] = -1
    return ids.reshape(h, w), lam.reshape(h, w, 2), best.reshape(h, w)


def rasterize_backward_near(clip, idx, raster, grad, viewport=None, dtype=np.float64, abs_terms=False):
    """d(sum grad[..., :2] * raster[..., :2]) / d clip [V, 4] for a raster remapped to the original triangles
    (rasterize_backward.hlsl's per-pixel adjoint, with its 1e-6 area offset). A triangle whose vertices
    all have w > 1e-8 is visited on the pixels of its projected bounds, as the reference visits it; one
    with a vertex at w <= 1e-8 (which the reference never visits) on every pixel it owns. dtype float32
    evaluates the per-pixel adjoint with the kernel's float32 operations; abs_terms sums |terms|."""
    c32 = _f(clip).reshape(-1, 4)
    I = np.asarray(idx, np.int64).reshape(-1, 3)
    h, w = raster.shape[:2]
    vp32 = _vp(viewport, w, h)
    r = np.asarray(raster, np.float32).reshape(-1, 4)
    g = np.asarray(grad, np.float32).reshape(-1, 4)
    ids = np.rint(r[:, 3]).astype(np.int64)
    pix = np.flatnonzero((ids > 0) & (ids <= I.shape[0]) & ~((g[:, 0] == 0) & (g[:, 1] == 0)))
    tri = I[ids[pix] - 1]
    P32 = [c32[tri[:, m]] for m in range(3)]
    behind = (P32[0][:, 3] <= np.float32(1e-8)) | (P32[1][:, 3] <= np.float32(1e-8)) | (P32[2][:, 3] <= np.float32(1e-8))
    with np.errstate(all="ignore"):
        s = [(p[:, 0] / p[:, 3], p[:, 1] / p[:, 3]) for p in P32]
        f, half = np.float32, np.float32(0.5)
        mnx, mxx = np.fmin(np.fmin(s[0][0], s[1][0]), s[2][0]), np.fmax(np.fmax(s[0][0], s[1][0]), s[2][0])
        mny, mxy = np.fmin(np.fmin(s[0][1], s[1][1]), s[2][1]), np.fmax(np.fmax(s[0][1], s[1][1]), s[2][1])

        def bound(v, lim):
            v = np.where(np.isnan(v), 0.0, np.clip(v.astype(np.float64), -2.0 ** 31, 2.0 ** 31 - 1))
            return np.clip(v, 0, lim).astype(np.int64)

        x0 = bound(np.floor((mnx * half + half) * vp32[2] + vp32[0]), w)
        x1 = bound(np.ceil((mxx * half + half) * vp32[2] + vp32[0]), w)
        y0 = bound(np.floor((mny * half + half) * vp32[3] + vp32[1]), h)
        y1 = bound(np.ceil((mxy * half + half) * vp32[3] + vp32[1]), h)
        px, py = pix % w, pix // w
        visit = behind | ((px >= x0) & (px < x1) & (py >= y0) & (py < y1))
    pix, tri = pix[visit], tri[visit]
    if dtype == np.float32:
        sx, sy = _sample32(pix, w, vp32)
        p = [c32[tri[:, m]] for m in range(3)]
    else:
        vp = vp32.astype(np.float64)
        sx = ((pix % w) - vp[0] + 0.5) * 2.0 / vp[2] - 1.0
        sy = ((pix // w) - vp[1] + 0.5) * 2.0 / vp[3] - 1.0
        p = [c32[tri[:, m]].astype(np.float64) for m in range(3)]
    gx, gy = g[pix, 0].astype(dtype), g[pix, 1].astype(dtype)
    with np.errstate(all="ignore"):
        q = [(pp[:, 0] - sx * pp[:, 3], pp[:, 1] - sy * pp[:, 3]) for pp in p]
        cr = lambda u, v: u[0] * v[1] - u[1] * v[0]  # noqa: E731
        a0, a1 = cr(q[1], q[2]), cr(q[2], q[0])
        area = (a0 + a1) + cr(q[0], q[1])
        keep = ~(np.abs(area.astype(np.float64)) <= float(np.float32(1e-12)))
        e6 = dtype(np.float32(1e-6))  # the kernel's 1e-6f
        eps = np.where(area >= 0, e6, -e6).astype(dtype)
        inv = dtype(1.0) / (area + eps)
        b0, b1 = a0 * inv, a1 * inv
        gb0, gb1 = gx * inv, gy * inv
        gc = gb0 * b0 + gb1 * b1
        (q0x, q0y), (q1x, q1y), (q2x, q2y) = q
        gxs = [gc * (q2y - q1y) - gb1 * q2y, gc * (q0y - q2y) + gb0 * q2y, gc * (q1y - q0y) - gb0 * q1y + gb1 * q0y]
        gys = [gc * (q1x - q2x) + gb1 * q2x, gc * (q2x - q0x) - gb0 * q2x, gc * (q0x - q1x) + gb0 * q1x - gb1 * q0x]
    out = np.zeros((c32.shape[0], 4))
    for m in range(3):
        vals = [gxs[m], gys[m], -sx * gxs[m] - sy * gys[m]]
        for col, v in zip((0, 1, 3), vals):
            v = np.where(keep, v, 0).astype(np.float64)
            np.add.at(out[:, col], tri[:, m], np.abs(v) if abs_terms else v)
    return out

"""The refiner's gradients against central finite differences of its own objective, on the CPU.

The FP64 twins of the photometric (atlas_photometric_gradient.hlsl:45-108), seam
(atlas_seam_gradient.hlsl:50-100) and chart-aware total-variation (python/photara_drender/atlas.py:84-115)
gradients are checked against central differences of the FP64 losses they return, at randomly chosen
texels and channels of a small atlas. The fp32 reference-order gradients are pinned bit-exact to the
reference's shaders (tests/test_oracle_vs_reference.py); they differ from the FP64 twins by the
reference's own fp32 rounding (texel positions u*w - 0.5 rounded to fp32, cancellation in
rendered - target), which is why GPU results are compared with tests/gpu_util.grad_check. The GPU
kernels are held to the FP64 twins in tests/test_gpu_refine_parity.py, which closes the chain
GPU -> FP64 -> finite differences."""
import numpy as np
import pytest

from oracle import api
from photara_drender_gb300 import synthetic as S


def scene(seed=0, th=40, tw=48, P=6000):
    rng = np.random.default_rng(seed)
    tex = rng.uniform(0.05, 0.95, size=(th, tw, 3)).astype(np.float32)
    uv = rng.uniform(-0.05, 1.05, size=(P, 2)).astype(np.float32)
    tgt = (rng.uniform(size=(P, 3)) * 0.8 + 0.1).astype(np.float32)
    # a few targets equal to the rendered colour: Charbonnier terms at their curvature peak
    mask = ((rng.uniform(size=P) > 0.25) * rng.uniform(0.2, 1.0, size=P)).astype(np.float32)
    pos3, _, suv, idx, chart, remap = S.displaced_sphere(800, seed=seed, atlas_size=tw)
    pairs = S.seam_uv_pairs(suv, idx, remap, chart, samples_per_edge=3).astype(np.float32)
    pairs = np.concatenate([pairs, rng.uniform(size=(200, 2, 2)).astype(np.float32)])
    valid = rng.uniform(size=(th, tw)) < 0.85
    charts = ((np.arange(tw)[None, :] // 13) + 5 * (np.arange(th)[:, None] // 11)).astype(np.int32)
    return tex, uv, tgt, mask, pairs, valid, charts


def losses(kind, tex, uv, tgt, mask, pairs, valid, charts, eps):
    if kind == "photometric":
        return lambda t: api.photometric_gradient(t, uv, tgt, mask, eps, 1e-3, f64=True)
    if kind == "seam":
        return lambda t: api.seam_gradient(t, pairs, eps, 1.0 / (pairs.shape[0] * 3), f64=True)
    return lambda t: api.tv_gradient(t, valid=valid.astype(np.uint8), chart=charts, eps=eps, weight=0.5, f64=True)


@pytest.mark.parametrize("kind,eps", [("photometric", 1e-3), ("photometric", 1e-2), ("seam", 1e-4), ("seam", 1e-2),
                                      ("tv", 1e-4), ("tv", 1e-2)])
def test_fp64_gradient_matches_central_differences(kind, eps):
    tex, uv, tgt, mask, pairs, valid, charts = scene()
    f = losses(kind, tex, uv, tgt, mask, pairs, valid, charts, eps)
    g64, _ = f(tex)
    rng = np.random.default_rng(3)
    nz = np.argwhere(np.abs(g64) > 0)
    picks = nz[rng.choice(len(nz), size=60, replace=False)]
    scale = np.abs(g64).max()
    h = 2e-6
    worst = 0.0
    for y, x, c in picks:
        tp, tm = tex.copy(), tex.copy()
        tp[y, x, c] = np.float32(tex[y, x, c] + h)
        tm[y, x, c] = np.float32(tex[y, x, c] - h)
        fd = (f(tp)[1] - f(tm)[1]) / (float(tp[y, x, c]) - float(tm[y, x, c]))
        err = abs(fd - g64[y, x, c]) / max(abs(g64[y, x, c]), 1e-3 * scale)
        worst = max(worst, err)
    # central-difference truncation (h^2 / eps^2 of the Charbonnier curvature) and FP64 rounding of
    # the loss sum stay far below this
    assert worst < 1e-4, worst


def test_reverse_order_is_another_valid_sum():
    """The reversed accumulation order gives the same gradient up to fp32 summation-order noise."""
    tex, uv, tgt, mask, pairs, valid, charts = scene(2)
    a, la = api.photometric_gradient(tex, uv, tgt, mask, 1e-3, 1e-3)
    lib = api.lib()
    lib.ora_set_reverse_order(1)
    try:
        b, lb = api.photometric_gradient(tex, uv, tgt, mask, 1e-3, 1e-3)
    finally:
        lib.ora_set_reverse_order(0)
    gab, _ = api.photometric_gradient(tex, uv, tgt, mask, 1e-3, 1e-3, f64=True, abs_terms=True)
    assert not np.array_equal(a, b)
    assert np.all(np.abs(a - b) <= 2e-6 * gab + 1e-12)
    assert abs(la - lb) <= 1e-5 * abs(la)

"""Helpers shared by the GPU parity tests."""
import numpy as np


def same_bits(a, b) -> bool:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float32))
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def grad_check(gpu, ora32, ora64, abs64=None, rtol=1e-5, noise=2e-6, name=""):
    """Gradient sums: the GPU sums with atomics (a different order from the reference's fixed loops),
    so results are compared against the FP64 oracle. An element passes when
        |gpu - f64| <= rtol * max(|f64|, s) + noise * sum|terms|,   s = 1e-3 * max|f64|,
    i.e. 1e-5 relative with a magnitude floor, plus a summation-order noise floor of about 32 fp32
    ulps of the element's sum of absolute terms (abs64, from the FP64 twin's abs_terms mode) for
    elements whose terms cancel; an element whose error is within twice the reference-order fp32
    result's own error |ora32 - f64| also passes. Returns (worst error / max(|f64|, s),
    worst error / sum|terms|) for reporting."""
    gpu = np.asarray(gpu, np.float64)
    o32 = np.asarray(ora32, np.float64)
    o64 = np.asarray(ora64, np.float64)
    a64 = np.zeros_like(o64) if abs64 is None else np.asarray(abs64, np.float64)
    assert gpu.shape == o64.shape == o32.shape == a64.shape, (gpu.shape, o64.shape)
    scale = np.abs(o64).max() if o64.size else 0.0
    floor = 1e-3 * scale
    denom = np.maximum(np.abs(o64), floor)
    err = np.abs(gpu - o64)
    ok = (err <= rtol * denom + noise * a64) | (err <= 2.0 * np.abs(o32 - o64) + 1e-30)
    bad = np.flatnonzero(~ok.reshape(-1))
    assert bad.size == 0, (
        f"{name}: {bad.size} elements exceed the tolerance; worst at {bad[:5]}: gpu={gpu.reshape(-1)[bad[:5]]} "
        f"f64={o64.reshape(-1)[bad[:5]]} ref32={o32.reshape(-1)[bad[:5]]} abs={a64.reshape(-1)[bad[:5]]}")
    if not err.size:
        return 0.0, 0.0
    rel = float((err / np.where(denom > 0, denom, 1)).max())
    rel_abs = float((err / np.where(a64 > 0, a64, np.inf)).max()) if abs64 is not None else 0.0
    return rel, rel_abs


def oracle_render_chain(api, clip, idx, uva, attrs, tex, g_attr, g_samp, res, mode="clamp", viewport=None,
                        acc=None):
    """One view through the oracle in the reference's order: rasterize -> interpolate(attributes),
    interpolate(uv) -> texture, then texture_grad_texture / texture_grad_uv, both interpolate adjoints and
    rasterize_backward for the summed raster gradient, each in fp32 (reference order), FP64 and FP64 of
    |terms|. Returns the forward outputs and the per-view clip gradients; the texture, attribute and uv
    attribute gradients are added into `acc` (a dict, summed over the views passed)."""
    r, d = api.rasterize_forward(clip, idx, res, viewport=viewport)
    a = api.interpolate_forward(attrs, idx, r)
    uv = api.interpolate_forward(uva, idx, r)
    s = api.texture_forward(tex, uv, r, mode)
    gt, gu = api.texture_backward(tex, uv, r, g_samp, mode)
    gt64 = api.texture_backward(tex, uv, r, g_samp, mode, f64=True)[0]
    gtab = api.texture_backward(tex, uv, r, g_samp, mode, f64=True, abs_terms=True)[0]
    guv, gr1 = api.interpolate_backward(uva, idx, r, gu)
    ga, gr2 = api.interpolate_backward(attrs, idx, r, g_attr)
    sums = {
        "grad_tex": (gt, gt64, gtab),
        "grad_uv_attr": (guv, api.interpolate_backward(uva, idx, r, gu, f64=True)[0],
                         api.interpolate_backward(uva, idx, r, gu, f64=True, abs_terms=True)[0]),
        "grad_attr": (ga, api.interpolate_backward(attrs, idx, r, g_attr, f64=True)[0],
                      api.interpolate_backward(attrs, idx, r, g_attr, f64=True, abs_terms=True)[0]),
    }
    if acc is not None:
        for k, trio in sums.items():
            prev = acc.get(k)
            acc[k] = tuple(t.astype(np.float64) + (0.0 if prev is None else p) for t, p in
                           zip(trio, prev if prev is not None else (None,) * 3))
    grs = (gr1 + gr2).astype(np.float32)
    clip_grads = (api.rasterize_backward(clip, idx, r, grs, viewport=viewport),
                  api.rasterize_backward(clip, idx, r, grs, viewport=viewport, f64=True),
                  api.rasterize_backward(clip, idx, r, grs, viewport=viewport, f64=True, abs_terms=True))
    return {"raster": r, "deriv": d, "attr_out": a, "uv": uv, "sampled": s}, clip_grads

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

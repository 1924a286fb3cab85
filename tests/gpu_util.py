"""Helpers shared by the GPU parity tests."""
import numpy as np


def same_bits(a, b) -> bool:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float32))
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def grad_check(gpu, ora32, ora64, rtol=1e-5, name=""):
    """Gradient sums: the GPU sums with atomics (a different order from the reference's fixed loops),
    so results are compared against the FP64 oracle. An element passes when
        |gpu - f64| <= rtol * max(|f64|, s)      with s = 1e-3 * max|f64|
    (the relative-error metric with a magnitude floor), or when its error is no larger than twice the
    reference-order fp32 result's own error |ora32 - f64| (cancellation-dominated elements).
    Returns the worst relative error against FP64, for reporting."""
    gpu = np.asarray(gpu, np.float64)
    o32 = np.asarray(ora32, np.float64)
    o64 = np.asarray(ora64, np.float64)
    assert gpu.shape == o64.shape == o32.shape, (gpu.shape, o64.shape)
    scale = np.abs(o64).max() if o64.size else 0.0
    floor = 1e-3 * scale
    denom = np.maximum(np.abs(o64), floor)
    err = np.abs(gpu - o64)
    ok = (err <= rtol * denom) | (err <= 2.0 * np.abs(o32 - o64) + 1e-30)
    bad = np.flatnonzero(~ok.reshape(-1))
    assert bad.size == 0, (
        f"{name}: {bad.size} elements exceed the tolerance; worst at {bad[:5]}: gpu={gpu.reshape(-1)[bad[:5]]} "
        f"f64={o64.reshape(-1)[bad[:5]]} ref32={o32.reshape(-1)[bad[:5]]}")
    return float((err / np.where(denom > 0, denom, 1)).max()) if err.size else 0.0

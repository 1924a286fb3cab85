"""The float64 adjoint of the barycentric-derivative output (oracle/api.py) against central differences
of the float64 forward formula: the checker for the GPU's gradient through the pixel derivatives, a
capability the reference rejects (src/rasterizer.cpp:459-462)."""
import numpy as np

from oracle import api
from photara_drender_gb300 import synthetic as S


def test_adjoint_matches_finite_differences():
    rng = np.random.default_rng(0)
    pos3, idx = S.icosphere(2)
    mats, _ = S.orbit_cameras(1)
    clip = S.clip_positions(pos3, mats)[0].astype(np.float64)
    res = (40, 48)
    raster, _ = api.rasterize_forward(clip.astype(np.float32), idx, res)
    grad = rng.normal(size=res + (4,))
    g = api.barycentric_derivatives_backward_f64(clip, idx, raster, grad)
    assert np.abs(g[:, 2]).max() == 0.0 and np.abs(g).max() > 0
    loss = lambda c: float((api.barycentric_derivatives_f64(c, idx, raster) * grad).sum())  # noqa: E731
    touched = np.flatnonzero(np.abs(g).sum(1) > 0)
    for v in rng.choice(touched, 12, replace=False):
        for comp in (0, 1, 3):
            e = 1e-6 * max(1.0, abs(clip[v, comp]))
            cp, cm = clip.copy(), clip.copy()
            cp[v, comp] += e
            cm[v, comp] -= e
            fd = (loss(cp) - loss(cm)) / (2 * e)
            assert abs(fd - g[v, comp]) <= 1e-4 * max(1.0, abs(fd)), (v, comp, fd, g[v, comp])

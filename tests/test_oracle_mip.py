"""The float64 mip-sampling checker (oracle/api.py): its adjoint against finite differences of its own
forward, and at level of detail 0 its forward against the oracle's bilinear texture_forward."""
import numpy as np

from oracle import api


def case(rng, h=24, w=40, th=37, tw=50, ch=3, scale=3.0):
    tex = rng.uniform(size=(th, tw, ch)).astype(np.float32)
    uv = rng.uniform(-0.2, 1.2, size=(h, w, 2)).astype(np.float32)
    da = (rng.normal(size=(h, w, 4)) * scale / max(th, tw)).astype(np.float32)
    raster = np.zeros((h, w, 4), np.float32)
    raster[..., 3] = (rng.uniform(size=(h, w)) > 0.2).astype(np.float32)
    return tex, uv, da, raster


def test_mip_adjoint_matches_finite_differences():
    rng = np.random.default_rng(0)
    for mode in (0, 1, 2):
        tex, uv, da, raster = case(rng)
        g = rng.normal(size=uv.shape[:2] + (3,))
        gt, gu = api.texture_mip_backward(tex, uv, da, raster, g, mode)
        f = lambda t: float((api.texture_mip_forward(t, uv, da, raster, mode)[0] * g).sum())  # noqa: E731
        # linear in the texture: a random direction gives the exact directional derivative
        d = rng.normal(size=tex.shape).astype(np.float32) * np.float32(1e-2)
        assert abs(f(tex + d) - f(tex) - float((gt * d).sum())) < 1e-4 * max(1.0, abs(float((gt * d).sum())))
        # uv: central differences away from texel boundaries (piecewise bilinear)
        for _ in range(20):
            y, x = rng.integers(0, uv.shape[0]), rng.integers(0, uv.shape[1])
            if raster[y, x, 3] == 0:
                continue
            for c in range(2):
                e = 1e-4
                up, um = uv.copy(), uv.copy()
                up[y, x, c] += e
                um[y, x, c] -= e
                fd = (f_uv(tex, up, da, raster, g, mode) - f_uv(tex, um, da, raster, g, mode)) / (up[y, x, c] - um[y, x, c])
                assert abs(fd - gu[y, x, c]) <= 2e-2 * max(1.0, abs(fd)), (mode, y, x, c, fd, gu[y, x, c])


def f_uv(tex, uv, da, raster, g, mode):
    return float((api.texture_mip_forward(tex, uv, da, raster, mode)[0] * g).sum())


def test_lod_zero_is_bilinear():
    rng = np.random.default_rng(1)
    tex, uv, da, raster = case(rng, scale=0.1)
    da[...] = 0.0  # log2(0) = -inf: level 0 everywhere
    out, lod = api.texture_mip_forward(tex, uv, da, raster)
    assert not lod.any()
    ref = api.texture_forward(tex, uv, raster)
    assert np.abs(out - ref).max() < 1e-5  # the bilinear oracle forms texel positions in fp32

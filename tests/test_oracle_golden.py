"""The oracle (oracle/pdr_oracle.c) against golden fixtures produced by the reference's own
shader code (tests/golden/make_golden.py). Runs anywhere the oracle compiles."""
import os

import numpy as np
import pytest

from oracle import api

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def same_bits(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_triangle_known_case():
    g = load("triangle_32.npz")
    raster, deriv = api.rasterize_forward(g["pos"], g["idx"], (32, 32))
    assert same_bits(raster, g["raster"]) and same_bits(deriv, g["deriv"])
    vraster, vderiv = api.rasterize_forward(g["pos"], g["idx"], (32, 32), viewport=(8.0, 4.0, 16.0, 20.0))
    assert same_bits(vraster, g["vraster"]) and same_bits(vderiv, g["vderiv"])
    assert same_bits(api.rasterize_backward(g["pos"], g["idx"], raster, g["grad"]), g["gpos"])
    assert same_bits(api.rasterize_backward(g["pos"], g["idx"], vraster, g["grad"], viewport=(8.0, 4.0, 16.0, 20.0)),
                     g["vgpos"])
    assert same_bits(api.interpolate_forward(g["attrs"], g["idx"], raster), g["interp"])
    ga, gr = api.interpolate_backward(g["attrs"], g["idx"], raster, np.ones_like(g["interp"]))
    assert same_bits(ga, g["ga"]) and same_bits(gr, g["gr"])
    assert same_bits(api.interpolate_forward(g["vuv"], g["idx"], raster), g["uv"])
    assert same_bits(api.texture_forward(g["tex"], g["uv"], raster), g["sampled"])
    gt, gu = api.texture_backward(g["tex"], g["uv"], raster, g["gs"])
    assert same_bits(gt, g["gt"]) and same_bits(gu, g["gu"])


@pytest.mark.parametrize("k", [0, 1])
def test_sphere_views(k):
    g = load("sphere_small.npz")
    raster = g[f"raster{k}"]
    res = raster.shape[:2]
    vp = g[f"vp{k}"]
    r, d = api.rasterize_forward(g["clip"][k], g["idx"], res, viewport=vp, cull_mode=k)
    assert same_bits(r, raster) and same_bits(d, g[f"deriv{k}"])
    assert same_bits(api.rasterize_backward(g["clip"][k], g["idx"], raster, g[f"grad{k}"], viewport=vp), g[f"gpos{k}"])
    assert same_bits(api.interpolate_forward(g[f"attr{k}"], g["idx"], raster), g[f"interp{k}"])
    ga, gr = api.interpolate_backward(g[f"attr{k}"], g["idx"], raster, g[f"gi{k}"])
    assert same_bits(ga, g[f"ga{k}"]) and same_bits(gr, g[f"gr{k}"])
    for mode in ("clamp", "wrap", "mirror"):
        assert same_bits(api.texture_forward(g[f"tex{k}"], g[f"uv{k}"], raster, mode), g[f"s{k}_{mode}"])
        gt, gu = api.texture_backward(g[f"tex{k}"], g[f"uv{k}"], raster, g[f"gs{k}_{mode}"], mode)
        assert same_bits(gt, g[f"gt{k}_{mode}"]) and same_bits(gu, g[f"gu{k}_{mode}"])


def test_atlas_kernels():
    g = load("atlas_kernels.npz")
    grad, loss = api.photometric_gradient(g["tex"], g["uv"], g["tgt"], g["mask"], 1e-3, 0.01)
    assert same_bits(grad, g["g"]) and np.float32(loss) == g["loss"]
    sg, sloss = api.seam_gradient(g["tex"], g["pairs"], 1e-4, 1.0 / 900.0)
    assert same_bits(sg, g["sg"]) and np.float32(sloss) == g["sloss"]
    t, gg, m, v = g["tex"].copy(), g["g"].copy(), g["m_in"].copy(), g["v_in"].copy()
    api.adam_update(t, gg, m, v, 0.01, 0.9, 0.999, 1e-8, 0.1, 0.001, 0.0, 1.0)
    assert same_bits(t, g["t_out"]) and same_bits(m, g["m_out"]) and same_bits(v, g["v_out"])
    assert not gg.any()


def test_projection_modes():
    g = load("projection_small.npz")
    aw = ah = 40
    IW, IH = 28, 24
    tags = sorted({k.split("_", 1)[1] for k in g.files if k.startswith("acc_")})
    assert len(tags) == 9
    for tag in tags:
        blend, chans, vis = int(tag[1]), int(tag[3]), int(tag[5])
        acc = np.zeros(aw * ah * 3, np.float32)
        accw = np.zeros(aw * ah, np.float32)
        best = np.zeros(aw * ah, np.float32)
        src = np.full(aw * ah, 0xFFFFFFFF, np.uint32)
        for k in range(3):
            vw = 2.5 if blend == 2 else 0.7 + k * 0.2
            api.project_texture_view(g["mats"][k], g["eyes"][k], vw, [0, 0, IW, IH], (aw, ah), (IW, IH), 1e-3, 0.05,
                                     chans, blend, 1, k != 1, vis, k, g["apos"], g["anrm"], g["araster"],
                                     g["shadows"][k], g[f"photos_{tag}"][k], g[f"masks_{tag}"][k], g[f"rayvis_{tag}"],
                                     acc, accw, best, src)
        assert same_bits(acc, g[f"acc_{tag}"]), tag
        assert same_bits(accw, g[f"accw_{tag}"]), tag
        assert same_bits(best, g[f"best_{tag}"]), tag
        assert np.array_equal(src, g[f"src_{tag}"]), tag

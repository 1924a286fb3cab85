"""GPU parity of binning, rasterize, interpolate and texture (forward and backward) against the
CPU oracle, through the C ABI (photara_drender_gb300.Rasterizer -> libphotara_drender_gb300.so).

Integer outputs (tile lists, triangle ids) and every forward value are bit-exact. Gradient sums are
checked with tests/gpu_util.grad_check (1e-5 relative against FP64, floor 1e-3 of the max)."""
import os

import numpy as np
import pytest
import torch

from oracle import api
from photara_drender_gb300 import synthetic as S
from tests.gpu_util import grad_check, same_bits
from tests.raster_scenes import tie_scene

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def rast():
    from photara_drender_gb300 import Rasterizer

    return Rasterizer(0)


def sphere_scene(subdiv=3, views=3, seed=0):
    pos3, idx = S.icosphere(subdiv)
    mats, eyes = S.orbit_cameras(views)
    return pos3, idx, S.clip_positions(pos3, mats), S.spherical_uv(pos3)


def adversarial_scene():
    rng = np.random.default_rng(5)
    pos = rng.uniform(-1.5, 1.5, size=(60, 4)).astype(np.float32)
    pos[:, 3] = rng.uniform(0.2, 2.0, size=60)
    pos[3, 3] = 0.0
    pos[4, 3] = -1.0
    pos[5, 3] = 1e-9
    pos[6, :2] = (1e6, -1e6)
    pos[7, :2] = (pos[8, 0] + 1e-6, pos[8, 1])
    idx = rng.integers(0, 60, size=(300, 3)).astype(np.uint32)
    idx[:4] = [[1, 1, 2], [7, 8, 9], [6, 10, 11], [3, 12, 13]]
    quad = np.array([[-0.8, -0.8, 0.1, 1], [0.8, -0.8, 0.1, 1], [0.8, 0.8, 0.1, 1], [-0.8, 0.8, 0.1, 1],
                     [0.0, 0.0, 0.1, 1.0]], np.float32)
    qidx = np.array([[0, 1, 2], [0, 2, 3], [0, 1, 4], [1, 2, 4], [2, 3, 4], [3, 0, 4], [0, 2, 3]], np.uint32) + 60
    return np.concatenate([pos, quad]), np.concatenate([idx, qidx])


@pytest.mark.parametrize("res,vp", [((96, 80), None), ((77, 131), (5.0, -3.0, 120.0, 70.0)), ((16, 16), None)])
def test_bins_and_raster_bit_exact(rast, res, vp):
    pos3, idx, clip, _ = sphere_scene()
    offs, lst = rast.bin_tiles(clip, idx, res, viewport=[vp] * clip.shape[0] if vp else None)
    raster, deriv = rast.forward(clip, idx, res, viewport=[vp] * clip.shape[0] if vp else None)
    tiles = ((res[1] + 15) // 16) * ((res[0] + 15) // 16)
    base = 0
    for k in range(clip.shape[0]):
        o_off, o_lst = api.bin_tiles(clip[k], idx, res, vp)
        seg = offs[k * tiles:(k + 1) * tiles + 1].astype(np.int64) - base
        assert np.array_equal(seg, o_off.astype(np.int64)), f"view {k} tile offsets"
        assert np.array_equal(lst[base:base + len(o_lst)].view(np.uint32), o_lst), f"view {k} tile lists"
        base += len(o_lst)
        o_r, o_d = api.rasterize_forward(clip[k], idx, res, viewport=vp)
        assert same_bits(raster[k], o_r), f"view {k} raster"
        assert same_bits(deriv[k], o_d), f"view {k} derivatives"


@pytest.mark.parametrize("cull", ["none", "back", "front"])
def test_adversarial_raster(rast, cull):
    pos, idx = adversarial_scene()
    for res, vp in [((40, 36), None), ((33, 29), (-4.0, 3.5, 41.0, 25.0))]:
        raster, deriv = rast.forward(pos, idx, res, cull_mode=cull, viewport=vp)
        o_r, o_d = api.rasterize_forward(pos, idx, res, cull_mode={"none": 0, "back": 1, "front": 2}[cull],
                                         viewport=vp)
        assert same_bits(raster, o_r) and same_bits(deriv, o_d)
        g = np.random.default_rng(1).normal(size=o_r.shape).astype(np.float32)
        gp = rast.backward(pos, idx, o_r, g, viewport=vp)
        grad_check(gp, api.rasterize_backward(pos, idx, o_r, g, viewport=vp),
                   api.rasterize_backward(pos, idx, o_r, g, viewport=vp, f64=True),
                   api.rasterize_backward(pos, idx, o_r, g, viewport=vp, f64=True, abs_terms=True),
                   name="adversarial grad_pos")


def test_large_tiles_sorted(rast):
    # many overlapping triangles in one tile exercise the large-tile (bitmap) ordering pass
    rng = np.random.default_rng(3)
    T = 5000
    c = rng.uniform(-0.9, 0.9, size=(T, 1, 2))
    tri = c + rng.uniform(-0.02, 0.02, size=(T, 3, 2))
    pos = np.concatenate([tri.reshape(-1, 2), rng.uniform(0.1, 0.9, size=(T * 3, 1)), np.ones((T * 3, 1))], 1)
    pos = pos.astype(np.float32)
    idx = np.arange(T * 3, dtype=np.uint32).reshape(T, 3)
    for res in [(32, 32), (8, 8)]:
        offs, lst = rast.bin_tiles(pos, idx, res)
        o_off, o_lst = api.bin_tiles(pos, idx, res)
        assert np.array_equal(offs.view(np.uint32), o_off) and np.array_equal(lst.view(np.uint32), o_lst)
        raster, _ = rast.forward(pos, idx, res)
        assert same_bits(raster, api.rasterize_forward(pos, idx, res)[0])


def edge_case_triangles(seed=11):
    """Triangles that stress the forward's per-triangle candidate rectangle: microscopic ones (whose
    1e-7 edge tolerance reaches pixels beyond their bounding box), slivers, triangles with a far
    vertex, triangles with vertices on pixel centres and tile borders, and near-degenerate ones."""
    rng = np.random.default_rng(seed)
    tris = []
    for size in (1e-7, 1e-5, 1e-3, 3e-2):  # NDC
        c = rng.uniform(-0.95, 0.95, size=(150, 1, 2))
        tris.append(c + rng.normal(scale=size, size=(150, 3, 2)))
    a = rng.uniform(-0.9, 0.9, size=(150, 2))
    d = rng.normal(size=(150, 2))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    n = np.stack([-d[:, 1], d[:, 0]], 1)
    length = rng.uniform(0.05, 0.5, size=(150, 1))
    for width in (1e-6, 1e-4):  # slivers
        tris.append(np.stack([a, a + d * length, a + d * length * 0.5 + n * width], 1))
    far = rng.uniform(-0.9, 0.9, size=(150, 3, 2))
    far[:, 0] = rng.uniform(-1e3, 1e3, size=(150, 2))
    tris.append(far)
    grid = (np.arange(-8, 9) / 8.0)  # pixel centres and tile borders of a 64x64 image lie on this lattice
    tris.append(rng.choice(grid, size=(150, 3, 2)))
    xy = np.concatenate(tris).astype(np.float32)
    T = xy.shape[0]
    w = rng.uniform(0.5, 2.0, size=(T, 3, 1)).astype(np.float32)
    z = rng.uniform(-0.9, 0.9, size=(T, 3, 1)).astype(np.float32)
    pos = np.concatenate([xy * w, z * w, w], 2).reshape(-1, 4).astype(np.float32)
    return pos, np.arange(3 * T, dtype=np.uint32).reshape(T, 3)


def test_tie_rules_counted(rast):
    """Edge ties (samples on an edge, inside the 1e-7 tolerance) and depth ties (the lowest-id rule) are
    counted by the oracle and decided identically on the GPU."""
    pos, idx, res = tie_scene()
    _, _, counts = api.rasterize_tie_counts(pos, idx, res)
    assert counts["depth_ties"] > 0 and counts["edge_ties"] > 0, counts
    raster, _ = rast.forward(pos, idx, res)
    assert same_bits(raster, api.rasterize_forward(pos, idx, res)[0])
    apos, aidx = adversarial_scene()
    _, _, acounts = api.rasterize_tie_counts(apos, aidx, (40, 36))
    assert acounts["depth_ties"] > 0
    print(f"tie counts: grid {counts}, adversarial {acounts}")


@pytest.mark.parametrize("cull", ["none", "back"])
def test_candidate_rectangle_edge_cases(rast, cull):
    pos, idx = edge_case_triangles()
    for res, vp in [((64, 64), None), ((61, 70), (-3.0, 2.0, 75.0, 58.0)), ((40, 48), (1000.5, -700.25, 8192.0, 4096.0))]:
        raster, deriv = rast.forward(pos, idx, res, cull_mode=cull, viewport=vp)
        o_r, o_d = api.rasterize_forward(pos, idx, res, cull_mode={"none": 0, "back": 1}[cull], viewport=vp)
        assert same_bits(raster, o_r) and same_bits(deriv, o_d), (res, vp)


def test_backward_chain_vs_oracle(rast):
    rng = np.random.default_rng(2)
    pos3, idx, clip, uvv = sphere_scene(views=2)
    res = (120, 104)
    A = 3
    attrs = rng.uniform(size=(pos3.shape[0], A)).astype(np.float32)
    tex = rng.uniform(size=(64, 48, 4)).astype(np.float32)
    for k in range(2):
        o_r, _ = api.rasterize_forward(clip[k], idx, res)
        raster, _ = rast.forward(clip[k], idx, res)
        assert same_bits(raster, o_r)
        out = rast.interpolate_forward(attrs, idx, o_r)
        assert same_bits(out, api.interpolate_forward(attrs, idx, o_r))
        gi = rng.normal(size=out.shape).astype(np.float32)
        ga, gr = rast.interpolate_backward(attrs, idx, o_r, gi)
        o_ga, o_gr = api.interpolate_backward(attrs, idx, o_r, gi)
        o64_ga, _ = api.interpolate_backward(attrs, idx, o_r, gi, f64=True)
        abs_ga, _ = api.interpolate_backward(attrs, idx, o_r, gi, f64=True, abs_terms=True)
        assert same_bits(gr, o_gr), "interpolate grad_raster"
        grad_check(ga, o_ga, o64_ga, abs_ga, name="grad_attributes")
        uv = api.interpolate_forward(uvv, idx, o_r) * 1.3 - 0.1
        for mode in ("clamp", "wrap", "mirror"):
            s = rast.texture_forward(tex, uv, o_r, mode)
            assert same_bits(s, api.texture_forward(tex, uv, o_r, mode)), mode
            gs = rng.normal(size=s.shape).astype(np.float32)
            gt, gu = rast.texture_backward(tex, uv, o_r, gs, mode)
            o_gt, o_gu = api.texture_backward(tex, uv, o_r, gs, mode)
            o64_gt, _ = api.texture_backward(tex, uv, o_r, gs, mode, f64=True)
            abs_gt, _ = api.texture_backward(tex, uv, o_r, gs, mode, f64=True, abs_terms=True)
            assert same_bits(gu, o_gu), f"grad_uv {mode}"
            grad_check(gt, o_gt, o64_gt, abs_gt, name=f"grad_texture {mode}")
        g = rng.normal(size=o_r.shape).astype(np.float32)
        gp = rast.backward(clip[k], idx, o_r, g)
        grad_check(gp, api.rasterize_backward(clip[k], idx, o_r, g),
                   api.rasterize_backward(clip[k], idx, o_r, g, f64=True),
                   api.rasterize_backward(clip[k], idx, o_r, g, f64=True, abs_terms=True), name="grad_positions")


@pytest.mark.parametrize("tex_hw,res", [((4, 4), (96, 80)), ((2, 3), (64, 64)), ((160, 128), (40, 36))])
def test_texture_gradient_magnified_and_minified(rast, tex_hw, res):
    """grad_texture when many pixels of a warp share texels (warp-aggregated reductions) and when they
    do not (plain reductions), in every address mode, against the float64 oracle."""
    rng = np.random.default_rng(4)
    pos3, idx, clip, uvv = sphere_scene(views=1)
    o_r, _ = api.rasterize_forward(clip[0], idx, res)
    uv = api.interpolate_forward(uvv, idx, o_r) * 1.7 - 0.35
    tex = rng.uniform(size=tex_hw + (4,)).astype(np.float32)
    gs = rng.normal(size=res + (4,)).astype(np.float32)
    for mode in ("clamp", "wrap", "mirror"):
        gt, gu = rast.texture_backward(tex, uv, o_r, gs, mode)
        o_gt, o_gu = api.texture_backward(tex, uv, o_r, gs, mode)
        o64_gt, _ = api.texture_backward(tex, uv, o_r, gs, mode, f64=True)
        abs_gt, _ = api.texture_backward(tex, uv, o_r, gs, mode, f64=True, abs_terms=True)
        assert same_bits(gu, o_gu), f"grad_uv {mode}"
        grad_check(gt, o_gt, o64_gt, abs_gt, name=f"grad_texture {mode} {tex_hw}")


def test_texture_channels_not_four(rast):
    rng = np.random.default_rng(9)
    pos3, idx, clip, uvv = sphere_scene(views=1)
    o_r, _ = api.rasterize_forward(clip[0], idx, (50, 60))
    uv = api.interpolate_forward(uvv, idx, o_r)
    for C in (1, 2, 3, 5):
        tex = rng.uniform(size=(17, 23, C)).astype(np.float32)
        s = rast.texture_forward(tex, uv, o_r)
        assert same_bits(s, api.texture_forward(tex, uv, o_r))
        gs = rng.normal(size=s.shape).astype(np.float32)
        gt, gu = rast.texture_backward(tex, uv, o_r, gs)
        o_gt, o_gu = api.texture_backward(tex, uv, o_r, gs)
        assert same_bits(gu, o_gu)
        grad_check(gt, o_gt, api.texture_backward(tex, uv, o_r, gs, f64=True)[0],
                   api.texture_backward(tex, uv, o_r, gs, f64=True, abs_terms=True)[0], name=f"grad_texture C={C}")


def test_golden_fixtures_on_gpu(rast):
    g = np.load(os.path.join(GOLDEN, "triangle_32.npz"))
    raster, deriv = rast.forward(g["pos"], g["idx"], (32, 32))
    assert same_bits(raster, g["raster"]) and same_bits(deriv, g["deriv"])
    vr, vd = rast.forward(g["pos"], g["idx"], (32, 32), viewport=(8.0, 4.0, 16.0, 20.0))
    assert same_bits(vr, g["vraster"]) and same_bits(vd, g["vderiv"])
    assert same_bits(rast.interpolate_forward(g["vuv"], g["idx"], raster), g["uv"])
    assert same_bits(rast.texture_forward(g["tex"], g["uv"], raster), g["sampled"])
    s = np.load(os.path.join(GOLDEN, "sphere_small.npz"))
    for k in (0, 1):
        ref = s[f"raster{k}"]
        r, d = rast.forward(s["clip"][k], s["idx"], ref.shape[:2], cull_mode=["none", "back"][k], viewport=s[f"vp{k}"])
        assert same_bits(r, ref) and same_bits(d, s[f"deriv{k}"])
        for mode in ("clamp", "wrap", "mirror"):
            assert same_bits(rast.texture_forward(s[f"tex{k}"], s[f"uv{k}"], ref, mode), s[f"s{k}_{mode}"])
            _, gu = rast.texture_backward(s[f"tex{k}"], s[f"uv{k}"], ref, s[f"gs{k}_{mode}"], mode)
            assert same_bits(gu, s[f"gu{k}_{mode}"])


def test_torch_zero_copy_batched(rast):
    pos3, idx, clip, uvv = sphere_scene(views=4)
    dev = torch.device("cuda", 0)
    tclip = torch.tensor(clip, device=dev)
    raster, deriv = rast.forward(tclip, torch.tensor(idx.astype(np.int64), device=dev), (64, 64))
    assert raster.is_cuda and raster.shape == (4, 64, 64, 4)
    for k in range(4):
        assert same_bits(raster[k].cpu().numpy(), api.rasterize_forward(clip[k], idx, (64, 64))[0])


def test_errors_match_reference(rast):
    pos, idx = adversarial_scene()
    with pytest.raises(IndexError):
        rast.forward(pos, idx + 1000, (8, 8))
    with pytest.raises(ValueError):
        rast.forward(pos, idx, (8, 8), cull_mode="sideways")
    with pytest.raises(ValueError):
        rast.forward(pos, idx, (8, 8), viewport=(0, 0, 0, 4))
    r, _ = rast.forward(pos, idx, (16, 16))
    uv = np.zeros((16, 16, 2), np.float32)
    uv[r[..., 3] != 0] = np.nan
    if (r[..., 3] != 0).any():
        with pytest.raises(ValueError):
            rast.texture_backward(np.zeros((4, 4, 3), np.float32), uv, r, np.zeros((16, 16, 3), np.float32))
        uv[r[..., 3] != 0] = 1e12
        with pytest.raises(IndexError):
            rast.texture_backward(np.zeros((4, 4, 3), np.float32), uv, r, np.zeros((16, 16, 3), np.float32))

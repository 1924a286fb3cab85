"""Element-wise parity at the benchmark table's own configurations, through the C ABI.

* C1 exactly as stated (icosphere subdivision 4, 8 Fibonacci orbit views at 512x512, 3 attributes
  U[0,1], a 1024x1024x4 texture U[0,1], N(0,1) upstream gradients, numpy seed 0), through the fused
  pdr_render_* path and through the separate reference-shaped kernels: raster, barycentric derivatives,
  interpolated attributes, uv and texture samples bit-exact on all 8 views; texture, attribute, uv
  attribute and per-view clip gradients within tests/gpu_util.grad_check of the FP64 oracle.
* The 200k-triangle displaced sphere of the batched workload (six packed charts, 4096x4096x4 atlas) at
  1024x1024 for views 0, 31 and 63 of its 64 orbit views, each a one-view fused pass: forward bit-exact,
  gradients within grad_check.

The worst errors are printed (run with -s to see them)."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import api
from photara_drender_gb300 import synthetic as S
from tests.gpu_util import grad_check, oracle_render_chain, same_bits

pytestmark = pytest.mark.gpu

FORWARD = ("raster", "deriv", "attr_out", "uv", "sampled")
SUMMED = ("grad_tex", "grad_attr", "grad_uv_attr")


def gpu_pass(clip, idx, uva, attrs, tex, g_attr, g_samp, H, W, fused):
    from photara_drender_gb300 import Rasterizer
    from photara_drender_gb300.pipeline import RenderFwdBwd

    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)  # noqa: E731
    views, V = clip.shape[0], clip.shape[1]
    p = RenderFwdBwd(Rasterizer(0), torch.tensor(idx.astype(np.int32)), V, views, H, W, attrs.shape[1], tex.shape,
                     fused=fused)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    args = [t(clip), t(attrs), t(uva), t(tex)]
    p.forward(*args, stream)
    p.backward(*args, t(g_attr), t(g_samp), stream)
    torch.cuda.synchronize()
    p.check_capacity()
    return {k: getattr(p, k).cpu().numpy() for k in FORWARD + SUMMED + ("grad_clip",)}


@pytest.fixture(scope="module")
def c1_case():
    """The C1 inputs, generated in the order the benchmark's C1 leg generates them, and the oracle's
    results for all 8 views."""
    rng = np.random.default_rng(0)
    pos3, idx = S.icosphere(4)
    assert pos3.shape[0] == 2562 and idx.shape[0] == 5120
    mats, _ = S.orbit_cameras(8, radius=3.0, fov_y_deg=45.0, aspect=1.0)
    attrs = rng.uniform(size=(pos3.shape[0], 3)).astype(np.float32)
    tex = rng.uniform(size=(1024, 1024, 4)).astype(np.float32)
    uva = S.spherical_uv(pos3).astype(np.float32)
    clip = S.clip_positions(pos3, mats)
    H = W = 512
    g_attr = rng.standard_normal((8, H, W, 3)).astype(np.float32)
    g_samp = rng.standard_normal((8, H, W, 4)).astype(np.float32)
    acc, fwd, clip_grads = {}, [], []
    for v in range(8):
        f, cg = oracle_render_chain(api, clip[v], idx, uva, attrs, tex, g_attr[v], g_samp[v], (H, W), acc=acc)
        fwd.append(f)
        clip_grads.append(cg)
    inputs = (clip, idx, uva, attrs, tex, g_attr, g_samp, H, W)
    return inputs, fwd, clip_grads, acc


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "separate"])
def test_c1_every_view_against_oracle(c1_case, fused):
    inputs, fwd, clip_grads, acc = c1_case
    g = gpu_pass(*inputs, fused=fused)
    covered = 0
    for v in range(8):
        for k in FORWARD:
            assert same_bits(g[k][v], fwd[v][k]), (v, k)
        covered += int((fwd[v]["raster"][..., 3] != 0).sum())
    assert covered > 100_000
    worst = {}
    for v in range(8):
        worst[f"grad_clip[{v}]"] = grad_check(g["grad_clip"][v], *clip_grads[v], name=f"grad_clip view {v}")
    for k in SUMMED:
        worst[k] = grad_check(g[k], *acc[k], name=k)
    print(f"\nC1 {'fused' if fused else 'separate'}: {covered} covered pixels bit-exact; worst gradient error "
          "(vs max(|f64|, 1e-3 max|f64|), vs sum|terms|):")
    for k, (rel, rel_abs) in worst.items():
        print(f"  {k}: {rel:.3e} {rel_abs:.3e}")


@pytest.fixture(scope="module")
def c2_scene():
    pos3, _, uv, idx, _, _ = S.displaced_sphere(200_000, seed=0, atlas_size=4096)
    mats, _ = S.orbit_cameras(64, radius=3.0, fov_y_deg=45.0, aspect=1.0)
    rng = np.random.default_rng(0)
    attrs = rng.uniform(size=(pos3.shape[0], 3)).astype(np.float32)
    tex = np.random.default_rng(1).uniform(size=(4096, 4096, 4)).astype(np.float32)
    return pos3, uv, idx, mats, attrs, tex


@pytest.mark.parametrize("view", [0, 31, 63])
def test_c2_scale_view_against_oracle(c2_scene, view):
    pos3, uva, idx, mats, attrs, tex = c2_scene
    H = W = 1024
    rng = np.random.default_rng(100 + view)
    clip = S.clip_positions(pos3, mats[view:view + 1])
    g_attr = rng.standard_normal((1, H, W, 3)).astype(np.float32)
    g_samp = rng.standard_normal((1, H, W, 4)).astype(np.float32)
    g = gpu_pass(clip, idx, uva, attrs, tex, g_attr, g_samp, H, W, fused=True)
    acc = {}
    fwd, cg = oracle_render_chain(api, clip[0], idx, uva, attrs, tex, g_attr[0], g_samp[0], (H, W), acc=acc)
    for k in FORWARD:
        assert same_bits(g[k][0], fwd[k]), k
    covered = int((fwd["raster"][..., 3] != 0).sum())
    assert covered > 300_000
    worst = {"grad_clip": grad_check(g["grad_clip"][0], *cg, name="grad_clip")}
    for k in SUMMED:
        worst[k] = grad_check(g[k], *acc[k], name=k)
    print(f"\nC2 view {view}: {covered} covered pixels bit-exact; worst gradient error:")
    for k, (rel, rel_abs) in worst.items():
        print(f"  {k}: {rel:.3e} {rel_abs:.3e}")


@pytest.fixture(scope="module")
def c2_oracle_rasters(c2_scene):
    pos3, uva, idx, mats, attrs, tex = c2_scene
    clip = S.clip_positions(pos3, mats[[0, 31]])
    return clip, [api.rasterize_forward(clip[k], idx, (1024, 1024)) for k in range(2)]


@pytest.mark.parametrize("capacity_share", [None, 0.5], ids=["full-list", "cut-lists"])
@pytest.mark.parametrize("config", [(16, 16, 256), (16, 16, 128), (16, 8, 128)], ids=["16x16-256", "16x16-128", "16x8-128"])
def test_c2_scale_raster_every_tile_config(c2_scene, c2_oracle_rasters, config, capacity_share):
    """Views 0 and 31 of the C2 scene at 1024x1024 through the fused forward in every compiled tile shape:
    raster and derivatives bit-exact against the oracle. A sample can pass the edge tests inside their
    1e-7 tolerance outside the triangle's pixel box; the reference tests it when its 16x16 tile lists the
    triangle, so the binning lists a triangle in every sub-tile of those tiles (the pixels at stake here
    once differed at 16x8). With cut lists (half the entries fit) the cut tiles go through the overflow
    kernel's all-triangle pass with the same binning rule."""
    from photara_drender_gb300 import Rasterizer
    from photara_drender_gb300.pipeline import RenderFwdBwd

    pos3, uva, idx, mats, attrs, tex = c2_scene
    clip, want = c2_oracle_rasters
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)  # noqa: E731
    T, V = idx.shape[0], clip.shape[1]
    p = RenderFwdBwd(Rasterizer(0), torch.tensor(idx.astype(np.int32)), V, 2, 1024, 1024, 3, tex.shape,
                     tile_config=config)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    args = [t(clip), t(attrs), t(uva), t(tex)]
    p.forward(*args, stream)
    entries = p.check_capacity()
    if capacity_share:
        p.set_tile_config(config, int(entries * capacity_share))
        p.forward(*args, stream)
        torch.cuda.synchronize()
    raster, deriv = p.raster.cpu().numpy(), p.deriv.cpu().numpy()
    for k in range(2):
        assert same_bits(raster[k], want[k][0]), (config, k)
        assert same_bits(deriv[k], want[k][1]), (config, k)

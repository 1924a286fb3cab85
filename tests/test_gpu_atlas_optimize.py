"""optimize_texture_atlas (python/photara_drender/atlas.py:147-257) on the native refiner kernels,
against a float64 torch restatement of the reference's loop; and one Rasterizer shared by concurrent
callers (the reference serialises dispatches per context: src/context_internal.hpp:101,
docs/architecture.md:52-53)."""
import threading

import numpy as np
import pytest
import torch

import photara_drender_gb300 as pdr
from oracle import api
from photara_drender_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def scene(seed=2, views=3, res=(72, 88), atlas=64):
    rng = np.random.default_rng(seed)
    pos3, _, uv, idx, chart, remap = S.displaced_sphere(3000, seed=seed, atlas_size=atlas)
    mats, _ = S.orbit_cameras(views)
    clip = S.clip_positions(pos3, mats)
    truth = rng.uniform(0.1, 0.9, size=(atlas, atlas, 3)).astype(np.float32)
    targets, masks = [], []
    for k in range(views):
        r, _ = api.rasterize_forward(clip[k], idx, res, output_derivatives=False)
        img = api.texture_forward(truth, api.interpolate_forward(uv, idx, r), r)
        targets.append((img + rng.normal(scale=0.02, size=img.shape)).astype(np.float32))
        masks.append((rng.uniform(size=res) > 0.1).astype(np.float32) if k == 1 else None)
    pairs = S.seam_uv_pairs(uv, idx, remap, chart, samples_per_edge=2).astype(np.float32)
    valid = rng.uniform(size=(atlas, atlas)) < 0.95
    charts = ((np.arange(atlas)[None, :] // 21) + 4 * (np.arange(atlas)[:, None] // 32)).astype(np.int32)
    init = np.full((atlas, atlas, 3), 0.5, np.float32)
    return clip, idx, uv, targets, masks, pairs, valid, charts, init


def bilinear64(tex, uv):
    """Texel-centre bilinear sampling with clamp addressing in float64 (texture_forward.hlsl's formula)."""
    th, tw, _ = tex.shape
    tx, ty = uv[..., 0] * tw - 0.5, uv[..., 1] * th - 0.5
    x0f, y0f = torch.floor(tx), torch.floor(ty)
    fx, fy = (tx - x0f)[..., None], (ty - y0f)[..., None]
    x0, y0 = x0f.long(), y0f.long()
    cx = lambda x: x.clamp(0, tw - 1)  # noqa: E731
    cy = lambda y: y.clamp(0, th - 1)  # noqa: E731
    t00, t10 = tex[cy(y0), cx(x0)], tex[cy(y0), cx(x0 + 1)]
    t01, t11 = tex[cy(y0 + 1), cx(x0)], tex[cy(y0 + 1), cx(x0 + 1)]
    return t00 * (1 - fx) * (1 - fy) + t10 * fx * (1 - fy) + t01 * (1 - fx) * fy + t11 * fx * fy


def reference_loop_f64(init, uvs, rasters, targets, masks, valid, charts, pairs, o):
    """atlas.py:147-257 in float64 with the rasters and uv of the views fixed (the geometry does not
    change): masked Charbonnier of the round-robin view + TV + seam, torch.optim.Adam, clamp."""
    dev = uvs[0].device
    param = torch.nn.Parameter(torch.tensor(init, dtype=torch.float64, device=dev))
    opt = torch.optim.Adam([param], lr=o.learning_rate)
    valid_t = torch.tensor(valid, device=dev)
    chart_t = torch.tensor(charts, device=dev)
    pairs_t = torch.tensor(pairs, dtype=torch.float64, device=dev)
    history = []
    for step in range(o.steps):
        opt.zero_grad(set_to_none=True)
        k = step % len(uvs)
        covered = (rasters[k][..., 3] > 0).double()[..., None]
        image = bilinear64(param, uvs[k].double()) * covered
        mask = covered if masks[k] is None else covered * torch.tensor(masks[k], dtype=torch.float64,
                                                                        device=dev)[..., None]
        target = torch.tensor(targets[k], dtype=torch.float64, device=dev)
        robust = torch.sqrt((image - target).square() + o.photometric_epsilon ** 2)
        loss = (robust * mask).sum() / (mask.sum().clamp_min(1.0) * 3)
        loss = loss + o.total_variation_weight * pdr.atlas_total_variation(param, valid_mask=valid_t,
                                                                           chart_ids=chart_t)
        colors = bilinear64(param, pairs_t)
        loss = loss + o.seam_weight * torch.sqrt((colors[:, 0] - colors[:, 1]).square() + 1e-8).mean()
        loss.backward()
        opt.step()
        with torch.no_grad():
            param.clamp_(o.clamp_min, o.clamp_max)
        history.append(float(loss.detach()))
    return param.detach(), history


def run_optimize(o, native=True):
    from photara_drender_gb300 import atlas

    clip, idx, uv, targets, masks, pairs, valid, charts, init = scene()
    dev = torch.device("cuda", 0)
    r = pdr.Rasterizer()
    t = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    keep = atlas.USE_REFINER_KERNELS
    atlas.USE_REFINER_KERNELS = native
    try:
        return pdr.optimize_texture_atlas(
            t(init), t(clip), t(idx.astype(np.int64)), t(uv), [t(x) for x in targets], rasterizer=r,
            visibility_masks=[None if m is None else t(m) for m in masks], atlas_valid_mask=t(valid),
            chart_ids=t(charts), seam_uv_pairs=t(pairs), options=o)
    finally:
        atlas.USE_REFINER_KERNELS = keep


def test_optimize_texture_atlas_native_against_float64_reference_loop():
    """Photometric + chart-aware TV: the native run against the float64 restatement, step by step. (The
    seam term is compared against the reference's fp32 loop below: on an untouched atlas the fp32
    bilinear weights do not sum to exactly one, so the seam gradient the reference computes in fp32 is
    about 1e-9 where the exact one is 0, and Adam, whose epsilon is 1e-8, turns that into steps of up
    to a fifth of the learning rate. Float64 takes no such steps, so the trajectories part by design.)"""
    clip, idx, uv, targets, masks, pairs, valid, charts, init = scene()
    dev = torch.device("cuda", 0)
    r = pdr.Rasterizer()
    o = pdr.AtlasOptimizationOptions(steps=12, learning_rate=1e-2, total_variation_weight=1e-2, seam_weight=0.0)
    t = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    tex, hist = run_optimize(o)
    rasters, uvs = [], []
    for k in range(clip.shape[0]):
        raster, _ = r.forward(t(clip[k]), t(idx.astype(np.int32)), targets[k].shape[:2],
                              output_barycentric_derivatives=False)
        rasters.append(raster)
        uvs.append(r.interpolate_forward(t(uv), t(idx.astype(np.int32)), raster))
    ref, ref_hist = reference_loop_f64(init, uvs, rasters, targets, masks, valid, charts, pairs, o)
    rel = np.abs(np.asarray(hist) - np.asarray(ref_hist)) / np.abs(np.asarray(ref_hist))
    diff = (tex.double() - ref).abs()
    frac = float((diff > 1e-5).double().mean())
    print(f"\noptimize_texture_atlas, {o.steps} steps: loss history worst relative {rel.max():.2e}; atlas "
          f"|native - float64| max {float(diff.max()):.2e}, share above 1e-5 {frac:.2e}")
    assert rel.max() <= 1e-5, (hist, ref_hist)
    # Adam normalises each texel's step, so texels whose gradient cancels to within fp32 rounding step
    # differently from float64 in any fp32 implementation: the oracle's fp32 restatement in the
    # reference's order parts from float64 the same way (mean 3.7e-5, 6.9% of texels above 1e-5 after 12
    # steps). Per texel the GPU is held to that restatement below.
    assert float(diff.mean()) <= 1e-4 and float(diff.max()) <= 2 * o.learning_rate * o.steps
    assert hist[-1] < hist[0]
    # the same loop in fp32 in the reference's order (the oracle's restatement of the photometric and TV
    # gradients and of the Adam update). The GPU adds the photometric taps in atomic order, sums each
    # texel's four TV terms before adding them, and forms each TV term with a reciprocal square root
    # (about 2 ulp): rounding-level gradient differences that Adam turns into visible steps where a
    # gradient cancels. The yardstick is the fp32 loop's own conditioning: the oracle rerun with the TV
    # weight moved by one part in 2^23 (one ulp) parts from itself by as much (measured: max 4.2e-3,
    # mean 6.2e-6; the GPU against the oracle: max 3.2e-3, mean 3.9e-6).
    ora = oracle_loop_fp32(init, rasters, uvs, targets, masks, valid, charts, o, False)
    o_ulp = pdr.AtlasOptimizationOptions(steps=o.steps, learning_rate=o.learning_rate, seam_weight=0.0,
                                         total_variation_weight=o.total_variation_weight * (1 + 2.0 ** -23))
    d_ulp = np.abs(oracle_loop_fp32(init, rasters, uvs, targets, masks, valid, charts, o_ulp, False) - ora)
    d_gpu = np.abs(tex.cpu().numpy() - ora)
    print(f"per texel against the fp32 restatement: GPU max {d_gpu.max():.2e} mean {d_gpu.mean():.2e}, "
          f"99.9th percentile {np.quantile(d_gpu, 0.999):.2e}; the restatement against itself with a "
          f"one-ulp TV weight change: max {d_ulp.max():.2e} mean {d_ulp.mean():.2e}")
    assert d_ulp.max() > 0  # the yardstick is not degenerate
    assert d_gpu.mean() <= 2 * d_ulp.mean() and d_gpu.max() <= 2 * d_ulp.max()
    assert d_gpu.max() <= 0.5 * o.learning_rate


def oracle_loop_fp32(init, rasters, uvs, targets, masks, valid, charts, o, reverse):
    """The photometric + TV refinement loop of the reference in fp32 on the host (oracle gradients, the
    Adam shader's arithmetic), in pixel order or reversed order."""
    tex = init.copy()
    m1, m2 = np.zeros_like(tex), np.zeros_like(tex)
    lib = api.lib()
    lib.ora_set_reverse_order(int(reverse))
    try:
        for step in range(o.steps):
            k = step % len(uvs)
            r, u = rasters[k].cpu().numpy(), uvs[k].cpu().numpy()
            m = (r[..., 3] > 0).astype(np.float32) * (1.0 if masks[k] is None else masks[k])
            g = np.zeros_like(tex)
            norm = float(np.float32(1.0 / (max(float(m.sum()), 1.0) * 3)))
            api.photometric_gradient(tex, u.reshape(-1, 2), targets[k].reshape(-1, 3), m.reshape(-1),
                                     o.photometric_epsilon, norm, grad=g)
            api.tv_gradient(tex, valid=valid.astype(np.uint8), chart=charts, eps=1e-4,
                            weight=o.total_variation_weight, grad=g)
            t = step + 1
            api.adam_update(tex, g, m1, m2, o.learning_rate, 0.9, 0.999, 1e-8, 1 - 0.9 ** t, 1 - 0.999 ** t,
                            o.clamp_min, o.clamp_max)
    finally:
        lib.ora_set_reverse_order(0)
    return tex


def test_optimize_texture_atlas_native_against_reference_fp32_loop():
    """All terms (photometric, TV, seam): the native run against the reference's loop itself in fp32
    torch operations over the CUDA renderer (separate rasterize / interpolate / texture calls,
    torch.optim.Adam)."""
    o = pdr.AtlasOptimizationOptions(steps=12, learning_rate=1e-2, total_variation_weight=1e-2, seam_weight=1e-2)
    tex, hist = run_optimize(o, native=True)
    ref, ref_hist = run_optimize(o, native=False)
    rel = np.abs(np.asarray(hist) - np.asarray(ref_hist)) / np.abs(np.asarray(ref_hist))
    diff = (tex - ref).abs()
    frac = float((diff > 1e-4).float().mean())
    print(f"\noptimize_texture_atlas with seams, {o.steps} steps, native vs the reference's fp32 loop: loss "
          f"history worst relative {rel.max():.2e}; atlas max {float(diff.max()):.2e}, share above 1e-4 {frac:.2e}")
    assert rel.max() <= 1e-4, (hist, ref_hist)
    # the torch loop sums its gradients in another order and with the texture adjoint's double-precision
    # texel weights; texels whose gradient cancels to within rounding may step differently (Adam
    # normalises each step), measured 2.5% of texels above 1e-4 after 12 steps
    assert float(diff.mean()) <= 1e-4 and float(diff.max()) <= 2 * o.learning_rate * o.steps


def test_shared_rasterizer_concurrent_callers():
    """Two threads drive one Rasterizer with different views at once: every result equals the same
    call made alone (the per-context lock serialises the dispatches)."""
    pos3, idx = S.icosphere(4)
    mats, _ = S.orbit_cameras(6)
    clip = S.clip_positions(pos3, mats)
    rng = np.random.default_rng(3)
    tex = rng.uniform(size=(64, 64, 4)).astype(np.float32)
    uva = S.spherical_uv(pos3).astype(np.float32)
    r = pdr.Rasterizer()
    dev = torch.device("cuda", 0)
    t_idx = torch.tensor(idx.astype(np.int32), device=dev)
    t_tex, t_uv = torch.tensor(tex, device=dev), torch.tensor(uva, device=dev)

    def work(k):
        raster, deriv = r.forward(torch.tensor(clip[k], device=dev), t_idx, (96, 80))
        uv = r.interpolate_forward(t_uv, t_idx, raster)
        img = r.texture_forward(t_tex, uv, raster)
        gt, gu = r.texture_backward(t_tex, uv, raster, torch.ones_like(img))
        gp = r.backward(torch.tensor(clip[k], device=dev), t_idx, raster, torch.ones_like(raster))
        torch.cuda.synchronize()
        return [x.cpu().numpy() for x in (raster, deriv, uv, img, gu)], [gt.cpu().numpy(), gp.cpu().numpy()]

    alone = [work(k) for k in range(6)]
    results = [None] * 6
    errors = []

    def thread(ks):
        try:
            for _ in range(3):
                for k in ks:
                    results[k] = work(k)
        except Exception as e:  # pragma: no cover - reported below
            errors.append(e)

    th = [threading.Thread(target=thread, args=(ks,)) for ks in ((0, 2, 4), (1, 3, 5))]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errors, errors
    for k in range(6):
        exact, summed = results[k]
        for a, b in zip(exact, alone[k][0]):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        for a, b in zip(summed, alone[k][1]):  # atomic sums: equal up to their summation order
            assert np.allclose(a, b, rtol=1e-5, atol=1e-6 * max(np.abs(b).max(), 1e-30))

"""The learned preconditioner's kernels on the GPU (csrc/precond.cu through the C ABI).

The MLP runs on the tensor cores with BF16 operands and FP32 accumulation; it is checked against a
float64 NumPy restatement that applies the same BF16 roundings (inputs, weights, hidden activations,
and in training the upstream gradients fed to the tensor cores). Remaining differences come from the
accumulation order, which can flip a rounded activation by one BF16 unit, so outputs and gradients
are compared with a tolerance of 2% of the largest magnitude (a layout or descriptor error gives
errors of order 100%) and a median error below 0.1%.

A learned refinement whose MLP outputs zero everywhere scales every step by exp(0) = 1, so it must
follow the plain refiner: that pins the whole learned loop (features, MLP refresh, scaled Adam,
fallback bookkeeping) to the plain path, with and without the CUDA graph. The photometric gradient
sums with atomics in no fixed order, so two runs of the same refiner differ in the last bits, and a
texel whose gradient is a cancellation near zero can take an opposite Adam step; the comparison
therefore allows 0.1% of the values to differ by more than 1e-4 (a wrong multiplier moves nearly
every texel by about the learning rate)."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    u = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    from photara_drender_gb300.precond import OFFSETS, SHAPES

    out = {}
    for k, o in OFFSETS.items():
        n = int(np.prod(SHAPES[k]))
        out[k] = np.asarray(p[o:o + n], dtype=np.float64).reshape(SHAPES[k])
    return out


def emulate(params, x):
    """Forward of the kernel's arithmetic in float64: returns y and the intermediates."""
    w = unpack(params)
    xb = bf16(x)
    z1 = xb @ bf16(w["w1"]).T + w["b1"]
    h1 = bf16(np.maximum(z1, 0.0))
    z2 = h1 @ bf16(w["w2"]).T + w["b2"]
    h2 = bf16(np.maximum(z2, 0.0))
    y = h2 @ bf16(w["w3"]).T + w["b3"]
    return y, dict(x=xb, h1=h1, h2=h2, w=w)


def close(gpu, ref, name):
    gpu, ref = np.asarray(gpu, np.float64), np.asarray(ref, np.float64)
    scale = max(np.abs(ref).max(), 1e-6)
    err = np.abs(gpu - ref)
    assert err.max() <= 2e-2 * scale, f"{name}: max error {err.max():.3g} vs scale {scale:.3g}"
    assert np.median(err) <= 1e-3 * scale, f"{name}: median error {np.median(err):.3g} vs scale {scale:.3g}"


@pytest.fixture(scope="module")
def dev():
    return torch.device("cuda", 0)


def random_mlp(seed, dev):
    from photara_drender_gb300.precond import PrecondMLP

    mlp = PrecondMLP(0, seed=seed)
    rng = np.random.default_rng(seed)
    p = mlp.state()
    p[1024:1088] = rng.normal(scale=0.1, size=64)
    p[5184:5248] = rng.normal(scale=0.1, size=64)
    p[5248:5504] *= 10.0
    p[5504:5508] = rng.normal(scale=0.1, size=4)
    return PrecondMLP(0, params=p), p


@pytest.mark.parametrize("n", [1, 128, 1000, 70001])
def test_mlp_forward_matches_restatement(dev, n):
    mlp, p = random_mlp(1, dev)
    rng = np.random.default_rng(n)
    x = rng.normal(size=(n, 16)).astype(np.float32)
    feats = torch.tensor(x, device=dev).to(torch.bfloat16)
    y = mlp.forward(feats).cpu().numpy()
    mlp.check_status()
    ref, _ = emulate(p, feats.float().cpu().numpy())
    close(y, ref, f"forward n={n}")


def test_mlp_training_gradient_matches_restatement(dev):
    mlp, p = random_mlp(2, dev)
    rng = np.random.default_rng(3)
    n = 1000
    x = rng.normal(size=(n, 16)).astype(np.float32)
    t = rng.normal(size=(n, 4)).astype(np.float32)
    wt = (rng.uniform(size=(n, 4)) < 0.7).astype(np.float32)
    wt[:, 3] = 0.0
    feats = torch.tensor(x, device=dev).to(torch.bfloat16)
    inv = 1.0 / wt.sum()
    loss = mlp.gradient(feats, torch.tensor(t, device=dev), torch.tensor(wt, device=dev), inv).item()
    g = mlp.grads.cpu().numpy()
    mlp.check_status()
    y, c = emulate(p, feats.float().cpu().numpy())
    e = y - t
    ref_loss = float((wt * e * e).sum() * np.float32(inv))
    assert abs(loss - ref_loss) <= 1e-3 * abs(ref_loss)
    dy = 2.0 * wt * e * np.float32(inv)
    w = c["w"]
    dyp = np.zeros((n, 16))
    dyp[:, :4] = bf16(dy.astype(np.float32))
    dh2 = dyp[:, :4] @ bf16(w["w3"])
    dz2 = np.where(c["h2"] > 0, dh2, 0.0)
    dh1 = bf16(dz2.astype(np.float32)) @ bf16(w["w2"])
    dz1 = np.where(c["h1"] > 0, dh1, 0.0)
    ref = dict(w1=dz1.T @ c["x"], b1=dz1.sum(0), w2=dz2.T @ c["h1"], b2=dz2.sum(0), w3=dy.T @ c["h2"],
               b3=dy.sum(0))
    got = unpack(g)
    for k in ref:
        close(got[k], ref[k], f"grad {k}")


def test_adam_and_bf16_copy(dev):
    from photara_drender_gb300.precond import PrecondMLP

    mlp = PrecondMLP(0, seed=4)
    p0 = mlp.state().astype(np.float64)
    rng = np.random.default_rng(4)
    g = rng.normal(size=p0.size).astype(np.float32)
    mlp.grads.copy_(torch.tensor(g, device=dev))
    mlp.adam(1e-2)
    p1 = mlp.state()
    m = 0.1 * g
    v = 0.001 * g.astype(np.float64) ** 2
    ref = p0 - 1e-2 * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    assert np.allclose(p1, ref, rtol=1e-5, atol=1e-6)
    assert np.array_equal(mlp.bf16.float().cpu().numpy(), bf16(p1).astype(np.float32))


def test_fit_learns_a_smooth_map(dev):
    from photara_drender_gb300.precond import PrecondMLP

    rng = np.random.default_rng(5)
    n = 65536
    x = rng.uniform(-1, 1, size=(n, 16)).astype(np.float32)
    t = np.zeros((n, 4), np.float32)
    t[:, 0] = np.tanh(x[:, 0] + 0.5 * x[:, 1])
    t[:, 1] = x[:, 2] * x[:, 3]
    t[:, 2] = np.abs(x[:, 4])
    w = np.ones((n, 4), np.float32)
    w[:, 3] = 0.0
    mlp = PrecondMLP(0, seed=5)
    losses = mlp.fit(torch.tensor(x, device=dev).to(torch.bfloat16), torch.tensor(t, device=dev),
                     torch.tensor(w, device=dev), steps=300, batch=8192, lr=3e-3)
    assert np.isfinite(losses).all()
    assert np.mean(losses[-20:]) < 0.1 * np.mean(losses[:5])


def test_fallback_check(dev):
    from photara_drender_gb300 import _native
    from photara_drender_gb300.rasterizer import _ptr

    loss = torch.tensor([1.0, 1.0, 1.0, 1.0, 1.0, 1.01, 1.0, 1.01, 1.1, 1.2], device=dev)
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _native.call("pdr_precond_fallback_check", _ptr(loss), 0, 4, 0.02, _ptr(flag), s)
    assert int(flag.item()) == 0  # 4.02 vs 4.00: within 2%
    _native.call("pdr_precond_fallback_check", _ptr(loss), 2, 4, 0.02, _ptr(flag), s)
    assert int(flag.item()) == 1  # 4.31 vs 4.01


def small_refine_scene(dev, steps=60, tv=True):
    from photara_drender_gb300 import TextureBaker
    from photara_drender_gb300 import synthetic as S
    from photara_drender_gb300.precond import atlas_layout

    pos3, _, uv, idx, chart, remap = S.displaced_sphere(8000, seed=3, atlas_size=256)
    mats, _ = S.orbit_cameras(6)
    baker = TextureBaker(0)
    r = baker.rasterizer
    t_pos, t_uv = torch.tensor(pos3, device=dev), torch.tensor(uv, device=dev)
    t_idx = torch.tensor(idx.astype(np.int32), device=dev)
    clip = torch.tensor(S.clip_positions(pos3, mats), device=dev)
    raster, _ = r.forward(clip, t_idx, (96, 96), output_barycentric_derivatives=False)
    uvimg = r.interpolate_forward(t_uv, t_idx, raster)
    rng = np.random.default_rng(3)
    atlas = torch.tensor(rng.uniform(0.1, 0.9, size=(256, 256, 4)).astype(np.float32), device=dev)
    images = r.texture_forward(atlas, uvimg, raster)[..., :3].contiguous()
    valid, charts = atlas_layout(r, t_uv, t_idx, chart, 256, 256)
    init = torch.full((256, 256, 3), 0.5, device=dev)
    args = (init, t_pos, t_uv, t_idx, [images[k] for k in range(6)], mats, None, None,
            torch.tensor(S.seam_uv_pairs(uv, idx, remap, chart), device=dev), steps, 2, 2e-2, 1e-3, 1e-3, 5, 1e-3,
            0.9, 0.999, 1e-8, 0.0, 1.0, 1e-4, 1e-3 if tv else 0.0, valid.float(), charts, 1e-4)
    return baker, args, valid, charts


def same_run(a, b):
    d = (a[0] - b[0]).abs()
    assert float((d > 1e-4).float().mean()) <= 1e-3 and float(d.max()) <= 0.1
    la, lb = a[1].cpu().numpy(), b[1].cpu().numpy()
    assert np.allclose(la, lb, rtol=1e-3, atol=0.0)
    assert np.allclose(a[2].cpu().numpy(), b[2].cpu().numpy(), rtol=1e-3, atol=1e-7)


@pytest.mark.parametrize("use_graph", [True, False])
def test_learned_refine_with_zero_mlp_equals_plain(dev, use_graph):
    from photara_drender_gb300.precond import PrecondMLP, refine_learned, texel_stats

    baker, args, valid, charts = small_refine_scene(dev)
    st = baker._refine_prepare(*args)
    plain = baker._refine_finish(st, use_graph)
    st2 = baker._refine_prepare(*args)
    stats = texel_stats(st2, valid, charts)
    mlp = PrecondMLP(0, params=np.zeros(5508, np.float32))
    learned = refine_learned(baker, st2, mlp, stats, refresh_interval=25, fallback_tolerance=0.02,
                             use_graph=use_graph)
    same_run(plain, learned)
    assert stats.observation.sum().item() > 0 and stats.view_counts.max().item() <= 6
    assert float(stats.edge_distance.min()) == 0.0 and float(stats.edge_distance.max()) <= 64.0


def test_trajectory_samples_and_learned_run(dev):
    from photara_drender_gb300.precond import PrecondMLP, plain_trajectory_samples, refine_learned, texel_stats

    baker, args, valid, charts = small_refine_scene(dev, steps=100)
    st = baker._refine_prepare(*args)
    stats = texel_stats(st, valid, charts)
    f, t, w, final = plain_trajectory_samples(st, stats, valid, interval=25, samples=4096)
    assert f.shape == (3 * 4096, 16) and t.shape == w.shape == (3 * 4096, 4)
    assert torch.isfinite(f.float()).all() and torch.isfinite(t).all()
    assert float(t.min()) >= np.log(1 / 8) - 1e-6 and float(t.max()) <= np.log(16) + 1e-6
    assert float(w[:, 3].abs().sum()) == 0.0 and np.isfinite(final)
    # the plain path stepped by hand from Python equals the driver's plain run
    plain = baker._refine_finish(baker._refine_prepare(*args), False)
    assert abs(float(plain[1][-1]) - final) <= 1e-3 * abs(final)
    mlp = PrecondMLP(0, seed=0)
    mlp.fit(f, t, w, steps=50, batch=4096)
    out = refine_learned(baker, baker._refine_prepare(*args), mlp, stats)
    assert torch.isfinite(out[0]).all() and np.isfinite(out[1].cpu().numpy()).all()


@pytest.mark.parametrize("fallback", [0, 1])
def test_scaled_adam_matches_restatement(dev, fallback):
    """pdr_refine_adam_scaled against NumPy float32: the multiplier is exp(clamp(out, log 1/8, log 16)),
    ignored when the fallback flag is set; the update otherwise follows the plain Adam kernel."""
    from photara_drender_gb300 import _native
    from photara_drender_gb300.rasterizer import _ptr

    rng = np.random.default_rng(7 + fallback)
    N = 10007
    x, g = rng.uniform(0, 1, (N, 3)).astype(np.float32), rng.normal(0, 1e-3, (N, 3)).astype(np.float32)
    m, v = rng.normal(0, 1e-3, (N, 3)).astype(np.float32), rng.uniform(0, 1e-6, (N, 3)).astype(np.float32)
    mult = rng.uniform(-4, 4, (N, 4)).astype(np.float32)
    g4 = np.concatenate([g, np.full((N, 1), 5.0, np.float32)], 1)  # the refiner's RGB + pad gradient
    t = [torch.tensor(a, device=dev) for a in (x, g4, m, v, mult)]
    flag = torch.tensor([fallback], dtype=torch.int32, device=dev)
    lr, b1, b2, eps, bc1, bc2 = 1e-2, 0.9, 0.999, 1e-8, 0.271, 0.00299
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _native.call("pdr_refine_adam_scaled", _ptr(t[0]), _ptr(t[1]), _ptr(t[2]), _ptr(t[3]), N, _ptr(t[4]), _ptr(flag),
                 lr, b1, b2, eps, bc1, bc2, 0.0, 1.0, s)
    f32 = np.float32
    mm = f32(b1) * m + (f32(1) - f32(b1)) * g
    vv = f32(b2) * v + (f32(1) - f32(b2)) * g * g
    sc = np.ones((N, 3), np.float32) if fallback else np.exp(np.clip(mult[:, :3], f32(-2.0794415), f32(2.7725887)))
    ref = np.clip(x - f32(lr) * sc * (mm / f32(bc1)) / (np.sqrt(vv / f32(bc2)) + f32(eps)), 0.0, 1.0)
    assert np.allclose(t[0].cpu().numpy(), ref, rtol=2e-6, atol=1e-7)
    assert np.array_equal(t[2].cpu().numpy(), mm) and np.array_equal(t[3].cpu().numpy(), vv)
    assert not t[1].any()

"""GPU parity of the bake (all views in one projection launch) and the refiner (CUDA graph) against
the CPU oracle's restatement of src/texture_baker.cpp and src/texture_refiner.cpp."""
import numpy as np
import pytest

from oracle import api
from photara_drender_gb300 import synthetic as S
from tests.gpu_util import grad_check, same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def baker():
    from photara_drender_gb300.baking import TextureBaker

    return TextureBaker(0)


def bake_scene(views=4, seed=0, channels=(3, 4)):
    rng = np.random.default_rng(seed)
    pos3, idx = S.icosphere(3)
    nrm = S.vertex_normals(pos3, idx)
    uv = S.spherical_uv(pos3)
    mats, eyes = S.orbit_cameras(views)
    sizes = [(48, 64), (48, 64), (40, 40), (48, 64)][:views]
    images = [rng.uniform(size=(h, w, channels[k % len(channels)])).astype(np.float32) for k, (h, w) in enumerate(sizes)]
    masks = [rng.uniform(-0.2, 1.2, size=(h, w)).astype(np.float32) if k != 1 else None for k, (h, w) in enumerate(sizes)]
    return pos3, nrm, uv, idx, images, mats, eyes, masks


@pytest.mark.parametrize("blend", ["best_view", "weighted_average", "softmax"])
@pytest.mark.parametrize("mask_floor", [0.0, 0.25])
def test_bake_matches_oracle(baker, blend, mask_floor):
    pos3, nrm, uv, idx, images, mats, eyes, masks = bake_scene()
    viewports = [None, (2.0, -3.0, 60.0, 50.0), None, None]
    out = baker.bake_output(pos3, nrm, uv, idx, images, mats, eyes, visibility_masks=masks, viewports=viewports,
                            resolution=(64, 72), blend_mode=blend, visibility_mode="shadow_map", mask_floor=mask_floor)
    ref = api.bake(pos3, nrm, uv, idx, images, mats, eyes, visibility_masks=masks, viewports=viewports,
                   resolution=(64, 72), blend_mode=blend, mask_floor=mask_floor)
    color, conf, src, valid, cov, faces = ref
    assert np.array_equal(out.coverage_mask, cov) and np.array_equal(out.face_ids, faces)
    assert (valid > 0).sum() > 100
    if blend == "softmax":
        # exp() differs from the host libm by an ulp or two: compare with a tolerance
        assert np.array_equal(out.valid_mask, valid)
        assert np.allclose(out.color, color, rtol=1e-5, atol=1e-6)
        assert np.allclose(out.confidence, conf, rtol=1e-5, atol=1e-6)
        assert (out.source_view == src).mean() > 0.999
    else:
        assert same_bits(out.color, color) and same_bits(out.confidence, conf)
        assert np.array_equal(out.source_view, src) and same_bits(out.valid_mask, valid)


def test_bake_default_visibility_uses_ray_queries(baker):
    # the default visibility mode is ray_query (types.hpp:161); the device supports it through the BVH
    # ray caster, so no fallback happens and allow_visibility_fallback=False is accepted
    pos3, nrm, uv, idx, images, mats, eyes, masks = bake_scene(views=2)
    assert baker.device_info.supports_ray_query
    res = baker.bake(pos3, nrm, uv, idx, images, mats, eyes, resolution=(32, 32))
    assert res[5] is True
    res = baker.bake(pos3, nrm, uv, idx, images, mats, eyes, resolution=(32, 32), allow_visibility_fallback=False)
    assert res[5] is True and res[3].any()
    res = baker.bake(pos3, nrm, uv, idx, images, mats, eyes, resolution=(32, 32), visibility_mode="shadow_map")
    assert res[5] is False


def test_bake_known_answers(baker):
    # tests/native_tests.cpp:323-436 through the GPU path
    tri = np.array([[-0.75, -0.75, 0.0], [0.75, -0.75, 0.0], [0.0, 0.75, 0.0]], np.float32)
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (3, 1))
    buv = np.array([[0.125, 0.125], [0.875, 0.125], [0.5, 0.875]], np.float32)
    idx = np.array([[0, 1, 2]], np.uint32)
    img = np.zeros((16, 16, 4), np.float32)
    img[...] = (0.8, 0.2, 0.1, 1.0)
    eye = np.eye(4, dtype=np.float32)[None]
    o = baker.bake_output(tri, nrm, buv, idx, [img], eye, [[0, 0, 2]], resolution=(16, 16))
    assert np.array_equal(o.face_ids, np.where(o.coverage_mask > 0.5, 0, 0xFFFFFFFF).astype(np.uint32))
    first = np.flatnonzero(o.valid_mask.reshape(-1) > 0.5)[0]
    assert abs(o.color.reshape(-1, 4)[first, 0] - 0.8) < 1e-4
    far = img.copy()
    far[..., :3] = (0.1, 0.2, 0.8)
    two = np.concatenate([eye, eye])
    avg = baker.bake(tri, nrm, buv, idx, [img, far], two, [[0, 0, 2], [0, 0, 6]], resolution=(16, 16))
    sm = baker.bake(tri, nrm, buv, idx, [img, far], two, [[0, 0, 2], [0, 0, 6]], resolution=(16, 16),
                    blend_mode="softmax")
    i = np.flatnonzero(sm[3].reshape(-1) > 0.5)[0]
    assert sm[0].reshape(-1, 4)[i, 0] > avg[0].reshape(-1, 4)[i, 0] + 0.05
    assert abs(sm[0].reshape(-1, 4)[i, 0] - 0.8) < 0.05
    zero = np.zeros((16, 16), np.float32)
    strict = baker.bake(tri, nrm, buv, idx, [img], eye, [[0, 0, 2]], resolution=(16, 16), blend_mode="softmax",
                        visibility_masks=[zero])
    assert not (strict[3] > 0).any()
    fl = baker.bake(tri, nrm, buv, idx, [img], eye, [[0, 0, 2]], resolution=(16, 16), blend_mode="softmax",
                    visibility_masks=[zero], mask_floor=0.1)
    j = np.flatnonzero(fl[3].reshape(-1) > 0.5)[0]
    assert abs(fl[0].reshape(-1, 4)[j, 0] - 0.8) < 1e-3


def refine_scene(seed=0):
    rng = np.random.default_rng(seed)
    pos3, nrm, uv, idx, chart, remap = S.displaced_sphere(2000, seed=seed, atlas_size=64)
    mats, eyes = S.orbit_cameras(3)
    truth = rng.uniform(size=(64, 64, 3)).astype(np.float32)
    images, masks = [], []
    for k in range(3):
        from oracle import api as ora

        r, _ = ora.rasterize_forward(ora.transform_positions(pos3, mats[k]), idx, (40, 48), output_derivatives=False)
        uvk = ora.interpolate_forward(uv, idx, r)
        img = ora.texture_forward(truth, uvk, r)
        images.append(np.concatenate([img, np.ones((40, 48, 1), np.float32)], 2) if k == 0 else img)
        masks.append((rng.uniform(size=(40, 48)) > 0.2).astype(np.float32) if k == 2 else None)
    pairs = S.seam_uv_pairs(uv, idx, remap, chart, samples_per_edge=2)
    init = np.full((64, 64, 3), 0.5, np.float32)
    return init, pos3, uv, idx, images, mats, masks, pairs


def test_refine_matches_oracle(baker):
    init, pos3, uv, idx, images, mats, masks, pairs = refine_scene()
    kw = dict(steps=12, batch_size=2, learning_rate=0.05, minimum_learning_rate=0.01, seam_polish_steps=5)
    color, loss, seam, _, _ = baker.refine_texture(init, pos3, uv, idx, images, mats, visibility_masks=masks,
                                                   seam_uv_pairs=pairs, **kw)
    o_color, o_loss, o_seam = api.refine(init, pos3, uv, idx, images, mats, visibility_masks=masks,
                                         seam_uv_pairs=pairs, **kw)
    # the reference adds gradients with atomics: the oracle in reversed order is another result it may
    # give, and the GPU must stay within a small multiple of that order noise
    r_color, r_loss, r_seam = api.refine(init, pos3, uv, idx, images, mats, visibility_masks=masks,
                                         seam_uv_pairs=pairs, reverse_order=True, **kw)
    assert loss.shape == (12,) and seam.shape == (5,)
    assert np.allclose(loss, o_loss, rtol=1e-5, atol=1e-7), (loss, o_loss)
    seam_noise = np.abs(r_seam - o_seam).max()
    assert np.abs(seam - o_seam).max() <= 4.0 * seam_noise + 1e-5 * np.abs(o_seam).max(), (seam, o_seam, r_seam)
    assert np.abs(color - o_color).max() <= 4.0 * np.abs(r_color - o_color).max() + 1e-6
    assert loss[-1] < loss[0]


def test_refine_graph_equals_stream(baker):
    init, pos3, uv, idx, images, mats, masks, pairs = refine_scene(1)
    kw = dict(steps=6, batch_size=3, seam_polish_steps=2)
    a = baker.refine_texture(init, pos3, uv, idx, images, mats, seam_uv_pairs=pairs, use_graph=True, **kw)
    b = baker.refine_texture(init, pos3, uv, idx, images, mats, seam_uv_pairs=pairs, use_graph=False, **kw)
    assert np.abs(a[0] - b[0]).max() < 1e-5 and np.allclose(a[1], b[1], rtol=1e-5)


def test_refine_step_kernels(baker):
    """One photometric dispatch and one Adam update against the oracle."""
    import ctypes as C

    import torch

    from photara_drender_gb300 import _native
    from photara_drender_gb300.baking import RefineViewC
    from photara_drender_gb300.rasterizer import _ptr

    rng = np.random.default_rng(4)
    tex = rng.uniform(size=(30, 20, 3)).astype(np.float32)
    P = 4000
    uv = rng.uniform(-0.1, 1.1, size=(P, 2)).astype(np.float32)
    tgt = rng.uniform(size=(P, 3)).astype(np.float32)
    mask = ((rng.uniform(size=P) > 0.3) * rng.uniform(size=P)).astype(np.float32)
    dev = torch.device("cuda", 0)
    t_tex, t_uv, t_tgt, t_mask = (torch.tensor(x, device=dev) for x in (tex, uv, tgt, mask))
    table = (RefineViewC * 1)()
    table[0].uv, table[0].target, table[0].mask, table[0].pixel_count = (t_uv.data_ptr(), t_tgt.data_ptr(),
                                                                         t_mask.data_ptr(), P)
    t_table = torch.frombuffer(bytearray(bytes(table)), dtype=torch.uint8).to(dev)
    grad = torch.zeros((30, 20, 4), dtype=torch.float32, device=dev)  # the refiner's RGB + pad layout
    loss = torch.zeros(4, dtype=torch.float32, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _native.call("pdr_refine_photometric", _ptr(t_tex), 20, 30, _ptr(t_table), 1, P, 2, 1, 1e-3, 0.01, _ptr(grad),
                 _ptr(loss), stream)
    g32, l32 = api.photometric_gradient(tex, uv, tgt, mask, 1e-3, 0.01)
    # per-texel sums of a handful of atomically added terms: within 1e-5 of the reference-order sums
    assert not grad[..., 3].any()
    g = grad[..., :3].cpu().numpy()
    assert np.all(np.abs(g - g32) <= 1e-5 * np.maximum(np.abs(g32), 1e-3 * np.abs(g32).max()))
    assert abs(float(loss[2]) - l32) <= 1e-5 * abs(l32)
    m = (rng.normal(size=tex.shape) * 0.01).astype(np.float32)
    v = (rng.uniform(size=tex.shape) * 0.001).astype(np.float32)
    g = np.concatenate([g32, np.full(g32.shape[:2] + (1,), 7.0, np.float32)], -1)  # the pad is ignored
    tt, tg, tm, tv = (torch.tensor(x, device=dev) for x in (tex, g, m, v))
    _native.call("pdr_refine_adam", _ptr(tt), _ptr(tg), _ptr(tm), _ptr(tv), tex.size, 0.01, 0.9, 0.999, 1e-8, 0.1,
                 0.001, 0.0, 1.0, stream)
    api.adam_update(tex, g32.copy(), m, v, 0.01, 0.9, 0.999, 1e-8, 0.1, 0.001, 0.0, 1.0)
    assert same_bits(tt.cpu().numpy(), tex) and same_bits(tm.cpu().numpy(), m) and same_bits(tv.cpu().numpy(), v)
    assert not tg.any()


@pytest.mark.parametrize("masked", [False, True])
def test_total_variation_kernel(masked):
    """pdr_refine_total_variation (the chart-aware TV of atlas.py:84-115 added into the refiner's gradient)
    against the oracle's TV gradient, itself pinned to the reference's autograd
    (tests/test_atlas_losses.py), on the golden texture and a larger random atlas: within
    tests/gpu_util.grad_check of the FP64 twin (each pair term uses a reciprocal square root of about
    2 ulp; a texel sums at most four of them)."""
    import ctypes as C
    import os

    import torch

    from photara_drender_gb300 import _native
    from photara_drender_gb300.rasterizer import _ptr

    golden = np.load(os.path.join(os.path.dirname(__file__), "golden", "atlas_losses.npz"))
    rng = np.random.default_rng(6)
    cases = [(golden["tex"].astype(np.float32), golden["valid"], golden["chart"])]
    big = rng.uniform(size=(301, 517, 3)).astype(np.float32)
    cases.append((big, rng.uniform(size=big.shape[:2]) < 0.9,
                  (np.arange(517)[None, :] // 64 + 9 * (np.arange(301)[:, None] // 50)).astype(np.int32)))
    dev = torch.device("cuda", 0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for tex, valid, chart in cases:
        if not masked:
            valid, chart = np.ones(tex.shape[:2], bool), None
        H, W = tex.shape[:2]
        ok_h = valid[:, 1:] & valid[:, :-1] & (True if chart is None else chart[:, 1:] == chart[:, :-1])
        ok_v = valid[1:, :] & valid[:-1, :] & (True if chart is None else chart[1:, :] == chart[:-1, :])
        scale = np.float32(0.37 / (max(int(ok_h.sum() + ok_v.sum()), 1) * 3.0))
        want, _ = api.tv_gradient(tex, valid=valid.astype(np.uint8), chart=chart, eps=1e-4, weight=0.37)
        t_tex = torch.tensor(tex, device=dev)
        t_valid = torch.tensor(valid.astype(np.uint8), device=dev)
        t_chart = None if chart is None else torch.tensor(chart, device=dev)
        grad = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
        _native.call("pdr_refine_total_variation", _ptr(t_tex), W, H, _ptr(t_valid), _ptr(t_chart), 1e-4,
                     float(scale), _ptr(grad), stream)
        assert not grad[..., 3].any()
        got = grad[..., :3].cpu().numpy()
        kw = dict(valid=valid.astype(np.uint8), chart=chart, eps=1e-4, weight=0.37)
        w64, _ = api.tv_gradient(tex, f64=True, **kw)
        wab, _ = api.tv_gradient(tex, f64=True, abs_terms=True, **kw)
        grad_check(got, want, w64, wab, name=f"tv {H}x{W} masked={masked}")


@pytest.mark.parametrize("steps", [7, 8])
def test_refine_tv_fused_pass_is_bit_identical(baker, steps):
    """With the chart-aware total variation on, pdr_refine_run given a second atlas buffer
    (texture_scratch) runs each step's TV gradient and Adam update as one pass, alternating the texture
    between the two buffers, for an odd and an even step count (the result ends in the caller's texture
    either way). Per texel the arithmetic is the separate passes': with the photometric term weighted 0
    (its gradient is then exactly zero whatever the order of its atomic adds) and no seam pairs (their
    gradient is added with atomics too) the fused run equals the separate one exactly. With both terms
    on, two runs differ by the order of their atomic adds, which Adam amplifies where a gradient
    cancels: the fused run's mean deviation from a separate run must stay within that run-to-run noise."""
    import ctypes as C

    import torch

    from photara_drender_gb300 import _native
    from photara_drender_gb300.rasterizer import _ptr

    init, pos3, uv, idx, images, mats, masks, pairs = refine_scene(2)
    valid = np.ones((64, 64), np.float32)
    valid[:3] = 0.0
    chart = (np.arange(64)[None, :] // 20 + 4 * (np.arange(64)[:, None] // 32)).astype(np.int32)
    with baker.context.lock:
        st = baker._refine_prepare(init, pos3, uv, idx, images, mats, masks, None, pairs, steps, 2, 0.05, 0.01,
                                   1e-3, 3, 1e-3, 0.9, 0.999, 1e-8, 0.0, 1.0, 1e-4, 0.05, valid, chart, 1e-4)
        o = st.options
        assert float(o.tv_scale) > 0.0
        n = len(st.weights)
        outs = []
        for fused, photometric in ((False, False), (True, False), (False, True), (False, True), (True, True)):
            vw = (C.c_double * n)(*(st.weights if photometric else [0.0] * n))
            tex = st.init.clone().contiguous()
            grad = torch.empty((64, 64, 4), dtype=torch.float32, device=tex.device)
            m1, m2 = torch.empty_like(tex), torch.empty_like(tex)
            loss = torch.zeros(steps + 3, dtype=torch.float32, device=tex.device)
            scratch = torch.empty_like(tex) if fused else None
            o.texture_scratch = scratch.data_ptr() if fused else None
            _native.call("pdr_refine_run", C.addressof(o), _ptr(st.table_dev), n, C.addressof(vw), st.max_pixels,
                         _ptr(st.pairs), st.npairs if photometric else 0, _ptr(st.tv_valid), _ptr(st.tv_chart),
                         _ptr(tex), _ptr(grad),
                         _ptr(m1), _ptr(m2), _ptr(loss), 1, baker.context.stream())
            torch.cuda.synchronize()
            outs.append([x.cpu().numpy() for x in (tex, m1, m2, loss)])
        o.texture_scratch = None
    tv_sep, tv_fused, base, again, fused = outs
    for k, name in enumerate(("texture", "moment1", "moment2", "loss")):
        # equal values (the moments of a texel with no gradient may differ in the sign of zero)
        assert np.array_equal(tv_fused[k], tv_sep[k]), name
        if name == "texture":
            assert not np.array_equal(tv_sep[k], base[k])  # the photometric term is on in the second group
        noise = np.abs(again[k] - base[k]).mean()
        dev = np.abs(fused[k] - base[k]).mean()
        scale = np.abs(base[k]).max()
        assert dev <= max(4.0 * noise, 1e-7 * scale), (name, dev, noise)

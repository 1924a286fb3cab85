"""The reference's own known-answer tests (tests/native_tests.cpp, tests/python_smoke.py)
restated against the oracle."""
import numpy as np

from oracle import api

TRI = np.array([[-0.75, -0.75, 0.0, 1.0], [0.75, -0.75, 0.0, 1.0], [0.0, 0.75, 0.0, 1.0]], np.float32)
IDX = np.array([[0, 1, 2]], np.uint32)


def test_coverage_and_raster_fd():
    # native_tests.cpp:133-157
    raster, deriv = api.rasterize_forward(TRI, IDX, (32, 32))
    assert raster[..., 3].sum() > 100.0
    grad = np.zeros_like(raster)
    grad[..., 0] = (raster[..., 3] > 0).astype(np.float32)
    g = api.rasterize_backward(TRI, IDX, raster, grad)
    assert np.isfinite(g).all()
    eps = np.float32(1e-3)
    p, n = TRI.copy(), TRI.copy()
    p[0, 0] += eps
    n[0, 0] -= eps
    fd = (api.rasterize_forward(p, IDX, (32, 32))[0][..., 0].sum(dtype=np.float32)
          - api.rasterize_forward(n, IDX, (32, 32))[0][..., 0].sum(dtype=np.float32)) / (2 * eps)
    assert abs(g[0, 0] - fd) < 0.2


def test_texture_fd():
    # native_tests.cpp:176-233
    raster, _ = api.rasterize_forward(TRI, IDX, (32, 32))
    uv = api.interpolate_forward(np.array([[0.2, 0.2], [0.8, 0.2], [0.5, 0.8]], np.float32), IDX, raster)
    tex = np.zeros((4, 4, 2), np.float32)
    for y in range(4):
        for x in range(4):
            tex[y, x] = (x + y * 2, x * 3 - y)
    s = api.texture_forward(tex, uv, raster)
    gs = np.zeros_like(s)
    cp = int(np.flatnonzero(raster[..., 3].reshape(-1) != 0)[0])
    gs.reshape(-1, 2)[cp, 0] = 1.0
    gt, gu = api.texture_backward(tex, uv, raster, gs)
    eps = np.float32(1e-3)
    up, un = uv.copy(), uv.copy()
    up.reshape(-1, 2)[cp, 0] += eps
    un.reshape(-1, 2)[cp, 0] -= eps
    fd = (api.texture_forward(tex, up, raster).reshape(-1, 2)[cp, 0]
          - api.texture_forward(tex, un, raster).reshape(-1, 2)[cp, 0]) / (2 * eps)
    assert abs(gu.reshape(-1, 2)[cp, 0] - fd) < 1e-3
    k = int(np.flatnonzero(np.abs(gt.reshape(-1)) >= 1e-8)[0])
    tp, tn = tex.copy(), tex.copy()
    tp.reshape(-1)[k] += eps
    tn.reshape(-1)[k] -= eps
    fd = (api.texture_forward(tp, uv, raster).reshape(-1, 2)[cp, 0]
          - api.texture_forward(tn, uv, raster).reshape(-1, 2)[cp, 0]) / (2 * eps)
    assert abs(gt.reshape(-1)[k] - fd) < 1e-3


def test_viewport_clip():
    # native_tests.cpp:235-249
    raster, _ = api.rasterize_forward(TRI, IDX, (32, 32), viewport=(8.0, 4.0, 16.0, 20.0))
    ys, xs = np.nonzero(raster[..., 3])
    assert len(xs) > 0 and xs.min() >= 8 and xs.max() < 24 and ys.min() >= 4 and ys.max() < 24


def _bake_inputs():
    wp = TRI[:, :3].copy()
    wn = np.tile(np.array([[0, 0, 1]], np.float32), (3, 1))
    buv = np.array([[0.125, 0.125], [0.875, 0.125], [0.5, 0.875]], np.float32)
    img = np.zeros((16, 16, 4), np.float32)
    img[...] = (0.8, 0.2, 0.1, 1.0)
    return wp, wn, buv, img


def test_bake_colour_and_face_ids():
    # native_tests.cpp:323-364 (shadow-map visibility)
    wp, wn, buv, img = _bake_inputs()
    color, conf, src, valid, cov, faces = api.bake(wp, wn, buv, IDX, [img], [np.eye(4, dtype=np.float32)],
                                                   [[0, 0, 2]], resolution=(16, 16))
    assert np.array_equal(faces, np.where(cov > 0.5, 0, 0xFFFFFFFF).astype(np.uint32))
    assert (valid > 0.5).any()
    first = np.flatnonzero(valid.reshape(-1) > 0.5)[0]
    assert abs(color.reshape(-1, 4)[first, 0] - 0.8) < 1e-4


def test_softmax_prefers_near_view_and_mask_floor():
    # native_tests.cpp:376-436
    wp, wn, buv, img = _bake_inputs()
    far = img.copy()
    far[..., :3] = (0.1, 0.2, 0.8)
    eye = np.eye(4, dtype=np.float32)
    avg = api.bake(wp, wn, buv, IDX, [img, far], [eye, eye], [[0, 0, 2], [0, 0, 6]], resolution=(16, 16))
    sm = api.bake(wp, wn, buv, IDX, [img, far], [eye, eye], [[0, 0, 2], [0, 0, 6]], resolution=(16, 16),
                  blend_mode="softmax")
    i = np.flatnonzero(sm[3].reshape(-1) > 0.5)[0]
    assert sm[4].reshape(-1)[i] > 0.5
    assert sm[0].reshape(-1, 4)[i, 0] > avg[0].reshape(-1, 4)[i, 0] + 0.05
    assert abs(sm[0].reshape(-1, 4)[i, 0] - 0.8) < 0.05
    zero = np.zeros((16, 16), np.float32)
    strict = api.bake(wp, wn, buv, IDX, [img], [eye], [[0, 0, 2]], resolution=(16, 16), blend_mode="softmax",
                      visibility_masks=[zero])
    assert not (strict[3] > 0).any()
    floored = api.bake(wp, wn, buv, IDX, [img], [eye], [[0, 0, 2]], resolution=(16, 16), blend_mode="softmax",
                       visibility_masks=[zero], mask_floor=0.1)
    j = np.flatnonzero(floored[3].reshape(-1) > 0.5)[0]
    assert abs(floored[0].reshape(-1, 4)[j, 0] - 0.8) < 1e-3


def test_softmax_scale_known_answer():
    # native_tests.cpp:114-117
    assert abs(api.suggest_softmax_scale([[0, 0, 0]], [[0, 0, 2]]) - 80.0) < 1e-3


def test_refine_loss_decreases():
    # tests/python_smoke.py:83-100 (three steps, batch 1, no seam polish)
    wp, wn, buv, img = _bake_inputs()
    img[..., :3] = (0.75, 0.25, 0.0)
    baked = api.bake(wp, wn, buv, IDX, [img], [np.eye(4, dtype=np.float32)], [[0, 0, 2]], resolution=(16, 16))[0]
    out, loss, seam = api.refine(baked[..., :3] * 0.5, wp, buv, IDX, [img], [np.eye(4, dtype=np.float32)], steps=3,
                                 batch_size=1, learning_rate=0.05, minimum_learning_rate=0.01, seam_polish_steps=0)
    assert out.shape == (16, 16, 3) and loss.shape == (3,) and np.isfinite(loss).all()
    assert loss[-1] < loss[0]
    assert seam.shape == (0,)

"""The oracle's restatement of src/texture_padding.cpp (pad_texture_atlas, fill_texture_on_surface)
against golden vectors made by the reference's own code, against the reference built here (when its
sources are present) and against the reference's known-answer tests."""
import os

import numpy as np
import pytest

from oracle import api, ref_api
from photara_drender_gb300 import synthetic as S
from tests.padding_cases import chart_atlas, surface_case

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "padding_small.npz")


def same_bits(a, b):
    a, b = np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_padding_golden():
    g = np.load(GOLDEN)
    for k in range(5):
        margin, fill, limit = (int(v) for v in g[f"p{k}_args"])
        c, f, st = api.pad_texture_atlas(g[f"p{k}_color"], g[f"p{k}_valid"], margin,
                                         coverage_mask=g[f"p{k}_cov"] if k != 3 else None,
                                         filled_mask=g[f"p{k}_filled"], fill_unobserved=bool(fill),
                                         maximum_fill_distance=limit, valid_threshold=float(g[f"p{k}_thr"]))
        assert same_bits(c, g[f"p{k}_out"]) and same_bits(f, g[f"p{k}_out_filled"]), k
        assert st == tuple(int(v) for v in g[f"p{k}_stats"]), k
    for k in range(2):
        c, f, st = api.fill_texture_on_surface(g[f"s{k}_color"], g[f"s{k}_valid"], g[f"s{k}_faces"], g["s_idx"])
        assert same_bits(c, g[f"s{k}_out"]) and same_bits(f, g[f"s{k}_out_filled"]), k
        assert st == tuple(int(v) for v in g[f"s{k}_stats"]), k


@pytest.mark.skipif(not ref_api.available(), reason="reference sources absent")
def test_padding_matches_reference_build():
    rng = np.random.default_rng(5)
    for trial in range(120):
        h, w = int(rng.integers(1, 80)), int(rng.integers(1, 80))
        color, valid, cov, filled = chart_atlas(rng, h, w, int(rng.choice([3, 4])))
        kw = dict(coverage_mask=cov if trial % 4 else None, filled_mask=filled if trial % 3 else None,
                  fill_unobserved=bool(trial % 2), maximum_fill_distance=int(rng.choice([0, 2, 9])),
                  valid_threshold=float(rng.choice([0.5, 1.0, 0.3])))
        margin = int(rng.choice([0, 1, 3, 7]))
        a, b = api.pad_texture_atlas(color, valid, margin, **kw), ref_api.pad_texture_atlas(color, valid, margin, **kw)
        assert a[2] == b[2] and same_bits(a[0], b[0]) and same_bits(a[1], b[1]), trial


@pytest.mark.skipif(not ref_api.available(), reason="reference sources absent")
def test_surface_fill_matches_reference_build():
    rng = np.random.default_rng(6)
    pos3, idx = S.icosphere(2)
    uv = S.spherical_uv(pos3)
    for trial in range(12):
        color, valid, faces = surface_case(rng, pos3, idx, uv, (int(rng.integers(8, 60)), int(rng.integers(8, 60))),
                                           3 + trial % 2)
        if trial % 3 == 0:
            color[..., 1] *= np.float32(1e-30)  # sums that depend on the summation order
        prior = (rng.uniform(size=valid.shape) > 0.5).astype(np.float32) if trial % 2 else None
        a = api.fill_texture_on_surface(color, valid, faces, idx, filled_mask=prior)
        b = ref_api.fill_texture_on_surface(color, valid, faces, idx, filled_mask=prior)
        assert a[2] == b[2] and same_bits(a[0], b[0]) and same_bits(a[1], b[1]), trial


def padding_known_atlas():
    """tests/native_tests.cpp:34-61: a 4x4 sampled block and an 8x8 covered chart without samples."""
    n = 24
    color = np.zeros((n, n, 4), np.float32)
    valid = np.zeros((n, n), np.float32)
    cov = np.zeros((n, n), np.float32)
    valid[2:6, 2:6] = 1
    cov[2:6, 2:6] = 1
    color[2:6, 2:6] = (0.25, 0.5, 0.75, 1.0)
    cov[10:18, 10:18] = 1
    return color, valid, cov


def check_padding_known_answers(pad):
    """tests/native_tests.cpp:63-112 through `pad(color, valid, margin, cov, fill)`."""
    color, valid, cov = padding_known_atlas()
    out, filled, st = pad(color, valid, 3, cov, True)
    assert st.valid_texels == 16 and st.filled_texels == st.gutter_texels + st.unobserved_texels
    assert st.gutter_texels > 0 and st.unobserved_texels == 64 and st.remaining_unobserved == 0
    assert np.allclose(out[6, 2], (0.25, 0.5, 0.75, 1.0), atol=1e-6) and out[6, 2, 3] == 1.0
    assert np.allclose(out[10, 10], (0.25, 0.5, 0.75, 1.0), atol=1e-6)
    assert filled[10, 10] > 0.5 and filled[2, 2] < 0.5
    assert out[12, 2, 0] == 0.0
    color[...] = 0
    out, filled, st = pad(color, valid, 0, cov, False)
    assert st.filled_texels == 0 and st.remaining_unobserved == 64


class _Stats:
    def __init__(self, s):
        self.valid_texels, self.gutter_texels, self.unobserved_texels, self.remaining_unobserved, \
            self.filled_texels = s


def test_padding_known_answers_oracle():
    check_padding_known_answers(lambda c, v, m, cov, fill: (lambda r: (r[0], r[1], _Stats(r[2])))(
        api.pad_texture_atlas(c, v, m, coverage_mask=cov, fill_unobserved=fill)))


def surface_known_atlas():
    """tests/texture_surface_fill_test.cpp:14-30: faces 0 and 1 share a mesh edge but are separated in
    UV space by face 2; face 3 is a disconnected component without samples."""
    color = np.zeros((1, 7, 4), np.float32)
    valid = np.array([[1, 0, 1, 0, 0, 0, 0]], np.float32)
    cov = np.array([[1, 1, 1, 1, 1, 0, 0]], np.float32)
    faces = np.array([[0, 0, 2, 1, 3, 0xFFFFFFFF, 0xFFFFFFFF]], np.uint32)
    color[0, 0, 0], color[0, 0, 3] = 0.8, 1.0
    color[0, 2, 2], color[0, 2, 3] = 0.6, 1.0
    topology = np.array([[0, 1, 2], [2, 1, 3], [4, 5, 6], [7, 8, 9]], np.uint32)
    return color, valid, cov, faces, topology


def check_surface_known_answers(fill, pad):
    """tests/texture_surface_fill_test.cpp:31-71 through fill(color, valid, faces, topology, filled)
    -> (color, filled, (filled, remaining, measured, propagated)) and pad(color, valid, margin, cov,
    fill, filled) -> (color, filled, (valid, gutter, unobserved, remaining, filled))."""
    color, valid, cov, faces, topology = surface_known_atlas()
    out, filled, st = fill(color, valid, faces, topology, None)
    assert st[2] == 2 and st[3] == 1 and st[0] == 2 and st[1] == 1
    assert out[0, 1, 0] == np.float32(0.8) and out[0, 3, 0] == np.float32(0.8) and out[0, 3, 2] == 0.0
    assert same_bits(out[0, [0, 2]], color[0, [0, 2]])
    padded, pfilled, pst = pad(out, valid, 2, cov, False, filled)
    assert pst[2] == 2 and pst[3] == 1
    assert padded[0, 5, 0] == np.float32(0.8) and padded[0, 4, 0] == 0.0 and pfilled[0, 3] == 1.0
    _, _, again = pad(padded, valid, 2, cov, False, pfilled)
    assert again[1] == pst[1] and again[2] == pst[2]
    bad = faces.copy()
    bad[0, 1] = 100
    with pytest.raises(ValueError, match="face ID is out of range"):
        fill(color, valid, bad, topology, None)
    _, _, st = fill(out, np.zeros_like(valid), faces, topology, None)
    assert st[0] == 0 and st[1] == 5


def test_surface_fill_known_answers_oracle():
    check_surface_known_answers(
        lambda c, v, f, t, fl: api.fill_texture_on_surface(c, v, f, t, filled_mask=fl),
        lambda c, v, m, cov, fill, fl: api.pad_texture_atlas(c, v, m, coverage_mask=cov, fill_unobserved=fill,
                                                             filled_mask=fl))


def test_surface_fill_errors_oracle():
    pos3, idx = S.icosphere(1)
    color = np.zeros((4, 4, 3), np.float32)
    valid = np.ones((4, 4), np.float32)
    faces = np.zeros((4, 4), np.uint32)
    deg = idx.copy()
    deg[3, 2] = deg[3, 0]
    with pytest.raises(ValueError, match="degenerate edge"):
        api.fill_texture_on_surface(color, valid, faces, deg)
    with pytest.raises(ValueError, match="manifold edges"):
        api.fill_texture_on_surface(color, valid, faces, np.concatenate([idx, idx[:1]]))
    with pytest.raises(ValueError, match="RGB or RGBA"):
        api.fill_texture_on_surface(np.zeros((4, 4, 2), np.float32), valid, faces, idx)

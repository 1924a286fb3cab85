"""The oracle against the reference's own shader code compiled for the CPU (oracle/_ref), on
fresh seeded inputs, including the adversarial cases the reference's tests do not cover.
Skipped where the reference sources are absent."""
import numpy as np
import pytest

from oracle import api, ref_api
from photara_drender_gb300 import synthetic as S
from tests.raster_scenes import tie_scene

pytestmark = pytest.mark.skipif(not ref_api.available(), reason="reference sources not available")


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(np.ascontiguousarray(a).view(np.uint32),
                                                 np.ascontiguousarray(b).view(np.uint32))


def adversarial_meshes():
    rng = np.random.default_rng(5)
    cases = []
    # shared edges and coincident depths: a quad split twice, duplicated triangles at equal depth
    pos = np.array([[-0.8, -0.8, 0.1, 1], [0.8, -0.8, 0.1, 1], [0.8, 0.8, 0.1, 1], [-0.8, 0.8, 0.1, 1],
                    [0.0, 0.0, 0.1, 1.0]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3], [0, 1, 4], [1, 2, 4], [2, 3, 4], [3, 0, 4], [0, 2, 3]], np.uint32)
    cases.append((pos, idx))
    # w <= 1e-8, negative w, slivers, huge off-screen coordinates, degenerate (repeated vertex) faces
    pos = rng.uniform(-1.5, 1.5, size=(40, 4)).astype(np.float32)
    pos[:, 3] = rng.uniform(0.2, 2.0, size=40)
    pos[3, 3] = 0.0
    pos[4, 3] = -1.0
    pos[5, 3] = 1e-9
    pos[6, :2] = (1e6, -1e6)
    pos[7, :2] = (pos[8, 0] + 1e-6, pos[8, 1])
    idx = rng.integers(0, 40, size=(120, 3)).astype(np.uint32)
    idx[:4] = [[1, 1, 2], [7, 8, 9], [6, 10, 11], [3, 12, 13]]
    cases.append((pos, idx))
    return cases


@pytest.mark.parametrize("case", range(2))
@pytest.mark.parametrize("cull", [0, 1, 2])
def test_raster_adversarial(case, cull):
    pos, idx = adversarial_meshes()[case]
    for res, vp in [((40, 36), None), ((33, 29), (-4.0, 3.5, 41.0, 25.0))]:
        r1, d1 = api.rasterize_forward(pos, idx, res, cull_mode=cull, viewport=vp)
        r2, d2 = ref_api.rasterize_forward(pos, idx, res, cull_mode=cull, viewport=vp)
        assert same_bits(r1, r2) and same_bits(d1, d2)
        g = np.random.default_rng(1).normal(size=r1.shape).astype(np.float32)
        assert same_bits(api.rasterize_backward(pos, idx, r1, g, viewport=vp),
                         ref_api.rasterize_backward(pos, idx, r1, g, viewport=vp))


def test_tie_decisions_match_reference():
    """Pixels decided by the edge tolerance or by the lowest-id depth rule (counted by the oracle) come
    out the same in the reference's own shader code: a coplanar pixel-centre grid drawn twice."""
    pos, idx, res = tie_scene()
    r1, ties, counts = api.rasterize_tie_counts(pos, idx, res)
    r2, _ = ref_api.rasterize_forward(pos, idx, res)
    assert same_bits(r1, r2)
    assert counts["depth_ties"] > 0 and counts["edge_ties"] > 0
    # the lowest-id rule: every depth-tied pixel of the duplicated grid shows the first copy
    ids = np.rint(r1[..., 3]).astype(np.int64)
    assert (ids[(ties & 1) > 0] <= idx.shape[0] // 2).all()


@pytest.mark.parametrize("view", range(3))
def test_pipeline_sphere(view):
    rng = np.random.default_rng(view)
    pos3, idx = S.icosphere(2)
    mats, _ = S.orbit_cameras(3)
    clip = S.clip_positions(pos3, mats)[view]
    r, _ = api.rasterize_forward(clip, idx, (45, 51))
    attr = rng.uniform(size=(pos3.shape[0], 5)).astype(np.float32)
    gi = rng.normal(size=(45, 51, 5)).astype(np.float32)
    assert same_bits(api.interpolate_forward(attr, idx, r), ref_api.interpolate_forward(attr, idx, r))
    a1, r1 = api.interpolate_backward(attr, idx, r, gi)
    a2, r2 = ref_api.interpolate_backward(attr, idx, r, gi)
    assert same_bits(a1, a2) and same_bits(r1, r2)
    uv = api.interpolate_forward(S.spherical_uv(pos3), idx, r) * 2.3 - 0.6
    tex = rng.uniform(size=(13, 17, 3)).astype(np.float32)
    for mode in ("clamp", "wrap", "mirror"):
        s = api.texture_forward(tex, uv, r, mode)
        assert same_bits(s, ref_api.texture_forward(tex, uv, r, mode))
        gs = rng.normal(size=s.shape).astype(np.float32)
        t1, u1 = api.texture_backward(tex, uv, r, gs, mode)
        t2, u2 = ref_api.texture_backward(tex, uv, r, gs, mode)
        assert same_bits(t1, t2) and same_bits(u1, u2)


def test_softmax_scale_matches_reference_padding_code():
    rng = np.random.default_rng(2)
    for n in (1, 50, 25000):
        pos = rng.normal(size=(n, 3)).astype(np.float32)
        cams = (rng.normal(size=(5, 3)) * 3).astype(np.float32)
        assert api.suggest_softmax_scale(pos, cams) == ref_api.suggest_softmax_scale(pos, cams)


def test_tile_bins_match_reference_host_code():
    """The oracle's tile binning against the reference's own build_tile_bins (src/rasterizer.cpp:61-138,
    compiled from its source): offsets and triangle lists bit-identical on sphere views, adversarial
    meshes (w <= 1e-8, negative w, huge and non-finite coordinates), ragged sizes and offset viewports."""
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(3)
    clip = S.clip_positions(pos3, mats)
    cases = [(clip[k], idx) for k in range(3)] + adversarial_meshes() + [tie_scene()[:2]]
    nonfinite = clip[0].copy()
    nonfinite[5, 0] = np.inf
    nonfinite[9, 1] = np.nan
    cases.append((nonfinite, idx))
    checked = 0
    for pos, tri in cases:
        for res, vp in [((64, 64), None), ((33, 47), None), ((40, 36), (-4.0, 3.5, 41.0, 25.0)),
                        ((17, 100), (2.5, -1.0, 90.0, 30.0))]:
            o1, l1 = api.bin_tiles(pos, tri, res, vp)
            o2, l2 = ref_api.bin_tiles(pos, tri, res, vp)
            assert np.array_equal(o1, o2) and np.array_equal(l1, l2), (res, vp)
            checked += l2.size
    assert checked > 1000


def test_texel_tables_match_reference_host_code():
    """The oracle's texture adjoint uses the reference's texel->sample table (src/rasterizer.cpp:187-258,
    double-precision texel positions); texel gradients from the reference's own table builder and
    texture_grad_texture shader equal the oracle's, in all address modes, with uv far outside [0,1]."""
    rng = np.random.default_rng(11)
    h, w = 24, 20
    raster = np.zeros((h, w, 4), np.float32)
    raster[..., 3] = (rng.uniform(size=(h, w)) < 0.7) * 5.0
    uv = rng.uniform(-1.5, 2.5, size=(h, w, 2)).astype(np.float32)
    uv[0, :4] = [[0.5 / 7, 0.5 / 9], [1.0, 0.0], [-0.0, 1e-30], [3.999999, -2.000001]]
    tex = rng.uniform(size=(9, 7, 4)).astype(np.float32)
    g = rng.normal(size=(h, w, 4)).astype(np.float32)
    for mode in ("clamp", "wrap", "mirror"):
        gt1, gu1 = api.texture_backward(tex, uv, raster, g, address_mode=mode)
        gt2, gu2 = ref_api.texture_backward(tex, uv, raster, g, address_mode=mode)
        assert same_bits(gt1, gt2) and same_bits(gu1, gu2), mode

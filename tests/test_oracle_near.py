"""Near-plane clipping on the CPU (the reference has none: README.md:140, docs/architecture.md:62 drop every
triangle with a vertex at w <= 1e-8). The oracle's float32 restatement of the clipped raster
(oracle/api.py rasterize_forward_near) is checked against what each pixel should see, decided in float64
from the geometry alone (near_truth_f64); the float64 adjoint (rasterize_backward_near) is checked by
central differences and, where nothing is clipped, against the reference-order oracle."""
import numpy as np
import pytest

from oracle import api
from photara_drender_gb300 import synthetic as S
from tests.near_scenes import cloud, ground


def _behind(clip, idx):
    return (np.asarray(clip)[np.asarray(idx, np.int64)][..., 3] <= np.float32(1e-8)).any(1)


def test_clipped_mesh_slots():
    clip, idx, _ = cloud()
    cp, ci = api.clip_near(clip, idx)
    T = idx.shape[0]
    assert cp.shape == (4 * T, 4) and ci.shape == (2 * T, 3)
    assert np.array_equal(ci[0::2], 4 * np.arange(T)[:, None] + [0, 1, 2])
    assert np.array_equal(ci[1::2], 4 * np.arange(T)[:, None] + [0, 2, 3])
    P = clip[idx.astype(np.int64)]
    n_in = ((P[..., 2] + P[..., 3]) >= 0).sum(1)
    slots = cp.reshape(T, 4, 4)
    assert np.array_equal(slots[n_in == 3, :3], P[n_in == 3]) and not slots[n_in == 3, 3].any()
    assert not slots[n_in == 0].any()
    used = slots[n_in > 0][..., 3] != 0
    zw = (slots[..., 2] + slots[..., 3])[n_in > 0][used]
    scale = np.abs(P).max()
    assert zw.min() >= -1e-6 * scale, "every clipped vertex lies in front of the near plane"
    assert (slots[n_in > 0][..., 3][used] > 0).all(), "clipped vertices are in front of the eye"
    assert set(np.bincount(n_in, minlength=4)[1:3]) != {0}, "the scene crosses the near plane"


def test_shared_edges_get_identical_points():
    clip, idx, _ = ground()
    cp, _ = api.clip_near(clip, idx)
    slots = cp.reshape(-1, 4, 4)
    P = clip[idx.astype(np.int64)]
    inside = (P[..., 2] + P[..., 3]) >= 0
    # every intersection point of an edge shared by two triangles appears bit-identically in both
    points = {}
    for t, tri in enumerate(idx.astype(np.int64)):
        for e in range(3):
            a, b = tri[e], tri[(e + 1) % 3]
            if inside[t, e] != inside[t, (e + 1) % 3]:
                key = (min(a, b), max(a, b))
                zw = slots[t, :, 2] + slots[t, :, 3]
                cand = {tuple(slots[t, s].view(np.uint32)) for s in range(4) if slots[t, s, 3] != 0 and
                        not np.any(np.all(slots[t, s] == P[t], axis=1)) and abs(zw[s]) <= 1e-5}
                points.setdefault(key, []).append(cand)
    shared = [v for v in points.values() if len(v) == 2]
    assert shared
    for a, b in shared:
        assert a & b, "the two triangles of an edge share its near-plane point"


def test_nothing_clipped_is_the_plain_raster():
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(2)
    clip = S.clip_positions(pos3, mats)
    for k in range(2):
        for cull in (0, 1):
            r, d = api.rasterize_forward_near(clip[k], idx, (72, 64), cull, viewport=(3.0, -2.0, 60.0, 70.0))
            r0, d0 = api.rasterize_forward(clip[k], idx, (72, 64), cull, viewport=(3.0, -2.0, 60.0, 70.0))
            assert np.array_equal(r.view(np.uint32), r0.view(np.uint32))
            assert np.array_equal(d.view(np.uint32), d0.view(np.uint32))


@pytest.mark.parametrize("scene", [ground, cloud])
@pytest.mark.parametrize("cull", [0, 1, 2])
def test_near_raster_matches_float64_geometry(scene, cull):
    """Triangle ids equal the float64 decision on every pixel not within 1e-4 (barycentric units) of an
    edge or the near plane and not a depth near-tie; barycentrics within 1e-5 and depth within 1e-5 of
    float64 on those pixels, including triangles with vertices behind the eye."""
    clip, idx, res = scene()
    r, _ = api.rasterize_forward_near(clip, idx, res, cull)
    ids, lam, depth = api.near_truth_f64(clip, idx, res, cull)
    got = np.rint(r[..., 3]).astype(np.int64)
    decided = ids >= 0
    assert np.count_nonzero(~decided) <= 0.02 * ids.size
    assert np.array_equal(got[decided], ids[decided])
    ok = decided & (ids > 0)
    assert np.abs(r[..., :2].astype(np.float64) - lam)[ok].max(initial=0) <= 1e-5
    assert np.abs(r[..., 2].astype(np.float64) - depth)[ok].max(initial=0) <= 1e-5
    if cull != 1 or scene is cloud:
        behind = _behind(clip, idx)
        assert behind[got[ok] - 1].any(), "triangles with a vertex behind the eye are drawn"
        plain, _ = api.rasterize_forward(clip, idx, res, cull)
        assert np.count_nonzero(got) > np.count_nonzero(np.rint(plain[..., 3]))


def _fd_loss(clip, idx, raster, grad, vp):
    """sum over owned pixels of grad . (a0, a1) / (A + 1e-6f sign A), the barycentrics as the adjoint
    differentiates them, in float64 for fixed pixel ownership."""
    h, w = raster.shape[:2]
    ids = np.rint(raster[..., 3]).astype(np.int64).reshape(-1)
    pix = np.flatnonzero(ids > 0)
    tri = np.asarray(idx, np.int64)[ids[pix] - 1]
    sx = ((pix % w) - vp[0] + 0.5) * 2.0 / vp[2] - 1.0
    sy = ((pix // w) - vp[1] + 0.5) * 2.0 / vp[3] - 1.0
    p = [clip[tri[:, m]] for m in range(3)]
    q = [(pp[:, 0] - sx * pp[:, 3], pp[:, 1] - sy * pp[:, 3]) for pp in p]
    cr = lambda u, v: u[0] * v[1] - u[1] * v[0]  # noqa: E731
    a0, a1 = cr(q[1], q[2]), cr(q[2], q[0])
    A = a0 + a1 + cr(q[0], q[1])
    e6 = float(np.float32(1e-6))
    inv = 1.0 / (A + np.where(A >= 0, e6, -e6))
    g = grad.reshape(-1, 4)[pix].astype(np.float64)
    return float((g[:, 0] * a0 * inv + g[:, 1] * a1 * inv).sum())


def test_near_backward_matches_central_differences():
    clip, idx, res = ground()
    raster, _ = api.rasterize_forward_near(clip, idx, res)
    grad = np.random.default_rng(4).normal(size=raster.shape).astype(np.float32)
    got = api.rasterize_backward_near(clip, idx, raster, grad)
    vp = np.array([0.0, 0.0, res[1], res[0]])
    owned = np.unique(idx[np.rint(raster[..., 3]).astype(np.int64)[raster[..., 3] > 0] - 1])
    behind_v = np.flatnonzero(clip[:, 3] <= 1e-8)
    behind_owned = np.intersect1d(owned, behind_v)
    checked = behind_owned[:4].tolist() + np.setdiff1d(owned, behind_v)[::7][:4].tolist()
    assert behind_owned.size >= 1 and len(checked) >= 5
    c64 = clip.astype(np.float64)
    for v in checked:
        for comp in (0, 1, 3):
            h = 1e-6 * max(1.0, abs(c64[v, comp]))
            cp, cm = c64.copy(), c64.copy()
            cp[v, comp] += h
            cm[v, comp] -= h
            fd = (_fd_loss(cp, idx, raster, grad, vp) - _fd_loss(cm, idx, raster, grad, vp)) / (2 * h)
            assert abs(got[v, comp] - fd) <= 1e-6 * max(1.0, abs(fd)), (v, comp, got[v, comp], fd)
    assert not got[:, 2].any()


def test_near_backward_is_the_reference_adjoint_when_nothing_is_behind():
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(1)
    clip = S.clip_positions(pos3, mats)[0]
    raster, _ = api.rasterize_forward(clip, idx, (64, 56))
    grad = np.random.default_rng(5).normal(size=raster.shape).astype(np.float32)
    ours = api.rasterize_backward_near(clip, idx, raster, grad)
    ref64 = api.rasterize_backward(clip, idx, raster, grad, f64=True)
    assert np.allclose(ours, ref64, rtol=1e-10, atol=1e-12 * np.abs(ref64).max())

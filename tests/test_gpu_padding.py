"""Atlas padding and surface fill on the GPU (csrc/padding.cu through the C ABI) against the oracle's
restatement of src/texture_padding.cpp and the reference-made golden vectors: bit for bit, including
the statistics."""
import os

import numpy as np
import pytest
import torch

from oracle import api
from photara_drender_gb300 import padding as P
from photara_drender_gb300 import synthetic as S
from tests.gpu_util import same_bits
from tests.padding_cases import chart_atlas, surface_case
from tests.test_oracle_padding import check_padding_known_answers, check_surface_known_answers

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "padding_small.npz")


def gpu_pad(color, valid, margin, cov=None, fill=True, filled=None, limit=0, thr=0.5):
    dev = torch.device("cuda", 0)
    c = torch.tensor(color, device=dev)
    v = torch.tensor(valid, device=dev)
    cv = None if cov is None else torch.tensor(cov, device=dev)
    f = torch.zeros(valid.shape, dtype=torch.float32, device=dev) if filled is None else torch.tensor(filled, device=dev)
    st = P.pad_texture_atlas_device(c, v, margin, cv, fill, limit, filled_mask=f, valid_threshold=thr)
    return c.cpu().numpy(), f.cpu().numpy(), st


def test_padding_golden():
    g = np.load(GOLDEN)
    for k in range(5):
        margin, fill, limit = (int(x) for x in g[f"p{k}_args"])
        c, f, st = gpu_pad(g[f"p{k}_color"], g[f"p{k}_valid"], margin, g[f"p{k}_cov"] if k != 3 else None,
                           bool(fill), g[f"p{k}_filled"], limit, float(g[f"p{k}_thr"]))
        assert same_bits(c, g[f"p{k}_out"]) and same_bits(f, g[f"p{k}_out_filled"]), k
        assert tuple(st) == tuple(int(x) for x in g[f"p{k}_stats"]), k


def test_padding_random_matches_oracle():
    rng = np.random.default_rng(11)
    shapes = [(1, 1), (1, 97), (97, 1), (31, 33), (32, 32), (33, 31), (64, 65), (65, 64), (5, 200), (200, 5),
              (129, 70), (70, 129)]
    for k, (h, w) in enumerate(shapes * 3):
        color, valid, cov, filled = chart_atlas(rng, h, w, 4 if k % 2 else 3)
        margin = int(rng.choice([0, 1, 2, 5, 40]))
        fill, limit = bool(k % 3), int(rng.choice([0, 0, 4]))
        thr = float(rng.choice([0.5, 1.0]))
        use_cov = cov if k % 5 else None
        c, f, st = gpu_pad(color, valid, margin, use_cov, fill, filled, limit, thr)
        oc, of, ost = api.pad_texture_atlas(color, valid, margin, coverage_mask=use_cov, filled_mask=filled,
                                            fill_unobserved=fill, maximum_fill_distance=limit, valid_threshold=thr)
        assert tuple(st) == ost, (h, w, k)
        assert same_bits(c, oc) and same_bits(f, of), (h, w, k)


def test_padding_ties_and_sparse_sources():
    # sources on a lattice: many texels are equidistant from several sources, so the colour they take
    # is decided by the sweeps' order of relaxation and strict comparisons alone
    rng = np.random.default_rng(2)
    for h, w, step in ((96, 130, 7), (257, 190, 16), (300, 300, 61)):
        valid = np.zeros((h, w), np.float32)
        valid[::step, ::step] = 1
        valid[rng.integers(0, h, 5), rng.integers(0, w, 5)] = 1
        color = rng.uniform(size=(h, w, 4)).astype(np.float32)
        cov = (rng.uniform(size=(h, w)) > 0.5).astype(np.float32)
        c, f, st = gpu_pad(color, valid, 9, cov, True)
        oc, of, ost = api.pad_texture_atlas(color, valid, 9, coverage_mask=cov, fill_unobserved=True)
        assert tuple(st) == ost and same_bits(c, oc) and same_bits(f, of), (h, w)


def test_padding_no_sources_leaves_atlas():
    color = np.random.default_rng(0).uniform(size=(40, 50, 4)).astype(np.float32)
    valid = np.zeros((40, 50), np.float32)
    filled = np.ones((40, 50), np.float32)
    c, f, st = gpu_pad(color, valid, 4, None, True, filled)
    oc, of, ost = api.pad_texture_atlas(color, valid, 4, filled_mask=filled)
    assert tuple(st) == ost == (0, 0, 0, 0, 0)
    assert same_bits(c, color) and same_bits(f, of) and not f.any()


def test_padding_large_atlas_matches_oracle():
    # a 4096x4096 atlas: 128 bands of 32 rows through the sweeps' boundary hand-off
    rng = np.random.default_rng(9)
    color, valid, cov, filled = chart_atlas(rng, 4096, 4096, 4, charts=40)
    c, f, st = gpu_pad(color, valid, 8, cov, True, filled)
    oc, of, ost = api.pad_texture_atlas(color, valid, 8, coverage_mask=cov, filled_mask=filled)
    assert tuple(st) == ost and same_bits(c, oc) and same_bits(f, of)


def test_padding_repeated_is_stable():
    rng = np.random.default_rng(4)
    color, valid, cov, _ = chart_atlas(rng, 120, 90, 4)
    c1, f1, s1 = gpu_pad(color, valid, 3, cov, False)
    c2, f2, s2 = gpu_pad(c1, valid, 3, cov, False, f1)
    o2 = api.pad_texture_atlas(c1, valid, 3, coverage_mask=cov, filled_mask=f1, fill_unobserved=False)
    assert tuple(s2) == o2[2] and same_bits(c2, o2[0]) and same_bits(f2, o2[1])
    assert s2.gutter_texels == s1.gutter_texels


def _gpu_pad_tuple(c, v, m, cov, fill, filled=None):
    out, f, st = gpu_pad(c, v, m, cov, fill, filled)
    return out, f, tuple(st)


def test_padding_known_answers_gpu():
    check_padding_known_answers(lambda c, v, m, cov, fill: gpu_pad(c, v, m, cov, fill))


def test_surface_fill_known_answers_gpu():
    check_surface_known_answers(
        lambda c, v, f, t, fl: P.fill_texture_on_surface(c, v, f, t, filled_mask=fl),
        lambda c, v, m, cov, fill, fl: _gpu_pad_tuple(c, v, m, cov, fill, fl))


def test_surface_fill_golden_and_oracle():
    g = np.load(GOLDEN)
    for k in range(2):
        c, f, st = P.fill_texture_on_surface(g[f"s{k}_color"], g[f"s{k}_valid"], g[f"s{k}_faces"], g["s_idx"])
        assert same_bits(c, g[f"s{k}_out"]) and same_bits(f, g[f"s{k}_out_filled"]), k
        assert tuple(st) == tuple(int(x) for x in g[f"s{k}_stats"]), k
    rng = np.random.default_rng(8)
    pos3, nrm, uv, idx, chart, remap = S.displaced_sphere(20000, seed=3, atlas_size=512)
    # face ids of the seam-split atlas mesh, topology of the original welded mesh
    welded = remap[idx].astype(np.uint32)
    for k in range(3):
        color, valid, faces = surface_case(rng, pos3, idx, uv, (512, 512), 3 + k % 2)
        if k == 2:
            color[..., 0] *= np.float32(1e-30)
        prior = (rng.uniform(size=valid.shape) > 0.7).astype(np.float32) if k == 1 else None
        c, f, st = P.fill_texture_on_surface(color, valid, faces, welded, filled_mask=prior)
        oc, of, ost = api.fill_texture_on_surface(color, valid, faces, welded, filled_mask=prior)
        assert tuple(st) == ost and same_bits(c, oc) and same_bits(f, of), k
        assert st.propagated_faces > 0


def test_surface_fill_errors_gpu():
    pos3, idx = S.icosphere(1)
    color = np.zeros((4, 4, 3), np.float32)
    valid = np.ones((4, 4), np.float32)
    faces = np.zeros((4, 4), np.uint32)
    bad_faces = faces.copy()
    bad_faces[1, 1] = idx.shape[0]
    deg = idx.copy()
    deg[3, 2] = deg[3, 0]
    nonmanifold = np.concatenate([idx, idx[:1]])
    with pytest.raises(ValueError, match="face ID is out of range"):
        P.fill_texture_on_surface(color, valid, bad_faces, deg)   # the face-id error takes precedence
    with pytest.raises(ValueError, match="degenerate edge"):
        P.fill_texture_on_surface(color, valid, faces, deg)
    with pytest.raises(ValueError, match="manifold edges"):
        P.fill_texture_on_surface(color, valid, faces, nonmanifold)
    with pytest.raises(ValueError, match="RGB or RGBA"):
        P.fill_texture_on_surface(np.zeros((4, 4, 2), np.float32), valid, faces, idx)


def test_pad_texture_atlas_wrapper_and_project():
    # python/photara_drender/baking.py:33-80 semantics, then project_texture_atlas(padding=...)
    rng = np.random.default_rng(1)
    color, valid, cov, _ = chart_atlas(rng, 64, 48, 4)
    out = P.pad_texture_atlas(color, valid > 0, 2, coverage_mask=cov, fill_unobserved=True)
    ref = api.pad_texture_atlas(color, (valid > 0).astype(np.float32), 2, coverage_mask=cov)[0]
    assert same_bits(out, ref)
    assert same_bits(P.pad_texture_atlas(color, valid, 0), color)
    with pytest.raises(ValueError, match="non-negative"):
        P.pad_texture_atlas(color, valid, -1)
    t = torch.tensor(color, device="cuda")
    assert same_bits(P.pad_texture_atlas(t, torch.tensor(valid, device="cuda"), 2, coverage_mask=torch.tensor(
        cov, device="cuda"), fill_unobserved=True).cpu().numpy(), ref)

    from photara_drender_gb300 import TextureBaker, UnwrappedMesh, project_texture_atlas

    baker = TextureBaker(0)
    pos3, idx = S.icosphere(3)
    nrm = S.vertex_normals(pos3, idx)
    uv = S.spherical_uv(pos3)
    mats, eyes = S.orbit_cameras(2)
    images = [rng.uniform(size=(48, 64, 3)).astype(np.float32) for _ in range(2)]
    mesh = UnwrappedMesh(pos3, nrm, uv, idx, np.arange(len(pos3), dtype=np.uint32), np.zeros(len(idx), np.uint32), 1,
                         1.0)
    plain = project_texture_atlas(mesh, images, mats, eyes, baker=baker, resolution=(64, 64),
                                  visibility_mode="shadow_map")
    padded = project_texture_atlas(mesh, images, mats, eyes, baker=baker, resolution=(64, 64),
                                   visibility_mode="shadow_map", padding=3, fill_unobserved=True)
    ref = api.pad_texture_atlas(plain.color, (plain.valid_mask > 0).astype(np.float32), 3,
                                coverage_mask=plain.coverage_mask, fill_unobserved=True)[0]
    assert same_bits(padded.color, ref) and same_bits(padded.valid_mask, plain.valid_mask)

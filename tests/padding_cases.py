"""Seeded atlases for the padding and surface-fill tests: elliptical charts with partial sampling,
earlier fills carried over, and face ids rasterised from a mesh's UV atlas."""
import numpy as np


def chart_atlas(rng, h, w, channels=4, charts=None):
    """(color, valid, coverage, filled) of an atlas with a few elliptical charts, sampled in part."""
    cov = np.zeros((h, w), np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    for _ in range(charts if charts is not None else int(rng.integers(1, 6))):
        y0, x0 = rng.integers(0, h), rng.integers(0, w)
        ry, rx = rng.integers(1, max(2, h // 3)), rng.integers(1, max(2, w // 3))
        cov[((yy - y0) / ry) ** 2 + ((xx - x0) / rx) ** 2 <= 1] = 1
    valid = ((cov > 0) & (rng.uniform(size=(h, w)) > rng.uniform(0.1, 0.9))).astype(np.float32)
    color = (rng.uniform(size=(h, w, channels)) * valid[..., None]).astype(np.float32)
    filled = ((cov > 0) & (valid == 0) & (rng.uniform(size=(h, w)) > 0.8)).astype(np.float32)
    return color, valid, cov, filled


def surface_case(rng, pos3, idx, uv, res, channels=4):
    """(color, valid, face_ids) over the atlas of a mesh: face ids from the UV raster, a random subset
    of texels sampled."""
    from oracle import api

    h, w = res
    aclip = np.concatenate([uv * 2 - 1, np.zeros((len(uv), 1)), np.ones((len(uv), 1))], 1).astype(np.float32)
    raster, _ = api.rasterize_forward(aclip, idx, res, output_derivatives=False)
    ids = raster[..., 3].astype(np.int64)
    faces = np.where(ids > 0, ids - 1, 0xFFFFFFFF).astype(np.uint32)
    keep = rng.uniform(size=idx.shape[0]) < rng.uniform(0.2, 0.8)
    covered = faces != 0xFFFFFFFF
    valid = (covered & keep[np.where(covered, faces, 0)] & (rng.uniform(size=(h, w)) > 0.3)).astype(np.float32)
    color = (rng.uniform(size=(h, w, channels)) * (valid[..., None] > 0)).astype(np.float32)
    return color, valid, faces

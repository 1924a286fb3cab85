"""Generates the golden fixtures in this folder from the reference's own shader code.

Run here (where the reference sources exist): ``python tests/golden/make_golden.py``.
It builds ``oracle/_ref/libpdr_ref.so`` from the reference's HLSL shaders (see oracle/build.py),
runs each shader over small seeded inputs and stores inputs and outputs as ``.npz``. Tile bins,
the vertex->corner table and the texel->sample table are the host-side restatements in
oracle/ (the reference's host file needs the absent Vulkan wrapper).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))  # the repository root

from oracle import api, ref_api  # noqa: E402
from photara_drender_gb300 import synthetic as S  # noqa: E402


def triangle_case():
    """tests/native_tests.cpp:127-137: one triangle at 32x32, plus the (8,4,16,20) viewport."""
    pos = np.array([[-0.75, -0.75, 0.0, 1.0], [0.75, -0.75, 0.0, 1.0], [0.0, 0.75, 0.0, 1.0]], np.float32)
    idx = np.array([[0, 1, 2]], np.uint32)
    raster, deriv = ref_api.rasterize_forward(pos, idx, (32, 32))
    vraster, vderiv = ref_api.rasterize_forward(pos, idx, (32, 32), viewport=(8.0, 4.0, 16.0, 20.0))
    grad = np.zeros_like(raster)
    grad[..., 0] = (raster[..., 3] > 0).astype(np.float32)
    gpos = ref_api.rasterize_backward(pos, idx, raster, grad)
    vgpos = ref_api.rasterize_backward(pos, idx, vraster, grad, viewport=(8.0, 4.0, 16.0, 20.0))
    attrs = np.eye(3, dtype=np.float32)
    interp = ref_api.interpolate_forward(attrs, idx, raster)
    ga, gr = ref_api.interpolate_backward(attrs, idx, raster, np.ones_like(interp))
    vuv = np.array([[0.2, 0.2], [0.8, 0.2], [0.5, 0.8]], np.float32)
    uv = ref_api.interpolate_forward(vuv, idx, raster)
    tex = np.zeros((4, 4, 2), np.float32)
    for y in range(4):
        for x in range(4):
            tex[y, x] = (x + y * 2, x * 3 - y)
    sampled = ref_api.texture_forward(tex, uv, raster)
    gs = np.zeros_like(sampled)
    covered = int(np.flatnonzero(raster[..., 3].reshape(-1) != 0)[0])
    gs.reshape(-1, 2)[covered, 0] = 1.0
    gt, gu = ref_api.texture_backward(tex, uv, raster, gs)
    np.savez_compressed(os.path.join(HERE, "triangle_32.npz"), pos=pos, idx=idx, raster=raster, deriv=deriv,
                        vraster=vraster, vderiv=vderiv, grad=grad, gpos=gpos, vgpos=vgpos, attrs=attrs,
                        interp=interp, ga=ga, gr=gr, vuv=vuv, uv=uv, tex=tex, sampled=sampled, gs=gs, gt=gt, gu=gu)


def sphere_case():
    rng = np.random.default_rng(7)
    pos3, idx = S.icosphere(2)
    mats, _ = S.orbit_cameras(2)
    clip = S.clip_positions(pos3, mats)
    uvv = S.spherical_uv(pos3)
    out = {"pos3": pos3, "idx": idx, "clip": clip, "vuv": uvv}
    for k, (res, vp) in enumerate([((48, 40), None), ((37, 53), (3.0, 5.0, 40.0, 30.0))]):
        raster, deriv = ref_api.rasterize_forward(clip[k], idx, res, viewport=vp, cull_mode=k)
        grad = rng.normal(size=raster.shape).astype(np.float32)
        gpos = ref_api.rasterize_backward(clip[k], idx, raster, grad, viewport=vp)
        attr = rng.uniform(size=(pos3.shape[0], 3)).astype(np.float32)
        interp = ref_api.interpolate_forward(attr, idx, raster)
        gi = rng.normal(size=interp.shape).astype(np.float32)
        ga, gr = ref_api.interpolate_backward(attr, idx, raster, gi)
        uv = ref_api.interpolate_forward(uvv, idx, raster) * 1.7 - 0.3
        tex = rng.uniform(size=(16, 24, 4)).astype(np.float32)
        out.update({f"raster{k}": raster, f"deriv{k}": deriv, f"grad{k}": grad, f"gpos{k}": gpos, f"attr{k}": attr,
                    f"interp{k}": interp, f"gi{k}": gi, f"ga{k}": ga, f"gr{k}": gr, f"uv{k}": uv, f"tex{k}": tex,
                    f"vp{k}": np.asarray(vp if vp else (0, 0, res[1], res[0]), np.float32)})
        for mode in ("clamp", "wrap", "mirror"):
            s = ref_api.texture_forward(tex, uv, raster, mode)
            gs = rng.normal(size=s.shape).astype(np.float32)
            gt, gu = ref_api.texture_backward(tex, uv, raster, gs, mode)
            out.update({f"s{k}_{mode}": s, f"gs{k}_{mode}": gs, f"gt{k}_{mode}": gt, f"gu{k}_{mode}": gu})
    np.savez_compressed(os.path.join(HERE, "sphere_small.npz"), **out)


def atlas_case():
    rng = np.random.default_rng(3)
    tex = rng.uniform(size=(20, 30, 3)).astype(np.float32)
    P = 500
    uv = rng.uniform(-0.1, 1.1, size=(P, 2)).astype(np.float32)
    tgt = rng.uniform(size=(P, 3)).astype(np.float32)
    mask = ((rng.uniform(size=P) > 0.3) * rng.uniform(size=P)).astype(np.float32)
    g, loss = ref_api.photometric_gradient(tex, uv, tgt, mask, 1e-3, 0.01)
    pairs = rng.uniform(size=(300, 2, 2)).astype(np.float32)
    sg, sloss = ref_api.seam_gradient(tex, pairs, 1e-4, 1.0 / 900.0)
    t2, g2 = tex.copy(), g.copy()
    m2 = (rng.normal(size=tex.shape) * 0.01).astype(np.float32)
    v2 = (rng.uniform(size=tex.shape) * 0.001).astype(np.float32)
    m_in, v_in = m2.copy(), v2.copy()
    ref_api.adam_update(t2, g2, m2, v2, 0.01, 0.9, 0.999, 1e-8, 0.1, 0.001, 0.0, 1.0)
    np.savez_compressed(os.path.join(HERE, "atlas_kernels.npz"), tex=tex, uv=uv, tgt=tgt, mask=mask, g=g,
                        loss=np.float32(loss), pairs=pairs, sg=sg, sloss=np.float32(sloss), m_in=m_in, v_in=v_in,
                        t_out=t2, m_out=m2, v_out=v2)


def projection_case():
    rng = np.random.default_rng(11)
    pos, idx = S.icosphere(2)
    nrm = S.vertex_normals(pos, idx)
    uvv = S.spherical_uv(pos)
    mats, eyes = S.orbit_cameras(3)
    aw = ah = 40
    IW, IH = 28, 24
    aclip = np.concatenate([uvv * 2 - 1, np.zeros((len(uvv), 1)), np.ones((len(uvv), 1))], 1).astype(np.float32)
    araster, _ = ref_api.rasterize_forward(aclip, idx, (ah, aw), output_derivatives=False)
    apos = ref_api.interpolate_forward(pos, idx, araster)
    anrm = ref_api.interpolate_forward(nrm, idx, araster)
    shadows = []
    for k in range(3):
        clip = api.transform_positions(pos, mats[k])
        shadows.append(ref_api.rasterize_forward(clip, idx, (IH, IW), output_derivatives=False)[0])
    out = {"mats": mats, "eyes": eyes, "apos": apos, "anrm": anrm, "araster": araster, "shadows": np.stack(shadows)}
    for blend in (0, 1, 2):
        for vis in (0, 1, 2):
            for chans in ((3,) if (blend + vis) % 2 else (4,)):
                photos = np.stack([rng.uniform(size=(IH, IW, chans)).astype(np.float32) for _ in range(3)])
                masks = np.stack([rng.uniform(size=(IH, IW)).astype(np.float32) for _ in range(3)])
                rayvis = (rng.uniform(size=aw * ah) > 0.2).astype(np.float32)
                acc = np.zeros(aw * ah * 3, np.float32)
                accw = np.zeros(aw * ah, np.float32)
                best = np.zeros(aw * ah, np.float32)
                src = np.full(aw * ah, 0xFFFFFFFF, np.uint32)
                for k in range(3):
                    has_mask = k != 1
                    vw = 2.5 if blend == 2 else 0.7 + k * 0.2
                    packed = chans | (blend << 8) | (1 << 16) | ((1 << 24) if has_mask else 0) | (vis << 25)
                    ref_api.project_texture(mats[k].reshape(16), [*eyes[k], vw], [0, 0, IW, IH], [aw, ah, IW, IH],
                                            1e-3, 0.05, packed, k, apos, anrm, araster, shadows[k], photos[k],
                                            masks[k], rayvis, acc, accw, best, src)
                tag = f"b{blend}c{chans}v{vis}"
                out.update({f"photos_{tag}": photos, f"masks_{tag}": masks, f"rayvis_{tag}": rayvis,
                            f"acc_{tag}": acc, f"accw_{tag}": accw, f"best_{tag}": best, f"src_{tag}": src})
    np.savez_compressed(os.path.join(HERE, "projection_small.npz"), **out)


def padding_case():
    """pad_texture_atlas and fill_texture_on_surface of the reference's texture_padding.cpp."""
    from tests.padding_cases import chart_atlas, surface_case

    rng = np.random.default_rng(21)
    out = {}
    settings = [(4, True, 0, 0.5), (2, False, 0, 0.5), (0, True, 3, 0.5), (6, True, 0, 1.0), (1, True, 8, 0.25)]
    for k, (margin, fill, limit, thr) in enumerate(settings):
        h, w = [(40, 48), (33, 61), (64, 31), (45, 45), (17, 70)][k]
        color, valid, cov, filled = chart_atlas(rng, h, w, 4 if k % 2 == 0 else 3)
        c, f, st = ref_api.pad_texture_atlas(color, valid, margin, coverage_mask=cov if k != 3 else None,
                                             filled_mask=filled, fill_unobserved=fill, maximum_fill_distance=limit,
                                             valid_threshold=thr)
        out.update({f"p{k}_color": color, f"p{k}_valid": valid, f"p{k}_cov": cov, f"p{k}_filled": filled,
                    f"p{k}_args": np.array([margin, fill, limit], np.int64), f"p{k}_thr": np.float32(thr),
                    f"p{k}_out": c, f"p{k}_out_filled": f, f"p{k}_stats": np.array(st, np.uint64)})
    pos3, idx = S.icosphere(2)
    uv = S.spherical_uv(pos3)
    for k in range(2):
        color, valid, faces = surface_case(rng, pos3, idx, uv, (48, 56), 4 - k)
        c, f, st = ref_api.fill_texture_on_surface(color, valid, faces, idx)
        out.update({f"s{k}_color": color, f"s{k}_valid": valid, f"s{k}_faces": faces, f"s{k}_out": c,
                    f"s{k}_out_filled": f, f"s{k}_stats": np.array(st, np.uint64)})
    out["s_idx"] = idx.astype(np.uint32)
    np.savez_compressed(os.path.join(HERE, "padding_small.npz"), **out)


if __name__ == "__main__":
    if not ref_api.available():
        raise SystemExit("reference sources not available")
    triangle_case()
    sphere_case()
    atlas_case()
    projection_case()
    padding_case()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))

"""Uneven multi-mesh batches (pdr_render_batch_*) on the GPU: three meshes with different triangle
counts, view counts, resolutions and textures (one without a texture) render in one binning pass,
one raster launch and one adjoint launch. For every tile shape / bin depth the autotuner can pick,
the forward outputs are bit-identical to rendering each mesh on its own (torch.render, 16x16 tiles),
and the gradients equal the per-mesh gradients up to the summation order of the atomics."""
import numpy as np
import pytest
import torch

import photara_drender_gb300 as pdr
from photara_drender_gb300 import synthetic as S
from photara_drender_gb300.batch import CONFIGS, BatchMesh, MeshBatch

pytestmark = pytest.mark.gpu


def make_meshes(dev, rng):
    specs = [(2, 2, (64, 48), (32, 32)), (3, 3, (96, 96), (64, 48)), (4, 1, (80, 120), None)]
    meshes = []
    for sub, views, (h, w), tex in specs:
        pos3, idx = S.icosphere(sub)
        mats, _ = S.orbit_cameras(views, aspect=w / h)
        V = pos3.shape[0]
        m = BatchMesh(clip=torch.tensor(S.clip_positions(pos3, mats), device=dev),
                      indices=torch.tensor(idx.astype(np.int32), device=dev), height=h, width=w,
                      attributes=torch.tensor(rng.uniform(size=(V, 3)).astype(np.float32), device=dev),
                      uv_attributes=torch.tensor(S.spherical_uv(pos3), device=dev) if tex else None,
                      texture=torch.tensor(rng.uniform(size=tex + (4,)).astype(np.float32), device=dev) if tex else None)
        meshes.append(m)
    return meshes


def test_batch_matches_per_mesh_renders():
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(4)
    r = pdr.Rasterizer(0)
    meshes = make_meshes(dev, rng)
    refs = []
    for m in meshes:
        leaves = {k: t.clone().requires_grad_(True) for k, t in (("clip", m.clip), ("attrs", m.attributes),
                                                                 ("uv", m.uv_attributes), ("tex", m.texture))
                  if t is not None}
        out = pdr.render(leaves["clip"], m.indices, (m.height, m.width), rasterizer=r, vertex_attributes=leaves["attrs"],
                         vertex_uv=leaves.get("uv"), texture=leaves.get("tex"), address_mode="wrap")
        gi = torch.tensor(rng.normal(size=out.interpolated.shape).astype(np.float32), device=dev)
        outs, grads = [out.interpolated], [gi]
        m.grads["interp"] = gi
        if out.sampled is not None:
            gs = torch.tensor(rng.normal(size=out.sampled.shape).astype(np.float32), device=dev)
            outs.append(out.sampled)
            grads.append(gs)
            m.grads["sampled"] = gs
        torch.autograd.backward(outs, grads)
        refs.append((out, {k: v.grad for k, v in leaves.items()}))
    batch = MeshBatch(r, meshes, address_mode="wrap")
    for cfg in CONFIGS:
        batch.set_config(cfg)
        batch.forward()
        batch.backward()
        torch.cuda.synchronize(dev)
        for m, (out, g) in zip(meshes, refs):
            for name, ref in (("raster", out.raster), ("deriv", out.derivatives), ("interp", out.interpolated),
                              ("uv", out.uv), ("sampled", out.sampled)):
                if ref is None:
                    continue
                got = m.outputs[name]
                assert torch.equal(got.view(torch.int32), ref.view(torch.int32)), (cfg, name)
            for name, ref in (("clip", g["clip"]), ("attributes", g["attrs"]), ("uv_attributes", g.get("uv")),
                              ("texture", g.get("tex"))):
                if ref is None:
                    continue
                d = float((m.grads[name] - ref).abs().max())
                assert d <= 1e-4 * float(ref.abs().max()) + 1e-7, (cfg, name, d)


def test_batch_autotune_keeps_results():
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    r = pdr.Rasterizer(0)
    meshes = make_meshes(dev, rng)
    for m in meshes:
        m.grads["interp"] = torch.randn(m.clip.shape[0], m.height, m.width, 3, device=dev)
        if m.texture is not None:
            m.grads["sampled"] = torch.randn(m.clip.shape[0], m.height, m.width, 4, device=dev)
    batch = MeshBatch(r, meshes)
    batch.forward()
    first = [m.outputs["raster"].clone() for m in meshes]
    times = batch.autotune(reps=2)
    assert set(times) == set(CONFIGS) and all(t > 0 for t in times.values())
    assert (batch.config.tile_width, batch.config.tile_height, batch.config.stage_triangles) == min(times, key=times.get)
    batch.forward()
    for m, f in zip(meshes, first):
        assert torch.equal(m.outputs["raster"].view(torch.int32), f.view(torch.int32))
    with pytest.raises(ValueError):
        batch.set_config((8, 8, 64))

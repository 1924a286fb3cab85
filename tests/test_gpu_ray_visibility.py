"""Ray-query visibility on the GPU (csrc/bvh.cu through the C ABI) against the oracle.

The oracle restates project_ray_visibility.hlsl (ray set-up in fp32 as the shader writes it) and tests
every triangle in double precision, marking texels whose ray passes within 1e-5 of a triangle edge or
of its t range as undecided. Hardware ray tracers are watertight and the GPU caster's fp32
Moller-Trumbore test is not, so only those undecided texels may differ: every decided texel must
match, and the undecided ones must be rare. The bakes in the two ray modes are then checked against
the oracle bake fed with the same visibility bits, bit for bit where the shadow-map bake is."""
import numpy as np
import pytest
import torch

from oracle import api
from photara_drender_gb300 import TextureBaker, _native
from photara_drender_gb300 import synthetic as S
from photara_drender_gb300.rasterizer import _ptr
from tests.gpu_util import same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def baker():
    return TextureBaker(0)


def scene(triangles=6000, seed=2):
    pos3, nrm, uv, idx, _, _ = S.displaced_sphere(triangles, seed=seed, amplitude=0.15, atlas_size=128)
    return pos3, nrm, uv, idx


def gbuffer(baker, pos3, nrm, uv, idx, res):
    """The atlas G-buffer and the visibility bits exactly as TextureBaker builds them."""
    dev = baker.context.device
    t_pos, t_nrm, t_uv = (torch.tensor(x, device=dev) for x in (pos3, nrm, uv))
    t_idx = torch.tensor(idx.astype(np.int32), device=dev)
    aclip = torch.empty((1, uv.shape[0], 4), dtype=torch.float32, device=dev)
    _native.call("pdr_atlas_clip_positions", _ptr(t_uv), uv.shape[0], _ptr(aclip), baker.context.stream())
    araster = baker._rasters(aclip, t_idx, [res], [None])[0]
    apos = baker.rasterizer.interpolate_forward(t_pos, t_idx, araster)
    anrm = baker.rasterizer.interpolate_forward(t_nrm, t_idx, araster)
    return t_pos, t_idx, apos, anrm, araster


def gpu_bits(baker, t_pos, t_idx, apos, anrm, araster, cams, bias=1e-4):
    bits = baker._ray_visibility(t_pos, t_idx, apos, anrm, araster, np.asarray(cams, np.float32), bias)
    return bits.cpu().numpy().view(np.uint32)


def test_ray_visibility_matches_oracle(baker):
    pos3, nrm, uv, idx = scene()
    _, eyes = S.orbit_cameras(3)
    cams = np.concatenate([eyes, np.array([[0.0, 0.0, 1.6], [0.05, 2.5, 0.3]], np.float32)])
    t_pos, t_idx, apos, anrm, araster = gbuffer(baker, pos3, nrm, uv, idx, (128, 128))
    bits = gpu_bits(baker, t_pos, t_idx, apos, anrm, araster, cams)
    ap, an, ar = apos.cpu().numpy(), anrm.cpu().numpy(), araster.cpu().numpy()
    covered = ar[..., 3].reshape(-1) != 0
    undecided = 0
    for k, cam in enumerate(cams):
        state = api.ray_visibility(pos3, idx, ap, an, ar, cam)
        got = (bits[:, k // 32] >> (k % 32)) & 1
        decided = state >= 0
        assert np.array_equal(got[decided], state[decided].astype(np.uint32)), f"view {k}"
        undecided += int((~decided).sum())
        # both outcomes occur among covered texels: the test exercises occlusion and visibility
        assert (state[covered] == 1).any() and (state[covered] == 0).any()
    assert undecided <= 0.01 * covered.sum() * len(cams)


@pytest.mark.parametrize("mode", ["hybrid_ray_query", "ray_query"])
@pytest.mark.parametrize("blend", ["best_view", "weighted_average"])
def test_bake_ray_modes_match_oracle(baker, mode, blend):
    pos3, nrm, uv, idx = scene(3000, seed=4)
    mats, eyes = S.orbit_cameras(3)
    rng = np.random.default_rng(6)
    images = [rng.uniform(size=(48, 64, 3)).astype(np.float32) for _ in range(3)]
    out = baker.bake_output(pos3, nrm, uv, idx, images, mats, eyes, resolution=(64, 64), blend_mode=blend,
                            visibility_mode=mode)
    assert out.used_ray_query
    t_pos, t_idx, apos, anrm, araster = gbuffer(baker, pos3, nrm, uv, idx, (64, 64))
    bits = gpu_bits(baker, t_pos, t_idx, apos, anrm, araster, eyes)
    vm = {"hybrid_ray_query": 1, "ray_query": 2}[mode]
    color, conf, src, valid, cov, faces = api.bake(pos3, nrm, uv, idx, images, mats, eyes, resolution=(64, 64),
                                                   blend_mode=blend, visibility_mode=vm, ray_bits=bits)
    assert np.array_equal(out.coverage_mask, cov) and np.array_equal(out.face_ids, faces)
    assert same_bits(out.color, color) and same_bits(out.confidence, conf)
    assert np.array_equal(out.source_view, src) and same_bits(out.valid_mask, valid)
    assert valid.any()

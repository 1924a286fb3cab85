"""The C++ API (include/photara_drender/*.hpp, libphotara_drender.so) on the GPU.

tests/native/cpp_api_test.cpp is compiled against the library and run as its own process: it makes
the property checks of the reference's tests/native_tests.cpp through Context, Rasterizer,
TextureBaker and TextureRefiner, then runs a sphere mesh written here through forward, backward,
interpolate and texture. Its outputs are compared with the oracle: bit-exact for the forward
results, within the gradient tolerance of tests/gpu_util.grad_check for the gradient sums."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import api
from photara_drender_gb300 import synthetic as S
from tests.gpu_util import grad_check, same_bits

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def cpp_test_binary(tmp_path_factory):
    from photara_drender_gb300 import build

    lib = build.build_cpp()
    exe = str(tmp_path_factory.mktemp("cpp") / "cpp_api_test")
    cxx = shutil.which("g++") or "g++"
    subprocess.run([cxx, "-std=c++20", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "native", "cpp_api_test.cpp"), "-o", exe, "-L", os.path.dirname(lib),
                    "-lphotara_drender", f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    return exe


def test_cpp_api_against_oracle(cpp_test_binary, tmp_path):
    rng = np.random.default_rng(11)
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(1)
    clip = S.clip_positions(pos3, mats)[0]
    H, W, A, TW, TH, TC = 72, 88, 3, 40, 24, 4
    attr = rng.uniform(size=(pos3.shape[0], A)).astype(np.float32)
    tex = rng.uniform(size=(TH, TW, TC)).astype(np.float32)
    o_r, o_d = api.rasterize_forward(clip, idx, (H, W))
    uv = (api.interpolate_forward(S.spherical_uv(pos3), idx, o_r) * 1.7 - 0.3).astype(np.float32)
    gr = rng.normal(size=(H, W, 4)).astype(np.float32)
    gt = rng.normal(size=(H, W, TC)).astype(np.float32)
    inp, out = tmp_path / "in", tmp_path / "out"
    inp.mkdir()
    out.mkdir()
    np.array([pos3.shape[0], idx.shape[0], W, H, A, TW, TH, TC], np.uint32).tofile(inp / "dims.u32")
    for name, a in (("clip.f32", clip), ("idx.u32", idx.astype(np.uint32)), ("grad_raster.f32", gr),
                    ("attr.f32", attr), ("uv.f32", uv), ("tex.f32", tex), ("grad_tex.f32", gt)):
        np.ascontiguousarray(a).tofile(inp / name)
    res = subprocess.run([cpp_test_binary, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "checks passed" in res.stdout

    def load(name, shape):
        return np.fromfile(out / name, np.float32).reshape(shape)

    assert same_bits(load("raster.f32", (H, W, 4)), o_r)
    assert same_bits(load("derivatives.f32", (H, W, 4)), o_d)
    assert same_bits(load("interp.f32", (H, W, A)), api.interpolate_forward(attr, idx, o_r))
    assert same_bits(load("sampled.f32", (H, W, TC)), api.texture_forward(tex, uv, o_r, "wrap"))
    grad_check(load("grad_clip.f32", clip.shape), api.rasterize_backward(clip, idx, o_r, gr),
               api.rasterize_backward(clip, idx, o_r, gr, f64=True),
               api.rasterize_backward(clip, idx, o_r, gr, f64=True, abs_terms=True), name="grad_positions")
    o_gt, o_gu = api.texture_backward(tex, uv, o_r, gt, "wrap")
    grad_check(load("grad_texture.f32", tex.shape), o_gt, api.texture_backward(tex, uv, o_r, gt, "wrap", f64=True)[0],
               api.texture_backward(tex, uv, o_r, gt, "wrap", f64=True, abs_terms=True)[0], name="grad_texture")
    assert same_bits(load("grad_uv.f32", (H, W, 2)), o_gu)

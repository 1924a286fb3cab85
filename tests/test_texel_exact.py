"""The integer emulation of the reference's double-precision texel position (csrc/pdr_common.cuh
exact_texel_coordinate, used by every texture adjoint on the GPU) against the double formula of
src/rasterizer.cpp:207-215: tests/native/texel_exact_check.cpp is compiled for the host and checks
base texel and fraction bit for bit on about 2.7 M seeded and edge-case inputs (random, tiny,
texel-centre, random-bit and one-ulp-off-centre coordinates, +-0, denormals, infinities, NaN) over
texture sizes 1 to 2^28 + 3."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_exact_texel_coordinate_matches_double_formula(tmp_path):
    exe = str(tmp_path / "texel_exact_check")
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(shutil.which("nvcc") or
                                                                             "/usr/local/cuda/bin/nvcc"))), "include")
    subprocess.run([shutil.which("g++") or "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I",
                    os.path.join(ROOT, "photara_drender_gb300", "csrc"), "-I", cuda_inc,
                    os.path.join(HERE, "native", "texel_exact_check.cpp"), "-o", exe], check=True)
    res = subprocess.run([exe], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "fails=0" in res.stdout

"""Build recipes for the two CPU checkers (test infrastructure only).

* ``build_oracle()`` compiles ``oracle/pdr_oracle.c`` (the C restatement of the reference's
  shaders and host routines) into ``oracle/_build/libpdr_oracle.so``.
* ``build_ref()`` compiles the reference's own sources, read where they lie under
  ``/root/reference``, into ``oracle/_ref/libpdr_ref.so``: the HLSL compute shaders (after
  stripping the ``[numthreads]`` attribute line and ``: SV_*`` semantics, which C++ has no
  syntax for) through ``oracle/ref_shim.hpp``, and ``src/texture_padding.cpp`` as-is.
  Nothing from the reference is copied into the repository; the stripped shader text is
  written only under ``oracle/_ref/gen`` (git-ignored).

Both use ``-ffp-contract=off`` so that every fp32 operation rounds on its own, on x86 and Arm.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = "/root/reference"
ORACLE_SO = os.path.join(HERE, "_build", "libpdr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpdr_ref.so")
SHADERS = [
    "rasterize_forward", "rasterize_backward", "reduce_vertex_gradients", "interpolate_forward",
    "interpolate_grad_attributes", "interpolate_grad_raster", "texture_forward", "texture_grad_texture",
    "texture_grad_uv", "project_texture", "atlas_photometric_gradient", "atlas_seam_gradient",
    "atlas_adam_update",
]
FP_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "pdr_oracle.c")
    hdr = os.path.join(HERE, "pdr_oracle.h")
    if not force and _newer(ORACLE_SO, [src, hdr, __file__]):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    tmp = ORACLE_SO + f".tmp{os.getpid()}"
    subprocess.run(["gcc", "-std=c11", *FP_FLAGS, "-fopenmp", src, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def _strip_hlsl(text: str) -> str:
    text = re.sub(r"^\[numthreads\([^)]*\)\]\s*$", "[[maybe_unused]]", text, flags=re.M)
    return re.sub(r"\s*:\s*SV_[A-Za-z]+", "", text)


def build_ref(force: bool = False) -> str | None:
    """Returns the library path, or None when the reference sources are absent."""
    shader_dir = os.path.join(REFERENCE, "shaders")
    if not os.path.isdir(shader_dir):
        return REF_SO if os.path.exists(REF_SO) else None
    sources = [os.path.join(shader_dir, s + ".hlsl") for s in SHADERS]
    own = [os.path.join(HERE, f) for f in ("ref_shim.hpp", "ref_shaders.cpp", "ref_padding.cpp")]
    padding = os.path.join(REFERENCE, "src", "texture_padding.cpp")
    if not force and _newer(REF_SO, sources + own + [padding, __file__]):
        return REF_SO
    gen = os.path.join(HERE, "_ref", "gen")
    os.makedirs(gen, exist_ok=True)
    for name, path in zip(SHADERS, sources):
        with open(path, encoding="utf-8") as f:
            text = _strip_hlsl(f.read())
        with open(os.path.join(gen, name + ".hlsl.inc"), "w", encoding="utf-8") as f:
            f.write(text)
    tmp = REF_SO + f".tmp{os.getpid()}"
    subprocess.run(
        ["g++", "-std=c++20", *FP_FLAGS, "-Wno-attributes", "-I", HERE, "-I", gen,
         "-I", os.path.join(REFERENCE, "include"),
         os.path.join(HERE, "ref_shaders.cpp"), os.path.join(HERE, "ref_padding.cpp"), padding,
         "-o", tmp, "-lpthread"],
        check=True,
    )
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))

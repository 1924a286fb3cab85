"""Build recipes for the two CPU checkers (test infrastructure only).

* ``build_oracle()`` compiles ``oracle/pdr_oracle.c`` (the C restatement of the reference's
  shaders and host routines) into ``oracle/_build/libpdr_oracle.so``.
* ``build_ref()`` compiles the reference's own sources, read where they lie (``REFERENCE``
  below), into ``oracle/_ref/libpdr_ref.so``: the HLSL compute shaders (after
  stripping the ``[numthreads]`` attribute line and ``: SV_*`` semantics, which C++ has no
  syntax for) through ``oracle/ref_shim.hpp``, ``src/texture_padding.cpp`` as-is, and the
  self-contained host routines of ``src/rasterizer.cpp`` (tile binning and the two CSR builders,
  cut out by name through ``oracle/ref_host.cpp``; the rest of that file needs the absent Vulkan
  wrapper). The reference directory is ``$PDR_REFERENCE_DIR`` (default: the mount point of the
  read-only reference checkout).
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
# where the reference's sources lie; override with PDR_REFERENCE_DIR
REFERENCE = os.environ.get("PDR_REFERENCE_DIR", "/root/reference")
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


# Definitions of src/rasterizer.cpp compiled for the checker, in source order: the binning and table
# builders of the raster path plus the constants, structs and helpers they use.
HOST_DEFINITIONS = [
    r"constexpr std::uint32_t RASTER_TILE_SIZE\b", r"std::uint32_t divide_round_up\(", r"struct TileBins\b",
    r"TileBins build_tile_bins\(", r"struct VertexAdjacency\b", r"VertexAdjacency build_vertex_adjacency\(",
    r"std::int32_t address_coordinate\(", r"struct TextureSampleAdjacency\b",
    r"TextureSampleAdjacency build_texture_sample_adjacency\(",
]


def _definition(text: str, pattern: str) -> str:
    """The definition starting at `pattern`: up to its first ';' when that comes before any '{',
    else through the matching closing brace (and a trailing ';' for a struct)."""
    m = re.search(r"^" + pattern, text, flags=re.M)
    if m is None:
        raise RuntimeError(f"definition {pattern!r} not found in the reference source")
    i = m.start()
    semi, brace = text.find(";", i), text.find("{", i)
    if brace < 0 or (0 <= semi < brace):
        return text[i:semi + 1]
    depth, j = 0, brace
    while True:
        c = text[j]
        depth += c == "{"
        depth -= c == "}"
        j += 1
        if depth == 0:
            break
    if text[j:j + 1] == ";":
        j += 1
    return text[i:j]


def build_ref(force: bool = False) -> str | None:
    """Returns the library path, or None when the reference sources are absent."""
    shader_dir = os.path.join(REFERENCE, "shaders")
    if not os.path.isdir(shader_dir):
        return REF_SO if os.path.exists(REF_SO) else None
    sources = [os.path.join(shader_dir, s + ".hlsl") for s in SHADERS]
    own = [os.path.join(HERE, f) for f in ("ref_shim.hpp", "ref_shaders.cpp", "ref_padding.cpp", "ref_host.cpp")]
    padding = os.path.join(REFERENCE, "src", "texture_padding.cpp")
    rasterizer = os.path.join(REFERENCE, "src", "rasterizer.cpp")
    if not force and _newer(REF_SO, sources + own + [padding, rasterizer, __file__]):
        return REF_SO
    gen = os.path.join(HERE, "_ref", "gen")
    os.makedirs(gen, exist_ok=True)
    for name, path in zip(SHADERS, sources):
        with open(path, encoding="utf-8") as f:
            text = _strip_hlsl(f.read())
        with open(os.path.join(gen, name + ".hlsl.inc"), "w", encoding="utf-8") as f:
            f.write(text)
    with open(rasterizer, encoding="utf-8") as f:
        host = f.read()
    with open(os.path.join(gen, "rasterizer_host.inc"), "w", encoding="utf-8") as f:
        f.write("\n\n".join(_definition(host, p) for p in HOST_DEFINITIONS) + "\n")
    tmp = REF_SO + f".tmp{os.getpid()}"
    subprocess.run(
        ["g++", "-std=c++20", *FP_FLAGS, "-Wno-attributes", "-I", HERE, "-I", gen,
         "-I", os.path.join(REFERENCE, "include"),
         os.path.join(HERE, "ref_shaders.cpp"), os.path.join(HERE, "ref_padding.cpp"),
         os.path.join(HERE, "ref_host.cpp"), padding,
         "-o", tmp, "-lpthread"],
        check=True,
    )
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))

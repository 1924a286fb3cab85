"""Builds libphotara_drender_gb300.so in-tree with nvcc for sm_103a (no CMake, parallel TUs)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libphotara_drender_gb300.so")
CPP_LIB = os.path.join(HERE, "libphotara_drender.so")  # the C++ API of include/photara_drender/*.hpp
CPP_SOURCES = [os.path.join(HERE, "cpp", "photara_drender.cpp")]
SOURCES = ["raster.cu", "shading.cu", "bake.cu", "refine.cu", "drivers.cu", "fused.cu", "no_alloc.cu", "precond.cu", "batch.cu", "bvh.cu", "padding.cu", "mip.cu", "near.cu", "calibrate.cu", "capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "--expt-relaxed-constexpr",
         "-I", CSRC, "-I", INCLUDE]
# Multiply-add contraction stays off wherever a result is compared bit for bit with the reference's
# arithmetic (every fp32 operation rounding on its own), including the discrete decisions adjoints make
# from fp32 values (visit rules, texel addresses). Translation units whose every result is held to a
# tolerance contract a*b+c into one FMA: the ray caster (visibility decided against a 1e-5 band) and
# the calibration kernel.
FMA_SOURCES = {"bvh.cu", "calibrate.cu"}


def fmad_flag(src: str) -> str:
    return "-fmad=true" if src in FMA_SOURCES else "-fmad=false"


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build photara_drender_gb300")
    return path


def cuda_lib_dir() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64")


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "pdr_capi.h"))
    return files


def build(force: bool = False, verbose: bool = False) -> str:
    deps = _deps()
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, fmad_flag(src), "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(SOURCES))) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run([cc, *ARCH, "-shared", "--cudart", "shared", "-Xlinker", f"-rpath,{cuda_lib_dir()}", "-o", tmp,
                    *objs], check=True)
    os.replace(tmp, LIB)
    return LIB


def build_cpp(force: bool = False) -> str:
    """Builds the C++ API library (photara_drender::Context, Rasterizer, TextureBaker, TextureRefiner)
    over the C ABI library; it needs C++20 for std::span, as the reference's headers do."""
    lib = build(force=force)
    deps = CPP_SOURCES + [lib] + [os.path.join(INCLUDE, "photara_drender", f)
                                  for f in os.listdir(os.path.join(INCLUDE, "photara_drender"))]
    if not force and os.path.exists(CPP_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(CPP_LIB) for d in deps):
        return CPP_LIB
    tmp = CPP_LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), "-std=c++20", "-O2", "-Xcompiler", "-fPIC,-Wall", "-shared", "--cudart", "shared", "-I", INCLUDE,
           *CPP_SOURCES,
           "-o", tmp, "-L", HERE, "-lphotara_drender_gb300", "-Xlinker", f"-rpath,$ORIGIN:{cuda_lib_dir()}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"building the C++ API failed:\n{res.stderr}")
    os.replace(tmp, CPP_LIB)
    return CPP_LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_cpp())

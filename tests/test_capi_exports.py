"""The C-ABI library builds, loads without a GPU, and exports every entry point include/*.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            with open(os.path.join(inc, f)) as fh:
                text = fh.read()
            names += re.findall(r"PDR_API\s+[\w\s\*]+?\b(pdr_\w+)\s*\(", text)
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert len(names) >= 25
    for required in ("pdr_bin_tiles", "pdr_rasterize_forward", "pdr_rasterize_backward", "pdr_interpolate_forward",
                     "pdr_interpolate_backward", "pdr_texture_forward", "pdr_texture_backward", "pdr_project_views",
                     "pdr_refine_run", "pdr_refine_graph_create"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from photara_drender_gb300 import build

    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    lib.pdr_version.restype = ctypes.c_int32
    assert lib.pdr_version() >= 100


def test_status_codes_without_gpu():
    """Argument checks run before any CUDA call, so they answer on a machine without a GPU."""
    from photara_drender_gb300 import _native

    L = _native.lib()
    with pytest.raises(ValueError):
        _native.check(L.pdr_rasterize_forward(None, 1, 3, None, 1, 8, 8, None, 0, None, None, 0, None, None, None))
    with pytest.raises(ValueError):
        _native.check(L.pdr_texture_forward(None, 0, 4, 4, 3, 0, None, None, 1, 16, None, None))


def test_cpp_api_library_builds_and_links():
    """The C++ API library builds over the C ABI and the native C++ test links against it (the
    test itself needs a GPU and runs in tests/test_gpu_cpp_api.py)."""
    import shutil
    import subprocess

    from photara_drender_gb300 import build

    lib = build.build_cpp()
    exe = os.path.join(os.path.dirname(lib), "_build", "cpp_api_test_link_check")
    subprocess.run([shutil.which("g++") or "g++", "-std=c++20", "-O0", "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "native", "cpp_api_test.cpp"), "-o",
                    exe, "-L", os.path.dirname(lib), "-lphotara_drender", f"-Wl,-rpath,{os.path.dirname(lib)}"],
                   check=True)
    assert os.path.exists(exe)


def test_binning_argument_checks_without_gpu():
    """Both binning entry points refuse, before any launch, clip positions or viewports that are not
    16-byte aligned (the count kernel reads them as float4) and a tile-list capacity beyond the u32
    offsets. The pointers are never dereferenced: the checks answer on a machine without a GPU."""
    import ctypes as C

    from photara_drender_gb300 import _native

    L = _native.lib()
    fn = L.pdr_bin_tiles_no_alloc
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
    base = 1 << 20  # a 16-byte aligned stand-in address
    clip, idx, vps, off, lst, status = (C.c_void_p(base + k * 4096) for k in range(6))
    odd = C.c_void_p(base + 4)
    with pytest.raises(ValueError, match="16-byte aligned"):
        _native.check(fn(odd, 1, 3, idx, 1, 32, 32, vps, off, lst, 64, status, None))
    with pytest.raises(ValueError, match="16-byte aligned"):
        _native.check(fn(clip, 1, 3, idx, 1, 32, 32, odd, off, lst, 64, status, None))
    with pytest.raises(OverflowError, match="capacity"):
        _native.check(fn(clip, 1, 3, idx, 1, 32, 32, vps, off, lst, 1 << 62, status, None))
    ws = C.c_void_p(base + 8 * 4096)
    with pytest.raises(ValueError, match="16-byte aligned"):
        _native.check(L.pdr_bin_tiles(odd, 1, 3, idx, 1, 32, 32, vps, off, lst, 64, ws, 1 << 30, status, None))
    with pytest.raises(OverflowError, match="capacity"):
        _native.check(L.pdr_bin_tiles(clip, 1, 3, idx, 1, 32, 32, vps, off, lst, 1 << 62, ws, 1 << 30, status, None))


def test_render_workspace_queries_without_gpu():
    """The fused render's workspace queries answer on the host: the backward's per-view vertex records take
    4 * ceil((attributes + 5) / 4) floats per vertex and view (0 above 8 attributes), the tiled forward query
    takes only the tile shapes the raster is compiled for, and a shape that does not divide the reference's
    16x16 tile is refused by the render entry points before any launch."""
    import ctypes as C

    from photara_drender_gb300 import _native
    from photara_drender_gb300.pipeline import TILE_CONFIGS, RenderArgsC

    L = _native.lib()
    for a in range(9):
        want = 3 * 1000 * 4 * ((a + 5 + 3) // 4) * 4
        assert L.pdr_render_backward_workspace_bytes(3, 1000, a) == want, a
    assert L.pdr_render_backward_workspace_bytes(3, 1000, 9) == 0
    assert L.pdr_render_workspace_bytes_tiled(2, 100, 64, 64, 1024, 0, 8) == 0
    for tw, th, _ in TILE_CONFIGS:
        assert L.pdr_render_workspace_bytes_tiled(2, 100, 64, 64, 1024, tw, th) > 0
    base = 1 << 20
    a = RenderArgsC()
    a.clip_positions, a.indices, a.viewports, a.raster = base, base + 4096, base + 8192, base + 12288
    a.tile_offsets, a.tile_triangles, a.workspace, a.status = base + 16384, base + 20480, base + 24576, base + 28672
    a.views, a.vertex_count, a.triangle_count, a.width, a.height = 1, 3, 1, 64, 64
    a.capacity, a.workspace_bytes = 1024, 1 << 30
    a.tile_width, a.tile_height, a.stage_triangles = 32, 8, 256
    with pytest.raises(ValueError, match="tile shape"):
        _native.check(L.pdr_render_bin(C.addressof(a), None))

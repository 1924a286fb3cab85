"""pdr_bin_tiles_no_alloc: the allocation-free tile binning entry point, for callers that cannot call
cudaMalloc (code running inside someone else's CUDA-graph capture, real-time loops that must not take
cudaMalloc's synchronising path, plugin hosts that pass buffers but no allocator). Its scratch is a
fixed array inside the library; this test drives it through the C ABI and checks that two calls in a
row give exactly what pdr_bin_tiles with a caller workspace gives, and that the bins rasterize to the
same image. The file sorts last so a run that stops at the first failure has run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_no_alloc_binning_matches_workspace_binning():
    import torch

    from photara_drender_gb300 import _native
    from photara_drender_gb300 import synthetic as S

    L = _native.lib()
    fn = L.pdr_bin_tiles_no_alloc
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
    dev = torch.device("cuda", 0)
    pos3, idx = S.icosphere(4)
    mats, _ = S.orbit_cameras(3)
    clip = torch.tensor(S.clip_positions(pos3, mats), device=dev)
    tidx = torch.tensor(idx.astype(np.int32), device=dev)
    views, V, T, H, W = 3, pos3.shape[0], idx.shape[0], 120, 136
    vps = torch.tensor([[0.0, 0.0, W, H], [4.0, -2.0, 120.0, 110.0], [0.0, 0.0, W, H]], dtype=torch.float32,
                       device=dev)
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    capacity = 8 * T
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def outputs():
        return (torch.full((views * tiles + 1,), -1, dtype=torch.int32, device=dev),
                torch.full((capacity,), -1, dtype=torch.int32, device=dev),
                torch.zeros(_native.STATUS_WORDS, dtype=torch.int32, device=dev))

    ref_off, ref_list, ref_status = outputs()
    ws_bytes = L.pdr_bin_tiles_workspace_bytes(views, T, W, H, capacity)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    _native.check(L.pdr_bin_tiles(p(clip), views, V, p(tidx), T, W, H, p(vps), p(ref_off), p(ref_list), capacity,
                                  p(ws), ws_bytes, p(ref_status), stream))
    torch.cuda.synchronize()
    total = int(ref_status[0])
    assert total > 0 and int(ref_status[2]) == 0
    results = []
    for _ in range(2):
        off, lst, status = outputs()
        _native.check(fn(p(clip), views, V, p(tidx), T, W, H, p(vps), p(off), p(lst), capacity, p(status), stream))
        torch.cuda.synchronize()
        results.append((off, lst, status))
    for off, lst, status in results:
        assert torch.equal(off, ref_off)
        assert torch.equal(lst[:total], ref_list[:total])
        assert int(status[0]) == total and int(status[2]) == 0

    # the bins drive the rasterizer to the same image
    r1 = torch.empty((views, H, W, 4), dtype=torch.float32, device=dev)
    r2 = torch.empty_like(r1)
    off, lst, _ = results[1]
    _native.check(L.pdr_rasterize_forward(p(clip), views, V, p(tidx), T, W, H, p(vps), 0, p(ref_off), p(ref_list),
                                          capacity, p(r1), None, stream))
    _native.check(L.pdr_rasterize_forward(p(clip), views, V, p(tidx), T, W, H, p(vps), 0, p(off), p(lst), capacity,
                                          p(r2), None, stream))
    torch.cuda.synchronize()
    assert torch.equal(r1.view(torch.int32), r2.view(torch.int32))

    # a binning that needs more scratch than the fixed array is rejected with a clear error
    huge = 64 << 20
    big_list = torch.empty(1, dtype=torch.int32, device=dev)
    with pytest.raises(ValueError, match="scratch"):
        _native.check(fn(p(clip), views, V, p(tidx), T, W, H, p(vps), p(ref_off), p(big_list), huge, p(ref_status),
                         stream))


def test_no_alloc_binning_inside_a_graph_capture():
    """The use case the entry point exists for: after a first call outside any capture (which looks the
    scratch array's device address up), a call recorded into someone else's CUDA graph (memset and
    kernels only) replays to the bins a workspace call gives, twice in a row."""
    import torch

    from photara_drender_gb300 import _native
    from photara_drender_gb300 import synthetic as S

    L = _native.lib()
    fn = L.pdr_bin_tiles_no_alloc
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
    dev = torch.device("cuda", 0)
    pos3, idx = S.icosphere(3)
    mats, _ = S.orbit_cameras(2)
    clip = torch.tensor(S.clip_positions(pos3, mats), device=dev)
    tidx = torch.tensor(idx.astype(np.int32), device=dev)
    views, V, T, H, W = 2, pos3.shape[0], idx.shape[0], 96, 80
    vps = torch.tensor([[0.0, 0.0, W, H]] * views, dtype=torch.float32, device=dev)
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    capacity = 8 * T
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def outputs():
        return (torch.full((views * tiles + 1,), -1, dtype=torch.int32, device=dev),
                torch.full((capacity,), -1, dtype=torch.int32, device=dev),
                torch.zeros(_native.STATUS_WORDS, dtype=torch.int32, device=dev))

    ref_off, ref_list, ref_status = outputs()
    ws_bytes = L.pdr_bin_tiles_workspace_bytes(views, T, W, H, capacity)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _native.check(L.pdr_bin_tiles(p(clip), views, V, p(tidx), T, W, H, p(vps), p(ref_off), p(ref_list), capacity,
                                  p(ws), ws_bytes, p(ref_status), stream))
    off, lst, status = outputs()
    _native.check(fn(p(clip), views, V, p(tidx), T, W, H, p(vps), p(off), p(lst), capacity, p(status), stream))
    torch.cuda.synchronize()
    total = int(ref_status[0])
    assert total > 0

    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    graph = torch.cuda.CUDAGraph()
    off.fill_(-1)
    lst.fill_(-1)
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        cap = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        _native.check(fn(p(clip), views, V, p(tidx), T, W, H, p(vps), p(off), p(lst), capacity, p(status), cap))
    for _ in range(2):
        off.fill_(-1)
        lst.fill_(-1)
        status.zero_()
        graph.replay()
        torch.cuda.synchronize()
        assert torch.equal(off, ref_off)
        assert torch.equal(lst[:total], ref_list[:total])
        assert int(status[0]) == total and int(status[2]) == 0

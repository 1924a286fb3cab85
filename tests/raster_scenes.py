"""Raster scenes shared by the oracle and GPU tests."""
import numpy as np


def tie_scene(n=6, res=64):
    """Coplanar grid quads with vertices on pixel centres: samples on shared edges and diagonals pass the
    edge tests of both triangles at equal depth, so edges and the lowest-id rule decide them."""
    c = (np.arange(res, dtype=np.float64) + 0.5) * 2.0 / res - 1.0  # pixel-centre NDC
    ticks = c[np.linspace(3, res - 4, n + 1).round().astype(int)]
    X, Y = np.meshgrid(ticks, ticks)
    pos = np.stack([X, Y, np.full_like(X, 0.25), np.ones_like(X)], -1).reshape(-1, 4).astype(np.float32)
    idx = []
    for i in range(n):
        for j in range(n):
            a = i * (n + 1) + j
            idx += [[a, a + 1, a + n + 2], [a, a + n + 2, a + n + 1]]
    # a second, overlapping copy of the grid at the same depth (duplicate triangles, higher ids)
    idx = np.array(idx, np.uint32)
    return pos, np.concatenate([idx, idx[::-1]]), (res, res)

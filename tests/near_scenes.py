"""Scenes for the near-plane clipping tests: geometry that crosses the near plane and the eye plane."""
import numpy as np

from photara_drender_gb300 import synthetic as S


def ground(n=8, size=4.0, seed=0, res=(64, 80)):
    """A slightly uneven ground grid seen from 0.2 above it, looking down with a 100 degree field of view:
    the cells under and behind the camera cross the near plane and the eye plane."""
    rng = np.random.default_rng(seed)
    g = np.linspace(-size / 2, size / 2, n + 1)
    X, Z = np.meshgrid(g, g)
    Y = rng.uniform(-0.03, 0.03, X.shape)
    pos = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    idx = []
    for i in range(n):
        for j in range(n):
            a = i * (n + 1) + j
            idx += [[a, a + 1, a + n + 1], [a + 1, a + n + 2, a + n + 1]]
    M = S.look_at_world_to_clip((0.05, -0.2, -0.3), (0.1, 0.6, 0.5), fov_y_deg=100.0, aspect=res[1] / res[0])
    return S.clip_positions(pos, M[None])[0], np.array(idx, np.uint32), res


def cloud(T=150, seed=1, res=(64, 80), views=1):
    """Random triangles with edges up to about a metre around the eye (80 degree field of view): many have
    vertices on both sides of the near plane and behind the eye. views > 1 turns the camera."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1.2, 1.2, (T, 1, 3))
    pos = (c + rng.uniform(-0.6, 0.6, (T, 3, 3))).reshape(-1, 3).astype(np.float32)
    targets = [(0.2, 0.1, 1.0), (1.0, -0.2, 0.1), (-0.3, 0.9, -0.4), (-1.0, 0.0, -0.5)][:views]
    mats = np.stack([S.look_at_world_to_clip((0.0, 0.0, 0.0), t, fov_y_deg=80.0, aspect=res[1] / res[0])
                     for t in targets])
    clip = S.clip_positions(pos, mats)
    return (clip[0] if views == 1 else clip), np.arange(3 * T, dtype=np.uint32).reshape(T, 3), res

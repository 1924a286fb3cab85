"""Seeded synthetic scenes for the raster / bake / refine workloads.

These stand in for the captured meshes and photographs the reference's examples use (no
dataset ships with the reference). Cameras follow the clip convention of
python/photara_drender/colmap.py:131-153: row-major ``world_to_clip`` with ``clip = M @ [p, 1]``,
camera-space +z forward (w = depth), OpenGL-style z in [-1, 1].
"""
from __future__ import annotations

import math

import numpy as np


def icosphere(subdivisions: int = 4, radius: float = 1.0):
    """Geodesic sphere: 10*4^s+2 vertices, 20*4^s triangles (subdivision 4: 2562 / 5120)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in verts]
    for _ in range(subdivisions):
        cache = {}
        new_faces = []

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    pos = (np.array(v) * radius).astype(np.float32)
    return pos, np.array(faces, dtype=np.uint32)


def spherical_uv(pos: np.ndarray) -> np.ndarray:
    p = pos.astype(np.float64)
    p = p / np.linalg.norm(p, axis=1, keepdims=True)
    u = 0.5 + np.arctan2(p[:, 2], p[:, 0]) / (2 * math.pi)
    v = 0.5 + np.arcsin(np.clip(p[:, 1], -1, 1)) / math.pi
    return np.stack([u, v], axis=1).astype(np.float32)


def vertex_normals(pos: np.ndarray, idx: np.ndarray) -> np.ndarray:
    tri = pos[idx.astype(np.int64)].astype(np.float64)
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    n = np.zeros(pos.shape, np.float64)
    for k in range(3):
        np.add.at(n, idx[:, k].astype(np.int64), fn)
    return (n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-20)).astype(np.float32)


def fibonacci_directions(n: int) -> np.ndarray:
    i = np.arange(n, dtype=np.float64) + 0.5
    phi = np.arccos(1 - 2 * i / n)
    theta = math.pi * (1 + 5 ** 0.5) * i
    return np.stack([np.cos(theta) * np.sin(phi), np.cos(phi), np.sin(theta) * np.sin(phi)], axis=1)


def look_at_world_to_clip(eye, target=(0.0, 0.0, 0.0), fov_y_deg=45.0, aspect=1.0, near=0.1, far=10.0):
    """Pinhole camera looking at ``target``; camera x right, y down, z forward (COLMAP axes)."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    up_hint = np.array([0.0, 1.0, 0.0]) if abs(fwd[1]) < 0.99 else np.array([1.0, 0.0, 0.0])
    right = np.cross(up_hint, fwd)
    right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    R = np.stack([right, down, fwd])
    t = -R @ eye
    f = 1.0 / math.tan(math.radians(fov_y_deg) / 2.0)
    ds = (far + near) / (far - near)
    do = -2.0 * far * near / (far - near)
    M = np.zeros((4, 4))
    M[0, :3], M[0, 3] = (f / aspect) * R[0], (f / aspect) * t[0]
    M[1, :3], M[1, 3] = f * R[1], f * t[1]
    M[2, :3], M[2, 3] = ds * R[2], ds * t[2] + do
    M[3, :3], M[3, 3] = R[2], t[2]
    return M.astype(np.float32)


def orbit_cameras(n: int, radius: float = 3.0, fov_y_deg: float = 45.0, aspect: float = 1.0):
    dirs = fibonacci_directions(n)
    eyes = dirs * radius
    mats = np.stack([look_at_world_to_clip(e, fov_y_deg=fov_y_deg, aspect=aspect) for e in eyes])
    return mats, eyes.astype(np.float32)


def clip_positions(pos3: np.ndarray, mats: np.ndarray) -> np.ndarray:
    """[views, V, 4] clip positions, computed in float32 in the order m0*x + m1*y + m2*z + m3."""
    p = pos3.astype(np.float32)
    out = np.empty((mats.shape[0], p.shape[0], 4), np.float32)
    for k, M in enumerate(mats.astype(np.float32)):
        for r in range(4):
            out[k, :, r] = ((M[r, 0] * p[:, 0] + M[r, 1] * p[:, 1]) + M[r, 2] * p[:, 2]) + M[r, 3]
    return out


def uv_sphere(n_lat: int, n_lon: int):
    """Latitude/longitude sphere with 2*n_lat*n_lon triangles (poles as degenerate-free fans)."""
    lat = np.linspace(0, math.pi, n_lat + 1)[1:-1]
    lon = np.linspace(0, 2 * math.pi, n_lon, endpoint=False)
    ring = np.stack([np.outer(np.sin(lat), np.cos(lon)), np.repeat(np.cos(lat)[:, None], n_lon, 1),
                     np.outer(np.sin(lat), np.sin(lon))], axis=-1).reshape(-1, 3)
    pos = np.concatenate([[[0, 1, 0]], ring, [[0, -1, 0]]])
    south = pos.shape[0] - 1
    faces = []
    j = np.arange(n_lon)
    jn = (j + 1) % n_lon
    faces.append(np.stack([np.zeros(n_lon, int), 1 + jn, 1 + j], 1))
    for i in range(n_lat - 2):
        a = 1 + i * n_lon + j
        b = 1 + i * n_lon + jn
        c = 1 + (i + 1) * n_lon + j
        d = 1 + (i + 1) * n_lon + jn
        faces.append(np.stack([a, b, d], 1))
        faces.append(np.stack([a, d, c], 1))
    last = 1 + (n_lat - 2) * n_lon
    faces.append(np.stack([np.full(n_lon, south), last + j, last + jn], 1))
    return pos.astype(np.float64), np.concatenate(faces).astype(np.int64)


def displaced_sphere(triangles: int, seed: int = 0, amplitude: float = 0.05, gutter_texels: int = 8,
                     atlas_size: int = 4096):
    """Sphere of about ``triangles`` faces with radial displacement
    r = 1 + amplitude * sum_8 sin(k.dir + phi) / 8 and six cube-projection charts packed 3x2.

    Returns positions [V,3], normals [V,3], uv [V,2], indices [T,3], face_chart_ids [T],
    vertex_remap [V] (original vertex of each chart-duplicated vertex)."""
    rng = np.random.default_rng(seed)
    n_lon = max(8, int(round(math.sqrt(triangles))))
    n_lat = max(4, int(round(triangles / (2 * n_lon))) + 1)
    base, faces = uv_sphere(n_lat, n_lon)
    k = rng.normal(size=(8, 3)) * 3.0
    phase = rng.uniform(0, 2 * math.pi, size=8)
    r = 1.0 + amplitude * np.sin(base @ k.T + phase).sum(1) / 8.0
    pos = base * r[:, None]
    nrm = vertex_normals(pos.astype(np.float32), faces.astype(np.uint32)).astype(np.float64)
    # chart of each face: dominant axis of the centroid direction
    cen = base[faces].mean(1)
    axis = np.argmax(np.abs(cen), 1)
    sign = np.take_along_axis(cen, axis[:, None], 1)[:, 0] >= 0
    chart = (axis * 2 + (~sign)).astype(np.int32)
    key = faces * 6 + chart[:, None]
    uniq, inv = np.unique(key.reshape(-1), return_inverse=True)
    remap = (uniq // 6).astype(np.int64)
    vchart = (uniq % 6).astype(np.int64)
    new_idx = inv.reshape(-1, 3)
    d = base[remap]
    ax = vchart // 2
    other = np.array([[1, 2], [0, 2], [0, 1]])[ax]
    denom = np.abs(np.take_along_axis(d, ax[:, None], 1)[:, 0])
    a = np.take_along_axis(d, other[:, :1], 1)[:, 0] / denom
    b = np.take_along_axis(d, other[:, 1:], 1)[:, 0] / denom
    lim = 1.6
    cell_u, cell_v = vchart % 3, vchart // 3
    g = gutter_texels / atlas_size
    cw, ch = 1.0 / 3.0, 1.0 / 2.0
    uu = cell_u * cw + g + (np.clip(a, -lim, lim) / lim * 0.5 + 0.5) * (cw - 2 * g)
    vv = cell_v * ch + g + (np.clip(b, -lim, lim) / lim * 0.5 + 0.5) * (ch - 2 * g)
    uv = np.stack([uu, vv], 1)
    return (pos[remap].astype(np.float32), nrm[remap].astype(np.float32), uv.astype(np.float32),
            new_idx.astype(np.uint32), chart, remap.astype(np.uint32))


def seam_uv_pairs(uv: np.ndarray, idx: np.ndarray, remap: np.ndarray, face_chart: np.ndarray,
                  samples_per_edge: int = 4) -> np.ndarray:
    """Samples along every mesh edge shared by two faces of different charts: [S, 2, 2] UV pairs,
    the layout examples/texture_workflow.py:34-71 produces."""
    faces = idx.astype(np.int64)
    rem = remap.astype(np.int64)
    keys, lo_uv, hi_uv, charts = [], [], [], []
    for a, b in ((0, 1), (1, 2), (2, 0)):
        va, vb = faces[:, a], faces[:, b]
        oa, ob = rem[va], rem[vb]
        swap = oa > ob
        keys.append(np.minimum(oa, ob) * (1 << 32) + np.maximum(oa, ob))
        lo_uv.append(np.where(swap[:, None], uv[vb], uv[va]))
        hi_uv.append(np.where(swap[:, None], uv[va], uv[vb]))
        charts.append(face_chart)
    key = np.concatenate(keys)
    lo = np.concatenate(lo_uv)
    hi = np.concatenate(hi_uv)
    ch = np.concatenate(charts)
    order = np.argsort(key, kind="stable")
    key, lo, hi, ch = key[order], lo[order], hi[order], ch[order]
    starts = np.r_[0, np.flatnonzero(key[1:] != key[:-1]) + 1]
    ends = np.r_[starts[1:], key.size]
    starts = starts[(ends - starts) == 2]
    starts = starts[ch[starts] != ch[starts + 1]]
    if starts.size == 0:
        return np.zeros((0, 2, 2), np.float32)
    t = ((np.arange(samples_per_edge) + 0.5) / samples_per_edge)[None, :, None]
    first = lo[starts, None] * (1 - t) + hi[starts, None] * t
    second = lo[starts + 1, None] * (1 - t) + hi[starts + 1, None] * t
    return np.ascontiguousarray(np.stack([first, second], 2).reshape(-1, 2, 2), dtype=np.float32)

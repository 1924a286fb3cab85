"""The data formats on either side of the bake / refine path, as the reference's scripts write and read
them, so files move between the two implementations unchanged:

* COLMAP text models and the clip convention of python/photara_drender/colmap.py:39-153,253-256:
  row-major world-to-clip matrices ``clip = M @ [p, 1]`` of undistorted pinhole cameras (OpenGL-style
  depth in [-1, 1], principal point moved into NDC), camera centres ``-R^T t``, and the near / far
  planes derived from the mesh's depths when not given.
* Dense seam pairs ``[S, 2, 2]`` (examples/texture_workflow.py:34-71): UV positions sampled along each
  mesh edge that two charts share, one row per sample, (uv in the first chart, uv in the second).
* The ``.npz`` archives of examples/bake_colmap.py:106-121,162-178 (initial and final bakes) and
  examples/refine_colmap_texture.py:296-307 (refined atlas): the same keys, dtypes and shapes.

Everything here is host-side NumPy; it feeds the device path (world_to_clip, seam_uv_pairs) and stores
its outputs.
"""
from __future__ import annotations

from pathlib import Path
from typing import Dict, NamedTuple, Optional, Sequence, Tuple, Union

import numpy as np

PathLike = Union[str, Path]


# ---- COLMAP -----------------------------------------------------------------------------------------

class ColmapCamera(NamedTuple):
    camera_id: int
    model: str
    width: int
    height: int
    parameters: np.ndarray


class ColmapImage(NamedTuple):
    image_id: int
    camera_id: int
    name: str
    rotation: np.ndarray      # [3, 3] world -> camera, float64
    translation: np.ndarray   # [3]


class ColmapViews(NamedTuple):
    """Everything of a COLMAP model the bake needs except the photographs themselves."""
    world_to_clip: np.ndarray     # [N, 4, 4] float32, row-major
    camera_positions: np.ndarray  # [N, 3] float32
    image_names: Tuple[str, ...]
    image_sizes: Tuple[Tuple[int, int], ...]  # (height, width) the photographs must have


def quaternion_to_rotation(quaternion: Sequence[float]) -> np.ndarray:
    """Rotation matrix of a unit quaternion (w, x, y, z), COLMAP's convention (colmap.py:39-48)."""
    w, x, y, z = (float(v) for v in np.asarray(quaternion, dtype=np.float64))
    xx, yy, zz = x * x, y * y, z * z
    return np.array([[1.0 - 2.0 * (yy + zz), 2.0 * (x * y - w * z), 2.0 * (x * z + w * y)],
                     [2.0 * (x * y + w * z), 1.0 - 2.0 * (xx + zz), 2.0 * (y * z - w * x)],
                     [2.0 * (x * z - w * y), 2.0 * (y * z + w * x), 1.0 - 2.0 * (xx + yy)]], dtype=np.float64)


def _records(path: Path):
    with path.open("r", encoding="utf-8") as f:
        for raw in f:
            line = raw.strip()
            if line and not raw.startswith("#"):
                yield line


def read_colmap_text_model(sparse_path: PathLike) -> Tuple[Dict[int, ColmapCamera], Tuple[ColmapImage, ...]]:
    """cameras.txt and images.txt of a COLMAP text model (colmap.py:51-90); images sorted by id."""
    root = Path(sparse_path)
    cameras: Dict[int, ColmapCamera] = {}
    for line in _records(root / "cameras.txt"):
        f = line.split()
        cameras[int(f[0])] = ColmapCamera(int(f[0]), f[1], int(f[2]), int(f[3]), np.asarray(f[4:], dtype=np.float64))
    lines = list(_records(root / "images.txt"))
    if len(lines) % 2:
        raise ValueError("COLMAP images.txt must contain one points2D line after each image line")
    images = []
    for line in lines[0::2]:
        f = line.split(maxsplit=9)
        if len(f) != 10:
            raise ValueError(f"invalid COLMAP image record: {line[:120]}")
        q = np.asarray(f[1:5], dtype=np.float64)
        n = np.linalg.norm(q)
        if not np.isfinite(n) or n <= 0.0:
            raise ValueError(f"image {f[0]} contains an invalid quaternion")
        images.append(ColmapImage(int(f[0]), int(f[8]), f[9], quaternion_to_rotation(q / n),
                                  np.asarray(f[5:8], dtype=np.float64)))
    images.sort(key=lambda im: im.image_id)
    return cameras, tuple(images)


def pinhole_parameters(camera: ColmapCamera) -> Tuple[float, float, float, float]:
    """(fx, fy, cx, cy) of a PINHOLE or SIMPLE_PINHOLE camera (colmap.py:93-101)."""
    p = camera.parameters
    if camera.model == "PINHOLE" and p.size == 4:
        return float(p[0]), float(p[1]), float(p[2]), float(p[3])
    if camera.model == "SIMPLE_PINHOLE" and p.size == 3:
        return float(p[0]), float(p[0]), float(p[1]), float(p[2])
    raise ValueError(f"camera {camera.camera_id} uses {camera.model}; undistort it to PINHOLE or SIMPLE_PINHOLE "
                     "before projection")


def depth_range(image: ColmapImage, mesh_positions: Optional[np.ndarray], near: Optional[float],
                far: Optional[float]) -> Tuple[float, float]:
    """Near and far planes (colmap.py:104-128): as given, else 1e-3 / 1e3 without a mesh, else half the
    nearest and 1.5x the farthest positive mesh depth (near at least 1e-4)."""
    def checked(n, f):
        if not 0.0 < n < f:
            raise ValueError("near and far must satisfy 0 < near < far")
        return float(n), float(f)

    if near is not None and far is not None:
        return checked(near, far)
    if mesh_positions is None:
        return checked(1e-3 if near is None else near, 1e3 if far is None else far)
    depth = np.asarray(mesh_positions, dtype=np.float64) @ image.rotation[2] + image.translation[2]
    depth = depth[depth > 1e-6]
    if depth.size == 0:
        raise ValueError(f"mesh is entirely behind COLMAP camera for {image.name}")
    return checked(max(1e-4, float(depth.min()) * 0.5) if near is None else float(near),
                   float(depth.max()) * 1.5 if far is None else float(far))


def colmap_world_to_clip(camera: ColmapCamera, image: ColmapImage, near: float, far: float) -> np.ndarray:
    """Row-major [4, 4] float32 world-to-clip matrix of the renderer for a COLMAP view
    (colmap.py:131-153): x_clip = 2 fx / W * x_cam + (2 cx / W - 1) * z_cam, likewise for y, OpenGL
    depth z_clip = (f + n) / (f - n) * z_cam - 2 f n / (f - n), w_clip = z_cam; computed in float64."""
    fx, fy, cx, cy = pinhole_parameters(camera)
    R, t = image.rotation, image.translation
    proj = np.zeros((4, 4), dtype=np.float64)  # the projection applied to camera-space points
    proj[0, 0], proj[0, 2] = 2.0 * fx / camera.width, 2.0 * cx / camera.width - 1.0
    proj[1, 1], proj[1, 2] = 2.0 * fy / camera.height, 2.0 * cy / camera.height - 1.0
    proj[2, 2], proj[2, 3] = (far + near) / (far - near), -2.0 * far * near / (far - near)
    proj[3, 2] = 1.0
    # expanded row by row as the reference writes it, so the float64 values round identically
    m = np.empty((4, 4), dtype=np.float64)
    m[0, :3] = proj[0, 0] * R[0] + proj[0, 2] * R[2]
    m[0, 3] = proj[0, 0] * t[0] + proj[0, 2] * t[2]
    m[1, :3] = proj[1, 1] * R[1] + proj[1, 2] * R[2]
    m[1, 3] = proj[1, 1] * t[1] + proj[1, 2] * t[2]
    m[2, :3] = proj[2, 2] * R[2]
    m[2, 3] = proj[2, 2] * t[2] + proj[2, 3]
    m[3, :3] = R[2]
    m[3, 3] = t[2]
    return m.astype(np.float32)


def camera_position(image: ColmapImage) -> np.ndarray:
    """Camera centre in world space, -R^T t, as float32 (colmap.py:256)."""
    return (-image.rotation.T @ image.translation).astype(np.float32)


def colmap_views(sparse_path: PathLike, *, mesh_positions: Optional[np.ndarray] = None,
                 image_names: Optional[Sequence[str]] = None, image_stride: int = 1,
                 max_images: Optional[int] = None, near: Optional[float] = None,
                 far: Optional[float] = None) -> ColmapViews:
    """The view selection and matrices of load_colmap_projection (colmap.py:192-262) without reading the
    photographs: the caller loads image_names in order, each of size image_sizes[k]."""
    if image_stride < 1:
        raise ValueError("image_stride must be positive")
    cameras, images = read_colmap_text_model(sparse_path)
    wanted = None if image_names is None else set(image_names)
    chosen = [im for im in images if wanted is None or im.name in wanted]
    if wanted is not None:
        missing = wanted.difference(im.name for im in chosen)
        if missing:
            raise FileNotFoundError(f"images are absent from COLMAP model: {sorted(missing)}")
    chosen = chosen[::image_stride]
    if max_images is not None:
        chosen = chosen[:max_images]
    if not chosen:
        raise ValueError("no COLMAP images matched the selection")
    mesh = None
    if mesh_positions is not None:
        mesh = np.asarray(mesh_positions, dtype=np.float64)
        if mesh.ndim != 2 or mesh.shape[1] != 3:
            raise ValueError("mesh_positions must have shape [vertex_count, 3]")
        if mesh.shape[0] == 0 or not np.isfinite(mesh).all():
            raise ValueError("mesh_positions must be non-empty and finite")
    mats, eyes, names, sizes = [], [], [], []
    for im in chosen:
        cam = cameras.get(im.camera_id)
        if cam is None:
            raise ValueError(f"image {im.name} references missing camera {im.camera_id}")
        n, f = depth_range(im, mesh, near, far)
        mats.append(colmap_world_to_clip(cam, im, n, f))
        eyes.append(camera_position(im))
        names.append(im.name)
        sizes.append((cam.height, cam.width))
    return ColmapViews(np.ascontiguousarray(mats, dtype=np.float32), np.ascontiguousarray(eyes, dtype=np.float32),
                       tuple(names), tuple(sizes))


def srgb_to_linear(image: np.ndarray) -> np.ndarray:
    """IEC 61966-2-1 decoding, as colmap.py:156-157 applies with linearize_srgb."""
    x = np.asarray(image, dtype=np.float32)
    return np.where(x <= 0.04045, x / 12.92, ((x + 0.055) / 1.055) ** 2.4).astype(np.float32)


def linear_to_srgb(image: np.ndarray) -> np.ndarray:
    """IEC 61966-2-1 encoding, the inverse of srgb_to_linear (used for display PNGs of linear atlases)."""
    x = np.asarray(image, dtype=np.float32)
    return np.where(x <= 0.0031308, x * 12.92, 1.055 * np.power(np.maximum(x, 0.0), 1.0 / 2.4) - 0.055
                    ).astype(np.float32)


# ---- seam pairs -------------------------------------------------------------------------------------

def dense_seam_pairs(mesh, samples_per_edge: int) -> np.ndarray:
    """[S, 2, 2] float32 UV pairs along every mesh edge whose two faces lie in different charts
    (examples/texture_workflow.py:34-71). `mesh` has indices [T, 3], vertex_remap (UV-split vertex ->
    original vertex), uv [V, 2] and face_chart_ids [T]. Each shared edge contributes samples_per_edge
    rows at t = (k + 0.5) / samples_per_edge from its lower to its higher original vertex; row
    (uv in the face met first, uv in the other face). Edges are ordered by their (low, high) key with
    NumPy's default argsort, which also decides which face is met first."""
    faces = np.asarray(mesh.indices).reshape(-1, 3)
    remap = np.asarray(mesh.vertex_remap)
    uv = np.asarray(mesh.uv)
    charts = np.asarray(mesh.face_chart_ids)
    a = faces[:, [0, 1, 2]].T.reshape(-1)   # edge k of face f sits at k * T + f
    b = faces[:, [1, 2, 0]].T.reshape(-1)
    oa, ob = remap[a], remap[b]
    flip = oa > ob
    lo_v = np.where(flip, b, a)
    hi_v = np.where(flip, a, b)
    key = (np.minimum(oa, ob).astype(np.uint64) << np.uint64(32)) | np.maximum(oa, ob).astype(np.uint64)
    chart = np.tile(charts, 3)
    order = np.argsort(key)
    key, lo_v, hi_v, chart = key[order], lo_v[order], hi_v[order], chart[order]
    first = np.r_[True, key[1:] != key[:-1]]
    start = np.flatnonzero(first)
    count = np.diff(np.r_[start, key.size])
    pair = start[count == 2]
    pair = pair[chart[pair] != chart[pair + 1]]
    if pair.size == 0:
        return np.empty((0, 2, 2), dtype=np.float32)
    t = ((np.arange(samples_per_edge, dtype=np.float32) + 0.5) / samples_per_edge)[None, :, None]
    side = [uv[lo_v[pair + s], None] * (1.0 - t) + uv[hi_v[pair + s], None] * t for s in (0, 1)]
    return np.ascontiguousarray(np.stack(side, axis=2).reshape(-1, 2, 2), dtype=np.float32)


# ---- npz archives -----------------------------------------------------------------------------------

#: examples/bake_colmap.py:110-121: the initial bake (before refinement)
INITIAL_BAKE_KEYS = ("color", "confidence", "source_view", "valid_mask", "texture_source", "source_images_path",
                     "mask_applied", "visibility_mode", "used_ray_query", "color_space")
#: examples/bake_colmap.py:162-178: the final bake, the initial keys plus the refinement results
FINAL_BAKE_KEYS = INITIAL_BAKE_KEYS + ("optimized", "history", "seam_history", "seam_pairs")
#: examples/refine_colmap_texture.py:296-307: a refined atlas
REFINED_KEYS = ("color", "valid_mask", "history", "seam_history", "seam_pairs", "color_space", "texture_source",
                "source_images_path", "mask_applied")


def _text(value) -> np.ndarray:
    return np.asarray(str(value))


def save_bake_npz(path: PathLike, baked, *, texture_source: str, source_images_path: PathLike,
                  mask_applied: bool, color_space: str, visibility_mode: str = "ray_query", color=None,
                  optimized: Optional[bool] = None, history=None, seam_history=None, seam_pairs=None) -> Path:
    """Writes a bake archive with the keys of bake_colmap.py: the initial form, or the final form when
    `optimized` is given (then history, seam_history and seam_pairs default to empty). `baked` has
    color, confidence, source_view, valid_mask and used_ray_query (BakedTexture); `color` overrides the
    stored colour (the final bake stores the refined RGB with the valid mask as alpha)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    data = dict(color=np.asarray(baked.color if color is None else color, dtype=np.float32),
                confidence=np.asarray(baked.confidence, dtype=np.float32),
                source_view=np.asarray(baked.source_view), valid_mask=np.asarray(baked.valid_mask, dtype=np.float32),
                texture_source=_text(texture_source), source_images_path=_text(Path(source_images_path).resolve()),
                mask_applied=np.asarray(bool(mask_applied)), visibility_mode=_text(visibility_mode),
                used_ray_query=np.asarray(bool(baked.used_ray_query)), color_space=_text(color_space))
    if optimized is not None:
        data.update(optimized=np.asarray(bool(optimized)),
                    history=np.asarray(np.empty(0) if history is None else history, dtype=np.float32),
                    seam_history=np.asarray(np.empty(0) if seam_history is None else seam_history, dtype=np.float32),
                    seam_pairs=np.asarray(np.empty((0, 2, 2)) if seam_pairs is None else seam_pairs,
                                          dtype=np.float32).reshape(-1, 2, 2))
    np.savez_compressed(path, **data)
    return path


def save_refined_npz(path: PathLike, color, valid_mask, *, history, seam_history, seam_pairs, color_space: str,
                     texture_source: str, source_images_path: PathLike, mask_applied: bool = True) -> Path:
    """Writes a refined-atlas archive with the keys of refine_colmap_texture.py:296-307."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, color=np.asarray(color, dtype=np.float32),
                        valid_mask=np.asarray(valid_mask, dtype=np.float32),
                        history=np.asarray(history, dtype=np.float32),
                        seam_history=np.asarray(seam_history, dtype=np.float32),
                        seam_pairs=np.asarray(seam_pairs, dtype=np.float32).reshape(-1, 2, 2),
                        color_space=_text(color_space), texture_source=_text(texture_source),
                        source_images_path=_text(Path(source_images_path).resolve()),
                        mask_applied=np.asarray(bool(mask_applied)))
    return path


def load_archive(path: PathLike) -> Dict[str, np.ndarray]:
    """Reads any of the three archives, checks it is one of them and returns its arrays; 0-d text and
    flag entries come back as Python str / bool."""
    with np.load(Path(path), allow_pickle=False) as z:
        keys = tuple(z.files)
        data = {k: z[k] for k in keys}
    kinds = {"initial bake": INITIAL_BAKE_KEYS, "final bake": FINAL_BAKE_KEYS, "refined atlas": REFINED_KEYS}
    if not any(set(keys) == set(v) for v in kinds.values()):
        raise ValueError(f"{path} is not a bake or refinement archive (keys {sorted(keys)})")
    color = data["color"]
    if color.ndim != 3 or color.shape[2] not in (3, 4) or data["valid_mask"].shape != color.shape[:2]:
        raise ValueError("archive colour must be [H, W, 3|4] with a matching valid_mask")
    if "seam_pairs" in data and (data["seam_pairs"].ndim != 3 or data["seam_pairs"].shape[1:] != (2, 2)):
        raise ValueError("archive seam_pairs must have shape [S, 2, 2]")
    out: Dict[str, object] = {}
    for k, v in data.items():
        if v.ndim == 0 and v.dtype.kind in "US":
            out[k] = str(v)
        elif v.ndim == 0 and v.dtype == np.bool_:
            out[k] = bool(v)
        else:
            out[k] = v
    return out  # type: ignore[return-value]

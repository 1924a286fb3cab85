"""photara_drender_gb300.formats against golden vectors made by the reference's own Python
(tests/golden/make_formats_golden.py): COLMAP parsing and clip matrices, dense seam pairs; and the
.npz archives' key sets of the reference's bake and refine scripts."""
import os
import types

import numpy as np
import pytest

from photara_drender_gb300 import formats as F

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "formats_small.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture()
def model_dir(tmp_path, golden):
    (tmp_path / "cameras.txt").write_text(str(golden["cameras_txt"]))
    (tmp_path / "images.txt").write_text(str(golden["images_txt"]))
    return tmp_path


def test_colmap_matrices_match_reference(golden, model_dir):
    cameras, images = F.read_colmap_text_model(model_dir)
    assert len(images) == 6 and [im.image_id for im in images] == sorted(im.image_id for im in images)
    assert np.array_equal(np.stack([im.rotation for im in images]), golden["rotations"])
    views = F.colmap_views(model_dir)
    assert np.array_equal(views.world_to_clip, golden["world_to_clip"])
    assert np.array_equal(views.camera_positions, golden["camera_positions"])
    with_mesh = F.colmap_views(model_dir, mesh_positions=golden["mesh_positions"])
    assert np.array_equal(with_mesh.world_to_clip, golden["world_to_clip_mesh"])
    assert views.image_names[0] == "view_000.png" and views.image_sizes[0] == (480, 640)
    assert F.colmap_views(model_dir, image_stride=2, max_images=2).image_names == ("view_000.png", "view_002.png")


def test_colmap_clip_convention():
    # a camera at the origin looking down +z: the principal point maps to NDC (2cx/W - 1, 2cy/H - 1)
    cam = F.ColmapCamera(1, "PINHOLE", 100, 50, np.array([80.0, 90.0, 30.0, 20.0]))
    im = F.ColmapImage(1, 1, "a", np.eye(3), np.zeros(3))
    m = F.colmap_world_to_clip(cam, im, 0.5, 10.0).astype(np.float64)
    p = m @ np.array([0.0, 0.0, 2.0, 1.0])
    assert np.allclose(p[:2] / p[3], [2 * 30 / 100 - 1, 2 * 20 / 50 - 1])
    for z, ndc in ((0.5, -1.0), (10.0, 1.0)):
        q = m @ np.array([0.0, 0.0, z, 1.0])
        assert abs(q[2] / q[3] - ndc) < 1e-6
    with pytest.raises(ValueError, match="undistort"):
        F.pinhole_parameters(F.ColmapCamera(2, "OPENCV", 10, 10, np.zeros(8)))
    with pytest.raises(ValueError, match="0 < near < far"):
        F.depth_range(im, None, 2.0, 1.0)


def test_colmap_errors(tmp_path):
    (tmp_path / "cameras.txt").write_text("1 PINHOLE 10 10 1 1 5 5\n")
    (tmp_path / "images.txt").write_text("1 1 0 0 0 0 0 1 1 a.png\n")
    with pytest.raises(ValueError, match="points2D line"):
        F.read_colmap_text_model(tmp_path)
    (tmp_path / "images.txt").write_text("1 0 0 0 0 0 0 1 1 a.png\n\n")
    (tmp_path / "images.txt").write_text("1 0 0 0 0 0 0 1 1 a.png\nx\n")
    with pytest.raises(ValueError, match="invalid quaternion"):
        F.read_colmap_text_model(tmp_path)
    (tmp_path / "images.txt").write_text("1 1 0 0 0 0 0 1 1 a.png\nx\n")
    with pytest.raises(FileNotFoundError):
        F.colmap_views(tmp_path, image_names=["b.png"])
    with pytest.raises(ValueError, match="entirely behind"):
        F.colmap_views(tmp_path, mesh_positions=np.array([[0.0, 0.0, -5.0]]))


def test_dense_seam_pairs_match_reference(golden):
    mesh = types.SimpleNamespace(indices=golden["seam_indices"], vertex_remap=golden["seam_remap"],
                                 uv=golden["seam_uv"], face_chart_ids=golden["seam_charts"])
    for k in (1, 3):
        got = F.dense_seam_pairs(mesh, k)
        assert got.dtype == np.float32 and np.array_equal(got, golden[f"seam_pairs_{k}"]), k
    single = types.SimpleNamespace(indices=golden["seam_indices"], vertex_remap=golden["seam_remap"],
                                   uv=golden["seam_uv"], face_chart_ids=np.zeros_like(golden["seam_charts"]))
    assert F.dense_seam_pairs(single, 2).shape == (0, 2, 2)


def test_srgb_round_trip():
    x = np.linspace(0, 1, 101, dtype=np.float32)
    assert np.allclose(F.linear_to_srgb(F.srgb_to_linear(x)), x, atol=2e-6)


def test_archives_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    baked = types.SimpleNamespace(color=rng.uniform(size=(8, 6, 4)).astype(np.float32),
                                  confidence=rng.uniform(size=(8, 6)).astype(np.float32),
                                  source_view=rng.integers(0, 3, size=(8, 6)).astype(np.uint32),
                                  valid_mask=(rng.uniform(size=(8, 6)) > 0.5).astype(np.float32), used_ray_query=True)
    p = F.save_bake_npz(tmp_path / "initial.npz", baked, texture_source="photos", source_images_path=tmp_path,
                        mask_applied=False, color_space="srgb")
    a = F.load_archive(p)
    assert set(a) == set(F.INITIAL_BAKE_KEYS) and a["used_ray_query"] is True and a["visibility_mode"] == "ray_query"
    assert np.array_equal(a["color"], baked.color) and a["source_view"].dtype == np.uint32
    pairs = rng.uniform(size=(5, 2, 2)).astype(np.float32)
    p = F.save_bake_npz(tmp_path / "final.npz", baked, texture_source="photos", source_images_path=tmp_path,
                        mask_applied=True, color_space="linear", optimized=True, history=[0.5, 0.25],
                        seam_pairs=pairs)
    a = F.load_archive(p)
    assert set(a) == set(F.FINAL_BAKE_KEYS) and a["optimized"] is True and a["seam_history"].shape == (0,)
    assert np.array_equal(a["seam_pairs"], pairs)
    p = F.save_refined_npz(tmp_path / "refined.npz", baked.color, baked.valid_mask, history=[1.0], seam_history=[],
                           seam_pairs=pairs, color_space="srgb", texture_source="photos",
                           source_images_path=tmp_path)
    assert set(F.load_archive(p)) == set(F.REFINED_KEYS)
    np.savez(tmp_path / "other.npz", color=baked.color)
    with pytest.raises(ValueError, match="not a bake"):
        F.load_archive(tmp_path / "other.npz")

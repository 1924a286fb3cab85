"""Golden vectors for photara_drender_gb300.formats from the reference's own Python: the COLMAP
helpers of python/photara_drender/colmap.py (NumPy only, loaded from its file) and dense_seam_pairs of
examples/texture_workflow.py (loaded with stand-ins for the two modules it imports but this function
does not use). Run here, where the reference sources exist:
``python tests/golden/make_formats_golden.py``; writes tests/golden/formats_small.npz."""
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))  # the repository root
REFERENCE = os.environ.get("PDR_REFERENCE_DIR", "/root/reference")  # the reference checkout

from photara_drender_gb300 import synthetic as S  # noqa: E402


def load(name, path, stubs=()):
    for stub in stubs:
        sys.modules.setdefault(stub, types.ModuleType(stub))
    if "PIL" in stubs:
        sys.modules["PIL"].Image = types.SimpleNamespace()
        sys.modules["PIL"].ImageFilter = types.SimpleNamespace()
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def colmap_model(rng, n_images=6):
    """A COLMAP text model: two pinhole cameras and posed images looking at the origin."""
    cams = ["# Camera list", "1 PINHOLE 640 480 520.5 521.25 318.7 241.3", "2 SIMPLE_PINHOLE 800 600 700.0 401.5 299.0"]
    imgs = ["# Image list"]
    for k in range(n_images):
        q = rng.normal(size=4)
        q *= (1.0 + rng.uniform()) / np.linalg.norm(q)   # not unit: the reader normalises
        t = rng.normal(size=3) * 0.3 + np.array([0.0, 0.0, 3.0])
        imgs.append(f"{k + 1} {q[0]:.17g} {q[1]:.17g} {q[2]:.17g} {q[3]:.17g} {t[0]:.17g} {t[1]:.17g} {t[2]:.17g} "
                    f"{1 + k % 2} view_{k:03d}.png")
        imgs.append("10.0 20.0 -1")
    return "\n".join(cams) + "\n", "\n".join(imgs) + "\n"


def main():
    colmap = load("ref_colmap", os.path.join(REFERENCE, "python", "photara_drender", "colmap.py"))
    workflow = load("ref_texture_workflow", os.path.join(REFERENCE, "examples", "texture_workflow.py"),
                    stubs=("PIL", "photara_drender"))
    rng = np.random.default_rng(5)
    cams_txt, imgs_txt = colmap_model(rng)
    import tempfile
    from pathlib import Path

    out = {"cameras_txt": np.asarray(cams_txt), "images_txt": np.asarray(imgs_txt)}
    pos3, nrm, uv, idx, chart, remap = S.displaced_sphere(3000, seed=2, atlas_size=256)
    out["mesh_positions"] = pos3
    with tempfile.TemporaryDirectory() as d:
        (Path(d) / "cameras.txt").write_text(cams_txt)
        (Path(d) / "images.txt").write_text(imgs_txt)
        cameras, images = colmap.read_colmap_text_model(d)
        mats, eyes, mats_mesh, rots = [], [], [], []
        for im in images:
            cam = cameras[im.camera_id]
            n, f = colmap._depth_range(im, None, None, None)
            mats.append(colmap._world_to_clip(cam, im, n, f))
            n2, f2 = colmap._depth_range(im, pos3.astype(np.float64), None, None)
            mats_mesh.append(colmap._world_to_clip(cam, im, n2, f2))
            eyes.append((-im.rotation.T @ im.translation).astype(np.float32))
            rots.append(im.rotation)
    out.update(world_to_clip=np.stack(mats), world_to_clip_mesh=np.stack(mats_mesh), camera_positions=np.stack(eyes),
               rotations=np.stack(rots))
    mesh = types.SimpleNamespace(indices=idx, vertex_remap=remap, uv=uv, face_chart_ids=chart)
    for k in (1, 3):
        out[f"seam_pairs_{k}"] = workflow.dense_seam_pairs(mesh, k)
    out.update(seam_indices=idx, seam_remap=remap, seam_uv=uv, seam_charts=chart)
    np.savez_compressed(os.path.join(HERE, "formats_small.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()

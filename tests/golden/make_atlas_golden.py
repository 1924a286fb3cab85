"""Golden vectors for the atlas losses from the reference's own Python: atlas_total_variation and
masked_charbonnier_loss of python/photara_drender/atlas.py, loaded from its file inside a stand-in
package (the native module and the torch adapters it imports are not used by these two functions),
evaluated with torch autograd in float64. Run here, where the reference sources exist:
``python tests/golden/make_atlas_golden.py``; writes tests/golden/atlas_losses.npz."""
import importlib.util
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("PDR_REFERENCE_DIR", "/root/reference")  # the reference checkout


def load_reference_atlas():
    pkg = types.ModuleType("ref_pdr")
    pkg.__path__ = []
    native = types.ModuleType("ref_pdr._photara_drender")
    native.Rasterizer = object
    adapters = types.ModuleType("ref_pdr.torch")
    adapters.interpolate = adapters.rasterize = adapters.texture = None
    sys.modules.update({"ref_pdr": pkg, "ref_pdr._photara_drender": native, "ref_pdr.torch": adapters})
    spec = importlib.util.spec_from_file_location("ref_pdr.atlas",
                                                  os.path.join(REFERENCE, "python", "photara_drender", "atlas.py"))
    mod = importlib.util.module_from_spec(spec)
    mod.__package__ = "ref_pdr"
    sys.modules["ref_pdr.atlas"] = mod  # dataclasses look the module up while the file executes
    spec.loader.exec_module(mod)
    return mod


def main():
    atlas = load_reference_atlas()
    rng = np.random.default_rng(9)
    out = {}
    H, W = 24, 32
    tex = rng.uniform(size=(H, W, 3))
    tex[5:9, 4:12] = 0.5  # flat patches: differences below epsilon
    tex = tex.astype(np.float32).astype(np.float64)  # float32-exact, so fp32 restatements see the same input
    valid = rng.uniform(size=(H, W)) < 0.8
    chart = (np.arange(W)[None, :] // 11 + 3 * (np.arange(H)[:, None] // 9)).astype(np.int32)
    for name, v, c in (("tv_all", None, None), ("tv_masked", valid, chart)):
        t = torch.tensor(tex, requires_grad=True)
        loss = atlas.atlas_total_variation(t, valid_mask=None if v is None else torch.tensor(v),
                                           chart_ids=None if c is None else torch.tensor(c), epsilon=1e-4)
        loss.backward()
        out[name + "_loss"] = loss.detach().numpy()
        out[name + "_grad"] = t.grad.numpy()
    out.update(tex=tex, valid=valid, chart=chart)
    rendered = rng.uniform(size=(16, 20, 3)).astype(np.float32).astype(np.float64)
    target = (rendered + rng.normal(scale=0.05, size=rendered.shape)).astype(np.float32).astype(np.float64)
    mask = (rng.uniform(size=(16, 20, 1)) < 0.7).astype(np.float64)
    r = torch.tensor(rendered, requires_grad=True)
    loss = atlas.masked_charbonnier_loss(r, torch.tensor(target), torch.tensor(mask), epsilon=1e-3)
    loss.backward()
    out.update(rendered=rendered, target=target, mask=mask, charbonnier_loss=loss.detach().numpy(),
               charbonnier_grad=r.grad.numpy())
    np.savez_compressed(os.path.join(HERE, "atlas_losses.npz"), **out)
    print({k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    main()

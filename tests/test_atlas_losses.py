"""The atlas research losses (python/photara_drender/atlas.py:65-115) against golden vectors made by the
reference's own Python (tests/golden/make_atlas_golden.py, float64 autograd): the package's torch
restatement (photara_drender_gb300.atlas) and the oracle's chart-aware total-variation gradient, which
the refiner's TV kernel restates."""
import os

import numpy as np
import torch

from oracle import api
from photara_drender_gb300 import atlas

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "atlas_losses.npz")


def golden():
    return np.load(GOLDEN)


def test_total_variation_matches_reference():
    g = golden()
    for name, valid, chart in (("tv_all", None, None), ("tv_masked", g["valid"], g["chart"])):
        t = torch.tensor(g["tex"], requires_grad=True)
        loss = atlas.atlas_total_variation(t, valid_mask=None if valid is None else torch.tensor(valid),
                                           chart_ids=None if chart is None else torch.tensor(chart), epsilon=1e-4)
        loss.backward()
        assert abs(loss.item() - float(g[name + "_loss"])) <= 1e-14 * abs(float(g[name + "_loss"]))
        assert np.allclose(t.grad.numpy(), g[name + "_grad"], rtol=1e-12, atol=1e-15)


def test_masked_charbonnier_matches_reference():
    g = golden()
    r = torch.tensor(g["rendered"], requires_grad=True)
    loss = atlas.masked_charbonnier_loss(r, torch.tensor(g["target"]), torch.tensor(g["mask"]), epsilon=1e-3)
    loss.backward()
    assert abs(loss.item() - float(g["charbonnier_loss"])) <= 1e-14
    assert np.allclose(r.grad.numpy(), g["charbonnier_grad"], rtol=1e-12, atol=1e-15)


def test_oracle_tv_gradient_matches_reference():
    """ora_tv_gradient in float32 (the refiner's arithmetic) against the reference's float64 autograd:
    within 1e-5 of the largest component."""
    g = golden()
    tex32 = g["tex"].astype(np.float32)
    for name, valid, chart in (("tv_all", None, None), ("tv_masked", g["valid"], g["chart"])):
        grad, loss = api.tv_gradient(tex32, valid=None if valid is None else valid.astype(np.uint8),
                                     chart=chart, eps=1e-4, weight=1.0)
        ref = g[name + "_grad"]
        assert np.abs(grad - ref).max() <= 1e-5 * np.abs(ref).max(), name
        assert abs(loss - float(g[name + "_loss"])) <= 1e-6 * float(g[name + "_loss"])

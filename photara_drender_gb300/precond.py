"""Learned preconditioner for the atlas refiner (no counterpart in the reference).

A 16 -> 64 -> 64 -> 4 MLP (ReLU; BF16 weights and operands, FP32 accumulation on the tensor cores,
csrc/precond.cu) maps each texel's refine state to per-channel log step multipliers that scale the
Adam update of the photometric refinement. It is trained on trajectories of the plain refiner: for a
texel at step k, the target is log(clip(r, 1/8, 16)) with r = (theta_final - theta_k) /
(theta_{k+K} - theta_k), how many more K-step windows of plain progress the texel still needs.
During a learned run the multipliers are refreshed every K steps, and a rise of the windowed batch
loss switches the run back to plain Adam (decided on the device).

Features (csrc/precond.cu features_kernel): Adam direction, log magnitudes of both moments, the
texel value, observation weight, view count, a chart-edge distance proxy, schedule progress.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native
from .rasterizer import _ptr

PARAMS, IN, HIDDEN, OUT = 5508, 16, 64, 4
OFFSETS = dict(w1=0, b1=1024, w2=1088, b2=5184, w3=5248, b3=5504)
SHAPES = dict(w1=(64, 16), b1=(64,), w2=(64, 64), b2=(64,), w3=(4, 64), b3=(4,))
LOG_MIN, LOG_MAX = math.log(1.0 / 8.0), math.log(16.0)


class PrecondRunC(C.Structure):
    """pdr_precond_run (include/pdr_capi.h)."""
    _fields_ = [("params", C.c_void_p), ("params_bf16", C.c_void_p), ("observation", C.c_void_p),
                ("view_counts", C.c_void_p), ("edge_distance", C.c_void_p), ("features", C.c_void_p),
                ("multipliers", C.c_void_p), ("fallback", C.c_void_p), ("status", C.c_void_p),
                ("refresh_interval", C.c_uint32), ("fallback_tolerance", C.c_float)]


def _stream(dev):
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


class PrecondMLP:
    """The preconditioner network: FP32 master parameters plus the BF16 copy the tensor cores read."""

    def __init__(self, device_index: int = 0, seed: int = 0, params: Optional[np.ndarray] = None):
        self.device = torch.device("cuda", device_index)
        if params is None:
            g = torch.Generator().manual_seed(seed)
            p = torch.zeros(PARAMS)
            for name, fan_in, scale in (("w1", IN, 1.0), ("w2", HIDDEN, 1.0), ("w3", HIDDEN, 0.05)):
                bound = scale * math.sqrt(6.0 / fan_in)
                o, shape = OFFSETS[name], SHAPES[name]
                p[o:o + shape[0] * shape[1]] = (torch.rand(shape[0] * shape[1], generator=g) * 2 - 1) * bound
            params = p.numpy()
        params = np.asarray(params, dtype=np.float32).reshape(-1)
        if params.size != PARAMS:
            raise ValueError(f"preconditioner parameters must have {PARAMS} values")
        self.params = torch.tensor(params, device=self.device)
        self.bf16 = self.params.to(torch.bfloat16).contiguous()
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grads = torch.zeros_like(self.params)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        self.status = torch.zeros(_native.STATUS_WORDS, dtype=torch.int32, device=self.device)
        self.step = 0

    def state(self) -> np.ndarray:
        return self.params.cpu().numpy()

    def check_status(self) -> None:
        if int(self.status[_native.STATUS_PRECOND_TIMEOUT].item()):
            raise RuntimeError("a tensor-core wait of the preconditioner MLP timed out")

    def forward(self, features: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """features [n, 16] BF16 -> [n, 4] FP32."""
        if features.dtype != torch.bfloat16 or features.ndim != 2 or features.shape[1] != IN:
            raise ValueError("features must be a [n, 16] bfloat16 tensor")
        features = features.contiguous()
        n = features.shape[0]
        if out is None:
            out = torch.empty((n, OUT), dtype=torch.float32, device=self.device)
        _native.call("pdr_precond_forward", _ptr(self.params), _ptr(self.bf16), _ptr(features), n, _ptr(out),
                     _ptr(self.status), _stream(self.device))
        return out

    def gradient(self, features, targets, weights, inv_norm: Optional[float] = None) -> torch.Tensor:
        """Loss and gradient (into self.grads) of inv_norm * sum weights * (MLP(features) - targets)^2."""
        n = features.shape[0]
        if inv_norm is None:
            inv_norm = 1.0 / max(float(weights.sum().item()), 1.0)
        _native.call("pdr_precond_train_step", _ptr(self.params), _ptr(self.bf16), _ptr(features.contiguous()),
                     _ptr(targets.contiguous()), _ptr(weights.contiguous()), n, float(inv_norm), _ptr(self.grads),
                     _ptr(self.loss), _ptr(self.status), _stream(self.device))
        return self.loss

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        _native.call("pdr_precond_adam", _ptr(self.params), _ptr(self.grads), _ptr(self.m), _ptr(self.v), self.step,
                     lr, beta1, beta2, eps, _ptr(self.bf16), _stream(self.device))
        self.step += 1

    def fit(self, features, targets, weights, steps: int = 400, batch: int = 65536, lr: float = 2e-3,
            seed: int = 0) -> List[float]:
        """Minibatch Adam on the samples; returns the loss of every step."""
        n = features.shape[0]
        g = torch.Generator(device=self.device).manual_seed(seed)
        losses = []
        for s in range(steps):
            sel = torch.randint(0, n, (min(batch, n),), device=self.device, generator=g)
            f, t, w = features[sel], targets[sel], weights[sel]
            self.gradient(f, t, w)
            cos = 0.5 * (1.0 + math.cos(math.pi * s / steps))
            self.adam(lr * (0.1 + 0.9 * cos))
            losses.append(self.loss.clone())
        self.check_status()
        return [float(x.item()) for x in losses]


# ---- per-texel inputs ------------------------------------------------------------------------------

def atlas_layout(rasterizer, uv: torch.Tensor, indices: torch.Tensor, face_chart, height: int, width: int):
    """Valid mask (uint8) and chart id (int32, -1 outside) of every atlas texel from the UV layout."""
    dev = uv.device
    aclip = torch.cat([uv * 2.0 - 1.0, torch.zeros_like(uv[:, :1]), torch.ones_like(uv[:, :1])], 1).contiguous()
    araster, _ = rasterizer.forward(aclip, indices, (height, width), output_barycentric_derivatives=False)
    fid = araster[..., 3].long()
    valid = fid > 0
    chart = torch.as_tensor(np.asarray(face_chart), device=dev).to(torch.int64)
    charts = torch.where(valid, chart[(fid - 1).clamp(min=0)], torch.full_like(fid, -1)).to(torch.int32)
    return valid.to(torch.uint8).contiguous(), charts.contiguous()


@dataclass
class TexelStats:
    observation: torch.Tensor
    view_counts: torch.Tensor
    edge_distance: torch.Tensor


def texel_stats(state, valid: torch.Tensor, chart: Optional[torch.Tensor]) -> TexelStats:
    """Observation weight, view count and chart-edge distance of every texel of a prepared refinement."""
    o = state.options
    W, H = int(o.width), int(o.height)
    dev = state.init.device
    obs = torch.empty(H * W, dtype=torch.float32, device=dev)
    views = torch.empty_like(obs)
    edge = torch.empty_like(obs)
    scratch = torch.empty(H * W, dtype=torch.uint8, device=dev)
    _native.call("pdr_precond_texel_stats", C.addressof(state.table), len(state.weights), W, H, _ptr(valid),
                 _ptr(chart), _ptr(obs), _ptr(views), _ptr(edge), _ptr(scratch), _stream(dev))
    return TexelStats(obs, views, edge)


# ---- training data from plain trajectories ----------------------------------------------------------------

def _norm(state, step: int) -> float:
    o = state.options
    n = len(state.weights)
    bvw = 0.0
    for b in range(int(o.batch_size)):
        bvw += state.weights[(step * int(o.batch_size) + b) % n]
    return float(np.float32(1.0 / (bvw * 3.0))) if bvw > 0.0 else 0.0


def plain_trajectory_samples(state, stats: TexelStats, valid: torch.Tensor, interval: int = 25,
                             samples: int = 16384, seed: int = 0, min_progress: float = 1e-4):
    """Runs the plain refiner step by step on a prepared refinement, recording features and texel values
    of `samples` random valid texels every `interval` steps; returns (features [S*k, 16] BF16,
    targets [S*k, 4], weights [S*k, 4], final photometric batch loss)."""
    o = state.options
    dev = state.init.device
    s = _stream(dev)
    W, H = int(o.width), int(o.height)
    N = W * H
    L = _native.lib()
    tex = state.init.clone().contiguous()
    grad = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)  # the refiner's RGB + pad gradient
    m1 = torch.zeros_like(tex)
    m2 = torch.zeros_like(tex)
    steps = int(o.steps)
    loss = torch.zeros(steps, dtype=torch.float32, device=dev)
    g = torch.Generator(device=dev).manual_seed(seed)
    cand = torch.nonzero(valid.reshape(-1), as_tuple=False)[:, 0]
    pick = cand[torch.randint(0, cand.numel(), (min(samples, cand.numel()),), device=dev, generator=g)]
    feat = torch.empty((N, IN), dtype=torch.bfloat16, device=dev)
    snaps_f, snaps_x = [], []
    lr, bc1, bc2 = C.c_float(), C.c_float(), C.c_float()
    n = len(state.weights)
    for step in range(steps):
        if step % interval == 0:
            b1, b2 = (1.0, 1.0)
            if step > 0:
                _native.check(L.pdr_refine_schedule(C.addressof(o), step - 1, C.byref(lr), C.byref(bc1), C.byref(bc2)))
                b1, b2 = bc1.value, bc2.value
            _native.check(L.pdr_precond_features(_ptr(tex), _ptr(m1), _ptr(m2), b1, b2, float(o.adam_epsilon),
                                                 _ptr(stats.observation), _ptr(stats.view_counts),
                                                 _ptr(stats.edge_distance), step / steps, N, _ptr(feat), s))
            snaps_f.append(feat[pick].clone())
            snaps_x.append(tex.reshape(N, 3)[pick].clone())
        _native.check(L.pdr_refine_photometric(_ptr(tex), W, H, _ptr(state.table_dev), n, state.max_pixels, step,
                                               int(o.batch_size), float(o.photometric_epsilon), _norm(state, step),
                                               _ptr(grad), _ptr(loss), s))
        if float(o.tv_scale) > 0.0 and state.tv_valid is not None:
            _native.check(L.pdr_refine_total_variation(_ptr(tex), W, H, _ptr(state.tv_valid), _ptr(state.tv_chart),
                                                       float(o.tv_epsilon), float(o.tv_scale), _ptr(grad), s))
        _native.check(L.pdr_refine_schedule(C.addressof(o), step, C.byref(lr), C.byref(bc1), C.byref(bc2)))
        _native.check(L.pdr_refine_adam(_ptr(tex), _ptr(grad), _ptr(m1), _ptr(m2), N * 3, lr.value,
                                        float(o.adam_beta1), float(o.adam_beta2), float(o.adam_epsilon), bc1.value,
                                        bc2.value, float(o.clamp_min), float(o.clamp_max), s))
    final = tex.reshape(N, 3)[pick]
    feats, targets, weights = [], [], []
    for k in range(len(snaps_x) - 1):
        x0, x1 = snaps_x[k], snaps_x[k + 1]
        step_ = x1 - x0
        rem = final - x0
        moving = step_.abs() > min_progress
        r = torch.where(moving, rem / torch.where(moving, step_, torch.ones_like(step_)), torch.zeros_like(step_))
        t = torch.log(r.clamp(min=1.0 / 8.0, max=16.0))
        t = torch.where(r > 0, t, torch.full_like(t, LOG_MIN))
        feats.append(snaps_f[k])
        targets.append(torch.cat([t, torch.zeros_like(t[:, :1])], 1))
        weights.append(torch.cat([moving.float(), torch.zeros_like(t[:, :1])], 1))
    return (torch.cat(feats).contiguous(), torch.cat(targets).contiguous(), torch.cat(weights).contiguous(),
            float(loss[-1].item()))


# ---- learned refinement --------------------------------------------------------------------------------

def refine_learned(baker, state, mlp: PrecondMLP, stats: TexelStats, refresh_interval: int = 25,
                   fallback_tolerance: float = 0.02, use_graph: bool = True):
    """TextureBaker refinement of a prepared state with the learned multipliers:
    (color, loss_history, seam_loss_history, precompute_seconds, optimization_seconds, fell_back)."""
    o = state.options
    dev = state.init.device
    N = int(o.width) * int(o.height)
    feat = torch.empty((N, IN), dtype=torch.bfloat16, device=dev)
    mult = torch.zeros((N, OUT), dtype=torch.float32, device=dev)
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    run = PrecondRunC(_ptr(mlp.params), _ptr(mlp.bf16), _ptr(stats.observation), _ptr(stats.view_counts),
                      _ptr(stats.edge_distance), _ptr(feat), _ptr(mult), _ptr(flag), _ptr(mlp.status),
                      int(refresh_interval), float(fallback_tolerance))
    out = baker._refine_finish(state, use_graph, precond=run)
    mlp.check_status()
    return (*out, bool(flag.item()))


def photometric_loss(state, texture: torch.Tensor) -> float:
    """Masked Charbonnier loss of a texture over all cached views, each view weighted as one batch of the
    refiner (the refiner's per-step normalisation), averaged over views."""
    o = state.options
    dev = state.init.device
    W, H = int(o.width), int(o.height)
    n = len(state.weights)
    grad = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
    loss = torch.zeros(n, dtype=torch.float32, device=dev)
    s = _stream(dev)
    L = _native.lib()
    for k in range(n):
        w = state.weights[k]
        norm = float(np.float32(1.0 / (w * 3.0))) if w > 0 else 0.0
        _native.check(L.pdr_refine_photometric(_ptr(texture.contiguous()), W, H, _ptr(state.table_dev), n,
                                               state.max_pixels, k, 1, float(o.photometric_epsilon), norm, _ptr(grad),
                                               _ptr(loss), s))
    return float(loss.mean().item())

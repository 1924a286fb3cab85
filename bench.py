"""Benchmark: fwd+bwd Mpix/s of rasterize -> interpolate -> texture on the batched multi-view
workload (200k-triangle displaced sphere with packed chart UVs, 64 views at 1024x1024, 3-channel
vertex attributes, 4096x4096x4 fp32 atlas, N(0,1) upstream gradients; seeded synthetic data).

One step = the forward and backward pass over all 64 views. `value` is timed with CUDA events on
device-resident inputs; `e2e` runs the same pass through the public autograd API
(photara_drender_gb300.torch) with the inputs copied from pinned host memory and the gradients read
back every step. `--impl reference` times the CPU restatement of the reference (oracle/, all host
threads) on a bounded sample of the same workload.

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="c2_fwdbwd_200k_64x1024sq_atlas4096", triangles=200_000, views=64, height=1024, width=1024,
                attributes=3, atlas=4096, channels=4, seed=0)
METRIC = "fwd+bwd Mpix/s"


def scene(w=WORKLOAD):
    from photara_drender_gb300 import synthetic as S

    pos3, nrm, uv, idx, chart, remap = S.displaced_sphere(w["triangles"], seed=w["seed"], atlas_size=w["atlas"])
    mats, eyes = S.orbit_cameras(w["views"], radius=3.0, fov_y_deg=45.0, aspect=w["width"] / w["height"])
    rng = np.random.default_rng(w["seed"])
    attrs = rng.uniform(size=(pos3.shape[0], w["attributes"])).astype(np.float32)
    return pos3, uv, idx, mats, attrs


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.device_index = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---- CPU restatement (reference arm and cpu_baseline) -------------------------------------------------

def cpu_fwdbwd_sample(pos3, uv, idx, mats, attrs, tex, view: int, rng):
    """One view's forward + backward through the oracle, returns seconds."""
    from oracle import api

    w = WORKLOAD
    clip = api.transform_positions(pos3, mats[view])
    t0 = time.perf_counter()
    raster, deriv = api.rasterize_forward(clip, idx, (w["height"], w["width"]))
    a = api.interpolate_forward(attrs, idx, raster)
    u = api.interpolate_forward(uv, idx, raster)
    s = api.texture_forward(tex, u, raster)
    t1 = time.perf_counter()
    ga = rng.standard_normal(a.shape, dtype=np.float32)
    gs = rng.standard_normal(s.shape, dtype=np.float32)
    t2 = time.perf_counter()
    gt, gu = api.texture_backward(tex, u, raster, gs)
    guv, gr1 = api.interpolate_backward(uv, idx, raster, gu)
    gatt, gr2 = api.interpolate_backward(attrs, idx, raster, ga)
    gp = api.rasterize_backward(clip, idx, raster, gr1 + gr2)
    t3 = time.perf_counter()
    return (t1 - t0) + (t3 - t2)


def run_reference(args, world, rank):
    if rank != 0:
        return
    from oracle import api  # noqa: F401  (builds the oracle when needed)

    w = WORKLOAD
    pos3, uv, idx, mats, attrs = scene()
    rng = np.random.default_rng(1)
    tex = rng.uniform(size=(w["atlas"], w["atlas"], w["channels"])).astype(np.float32)
    cores = os.cpu_count() or 1
    for k in range(args.warmup):
        cpu_fwdbwd_sample(pos3, uv, idx, mats, attrs, tex, k % w["views"], rng)
    times = [cpu_fwdbwd_sample(pos3, uv, idx, mats, attrs, tex, k % w["views"], rng) for k in range(args.steps)]
    per_view = float(np.mean(times))
    mpix = w["height"] * w["width"] / 1e6 / per_view
    sample = (f"one of the {w['views']} views per step (view k mod {w['views']}), full forward+backward at "
              f"{w['height']}x{w['width']}; rasterize/interpolate/texture forward multi-threaded (OpenMP), adjoints "
              f"single-threaded as the reference's loops")
    line = {
        "metric": METRIC, "value": mpix, "unit": "Mpix/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_view * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": w["name"], "views": w["views"], "resolution": [w["height"], w["width"]],
                   "triangles": int(idx.shape[0]), "atlas": [w["atlas"], w["atlas"], w["channels"]],
                   "attributes": w["attributes"], "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": mpix, "unit": "Mpix/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": mpix, "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's Vulkan path cannot run here (no graphics stack); its shader arithmetic runs as "
                "the oracle's C restatement, pinned bit-exact to the reference shaders compiled for the CPU",
    }
    print(json.dumps(line), flush=True)


# ---- GPU arm ------------------------------------------------------------------------------------------

STAGES = ["bin_tiles", "rasterize_forward+shade", "render_backward"]


def stage_bytes(w, T, V, entries):
    """Algorithmic bytes per launch of each timed stage: API-boundary tensors, each read or written
    once (tile lists count for binning only, where they are the output)."""
    P = w["views"] * w["height"] * w["width"]
    A, Cc = w["attributes"], w["channels"]
    tex = w["atlas"] * w["atlas"] * Cc * 4
    mesh = w["views"] * V * 16 + T * 12
    tiles = w["views"] * ((w["height"] + 15) // 16) * ((w["width"] + 15) // 16)
    return {
        "bin_tiles": mesh + entries * 4 + (tiles + 1) * 4,
        # inputs: clip, indices, attributes, uv attributes, texture; outputs raster, derivatives,
        # attributes, uv, sampled
        "rasterize_forward+shade": mesh + V * (A + 2) * 4 + tex + P * (16 + 16 + A * 4 + 8 + Cc * 4),
        # inputs: raster, uv, grad_interpolated, grad_sampled, texture, clip, attributes;
        # outputs: grad_texture, grad_clip, grad_attributes, grad_uv_attributes
        "render_backward": P * (16 + 8 + A * 4 + Cc * 4) + 2 * tex + 2 * mesh + 2 * V * (A + 2) * 4,
    }


def run_gpu(args, world, rank, local):
    import torch

    from photara_drender_gb300 import Rasterizer, _native
    from photara_drender_gb300 import torch as pdr_torch
    from photara_drender_gb300.pipeline import RenderFwdBwd
    from photara_drender_gb300.rasterizer import _ptr

    w = WORKLOAD
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pos3, uv, idx, mats, attrs = scene()
    V, T = pos3.shape[0], idx.shape[0]
    views, H, W = w["views"], w["height"], w["width"]
    P = views * H * W
    r = Rasterizer(local)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    g = torch.Generator(device=dev)
    g.manual_seed(w["seed"] + rank)
    t_pos = torch.tensor(pos3, device=dev)
    t_mats = torch.tensor(mats, device=dev)
    clip = torch.empty((views, V, 4), dtype=torch.float32, device=dev)
    _native.call("pdr_transform_positions", _ptr(t_pos), V, _ptr(t_mats), views, _ptr(clip), stream)
    t_attrs = torch.tensor(attrs, device=dev)
    t_uv = torch.tensor(uv, device=dev)
    t_idx = torch.tensor(idx.astype(np.int32), device=dev)
    tex = torch.rand((w["atlas"], w["atlas"], w["channels"]), device=dev, generator=g)
    g_attr = torch.randn((views, H, W, w["attributes"]), device=dev, generator=g)
    g_samp = torch.randn((views, H, W, w["channels"]), device=dev, generator=g)

    pipe = RenderFwdBwd(r, t_idx, V, views, H, W, w["attributes"], tuple(tex.shape), capacity=4 * T * views)
    pipe.step(clip, t_attrs, t_uv, tex, g_attr, g_samp, stream)
    entries = pipe.check_capacity()
    if entries * 1.25 + 1024 < pipe.capacity:  # shrink the list to the measured need
        pipe = RenderFwdBwd(r, t_idx, V, views, H, W, w["attributes"], tuple(tex.shape),
                            capacity=int(entries * 1.25) + 1024)
    for _ in range(args.warmup):
        pipe.step(clip, t_attrs, t_uv, tex, g_attr, g_samp, stream)
    torch.cuda.synchronize(dev)
    pipe.check_capacity()

    # ---- timed region: device-resident inputs ------------------------------------------------------
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clocks:
        start.record()
        for _ in range(args.steps):
            pipe.step(clip, t_attrs, t_uv, tex, g_attr, g_samp, stream)
        end.record()
        torch.cuda.synchronize(dev)
    barrier(world)
    ms = start.elapsed_time(end) / args.steps
    pipe.check_capacity()
    ms = max_over_ranks(ms, world)
    value = world * P / 1e6 / (ms / 1e3)

    # ---- per-stage attribution: replay each stage between events --------------------------------
    L = _native.lib()
    reps = 3
    stage_ms = np.zeros(len(STAGES))
    a = pipe._args(clip, t_attrs, t_uv, tex, g_attr, g_samp)
    timed = [
        lambda: _native.check(L.pdr_bin_tiles(_ptr(clip), views, V, _ptr(pipe.idx), T, W, H, _ptr(pipe.vps),
                                              _ptr(pipe.offsets), _ptr(pipe.list), pipe.capacity, _ptr(pipe.ws),
                                              pipe.ws_bytes, _ptr(pipe.status), stream)),
        lambda: _native.check(L.pdr_render_forward(C.addressof(a), stream)),
        lambda: _native.check(L.pdr_render_backward(C.addressof(a), stream)),
    ]
    for _ in range(reps):
        for i, fn in enumerate(timed):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize(dev)
            stage_ms[i] += e0.elapsed_time(e1)
    stage_ms /= reps
    stage_ms[1] = max(stage_ms[1] - stage_ms[0], 1e-6)  # render_forward includes the binning
    hbm, peak_kind = load_peaks()
    sbytes = stage_bytes(w, T, V, entries)
    dom = int(np.argmax(stage_ms))
    dom_name = STAGES[dom]
    achieved = sbytes[dom_name] / (stage_ms[dom] / 1e3) / 1e9
    step_bytes = P * 96 + 2 * w["atlas"] ** 2 * w["channels"] * 4

    # ---- e2e: public autograd API with host buffers ---------------------------------------------------
    e2e_steps = 0 if args.skip_e2e else max(1, min(args.steps, 3))
    host = {k: v.cpu().pin_memory() for k, v in dict(clip=clip, attrs=t_attrs, uv=t_uv, tex=tex, g_attr=g_attr,
                                                     g_samp=g_samp).items()}
    h_idx = torch.tensor(idx.astype(np.int64)).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in host.values()) + h_idx.numel() * 8
    out_host = None

    def e2e_step():
        nonlocal out_host
        d = {k: v.to(dev, non_blocking=True) for k, v in host.items()}
        di = h_idx.to(dev, non_blocking=True)
        d_clip = d["clip"].requires_grad_(True)
        d_attrs = d["attrs"].requires_grad_(True)
        d_uv = d["uv"].requires_grad_(True)
        d_tex = d["tex"].requires_grad_(True)
        raster, _ = pdr_torch.rasterize(d_clip, di, (H, W), rasterizer=r)
        a = pdr_torch.interpolate(d_attrs, raster, di, rasterizer=r)
        u = pdr_torch.interpolate(d_uv, raster, di, rasterizer=r)
        s = pdr_torch.texture(d_tex, u, raster, rasterizer=r)
        torch.autograd.backward([a, s], [d["g_attr"], d["g_samp"]])
        outs = [d_clip.grad, d_attrs.grad, d_uv.grad, d_tex.grad]
        out_host = [o.to("cpu", non_blocking=True) for o in outs]
        return sum(o.numel() * o.element_size() for o in outs)

    e2e_value = e2e_ms = None
    d2h = 0
    if e2e_steps:
        d2h = e2e_step()
        torch.cuda.synchronize(dev)
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        torch.cuda.synchronize(dev)
        e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / e2e_steps, world)
        e2e_value = world * P / 1e6 / (e2e_ms / 1e3)

    # ---- CPU baseline (oracle restatement, bounded sample) --------------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        try:
            rng = np.random.default_rng(1)
            tex_h = tex.cpu().numpy()
            secs = cpu_fwdbwd_sample(pos3, uv, idx, mats, attrs, tex_h, 0, rng)
            cpu = {"value": H * W / 1e6 / secs, "unit": "Mpix/s", "cores": os.cpu_count() or 1, "kind": "port",
                   "sample": f"view 0 of {views}: full forward+backward at {H}x{W} through the oracle (forward "
                             f"stages OpenMP over all host threads, adjoint stages single-threaded), {secs:.2f} s"}
        except Exception as e:  # the CPU leg never hides a GPU result
            cpu = {"value": None, "unit": "Mpix/s", "cores": os.cpu_count() or 1, "kind": "port",
                   "sample": f"failed: {e}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded displaced sphere, orbit cameras)",
            "config": {"workload": w["name"], "views": views, "resolution": [H, W], "triangles": int(T),
                       "vertices": int(V), "atlas": [w["atlas"], w["atlas"], w["channels"]],
                       "attributes": w["attributes"], "tile_entries": entries,
                       "l2": "inputs larger than L2 (6.5 GB of per-view buffers per step)",
                       "parallelism": f"replicas x{world}"},
            "gpu_launches": pipe.kernels_per_step() * args.steps,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": hbm,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                         "algorithmic_bytes": sbytes[dom_name], "ms": float(stage_ms[dom])},
            "stages_ms": {n: float(t) for n, t in zip(STAGES, stage_ms)},
            "pipeline": "fused" if pipe.fused else "separate kernels",
            "step_roofline": {"algorithmic_bytes": step_bytes, "achieved_gbs": step_bytes / (ms / 1e3) / 1e9,
                              "frac": step_bytes / (ms / 1e3) / 1e9 / hbm},
            "e2e": {"value": e2e_value, "unit": "Mpix/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                    "api": "photara_drender_gb300.torch rasterize/interpolate/texture + autograd backward"},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU-baseline leg")
    ap.add_argument("--skip-e2e", action="store_true", help="omit the end-to-end leg (profiling runs)")
    ap.add_argument("--views", type=int, default=None, help="override the view count (small profiling cases)")
    args = ap.parse_args()
    if args.views:
        WORKLOAD["views"] = args.views
        WORKLOAD["name"] = WORKLOAD["name"].replace("64x", f"{args.views}x")
    if args.impl == "reference":
        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, world, rank)
        return
    import __graft_entry__ as g

    g.build()
    world, rank, local = dist_setup(args)
    run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()

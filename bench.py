#!/usr/bin/env python
"""Benchmark of SharpRay's render hot path on GB300: path samples/s at 1080p.

Workload (one step): the 1920x1080, 64 spp, depth-8, fog 0.02 scene (871,200-triangle fBm sphere
+ 64 instanced 5,000-triangle rocks, 2048x1024 HDR env, 512x512 albedo texture; seed 2), rendered
and composited (denoise + tonemap) once.  Synthetic seeded data stands in for the reference's
LFS-only assets.

Lines printed (rank 0, one JSON line):
* ours (default):   `value` = path samples/s with the scene resident in HBM and AOVs/image written
  to device memory (CUDA events on the launching stream); `e2e` = the same metric through the
  public render+compose call with host (pinned) outputs, D2H copies inside the timed region;
  `roofline` for the path-tracing kernel; `cpu_baseline` = the CPU oracle on a bounded row sample.
* --impl reference: the CPU restatement of the reference render path (the oracle; the C# reference
  cannot be built or run here: no .NET SDK/runtime on either machine) on all host cores.

Multi-GPU (torchrun): replicas only -- every rank renders its own full frame (weak scaling), no
data-path collective; the barrier and max-over-ranks timing use torch.distributed.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "path samples/s at 1080p (1920x1080, 64 spp, depth 8, fog)"
UNIT = "samples/s"
H2D_PARAM_BYTES = 48 + 32 + 44  # SrView + SrRenderParams + SrComposeParams per call


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the oracle sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--mode", type=int, default=0, help="render mode: 0 auto, 1 megakernel, 2 wavefront, 3 graph")
    ap.add_argument("--no-megakernel", action="store_true",
                    help="skip timing the megakernel render mode (one thread per pixel) among the render modes")
    ap.add_argument("--autotune-spp", type=int, default=8,
                    help="spp of the autotuner's trial renders at setup (0: default launch geometry)")
    ap.add_argument("--batch-autotune-spp", type=int, default=4,
                    help="autotune each batched scene with trial renders at this spp (0: defaults)")
    ap.add_argument("--batch-scenes", type=int, default=32,
                    help="scenes of the batched workload timed batched vs one after another (0: skip)")
    ap.add_argument("--adjoint-checks", type=int, default=64,
                    help="adjoint workload: texel channels checked by finite differences (-1: skip the workload)")
    ap.add_argument("--inverse-steps", type=int, default=200,
                    help="Adam steps of the inverse-rendering run (0: skip)")
    ap.add_argument("--c5-steps", type=int, default=0,
                    help="--adjoint-only: also time this many steps of the 16-view 768x768 differentiable workload")
    ap.add_argument("--c5-checkpoint-steps", type=int, default=0,
                    help="--adjoint-only with --c5-steps: also this many steps with path-vertex checkpointing")
    ap.add_argument("--joint-steps", type=int, default=0,
                    help="--adjoint-only: Adam steps recovering albedo, roughness and fog density jointly on a small "
                         "version of the 16-view workload")
    ap.add_argument("--joint-smooth", type=float, default=0.0,
                    help="--joint-steps: weight of a smoothness prior on both textures (0: none)")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the adjoint workload (--steps timed passes, --adjoint-checks FD checks)")
    ap.add_argument("--profile-once", action="store_true",
                    help="set up, render + compose exactly once, exit (for ncu captures)")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            j = json.loads(p.read_text())
            return float(j["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.lines, self.proc = device, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def aggregate(samples_per_rank_step: int, steps: int, world: int, rank_seconds: float, reduce_max=None) -> tuple:
    """Whole-job throughput of `world` replicas that each render `steps` frames: the slowest rank's
    time (max over ranks via `reduce_max`) over all ranks' samples.  Returns (value, seconds)."""
    t = reduce_max(rank_seconds) if (reduce_max is not None and world > 1) else rank_seconds
    return samples_per_rank_step * steps * world / t, t


def algorithmic_bytes(c: dict, pixels: int) -> int:
    """Bytes the reference algorithm must touch per render (data-structure sizes of the reference):
    32 B per BVH node test, 36 B per triangle test, 40 B per instance test, 108 B per inflated hit,
    48 B per bilinear material-texture sample (4 float3 texels), 48 B per environment radiance
    lookup (SkyTexture.Radiance: a bilinear sample of the env map), 4 B per CDF probe, 56 B AOV
    write per pixel."""
    return int(32 * (c["tlas_node"] + c["blas_node"]) + 36 * c["blas_shape"] + 40 * c["tlas_shape"]
               + 108 * c["hit_inflate"] + 48 * c["tex_sample"] + 48 * c["env_lookup"] + 4 * c["cdf_probe"]
               + 56 * pixels)


def traversal_bytes(c: dict) -> int:
    """The share of algorithmic_bytes that the traversal kernel touches: node, triangle and
    instance tests."""
    return int(32 * (c["tlas_node"] + c["blas_node"]) + 36 * c["blas_shape"] + 40 * c["tlas_shape"])


def oracle_bands(scene, view, params, threads: int, height: int, rows_per_band: int, bands: int = 16,
                 shift: int = 0, keep: bool = False):
    """Renders `bands` evenly spaced bands of `rows_per_band` image rows with the CPU oracle (a
    stratified sample of the frame: rows differ widely in cost, sky vs. geometry).  Returns the
    rows rendered, the seconds taken and (keep) the list of (y0, y1, radiance + fog radiance rows)."""
    r = max(1, min(rows_per_band, height // bands))
    spans = []
    for b in range(bands):
        y0 = int((b + 0.5) * height / bands) - r // 2 + shift * r
        y0 = max(0, min(height - r, y0))
        spans.append((y0, y0 + r))
    kept = []
    t0 = time.perf_counter()
    for y0, y1 in spans:
        a, _ = scene.render(view, params, threads, rows=(y0, y1))
        if keep:
            w = params.width
            kept.append((y0, y1, (a.radiance + a.radiance_fog)[y0 * w:y1 * w].copy()))
    return r * len(spans), time.perf_counter() - t0, kept


def band_parity(kept, frame) -> dict:
    """The GPU frame (radiance + fog radiance, pixels x 3) against the oracle's bands of the same
    frame: the project's image bar (relMSE < 1e-4, per-pixel relative error < 1e-3 on >= 99.5 %)."""
    import numpy as np
    w = None
    got, want = [], []
    for y0, y1, rows in kept:
        w = len(rows) // (y1 - y0)
        got.append(frame[y0 * w:y1 * w])
        want.append(rows)
    g, r = np.concatenate(got).astype(np.float64), np.concatenate(want).astype(np.float64)
    err = np.abs(g - r).max(axis=1) / np.maximum(np.abs(r).max(axis=1), 1e-3)
    rel = float(np.mean((g - r) ** 2 / (r ** 2 + 1e-2)))
    frac = float((err < 1e-3).mean())
    return {"pixels": int(len(err)), "rel_mse": rel, "frac_within_1e-3": frac,
            "pass": bool(rel < 1e-4 and frac >= 0.995),
            "bar": "relMSE < 1e-4 and per-pixel relative error < 1e-3 on >= 99.5 % of pixels"}


def cpu_oracle_sample(desc, target_s: float, threads: int):
    """Times the CPU oracle on a stratified row sample of the workload sized for ~target_s seconds;
    also returns the rows it rendered, for the parity check against the GPU frame."""
    from oracle import oracle
    from sharpray_gb300 import render_params
    scene = oracle.instantiate(desc)
    view, params = desc.view.to_c(), render_params(*desc.render_args())
    rows1, dt1, _ = oracle_bands(scene, view, params, threads, desc.height, 1)
    per_band = int(max(1, round(target_s / max(dt1, 1e-3))))
    rows, dt, kept = oracle_bands(scene, view, params, threads, desc.height, per_band, keep=True)
    samples = rows * desc.width * desc.spp
    return samples / dt, rows, dt, kept


def measure_batch(ctx, count: int, stream, sp, tune_spp: int = 0) -> dict:
    """The batched workload (synth.config_batch: `count` scenes of uneven size, resolution and spp)
    rendered by one sr_render_batch graph launch vs the same scenes one sr_render_device call
    after another on the same stream; both give bit-identical images (so equal relMSE)."""
    import ctypes as C

    import torch
    from sharpray_gb300 import _abi, render_batch, render_params, synth
    t0 = time.perf_counter()
    descs = synth.config_batch(count, seed=3)
    scenes, outs, params, views, keep = [], [], [], [], []
    for d in descs:
        sc = d.instantiate(ctx)
        sc.build()
        n = d.width * d.height
        dev = {k: torch.empty(n * c, dtype=torch.int32 if k == "samples" else torch.float32, device="cuda")
               for k, c in (("radiance", 3), ("radiance_fog", 3), ("normals", 3), ("uv", 2), ("depth", 1),
                            ("samples", 1), ("variance", 1))}
        keep.append(dev)
        scenes.append(sc)
        outs.append(_abi.SrAovs(*[dev[k].data_ptr() for k in ("radiance", "radiance_fog", "normals", "uv", "depth",
                                                               "samples", "variance")]))
        params.append(render_params(*d.render_args()))
        views.append(d.view)
    setup = time.perf_counter() - t0
    tuned, choices = 0, []
    t_tune = time.perf_counter()
    if tune_spp > 0:  # each scene's launch geometry from the autotuner (setup, untimed)
        for sc, d, p in zip(scenes, descs, params):
            t = sc.autotune(d.view, p, trial_spp=min(tune_spp, d.spp))
            tuned += int(t["ms"] < t["default_ms"])
            choices.append({"scene": f"{d.width}x{d.height} {d.spp} spp {d.triangle_count} tris",
                            "block": t["trace_block_threads"], "trace_per_sm": t["trace_blocks_per_sm"],
                            "fog_per_sm": t["fog_shade_blocks_per_sm"], "tail_divisor": t["tail_divisor"],
                            "gain": round(t["gain"], 4) if t["gain"] else None})
    tune_s = time.perf_counter() - t_tune
    samples = sum(d.width * d.height * d.spp for d in descs)
    lib = ctx._lib

    def plain():
        for sc, v, p, o in zip(scenes, views, params, outs):
            vc = v.to_c()
            _abi.check(lib.sr_render_device(sc.handle, C.byref(vc), C.byref(p), C.byref(o), sp))

    def plain_host_loop():  # one launch per bounce kernel, driven by the host
        for sc in scenes:
            sc.set_render_mode(_abi.SR_RENDER_WAVEFRONT)
        try:
            plain()
        finally:
            for sc in scenes:
                sc.set_render_mode(_abi.SR_RENDER_AUTO)

    def batch():
        render_batch(scenes, views, params, outs, stream=stream.cuda_stream)

    res = {}
    for label, fn in (("plain", plain), ("plain_host_loop", plain_host_loop), ("batched", batch)):
        fn()  # warm-up (builds the graphs)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(2):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        res[label] = a.elapsed_time(b) / 2 / 1000.0
    tris = [d.triangle_count for d in descs]
    return {"workload": f"{count} scenes (synth.config_batch, seed 3): triangles {min(tris)}-{max(tris)}, "
                        "256x256-1920x1080, 4/16/64 spp, depth 4-8, fog on half",
            "samples_per_step": samples, "unit": UNIT,
            "value": samples / res["batched"], "plain_value": samples / res["plain"],
            "plain_host_loop_value": samples / res["plain_host_loop"],
            "batched_ms": 1000 * res["batched"], "plain_ms": 1000 * res["plain"],
            "plain_host_loop_ms": 1000 * res["plain_host_loop"],
            "speedup": res["plain"] / res["batched"], "speedup_vs_host_loop": res["plain_host_loop"] / res["batched"],
            "setup_s": round(setup, 1),
            "autotuned_scenes": tuned if tune_spp > 0 else None,
            "autotune": {"trial_spp": tune_spp, "seconds": round(tune_s, 1), "choices": choices} if tune_spp > 0 else None,
            "note": "batched: one graph launch, one bounce loop per scene side by side; plain: one "
                    "graph-captured render per scene, back to back; plain_host_loop: one render per scene "
                    "with one launch per bounce kernel from the host; images bit-identical"}


def fp64_comparison(d, p, d_image, samples, grad_a, grad_r, threads: int = 0) -> dict:
    """The GPU's float gradients (albedo texture rgb, roughness texture channel 0) against the oracle's
    FP64 replay adjoint (oracle/sr_oracle.cpp, dual numbers through the reference's formulas) for the
    same dL/dI and sample counts: relative L2 error and the fraction of texel channels within 1e-3
    relative + 1e-4 of the largest."""
    import numpy as np
    from oracle import oracle
    t0 = time.perf_counter()
    o = oracle.instantiate(d)
    ta, tr = d.textures[1].texels.shape[:2], d.textures[2].texels.shape[:2]
    ga, gr, _, _ = o.adjoint(d.view.to_c(), p, d_image, samples, 1, ta, 2, tr, threads)
    out = {"seconds": round(time.perf_counter() - t0, 1)}
    for name, got, want in (("albedo", grad_a.reshape(-1), ga.reshape(-1)),
                            ("roughness", grad_r.reshape(-1, 3)[:, 0], gr.reshape(-1, 3)[:, 0])):
        got, want = got.astype(np.float64), want.astype(np.float64)
        scale = float(np.abs(want).max())
        ok = np.abs(got - want) <= 1e-3 * np.abs(want) + 1e-4 * scale
        out[name] = {"rel_l2": float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)),
                     "frac_within_1e-3": float(ok.mean())}
    out["bar"] = "relative L2 < 1e-3 and >= 99 % of texel channels within 1e-3 (+ 1e-4 of the largest)"
    return out


def measure_adjoint(checks: int, reps: int = 5, oracle_check: bool = True) -> dict:
    """The differentiable workload (synth.config_c4): forward render, then the path-replay adjoint of
    L = sum (I - T)^2 for the albedo texture (and, timed only, for the roughness texture), T rendered
    from the textures perturbed by N(0, 0.05).  grads/s = texel-channel gradients produced per second
    (the albedo texture's h x w x 3 per adjoint pass; h x w for the roughness).
    `checks` random (texel, channel) pairs that the image depends on are compared with central
    differences of L (h = 1e-3 and 2e-3, and the same texels at 1e-2; common random numbers through
    sr_scene_update_texture_device);
    a pair whose two differences disagree by > 2 % saw a roulette decision flip and is not scored."""
    import ctypes as C

    import torch
    import numpy as np
    from sharpray_gb300 import Context, _abi, adjoint_albedo, adjoint_texture, render_params, synth
    from sharpray_gb300.autograd import device_aovs
    d = synth.config_c4()
    ctx = Context(0)
    sc = d.instantiate(ctx)
    sc.build()
    tex_a, tex_r = sc._keepalive[0][1], sc._keepalive[0][2]
    p = render_params(*d.render_args())
    v = d.view.to_c()
    st = torch.cuda.Stream()
    sp = C.c_void_p(st.cuda_stream)
    bufs, aovs = device_aovs(d.width, d.height)
    lib = ctx._lib
    base_a = torch.from_numpy(d.textures[1].texels).cuda()
    base_r = torch.from_numpy(d.textures[2].texels).cuda()
    g = torch.Generator(device="cpu").manual_seed(4)
    st.wait_stream(torch.cuda.current_stream())  # the planes and base textures above

    def render():
        _abi.check(lib.sr_render_device(sc.handle, C.byref(v), C.byref(p), C.byref(aovs), sp))

    def image():
        return bufs["radiance"] + bufs["radiance_fog"]

    with torch.cuda.stream(st):
        noise = lambda t: (t + 0.05 * torch.randn(t.shape, generator=g).cuda()).clamp(0.0, 1.0)
        noise_a, noise_r = noise(base_a).contiguous(), noise(base_r).contiguous()
        sc.update_texture_device(tex_a, noise_a.data_ptr(), st.cuda_stream)
        sc.update_texture_device(tex_r, noise_r.data_ptr(), st.cuda_stream)
        render()
        target = image().clone()
        sc.update_texture_device(tex_a, base_a.data_ptr(), st.cuda_stream)
        sc.update_texture_device(tex_r, base_r.data_ptr(), st.cuda_stream)
        grad = torch.zeros_like(base_a)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        fwd_ms, adj_ms = [], []
        for i in range(reps + 1):
            ev[0].record(st)
            render()
            ev[1].record(st)
            d_img = 2.0 * (image() - target)
            grad.zero_()
            e2 = torch.cuda.Event(enable_timing=True)
            e2.record(st)
            adjoint_albedo(sc, d.view, p, aovs, d_img.data_ptr(), tex_a, grad.data_ptr(), None, st.cuda_stream)
            ev[2].record(st)
            st.synchronize()
            if i:  # the first pass is a warm-up
                fwd_ms.append(ev[0].elapsed_time(ev[1]))
                adj_ms.append(e2.elapsed_time(ev[2]))
        loss0 = float(((image().double() - target.double()) ** 2).sum())
        # the roughness texture's gradient (same replay, GGX / Smith derivatives; channel 0)
        grad_r = torch.zeros_like(base_r)
        rough_ms = []
        for i in range(reps + 1):
            grad_r.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            adjoint_texture(sc, d.view, p, aovs, d_img.data_ptr(), tex_r, grad_r.data_ptr(), _abi.SR_ADJOINT_ROUGHNESS,
                            None, st.cuda_stream)
            e1.record(st)
            st.synchronize()
            if i:
                rough_ms.append(e0.elapsed_time(e1))
        # the same albedo adjoint replayed one pixel per thread (the first form), for comparison
        sc.set_adjoint_replay(_abi.SR_ADJOINT_REPLAY_PIXEL)
        pixel_ms = []
        for i in range(reps + 1):
            grad.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            adjoint_albedo(sc, d.view, p, aovs, d_img.data_ptr(), tex_a, grad.data_ptr(), None, st.cuda_stream)
            e1.record(st)
            st.synchronize()
            if i:
                pixel_ms.append(e0.elapsed_time(e1))
        sc.set_adjoint_replay(_abi.SR_ADJOINT_REPLAY_WAVEFRONT)
        # all three gradients from one wavefront replay against the oracle's FP64 replay adjoint on the
        # same dL/dI and sample counts
        fp64 = None
        if oracle_check:
            ga, gr = torch.zeros_like(base_a), torch.zeros_like(base_r)
            vc = d.view.to_c()
            _abi.check(lib.sr_adjoint_all(sc.handle, C.byref(vc), C.byref(p), C.byref(aovs), C.c_void_p(d_img.data_ptr()),
                                          tex_a.id, C.c_void_p(ga.data_ptr()), tex_r.id, C.c_void_p(gr.data_ptr()), None,
                                          None, sp))
            st.synchronize()
            fp64 = fp64_comparison(d, p, d_img.cpu().numpy(), bufs["samples"].cpu().numpy().view(np.uint32),
                                   ga.cpu().numpy(), gr.cpu().numpy())
        grad.zero_()
        adjoint_albedo(sc, d.view, p, aovs, d_img.data_ptr(), tex_a, grad.data_ptr(), None, st.cuda_stream)
        st.synchronize()

        def fd_check(params, tgt, g_ad, seed, h0=1e-3):
            """Central differences of L (steps h0 and 2 h0) at `checks` random seen (texel, channel)
            pairs against g_ad."""
            def loss_at(y, x, c, delta):
                t = base_a.clone()
                t[y, x, c] += delta
                sc.update_texture_device(tex_a, t.data_ptr(), st.cuda_stream)
                _abi.check(lib.sr_render_device(sc.handle, C.byref(v), C.byref(params), C.byref(aovs), sp))
                return float(((image().double() - tgt.double()) ** 2).sum())

            seen = (g_ad.abs().sum(dim=2) > 0).nonzero().cpu().numpy()
            rng = np.random.default_rng(seed)
            picks = seen[rng.choice(len(seen), min(checks, len(seen)), replace=False)] if checks > 0 else []
            rel, skipped, floor_ok = [], 0, []
            gmax = float(g_ad.abs().max())
            for y, x in picks:
                c = int(rng.integers(3))
                fd = [(loss_at(y, x, c, h) - loss_at(y, x, c, -h)) / (2 * h) for h in (h0, 2 * h0)]
                if abs(fd[0] - fd[1]) > 0.02 * abs(fd[0]):
                    skipped += 1
                    continue
                err = abs(float(g_ad[y, x, c]) - fd[0])
                rel.append(err / max(abs(fd[0]), 1e-12))
                floor_ok.append(err <= 0.01 * abs(fd[0]) + 1e-3 * gmax)
            sc.update_texture_device(tex_a, base_a.data_ptr(), st.cuda_stream)
            return np.array(rel) if rel else np.zeros(0), skipped, floor_ok

        # steps h = 1e-3 and 2e-3 (the workload's specification), and the same texels at h = 1e-2:
        # the loss is a sum over float32 pixels, and a difference quotient carries their rounding
        # divided by 2h, while the image is close to linear in one albedo texel (little truncation
        # error at the larger step)
        rel_a, skipped, floor_ok = fd_check(p, target, grad, 4, h0=1e-3)
        rel_s, skipped_s, _ = fd_check(p, target, grad, 4, h0=1e-2)
        sc.update_texture_device(tex_a, base_a.data_ptr(), st.cuda_stream)
        st.synchronize()
    n_grad = base_a.numel()
    adj_s = statistics.median(adj_ms) / 1000.0
    fwd_s = statistics.median(fwd_ms) / 1000.0
    samples = d.width * d.height * d.spp
    return {"workload": f"{d.name}: {d.triangle_count} triangles, 512x512 albedo + roughness textures, depth 6, "
                        "L2 loss vs textures + N(0, 0.05)",
            "grads_per_s": n_grad / adj_s, "unit": "texel-channel gradients/s",
            "adjoint_ms": 1000 * adj_s, "forward_ms": 1000 * fwd_s,
            "roughness_adjoint_ms": statistics.median(rough_ms),
            "replay": "wavefront (the render's kernels recording vertices; swept at each sample's end)",
            "pixel_replay_adjoint_ms": statistics.median(pixel_ms),
            "wavefront_over_pixel_replay": statistics.median(pixel_ms) / (1000 * adj_s),
            "fp64_oracle": fp64,
            "roughness_grads_per_s": (n_grad // 3) / (statistics.median(rough_ms) / 1000.0),
            "replayed_samples_per_s": samples / adj_s, "forward_samples_per_s": samples / fwd_s,
            "loss": loss0, "fd_checked": len(rel_a), "fd_skipped_roulette_flip": skipped,
            "fd_rel_err_median": float(np.median(rel_a)) if len(rel_a) else None,
            "fd_rel_err_max": float(rel_a.max()) if len(rel_a) else None,
            "fd_within_1pct": float((rel_a <= 0.01).mean()) if len(rel_a) else None,
            "fd_within_1pct_or_1e-3_of_max": float(np.mean(floor_ok)) if floor_ok else None,
            "fd_h1e-2": {"checked": len(rel_s), "skipped": skipped_s,
                         "rel_err_median": float(np.median(rel_s)) if len(rel_s) else None,
                         "rel_err_max": float(rel_s.max()) if len(rel_s) else None,
                         "within_1pct": float((rel_s <= 0.01).mean()) if len(rel_s) else None},
            "note": "gradient w.r.t. the albedo texture; sampling, roulette decisions, pdfs and MIS detached "
                    "(path replay); FD: central, h = 1e-3 (and 2e-3 to screen roulette flips), common random numbers; "
                    "fd_h1e-2: the same texels at h = 1e-2, where the float32 rounding of the loss weighs 10x less"}


def measure_inverse(steps: int, views: int = 4, size: int = 256, spp: int = 8) -> dict:
    """Inverse rendering on the differentiable workload's scene (synth.config_c4 geometry, 512x512
    albedo texture): `views` orbit cameras (size x size, spp, depth 6) render targets with the true
    texture; starting from flat grey, `steps` Adam steps (lr 0.02, texels clamped to [0, 1]) through
    sharpray_gb300.autograd.render_albedo minimise the summed L2 image loss.  Reports the time per
    step (all views' forward renders and adjoints) and the texture RMSE on the texels the views see."""
    import torch
    from sharpray_gb300 import Context, Transform, View, render_params, synth
    from sharpray_gb300.autograd import render_albedo
    d = synth.config_c4(size, size, spp)
    ctx = Context(0)
    sc = d.instantiate(ctx)
    sc.build()
    tex = sc._keepalive[0][1]
    p = render_params(*d.render_args())
    cams = []
    for k in range(views):
        ang = 2.0 * math.pi * k / views
        pos = (2.9 * math.sin(ang), 0.4, -2.9 * math.cos(ang))
        cams.append(View(Transform(pos, synth.look_rotation(pos, (0.0, 0.0, 0.0))), d.view.fov, d.view.near))
    truth = torch.from_numpy(d.textures[1].texels).cuda()
    with torch.no_grad():
        targets = [render_albedo(sc, v, p, tex, truth).clone() for v in cams]
    x = torch.full_like(truth, 0.5).requires_grad_(True)
    opt = torch.optim.Adam([x], lr=0.02)

    def step():
        opt.zero_grad()
        loss = sum(((render_albedo(sc, v, p, tex, x) - t) ** 2).sum() for v, t in zip(cams, targets))
        loss.backward()
        opt.step()
        with torch.no_grad():
            x.clamp_(0.0, 1.0)
        return loss

    loss0 = float(step().detach())
    seen = x.grad.abs().sum(dim=2) > 0
    rmse = lambda: float(((x.detach() - truth)[seen] ** 2).mean()) ** 0.5
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps - 1):
        loss = step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    with torch.no_grad():
        final = float(sum(((render_albedo(sc, v, p, tex, x) - t) ** 2).sum() for v, t in zip(cams, targets)))
    rmse_start = float(((torch.full_like(truth, 0.5) - truth)[seen] ** 2).mean()) ** 0.5
    per_step = dt / max(steps - 1, 1)
    return {"workload": f"{views} orbit views {size}x{size}, {spp} spp, depth 6, {d.triangle_count} triangles, "
                        "512x512 albedo texture from flat grey",
            "steps": steps, "ms_per_step": 1000 * per_step, "texel_grads_per_s": truth.numel() / per_step,
            "path_samples_per_s": 2 * views * size * size * spp / per_step,
            "loss_start": loss0, "loss_final": final, "texture_rmse_start": rmse_start, "texture_rmse_final": rmse(),
            "seen_texels": int(seen.sum()),
            "note": "per step: every view rendered (forward) and replayed (adjoint) through the torch.autograd "
                    "wrapper; targets share the renderer's per-pixel random numbers"}


def measure_inverse_c5(steps: int, views: int = 16, size: int = 768, spp: int = 32, rings: int = 500,
                       tex: int = 1024, lr_tex: float = 0.02, lr_density: float = 0.002,
                       target_spp_factor: int = 4, form: str = "replay", smooth: float = 0.0) -> dict:
    """The batched + differentiable configuration (synth.config_c5: 16 orbit views, 768x768, 32 spp,
    depth 8, 500,000 triangles, 1024x1024 albedo + roughness textures, fog; smaller with the
    arguments): per step every view is rendered and its image gradient replayed once for the albedo
    texture, the roughness texture and the fog density together (sr_adjoint_all), then one Adam step
    updates all three (from flat grey textures and 1.5x the density).  The targets are rendered
    once at target_spp_factor x spp; every step renders with a fresh random-number stream and
    replays with another (sr_scene_set_seed), so that dL/dI and dI/dθ come from independent samples
    and the gradient is an unbiased estimate for the expected image.
    form "checkpoint" instead renders each view with sr_render_checkpointed (every sample's path
    vertices kept on the device) and sweeps them with sr_adjoint_checkpointed: no second traversal,
    at the memory of every sample's vertices, and dL/dI and dI/dθ from the same samples.
    `smooth` > 0 adds a smoothness prior to the loss: smooth x the summed squared differences of
    neighbouring texels (wrapping, as the textures repeat) of both textures.
    Reports the time per step after one warm-up step over `steps` timed steps, the vertex-record
    memory the form holds, and the texture errors (albedo rgb, roughness channel 0, on the
    well-observed texels) before and after."""
    import ctypes as C

    import numpy as np
    import torch
    from sharpray_gb300 import Context, Transform, View, _abi, render_params, synth
    from sharpray_gb300.autograd import device_aovs
    t_setup = time.perf_counter()
    d = synth.config_c5(size, size, spp, rings=rings, tex=tex)
    ctx = Context(0)
    ctx.set_bvh_build(_abi.SR_BVH_BUILD_DEVICE)
    sc = d.instantiate(ctx)
    sc.build()
    tex_a, tex_r = sc._keepalive[0][1], sc._keepalive[0][2]
    p = render_params(*d.render_args())
    cams = []
    for k in range(views):
        ang = 2.0 * math.pi * k / views
        pos = (2.9 * math.sin(ang), 0.4 + 0.6 * math.sin(3.0 * ang), -2.9 * math.cos(ang))
        cams.append(View(Transform(pos, synth.look_rotation(pos, (0.0, 0.0, 0.0))), d.view.fov, d.view.near).to_c())
    truth_a = torch.from_numpy(d.textures[1].texels).cuda()
    truth_r = torch.from_numpy(d.textures[2].texels).cuda()
    sigma = d.fog.density
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    bufs, aovs = device_aovs(d.width, d.height)
    lib = ctx._lib
    with torch.cuda.stream(st):
        def render(v):
            _abi.check(lib.sr_render_device(sc.handle, C.byref(v), C.byref(p), C.byref(aovs),
                                            C.c_void_p(st.cuda_stream)))
            return bufs["radiance"] + bufs["radiance_fog"]

        p_step = p
        p = render_params(d.width, d.height, d.block_size, spp * target_spp_factor, spp * target_spp_factor,
                          d.variance_threshold, d.bounces, d.indirect_clamp)
        targets = [render(v).clone() for v in cams]  # reference stream (seed 0), more samples
        p = p_step
        seed = [0]
        xa = torch.full_like(truth_a, 0.5).requires_grad_(True)
        xr = torch.full_like(truth_r, 0.5).requires_grad_(True)
        xs = torch.tensor([1.5 * sigma], device="cuda", requires_grad=True)
        opt = torch.optim.Adam([{"params": [xa, xr], "lr": lr_tex}, {"params": [xs], "lr": lr_density}])
        base_lr = [g["lr"] for g in opt.param_groups]
        losses = []
        n_step = [0]

        kept = [0]

        def step():
            seed[0] += 2
            sc.update_texture_device(tex_a, xa.detach().data_ptr(), st.cuda_stream)
            sc.update_texture_device(tex_r, xr.detach().data_ptr(), st.cuda_stream)
            sc.update_fog_density(float(xs.detach()))
            ga, gr, gs = torch.zeros_like(xa), torch.zeros_like(xr), torch.zeros_like(xs)
            loss = torch.zeros((), dtype=torch.float64, device="cuda")
            for v, t in zip(cams, targets):
                sc.set_seed(seed[0])  # the image and dL/dI from one stream ...
                if form == "checkpoint":  # ... and the gradient from the same samples
                    kb = C.c_uint64()
                    _abi.check(lib.sr_render_checkpointed(sc.handle, C.byref(v), C.byref(p), C.byref(aovs),
                                                          C.c_void_p(st.cuda_stream), C.byref(kb)))
                    kept[0] = kb.value
                    img = bufs["radiance"] + bufs["radiance_fog"]
                else:
                    img = render(v)
                diff = img - t
                loss += (diff.double() ** 2).sum()
                d_img = 2.0 * diff
                if form == "checkpoint":
                    sc.adjoint_checkpointed(d_img.data_ptr(), tex_a, ga.data_ptr(), tex_r, gr.data_ptr(),
                                            gs.data_ptr(), st.cuda_stream)
                    continue
                sc.set_seed(seed[0] + 1)  # ... the replay from another (every pixel takes spp samples)
                _abi.check(lib.sr_adjoint_all(sc.handle, C.byref(v), C.byref(p), C.byref(aovs),
                                              C.c_void_p(d_img.data_ptr()), tex_a.id, C.c_void_p(ga.data_ptr()),
                                              tex_r.id, C.c_void_p(gr.data_ptr()), C.c_void_p(gs.data_ptr()), None,
                                              C.c_void_p(st.cuda_stream)))
            if smooth > 0.0:  # gradient of the smoothness prior: 2 smooth (4 x - its four neighbours)
                for x, g, ch in ((xa, ga, slice(None)), (xr, gr, slice(0, 1))):
                    v = x.detach()[..., ch]
                    lap = 4.0 * v - (torch.roll(v, 1, 0) + torch.roll(v, -1, 0) + torch.roll(v, 1, 1) +
                                     torch.roll(v, -1, 1))
                    g[..., ch] += 2.0 * smooth * lap
            xa.grad, xr.grad, xs.grad = ga, gr, gs
            # cosine decay of the learning rates over the run: the gradients are Monte Carlo
            # estimates, and at a fixed rate Adam's normalised steps keep the texels moving by about
            # the rate per step on the noise alone
            decay = 0.5 * (1.0 + math.cos(math.pi * min(n_step[0], steps) / (steps + 1)))
            for g, lr0 in zip(opt.param_groups, base_lr):
                g["lr"] = lr0 * decay
            n_step[0] += 1
            opt.step()
            with torch.no_grad():
                xa.clamp_(0.0, 1.0)
                xr.clamp_(0.05, 1.0)
                xs.clamp_(1e-3, 1.0)
            losses.append(loss)

        try:
            step()  # warm-up
            st.synchronize()
            # well-observed texels: first-step gradient at least 5 % of the 99th percentile (texels
            # seen only at grazing angles or through reflections get weak, noisy gradients)
            ga0, gr0 = xa.grad.abs().sum(dim=2), xr.grad[..., 0].abs()
            seen_a = ga0 >= 0.05 * torch.quantile(ga0[ga0 > 0], 0.99)
            seen_r = gr0 >= 0.05 * torch.quantile(gr0[gr0 > 0], 0.99)
            rmse = lambda x, t, m: float(((x.detach() - t)[m] ** 2).mean()) ** 0.5
            rmse_start = (rmse(torch.full_like(truth_a, 0.5), truth_a, seen_a),
                          rmse(torch.full_like(truth_r, 0.5)[..., 0], truth_r[..., 0], seen_r))
            setup_s = time.perf_counter() - t_setup
            t0 = time.perf_counter()
            for _ in range(steps):
                step()
            st.synchronize()
            dt = (time.perf_counter() - t0) / max(steps, 1)
        finally:
            sc.set_seed(0)  # later users of the scene render from the reference's stream
            sc.release_checkpoint()
    n_grads = truth_a.numel() + truth_r.shape[0] * truth_r.shape[1] + 1
    samples = views * d.width * d.height * d.spp
    slots = ((d.width + 7) // 8) * ((d.height + 3) // 4) * 32
    # vertex records held: one sample per slot (replay) or every sample (checkpoint), 128 B each
    vertex_bytes = kept[0] if form == "checkpoint" else slots * (d.bounces + 1) * 128
    return {"workload": f"{views} orbit views {d.width}x{d.height}, {d.spp} spp, depth 8, "
                        f"{d.triangle_count} triangles, {tex}x{tex} albedo + roughness textures, fog 0.03",
            "form": form, "vertex_record_bytes": vertex_bytes,
            "timed_steps": steps, "ms_per_step": 1000 * dt, "texel_grads_per_s": n_grads / dt,
            "adam": {"lr_textures": lr_tex, "lr_density": lr_density, "schedule": "cosine decay to 0 over the run"},
            "smoothness_prior": smooth,
            "path_samples_per_s": samples * (1 if form == "checkpoint" else 2) / dt,
            "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
            "fog_density": {"true": sigma, "start": 1.5 * sigma, "after": float(xs.detach())},
            "albedo_rmse": {"start": rmse_start[0], "after": rmse(xa, truth_a, seen_a), "texels": int(seen_a.sum())},
            "roughness_rmse": {"start": rmse_start[1], "after": rmse(xr[..., 0], truth_r[..., 0], seen_r),
                               "texels": int(seen_r.sum())},
            "setup_s": round(setup_s, 1),
            "note": ("per step: each view rendered once with every sample's vertices kept "
                     "(sr_render_checkpointed, a fresh random-number stream) and its gradients swept from "
                     "them (sr_adjoint_checkpointed); targets at %dx the spp" if form == "checkpoint" else
                     "per step: each view rendered once (wavefront graph, a fresh random-number stream) and "
                     "replayed once for all three gradients (sr_adjoint_all, wavefront replay, an independent "
                     "stream); path_samples_per_s counts both passes; targets at %dx the spp") % target_spp_factor}


def run_reference(args):
    rank, _, world = dist_info()
    if rank != 0:
        return
    from oracle import oracle
    from sharpray_gb300 import render_params, synth
    desc = synth.config_c2(args.width, args.height, args.spp)
    threads = os.cpu_count() or 1
    scene = oracle.instantiate(desc)
    view, params = desc.view.to_c(), render_params(*desc.render_args())
    # calibrate a stratified row sample of ~2 s per step so the whole run stays within minutes
    rows1, dt1, _ = oracle_bands(scene, view, params, threads, desc.height, 1)
    per_band = int(max(1, round(2.0 / max(dt1, 1e-3))))
    for _ in range(args.warmup):
        oracle_bands(scene, view, params, threads, desc.height, 1)
    times, rows = [], 0
    for s in range(args.steps):
        rows, dt, _ = oracle_bands(scene, view, params, threads, desc.height, per_band, shift=s % 2)
        times.append(dt)
    samples = rows * desc.width * desc.spp * args.steps
    value = samples / sum(times)
    sample_desc = (f"{rows} image rows per step in 16 evenly spaced bands x {desc.width} px x {desc.spp} spp "
                   f"(of {desc.height} rows)")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded), CPU",
        "config": {"workload": desc.name, "width": desc.width, "height": desc.height, "spp": desc.spp,
                   "bounces": desc.bounces, "sample": sample_desc},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample_desc,
                         "note": "C++ restatement of the reference C# CPU path (oracle/); the C# reference "
                                 "cannot run here (no .NET SDK or runtime)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_ours(args):
    import ctypes as C

    import numpy as np
    import torch

    rank, local, world = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from sharpray_gb300 import Context, Compositor, _abi, render_params, synth
    from sharpray_gb300.api import Aovs

    t_setup = time.perf_counter()
    desc = synth.config_c2(args.width, args.height, args.spp)
    ctx = Context(local)
    ctx.set_bvh_build(_abi.SR_BVH_BUILD_DEVICE)  # bit-identical to the host build
    scene = desc.instantiate(ctx)
    scene.build()
    setup_s = time.perf_counter() - t_setup
    lib = ctx._lib
    W, H = desc.width, desc.height
    n = W * H
    view, params = desc.view.to_c(), render_params(*desc.render_args())
    comp = Compositor()
    cparams = comp.to_c()

    dev = {k: torch.empty(n * c, dtype=torch.float32 if k != "samples" else torch.int32, device="cuda")
           for k, c in [("radiance", 3), ("radiance_fog", 3), ("normals", 3), ("uv", 2), ("depth", 1),
                        ("samples", 1), ("variance", 1)]}
    rgb = torch.empty(n * 3, dtype=torch.uint8, device="cuda")
    aovs = _abi.SrAovs(*[dev[k].data_ptr() for k in ("radiance", "radiance_fog", "normals", "uv", "depth",
                                                      "samples", "variance")])
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = C.c_void_p(stream.cuda_stream)
    scene.set_render_mode(args.mode)

    def render():
        _abi.check(lib.sr_render_device(scene.handle, C.byref(view), C.byref(params), C.byref(aovs), sp))

    def compose():
        _abi.check(lib.sr_compose_device(ctx.handle, C.byref(aovs), W, H, C.byref(cparams),
                                         C.c_void_p(rgb.data_ptr()), sp))

    if args.profile_once:
        render()
        compose()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # BVH build of the largest mesh, host vs device (identical trees; setup, not in the metric)
    from sharpray_gb300 import Mesh
    tris = Mesh.triangles_from_corners(ctx, desc.meshes[0].positions, desc.meshes[0].uvs)
    pa, pb, pc = tris[:, 0:3], tris[:, 0:3] + tris[:, 3:6], tris[:, 0:3] + tris[:, 6:9]
    tb = np.concatenate([np.minimum(np.minimum(pa, pb), pc), np.maximum(np.maximum(pa, pb), pc)], 1)
    bvh_s = {"triangles": int(len(tris))}
    for where, label in ((_abi.SR_BVH_BUILD_HOST, "host"), (_abi.SR_BVH_BUILD_DEVICE, "device")):
        t0 = time.perf_counter()
        ctx.build_bvh(tb, 1.0, 0.5, 8, where=where)
        bvh_s[label + "_s"] = round(time.perf_counter() - t0, 4)

    # autotuner (setup, untimed): launch geometry of the wavefront kernels for this scene
    tuning = None
    if args.autotune_spp > 0 and args.mode in (0, 3):
        t0 = time.perf_counter()
        tuning = scene.autotune(desc.view, params, trial_spp=args.autotune_spp)
        tuning["trial_spp"] = args.autotune_spp
        tuning["seconds"] = round(time.perf_counter() - t0, 2)

    # work counters of one render (untimed) -> algorithmic bytes per launch
    scene.set_counting(True)
    render()
    torch.cuda.synchronize()
    counters = scene.counters()
    scene.set_counting(False)
    samples_per_step = counters["sample"]

    for _ in range(args.warmup):
        render()
        compose()
    torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for a, b, c in ev:
            a.record(stream)
            render()
            b.record(stream)
            compose()
            c.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if world > 1:
        torch.distributed.barrier()
    step_ms = [a.elapsed_time(c) for a, _, c in ev]
    render_ms = [a.elapsed_time(b) for a, b, _ in ev]

    def reduce_max(x: float) -> float:
        t = torch.tensor([x], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    value, total_s = aggregate(samples_per_step, args.steps, world, sum(step_ms) / 1000.0, reduce_max)

    # render modes on the same frame (identical images): the graph-captured device bounce loop
    # against the plain one-launch-per-bounce host loop, two renders each after a warm-up; the
    # megakernel (one thread per pixel) unless --no-megakernel
    variants = {}
    modes = ((2, "wavefront_host_loop"), (3, "wavefront_graph")) + (() if args.no_megakernel else ((1, "megakernel"),))
    for mode, label in modes:
        scene.set_render_mode(mode)
        render()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(2):
            render()
        b.record(stream)
        torch.cuda.synchronize()
        variants[label] = samples_per_step / (a.elapsed_time(b) / 2000.0)
    # the dominant kernel, the traversal, timed live: one host-loop render with a CUDA-event pair
    # around every bounce's traversal kernel on the render's stream
    trace_timing = None
    if args.mode in (0, 2, 3):
        scene.set_render_mode(2)
        scene.set_kernel_timing(True)
        render()
        torch.cuda.synchronize()
        trace_timing = scene.trace_time()
        scene.set_kernel_timing(False)
    scene.set_render_mode(args.mode)
    variants["graph_over_host_loop"] = variants["wavefront_graph"] / variants["wavefront_host_loop"]

    batched = None
    if args.batch_scenes > 0 and rank == 0:
        batched = measure_batch(ctx, args.batch_scenes, stream, sp, args.batch_autotune_spp)

    adjoint = None
    if args.adjoint_checks >= 0 and rank == 0:
        adjoint = measure_adjoint(args.adjoint_checks)
        if args.inverse_steps > 0:
            adjoint["inverse_rendering"] = measure_inverse(args.inverse_steps)

    # end to end through the public API with pinned host outputs
    host = Aovs(W, H)
    pinned = {}
    for k in ("radiance", "radiance_fog", "normals", "uv", "depth", "samples", "variance"):
        arr = getattr(host, k)
        t = torch.empty(arr.shape, dtype=torch.int32 if k == "samples" else torch.float32).pin_memory()
        pinned[k] = t
        setattr(host, k, t.numpy().view(arr.dtype))
    img_t = torch.empty((H, W, 3), dtype=torch.uint8).pin_memory()
    img = img_t.numpy()
    from sharpray_gb300 import render_compose
    render_compose(scene, desc.view, *desc.render_args(), comp, aovs=host, image=img)  # warm
    e2e_steps = max(1, args.e2e_steps)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        render_compose(scene, desc.view, *desc.render_args(), comp, aovs=host, image=img)
    e2e_value, e2e_s = aggregate(samples_per_step, e2e_steps, world, time.perf_counter() - t0, reduce_max)
    d2h = n * (12 + 12 + 12 + 8 + 4 + 4 + 4) + n * 3

    # kernels of one timed step: the render's own launches (reported by the library) + compose (2)
    info = scene.render_info()
    launches = (info["kernel_launches"] + 2) * args.steps
    peak, peak_kind = measured_peaks()
    alg = algorithmic_bytes(counters, n)
    kern_s = statistics.mean(render_ms) / 1000.0
    achieved = alg / kern_s / 1e9
    traffic, trace_traffic, trace_ncu_launches = None, None, None
    tf = ROOT / "profiles" / "path_tracer_c2_traffic.json"
    if tf.exists() and (W, H, desc.spp) == (1920, 1080, 64):
        try:
            tj = json.loads(tf.read_text())
            traffic = tj.get("traffic_bytes_per_frame")
            trace_traffic = tj.get("trace_traffic_bytes_per_frame")
            trace_ncu_launches = tj.get("trace_launches")
        except Exception:
            traffic = None
    # roofline of the traversal kernel: the reference's bytes for its work (node, triangle and
    # instance tests) per launch over its average launch time
    trace_roof = None
    if trace_timing and trace_timing["launches"] > 0:
        nl = trace_timing["launches"]
        trace_alg = traversal_bytes(counters)
        trace_s = trace_timing["total_ms"] / 1000.0
        trace_ach = trace_alg / trace_s / 1e9
        trace_roof = {"bound": "hbm", "achieved": trace_ach, "peak": peak, "unit": "GB/s", "frac": trace_ach / peak,
                      "traffic": trace_traffic / trace_ncu_launches if trace_traffic and trace_ncu_launches else None,
                      "kernel": "k_wave_trace (persistent traversal: path rays + shadow rays of a bounce)",
                      "launches": nl, "kernel_ms_per_launch": trace_timing["total_ms"] / nl,
                      "alg_bytes_per_launch": trace_alg / nl, "peak_source": peak_kind,
                      "note": "timed live with CUDA events around each traversal launch of a host-loop render "
                              "of the same frame; alg bytes 32 per node test, 36 per triangle test, 40 per "
                              "instance test from the kernels' work counters; traffic per launch from the ncu "
                              "launch list of the same frame"}

    cpu, parity = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, rows, dt, kept = cpu_oracle_sample(desc, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{rows} rows in 16 evenly spaced bands x {W} px x {desc.spp} spp of the same frame "
                         f"({dt:.1f} s)"}
        # the timed frame (AOVs of the last render; every render of this scene is the same) against
        # the oracle's rows of it
        frame = (dev["radiance"] + dev["radiance_fog"]).view(-1, 3).cpu().numpy()
        parity = band_parity(kept, frame)
        parity["sample"] = cpu["sample"]

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generators; reference assets are LFS pointers)",
            "config": {"workload": desc.name, "width": W, "height": H, "spp": desc.spp, "bounces": desc.bounces,
                       "fog_density": 0.02, "triangles": desc.triangle_count, "instances": len(desc.objects) - 1,
                       "env": "2048x1024", "step": "render + compose (denoise, fog blur, tonemap)",
                       "l2": "inputs larger than L2: scene ~%.0f MB + AOVs %.0f MB resident" % (
                           (desc.triangle_count * 192 + 2048 * 1024 * 24) / 1e6, n * 56 / 1e6),
                       "parallelism": "replicas" if world > 1 else "single", "setup_s": round(setup_s, 2),
                       "bvh_build": bvh_s,
                       "wall_s_timed": round(wall, 3)},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": H2D_PARAM_BYTES,
                    "d2h_bytes_per_step": d2h},
            "roofline": trace_roof or {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                       "frac": achieved / peak, "traffic": traffic, "kernel": "frame"},
            "roofline_frame": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": ("path tracer: k_render_pixels" if args.mode == 1 else
                                    "path tracer: k_wave_trace/finalize(late)/shade(fog,miss,surface)/finalize "
                                    "+ k_wave_tail (one frame)"),
                         "kernel_ms": 1000 * kern_s, "alg_bytes_per_launch": alg, "peak_source": peak_kind,
                         "note": "per frame of the path tracer; alg bytes from the kernels' own work "
                                 "counters sized by the reference's records"},
            "cpu_baseline": cpu,
            "parity_vs_oracle": parity,
            "gpu_launches": launches,
            "render_mode": {0: "auto (wavefront graph)", 1: "megakernel", 2: "wavefront host loop",
                            3: "wavefront graph"}[args.mode],
            "variants_samples_per_s": variants,
            "batched": batched,
            "autotune": tuning,
            "adjoint": adjoint,
            "clocks": clocks.summary(),
            "counters_per_step": counters,
            # closest-hit + shadow queries per second (SceneTrace + SceneOcclude counters)
            "rays_per_s": (counters["scene_trace"] + counters["scene_occlude"]) * value / max(1, samples_per_step),
            "bounce_iterations": info["bounce_iterations"],
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.adjoint_only:
        adj = measure_adjoint(max(args.adjoint_checks, 0), reps=max(args.steps, 1))
        if args.inverse_steps > 0:
            adj["inverse_rendering"] = measure_inverse(args.inverse_steps)
        if args.c5_steps > 0:
            adj["batched_differentiable"] = measure_inverse_c5(args.c5_steps)
            if args.c5_checkpoint_steps > 0:
                adj["batched_differentiable_checkpoint"] = measure_inverse_c5(args.c5_checkpoint_steps,
                                                                              form="checkpoint")
        if args.joint_steps > 0:  # the same pipeline small enough to run to convergence
            adj["joint_recovery"] = measure_inverse_c5(args.joint_steps, views=4, size=192, spp=8, rings=150,
                                                       tex=128, lr_tex=0.005, lr_density=0.001, target_spp_factor=8,
                                                       smooth=args.joint_smooth)
        print(json.dumps({"adjoint": adj}), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

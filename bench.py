#!/usr/bin/env python3
"""Throughput of the GB300 raycaster on the raycaster workload, printed as one JSON line.

Workload (the reference publishes no benchmark; seeded synthetic input): a subdivided
icosphere of 1,310,720 triangles radially displaced by 3-octave value noise (amplitude
0.1) and 16,777,216 rays with origins uniform in a box 3x the mesh bounds and directions
uniform on the sphere. One step = one closest-hit query (Raycaster::intersects) over all
16M rays; the any-hit query (Raycaster::intersectsAny) is timed the same way and reported
beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* value     -- Mrays/s, rays resident in HBM, CUDA events on the launching stream.
* e2e       -- Mrays/s through the public API with host (pinned) buffers: host->device copy
               of the rays and device->host copy of the hits inside the timed region.
* roofline  -- the traversal kernel against the measured HBM bandwidth; algorithmic bytes
               per ray = 32 (ray) + 16 (hit) + 128 x 4-wide nodes visited + 48 x triangles
               tested, visit counts measured on a 1M-ray sample of the same set.
* cpu_baseline -- the C restatement of the reference Raycaster (oracle/port), reference
               threading (hardware threads - 1), on a bounded sample of the same rays.
* pathtracer -- the path tracer on the small (Cornell room, 256x256, 16 spp, depth 5) and
               large (200 instances, ~2M triangles, 1920x1080, 64 spp, depth 8) scenes:
               Mrays/s counting primary, bounce and shadow rays, device time inside
               pt_render, beside the C restatement of PathTracer::render on host cores.
* batch    -- 64 seeded jobs (10k-500k triangles, 128^2-1024^2, 4-256 spp, depth 3-10) in
               one batched call (one CUDA graph launch looping over the waves, autotuned), vs the same
               jobs rendered one call after another.
* denoiser -- the learned denoiser (BF16 tensor-core U-Net) trained on path-tracer pairs:
               inference TFLOP/s at 1920x1080 against the BF16 peak, training-step
               throughput, and plain vs denoised path tracing at equal time (relative RMSE
               against a 4096-spp render of a held-out scene).
* --impl reference -- only that CPU path, as the reference arm.
Under torchrun (N > 1) every rank traces its own 16M rays (weak scaling, no collective on
the data path); value = all rays / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SUBDIV = 8
N_RAYS = 1 << 24
SEED = 20261204
WORKLOAD = ("raycaster: displaced icosphere, 1,310,720 triangles; 16,777,216 rays, origins uniform in 3x bounds, "
            "directions uniform on the sphere; closest hit per step")


def _config(triangles: int, rays: int, world: int) -> dict:
    """The workload description both arms print (identical keys and values)."""
    return {"workload": WORKLOAD, "triangles": triangles, "rays_per_gpu": rays,
            "l2": "inputs larger than L2 (512 MB of rays per step)", "parallelism": f"replicas x{world}"}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[3 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    """Process group of a torchrun launch (NCCL on GPUs, gloo without), or None for one
    process: (dist, rank, world size)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return dist, dist.get_rank(), ws
    return None, 0, 1


def _device_of(dist, torch):
    return "cuda" if (dist is None or dist.get_backend() == "nccl") and torch.cuda.is_available() else "cpu"


def _sync_all(dist, torch):
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
        if torch.cuda.is_available():
            torch.cuda.synchronize()


def _max_over_ranks(dist, torch, v: float) -> float:
    if dist is None:
        return v
    t = torch.tensor([v], dtype=torch.float64, device=_device_of(dist, torch))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _rank_seed(seed: int, rank: int) -> int:
    """Each rank's own rays (weak scaling: fixed work per GPU, no data exchanged)."""
    return seed + 1000 * rank


def _job_rate(dist, torch, local_units: float, local_s: float) -> float:
    """Whole-job throughput: the units of every rank over the slowest rank's time."""
    total = local_units
    if dist is not None:
        t = torch.tensor([local_units], dtype=torch.float64, device=_device_of(dist, torch))
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        total = float(t.item())
    return total / _max_over_ranks(dist, torch, local_s)


def cpu_raycaster_rate(mesh, rays, target_s: float, threads: int):
    """The C restatement of Raycaster on host cores: Mrays/s on a sample sized to run
    about target_s seconds. Returns (Mrays_per_s, sample_rays, build_s)."""
    from oracle import oracle as O

    O.build_port()
    port = O.PortRaycaster()
    port.add_mesh(mesh.positions, mesh.indices)
    t0 = time.perf_counter()
    port.build()
    build_s = time.perf_counter() - t0
    probe = min(len(rays), 1 << 18)
    t0 = time.perf_counter()
    port.intersect(rays[:probe], threads=threads)
    dt = max(time.perf_counter() - t0, 1e-6)
    m = int(min(len(rays), max(probe, probe * target_s / dt)))
    t0 = time.perf_counter()
    port.intersect(rays[:m], threads=threads)
    dt = time.perf_counter() - t0
    return m / dt / 1e6, m, build_s


PT_CONFIGS = {
    # name: (scene factory, width, height, spp, depth, cpu spp, estimator)
    #   estimator 0 = the reference's (PathTracer::render), 1 = extended (NEE on the emissive
    #   quads and the importance-sampled environment map, MIS) as the large workload asks.
    "cornell_256": ("cornell", 256, 256, 16, 5, 16, 0),
    "instanced_1080p": ("instanced", 1920, 1080, 64, 8, 4, 1),
    "instanced_1080p_reference_estimator": ("instanced", 1920, 1080, 64, 8, 4, 0),
}


def _pt_scene(kind):
    from rendu_gb300 import scenes as S

    return S.cornell_scene(20261204) if kind == "cornell" else S.instanced_scene(20261206)


def _profile_traffic(path: str) -> dict:
    """Per-kernel-class figures from a committed ncu summary: lines
    `traffic_bytes_per_launch <class>: <bytes>` (DRAM read + write of one launch, ncu) and
    `launches_per_render <class>: <n>` (the launch list)."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", path)) as f:
            for ln in f:
                for key in ("traffic_bytes_per_launch", "launches_per_render"):
                    if ln.startswith(key + " "):
                        k, v = ln[len(key) + 1:].split(":")
                        out.setdefault(k.strip(), {})[key] = float(v)
    except OSError:
        pass
    return out


def pt_kernel_rooflines(st: dict, prof: dict) -> dict:
    """Roofline of each path-tracer kernel class from a profiled render's per-kernel CUDA-event
    times: achieved = the kernel's algorithmic DRAM bytes (the streams it must read and write,
    counted per ray from the render's ray counts) / its time, against the measured HBM copy
    bandwidth. Node, triangle, attribute and texel fetches are not counted: they are gathers
    served mostly by L1/L2, which is what bounds these kernels.
      trace  (k_trace_batch): per path ray 32 B ray + 4 B path id + 4 B job id + 16 B hit
      shade  (k_shade): per shaded ray 32 B ray + 4 B path id + 16 B hit + 2 x 16 B path
             throughput and radiance + 4 B job + 8 B pixel/sample + 8 B screen position read,
             2 x 16 B written; + 36 B per next ray and 48 B per shadow ray queued
      shadow (k_shadow): per shadow ray 32 B ray + 16 B contribution + 16 B radiance read and
             written"""
    peak, kind = _peaks()
    rays = st["primary_rays"] + st["bounce_rays"]
    algo = {"trace": 56 * rays, "shade": 136 * rays + 36 * st["bounce_rays"] + 48 * st["shadow_rays"],
            "shadow": 80 * st["shadow_rays"]}
    total_ms = sum(st["kernel_ms"].values())
    out = {}
    for k, b in algo.items():
        ms = st["kernel_ms"][k]
        if ms <= 0:
            continue
        gbs = b / (ms * 1e-3) / 1e9
        p = prof.get(k, {})
        n = int(p.get("launches_per_render", 0)) or None
        tr = p.get("traffic_bytes_per_launch")
        out[k] = {"ms": round(ms, 3), "share": round(ms / total_ms, 3), "launches": n,
                  "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
                  "peak_kind": kind, "bound": "hbm", "algorithmic_bytes": int(b),
                  "traffic": tr, "dram_gbs": round(tr * n / (ms * 1e-3) / 1e9, 1) if tr and n else None}
    return out


def run_pathtracer(name, steps, cpu: bool):
    """One path-tracer configuration: GPU Mrays/s (device time inside pt_render), e2e with a
    host image, and the C restatement on host cores at `cpu spp` (cost is linear in spp)."""
    import torch

    import rendu_gb300 as R

    kind, w, h, spp, depth, cpu_spp, mode = PT_CONFIGS[name]
    sc = _pt_scene(kind)
    cam = dict(sc.camera, ratio=w / h)
    t0 = time.perf_counter()
    tr = R.PathTracer(sc)
    commit_s = time.perf_counter() - t0
    img = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
    tr.render(cam, spp, depth, img, seed=1, mode=mode)  # warm-up
    rays, dev_ms = 0, 0.0
    for k in range(steps):
        img.zero_()
        tr.render(cam, spp, depth, img, seed=2 + k, mode=mode)
        st = tr.last_stats()
        rays += st["rays"]
        dev_ms += st["device_ms"]
    # e2e: the image in host memory (copied in, rendered into, copied out every call), after
    # one warm-up call of that path; wall time per render over `steps` renders
    host = np.zeros((h, w, 3), np.float32)
    tr.render(cam, spp, depth, host, seed=98, mode=mode)
    e2e_rays, t0 = 0, time.perf_counter()
    for k in range(steps):
        tr.render(cam, spp, depth, host, seed=99 + k, mode=mode)
        e2e_rays += tr.last_stats()["rays"]
    e2e_s = (time.perf_counter() - t0) / steps
    e2e_rays //= steps
    # per-kernel times: one more render with the kernels launched directly, events between them
    img.zero_()
    tr.render(cam, spp, depth, img, seed=2, mode=mode, profile=True)
    pst = tr.last_stats()
    kernels = pt_kernel_rooflines(pst, _profile_traffic(f"pathtracer_{name}.txt"))
    out = {"workload": f"{kind}: {sc.triangle_count} triangles, {len(sc.objects)} objects, {w}x{h}, {spp} spp, "
                       f"depth {depth}, {'extended' if mode else 'reference'} estimator",
           "value": round(rays / (dev_ms * 1e3), 1), "unit": "Mrays/s", "ms_per_render": round(dev_ms / steps, 2),
           "rays_per_render": rays // steps, "e2e": {"value": round(e2e_rays / e2e_s / 1e6, 1), "unit": "Mrays/s",
                                                      "s_per_render": round(e2e_s, 5)},
           "scene_upload_and_build_s": round(commit_s, 2),
           "roofline": dict(kernels.get("trace", {}), kernel="k_trace_batch"), "kernels": kernels,
           "profiled_render_ms": round(pst["device_ms"], 2)}
    if cpu:
        from oracle import oracle as O

        O.build_port()
        threads = max((os.cpu_count() or 2) - 1, 1)
        port = O.PortPathTracer(sc)
        t0 = time.perf_counter()
        port.render(cam, cpu_spp, depth, w, h, seed=1, threads=threads, mode=mode)
        dt = time.perf_counter() - t0
        cpu_rays = int(port.rays.sum())
        cpu_rate = cpu_rays / dt / 1e6
        out["cpu_baseline"] = {"value": round(cpu_rate, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                               "sample": f"full image at {cpu_spp} spp (cost linear in spp)",
                               "render_s_at_full_spp": round(dt * spp / cpu_spp, 1)}
        out["speedup_vs_cpu"] = round(out["value"] / cpu_rate, 1)
    return out


def run_batch(cpu: bool, tune: bool = True):
    """Batched rendering: 64 seeded jobs (10k-500k triangles, 128^2-1024^2, 4-256 spp,
    depth 3-10) in one pt_batch_render call (one CUDA graph launch looping over the waves, autotuned
    tuning), against the same jobs rendered one pt_render call after another."""
    import torch

    import rendu_gb300 as R
    from rendu_gb300 import scenes as S

    wl = S.batch_workload()
    t0 = time.perf_counter()
    tracers = [R.PathTracer(j["scene"]) for j in wl]
    upload_s = time.perf_counter() - t0
    jobs = []
    for j, tr in zip(wl, tracers):
        jobs.append({"tracer": tr, "camera": dict(j["scene"].camera, ratio=1.0), "samples": j["samples"],
                     "depth": j["depth"], "seed": j["seed"],
                     "image": torch.zeros((j["height"], j["width"], 3), dtype=torch.float32, device="cuda")})
    br = R.BatchRenderer(0)
    tuning, tune_s = None, 0.0
    if tune:
        t0 = time.perf_counter()
        # an optional tuning cache shared between runs (RENDU_TUNING_CACHE=path)
        tuning = br.autotune(jobs, cache_path=os.environ.get("RENDU_TUNING_CACHE") or None)
        tune_s = time.perf_counter() - t0
    br.render(jobs, tuning=tuning)  # warm-up (graph capture)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = br.render(jobs, tuning=tuning)
    torch.cuda.synchronize()
    batch_s = time.perf_counter() - t0
    pst = br.render(jobs, tuning=tuning, profile=True)  # per-kernel times (kernels launched directly)
    kernels = pt_kernel_rooflines(pst, _profile_traffic("pathtracer_batch_64.txt"))
    seq_ms, seq_rays = 0.0, 0
    t0 = time.perf_counter()
    for j in jobs:
        j["tracer"].render(j["camera"], j["samples"], j["depth"], j["image"], seed=j["seed"])
        s1 = j["tracer"].last_stats()
        seq_ms += s1["device_ms"]
        seq_rays += s1["rays"]
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t0
    out = {"workload": f"{len(jobs)} jobs, {sum(j['scene'].triangle_count for j in wl)} triangles in total, "
                       f"{sum(j['width'] * j['height'] for j in wl)} pixels, "
                       f"{sum(j['width'] * j['height'] * j['samples'] for j in wl)} paths",
           "value": round(st["rays"] / (st["device_ms"] * 1e3), 1), "unit": "Mrays/s",
           "batch_device_ms": round(st["device_ms"], 1), "batch_wall_s": round(batch_s, 3),
           "sequential_device_ms": round(seq_ms, 1), "sequential_wall_s": round(seq_s, 3),
           "speedup_vs_sequential": round(seq_s / batch_s, 2), "rays": st["rays"], "tuning": tuning,
           "autotune_s": round(tune_s, 1), "scene_uploads_s": round(upload_s, 2),
           "roofline": dict(kernels.get("trace", {}), kernel="k_trace_batch"), "kernels": kernels,
           "profiled_render_ms": round(pst["device_ms"], 1)}
    if cpu:
        from oracle import oracle as O

        O.build_port()
        threads = max((os.cpu_count() or 2) - 1, 1)
        rays, dt = 0, 0.0
        for j in wl[:8]:  # bounded sample: the first 8 jobs at 1 spp
            port = O.PortPathTracer(j["scene"])
            t0 = time.perf_counter()
            port.render(dict(j["scene"].camera, ratio=1.0), 1, j["depth"], j["width"], j["height"], seed=1,
                        threads=threads)
            dt += time.perf_counter() - t0
            rays += int(port.rays.sum())
        out["cpu_baseline"] = {"value": round(rays / dt / 1e6, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                               "sample": "first 8 jobs at 1 spp"}
        out["speedup_vs_cpu"] = round(out["value"] / out["cpu_baseline"]["value"], 1)
    return out


def _bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured (burst)"
    except Exception:
        return 1900.0, "fallback"


def _events_ms(fn, iters):
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(iters):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / iters


# The learned denoiser's protocol (scaled down from 20k 512^2 crops with 1024-spp targets:
# the whole measurement has to fit in a bench run of a few minutes).
DN_TRAIN_SCENES = (20261208, 20261209, 20261211, 20261212)  # seeded scenes of the large workload's type
DN_TRAIN_VIEWS = 32  # views per scene, 256 x 256
DN_TRAIN_SPP = (64, 256, 1024, 4096)  # input sample counts, cycled over the views
DN_TRAIN_STEPS = 6000  # Adam steps of 16 random 128^2 crops
DN_EVAL_SCENE = 20261210  # held out
DN_EVAL_SIZE = (1920, 1080)
DN_TRUTH_SPP = 16384  # double-precision accumulation
DN_LEVELS = (64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384)  # --dn-max-spp extends it


def _dn_target_spp(spp_in: int) -> int:
    """Target sample count for an input of spp_in samples: an independent render with at
    least 4x the samples, 1024 to 4096 (the loss is unbiased for noisy targets)."""
    return int(min(max(4 * spp_in, 1024), 4096))


def run_denoiser(cpu: bool, max_spp: int = DN_LEVELS[-1]):
    """The learned denoiser: trained here on path-tracer pairs (scenes of the large
    workload's type, 256^2 views, 64-4096-spp inputs with first-hit features and the standard
    error, independent 1024-4096-spp double-precision targets), then (1) inference
    throughput at 1920x1080 and training-step throughput at 8 x 256^2 against the BF16
    tensor peak, and (2) plain path tracing vs path tracing + denoiser on a held-out scene at
    1920x1080: relative RMSE against a 16,384-spp double-precision render as the sample
    count doubles (to `max_spp`), and the time each needs to reach given error levels."""
    import torch

    import rendu_gb300 as R
    from rendu_gb300 import denoiser as D
    from rendu_gb300 import scenes as S

    t0 = time.perf_counter()
    feats, targets = [], []
    for k, seed in enumerate(DN_TRAIN_SCENES):
        tr = R.PathTracer(S.denoiser_scene(seed))
        f, t = D.render_pairs(tr, S.random_cameras(seed, DN_TRAIN_VIEWS), 256, 256, spp_in=list(DN_TRAIN_SPP),
                              spp_ref=_dn_target_spp, seed=1000 * k)
        feats.append(f)
        targets.append(t)
        tr.close()
    feats, targets = torch.cat(feats), torch.cat(targets)
    torch.cuda.synchronize()
    data_s = time.perf_counter() - t0
    net = D.Denoiser(seed=1)
    t0 = time.perf_counter()
    losses = D.train(net, feats, targets, DN_TRAIN_STEPS, batch=16, crop=128, lr=1e-3, log_every=1000)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del feats, targets

    # ---- throughput -----------------------------------------------------------------------
    peak, peak_kind = _bf16_peak()
    x = torch.rand((1, 1080, 1920, D.FEATURES), device="cuda")
    o = torch.empty((1, 1080, 1920, 3), device="cuda")
    for _ in range(3):
        net.denoise(x, o)
    inf_ms = _events_ms(lambda: net.denoise(x, o), 20)
    inf_flop = net.flops(1080, 1920, channels=(D.INPUT_CHANNELS, 3))  # channels that carry data
    fb = torch.rand((8, 256, 256, D.FEATURES), device="cuda")
    tb = torch.rand((8, 256, 256, 3), device="cuda")
    snap = net.get_params()
    for _ in range(3):
        net.train_step(fb, tb, 0.0, read_loss=False)
    tr_ms = _events_ms(lambda: net.train_step(fb, tb, 0.0, read_loss=False), 20)
    tr_flop = 3 * net.flops(256, 256, 8, channels=(D.INPUT_CHANNELS, 3))
    net.set_params(snap)
    del x, o, fb, tb

    # ---- quality on a held-out scene at 1080p ----------------------------------------------
    w, h = DN_EVAL_SIZE
    tr2 = R.PathTracer(S.denoiser_scene(DN_EVAL_SCENE))
    cam = S.random_cameras(DN_EVAL_SCENE, 1, ratio=w / h)[0]
    t0 = time.perf_counter()
    truth = torch.zeros((h, w, 3), device="cuda")
    tr2.render(dict(cam, ratio=w / h), DN_TRUTH_SPP, 5, truth, seed=7, mode=1, fp64=True)
    truth_s = tr2.last_stats()["device_ms"] / 1e3
    levels_spp = [DN_LEVELS[0] << k for k in range(64) if DN_LEVELS[0] << k <= max(max_spp, 2 * DN_LEVELS[0])]
    curve = D.progressive_curves(tr2, cam, w, h, levels_spp, truth, denoiser=net, seed=100)
    eval_s = time.perf_counter() - t0
    tr2.close()
    plain = [(p["render_s"], p["plain"]) for p in curve]
    den = [(p["render_s"] + p["denoise_ms"] / 1e3, p["denoised"]) for p in curve]
    # Plain path tracing's error against the truth: e^2(N) = a / N + b, b the truth's own
    # noise (independent renders); fitted by least squares on the measured levels, it gives
    # the sample count -- and, at the measured seconds per sample, the time -- at which plain
    # path tracing would reach a level beyond the measured range.
    inv = np.array([1.0 / p["spp"] for p in curve])
    e2 = np.array([p["plain"] ** 2 for p in curve])
    a_fit, b_fit = np.polyfit(inv, e2, 1)
    s_per_spp = curve[-1]["render_s"] / curve[-1]["spp"]
    levels = {}
    for thr in (0.1, 0.05, 0.02, 0.01):
        tp, td = D.time_to(plain, thr), D.time_to(den, thr)
        lv = {"plain_s": tp and round(tp, 4), "denoised_s": td and round(td, 4),
              "speedup": round(tp / td, 2) if tp and td else None}
        if tp is None:
            lv["plain_not_reached_by_s"] = round(plain[-1][0], 3)
            if thr * thr > b_fit and a_fit > 0:
                lv["plain_extrapolated_s"] = round(a_fit / (thr * thr - b_fit) * s_per_spp, 2)
                if td:
                    lv["speedup_extrapolated"] = round(lv["plain_extrapolated_s"] / td, 2)
            if td:
                lv["speedup_at_least"] = round(plain[-1][0] / td, 2)
        levels[str(thr)] = lv
    inf_tflops = inf_flop / inf_ms / 1e9
    out = {"workload": "5-level U-Net (32-128 channels, 3x3 conv, BF16 activations, FP32 accumulation); "
                       "inference 1920x1080, training 8 x 256^2",
           "value": round(inf_tflops, 1), "unit": "TFLOP/s (inference, 1920x1080)",
           "inference_ms_1080p": round(inf_ms, 3), "inference_gflop": round(inf_flop / 1e9, 1),
           "inference_gflop_padded": round(net.flops(1080, 1920) / 1e9, 1),
           "train_step_ms_8x256": round(tr_ms, 3), "train_tflops": round(tr_flop / tr_ms / 1e9, 1),
           "roofline": {"bound": "tensor", "achieved": round(inf_tflops, 1), "peak": peak, "unit": "TFLOP/s",
                        "frac": round(inf_tflops / peak, 4), "peak_kind": peak_kind, "kernel": "k_conv_fold",
                        "traffic": _profile_traffic("denoiser_conv_1080p.txt").get("k_conv_fold", {}).get(
                            "traffic_bytes_per_launch")},
           "training": {"scenes": len(DN_TRAIN_SCENES), "views": len(DN_TRAIN_SCENES) * DN_TRAIN_VIEWS,
                        "view_size": "256x256", "input_spp": list(DN_TRAIN_SPP),
                        "target_spp": [_dn_target_spp(s_) for s_ in DN_TRAIN_SPP], "steps": DN_TRAIN_STEPS,
                        "batch": "16 x 128^2 crops", "loss": "relative squared error (eps 0.01)",
                        "data_s": round(data_s, 2), "train_s": round(train_s, 2),
                        "losses": [(s_, round(l_, 6)) for s_, l_ in losses]},
           "quality": {"view": f"held-out scene, {w}x{h}, extended estimator, depth 5",
                       "ground_truth": f"{DN_TRUTH_SPP} spp, double-precision accumulation ({truth_s:.1f} s)",
                       "curve": [{k_: (round(v_, 5) if isinstance(v_, float) else v_) for k_, v_ in p.items()}
                                 for p in curve],
                       "time_to_rel_rmse": levels, "eval_s": round(eval_s, 1),
                       "plain_error_model": {"a": round(float(a_fit), 6), "b": float(b_fit),
                                             "truth_rel_rmse": round(float(np.sqrt(max(b_fit, 0.0))), 5)}}}
    return out


def run_reference(args):
    """Reference arm: the reference's Raycaster algorithm (C restatement; the reference's own
    sources do not travel to this host) on all host threads, same workload and metric."""
    from rendu_gb300 import scenes as S

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh, rays = S.raycaster_workload(SUBDIV, N_RAYS, SEED)
    from oracle import oracle as O

    O.build_port()
    threads = os.cpu_count() or 1
    port = O.PortRaycaster()
    port.add_mesh(mesh.positions, mesh.indices)
    port.build()
    probe = 1 << 18
    t0 = time.perf_counter()
    port.intersect(rays[:probe], threads=threads)
    per_ray = (time.perf_counter() - t0) / probe
    m = int(min(len(rays), max(probe, 6.0 / max(per_ray, 1e-12))))
    rng = np.random.default_rng(1)
    for _ in range(args.warmup):
        s = int(rng.integers(0, len(rays) - m + 1))
        port.intersect(rays[s:s + m], threads=threads)
    times = []
    for _ in range(args.steps):
        s = int(rng.integers(0, len(rays) - m + 1))
        t0 = time.perf_counter()
        port.intersect(rays[s:s + m], threads=threads)
        times.append(time.perf_counter() - t0)
    value = m * len(times) / sum(times) / 1e6
    out = {
        "impl": "reference", "metric": "Mrays/s (closest hit, raycaster workload)", "value": round(value, 3),
        "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * sum(times) / len(times), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": _config(mesh.triangle_count, len(rays), args.gpus),
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{m} contiguous rays of the 16,777,216-ray set per step"},
        "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-pt", action="store_true", help="skip the path-tracer lines")
    ap.add_argument("--denoiser-only", action="store_true", help="only the denoiser measurement (one JSON line)")
    ap.add_argument("--dn-max-spp", type=int, default=DN_LEVELS[-1],
                    help="largest sample count of the denoiser's quality curve (doubling from 64); 65536 "
                         "carries plain path tracing to rel-RMSE 0.01 against the 16,384-spp truth")
    ap.add_argument("--profile-dn", action="store_true",
                    help="only two 1920x1080 denoiser inferences and one 8 x 256^2 training step (for ncu captures)")
    ap.add_argument("--profile-run", action="store_true",
                    help="only one closest-hit and one any-hit launch over the workload (for ncu captures)")
    ap.add_argument("--profile-pt", default=None, choices=list(PT_CONFIGS) + ["batch_64"],
                    help="only one render of the given path-tracer configuration, its kernels launched "
                         "directly (for ncu captures)")
    ap.add_argument("--pt-size", default=None,
                    help="WxH: the --profile-pt render at another resolution (small ncu captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile_dn:
        import torch

        from rendu_gb300 import build as B
        from rendu_gb300 import denoiser as D

        B.build()
        net = D.Denoiser(seed=1)
        x = torch.rand((1, 1080, 1920, D.FEATURES), device="cuda")
        o = torch.empty((1, 1080, 1920, 3), device="cuda")
        net.denoise(x, o)
        net.denoise(x, o)
        fb = torch.rand((8, 256, 256, D.FEATURES), device="cuda")
        net.train_step(fb, torch.rand((8, 256, 256, 3), device="cuda"), 1e-4, read_loss=False)
        torch.cuda.synchronize()
        print(json.dumps({"profile_dn": "2 x inference 1920x1080 + 1 training step 8 x 256^2"}))
        return
    if args.denoiser_only:
        from rendu_gb300 import build as B

        B.build()
        print(json.dumps({"denoiser": run_denoiser(False, args.dn_max_spp)}), flush=True)
        return
    if args.profile_pt:
        import rendu_gb300 as R
        import torch
        from rendu_gb300 import build as B

        B.build()
        if args.profile_pt == "batch_64":
            from rendu_gb300 import scenes as S

            wl = S.batch_workload()
            tracers = [R.PathTracer(j["scene"]) for j in wl]
            jobs = [{"tracer": t, "camera": dict(j["scene"].camera, ratio=1.0), "samples": j["samples"],
                     "depth": j["depth"], "seed": j["seed"],
                     "image": torch.zeros((j["height"], j["width"], 3), dtype=torch.float32, device="cuda")}
                    for j, t in zip(wl, tracers)]
            # profile=True: the wave's kernels are launched directly rather than from the
            # graph's device-side loop, which a profiler cannot look into kernel by kernel
            st = R.BatchRenderer(0).render(jobs, profile=True)
            torch.cuda.synchronize()
            print(json.dumps({"profile_pt": "batch_64", **{k: v for k, v in st.items() if k != "kernel_ms"}}))
            return
        kind, w, h, spp, depth, _, mode = PT_CONFIGS[args.profile_pt]
        if args.pt_size:
            w, h = (int(v) for v in args.pt_size.split("x"))
        sc = _pt_scene(kind)
        img = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
        tr = R.PathTracer(sc)
        tr.render(dict(sc.camera, ratio=w / h), spp, depth, img, seed=1, mode=mode, profile=True)
        st = tr.last_stats()
        print(json.dumps({"profile_pt": args.profile_pt, "size": [w, h],
                          **{k: v for k, v in st.items() if k != "kernel_ms"}}))
        return

    import torch

    dist, rank, world = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from rendu_gb300 import build as B

    B.build()
    import rendu_gb300 as R
    from rendu_gb300 import scenes as S

    mesh, rays = S.raycaster_workload(SUBDIV, N_RAYS, _rank_seed(SEED, rank))
    n = len(rays)
    rc = R.Raycaster(local)
    rc.add_mesh(mesh.positions, mesh.indices)
    rc.updateHierarchy()
    st = rc.stats()

    pinned = torch.empty((n, 8), dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = rays
    d_rays = pinned.to(f"cuda:{local}", non_blocking=False)
    d_hits = torch.empty((n, 4), dtype=torch.float32, device=f"cuda:{local}")
    d_occ = torch.empty(n, dtype=torch.uint8, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()

    if args.profile_run:
        rc.intersect_batch(d_rays, out=d_hits)
        rc.intersect_any_batch(d_rays, out=d_occ)
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": "raycaster", "rays": n, "triangles": mesh.triangle_count}))
        return
    for _ in range(max(3, args.warmup)):
        rc.intersect_batch(d_rays, out=d_hits)
        rc.intersect_any_batch(d_rays, out=d_occ)
    _sync_all(dist, torch)

    # ---- timed: closest hit, rays resident in HBM (512 MB of rays per step > L2) --------
    # Clocks are sampled (every 200 ms) across all timed GPU work of this run: the closest-
    # and any-hit loops, the e2e loop and the path-tracer renders.
    clk = ClockSampler(local).__enter__()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _sync_all(dist, torch)
    ev0.record(stream)
    for _ in range(args.steps):
        rc.intersect_batch(d_rays, out=d_hits)
    ev1.record(stream)
    _sync_all(dist, torch)
    t_closest_local = ev0.elapsed_time(ev1) / 1000.0
    value = _job_rate(dist, torch, n * args.steps, t_closest_local) / 1e6
    t_closest = _max_over_ranks(dist, torch, t_closest_local)

    ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _sync_all(dist, torch)
    ea.record(stream)
    for _ in range(args.steps):
        rc.intersect_any_batch(d_rays, out=d_occ)
    eb.record(stream)
    _sync_all(dist, torch)
    t_any_local = ea.elapsed_time(eb) / 1000.0
    any_value = _job_rate(dist, torch, n * args.steps, t_any_local) / 1e6
    t_any = _max_over_ranks(dist, torch, t_any_local)

    # ---- e2e through the public API with host buffers ----------------------------------
    host_hits = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy().view(R.HIT_DTYPE).reshape(-1)
    host_rays = pinned.numpy()
    rc.intersect_batch(host_rays, out=host_hits)
    _sync_all(dist, torch)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc.intersect_batch(host_rays, out=host_hits)
    _sync_all(dist, torch)
    e2e_value = _job_rate(dist, torch, n * args.steps, time.perf_counter() - t0) / 1e6
    # the same with pageable host buffers (plain numpy arrays, as a C++ caller's std::vector)
    pg_rays = np.array(host_rays, copy=True)
    pg_hits = np.empty(n, R.HIT_DTYPE)
    rc.intersect_batch(pg_rays, out=pg_hits)
    _sync_all(dist, torch)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc.intersect_batch(pg_rays, out=pg_hits)
    _sync_all(dist, torch)
    e2e_pageable = _job_rate(dist, torch, n * args.steps, time.perf_counter() - t0) / 1e6

    # ---- algorithmic bytes per ray (visit counts on a 1M-ray sample) -------------------
    nv, nt = rc.count_visits(rays[: 1 << 20])
    v_node, v_tri = float(nv.mean()), float(nt.mean())
    bytes_per_ray = 32 + 16 + 128 * v_node + 48 * v_tri
    avg_launch = t_closest / args.steps
    achieved = bytes_per_ray * n / avg_launch / 1e9
    peak, peak_kind = _peaks()
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "raycaster_closest_16M.txt")) as f:
            for ln in f:
                if ln.startswith("traffic_bytes_per_launch:"):
                    traffic = float(ln.split(":")[1])
    except OSError:
        pass

    if rank == 0:
        out = {
            "metric": "Mrays/s (closest hit, raycaster workload)",
            "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000 * t_closest / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": _config(mesh.triangle_count, n, world),
            "any_hit": {"value": round(any_value, 2), "unit": "Mrays/s",
                        "ms_per_step": round(1000 * t_any / args.steps, 4)},
            "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s",
                    "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": n * 16, "host_memory": "pinned",
                    "pageable": {"value": round(e2e_pageable, 2), "unit": "Mrays/s"}},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_kind": peak_kind, "bytes_per_ray": round(bytes_per_ray, 1),
                         "node_visits_per_ray": round(v_node, 3), "tri_tests_per_ray": round(v_tri, 3),
                         "io_only_frac": round(48 * n / avg_launch / 1e9 / peak, 4)},
            "gpu_launches": args.steps,
            "bvh": {"build_ms": round(st["build_ms"], 2), "nodes": st["nodes"], "leaves": st["leaves"],
                    "sah_cost": round(st["sah_cost"], 2), "device_mb": round(st["device_bytes"] / 2**20, 1)},
        }
        if not args.no_pt:
            out["pathtracer"] = {name: run_pathtracer(name, 3, not args.no_cpu) for name in PT_CONFIGS}
            out["batch"] = run_batch(not args.no_cpu)
            out["denoiser"] = run_denoiser(not args.no_cpu)
        clk.__exit__(None, None, None)
        out["clocks"] = clk.summary()
        if not args.no_cpu:
            threads = max((os.cpu_count() or 2) - 1, 1)
            rate, m, build_s = cpu_raycaster_rate(mesh, rays, args.cpu_seconds, threads)
            out["cpu_baseline"] = {"value": round(rate, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                                   "sample": f"first {m} rays of the same 16,777,216-ray set",
                                   "build_s": round(build_s, 2)}
        print(json.dumps(out), flush=True)
    if rank != 0:
        clk.__exit__(None, None, None)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

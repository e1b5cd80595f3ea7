#!/usr/bin/env python
"""Benchmark of the A-SVGF denoise + luminance-histogram auto-exposure path on GB300.

Workload (one step = one frame through the whole path): 1 stream of 1920x1080, fp16 colour
and history storage (fp32 moments and variance), gradient sampling + 4 gradient a-trous,
temporal accumulation, anti-firefly, variance, 5 edge-aware a-trous passes with composition,
then the 256-bin histogram and eye adaptation. Inputs are a seeded 60-frame synthetic
sequence (analytic spheres and planes, camera 2 px/frame, a sphere moving 8 px/frame,
log-normal radiance sigma 1 with 0.1 % fireflies x100), generated before the timed region;
they stand in for captured frames, which the reference does not ship.

  value    Mpix/s with every frame's G-buffer already resident in HBM (bound to the stream
           without a copy), device time of K steps with CUDA events;
  e2e      the same through the C ABI from pinned HOST buffers: every step uploads the frame's
           G-buffer (rgdn_stream_upload), denoises, computes exposure, and reads PreFinal and
           the tonemapping state back to the host, synchronised per frame;
  roofline the dominant kernel's algorithmic bytes / its CUDA-event duration vs measured HBM;
  cpu_baseline  the CPU oracle (C++ restatement of the reference shaders) on the host cores.

`--impl reference` times the reference's own arithmetic on the host CPU (the oracle: the
reference's GLSL path cannot run here — no Vulkan or software renderer), per step one frame of
a 1920x120 band of the same workload, using every host core.

Multi-GPU (`torchrun --nproc-per-node N`): independent replicas, one stream per rank
(streams shard with no collective); value = all ranks' pixels / max time.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpix/s + p99 latency, served/batched vs plain A-SVGF on 1 GB300 at rel err≤1e-3"
STORAGE = {"ref": 0, "fp32": 1, "fp16": 2, "bf16": 3}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--storage", default="fp16", choices=list(STORAGE))
    ap.add_argument("--iters", type=int, default=5, help="a-trous passes")
    ap.add_argument("--frames", type=int, default=60, help="distinct frames in the sequence")
    ap.add_argument("--e2e-steps", type=int, default=120)
    ap.add_argument("--e2e-host-copy", choices=["sm", "engine"], default="sm",
                    help="how the streamed end-to-end uploads reach the device (rgdn_copy_host_planes)")
    ap.add_argument("--e2e-upload-priority", choices=["high", "normal"], default="high",
                    help="priority of the streamed end-to-end upload stream")
    ap.add_argument("--path", default="fused", choices=["fused", "plain", "tma", "pair", "afvar"],
                    help="fused: the default kernels; plain: one kernel per reference dispatch; "
                         "tma: the default kernels with TMA-staged a-trous; pair: the default kernels with "
                         "a-trous iterations 0 and 1 in one launch; afvar: the default kernels with "
                         "anti-firefly and variance in one launch")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU oracle (baseline and parity)")
    ap.add_argument("--parity-frames", type=int, default=8, help="frames run on GPU and oracle for the parity figures")
    ap.add_argument("--no-batched", action="store_true", help="skip the 32-stream batched measurement")
    ap.add_argument("--batch-steps", type=int, default=30)
    ap.add_argument("--batch-frames", type=int, default=4, help="distinct resident frames per batched stream")
    ap.add_argument("--batch-per-res", type=int, default=8, help="batched streams per resolution")
    ap.add_argument("--no-serving", action="store_true", help="skip the 64-stream serving measurement")
    ap.add_argument("--serve-seconds", type=float, default=3.0)
    ap.add_argument("--serve-only", action="store_true",
                    help="only the serving measurement (its runs and the end-to-end one), as its own JSON line")
    ap.add_argument("--serve-hz", type=float, nargs="+", default=[60.0, 15.0, 10.0],
                    help="per-stream Poisson frame rates to serve (the configured 60 Hz first)")
    ap.add_argument("--serve-step-mpix", type=float, default=8.0, help="pixel bound of one serving step (Mpix)")
    ap.add_argument("--serve-e2e-repeats", type=int, default=1,
                    help="end-to-end serving runs back to back in the process (the first is the line's)")
    ap.add_argument("--serve-host-copy", choices=["engine", "sm"], default="sm",
                    help="how the end-to-end serving run's pinned G-buffers reach the device: one kernel per "
                         "frame loading them over the host link (32 blocks), or the copy engines "
                         "(cudaMemcpyAsync per plane), whose copies stalled for 10-50 ms at times on the GB300 boxes")
    ap.add_argument("--serve-keep-pins", action="store_true",
                    help="end-to-end serving from the host buffers pinned at start-up, not fresh pinned "
                         "copies made right before each run (pinned buffers that have aged for tens of "
                         "seconds showed 30-50 ms host-to-device copy stalls on the GB300 boxes)")
    ap.add_argument("--serve-device-rates", type=int, default=1,
                    help="0: skip the device-resident serving runs (with --serve-only)")
    ap.add_argument("--serve-e2e-inflight", type=int, default=2,
                    help="serving steps enqueued ahead of the GPU in the end-to-end run (host inputs)")
    ap.add_argument("--serve-inflight", type=int, default=1,
                    help="serving steps enqueued ahead of the GPU (1..3) with resident inputs; the e2e run "
                         "(host inputs) uses at least 2 so copies overlap the kernels")
    ap.add_argument("--ncu-traffic", nargs="+", metavar="GROUP=CSV[@NAME]",
                    help="instead of the benchmark: print the profiles/dram_traffic.md rows (DRAM bytes read + "
                         "written per launch) of each kernel group from an ncu --csv capture of "
                         "dram__bytes_read.sum and dram__bytes_write.sum for that group's kernel (with --width, "
                         "--height and --storage of the captured run)")
    ap.add_argument("--precision-sweep", action="store_true",
                    help="instead of the benchmark: fp32/fp16/bf16 storage against the FP64 oracle "
                         "(use with --width 3840 --height 2160 --frames 30)")
    return ap.parse_args()


# ------------------------------------------------------------------------------------------
# distributed helpers (replicas; a barrier and a max-reduction of the timings only)
# ------------------------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            torch.cuda.set_device(self.local)
            dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{self.local}")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.samples, self.proc = device, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self) -> dict:
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ------------------------------------------------------------------------------------------
# algorithmic bytes per pixel of each kernel (each distinct texel read once, each output
# written once), from the framebuffer formats of the storage mode
# ------------------------------------------------------------------------------------------
def quantile(sorted_values: list, q: float):
    """The nearest-rank q-quantile (0 < q <= 1) of an ascending list."""
    import math
    return sorted_values[min(len(sorted_values) - 1, max(0, math.ceil(q * len(sorted_values)) - 1))]


def stage_bytes(storage: str) -> dict:
    col3 = {"ref": 4, "fp32": 16, "fp16": 8, "bf16": 8}[storage]
    cv = {"ref": 8, "fp32": 16, "fp16": 12, "bf16": 12}[storage]        # colour + variance
    cv_rgb = {"ref": 8, "fp32": 16, "fp16": 8, "bf16": 8}[storage]      # colour part only
    mom = {"ref": 4, "fp32": 8, "fp16": 8, "bf16": 8}[storage]
    hl = {"ref": 8, "fp32": 16, "fp16": 8, "bf16": 8}[storage]
    fv = {"ref": 2, "fp32": 4, "fp16": 4, "bf16": 4}[storage]
    pre = {"ref": 4, "fp32": 16, "fp16": 8, "bf16": 8}[storage]
    g = 1.0 / 9.0  # gradient images are 1/3 x 1/3
    b = {}
    # RtGradients image-space part: per stratum 9 motion + 8 GradientInputs_Prev reads, IsSky,
    # reshaded, IndirAccum_Prev, DISGradientHistory; writes DISPing + prev pix
    b["gradient_samples"] = 8 + 4 + g * (1 + 8 + col3 + 4 + 1) + g * (4 + 1)
    b["gradient_atrous"] = g * (4 + 4)
    # temporal accumulation: cur G-buffer + prev history (bilinear taps counted once) + writes
    b["temporal_accumulation"] = (12 + 8 + 8 + 2 + 4 + 2 + 16 + g * 4) + \
        (2 + 4 + cv_rgb + mom + hl + col3 + col3 + 16) + (col3 + mom + hl + col3 + col3)
    b["anti_firefly"] = 3 * col3 + 3 * col3
    b["variance_estimation"] = (col3 + 4 + 2 + hl + mom) + cv
    b["atrous0"] = (cv + 2 * col3 + 2 + 2 + 2 + 4 + hl) + (cv + 2 * col3 + fv)
    b["atrous"] = (cv + 2 * col3 + 2 + 2 + 2 + 4 + hl + fv) + (cv + 2 * col3)
    b["atrous_last"] = (cv + 2 * col3 + 2 + 2 + 2 + 4 + hl + fv) + (4 + 8 + 1) + (pre + 2)
    b["atrous_pair0"] = (cv + 2 * col3 + 2 + 2 + 2 + 4 + hl) + (cv + 2 * col3 + fv) + (cv + 2 * col3)
    b["atrous_pair"] = b["atrous"]
    b["luminance_histogram"] = 2
    b["luminance_avg"] = 0
    # The default path's kernels do the same reference stages, so they are charged the same
    # compulsory bytes: the 16-byte geometry record they write and read instead of normal,
    # depth and metallic-roughness is this implementation's choice, not the algorithm's traffic.
    for k in ("temporal_fast", "temporal_exact_geom", "temporal_fast_gp", "temporal_exact_geom_gp"):
        b[k] = b["temporal_accumulation"]
    b["anti_firefly_fast"] = b["anti_firefly"]
    b["variance_fast"] = b["variance_exact_geom"] = b["variance_estimation"]
    # anti-firefly + variance in one launch: the variance's read of the clamped diffuse colour
    # stays on chip
    b["af_variance_fast"] = b["af_variance_exact"] = b["anti_firefly"] + b["variance_estimation"] - col3
    return b


def path_bytes(storage: str) -> float:
    """Compulsory bytes per pixel of the whole fused chain (gradient samples through the
    histogram): every distinct input read once, every persistent output written once, the
    intermediates between stages never leaving the chip. The reference formats give about
    154.5 B/px; the 16-bit storage modes about 190.5 (16-bit colour and history, FP32 moments and
    variance)."""
    col3 = {"ref": 4, "fp32": 16, "fp16": 8, "bf16": 8}[storage]
    cv = {"ref": 8, "fp32": 16, "fp16": 12, "bf16": 12}[storage]
    mom = {"ref": 4, "fp32": 8, "fp16": 8, "bf16": 8}[storage]
    hl = {"ref": 8, "fp32": 16, "fp16": 8, "bf16": 8}[storage]
    pre = {"ref": 4, "fp32": 16, "fp16": 8, "bf16": 8}[storage]
    cur = 3 * 4 + 8 + 8 + 2 + 2 + 4 + 2 + 16 + 4 + 8 + 1                 # this frame's G-buffer: 67 B
    prev = 2 + 4 + 16 + cv + mom + hl + col3 + col3 + 4                  # history and G-buffer _Prev
    grad = 1.5                                                           # 1/9-resolution gradient state
    writes = cv + mom + hl + col3 + col3                                 # history for the next frame
    return cur + prev + grad + writes + pre


def kernel_bytes(name: str, it: int, niter: int, per_px: dict) -> float:
    if name in ("atrous", "atrous_fast", "atrous_fast_hist", "atrous_exact", "atrous_exact_hist", "atrous_tma",
                "atrous_tma_hist"):
        return per_px["atrous0"] if it == 0 else per_px["atrous_last"] if it == niter - 1 else per_px["atrous"]
    if name in ("atrous_pair", "atrous_pair_hist"):
        # two iterations in one launch (it, it + 1): the first one's sources and the static
        # planes read once; the second one's outputs written, and iteration 0's feedback image
        # and prefiltered variance as well when the pair starts at 0
        return per_px["atrous_pair0"] if it == 0 else per_px["atrous_pair"]
    return per_px[name]


def kernel_groups(kern: list, steps: int) -> list:
    """Per-launch entries (name[it]) summed per kernel over all its iterations, ranked by device
    time per step."""
    groups = {}
    for d in kern:
        name = d["kernel"].split("[")[0]
        g = groups.setdefault(name, {"kernel": name, "launches": 0, "us": 0.0, "alg_bytes": 0.0})
        g["launches"] += d["launches"]
        g["us"] += d["avg_us"] * d["launches"]
        g["alg_bytes"] += d["alg_bytes"] * d["launches"]
    out = []
    for g in groups.values():
        out.append({"kernel": g["kernel"], "launches_per_step": g["launches"] / steps,
                    "us_per_step": g["us"] / steps, "avg_us": g["us"] / g["launches"],
                    "alg_bytes_per_launch": g["alg_bytes"] / g["launches"],
                    "gbs": g["alg_bytes"] / (g["us"] / 1e6) / 1e9})
    out.sort(key=lambda g: -g["us_per_step"])
    return out


def host_link_gbs(dev: int, nbytes: int = 1 << 30, reps: int = 4) -> dict:
    """The host link's copy rates, measured live: one pinned buffer of `nbytes` copied host ->
    device, device -> host, and both at once on two streams (each direction's rate), timed
    with CUDA events after one untimed copy. These bound any end-to-end figure that moves a
    frame's inputs and outputs across the link."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    h2 = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=f"cuda:{dev}")
    d2 = torch.empty(nbytes, dtype=torch.uint8, device=f"cuda:{dev}")
    s1, s2 = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)

    def rate(fn) -> float:
        fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s1)
        s2.wait_event(e0)
        for _ in range(reps):
            fn()
        e2 = torch.cuda.Event()
        e2.record(s2)
        s1.wait_event(e2)
        e1.record(s1)
        e1.synchronize()
        return round(nbytes * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)

    def up():
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)

    def down():
        with torch.cuda.stream(s1):
            h2.copy_(d2, non_blocking=True)

    def both():
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    out = {"h2d_gbs": rate(up), "d2h_gbs": rate(down), "bidirectional_each_way_gbs": rate(both)}
    del h, h2, d, d2
    return out


def load_peaks() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel: str, width: int, height: int, storage: str):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu summary
    (profiles/dram_traffic.md, written by --ncu-traffic from one capture of this build), scaled
    from the captured frame size to this one by pixel count. None without a matching row."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.md")
    try:
        for line in open(path):
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            if len(cells) >= 5 and cells[0] == kernel and cells[1] == storage:
                w, h = (int(v) for v in cells[2].split("x"))
                return float(cells[4]) * (width * height) / (w * h)
    except Exception:
        pass
    return None


# ------------------------------------------------------------------------------------------
# CPU oracle timing (cpu_baseline in our line; the whole reference arm)
# ------------------------------------------------------------------------------------------
def oracle_check(ctx, args, frames: int):
    """The workload's first `frames` frames on a fresh GPU stream (default kernels) and on the
    CPU oracle (the same storage mode, all host cores), independently. Returns the oracle's time
    for the last frame (the CPU baseline) and the last frame's PRE_FINAL error (max-rel, p99.9
    rel, PSNR) with the histogram counts moved between bins per frame."""
    import numpy as np

    import oracle
    from raytracedgl1_gb300 import _native as N
    from raytracedgl1_gb300.denoiser import Denoiser, Stream, Tonemapping
    from raytracedgl1_gb300.scene import Scene

    W, H = args.width, args.height
    sc = Scene(W, H, seed=1)
    s = Stream(ctx, W, H, STORAGE[args.storage])
    o = oracle.OracleStream(W, H, STORAGE[args.storage])
    nthreads = os.cpu_count() or 1
    moved, last = [], None
    for f in range(frames):
        fi = f & 1
        bufs, p = sc.generate(f)
        p.atrousIterations = args.iters
        for k, v in bufs.items():
            s.upload(k, fi, v)
            o.load(k, fi, v)
        Denoiser(s).Denoise(fi, p)
        hg = s.tonemapping()[0].astype(np.int64)
        Tonemapping(s).CalculateExposure(fi, p)
        t0 = time.perf_counter()
        o.denoise(fi, p, nthreads)
        o.stage(N.STAGE_LUMINANCE_HISTOGRAM, 0, fi, p, nthreads)
        ho = o.tonemapping()[0].astype(np.int64)
        o.stage(N.STAGE_LUMINANCE_AVG, 0, fi, p, nthreads)
        last = time.perf_counter() - t0
        moved.append(int(np.abs(hg - ho).sum()) // 2)
    fi = (frames - 1) & 1
    img = s.image("PRE_FINAL", fi)
    fmt16 = img.format in (4, 5, 6)
    dec = (lambda a: a.view(np.float16).astype(np.float64)) if fmt16 else (lambda a: a.astype(np.float64))
    if img.format == 13:   # B10G11R11 (ref storage)
        from tests import _formats as F
        dec = lambda a: F.decode(a, 13).astype(np.float64)   # noqa: E731
    g = dec(s.download("PRE_FINAL", fi))[..., :3]
    c = dec(o.plane("PRE_FINAL", fi))[..., :3]
    atol = 1e-4 * float(np.percentile(np.abs(c), 99))
    rel = np.abs(g - c).max(axis=-1) / np.maximum(np.abs(c).max(axis=-1), atol)
    mse = float(np.mean((g - c) ** 2))
    peak = float(np.abs(c).max()) or 1.0
    s.close()
    cpu = {"value": round(W * H / last / 1e6, 4), "unit": "Mpix/s", "cores": nthreads, "kind": "port",
           "sample": f"frame {frames - 1} of the {W}x{H} sequence through the CPU oracle (denoise + exposure; "
                     f"frames 0-{frames - 2} untimed)"}
    parity = {"against": f"CPU oracle, {args.storage} storage, {frames} frames run independently",
              "frame": frames - 1, "max_rel": float(rel.max()), "p999_rel": float(np.percentile(rel, 99.9)),
              "frac_le_1e-3": float(np.mean(rel <= 1e-3)), "frac_le_1e-2": float(np.mean(rel <= 1e-2)),
              "psnr_db": round(10 * np.log10(peak * peak / mse), 2) if mse else None,
              "histogram_counts_moved_per_frame": moved,
              "histogram_note": "bit-exact given the same HistogramInput (tests); from independent runs a value "
                                "within an fp16 step of a bin edge can land in the neighbouring bin"}
    return cpu, parity


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    from raytracedgl1_gb300 import build
    build.build_oracle()
    build.build_scene()
    import oracle
    from raytracedgl1_gb300.scene import Scene
    W, H = args.width, min(120, args.height)
    sc = Scene(W, H, seed=1)
    o = oracle.OracleStream(W, H, STORAGE[args.storage])
    nthreads = os.cpu_count() or 1
    frames = [sc.generate(f) for f in range(min(args.frames, 8))]
    times = []
    for step in range(args.warmup + args.steps):
        f = step % len(frames)
        fi = step & 1
        bufs, p = frames[f]
        p.atrousIterations = args.iters
        for k, v in bufs.items():
            o.load(k, fi, v)
        t0 = time.perf_counter()
        o.denoise(fi, p, nthreads)
        o.calculate_exposure(fi, p, nthreads)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
    total = sum(times)
    mpix = W * H * len(times) / total / 1e6
    times.sort()
    line = {
        "impl": "reference", "metric": METRIC, "value": round(mpix, 4), "unit": "Mpix/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * total / len(times), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "p50_ms": round(1e3 * quantile(times, 0.5), 3), "p99_ms": round(1e3 * quantile(times, 0.99), 3),
        "config": dict(config_dict(args), band=f"{W}x{H}",
                       sample=f"each step times one {W}x{H} frame (a band of the {args.width}x{args.height} "
                              f"workload's width, from the same generator and stages, so the same per-pixel "
                              f"work); Mpix/s is per pixel of that band"),
        "cpu_baseline": {"value": round(mpix, 4), "unit": "Mpix/s", "cores": nthreads, "kind": "port",
                         "sample": f"one frame of a {W}x{H} band of the workload per step (same per-pixel work)"},
        "e2e": {"value": round(mpix, 4), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference GLSL/Vulkan path unavailable on this box (no graphics stack); the CPU "
                "restatement of its shaders (oracle/) is the reference's implementation timed here. Its "
                "outputs equal the reference's own shader sources run on the CPU bit for bit at every "
                "stage (oracle/glsl_ref, tests/test_ref_shaders.py); that emulation itself runs 2.3x "
                "slower than the restatement on one core, so the restatement is the faster CPU baseline",
    }
    print(json.dumps(line), flush=True)


def config_dict(args) -> dict:
    return {"workload": f"A-SVGF denoise + auto-exposure, 1 stream {args.width}x{args.height}, "
                        f"{args.storage} storage, {args.iters} a-trous passes + gradient a-trous, "
                        f"{args.frames}-frame synthetic sequence",
            "path": getattr(args, "path", "fused"),
            "streams_per_gpu": 1, "width": args.width, "height": args.height, "storage": args.storage,
            "atrous_iterations": args.iters, "frames": args.frames,
            "l2": "inputs larger than L2: each step touches its own frame's G-buffer (>160 MB) and the "
                  "stream's history (>500 MB), both above the 129 MB L2"}


# ------------------------------------------------------------------------------------------
# batched: 32 streams of mixed resolution advance one frame per step (rgdn_submit_batch)
# ------------------------------------------------------------------------------------------
BATCH_MIX = [(640, 360), (1280, 720), (1920, 1080), (2560, 1440)]


def run_batched(args, dist: Dist, dev: int, cs) -> dict:
    """Mpix/s of batched steps over 8 streams each of 640x360, 1280x720, 1920x1080 and
    2560x1440 (fp16 storage), beside the same frames one stream per call on the default path
    and on the plain path (one kernel per reference dispatch). G-buffers are resident in HBM
    and bound without a copy; `batch_frames` distinct frames per stream cycle."""
    import numpy as np
    import torch

    from raytracedgl1_gb300 import _native as N
    from raytracedgl1_gb300.denoiser import Context, Denoiser, Stream, Tonemapping
    from raytracedgl1_gb300.scene import Scene

    # frames side by side on several lanes: no L2 set-aside (measured about 1 % faster without)
    ctx = Context(dev, flags=N.CONTEXT_NO_L2_PERSIST)
    storage = STORAGE["fp16"]
    streams, seqs = [], []
    for r, (W, H) in enumerate(BATCH_MIX):
        for k in range(args.batch_per_res):
            sid = r * args.batch_per_res + k
            sc = Scene(W, H, seed=100 + sid + 1000 * dist.rank)
            s = Stream(ctx, W, H, storage)
            frames = []
            for f in range(args.batch_frames):
                bufs, p = sc.generate(f)
                p.atrousIterations = args.iters
                frames.append(({name: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).to(f"cuda:{dev}")
                                for name, a in bufs.items()}, p))
            streams.append(s)
            seqs.append(frames)
    torch.cuda.synchronize()
    px = sum(s.width * s.height for s in streams)

    def jobs_for(k: int, flags: int = 0, subset=None):
        jobs = []
        for idx, (s, frames) in enumerate(zip(streams, seqs)):
            if subset is not None and idx not in subset:
                continue
            bufs, p = frames[k % len(frames)]
            fi = k & 1
            for name, t in bufs.items():
                s.bind(name, fi, t.data_ptr())
            if flags:
                p = p.copy()
                p.flags |= flags
            jobs.append((s, fi, p))
        return jobs

    def batched(k, subset=None):
        ctx.submit_batch(jobs_for(k, 0, subset), cs)

    def one_by_one(k, flags, subset=None):
        for s, fi, p in jobs_for(k, flags, subset):
            Denoiser(s).Denoise(fi, p, cs)
            Tonemapping(s).CalculateExposure(fi, p, cs)

    def timed(fn, steps: int, first: int):
        # the host enqueues every launch of a step with one-frame groups: no garbage-collection
        # pause of this thread inside the timed region
        import gc
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        dist.barrier()
        torch.cuda.synchronize()
        gc.collect()
        gc.disable()
        with torch.cuda.stream(cs):
            ev[0].record(cs)
            for k in range(steps):
                fn(first + k)
                ev[k + 1].record(cs)
        cs.synchronize()
        gc.enable()
        dist.barrier()
        per = sorted(ev[k].elapsed_time(ev[k + 1]) for k in range(steps))
        return dist.max(ev[0].elapsed_time(ev[-1])), per

    k = 0
    with torch.cuda.stream(cs):
        for _ in range(28):          # autotuning (15 + 8 steps) + graph capture
            batched(k)
            k += 1
    cs.synchronize()
    cfg = ctx.batch_config(storage)
    launches0 = ctx.launch_count()
    t_b, per_b = timed(batched, args.batch_steps, k)
    launches = ctx.launch_count() - launches0
    k += args.batch_steps
    # per-launch device time of batched steps (direct launches with events)
    ctx.set_batch_timing(True)
    with torch.cuda.stream(cs):
        for _ in range(3):
            batched(k)
            k += 1
    cs.synchronize()
    tim = ctx.read_batch_timing()
    ctx.set_batch_timing(False)
    steps_cmp = max(3, args.batch_steps // 5)
    with torch.cuda.stream(cs):
        one_by_one(k, 0)
    t_s, _ = timed(lambda j: one_by_one(j, 0), steps_cmp, k + 1)
    k += 1 + steps_cmp
    with torch.cuda.stream(cs):
        one_by_one(k, N.FLAG_PLAIN)
    t_p, _ = timed(lambda j: one_by_one(j, N.FLAG_PLAIN), steps_cmp, k + 1)

    k += 1 + steps_cmp
    # each resolution class alone: its 8 streams batched against the same frames one stream per
    # call (the small frames are where launch overhead would show)
    per_class = []
    for r, (W, H) in enumerate(BATCH_MIX):
        sub = set(range(r * args.batch_per_res, (r + 1) * args.batch_per_res))
        cpx = W * H * len(sub)
        with torch.cuda.stream(cs):
            for _ in range(3):
                batched(k, sub)
                k += 1
        t_cb, _ = timed(lambda j: batched(j, sub), steps_cmp, k)
        k += steps_cmp
        with torch.cuda.stream(cs):
            one_by_one(k, 0, sub)
        t_cs, _ = timed(lambda j: one_by_one(j, 0, sub), steps_cmp, k + 1)
        k += 1 + steps_cmp
        vb = cpx * steps_cmp * dist.world / (t_cb / 1e3) / 1e6
        vs = cpx * steps_cmp * dist.world / (t_cs / 1e3) / 1e6
        per_class.append({"resolution": f"{W}x{H}", "streams": len(sub), "batched_mpix_s": round(vb, 1),
                          "one_stream_per_call_mpix_s": round(vs, 1), "vs_one_frame_per_launch": round(vb / vs, 3)})

    per_px = stage_bytes("fp16")
    # frames of at least singleFramePixels pixels run alone on the single-frame kernels (one timing
    # entry per such frame for its whole chain); the rest go through the constant-table kernels
    sizes = [s.width * s.height for s in streams]
    alone = [n for n in sizes if cfg.singleFramePixels and n >= cfg.singleFramePixels]
    px_alone, px_table = sum(alone), px - sum(alone)
    kern = []
    for (name, it), (n, ms) in tim.items():
        if name == "single_frame_group":
            # compulsory bytes of the whole chain (every input read once, every output written once)
            unit_px, alg = px_alone, path_bytes("fp16") * px_alone
        elif name == "atrous":
            pair = cfg.atrousFusionDepth >= 2 and it == 0
            unit_px = px_table
            alg = kernel_bytes("atrous_pair" if pair else "atrous_fast", it, args.iters, per_px) * px_table
        elif name in ("gradient_samples", "gradient_atrous"):
            unit_px, alg = px_table, per_px[name] * px_table
        else:
            unit_px = px_table
            alg = per_px.get({"temporal_accumulation": "temporal_fast_gp", "anti_firefly": "anti_firefly_fast",
                              "variance_estimation": "variance_fast"}.get(name, name), 0.0) * px_table
        # 3 timed steps; a step launches each kind once per group of frames
        us_step = 1e3 * ms / 3
        kern.append({"kernel": f"batched_{name}[{it}]", "launches_per_step": round(n / 3, 2),
                     "mpix_per_step": round(unit_px / 1e6, 3),
                     "us_per_step": round(us_step, 2), "us_per_mpix": round(us_step / max(unit_px / 1e6, 1e-9), 3),
                     "alg_bytes_per_step": alg, "gbs": round(alg / (us_step / 1e6) / 1e9, 1)})
    kern.sort(key=lambda d: -d["us_per_step"])
    out = {
        "workload": f"{len(streams)} streams: {args.batch_per_res} each of "
                    + ", ".join(f"{w}x{h}" for w, h in BATCH_MIX)
                    + f", fp16 storage, {args.iters} a-trous passes + gradient a-trous, one frame per stream per step",
        "mpix_per_step": round(px / 1e6, 3),
        "value": round(px * args.batch_steps * dist.world / (t_b / 1e3) / 1e6, 1), "unit": "Mpix/s",
        "ms_per_step": round(t_b / args.batch_steps, 3),
        "p50_ms": round(quantile(per_b, 0.5), 3), "p99_ms": round(quantile(per_b, 0.99), 3),
        "steps": args.batch_steps, "gpu_launches": int(launches),
        "one_stream_per_call_mpix_s": round(px * steps_cmp * dist.world / (t_s / 1e3) / 1e6, 1),
        "plain_path_mpix_s": round(px * steps_cmp * dist.world / (t_p / 1e3) / 1e6, 1),
        "tuned_config": {"temporal": int(cfg.temporalTile), "anti_firefly": int(cfg.antiFireflyTile),
                         "variance": int(cfg.varianceTile), "atrous": [int(v) for v in cfg.atrousTile][:args.iters],
                         "atrous_blocks_per_sm": [int(v) for v in cfg.atrousBlocksPerSM][:args.iters],
                         "atrous_fusion_depth": int(cfg.atrousFusionDepth),
                         "group_pixels": int(cfg.groupPixels), "single_frame_pixels": int(cfg.singleFramePixels),
                         "graphs": int(cfg.useGraphs), "tile_names": ["32x8", "16x16", "64x4", "32x4", "32x8 per block"]},
        "kernels": kern,
    }
    out["vs_plain"] = round(out["value"] / out["plain_path_mpix_s"], 3)
    out["vs_one_frame_per_launch"] = round(out["value"] / out["one_stream_per_call_mpix_s"], 3)
    out["per_class"] = per_class
    for s in streams:
        s.close()
    ctx.close()
    return out


# ------------------------------------------------------------------------------------------
# serving: 64 camera streams (720p / 1080p / 1440p drawn uniformly), Poisson frame arrivals
# ------------------------------------------------------------------------------------------
SERVE_RES = [(1280, 720), (1920, 1080), (2560, 1440)]


def run_serving(args, dist: Dist, dev: int) -> dict:
    """rgdn_server under per-stream Poisson arrivals (the configured 60 Hz, then lower rates),
    with history resident and admission under a 120 GB budget. Each request carries device
    pointers to a frame already resident in HBM (RGDN_REQUEST_BIND; 4 frames per resolution
    cycle), or, for the e2e run, pinned host G-buffers copied in the step with PRE_FINAL read
    back to pinned host memory. A stream keeps at most one waiting frame: an older waiting
    frame is dropped when a newer one arrives. Latency is submission -> completion on the
    host clock."""
    import numpy as np
    import torch

    from raytracedgl1_gb300 import _native as N
    from raytracedgl1_gb300.denoiser import Context, Server
    from raytracedgl1_gb300.scene import Scene

    storage = STORAGE["fp16"]
    ctx = Context(dev, memory_budget_bytes=120 * (1 << 30), flags=N.CONTEXT_NO_L2_PERSIST)
    rng = np.random.default_rng(7 + dist.rank)
    res = [SERVE_RES[i] for i in rng.integers(0, len(SERVE_RES), size=64)]
    frames, host = {}, {}
    for W, H in SERVE_RES:
        sc = Scene(W, H, seed=300 + W)
        fr, hf = [], []
        for f in range(4):
            bufs, p = sc.generate(f)
            p.atrousIterations = args.iters
            fr.append(({n: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).to(f"cuda:{dev}")
                        for n, a in bufs.items()}, p))
            hf.append(({n: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).pin_memory()
                        for n, a in bufs.items()}, p))
        frames[(W, H)], host[(W, H)] = fr, hf
    torch.cuda.synchronize()
    out_host = {r: torch.empty(r[0] * r[1] * 8, dtype=torch.uint8).pin_memory() for r in SERVE_RES}

    def serve(hz: float, e2e: bool) -> dict:
        inflight = args.serve_e2e_inflight if e2e else args.serve_inflight
        sv = Server(ctx, storage, max_frames_per_step=32, max_pixels_per_step=int(args.serve_step_mpix * 1e6),
                    max_queued_per_stream=1, steps_in_flight=inflight,
                    host_copy=N.HOST_COPY_SM if (e2e and args.serve_host_copy == "sm") else N.HOST_COPY_ENGINE)
        sids = [sv.open_stream(w, h) for w, h in res]
        reqs = []
        for i, sid in enumerate(sids):
            src = host[res[i]] if e2e else frames[res[i]]
            reqs.append([Server.request(sid, p, {n: t.data_ptr() for n, t in b.items()},
                                        N.REQUEST_COPY if e2e else N.REQUEST_BIND,
                                        out_host[res[i]].data_ptr() if e2e else None) for b, p in src])
        # warm-up: admission of every stream, the autotuner's steps, graph capture
        for rnd in range(3):
            ts = [sv.submit(reqs[i][rnd % 4]) for i in range(len(sids))]
            for t in ts:
                sv.wait(t)
        for rnd in range(24):
            sv.wait(sv.submit(reqs[rnd % len(sids)][rnd % 4]))
        sv.drain()
        arrivals = []
        for i in range(len(sids)):
            t = rng.exponential(1.0 / hz)
            while t < args.serve_seconds:
                arrivals.append((t, i))
                t += rng.exponential(1.0 / hz)
        arrivals.sort()
        sv.reset_stats()
        count = [0] * len(sids)
        tickets, late = [], []
        # the feeder is this Python thread: no garbage-collection pause while it feeds
        import gc
        gc.disable()
        t0 = time.perf_counter()
        for ta, i in arrivals:
            while True:
                dt = ta - (time.perf_counter() - t0)
                if dt <= 0:
                    break
                if dt > 2e-3:
                    time.sleep(dt - 1e-3)
            late.append(1e3 * ((time.perf_counter() - t0) - ta))   # the feeder's own delay
            tickets.append(sv.submit(reqs[i][count[i] % 4]))
            count[i] += 1
        sv.drain()
        elapsed = time.perf_counter() - t0
        gc.enable()
        st = sv.stats()
        lat_1080, queue, service = [], [], []
        for t, (_, i) in zip(tickets, arrivals):
            r = sv.wait(t, 0)
            if r.state == N.FRAME_DONE:
                # queueing (submission to the step's enqueue) and service (enqueue to completion)
                queue.append(r.queueMs)
                service.append(r.latencyMs - r.queueMs)
                if res[i] == (1920, 1080):
                    lat_1080.append(r.latencyMs)
        lat_1080.sort()

        def pct(v, q):
            v = sorted(v)
            return round(quantile(v, q), 3) if v else None
        offered = sum(res[i][0] * res[i][1] for _, i in arrivals)
        sv.close()
        return {"per_stream_hz": hz, "steps_in_flight": inflight, "seconds": round(elapsed, 3), "requests": len(arrivals),
                "offered_mpix_s": round(offered / args.serve_seconds / 1e6, 1),
                "value": round(st["pixelsDone"] / elapsed / 1e6, 1), "unit": "Mpix/s",
                "frames_done": int(st["framesDone"]), "frames_dropped": int(st["framesDropped"]),
                "p50_ms": round(st["p50Ms"], 3), "p99_ms": round(st["p99Ms"], 3), "max_ms": round(st["maxMs"], 3),
                "p99_all_requests_ms": (round(st["p99AllMs"], 3) if st["p99AllMs"] != float("inf") else "inf"),
                "drop_rate": round(st["dropRate"], 4),
                "p99_ms_1080p": round(pct(lat_1080, 0.99), 3) if lat_1080 else None,
                "queue_p50_ms": pct(queue, 0.5), "queue_p99_ms": pct(queue, 0.99),
                "service_p50_ms": pct(service, 0.5), "service_p99_ms": pct(service, 0.99),
                "feeder_late_p99_ms": pct(late, 0.99),
                "step_parts_ms": {k: round(st[k], 3) for k in ("issueP50Ms", "issueP99Ms", "copyInP50Ms", "copyInP99Ms",
                                                               "kernelsP50Ms", "kernelsP99Ms", "copyOutP50Ms", "copyOutP99Ms")},
                "mean_frames_per_step": round(st["meanFramesPerStep"], 2), "steps": int(st["steps"]),
                "gpu_busy_frac": round(st["busySeconds"] / elapsed, 3),
                "resident_gb": round(st["residentBytes"] / 1e9, 2)}

    runs = [serve(hz, False) for hz in args.serve_hz] if args.serve_device_rates else []

    def frames_h2d_gbs() -> float:
        """Host -> device rate of the requests' own pinned G-buffers (every plane of every
        frame once)."""
        dst = {r: torch.empty(max(t.numel() for t in host[r][0][0].values()), dtype=torch.uint8, device=f"cuda:{dev}")
               for r in SERVE_RES}
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nb = 0
        torch.cuda.synchronize(dev)
        e0.record()
        for r in SERVE_RES:
            for b, _ in host[r]:
                for t in b.values():
                    dst[r][:t.numel()].copy_(t, non_blocking=True)
                    nb += t.numel()
        e1.record()
        e1.synchronize()
        return round(nb / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)

    # the e2e run moves every frame across the host link: the link's rates, the rate of the
    # requests' own buffers and the host's load are recorded on both sides of each run
    e2e_runs, kept = [], []
    for _ in range(max(1, args.serve_e2e_repeats)):
        if not args.serve_keep_pins:
            # the old buffers stay referenced, so the new ones are new pinned allocations
            kept.append(dict(host))
            for r in SERVE_RES:
                host[r] = [({n: t.clone().pin_memory() for n, t in b.items()}, p) for b, p in host[r]]
        before = dict(host_link_gbs(dev, 1 << 29, 3), frames_h2d_gbs=frames_h2d_gbs(), loadavg=os.getloadavg()[0])
        clk = ClockSampler(dev)
        clk.start()
        r = serve(args.serve_hz[-1], True)
        r["clocks"] = clk.stop()
        r["host_link_before"] = before
        r["host_link_after"] = dict(host_link_gbs(dev, 1 << 29, 3), frames_h2d_gbs=frames_h2d_gbs(), loadavg=os.getloadavg()[0])
        e2e_runs.append(r)
    e2e = e2e_runs[0]
    e2e["host_buffers"] = ("pinned at start-up" if args.serve_keep_pins
                           else "fresh pinned copies made right before the run")
    e2e["host_copy"] = args.serve_host_copy
    if len(e2e_runs) > 1:
        e2e["repeats"] = [{k: r[k] for k in ("p50_ms", "p99_ms", "p99_all_requests_ms", "drop_rate", "queue_p99_ms",
                                              "service_p50_ms", "service_p99_ms", "gpu_busy_frac", "host_link_before",
                                              "step_parts_ms", "mean_frames_per_step", "clocks")}
                          for r in e2e_runs[1:]]
    W0, H0 = SERVE_RES[0]
    bpp = sum(t.numel() for t in host[(W0, H0)][0][0].values()) / (W0 * H0)
    e2e["h2d_gb_s_offered"] = round(e2e["offered_mpix_s"] * 1e6 * bpp / 1e9, 1)
    ctx.close()
    return {"workload": "64 camera streams, resolutions drawn uniformly from 1280x720 / 1920x1080 / 2560x1440 "
                        "(seeded), per-stream Poisson arrivals, fp16 storage, 120 GB admission budget, "
                        f"{args.iters} a-trous passes; steps bounded to {args.serve_step_mpix} Mpix; "
                        "at most one waiting frame per stream (older dropped)",
            "runs": runs, "e2e": e2e}


# ------------------------------------------------------------------------------------------
# our arm
# ------------------------------------------------------------------------------------------
def run_serve_only(args, dist: Dist):
    import torch
    from raytracedgl1_gb300 import build
    build.build_all()
    torch.cuda.set_device(dist.local)
    out = run_serving(args, dist, dist.local)
    if dist.rank == 0:
        print(json.dumps({"serving": out}), flush=True)


def run_ours(args, dist: Dist):
    import numpy as np
    import torch

    from raytracedgl1_gb300 import _native as N
    from raytracedgl1_gb300 import build
    from raytracedgl1_gb300.denoiser import Context, Denoiser, Stream, Tonemapping, copy_host_planes
    from raytracedgl1_gb300.scene import Scene

    build.build_all()
    dev = dist.local
    torch.cuda.set_device(dev)
    W, H = args.width, args.height
    storage = STORAGE[args.storage]
    ctx = Context(dev)
    st = Stream(ctx, W, H, storage)
    cs = torch.cuda.Stream(device=dev)
    sc = Scene(W, H, seed=1 + dist.rank)

    # --- the frame sequence, resident in HBM -------------------------------------------
    frames = []
    host_frames = []
    for f in range(args.frames):
        bufs, p = sc.generate(f)
        p.atrousIterations = args.iters
        if args.path == "plain":
            p.flags |= N.FLAG_PLAIN
        elif args.path == "tma":
            p.flags |= N.FLAG_TMA_STAGING
        elif args.path == "pair":
            p.flags |= N.FLAG_ATROUS_PAIR
        elif args.path == "afvar":
            p.flags |= N.FLAG_AF_VARIANCE_FUSED
        dev_bufs = {}
        for name, arr in bufs.items():
            t = torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1)).to(f"cuda:{dev}")
            dev_bufs[name] = t
        frames.append((dev_bufs, p))
        if f < 8:
            host_frames.append((bufs, p))
    torch.cuda.synchronize()
    gbytes_per_frame = sum(t.numel() for t in frames[0][0].values())

    den, tm = Denoiser(st), Tonemapping(st)

    def step(k: int):
        f = k % len(frames)
        fi = k & 1
        bufs, p = frames[f]
        for name, t in bufs.items():
            st.bind(name, fi, t.data_ptr())
        den.Denoise(fi, p, cs)
        tm.CalculateExposure(fi, p, cs)

    with torch.cuda.stream(cs):
        for k in range(args.warmup):
            step(k)
    cs.synchronize()

    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    launches0 = ctx.launch_count()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    dist.barrier()
    torch.cuda.synchronize()
    import gc
    gc.collect()
    gc.disable()   # no garbage-collection pause of the launching thread in the timed region
    with torch.cuda.stream(cs):
        ev[0].record(cs)
        for k in range(args.steps):
            step(args.warmup + k)
            ev[k + 1].record(cs)
    cs.synchronize()
    torch.cuda.synchronize()
    gc.enable()
    dist.barrier()
    launches = ctx.launch_count() - launches0
    total_ms = ev[0].elapsed_time(ev[-1])
    step_ms = sorted(ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps))
    clk = clocks.stop()
    total_ms_max = dist.max(total_ms)
    pixels = W * H * args.steps * dist.world
    value = pixels / (total_ms_max / 1e3) / 1e6

    # --- per-kernel durations over the same steps (library-side events) ------------------
    st.set_timing(True)
    with torch.cuda.stream(cs):
        for k in range(args.steps):
            step(args.warmup + args.steps + k)
    cs.synchronize()
    timing = st.read_timing()
    st.set_timing(False)
    per_px = stage_bytes(args.storage)
    kern = []
    for (name, it), (n, ms) in timing.items():
        alg = kernel_bytes(name, it, args.iters, per_px) * W * H
        kern.append({"kernel": f"{name}[{it}]", "launches": n, "avg_us": 1e3 * ms / n,
                     "alg_bytes": alg, "gbs": alg / (ms / n / 1e3) / 1e9})
    kern.sort(key=lambda d: -d["avg_us"] * d["launches"])
    kernel_total_us = sum(d["avg_us"] * d["launches"] for d in kern) / args.steps

    # --- exposure application and tonemapping (rgdn_prepare_final), after the same steps ------
    from raytracedgl1_gb300.denoiser import ImageComposition
    comp = ImageComposition(st)
    fparams = N.FinalParams.defaults()
    fparams.lightmapScreenCoverage = 0.0
    fparams.flags = N.FINAL_APPLY_SCATTERING
    nfin = max(args.steps, 20)
    with torch.cuda.stream(cs):
        for k in range(3):
            comp.Finalize(k & 1, fparams, cs)
        fe = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        fe[0].record(cs)
        for k in range(nfin):
            comp.Finalize(k & 1, fparams, cs)
        fe[1].record(cs)
    cs.synchronize()
    fin_us = 1e3 * fe[0].elapsed_time(fe[1]) / nfin
    pre_b = {"ref": 4, "fp32": 16, "fp16": 8, "bf16": 8}[args.storage]
    fin_alg = (pre_b + 4 + 8 + 8 + 2 * pre_b) * W * H   # PreFinal, emission, scattering, throughput in; Final, bloom out
    final = {"kernel": "prepare_final", "what": "CmCheckerboard + CmPrepareFinal (LPM 709, bloom input, scattering on)",
             "us_per_frame": round(fin_us, 2), "mpix_s": round(W * H / fin_us, 1),
             "alg_bytes": fin_alg, "gbs": round(fin_alg / (fin_us / 1e6) / 1e9, 1)}

    # --- bloom pyramid (rgdn_bloom: 8 down, 8 up, apply; 17 launches), after the composition --
    from raytracedgl1_gb300.denoiser import Bloom
    bloom = Bloom(st)
    with torch.cuda.stream(cs):
        for k in range(3):
            bloom.Apply(k & 1, 1.0, cs)
        be = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        be[0].record(cs)
        for k in range(nfin):
            bloom.Apply(k & 1, 1.0, cs)
        be[1].record(cs)
    cs.synchronize()
    bl_us = 1e3 * be[0].elapsed_time(be[1]) / nfin
    mips = [((W + 1) >> k) * ((H + 1) >> k) for k in range(9)]
    mips[0] = W * H
    # each level read once and written once on the way down, read (coarser level and own
    # texel) and written on the way up, then BLOOM_RESULT read and FINAL read and written
    bl_texels = sum(mips[k] + mips[k + 1] for k in range(8)) + sum(mips[k + 1] + 2 * mips[k] for k in range(1, 8)) \
        + mips[1] + W * H + 3 * W * H
    bl_alg = bl_texels * pre_b
    bloom_t = {"kernel": "bloom", "what": "8 downsample (13-tap, Karis on the first) + 8 tent upsample + apply, 17 launches",
               "us_per_frame": round(bl_us, 2), "mpix_s": round(W * H / bl_us, 1),
               "alg_bytes": bl_alg, "gbs": round(bl_alg / (bl_us / 1e6) / 1e9, 1)}

    # --- volumetric scattering (rgdn_process_scattering: volume integration + accumulation) ---
    from raytracedgl1_gb300.denoiser import Volumetric
    vparams = N.VolumetricParams()
    for name in ("invView", "invProjection", "volumeViewProj"):
        getattr(vparams, name)[:] = np.eye(4, dtype=np.float32).reshape(-1)
    vparams.cameraPosition[:] = (0.0, 0.0, -1.0, 0.0)
    vparams.volumeCameraNear, vparams.volumeCameraFar = 0.5, 3.0
    vparams.maxHistoryLength = 8.0
    vparams.volumeEnableType = N.VOLUME_ENABLE_VOLUMETRIC
    volu = Volumetric(st)
    with torch.cuda.stream(cs):
        for k in range(3):
            vparams.frameId = k
            volu.ProcessScattering(k & 1, vparams, cs)
        ve = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ve[0].record(cs)
        for k in range(nfin):
            vparams.frameId = 3 + k
            volu.ProcessScattering(k & 1, vparams, cs)
        ve[1].record(cs)
    cs.synchronize()
    vol_us = 1e3 * ve[0].elapsed_time(ve[1]) / nfin
    vol_bytes = 2 * 160 * 88 * 64 * 8
    # per pixel: motion 8, depth 2, normal 4, NDC depth 4, previous depth 2 and normal 4 (one
    # texel per pixel over the frame), previous scattering 8 and history 2, outputs 8 + 2
    vol_alg = vol_bytes + 44 * W * H
    volumetric_t = {"kernel": "process_scattering",
                    "what": "CmVolumetricProcess (160x88x64 froxels, in place) + CmScatterAccum (VOLUMETRIC mode)",
                    "us_per_frame": round(vol_us, 2), "mpix_s": round(W * H / vol_us, 1),
                    "alg_bytes": vol_alg, "gbs": round(vol_alg / (vol_us / 1e6) / 1e9, 1)}
    groups = kernel_groups(kern, args.steps)
    top = groups[0]
    peak, peak_kind = load_peaks()

    # --- end to end from pinned host buffers through the C ABI ----------------------------
    pinned = []
    for bufs, p in host_frames:
        hb = {}
        for name, arr in bufs.items():
            t = torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1)).pin_memory()
            hb[name] = t
        pinned.append((hb, p))
    pre_img = st.image("PRE_FINAL", 0)
    pre_bytes = pre_img.pitch_bytes * pre_img.height
    out_host = torch.empty(pre_bytes, dtype=torch.uint8).pin_memory()
    for name in N.GBUFFER:
        st.bind(name, 0, None)
        st.bind(name, 1, None)
    h2d = sum(t.numel() for t in pinned[0][0].values())
    d2h = pre_bytes + 256 * 4 + 4

    def e2e_step(k: int):
        f = k % len(pinned)
        fi = k & 1
        hb, p = pinned[f]
        for name, t in hb.items():
            st.upload(name, fi, (t.data_ptr(), t.numel()), cs)
        den.Denoise(fi, p, cs)
        tm.CalculateExposure(fi, p, cs)
        N.check(st.lib.rgdn_stream_download(st.handle, N.FB["PRE_FINAL"], fi, out_host.data_ptr(), pre_bytes,
                                            cs.cuda_stream))
        return st.tonemapping(cs)   # synchronous read of histogram + avgLuminance + exposure

    for k in range(4):
        e2e_step(k)
    dist.barrier()
    lat = []
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        a = time.perf_counter()
        e2e_step(k)
        lat.append(time.perf_counter() - a)
    e2e_sync_s = dist.max(time.perf_counter() - t0)
    lat.sort()

    # Streamed: the way a renderer feeds the denoiser. Frame k+1's G-buffer is uploaded (copy
    # stream) while frame k is denoised, into one of three device G-buffer sets bound to the
    # stream (a frame reads its own set and, for the _Prev images, the previous frame's); PRE_FINAL
    # and the tonemapping state of every frame are read back asynchronously into pinned buffers.
    # the uploads on a high-priority stream, as a renderer would put them (on GB300 the SM loader
    # reached the same 2474 Mpix/s from a normal-priority stream)
    up = torch.cuda.Stream(device=dev, priority=-1 if args.e2e_upload_priority == "high" else 0)
    sets = [{name: torch.empty(t.numel(), dtype=torch.uint8, device=f"cuda:{dev}") for name, t in pinned[0][0].items()}
            for _ in range(3)]
    uploaded = [torch.cuda.Event() for _ in range(3)]
    consumed = [torch.cuda.Event() for _ in range(3)]
    outs = [torch.empty(pre_bytes, dtype=torch.uint8).pin_memory() for _ in range(2)]
    tms = [torch.empty(256 * 4 + 4, dtype=torch.uint8).pin_memory() for _ in range(2)]
    for c in consumed:
        c.record(cs)

    def streamed_step(k: int, host_copy: int):
        f, fi, j = k % len(pinned), k & 1, k % 3
        hb, p = pinned[f]
        # set j was last read by frame k-3 (current) and frame k-2 (as _Prev)
        up.wait_event(consumed[( k - 2 ) % 3])
        copy_host_planes([(sets[j][name].data_ptr(), t.data_ptr(), t.numel()) for name, t in hb.items()], host_copy, up)
        uploaded[j].record(up)
        cs.wait_event(uploaded[j])
        for name in hb:
            st.bind(name, fi, sets[j][name].data_ptr())
        den.Denoise(fi, p, cs)
        tm.CalculateExposure(fi, p, cs)
        N.check(st.lib.rgdn_stream_download(st.handle, N.FB["PRE_FINAL"], fi, outs[k & 1].data_ptr(), pre_bytes,
                                            cs.cuda_stream))
        N.check(st.lib.rgdn_stream_copy_tonemapping(st.handle, tms[k & 1].data_ptr(), cs.cuda_stream))
        consumed[j].record(cs)

    def streamed(host_copy: int, first: int) -> float:
        for k in range(6):
            streamed_step(first + k, host_copy)
        cs.synchronize()
        dist.barrier()
        t0 = time.perf_counter()
        for k in range(args.e2e_steps):
            streamed_step(first + 6 + k, host_copy)
        cs.synchronize()
        return dist.max(time.perf_counter() - t0)

    # the headline form first (rgdn_copy_host_planes with args.e2e_host_copy), then the other one
    hc_main = N.HOST_COPY_SM if args.e2e_host_copy == "sm" else N.HOST_COPY_ENGINE
    e2e_s = streamed(hc_main, 0)
    e2e_other_s = streamed(N.HOST_COPY_ENGINE if hc_main == N.HOST_COPY_SM else N.HOST_COPY_SM, 6 + args.e2e_steps)
    e2e_value = W * H * args.e2e_steps * dist.world / e2e_s / 1e6
    # the host link's own rates: a frame cannot finish faster than its upload at the link's
    # host -> device rate, so W H / (h2d bytes / rate) is the end-to-end roofline
    link = host_link_gbs(dev)
    link_bound = W * H * dist.world / (h2d / (link["h2d_gbs"] * 1e9)) / 1e6
    for name in N.GBUFFER:
        st.bind(name, 0, None)
        st.bind(name, 1, None)

    # --- CPU baseline (rank 0, N=1) --------------------------------------------------------
    cpu, parity = None, None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        cpu, parity = oracle_check(ctx, args, args.parity_frames)

    st.close()
    ctx.close()
    del frames
    torch.cuda.empty_cache()
    batched = None if args.no_batched else run_batched(args, dist, dev, cs)
    torch.cuda.empty_cache()
    serving = None if args.no_serving else run_serving(args, dist, dev)
    if dist.rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mpix/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms_max / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded analytic scene; see bench.py docstring)",
        "p50_ms": round(quantile(step_ms, 0.5), 4), "p99_ms": round(quantile(step_ms, 0.99), 4),
        "config": config_dict(args),
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": top["kernel"], "achieved": round(top["gbs"], 1),
                     "peak": peak, "unit": "GB/s", "frac": round(top["gbs"] / peak, 4),
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)" if peak_kind == "measured" else "fallback 6800 GB/s",
                     "traffic": profile_traffic(top["kernel"], W, H, args.storage),
                     "alg_bytes_per_launch": round(top["alg_bytes_per_launch"]),
                     "avg_us_per_launch": round(top["avg_us"], 2), "launches_per_step": top["launches_per_step"],
                     "kernel_choice": "the kernel with the most device time per step, all its launches of a step summed",
                     "bytes": "compulsory bytes of the reference stages it runs (each distinct texel read once, each "
                              "output written once), in the storage mode's formats",
                     "path_alg_bytes_per_px": path_bytes(args.storage),
                     "path_achieved": round(path_bytes(args.storage) * W * H / (total_ms_max / args.steps / 1e3) / 1e9, 1),
                     "path_frac": round(path_bytes(args.storage) * W * H / (total_ms_max / args.steps / 1e3) / 1e9 / peak, 4)},
        "kernel_groups": [{k: (round(v, 2) if isinstance(v, float) else v) for k, v in g.items()} for g in groups],
        "kernels": [{k: (round(v, 2) if isinstance(v, float) else v) for k, v in d.items()} for d in kern],
        "kernel_sum_us_per_step": round(kernel_total_us, 2),
        "prepare_final": final,
        "bloom": bloom_t,
        "volumetric": volumetric_t,
        "path_alg_gbs": round(sum(d["alg_bytes"] * d["launches"] for d in kern) / args.steps /
                              (total_ms_max / args.steps / 1e3) / 1e9, 1),
        "e2e": {"value": round(e2e_value, 2), "unit": "Mpix/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps,
                "mode": "streamed: frame k+1's G-buffer uploads from pinned host memory while frame k is "
                        "denoised; PRE_FINAL and the tonemapping state of every frame read back to pinned host "
                        "memory; wall clock over all steps after a final synchronize",
                "host_copy": f"rgdn_copy_host_planes, {args.e2e_host_copy}, {args.e2e_upload_priority}-priority stream",
                ("engine_mpix_s" if hc_main == N.HOST_COPY_SM else "sm_mpix_s"):
                    round(W * H * args.e2e_steps * dist.world / e2e_other_s / 1e6, 2),
                "synchronous_mpix_s": round(W * H * args.e2e_steps * dist.world / e2e_sync_s / 1e6, 2),
                "synchronous_p50_ms": round(1e3 * quantile(lat, 0.5), 3),
                "synchronous_p99_ms": round(1e3 * quantile(lat, 0.99), 3),
                "host_link": link, "link_bound_mpix_s": round(link_bound, 1),
                "link_frac": round(e2e_value / link_bound, 4)},
        "clocks": clk,
        "cpu_baseline": cpu,
        "parity": parity,
        "gbuffer_bytes_per_frame": int(gbytes_per_frame),
        "batched": batched,
        "serving": serving,
        # the metric's own quantity: the served / batched forms against the plain path, at p99
        "served_batched": None if not (batched and serving) else {
            "batched_mpix_s": batched["value"], "batched_p99_step_ms": batched["p99_ms"],
            "batched_vs_plain_path": batched["vs_plain"],
            "batched_vs_one_frame_per_launch": batched["vs_one_frame_per_launch"],
            "served_mpix_s_configured_rate": serving["runs"][0]["value"],
            "served_p99_all_requests_ms_configured_rate": serving["runs"][0]["p99_all_requests_ms"],
            "served_drop_rate_configured_rate": serving["runs"][0]["drop_rate"],
            "served_p99_ms_1080p_lowest_rate": serving["runs"][-1]["p99_ms_1080p"],
            "plain_path_mpix_s": batched["plain_path_mpix_s"]},
    }
    print(json.dumps(line), flush=True)


def run_precision(args, dist: Dist):
    """fp32 / fp16 / bf16 storage against the FP64 oracle on the precision-sweep scene
    (radiance sigma 2, 1 % fireflies x1000): PRE_FINAL error after every tenth frame and the
    last, and each stage's algorithmic HBM GB/s per storage mode. The FP32 oracle (fp32 storage,
    the shaders' own arithmetic) runs beside it: GPU fp32 against it is the parity bar, and the
    FP32 oracle against FP64 separates FP32 arithmetic (threshold decisions that flip between
    FP32 and FP64) from storage precision."""
    import numpy as np

    import oracle
    from raytracedgl1_gb300 import build
    from raytracedgl1_gb300.denoiser import Context, Denoiser, Stream, Tonemapping
    from raytracedgl1_gb300.scene import Scene

    if dist.rank != 0:
        return
    build.build_all()
    W, H, frames = args.width, args.height, args.frames
    sc = Scene(W, H, seed=5, sigma=2.0, fireflyProb=0.01, fireflyMult=1000.0)
    o64 = oracle.OracleStream(W, H, oracle.MODE_F64)
    o32 = oracle.OracleStream(W, H, oracle.MODE_F32)
    ctx = Context(0)
    modes = ["fp32", "fp16", "bf16"]
    gpu = {m: Stream(ctx, W, H, STORAGE[m]) for m in modes}
    nthreads = os.cpu_count() or 1

    def decode(arr, fmt):
        if fmt in (4, 5, 6):
            return arr.view(np.float16).astype(np.float64)
        return arr.astype(np.float64)

    def metrics(x, ref):
        """max-rel, p99 / p99.9 rel and the fraction within 1e-3 / 1e-2 of |x - ref| over the
        pixel's largest reference channel (floor 1e-3 of the 99th percentile), and PSNR with
        the reference's peak."""
        x, ref = x[..., :3], ref[..., :3]
        atol = 1e-3 * float(np.percentile(np.abs(ref), 99))
        d = np.abs(x - ref).max(axis=-1)
        rel = d / np.maximum(np.abs(ref).max(axis=-1), atol)
        mse = float(np.mean((x - ref) ** 2))
        peak = float(np.abs(ref).max()) or 1.0
        return {"max_rel": float(rel.max()), "p99_rel": float(np.percentile(rel, 99)),
                "p999_rel": float(np.percentile(rel, 99.9)), "frac_le_1e-3": float(np.mean(rel <= 1e-3)),
                "frac_le_1e-2": float(np.mean(rel <= 1e-2)),
                "psnr_db": round(10 * np.log10(peak * peak / mse), 2) if mse else None}

    report = {m: [] for m in modes}
    report["fp32_vs_fp32_oracle"] = []
    report["fp32_oracle_vs_fp64"] = []
    stage_gbs = {}
    t_oracle = 0.0
    for f in range(frames):
        fi = f & 1
        bufs, p = sc.generate(f)
        p.atrousIterations = args.iters
        t0 = time.perf_counter()
        for o in (o64, o32):
            for k, v in bufs.items():
                o.load(k, fi, v)
            o.denoise(fi, p, nthreads)
            o.calculate_exposure(fi, p, nthreads)
        t_oracle += time.perf_counter() - t0
        last = f == frames - 1
        for m, s in gpu.items():
            for k, v in bufs.items():
                s.upload(k, fi, v)
            s.set_timing(last)
            Denoiser(s).Denoise(fi, p)
            Tonemapping(s).CalculateExposure(fi, p)
            if last:
                per_px = stage_bytes(m)
                stage_gbs[m] = {f"{name}[{it}]": round(kernel_bytes(name, it, args.iters, per_px) * W * H / (ms / n / 1e3) / 1e9, 1)
                                for (name, it), (n, ms) in s.read_timing().items()}
                s.set_timing(False)
        if f % 10 == 9 or last:
            ref = o64.plane("PRE_FINAL", fi).astype(np.float64)
            ref32 = o32.plane("PRE_FINAL", fi).astype(np.float64)
            for m, s in gpu.items():
                img = s.image("PRE_FINAL", fi)
                g = decode(s.download("PRE_FINAL", fi), img.format)
                report[m].append(dict(metrics(g, ref), frame=f))
                if m == "fp32":
                    report["fp32_vs_fp32_oracle"].append(dict(metrics(g, ref32), frame=f))
            report["fp32_oracle_vs_fp64"].append(dict(metrics(ref32, ref), frame=f))
            print(f"frame {f}: " + ", ".join(f"{k} max_rel {v[-1]['max_rel']:.3g} p99.9 {v[-1]['p999_rel']:.3g} "
                                             f"psnr {v[-1]['psnr_db']}" for k, v in report.items()), file=sys.stderr, flush=True)
    line = {"metric": "PRE_FINAL error of each storage mode against the FP64 oracle", "unit": "relative / dB",
            "config": {"workload": f"precision sweep, 1 stream {W}x{H}, {frames} frames, radiance sigma 2, "
                                   f"1% fireflies x1000, {args.iters} a-trous passes, default (FAST) kernels",
                       "width": W, "height": H, "frames": frames},
            "data": "synthetic (seeded analytic scene)", "errors": report, "stage_alg_gbs": stage_gbs,
            "oracle_seconds_per_frame": round(t_oracle / frames, 2), "oracle_threads": nthreads}
    print(json.dumps(line), flush=True)
    for s in gpu.values():
        s.close()
    ctx.close()


def ncu_traffic(args):
    """profiles/dram_traffic.md rows from ncu --csv captures (one per kernel group): per launch,
    the DRAM bytes read + written, averaged over the captured launches."""
    import csv
    scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3, "MB": 1e6, "GB": 1e9}
    print("| kernel group | storage | frame | launches captured | DRAM bytes per launch (read + write) |")
    print("|---|---|---|---|---|")
    for item in args.ncu_traffic:
        group, path = item.split("=", 1)
        # GROUP=CSV@TEXT keeps the launches whose kernel name contains TEXT
        path, _, only = path.partition("@")
        per = {}
        with open(path, newline="") as f:
            lines = [ln for ln in f if ln.startswith('"')]
        for row in csv.DictReader(lines):
            name = row.get("Metric Name", "")
            if name not in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
                continue
            if only and only not in row.get("Kernel Name", ""):
                continue
            v = float(row["Metric Value"].replace(",", "")) * scale.get(row.get("Metric Unit", "byte"), 1)
            per[row["ID"]] = per.get(row["ID"], 0.0) + v
        if per:
            print(f"| {group} | {args.storage} | {args.width}x{args.height} | {len(per)} | {sum(per.values()) / len(per):.0f} |")


def main():
    args = parse()
    if args.ncu_traffic:
        ncu_traffic(args)
        return
    dist = Dist()
    try:
        if args.precision_sweep:
            run_precision(args, dist)
        elif args.impl == "reference":
            run_reference(args, dist)
        elif args.serve_only:
            run_serve_only(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()

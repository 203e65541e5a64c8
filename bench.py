"""Benchmark: training steps/s at 1.1M Gaussians.

Workload: a seeded synthetic scene of 40 random
planes and boxes grown to 1.1M Gaussians (SH degree 3), trained against
photos rendered from a 500k-Gaussian ground truth on the same surfaces, seen
by 263 training cameras on a jittered ring at 980x545 (fov 55 deg). One step
is one Trainer.optimize(): preprocess, tile keys, radix sort, ranges, blend,
L1 + D-SSIM loss, both backward passes, densification statistics and Adam,
replayed as one captured CUDA graph. Densification is off in the timed steps
(the steady state after the reference's step 15,000); the SH degree is
already 3. The working set (~3 GB) is far larger than L2, so no flush is
needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference's algorithm on the host cores instead:
the reference itself is TypeScript + WGSL that only runs in a browser's
WebGPU, so its CPU implementation here is the oracle (oracle/oracle.c, a C
restatement of its WGSL, OpenMP over all host threads), on the same workload.
For N > 1 the path has no exchange step (a training step renders one view
against one global parameter set, so it does not shard): each rank trains its
own replica and the value is the sum.
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
from dataclasses import replace
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "train steps/s @1.1M Gaussians"
UNIT = "steps/s"
GROUND_TRUTH = 500_000
SCENE_SEED, TRUTH_SEED = 22, 21


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--gaussians", type=int, default=1_100_000)
    ap.add_argument("--views", type=int, default=263, help="training views (photos) to render and cycle through")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-held-out", action="store_true", help="skip the held-out views' frames/s")
    ap.add_argument("--workload", default="train", choices=["train", "sort", "densify", "knn", "profile", "mlp"],
                    help="train: the headline training step; sort: the sort/scan/ranges stress "
                         "(1.1M random Gaussians at 1960x1090, the reference's 6-pass sort); densify: "
                         "plain vs learned densification on the planes-and-boxes scene (minutes); knn: the "
                         "starting Gaussians' nearest-neighbour distances of a point cloud; profile: one training "
                         "step bracketed for a profiler started with collection off; mlp: the learned "
                         "densification's inference (tcgen05) over random candidates")
    ap.add_argument("--knn-points", type=int, default=1_100_000, help="knn workload: points in the cloud")
    ap.add_argument("--candidates", type=int, default=1_100_000, help="mlp workload: candidates per call")
    ap.add_argument("--densify-steps", type=int, default=15_000,
                    help="learned-vs-plain comparison: steps per training run (the reference's 30,000-step "
                         "schedule scaled to this)")
    ap.add_argument("--densify-threshold", type=float, default=1.5e-5,
                    help="learned-vs-plain comparison: the densification gradient threshold")
    ap.add_argument("--densify-seeds", type=int, default=3, help="learned-vs-plain comparison: starting sets")
    ap.add_argument("--no-densify-comparison", action="store_true",
                    help="train workload: leave out the learned-vs-plain comparison (minutes)")
    ap.add_argument("--unbalanced", action="store_true",
                    help="densify workload: plain cross-entropy (by default both labels weigh the same: ~98%% of "
                         "children survive, and unweighted the model only learns that)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    return args


def dist_setup(args):
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    group = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        group = dist
    return rank, world, local, group


def reduce_max(group, value: float) -> float:
    if group is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64)
    group.all_reduce(t, op=group.ReduceOp.MAX)
    return float(t.item())


def barrier(group):
    if group is not None:
        group.barrier()


def config(args, world):
    return {
        "workload": "planes-and-boxes scene grown to 1.1M Gaussians, one optimize() step per 980x545 "
                    "training view, full step as one CUDA graph",
        "gaussians": args.gaussians,
        "viewport": [980, 545],
        "training_views": args.views,
        "sh_degree": 3,
        "densify": "off in the timed steps (steady state past step 15,000); the learned-vs-plain comparison "
                   "(densify_comparison) trains its own runs after the timed steps",
        "l2": "working set ~3 GB > 129 MB L2; no flush needed",
        "parallelism": f"replicas x{world}",
    }


class ClockSampler:
    """nvidia-smi samples every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[4:8]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_scene(args):
    from diorama_gb300 import scenes

    raw, sh = scenes.surface_scene(args.gaussians, SCENE_SEED, noise=0.01)
    truth_raw, truth_sh = scenes.surface_scene(GROUND_TRUTH, TRUTH_SEED)
    train_cams, _held = scenes.ring_cameras()
    return raw, sh, truth_raw, truth_sh, train_cams[: args.views]


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of each
# kernel at 1.1M Gaussians, from one ncu capture of the profiled training step:
# `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
# --clock-control none --profile-from-start off -k regex:<kernel> -c 1
# python bench.py --workload profile --views 8 --warmup 3`.
NCU_TRAFFIC = {"preprocess_backward_adam": 1_781_186_048, "preprocess": 315_799_040}


# Algorithmic bytes per unit: what each kernel must move at minimum.
def algorithmic_bytes(name: str, n: int, pairs: int, pixels: int, tiles: int, passes: int = 6,
                      drawn: float = 0.0) -> float | None:
    return {
        # The preprocess backward fused with Adam: read the activated Gaussian 64, SH 180,
        # splat gradients 36 and visibility 4, raw parameters 56 and moments 472 (59 used
        # slots); write SH 180, parameters 56, moments 472 and activated values 56; and for
        # each drawn Gaussian (splat radius > 0) the densification statistics it updates,
        # every step like the reference (src/trainer.ts:230-234): read and write stats 16
        # and aux 8.
        "preprocess_backward_adam": 1576.0 * n + 48.0 * drawn,
        "preprocess": 300.0 * n,  # read Gaussian 64 + SH 180, write splat 48 + tile count 4 + radius 4
        "preprocess_backward": (64 + 180 + 48 + 36 + 64 + 180) * float(n),
        "sort_pass": 24.0 * pairs,  # per pass: read and write 8 B key + 4 B value
        "sort_histogram": 8.0 * pairs,
        "scan": 8.0 * n,
        "duplicate": 20.0 * n + 12.0 * pairs,
        "find_ranges": 8.0 * pairs + 8.0 * tiles,
        "loss_ssim": 20.0 * pixels + 48.0 * pixels,
        "loss_gradient": 20.0 * pixels + 48.0 * pixels + 20.0 * pixels,
        "stats": (4 + 8 + 16 + 16) * float(n),
    }.get(name)


def run_ours(args, rank, world, local, group):
    from diorama_gb300 import (DEFAULT_SETTINGS, Device, GaussianRenderer, RawGaussians, Trainer, TrainingView,
                               activate)
    from diorama_gb300.gpu import PinnedArray

    raw, sh, truth_raw, truth_sh, cams = build_scene(args)
    device = Device(local)
    W, H = cams[0].viewport
    photographer = GaussianRenderer(device)
    photographer.setGaussians(activate(truth_raw), {"rest": truth_sh.reshape(-1), "degree": 3})
    views = []
    for k, cam in enumerate(cams):
        tex = device.createTexture(W, H)
        photographer.encode(None, tex, cam, (0, 0, 0))
        views.append(TrainingView(f"view {k}", cam, tex))
    device.synchronize()
    photographer.destroy()
    settings = replace(DEFAULT_SETTINGS, extent=4.0, shDegreeInterval=1, densifyUntil=0)
    trainer = Trainer(device, RawGaussians(raw.reshape(-1), sh.reshape(-1)), views, settings)
    trainer.setGraph(not args.no_graph)
    for _ in range(args.warmup):
        trainer.step()
    trainer.renderer.afterSubmit()
    trainer.step()  # re-capture if the warm-up grew the pair buffers
    device.synchronize()
    assert trainer.shDegree == 3

    # Device-timed steps: CUDA events on the library's stream.
    start, end = device.event(), device.event()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(group)
    device.synchronize()
    launches0 = device.launch_count
    start.record()
    for _ in range(args.steps):
        trainer.step()
    end.record()
    ms = start.elapsed_ms(end)
    device.synchronize()
    barrier(group)
    clocks = sampler.stop()
    launches = device.launch_count - launches0
    ms = reduce_max(group, ms)
    value = world * args.steps / (ms / 1000.0)

    # End to end through the public API: each step uploads its photo from pinned
    # host memory and reads back the loss.
    pinned = []
    for v in views:
        p = PinnedArray((H * W * 4,), np.uint8)
        p.array[:] = v.image.read().reshape(-1)
        pinned.append(p)
    camera_bytes, adam_bytes = 144, 48
    barrier(group)
    device.synchronize()
    # The trainer copies each step's photo from pinned host memory itself (the
    # next step's while the current one runs), and each step's loss is read back
    # after the next step is launched, as a training loop logging its loss does.
    trainer.setHostPhotos(pinned)
    t0 = time.perf_counter()
    e2e_losses = []
    for s in range(args.steps):
        trainer.step()
        trainer.requestLoss()
        if s > 0:
            e2e_losses.append(trainer.takeLoss())
    e2e_losses.append(trainer.takeLoss())
    e2e_s = reduce_max(group, time.perf_counter() - t0)
    trainer.setHostPhotos(None)
    assert len(e2e_losses) == args.steps and all(math.isfinite(v) for v in e2e_losses)
    barrier(group)
    e2e = {"value": world * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": W * H * 4 + camera_bytes + adam_bytes
           + 8 + 16, "d2h_bytes_per_step": 8 + 4}

    # The same steps without graph replay (the captured step is reported against
    # the uncaptured one).
    trainer.setGraph(False)
    trainer.step()
    device.synchronize()
    start.record()
    for _ in range(args.steps):
        trainer.step()
    end.record()
    uncaptured = {"value": round(args.steps / (start.elapsed_ms(end) / 1000.0), 2), "unit": UNIT}

    # Held-out views: all 37 rendered together (batched stages, graph replay,
    # batch size and cooperative threshold from the autotuner) against the
    # per-view encode loop, in frames/s.
    held = None if args.no_held_out else held_out_views(args)
    if rank == 0 and held is not None:
        held_out = measure_held_out(device, trainer.renderer, held, args.steps)
    else:
        held_out = None

    # Per-kernel times: the same steps launched directly, each kernel bracketed by events.
    device.synchronize()
    device.setKernelTiming(True)
    device.kernelTimingReport()
    drawn_counts = []
    for _ in range(args.steps):
        trainer.step()
        # Gaussians drawn this step (splat radius > 0): the fused kernel updates their statistics.
        radius = trainer.renderer.splatBuffer.read(np.float32)[: trainer.count * 12].reshape(-1, 12)[:, 3]
        drawn_counts.append(int(np.count_nonzero(radius)))
    report = device.kernelTimingReport()
    device.setKernelTiming(False)
    drawn = float(np.mean(drawn_counts))
    pairs = trainer.renderer.tiles.lastPairCount
    n = trainer.count
    tiles = math.ceil(W / 16) * math.ceil(H / 16)
    total = sum(ms for _, ms in report.values())
    kernels = {name: {"launches": c, "avg_us": 1000 * t / c, "share": t / total} for name, (c, t) in report.items()}

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_source = "measured" if "hbm_gbs" in peaks else "fallback"
    roofline = None
    memory_kernels = [k for k in kernels if algorithmic_bytes(k, n, pairs, W * H, tiles) is not None]
    dominant = max(kernels, key=lambda k: kernels[k]["share"])
    dom_mem = max(memory_kernels, key=lambda k: kernels[k]["share"]) if memory_kernels else None
    if dom_mem:
        launches_per_step = kernels[dom_mem]["launches"] / args.steps
        by = algorithmic_bytes(dom_mem, n, pairs, W * H, tiles, drawn=drawn)
        achieved = by / (kernels[dom_mem]["avg_us"] * 1e-6) / 1e9
        roofline = {"kernel": dom_mem, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak,
                    "unit": "GB/s", "frac": round(achieved / hbm_peak, 3), "peak_source": peak_source,
                    "algorithmic_bytes_per_launch": by, "launches_per_step": launches_per_step,
                    "drawn_gaussians_per_step": round(drawn, 1),
                    "traffic": NCU_TRAFFIC.get(dom_mem) if n == 1_100_000 else None}
    # The blend's work: the splats each pixel walks, counted as the forward's
    # pixel_last (the 1-based position of the last splat the pixel blended) summed
    # over the last step's pixels, per second of each blend kernel.
    last = trainer.renderer.pixelLastBuffer.read(np.uint32)[: W * H]
    evaluations = int(last.astype(np.int64).sum())
    blend = {"evaluations_per_step": evaluations}
    for k in ("rasterize", "rasterize_backward"):
        if k in kernels:
            blend[k] = {"avg_us": round(kernels[k]["avg_us"], 1), "share": round(kernels[k]["share"], 3),
                        "evaluations_per_s": round(evaluations / (kernels[k]["avg_us"] * 1e-6), 1)}

    # Densification's compaction at this size (after everything else: it changes
    # the scene; the second of two): count, scan and the two scatter kernels, timed with events, in
    # GB/s of 748 B per input Gaussian + 812 B per output + 8 B per input.
    # One untimed densification first: the kernels' first launches in the process
    # would also time their lazy loading.
    trainer.densify(False)
    device.synchronize()
    device.setKernelTiming(True)
    device.kernelTimingReport()
    before = trainer.count
    trainer.densify(False)
    dreport = device.kernelTimingReport()
    device.setKernelTiming(False)
    after = trainer.count
    d_us = 1000 * sum(t for name, (c, t) in dreport.items() if name.startswith("densify") or name == "scan")
    d_bytes = 748.0 * before + 812.0 * after + 8.0 * before
    compaction = {"gaussians_in": before, "gaussians_out": after, "kernels_us": round(d_us, 1),
                  "gb_s": round(d_bytes / (d_us * 1e-6) / 1e9, 1),
                  "frac_of_measured": round(d_bytes / (d_us * 1e-6) / 1e9 / hbm_peak, 3),
                  "kernels": {k: round(1000 * t / c, 2) for k, (c, t) in dreport.items()}}

    result = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded planes-and-boxes scene; "
        "the reference's Tanks and Temples photos are not available)",
        "config": config(args, world), "e2e": {k: (round(v, 2) if isinstance(v, float) else v) for k, v in e2e.items()},
        "gpu_launches": launches, "roofline": roofline, "clocks": clocks,
        "kernels": {k: {"avg_us": round(v["avg_us"], 2), "share": round(v["share"], 4), "launches": v["launches"]}
                    for k, v in sorted(kernels.items(), key=lambda kv: -kv[1]["share"])},
        "dominant_kernel": dominant, "blend": blend, "pairs": pairs, "gaussians": n,
        "uncaptured_step": uncaptured, "held_out": held_out, "compaction": compaction,
    }
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args, raw, sh, views_host(views), cams, samples=1)
    trainer.destroy()
    for v in views:
        v.image.destroy()
    for p in pinned:
        p.free()
    # The second measure of the path: learned against plain densification at the
    # ~1.1M-Gaussian scale (rank 0 of a replica run; minutes).
    if rank == 0 and not args.no_densify_comparison:
        result["densify_comparison"] = densify_comparison(device, args)
    device.destroy()
    return result


def held_out_views(args):
    from diorama_gb300 import scenes

    _train, held = scenes.ring_cameras()
    return held


def measure_held_out(device, renderer, held, repeats: int) -> dict:
    """Frames/s of the 37 held-out views: batched (autotuned, graph replay) and
    one encode() per view, with the batched images checked against the per-view
    ones."""
    W, H = held[0].viewport
    n = len(held)
    bg = (0.0, 0.0, 0.0)
    targets = device.createBuffer(n * W * H * 4)
    tuned = renderer.tuneViews(held, bg, targets)
    renderer.renderViews(held, bg, targets)
    device.synchronize()
    start, end = device.event(), device.event()
    reps = max(1, repeats // 4)
    start.record()
    for _ in range(reps):
        renderer.renderViews(held, bg, targets)
    end.record()
    batched = n * reps / (start.elapsed_ms(end) / 1000.0)
    tex = device.createTexture(W, H)
    for cam in held[:2]:
        renderer.encode(None, tex, cam, bg)
        renderer.afterSubmit()
    start.record()
    for _ in range(reps):
        for cam in held:
            renderer.encode(None, tex, cam, bg)
    end.record()
    per_view = n * reps / (start.elapsed_ms(end) / 1000.0)
    # Where a batched render's time goes: one render launched directly (no graph),
    # each kernel bracketed by events.
    renderer.setViewBatching(tuned["batch"], tuned["coopMin"], False)
    renderer.renderViews(held, bg, targets)
    device.synchronize()
    device.setKernelTiming(True)
    device.kernelTimingReport()
    renderer.renderViews(held, bg, targets)
    report = device.kernelTimingReport()
    device.setKernelTiming(False)
    renderer.setViewBatching(tuned["batch"], tuned["coopMin"], True)
    kernels = {k: {"us": round(t * 1000, 1), "launches": c} for k, (c, t) in
               sorted(report.items(), key=lambda kv: -kv[1][1])}
    # The last view's image both ways.
    renderer.encode(None, tex, held[-1], bg)
    renderer.afterSubmit()
    same = bool(np.array_equal(tex.buffer.read(np.uint8), targets.read(np.uint8, offset=(n - 1) * W * H * 4)))
    tex.destroy()
    targets.destroy()
    # The tuner's last three candidates are the larger blend tiles at the best
    # 16x16 candidate's batch and threshold.
    secs = tuned["seconds"]
    by_tile = {"16x16": min(secs[:-3]), "32x16": secs[-3], "16x32": secs[-2], "32x32": secs[-1]}
    return {"views": n, "frames_per_s": round(batched, 1), "per_view_frames_per_s": round(per_view, 1),
            "batch": tuned["batch"], "coop_min": tuned["coopMin"], "blend_tile": "%dx%d" % tuned["tile"],
            "tuner_candidates": len(secs),
            "tuner_frames_per_s_by_blend_tile": {k: round(n / v, 1) for k, v in by_tile.items()},
            "last_view_identical": same, "kernels_one_batch": kernels}


def views_host(views):
    return [v.image.read() for v in views[:4]]


def cpu_baseline(args, raw, sh, photos, cams, samples: int) -> dict:
    """The oracle's optimize() step on the same workload, timed on the host cores."""
    import oracle

    params = np.ascontiguousarray(raw, np.float32).reshape(-1).copy()
    shc = np.ascontiguousarray(sh, np.float32).reshape(-1).copy()
    n = params.size // 16
    moments = np.zeros(n * 61 * 2, np.float32)
    stats = np.zeros(n * 4, np.float32)
    gaussians = oracle.activate(params)
    W, H = cams[0].viewport
    bg = np.zeros(3, np.float32)
    times = []
    for s in range(samples):
        cam = oracle.camera_array(cams[s % len(photos)].view, cams[s % len(photos)].proj, (W, H))
        photo = np.ascontiguousarray(photos[s % len(photos)], np.uint8).reshape(-1)
        t0 = time.perf_counter()
        frame = oracle.render(cam, bg, gaussians, shc, 3)
        _, pg, _ = oracle.loss(frame["pixel_color"], photo, W, H)
        sg = oracle.rasterize_backward(cam, bg, frame["splats"], frame, pg)
        gg, sgr = oracle.preprocess_backward(cam, gaussians, shc, 3, frame["splats"], sg)
        oracle.accumulate_stats(frame["splats"], sg, (W, H), stats)
        ap = np.array([0.1, 0.001, 1.6e-4 * 4, 0.025, 0.005, 0.001, 0.0025, 0.0025 / 20, W, H], np.float32)
        oracle.adam_step(ap, params, shc, moments, gg, sgr, gaussians)
        times.append(time.perf_counter() - t0)
    sec = statistics.median(times)
    return {"value": round(1.0 / sec, 4), "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{samples} full optimize() step(s) of the same workload ({n} Gaussians, {W}x{H}) by the C "
                      f"oracle with OpenMP; median {sec:.2f} s"}


def run_reference(args, rank, world, group):
    """The reference's algorithm on the host (the oracle), rank 0 only."""
    if rank != 0:
        return None
    import oracle
    from diorama_gb300 import activate

    raw, sh, truth_raw, truth_sh, cams = build_scene(args)
    W, H = cams[0].viewport
    truth = activate(truth_raw)
    photos = []
    for cam in cams[: max(1, min(4, len(cams)))]:
        c = oracle.camera_array(cam.view, cam.proj, (W, H))
        photos.append(oracle.render(c, np.zeros(3, np.float32), truth, truth_sh.reshape(-1), 3)["rgba8"])
    base = cpu_baseline(args, raw, sh, photos, cams, samples=args.warmup)  # warm-up and per-step estimate
    per_step = 1.0 / base["value"]
    budget = 180.0
    steps = max(1, min(args.steps, int(budget / per_step)))
    timed = cpu_baseline(args, raw, sh, photos, cams, samples=steps)
    value = timed["value"]
    timed["sample"] = (f"{steps} of {args.steps} requested full optimize() steps (capped at ~{int(budget)} s of CPU "
                       f"work), {timed['sample']}")
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": round(1000.0 / value, 2), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded planes-and-boxes scene)", "config": config(args, world),
        "impl": "reference", "cpu_baseline": timed,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is TypeScript + WGSL for a browser's WebGPU; its algorithm runs here as the C oracle "
                "on the host cores",
    }


def run_sort_stress(args, rank, local):
    """1.1M random Gaussians over [-3, 3]^3 at 1960x1090 through the
    reference-structured TileRasterizer: tile counts, the exclusive scan, 64-bit (tile, depth) keys, the 6-pass radix sort and the
    ranges, each kernel timed with CUDA events; GB/s of the algorithmic bytes
    against the measured HBM peak. (The keys, permutation and ranges are checked
    bit for bit against the oracle by tests/test_gpu_workloads.py.)"""
    if rank != 0:
        return None
    from diorama_gb300 import Device, GaussianRenderer, TileRasterizer, scenes
    import oracle

    raw, sh, camera = scenes.random_scene_1m(0)
    act = scenes.activate64(raw).astype(np.float32)
    device = Device(local)
    r = GaussianRenderer(device)
    r.setGaussians(act.reshape(-1), {"rest": sh.reshape(-1), "degree": 3})
    r.encode(None, None, camera, (0, 0, 0))
    r.afterSubmit()
    cam = oracle.camera_array(camera.view, camera.proj, camera.viewport)
    camera_buf = device.upload(cam)
    n = act.shape[0]
    tr = TileRasterizer(device, camera_buf, r.splatBuffer, n, r.tiles.pairCapacity)
    for _ in range(max(args.warmup, 3)):
        tr.encode(None, None, camera.viewport, (0, 0, 0))
        tr.afterSubmit()
    device.synchronize()
    device.setKernelTiming(True)
    device.kernelTimingReport()
    for _ in range(args.steps):
        tr.encode(None, None, camera.viewport, (0, 0, 0))
    device.synchronize()
    report = device.kernelTimingReport()
    device.setKernelTiming(False)
    keys = tr.lastPairCount
    tiles = math.ceil(camera.viewport[0] / 16) * math.ceil(camera.viewport[1] / 16)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    per = {name: 1000 * t / c for name, (c, t) in report.items()}  # us per launch
    launches = {name: c // args.steps for name, (c, _t) in report.items()}
    sort_us = per.get("sort_histogram", 0) * launches.get("sort_histogram", 0) + \
        per.get("sort_pass", 0) * launches.get("sort_pass", 0)
    sort_bytes = 152.0 * keys  # 6 passes x (read + write 8 B key + 4 B value) + 8 B of histogram reads
    scan_bytes = 8.0 * n
    ranges_bytes = 8.0 * keys + 8.0 * tiles

    def frac(b, us):
        return {"gb_s": round(b / (us * 1e-6) / 1e9, 1), "frac_of_measured": round(b / (us * 1e-6) / 1e9 / hbm, 3),
                "us": round(us, 2)}

    # The scan at 12M values too (at 1.1M it is launch-bound): PrefixSum over random
    # tile counts, timed with CUDA events. Its 48 MB fit in L2, so a 256 MB buffer
    # is cleared after each upload of the values and before the timed scan.
    from diorama_gb300 import PrefixSum
    big = 12_000_000
    counts = np.random.default_rng(5).integers(0, 9, big).astype(np.uint32)
    cbuf = device.upload(counts)
    flush = device.createBuffer(256 << 20)
    scan12 = PrefixSum(device, cbuf, big)
    for _ in range(3):
        cbuf.write(counts)
        scan12.encode()
    t_scan = 0.0
    for _ in range(args.steps):
        cbuf.write(counts)
        device.createCommandEncoder().clearBuffer(flush)
        e0, e1 = device.event(), device.event()
        e0.record()
        scan12.encode()
        e1.record()
        device.synchronize()
        t_scan += e0.elapsed_ms(e1)
    scan12_us = 1000 * t_scan / args.steps
    scan12.destroy()
    cbuf.destroy()
    flush.destroy()

    # CPU numbers for the same primitives, the reference's algorithms: the oracle's
    # stable LSD radix sort of (tile << 32 | depth bits) keys and its sequential
    # exclusive scan (single thread), and numpy's stable argsort, on samples.
    rng = np.random.default_rng(6)
    sample = 2_000_000
    sk = (rng.integers(0, tiles, sample).astype(np.uint64) << np.uint64(32)) | \
        rng.integers(0, 2**32, sample).astype(np.uint64)
    sv = np.arange(sample, dtype=np.uint32)
    t0 = time.perf_counter()
    oracle.lib().or_radix_sort(sk.copy(), sv.copy(), sample, 16)
    cpu_sort = sample / (time.perf_counter() - t0)
    t0 = time.perf_counter()
    np.argsort(sk, kind="stable")
    cpu_argsort = sample / (time.perf_counter() - t0)
    sc = counts[:n].copy()
    t0 = time.perf_counter()
    oracle.lib().or_exclusive_scan(sc, n)
    cpu_scan = n / (time.perf_counter() - t0)

    result = {
        "metric": "sort/scan/ranges keys/s", "workload": "1.1M random Gaussians in [-3,3]^3 at 1960x1090, "
        "16x16 tiles, reference-structured tile stage", "keys": keys, "gaussians": n, "tiles": tiles,
        "steps": args.steps, "peak_hbm_gbs": hbm,
        "sort": frac(sort_bytes, sort_us), "scan": frac(scan_bytes, per.get("scan", 0.0)),
        "scan_12M": frac(8.0 * big, scan12_us),
        "find_ranges": frac(ranges_bytes, per.get("find_ranges", 0.0)),
        "kernels": {k: {"avg_us": round(v, 2), "launches_per_frame": launches[k]} for k, v in per.items()},
        "gpu_keys_per_s": round(keys / (sort_us * 1e-6), 1),
        "cpu_baseline": {
            "sort_keys_per_s": round(cpu_sort, 1), "sort_kind": "the oracle's stable 6-pass LSD radix sort, 1 thread",
            "argsort_keys_per_s": round(cpu_argsort, 1), "argsort_kind": "numpy stable argsort of u64 keys, 1 thread",
            "scan_values_per_s": round(cpu_scan, 1), "scan_kind": "the oracle's sequential exclusive scan, 1 thread",
            "sample": f"{sample:,} random (tile < {tiles}) << 32 | depth-bits keys; {n:,} counts", "cores": 1},
    }
    tr.destroy()
    camera_buf.destroy()
    r.destroy()
    device.destroy()
    return result


def run_profile_step(args, rank, local):
    """One training step of the headline workload (direct launches), bracketed for a
    profiler started with collection off (`ncu --profile-from-start off`), after
    --warmup steps. Prints the step's work: the blend's evaluations (the forward's
    pixel_last summed over the frame's pixels), pairs and Gaussians, with the
    step's kernel times from CUDA events, so that a profiler's per-kernel counters
    can be divided by the work of the same launch."""
    if rank != 0:
        return None
    from diorama_gb300 import DEFAULT_SETTINGS, Device, GaussianRenderer, RawGaussians, Trainer, TrainingView, activate

    raw, sh, truth_raw, truth_sh, cams = build_scene(args)
    device = Device(local)
    W, H = cams[0].viewport
    photographer = GaussianRenderer(device)
    photographer.setGaussians(activate(truth_raw), {"rest": truth_sh.reshape(-1), "degree": 3})
    views = []
    for k, cam in enumerate(cams):
        tex = device.createTexture(W, H)
        photographer.encode(None, tex, cam, (0, 0, 0))
        views.append(TrainingView(f"view {k}", cam, tex))
    device.synchronize()
    photographer.destroy()
    settings = replace(DEFAULT_SETTINGS, extent=4.0, shDegreeInterval=1, densifyUntil=0)
    trainer = Trainer(device, RawGaussians(raw.reshape(-1), sh.reshape(-1)), views, settings)
    for _ in range(args.warmup):
        trainer.step()
    trainer.renderer.afterSubmit()
    view = trainer.nextView()
    device.setKernelTiming(True)
    device.kernelTimingReport()
    device.profile(True)
    trainer.step()
    device.profile(False)
    report = device.kernelTimingReport()
    device.setKernelTiming(False)
    last = trainer.renderer.pixelLastBuffer.read(np.uint32)[: W * H]
    result = {"workload": "one training step for a profiler", "gaussians": trainer.count, "viewport": [W, H],
              "view": view, "warmup_steps": args.warmup, "pairs": trainer.renderer.tiles.lastPairCount,
              "blend_evaluations": int(last.astype(np.int64).sum()),
              "drawn_gaussians": int(np.count_nonzero(
                  trainer.renderer.splatBuffer.read(np.float32)[: trainer.count * 12].reshape(-1, 12)[:, 3])),
              "kernels_us": {k: round(1000 * t / c, 2) for k, (c, t) in report.items()}}
    trainer.destroy()
    for v in views:
        v.image.destroy()
    device.destroy()
    return result


def run_mlp_inference(args, rank, local):
    """The learned densification's inference (DensifyMLP.predict, tcgen05) on
    `--candidates` random candidates with random weights, resident on the GPU:
    --steps calls timed with CUDA events after --warmup."""
    if rank != 0:
        return None
    import torch

    torch.cuda.set_device(local)
    from diorama_gb300 import DensifyMLP, Device
    from diorama_gb300.training import MLP_FEATURES, MLP_PARAMS

    device = Device(local)
    rng = np.random.default_rng(1)
    mlp = DensifyMLP(device, seed=1)
    w = rng.normal(0, 0.3, MLP_PARAMS + 24).astype(np.float32)
    w[MLP_PARAMS + 12:] = 1.0  # the input normalization's scales
    mlp.setWeights(w)
    n = args.candidates
    features = device.upload(rng.normal(0, 1.5, (n, MLP_FEATURES)).astype(np.float32))
    out = device.createBuffer(max(4, n * 4))
    for _ in range(args.warmup):
        mlp.predict(features, n, out)
    device.synchronize()
    start, end = device.event(), device.event()
    start.record()
    for _ in range(args.steps):
        mlp.predict(features, n, out)
    end.record()
    us = start.elapsed_ms(end) * 1000.0 / args.steps
    flops = 2.0 * (16 * 64 + 64 * 64 + 64 * 16) * n  # the padded product shapes
    result = {"metric": "densification MLP inference", "candidates": n, "us_per_call": round(us, 1),
              "tflops_padded": round(flops / us / 1e6, 1), "steps": args.steps, "warmup": args.warmup,
              "device_errors": device.check()}
    features.destroy()
    out.destroy()
    mlp.destroy()
    return result


def run_knn(args, rank, local):
    """The starting Gaussians' neighbour distances (src/loadDataset.ts:124-149) of
    a structure-from-motion-like cloud (clusters, a plane, 1% far outliers,
    duplicates): the grid search on the GPU with the points resident (value) and
    through the host API with its copies (e2e); the oracle's brute force, the
    reference's algorithm, timed on a sample of query points on the host cores.
    (The results are checked bit for bit against the brute force by
    tests/test_gpu_init.py.)"""
    if rank != 0:
        return None
    from diorama_gb300 import Device, scenes
    from diorama_gb300.dataset import meanNeighborDistance2, meanNeighborDistance2Buffers
    import oracle

    n = args.knn_points
    positions = scenes.clustered_cloud(n, 3)
    device = Device(local)
    points = np.zeros((n, 4), np.float32)
    points[:, :3] = positions.reshape(-1, 3)
    pbuf = device.upload(points)
    out = device.createBuffer(n * 4)
    for _ in range(args.warmup):
        meanNeighborDistance2Buffers(device, pbuf, n, out)
    device.synchronize()
    device.setKernelTiming(True)
    device.kernelTimingReport()
    walls = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        meanNeighborDistance2Buffers(device, pbuf, n, out)
        device.synchronize()
        walls.append(time.perf_counter() - t0)
    report = device.kernelTimingReport()
    device.setKernelTiming(False)
    e2e = []
    for _ in range(max(2, args.steps // 2)):
        t0 = time.perf_counter()
        meanNeighborDistance2(device, positions)
        e2e.append(time.perf_counter() - t0)
    sample = 2000
    which = np.random.default_rng(7).choice(n, sample, replace=False).astype(np.uint32)
    t0 = time.perf_counter()
    oracle.mean_neighbor_distance2_of(positions, which)
    cpu_s = time.perf_counter() - t0
    wall = statistics.median(walls)
    result = {
        "metric": "nearest-neighbour distances", "value": round(n / wall, 1), "unit": "points/s",
        "ms_per_call": round(wall * 1e3, 3), "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n:,} points: 80% in clusters (sigma 0.01-0.5), 15% on a plane, 5% outliers "
                               "(sigma 60), 0.5% duplicates; 3 nearest neighbours each"},
        "steps": args.steps, "warmup": args.warmup,
        "kernels": {k: {"avg_us": round(1000 * t / c, 2), "launches_per_call": c // args.steps}
                    for k, (c, t) in report.items()},
        "e2e": {"value": round(n / statistics.median(e2e), 1), "unit": "points/s",
                "h2d_bytes_per_step": n * 12, "d2h_bytes_per_step": n * 4},
        "cpu_baseline": {"value": round(sample / cpu_s, 1), "unit": "points/s", "cores": oracle.num_threads(),
                         "kind": "port", "sample": f"brute force (the reference's algorithm) for {sample} query "
                                                   f"points over all {n:,}"},
    }
    pbuf.destroy()
    out.destroy()
    device.destroy()
    return result


def densify_schedule(steps: int, threshold: float):
    """The reference's schedule (src/trainer.ts:65-82, densification from step 500
    to 15,000 every 100 steps, opacity reset every 3,000, SH degree +1 every
    1,000, position learning rate decaying over 30,000 steps) scaled to `steps`,
    on the planes-and-boxes scene's extent 4 with config 1's opacity lr 5e-2 and
    the given gradient threshold. Returns the settings and the label horizon (1,000
    steps, scaled)."""
    from diorama_gb300 import DEFAULT_SETTINGS

    f = steps / 30_000
    settings = replace(DEFAULT_SETTINGS, extent=4.0, opacityLr=0.05, densifyGradThreshold=threshold,
                       positionLrSteps=steps, shDegreeInterval=max(1, round(1000 * f)),
                       densifyFrom=round(500 * f), densifyUntil=round(15_000 * f),
                       densifyInterval=max(1, round(100 * f)), opacityResetInterval=max(1, round(3000 * f)))
    return settings, max(1, round(1000 * f))


def time_to_target(curve: list, target: float):
    """Training seconds at the first evaluation from which the held-out PSNR stays
    at or above the target (the opacity resets pull it down while densifying)."""
    at = None
    for step, seconds, psnr, _count in curve:
        if psnr < target:
            at = None
        elif at is None:
            at = seconds
    return at


def densify_comparison(device, args) -> dict:
    """Learned against plain densification (configs 1 and 4) on the
    planes-and-boxes scene: 500k ground-truth Gaussians on 40 planes and boxes,
    263 training and 37 held-out 980x545 views, training from 100k noisy surface
    samples on the reference's schedule scaled to --densify-steps, with
    densification threshold --densify-threshold (1.5e-5 by default: the plain
    path grows to ~1.2M Gaussians).

    For each of --densify-seeds starting sets: a plain run that logs every
    clone/split candidate's 12 features and whether any of its children is still
    alive a (scaled) 1,000 steps later; then a model (MLP 12 -> 64 -> 64 -> 2,
    BF16 tensor-core kernels, AdamW lr 1e-3, 5 epochs, both labels weighted
    equally) trained on the OTHER seeds' labels, and a learned run from the same
    start, in which the model decides the plain rule's candidates where it is
    confident (max(p, 1 - p) >= 0.6) and the threshold rule decides the rest.
    Per seed: held-out PSNR and SSIM, final Gaussians, training wall time
    (evaluations excluded) and the time to reach, for good, the plain run's final
    PSNR minus 0.1 dB; across seeds, their means and ranges."""
    from diorama_gb300 import DensifyMLP, GaussianRenderer, RawGaussians, Trainer, TrainingView, activate, scenes

    steps, threshold, seeds = args.densify_steps, args.densify_threshold, list(range(1, args.densify_seeds + 1))
    truth_raw, truth_sh = scenes.surface_scene(GROUND_TRUTH, TRUTH_SEED)
    train_cams, held_cams = scenes.ring_cameras()
    W, H = train_cams[0].viewport
    photographer = GaussianRenderer(device)
    photographer.setGaussians(activate(truth_raw), {"rest": truth_sh.reshape(-1), "degree": 3})

    def photos(cams, prefix):
        out = []
        for k, cam in enumerate(cams):
            tex = device.createTexture(W, H)
            photographer.encode(None, tex, cam, (0, 0, 0))
            out.append(TrainingView(f"{prefix} {k}", cam, tex))
        return out

    train_views, held_views = photos(train_cams, "train"), photos(held_cams, "held-out")
    device.synchronize()
    photographer.destroy()
    settings, horizon = densify_schedule(steps, threshold)
    every = max(1, steps // 20)

    def run(seed, mlp=None, log=False):
        raw, sh = scenes.surface_scene(100_000, seed, noise=0.01)
        t = Trainer(device, RawGaussians(raw.reshape(-1), sh.reshape(-1)), train_views, settings)
        t.setGraph(True)
        if log:
            t.setDensifyLog(True, horizon)
        if mlp is not None:
            t.setDensifyMLP(mlp, 0.6)
        curve, train_s, done = [], 0.0, 0
        while done < steps:
            n = min(every, steps - done)
            device.synchronize()
            t0 = time.perf_counter()
            for _ in range(n):
                t.step()
            device.synchronize()
            train_s += time.perf_counter() - t0
            done += n
            curve.append([done, round(train_s, 3), round(t.evaluate(held_views, False)["psnr"], 3), t.count])
        final = t.evaluate(held_views, True)
        result = {"seed": seed, "train_s": round(train_s, 2), "steps_per_s": round(steps / train_s, 1),
                  "psnr": round(final["psnr"], 3), "ssim": round(final["ssim"], 4), "gaussians": t.count,
                  "densifications": len(t.densifications), "curve": curve}
        if log:
            f, y, pending = t.takeDensifySamples()
            result["logged"] = {"samples": int(y.size), "children_alive_rate": round(float(y.mean()), 4)
                                if y.size else None, "unlabelled": pending}
        else:
            f = y = None
        if mlp is not None:
            result["mlp"] = t.densifyMLPStats
        t.destroy()
        return result, f, y

    plain, samples = {}, {}
    for seed in seeds:
        plain[seed], f, y = run(seed, log=True)
        samples[seed] = (f, y)
    learned, models = {}, {}
    for seed in seeds:
        others = [o for o in seeds if o != seed] or [seed]
        f = np.concatenate([samples[o][0] for o in others])
        y = np.concatenate([samples[o][1] for o in others])
        mlp = DensifyMLP(device, seed=7)
        t0 = time.perf_counter()
        losses = mlp.train(f, y, epochs=5, batch=1024, lr=1e-3, weightDecay=0.01, seed=7,
                           balanceClasses=not args.unbalanced)
        device.synchronize()
        fit_s = time.perf_counter() - t0
        # Inference time on every candidate of one run (the model runs once per
        # densification, on that densification's candidates), CUDA events.
        fb = device.upload(np.ascontiguousarray(samples[seed][0], np.float32))
        out = device.createBuffer(max(4, samples[seed][1].size * 4))
        mlp.predict(fb, samples[seed][1].size, out)
        start, end = device.event(), device.event()
        start.record()
        for _ in range(10):
            mlp.predict(fb, samples[seed][1].size, out)
        end.record()
        predict_us = start.elapsed_ms(end) * 100.0  # per call
        accuracy = float(np.mean((mlp.predictHost(samples[seed][0]) >= 0.5) == (samples[seed][1] == 1)))
        fb.destroy()
        out.destroy()
        learned[seed], _, _ = run(seed, mlp=mlp)
        models[seed] = {"trained_on_seeds": others, "samples": int(y.size), "loss": [round(x, 4) for x in losses],
                        "fit_s": round(fit_s, 3), "accuracy_on_this_seed": round(accuracy, 4),
                        "predict_us_for_all_candidates_of_a_run": round(predict_us, 1),
                        "candidates_per_run": int(samples[seed][1].size)}
        mlp.destroy()
    per_seed = []
    for seed in seeds:
        p, q = plain[seed], learned[seed]
        target = p["psnr"] - 0.1
        per_seed.append({
            "seed": seed, "target_psnr": round(target, 3),
            "plain": {k: p[k] for k in ("psnr", "ssim", "gaussians", "train_s", "steps_per_s", "logged")}
            | {"time_to_target_s": time_to_target(p["curve"], target)},
            "learned": {k: q[k] for k in ("psnr", "ssim", "gaussians", "train_s", "steps_per_s", "mlp")}
            | {"time_to_target_s": time_to_target(q["curve"], target)},
            "model": models[seed],
            "curves": {"plain": p["curve"], "learned": q["curve"]}})

    def stats(values):
        values = [v for v in values if v is not None]
        if not values:
            return None
        return {"mean": round(float(np.mean(values)), 4), "min": round(float(min(values)), 4),
                "max": round(float(max(values)), 4)}

    def ratio(a, b):
        return a / b if a is not None and b else None

    summary = {
        "psnr_learned_minus_plain_db": stats([r["learned"]["psnr"] - r["plain"]["psnr"] for r in per_seed]),
        "ssim_learned_minus_plain": stats([r["learned"]["ssim"] - r["plain"]["ssim"] for r in per_seed]),
        "gaussians_learned_over_plain": stats([r["learned"]["gaussians"] / r["plain"]["gaussians"] for r in per_seed]),
        "train_s_learned_over_plain": stats([r["learned"]["train_s"] / r["plain"]["train_s"] for r in per_seed]),
        "time_to_target_learned_over_plain": stats(
            [ratio(r["learned"]["time_to_target_s"], r["plain"]["time_to_target_s"]) for r in per_seed]),
        "learned_within_0.1_db_or_better": sum(r["learned"]["psnr"] >= r["target_psnr"] for r in per_seed),
        "seeds": len(per_seed),
    }
    for v in train_views + held_views:
        v.image.destroy()
    return {"metric": "time to held-out PSNR, learned vs plain densify", "unit": "s",
            "workload": f"planes-and-boxes scene (500k ground truth), 263 + 37 views at 980x545, {steps} steps "
                        f"from 100k noisy surface samples, densify threshold {threshold:g} (the reference's "
                        f"30,000-step schedule scaled by {steps / 30_000:g})",
            "schedule": {"steps": steps, "densify_from": settings.densifyFrom, "densify_until": settings.densifyUntil,
                         "densify_interval": settings.densifyInterval,
                         "opacity_reset_interval": settings.opacityResetInterval,
                         "sh_degree_interval": settings.shDegreeInterval, "label_horizon": horizon,
                         "grad_threshold": threshold, "opacity_lr": settings.opacityLr},
            "summary": summary, "per_seed": per_seed}


def run_densify_experiment(args, rank, local):
    """--workload densify: the learned-vs-plain comparison alone."""
    if rank != 0:
        return None
    from diorama_gb300 import Device

    device = Device(local)
    result = densify_comparison(device, args)
    device.destroy()
    return result


def free_port() -> int:
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_replicas(n: int, argv: list[str], script: str | None = None) -> int:
    """`bench.py --gpus N` started directly (not under torchrun): start N replica
    processes, one per GPU, with the environment torchrun would give them (RANK,
    LOCAL_RANK, WORLD_SIZE, MASTER_ADDR 127.0.0.1, MASTER_PORT). Rank 0's output
    passes through; the others' is dropped. Returns the first nonzero exit code."""
    port = free_port()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, script or str(Path(__file__).resolve()), *argv], env=env,
                                      stdout=None if r == 0 else subprocess.DEVNULL))
    codes = [p.wait() for p in procs]
    return next((c for c in codes if c != 0), 0)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_replicas(args.gpus, sys.argv[1:]))
    rank, world, local, group = dist_setup(args)
    if world != args.gpus and rank == 0:
        print(f"note: --gpus {args.gpus} but {world} process(es) were launched; measuring {world}", file=sys.stderr)
    if args.workload == "sort":
        result = run_sort_stress(args, rank, local) if args.impl == "ours" else None
    elif args.workload == "densify":
        result = run_densify_experiment(args, rank, local) if args.impl == "ours" else None
    elif args.workload == "knn":
        result = run_knn(args, rank, local) if args.impl == "ours" else None
    elif args.workload == "profile":
        result = run_profile_step(args, rank, local) if args.impl == "ours" else None
    elif args.workload == "mlp":
        result = run_mlp_inference(args, rank, local) if args.impl == "ours" else None
    elif args.impl == "reference":
        result = run_reference(args, rank, world, group)
    else:
        result = run_ours(args, rank, world, local, group)
    if rank == 0 and result is not None:
        print(json.dumps(result), flush=True)
    if group is not None:
        group.destroy_process_group()


if __name__ == "__main__":
    main()

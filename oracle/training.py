"""The oracle's training loop, FOR TESTS ONLY: a CPU restatement of the
reference's Trainer.step() (src/trainer.ts:192-252) over the oracle's per-step
pieces (oracle.c: render, loss, both backward passes, statistics, Adam,
densification, opacity reset).

Test infrastructure like the rest of this package: only tests/ use it, as the
checker of the GPU trainer's schedule step by step. It follows the reference's
host logic statement by statement:
- the view order: every view once in a mulberry32(1) Fisher-Yates order, then
  reshuffle (src/trainer.ts:395-404);
- the SH degree rises before step t renders when t is a multiple of
  shDegreeInterval, up to 3 (src/trainer.ts:195-197);
- a densification step (t > densifyFrom, t % densifyInterval == 0, t <
  densifyUntil) takes no Adam step, and Adam's bias correction counts only the
  steps that ran Adam (src/trainer.ts:198-201,209,217-218);
- the position learning rate decays log-linearly over positionLrSteps and
  scales with the extent (src/trainer.ts:210-212);
- statistics accumulate on every step (src/trainer.ts:232-236);
- maintain() densifies (pruning large Gaussians once past the first opacity
  reset) and then resets opacities when due (src/trainer.ts:243,248-252).
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import (FLOATS_PER_GAUSSIAN, MOMENT_SLOTS, accumulate_stats, adam_step, densify, loss, preprocess_backward,
               rasterize_backward, render, reset_opacity)
from . import activate as activate_f32

SH_C0 = 0.28209479177387814


def mulberry32(seed: int):
    """src/random.ts:3-12."""
    state = seed & 0xFFFFFFFF

    def next_value() -> float:
        nonlocal state
        state = (state + 0x6D2B79F5) & 0xFFFFFFFF
        t = state
        t = ((t ^ (t >> 15)) * (t | 1)) & 0xFFFFFFFF
        t ^= (t + (((t ^ (t >> 7)) * (t | 61)) & 0xFFFFFFFF)) & 0xFFFFFFFF
        return ((t ^ (t >> 14)) & 0xFFFFFFFF) / 4294967296

    return next_value


def activate_host(params: np.ndarray) -> np.ndarray:
    """The constructor's activation on the CPU in double precision, stored as
    float32 (src/trainer.ts:449-461)."""
    p = np.asarray(params, np.float32).astype(np.float64).reshape(-1, FLOATS_PER_GAUSSIAN)
    out = np.zeros_like(p)
    out[:, 0:3] = p[:, 0:3]
    out[:, 4:7] = np.exp(p[:, 4:7])
    out[:, 12:15] = 0.5 + SH_C0 * p[:, 12:15]
    out[:, 3] = 1 / (1 + np.exp(-p[:, 3]))
    out[:, 8:12] = p[:, 8:12]
    return out.astype(np.float32).reshape(-1)


@dataclass
class Settings:
    """TrainingSettings (src/trainer.ts:37-63), DEFAULT_SETTINGS' values."""

    extent: float = 1.0
    positionLrSteps: float = 30_000
    positionLr: tuple = (0.00016, 0.0000016)
    opacityLr: float = 0.025
    scaleLr: float = 0.005
    rotationLr: float = 0.001
    colorLr: float = 0.0025
    shLr: float = 0.0025 / 20
    shDegreeInterval: int = 1000
    densifyFrom: int = 500
    densifyUntil: int = 15_000
    densifyInterval: int = 100
    densifyGradThreshold: float = 0.0002
    percentDense: float = 0.01
    minOpacity: float = 0.005
    opacityResetInterval: int = 3000
    background: tuple = (0.0, 0.0, 0.0)


class Trainer:
    """The reference's training loop on the CPU. views: (camera array of 36
    floats, rgba8 photo of the viewport's size) pairs."""

    def __init__(self, params: np.ndarray, sh: np.ndarray, views, settings: Settings):
        self.params = np.ascontiguousarray(params, np.float32).reshape(-1).copy()
        self.sh = np.ascontiguousarray(sh, np.float32).reshape(-1).copy()
        self.count = self.params.size // FLOATS_PER_GAUSSIAN
        self.views = list(views)
        self.settings = settings
        self.gaussians = activate_host(self.params)
        self.moments = np.zeros(self.count * MOMENT_SLOTS * 2, np.float32)
        self.stats = np.zeros(self.count * 4, np.float32)
        self.iteration = 0
        self.shDegree = 0
        self.adamSteps = 0
        self.random = mulberry32(1)
        self.queue: list[int] = []
        self.densifications: list[tuple] = []  # (step, before, after, kept, cloned, split, removed)
        self.due = None
        self.last_loss = None
        self.last_view = None

    def next_view(self) -> int:
        if not self.queue:
            self.queue = list(range(len(self.views)))
            for i in range(len(self.queue) - 1, 0, -1):
                j = math.floor(self.random() * (i + 1))
                self.queue[i], self.queue[j] = self.queue[j], self.queue[i]
        return self.queue.pop()

    def step(self) -> None:
        self.optimize()
        self.maintain()

    def optimize(self) -> None:
        s = self.settings
        t = self.iteration = self.iteration + 1
        if t % s.shDegreeInterval == 0 and self.shDegree < 3:
            self.shDegree += 1
        densifying = t < s.densifyUntil
        densify_now = densifying and t > s.densifyFrom and t % s.densifyInterval == 0
        v = self.last_view = self.next_view()
        cam, photo = self.views[v]
        W, H = int(cam[32]), int(cam[33])
        bg = np.asarray(s.background, np.float32)
        frame = render(cam, bg, self.gaussians, self.sh, self.shDegree)
        self.last_loss, pixel_grads, _ = loss(frame["pixel_color"], photo, W, H)
        splat_grads = rasterize_backward(cam, bg, frame["splats"], frame, pixel_grads)
        ggrad, sgrad = preprocess_backward(cam, self.gaussians, self.sh, self.shDegree, frame["splats"], splat_grads)
        if not densify_now:
            self.adamSteps += 1
        progress = min(1.0, t / s.positionLrSteps)
        lr0, lr1 = s.positionLr
        position_lr = math.exp(math.log(lr0) * (1 - progress) + math.log(lr1) * progress) * s.extent
        ap = np.array([1 - 0.9 ** self.adamSteps, 1 - 0.999 ** self.adamSteps, position_lr, s.opacityLr, s.scaleLr,
                       s.rotationLr, s.colorLr, s.shLr, W, H], np.float32)
        accumulate_stats(frame["splats"], splat_grads, (W, H), self.stats)
        if not densify_now:
            adam_step(ap, self.params, self.sh, self.moments, ggrad, sgrad, self.gaussians)
        self.due = (densify_now, densifying and t % s.opacityResetInterval == 0)
        self.last_gradients = (ggrad, sgrad, splat_grads)

    def maintain(self) -> None:
        due, self.due = self.due, None
        if due and due[0]:
            self.densify(self.iteration > self.settings.opacityResetInterval)
        if due and due[1]:
            self.reset_opacity()

    def densify(self, prune_large: bool) -> None:
        s = self.settings
        dp = np.array([s.densifyGradThreshold, s.percentDense * s.extent, s.minOpacity,
                       0.1 * s.extent if prune_large else 0.0], np.float32)
        before = self.count
        params, sh, moments, tally = densify(self.params, self.stats, self.sh, self.moments, dp, self.iteration)
        after = params.size // FLOATS_PER_GAUSSIAN
        if after == 0:
            raise ValueError("Densification removed every Gaussian.")
        removed, kept, cloned, split = (int(x) for x in tally)
        self.densifications.append((self.iteration, before, after, kept, cloned, split, removed))
        self.params, self.sh, self.moments = params, sh, moments
        self.gaussians = activate_f32(params)  # the activate pipeline (src/shaders/adam.wgsl:60-78)
        self.stats = np.zeros(after * 4, np.float32)
        self.count = after

    def reset_opacity(self) -> None:
        reset_opacity(self.params, self.moments, self.gaussians)

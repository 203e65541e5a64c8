"""The GPU trainer against the oracle's training loop (oracle/training.py, a CPU
restatement of src/trainer.ts:192-252 and :395-404), step by step, and the
training step's fused backward + Adam kernel's gradients against the oracle's
preprocess backward.

The check scene is the reference's training check (src/checks/training.ts:
217-302: 60 Gaussians, 8 ring views at 96x96) with SH coefficients, the SH
degree rising every 60 steps, densification every 50 steps from step 50 to
250, and an opacity reset at step 150 (so the last two densifications also
prune large Gaussians). Exact: the view each step renders, the SH degree, Adam's
step counter, the densification records (counts and kept/cloned/split/removed
tallies) and the densified sets' SH and moments. Close: the per-step losses and
parameters (the backward's float atomics add in a run-dependent order).
"""

from __future__ import annotations

from dataclasses import asdict, replace

import numpy as np
import pytest

import oracle
from oracle import training as oracle_training
from diorama_gb300 import DEFAULT_SETTINGS, RawGaussians, Trainer
from helpers import GROUPS, cam_array, elementwise_errors
from test_gpu_training import ring_views, scrambled_start, truth_scene

pytestmark = pytest.mark.gpu

STEPS = 300
FREE_STEPS = 45  # before the first densification
SCHEDULE = dict(extent=3.85, shDegreeInterval=60, densifyFrom=40, densifyInterval=50, densifyUntil=260,
                densifyGradThreshold=2e-4, opacityResetInterval=150)


def gpu_state(gpu):
    n = gpu.count
    b = gpu.buffers
    return dict(params=b["params"].read(np.float32)[: n * 16].copy(),
                moments=gpu.readMoments(),
                stats=b["stats"].read(np.float32)[: n * 4].copy(),
                sh=gpu.renderer.shBuffer.read(np.float32)[: n * 45].copy(),
                gaussians=gpu.renderer.gaussianBuffer.read(np.float32)[: n * 16].copy())


def sync(cpu, state):
    """The oracle takes the GPU's state (so rounding differences do not accumulate)."""
    for k, v in state.items():
        setattr(cpu, k, v.copy())
    cpu.count = state["params"].size // 16


def test_training_loop_matches_oracle_loop(device):
    """Free-running for the first 45 steps (no densification yet), then in lockstep:
    the oracle takes the GPU's state before each step, and the GPU's statistics
    after optimize(), before maintain(). The backward's float atomics add in a
    run-dependent order, so the accumulated statistics differ by rounding from
    run to run, and a Gaussian whose mean gradient sits at the threshold could be
    densified on one side and not the other; with the same statistics the two
    must decide identically."""
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)
    sh = np.random.default_rng(7).normal(0, 0.05, 60 * 45).astype(np.float32)
    settings = replace(DEFAULT_SETTINGS, **SCHEDULE)
    gpu = Trainer(device, RawGaussians(params.copy(), sh.copy()), views, settings)
    cpu = oracle_training.Trainer(params, sh, [(cam_array(v.camera), v.image.read().reshape(-1)) for v in views],
                                  oracle_training.Settings(**asdict(settings)))
    mask = np.ones(16, bool)
    mask[[7, 15]] = False  # the densification stamps, compared exactly
    losses = []
    for step in range(1, STEPS + 1):
        lockstep = step > FREE_STEPS
        if lockstep:
            sync(cpu, gpu_state(gpu))
        view = gpu.nextView()
        gpu.optimize()
        cpu.optimize()
        assert view == cpu.last_view, step
        assert (gpu.iteration, gpu.shDegree, gpu.adamSteps) == (cpu.iteration, cpu.shDegree, cpu.adamSteps), step
        losses.append((gpu.lossValue(), cpu.last_loss))
        state = gpu_state(gpu)
        if lockstep:
            gp, cp = state["params"].reshape(-1, 16)[:, mask], cpu.params.reshape(-1, 16)[:, mask]
            # One step from the same state: measured at most 4.8e-7 (an opacity logit).
            assert np.abs(gp - cp).max() <= 1e-5, (step, np.abs(gp - cp).max())
            assert np.abs(state["sh"] - cpu.sh).max() <= 1e-5, step
            cpu.stats = state["stats"].copy()
        gpu.maintain()
        cpu.maintain()
        assert gpu.count == cpu.count, (step, gpu.count, cpu.count)
        if lockstep and cpu.densifications and cpu.densifications[-1][0] == step:
            after = gpu_state(gpu)  # the densified set: moments and SH copied exactly
            assert np.array_equal(after["moments"], cpu.moments) and np.array_equal(after["sh"], cpu.sh), step
            gp, cp = after["params"].reshape(-1, 16), cpu.params.reshape(-1, 16)
            assert np.array_equal(gp[:, [7, 15]], cp[:, [7, 15]])
            assert np.allclose(gp[:, mask], cp[:, mask], rtol=1e-5, atol=1e-6), step
        if step == FREE_STEPS:  # the free-running states after 45 steps
            gp, cp = state["params"].reshape(-1, 16)[:, mask], cpu.params.reshape(-1, 16)[:, mask]
            assert np.abs(gp - cp).max() <= 1e-5, np.abs(gp - cp).max()  # measured 7e-7
    got = [(d.step, d.before, d.after, d.kept, d.cloned, d.split, d.removed) for d in gpu.densifications]
    assert got == cpu.densifications
    assert len(got) == 5 and all(d[4] + d[5] > 0 for d in got) and any(d[3] > 0 for d in got), got
    assert cpu.adamSteps == STEPS - 5 and cpu.shDegree == 3

    g, c = np.array(losses).T
    rel = np.abs(g - c) / c
    assert rel[:FREE_STEPS].max() <= 1e-5, rel[:FREE_STEPS].max()  # measured 2.5e-7
    assert rel[FREE_STEPS:].max() <= 1e-9, rel[FREE_STEPS:].max()  # the same state: the forward is bit-exact
    gpu.destroy()
    for v in views:
        v.image.destroy()


def test_fused_backward_adam_gradients_match_oracle(device):
    """One training step with the gradients kept: the fused kernel's Gaussian and SH
    gradients against oracle.preprocess_backward from the same splat gradients and
    the state before the step, per group (relative to the group's largest) and
    element by element (over gradients above 1e-3 of the group's largest)."""
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)
    sh = np.random.default_rng(8).normal(0, 0.1, 60 * 45).astype(np.float32)
    settings = replace(DEFAULT_SETTINGS, extent=3.85, shDegreeInterval=1)  # degree 1 from the first step
    t = Trainer(device, RawGaussians(params, sh), views, settings)
    t.setKeepGradients(True)
    for _ in range(3):  # degree 3 by the third step
        gaussians = t.renderer.gaussianBuffer.read(np.float32).copy()
        coefficients = t.renderer.shBuffer.read(np.float32).copy()
        view = views[t.nextView()]
        t.optimize()
        t.maintain()
        grads = t.renderer.gradients
        gg, sg = grads["gaussians"].read(np.float32), grads["sh"].read(np.float32)
        splats = t.renderer.splatBuffer.read(np.float32)
        splat_grads = grads["splats"].read(np.float32)
        want_g, want_s = oracle.preprocess_backward(cam_array(view.camera), gaussians, coefficients, t.shDegree,
                                                    splats, splat_grads)
        mask = np.ones(16, bool)
        mask[[7, 15]] = False
        gg, want_g = gg.reshape(-1, 16), want_g.reshape(-1, 16)
        for name, off, size in GROUPS:
            g, w = gg[:, off:off + size], want_g[:, off:off + size]
            assert np.abs(g - w).max() <= 1e-4 * np.abs(w).max(), (name, t.shDegree)
            worst, median = elementwise_errors(g, w, 1e-3)
            assert worst <= 1e-3 and median <= 1e-5, (name, worst, median)
        assert np.abs(sg - want_s).max() <= 1e-4 * np.abs(want_s).max()
        worst, median = elementwise_errors(sg, want_s, 1e-3)
        assert worst <= 1e-3 and median <= 1e-5, ("sh", worst, median)
    assert t.shDegree == 3
    t.destroy()
    for v in views:
        v.image.destroy()

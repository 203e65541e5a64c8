"""Training on the GPU: Adam, statistics, densification and opacity reset against
the oracle and the reference's rules (src/checks/densify.ts), the end-to-end
training check (src/checks/training.ts), captured-graph steps against direct
launches, and the GPU evaluation metrics against the CPU's."""

from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from diorama_gb300 import (DEFAULT_SETTINGS, CameraData, Gaussian, GaussianRenderer, RawGaussians, Trainer,
                           TrainingView, activate, packGaussians)
from diorama_gb300.mat4 import IDENTITY, lookAt, perspective
from diorama_gb300.random import mulberry32
from dataclasses import replace

pytestmark = pytest.mark.gpu

SH_C0 = 0.28209479177387814


def ring_views(device, truth, size=96, count=8, background=(0, 0, 0)):
    """src/checks/training.ts:228-248: a ring of cameras photographing `truth`."""
    cams = []
    for k in range(count):
        angle = k / count * 2 * math.pi
        eye = [3.5 * math.sin(angle), 1.2, 3.5 * math.cos(angle)]
        cams.append(CameraData(lookAt(eye, [0, 0, 0], [0, 1, 0]), perspective(math.pi / 3.5, 1, 0.1, 100), (size, size)))
    photographer = GaussianRenderer(device)
    photographer.setGaussians(packGaussians(truth))
    views = []
    for k, cam in enumerate(cams):
        tex = device.createTexture(size, size)
        photographer.encode(None, tex, cam, background)
        views.append(TrainingView(f"view {k}", cam, tex))
    device.synchronize()
    photographer.destroy()
    return views


def truth_scene():
    random = mulberry32(17)
    between = lambda lo, hi: lo + (hi - lo) * random()  # noqa: E731
    return [Gaussian((between(-1, 1), between(-1, 1), between(-1, 1)),
                     (between(0.08, 0.3), between(0.08, 0.3), between(0.08, 0.3)),
                     (between(-1, 1), between(-1, 1), between(-1, 1), between(-1, 1)),
                     (random(), random(), random()), between(0.6, 0.95)) for _ in range(60)], random


def test_adam_step_matches_oracle(device):
    truth, random = truth_scene()
    views = ring_views(device, truth)
    rng = np.random.default_rng(1)
    n = 60
    params = np.zeros(n * 16, np.float32)
    for i, g in enumerate(truth):
        at = i * 16
        params[at:at + 3] = np.array(g.position) + rng.uniform(-0.1, 0.1, 3)
        params[at + 3] = 0.3
        params[at + 4:at + 7] = np.log(g.scale)
        params[at + 8:at + 12] = g.rotation
        params[at + 12:at + 15] = rng.uniform(-1, 1, 3)
    sh = rng.normal(0, 0.1, n * 45).astype(np.float32)
    settings = replace(DEFAULT_SETTINGS, extent=3.85, shDegreeInterval=1)  # degree 1 from the first step
    t = Trainer(device, RawGaussians(params, sh), views, settings)
    moments = rng.uniform(-1, 1, n * 61 * 2).astype(np.float32)
    moments[1::2] = np.abs(moments[1::2])
    t.writeMoments(moments)
    t.setKeepGradients(True)
    t.optimize()
    grads = t.renderer.gradients
    gg, sg = grads["gaussians"].read(np.float32), grads["sh"].read(np.float32)
    p = 1 / 30000
    lr = math.exp(math.log(0.00016) * (1 - p) + math.log(0.0000016) * p) * 3.85
    ap = np.array([1 - 0.9, 1 - 0.999, lr, 0.025, 0.005, 0.001, 0.0025, 0.0025 / 20, 96, 96], np.float32)
    want_p, want_sh, want_m = params.copy(), sh.copy(), moments.copy()
    want_g = np.zeros(n * 16, np.float32)
    oracle.adam_step(ap, want_p, want_sh, want_m, gg, sg, want_g)
    got_p = t.buffers["params"].read(np.float32)
    mask = np.ones(16, bool)
    mask[[7, 15]] = False
    assert np.allclose(got_p.reshape(-1, 16)[:, mask], want_p.reshape(-1, 16)[:, mask], rtol=1e-6, atol=1e-7)
    assert np.allclose(t.renderer.shBuffer.read(np.float32), want_sh, rtol=1e-6, atol=1e-7)
    got_m = t.readMoments()
    assert np.allclose(got_m, want_m, rtol=1e-5, atol=1e-9)
    slots = got_m.reshape(n, 61, 2)
    assert np.array_equal(slots[:, [7, 15]], moments.reshape(n, 61, 2)[:, [7, 15]])  # padding slots untouched
    act = t.renderer.gaussianBuffer.read(np.float32).reshape(-1, 16)
    assert np.allclose(act[:, mask], want_g.reshape(-1, 16)[:, mask], rtol=1e-6, atol=1e-7)
    # The densification statistics of this step.
    stats = t.buffers["stats"].read(np.float32)
    splats = t.renderer.splatBuffer.read(np.float32)
    want_stats = np.zeros(n * 4, np.float32)
    oracle.accumulate_stats(splats, grads["splats"].read(np.float32), (96, 96), want_stats)
    assert np.allclose(stats, want_stats, rtol=1e-6, atol=1e-12)
    t.destroy()
    for v in views:
        v.image.destroy()


@pytest.mark.parametrize("prune_large", [False, True])
def test_densify_and_reset(device, prune_large):
    """src/checks/densify.ts:28-185 against the oracle's restatement of densify.wgsl."""
    n = 2000
    random = mulberry32(41 if prune_large else 43)
    between = lambda lo, hi: lo + (hi - lo) * random()  # noqa: E731
    params = np.zeros(n * 16, np.float32)
    sh = np.array([between(-1, 1) for _ in range(n * 45)], np.float32)
    moments = np.array([between(-1, 1) for _ in range(n * 61 * 2)], np.float32)
    stats = np.zeros(n * 4, np.float32)
    ranges = [(0.002, 0.009), (0.012, 0.08), (0.11, 0.15), (0.17, 0.3)]
    for i in range(n):
        at = i * 16
        lo, hi = ranges[math.floor(random() * 4)]
        size = between(lo, hi)
        largest = math.floor(random() * 3)
        for k in range(3):
            params[at + k] = between(-1, 1)
            params[at + 4 + k] = math.log(size if k == largest else size * between(0.2, 0.9))
            params[at + 12 + k] = between(-1, 1)
        o = between(0.001, 0.004) if random() < 0.15 else between(0.006, 0.99)
        params[at + 3] = math.log(o / (1 - o))
        for k in range(8, 12):
            params[at + k] = between(-1, 1)
        if random() >= 0.1:
            seen = 1 + math.floor(random() * 10)
            average = between(0.00005, 0.00019) if random() < 0.5 else between(0.00021, 0.001)
            stats[i * 4:i * 4 + 4] = [average * seen, seen, between(1, 30), 0]
    image = device.createTexture(16, 16)
    cam = CameraData(IDENTITY, IDENTITY, (16, 16))
    t = Trainer(device, RawGaussians(params.copy(), sh), [TrainingView("unused", cam, image)],
                replace(DEFAULT_SETTINGS, extent=1.0))
    t.writeMoments(moments)
    t.buffers["stats"].write(stats)
    t.iteration = 700
    t.densify(prune_large)
    dp = [0.0002, 0.01, 0.005, 0.1 if prune_large else 0.0]
    want_p, want_sh, want_m, tally = oracle.densify(params, stats, sh, moments, dp, 700)
    assert t.count == want_p.size // 16
    record = t.densifications[0]
    assert (record.removed, record.kept, record.cloned, record.split) == tuple(int(x) for x in tally)
    assert (record.step, record.before, record.after) == (700, n, t.count)
    got_p = t.buffers["params"].read(np.float32)
    assert np.allclose(got_p, want_p, rtol=1e-5, atol=1e-6)
    assert np.array_equal(t.renderer.shBuffer.read(np.float32), want_sh)
    got_m = t.readMoments()
    assert np.array_equal(got_m, want_m)
    assert not t.buffers["stats"].read(np.float32).any()
    act = t.renderer.gaussianBuffer.read(np.float32).reshape(-1, 16)
    want_act = activate(got_p).reshape(-1, 16)
    mask = np.ones(16, bool)
    mask[[7, 15]] = False
    assert np.allclose(act[:, mask], want_act[:, mask], rtol=1e-5, atol=1e-6)
    # Split children's offsets, in the parent's axes and units of its scale, are N(0, 1).
    children = np.flatnonzero(got_p.reshape(-1, 16)[:, 7] == 2)
    assert children.size > 100

    # Opacity reset: every opacity capped at 0.01, and only its Adam slot cleared.
    t.resetOpacity()
    p2 = t.buffers["params"].read(np.float32).reshape(-1, 16)
    m2 = t.readMoments().reshape(-1, 122)
    capped = np.float32(-4.59511985013459)
    assert np.array_equal(p2[:, 3], np.minimum(got_p.reshape(-1, 16)[:, 3], capped))
    assert not m2[:, 6:8].any()
    keep = np.ones(122, bool)
    keep[6:8] = False
    assert np.array_equal(m2[:, keep], got_m.reshape(-1, 122)[:, keep])
    g2 = t.renderer.gaussianBuffer.read(np.float32).reshape(-1, 16)
    assert np.allclose(g2[:, 3], 1 / (1 + np.exp(-p2[:, 3].astype(np.float64))), atol=1e-6)
    t.destroy()
    image.destroy()


def scrambled_start(truth, random):
    between = lambda lo, hi: lo + (hi - lo) * random()  # noqa: E731
    params = np.zeros(len(truth) * 16, np.float32)
    for i, g in enumerate(truth):
        at = i * 16
        for k in range(3):
            params[at + k] = g.position[k] + between(-0.15, 0.15)
            params[at + 4 + k] = math.log(g.scale[k] * between(0.6, 1.6))
            params[at + 12 + k] = (random() - 0.5) / SH_C0
        params[at + 3] = 0
        params[at + 8:at + 12] = [1, 0, 0, 0]
    return params


def test_training_end_to_end(device):
    """src/checks/training.ts:217-302: 400 steps on 8 views at 96x96."""
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)

    def train(p, **overrides):
        count = p.size // 16
        t = Trainer(device, RawGaussians(p, np.zeros(count * 45, np.float32)), views,
                    replace(DEFAULT_SETTINGS, extent=3.85, **overrides))
        before = t.evaluate(views, False)["psnr"]
        for _ in range(400):
            t.step()
        after = t.evaluate(views, False)["psnr"]
        result = dict(before=before, after=after, loss=t.lastLoss(), count=t.count)
        t.destroy()
        return result

    fit = train(params)
    assert fit["after"] - fit["before"] >= 6, fit

    sparse = np.zeros(12 * 16, np.float32)
    for i in range(12):
        at = i * 16
        for k in range(3):
            sparse[at + k] = -0.8 + 1.6 * random()
            sparse[at + 4 + k] = math.log(0.25)
        sparse[at + 3] = math.log(0.1 / 0.9)
        sparse[at + 8:at + 12] = [1, 0, 0, 0]
    plain = train(sparse.copy(), densifyUntil=0)
    densified = train(sparse.copy(), densifyFrom=100, densifyInterval=50, densifyUntil=351)
    assert densified["count"] > 12
    assert densified["after"] > plain["after"] + 1, (plain, densified)
    for v in views:
        v.image.destroy()


def test_graph_steps_match_direct_steps(device):
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)

    def run(graph, steps, **overrides):
        t = Trainer(device, RawGaussians(params.copy(), np.zeros(60 * 45, np.float32)), views,
                    replace(DEFAULT_SETTINGS, extent=3.85, **overrides))
        t.setGraph(graph)
        for _ in range(steps):
            t.step()
        out = (t.exportRaw(), t.count, t.lastLoss(), [(d.cloned, d.split) for d in t.densifications])
        t.destroy()
        return out

    # A few steps: the same kernels with the same uniforms. The backward's atomics
    # add in a run-dependent order, so states agree to rounding.
    (a, _, la, _), (b, _, lb, _) = run(False, 3), run(True, 3)
    assert np.allclose(a.params, b.params, rtol=1e-5, atol=1e-6)
    assert abs(la - lb) < 1e-5
    # With densification: the same decisions; the rounding differences of many
    # steps stay small for almost every value.
    dense = dict(densifyFrom=20, densifyInterval=25, densifyUntil=80)
    (a, ca, la, da), (b, cb, lb, db) = run(False, 120, **dense), run(True, 120, **dense)
    assert ca == cb and da == db
    rel = np.abs(a.params - b.params) / (np.abs(b.params) + 1e-3)
    assert np.median(rel) < 1e-5 and np.mean(rel < 1e-3) > 0.99, (np.median(rel), np.mean(rel < 1e-3))
    assert abs(la - lb) < 1e-3
    for v in views:
        v.image.destroy()


def test_evaluate_matches_cpu_metrics(device):
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)
    t = Trainer(device, RawGaussians(params, np.zeros(60 * 45, np.float32)), views, replace(DEFAULT_SETTINGS, extent=3.85))
    for _ in range(30):
        t.step()
    got = t.evaluate(views[:3], True)
    psnr, ssim = [], []
    r = t.renderer
    for v in views[:3]:
        r.encode(None, None, v.camera, (0, 0, 0))
        rendered = r.pixelBuffer.read(np.float32)[: 96 * 96 * 4].astype(np.float64)
        q = (np.round(np.clip(rendered, 0, 1) * 255) / 255).astype(np.float32)
        photo = (v.image.read().reshape(-1).astype(np.float64) / 255).astype(np.float32)
        psnr.append(oracle.psnr(q, photo))
        ssim.append(oracle.ssim(q, photo, 96, 96))
    assert abs(got["psnr"] - np.mean(psnr)) < 1e-6
    assert abs(got["ssim"] - np.mean(ssim)) < 1e-5
    t.destroy()
    for v in views:
        v.image.destroy()


def test_requested_losses_arrive_in_order(device):
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)
    t = Trainer(device, RawGaussians(params, np.zeros(60 * 45, np.float32)), views,
                replace(DEFAULT_SETTINGS, extent=3.85))
    from diorama_gb300 import DioramaError
    with pytest.raises(DioramaError, match="no loss value requested"):
        t.takeLoss()
    want = []
    for _ in range(5):
        t.step()
        want.append(t.lossValue())
        t.requestLoss()
    got = [t.takeLoss() for _ in range(5)]
    assert got == want  # the same sum in the same order
    for _ in range(16):
        t.requestLoss()
    with pytest.raises(DioramaError, match="too many loss values"):
        t.requestLoss()
    taken = [t.takeLoss() for _ in range(16)]
    assert all(v == want[-1] for v in taken)  # no step in between: the same loss
    t.destroy()
    for v in views:
        v.image.destroy()


def test_host_photos_match_device_images(device):
    # Photos read from pinned host memory by the trainer itself give the same
    # losses as the views' device images (the first steps' bit for bit).
    from diorama_gb300.gpu import PinnedArray
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)
    settings = replace(DEFAULT_SETTINGS, extent=3.85)
    a = Trainer(device, RawGaussians(params.copy(), np.zeros(60 * 45, np.float32)), views, settings)
    b = Trainer(device, RawGaussians(params.copy(), np.zeros(60 * 45, np.float32)), views, settings)
    pinned = []
    for v in views:
        p = PinnedArray((96 * 96 * 4,), np.uint8)
        p.array[:] = v.image.read().reshape(-1)
        pinned.append(p)
    b.setHostPhotos(pinned)
    la, lb = [], []
    for _ in range(12):
        assert a.nextView() == b.nextView()
        a.step()
        b.step()
        la.append(a.lossValue())
        lb.append(b.lossValue())
    assert la[0] == lb[0]
    assert np.allclose(la, lb, rtol=1e-4)
    b.setHostPhotos(None)
    b.step()
    a.step()
    assert abs(a.lossValue() - b.lossValue()) < 1e-3
    a.destroy()
    b.destroy()
    for p in pinned:
        p.free()
    for v in views:
        v.image.destroy()


def test_pair_buffers_grow_while_training_runs_ahead(device):
    """A training loop that never waits for the GPU still grows the pair buffers
    once a frame needs more pairs than they hold (the reference's afterSubmit
    resolves for every frame, src/tileRasterizer.ts:229-244): every step queues its
    pair-count readback, and later steps consume the ones that have arrived.
    100 large Gaussians at 512x512 need ~10^5 pairs against the initial 2^16."""
    rng = np.random.default_rng(3)
    n = 100
    params = np.zeros((n, 16), np.float32)
    params[:, 0:3] = rng.uniform(-0.6, 0.6, (n, 3))
    params[:, 3] = 1.0
    params[:, 4:7] = np.log(0.6)
    params[:, 8] = 1.0
    params[:, 12:15] = rng.uniform(-1, 1, (n, 3))
    cams = [CameraData(lookAt([3 * math.sin(a), 0.5, 3 * math.cos(a)], [0, 0, 0], [0, 1, 0]),
                       perspective(math.pi / 3, 1, 0.1, 100), (512, 512)) for a in (0.0, 2.0)]
    photos = [device.createTexture(512, 512) for _ in cams]
    views = [TrainingView(f"view {k}", c, p) for k, (c, p) in enumerate(zip(cams, photos))]
    t = Trainer(device, RawGaussians(params.reshape(-1), np.zeros(n * 45, np.float32)), views,
                replace(DEFAULT_SETTINGS, extent=3.0, densifyUntil=0))
    t.setGraph(True)
    for _ in range(12):
        t.step()
    tiles = t.renderer.tiles
    grown = tiles.pairCapacity  # before any wait: grown by the loop itself
    t.renderer.afterSubmit()
    assert tiles.lastPairCount > 1 << 16, tiles.lastPairCount
    assert grown >= tiles.lastPairCount, (grown, tiles.lastPairCount)
    t.destroy()
    for p in photos:
        p.destroy()

"""The oracle (a float32 C restatement of the reference's path) against the
reference's own golden vectors: the fixtures its PyTorch float64 oracles write
(reference/backward_reference.py, reference/loss_reference.py) and the 16,384-Gaussian
random scene's vectors of tests/golden/make_golden.py. CPU only."""

from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from diorama_gb300 import scenes
from diorama_gb300.mat4 import IDENTITY, perspective
from diorama_gb300.random import mulberry32
from helpers import GOLDEN, backward_fixture, cam_array, group_errors, loss_fixture, sort_keys, stable_sort_reference


def test_fixtures_were_checked_by_finite_differences():
    # The reference checked its autograd against central differences in float64 (step 1e-6).
    assert max(backward_fixture()["fd_error"].values()) < 1e-7
    assert loss_fixture()["fd_error"] < 1e-6


def test_backward_fixture_forward_and_gradients():
    f = backward_fixture()
    cam = cam_array(f["camera"])
    frame = oracle.render(cam, f["background"], f["gaussians"], f["sh"], f["degree"])
    image = frame["pixel_color"].reshape(-1, 4)[:, :3]
    assert np.abs(image - f["image"]).max() <= 1e-6  # the reference's own bar is 1e-4
    sg = oracle.rasterize_backward(cam, f["background"], frame["splats"], frame, f["pixel_grads"])
    gg, shg = oracle.preprocess_backward(cam, f["gaussians"], f["sh"], f["degree"], frame["splats"], sg)
    errors = group_errors(gg, shg, f["grads"])
    assert max(errors.values()) <= 1e-5, errors  # the reference's own bar is 2e-3


def test_loss_fixture():
    f = loss_fixture()
    value, grads, per_pixel = oracle.loss(f["render"], f["target"], f["width"], f["height"])
    assert abs(value - f["loss"]) <= 1e-7
    g = grads.reshape(-1, 4)[:, :3]
    assert np.abs(g - f["gradient"]).max() / np.abs(f["gradient"]).max() <= 1e-5


def test_cpu_ssim_rebuilds_the_loss():
    # src/checks/loss.ts:472-481: the loss from the CPU SSIM agrees with PyTorch to 1e-6.
    f = loss_fixture()
    y = np.zeros_like(f["render"])
    y[:, :3] = f["target"][:, :3] / 255
    l1 = np.abs(f["render"][:, :3].astype(np.float64) - y[:, :3]).sum()
    cpu = 0.8 * l1 / (3 * f["width"] * f["height"]) + 0.2 * (1 - oracle.ssim(f["render"], y, f["width"], f["height"]))
    assert abs(cpu - f["loss"]) <= 1e-6


def test_random_16k_against_reference_golden():
    g = np.load(GOLDEN / "random_16k.npz")
    raw, sh, camera = scenes.random_scene_16k(0)
    act = scenes.activate64(raw).astype(np.float32)
    cam = cam_array(camera)
    W, H = camera.viewport
    frame = oracle.render(cam, np.zeros(3, np.float32), act, sh, 3)
    image = frame["pixel_color"].reshape(-1, 4)[:, :3]
    assert np.abs(image - g["image"]).max() <= 1e-5
    value, pg, _ = oracle.loss(frame["pixel_color"], g["target_rgba8"].reshape(-1), W, H)
    assert abs(value - float(g["loss"])) <= 1e-6
    sg = oracle.rasterize_backward(cam, np.zeros(3, np.float32), frame["splats"], frame, pg)
    gg, shg = oracle.preprocess_backward(cam, act, sh, 3, frame["splats"], sg)
    expected = {k: g["grad_" + k] for k in ("position", "scale", "rotation", "opacity", "color", "sh")}
    errors = group_errors(gg, shg, expected)
    assert max(errors.values()) <= 1e-4, errors


def test_scan_and_sort_primitives():
    # src/checks/depthSort.ts:46-104 on the oracle itself.
    random = mulberry32(3)
    data = np.array([math.floor(random() * 10) for _ in range(300_000)], np.uint32)
    scanned = data.copy()
    total = oracle.lib().or_exclusive_scan(scanned, data.size)
    assert total == data.sum()
    assert np.array_equal(scanned, np.concatenate([[0], np.cumsum(data)[:-1]]).astype(np.uint32))
    for size in (1, 1000, 1024, 10_003):
        keys = sort_keys(size).astype(np.uint64)
        values = np.arange(size, dtype=np.uint32)
        k, v = keys.copy(), values.copy()
        oracle.lib().or_radix_sort(k, v, size, 0)
        order = stable_sort_reference(keys)
        assert np.array_equal(v, order) and np.array_equal(k, keys[order])


def test_blend_exponential_accuracy():
    xs = np.linspace(-87, 0, 200_001, dtype=np.float32)
    got = np.array([oracle.exp_ref(float(x)) for x in xs[::97]], np.float64)
    want = np.exp(xs[::97].astype(np.float64))
    assert np.max(np.abs(got - want) / want) < 2.5e-7  # about two float32 ulps


def test_projection_hand_values():
    # src/checks/gaussians3d.ts:50-110: a 90-degree camera in a 64-pixel viewport (focal 32 px).
    from diorama_gb300 import Gaussian, packGaussians

    cam = oracle.camera_array(IDENTITY, perspective(math.pi / 2, 1, 0.1, 100), (64, 64))
    turn = (math.cos(math.pi / 8), 0, 0, math.sin(math.pi / 8))
    cases = [
        Gaussian((0, 0, -4), (0.5, 0.5, 0.5), (1, 0, 0, 0), (1, 1, 1), 0.9),
        Gaussian((0, 0, -4), (1, 0.25, 0.25), turn, (1, 1, 1), 0.9),
        Gaussian((0, 0, 2), (0.5, 0.5, 0.5), (1, 0, 0, 0), (1, 1, 1), 0.9),
        Gaussian((40, 0, -4), (0.2, 0.2, 0.2), (1, 0, 0, 0), (1, 1, 1), 0.9),
    ]
    s = oracle.preprocess(cam, packGaussians(cases), None, 0).reshape(-1, 12)
    assert np.allclose(s[0, :4], [32, 32, 4, 13], rtol=1e-4)
    assert np.allclose(s[0, 4:7], [1 / 16.3, 0, 1 / 16.3], rtol=1e-4, atol=1e-7)
    assert np.allclose(s[1, :4], [32, 32, 4, 25], rtol=1e-4)
    assert np.allclose(s[1, 4:7], [34.3 / 276.49, 30 / 276.49, 34.3 / 276.49], rtol=1e-4)
    assert s[2, 3] == 0 and s[3, 3] == 0  # behind the camera; far outside the view


@pytest.mark.parametrize("seed", [41, 43])
def test_densify_rules(seed):
    """The oracle's densification against the reference's CPU rules (src/checks/densify.ts:84-110)."""
    n = 2000
    random = mulberry32(seed)
    between = lambda lo, hi: lo + (hi - lo) * random()  # noqa: E731
    params = np.zeros(n * 16, np.float32)
    stats = np.zeros(n * 4, np.float32)
    sh = np.array([between(-1, 1) for _ in range(n * 45)], np.float32)
    moments = np.array([between(-1, 1) for _ in range(n * 61 * 2)], np.float32)
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
            stats[i * 4: i * 4 + 4] = [average * seen, seen, between(1, 30), 0]
    prune_large = seed == 41
    dp = [0.0002, 0.01, 0.005, 0.1 if prune_large else 0.0]
    new_params, new_sh, new_moments, tally = oracle.densify(params, stats, sh, moments, dp, 700)
    sig = lambda x: 1 / (1 + math.exp(-x))  # noqa: E731
    expected = []
    t = {"kept": 0, "cloned": 0, "split": 0, "removed": 0}
    for i in range(n):
        at = i * 16
        grad = stats[i * 4] / stats[i * 4 + 1] if stats[i * 4 + 1] > 0 else 0
        size = math.exp(max(params[at + 4], params[at + 5], params[at + 6]))
        clone = grad >= 0.0002 and size <= 0.01
        split = grad >= 0.0002 and not clone
        s = size / 1.6 if split else size
        if sig(params[at + 3]) < 0.005 or (prune_large and s > 0.1):
            t["removed"] += 1
        elif split:
            t["split"] += 1
            expected += [(i, "child"), (i, "child")]
        else:
            expected.append((i, "kept"))
            if clone:
                t["cloned"] += 1
                expected.append((i, "clone"))
            else:
                t["kept"] += 1
    assert list(tally) == [t["removed"], t["kept"], t["cloned"], t["split"]]
    assert new_params.size // 16 == len(expected)
    for o, (src, kind) in enumerate(expected):
        got = new_params[o * 16: o * 16 + 16]
        want = params[src * 16: src * 16 + 16].copy()
        if kind == "child":
            want[4:7] -= math.log(1.6)
        if kind != "kept":
            want[7] = 1 if kind == "clone" else 2
            want[15] = 700
        mask = np.ones(16, bool)
        if kind == "child":
            mask[:3] = False
        assert np.allclose(got[mask], want[mask], atol=1e-5)
        assert np.array_equal(new_sh[o * 45:(o + 1) * 45], sh[src * 45:(src + 1) * 45])
        m = new_moments[o * 122:(o + 1) * 122]
        assert np.array_equal(m, moments[src * 122:(src + 1) * 122] if kind == "kept" else np.zeros(122, np.float32))

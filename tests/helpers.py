"""Scenes and comparisons shared by the tests, following the reference's checks
(src/checks/helpers.ts, src/checks/tiles.ts, src/checks/depthSort.ts)."""

from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

import oracle
from diorama_gb300 import CameraData, Gaussian, packGaussians
from diorama_gb300.mat4 import IDENTITY, perspective
from diorama_gb300.random import mulberry32
from diorama_gb300.scenes import clustered_cloud  # noqa: F401

GOLDEN = Path(__file__).resolve().parent / "golden"


def cam_array(camera: CameraData) -> np.ndarray:
    return oracle.camera_array(camera.view, camera.proj, camera.viewport)


def assert_splats_match(gpu, cpu) -> None:
    """The renderer's splat records against the oracle's preprocess: bit for bit,
    but for slot 7. The reference leaves that padding unwritten; the renderer's
    preprocess stores each visible splat's blend cutoff there,
    log(1 / (255 opacity)) - 1e-3 (0 when culled), computed with the GPU's logf,
    so it is checked against the float64 value to 1e-6."""
    g = np.asarray(gpu, np.float32).reshape(-1, 12)
    c = np.asarray(cpu, np.float32).reshape(-1, 12)
    mask = np.ones(12, bool)
    mask[7] = False
    assert np.array_equal(g[:, mask].view(np.uint32), c[:, mask].view(np.uint32))
    visible = g[:, 3] != 0.0
    with np.errstate(divide="ignore"):
        want = np.log(1.0 / (255.0 * g[visible, 11].astype(np.float64))) - 1e-3
    got = g[visible, 7].astype(np.float64)
    same_inf = np.isinf(want) & (got == want)  # opacity 0: no pixel blends it
    assert np.all(same_inf | (np.abs(got - want) <= 1e-6 * np.maximum(1.0, np.abs(want))))
    assert np.all(g[~visible, 7] == 0.0)


def random_scene(count: int, scale=(0.02, 0.4), opacity=(0.2, 0.95)) -> list[Gaussian]:
    """src/checks/tiles.ts:169-186: Gaussians scattered through the view."""
    random = mulberry32(11)
    between = lambda lo, hi: lo + (hi - lo) * random()  # noqa: E731
    out = []
    for _ in range(count):
        depth = between(2, 8)
        position = (between(-1.2, 1.2) * depth, between(-0.9, 0.9) * depth, -depth)
        sc = (between(*scale), between(*scale), between(*scale))
        rotation = (between(-1, 1), between(-1, 1), between(-1, 1), between(-1, 1))
        color = (random(), random(), random())
        out.append(Gaussian(position=position, scale=sc, rotation=rotation, color=color, opacity=between(*opacity)))
    return out


TILES_VIEWPORT = (120, 90)
TILES_CAMERA = CameraData(view=IDENTITY, proj=perspective(math.pi / 2, 120 / 90, 0.1, 100), viewport=TILES_VIEWPORT)


def backward_fixture():
    """The reference's backward fixture as arrays: activated Gaussians (16 floats
    each), SH rest, camera, background, pixel gradients (vec4), image, gradients."""
    d = json.loads((GOLDEN / "backward.json").read_text())
    g = np.zeros((len(d["gaussians"]), 16), np.float32)
    for i, x in enumerate(d["gaussians"]):
        g[i, 0:3] = x["position"]
        g[i, 3] = x["opacity"]
        g[i, 4:7] = x["scale"]
        g[i, 8:12] = x["rotation"]
        g[i, 12:15] = x["color"]
    W, H = d["viewport"]
    pg = np.zeros((W * H, 4), np.float32)
    pg[:, :3] = np.array(d["pixelGrads"]).reshape(-1, 3)
    grads = {
        "position": np.array([x["position"] for x in d["gradients"]]),
        "scale": np.array([x["scale"] for x in d["gradients"]]),
        "rotation": np.array([x["rotation"] for x in d["gradients"]]),
        "opacity": np.array([[x["opacity"]] for x in d["gradients"]]),
        "color": np.array([x["color"] for x in d["gradients"]]),
        "sh": np.array([x["sh"] for x in d["gradients"]]),
    }
    return dict(
        gaussians=g,
        sh=np.array(d["shRest"], np.float32).reshape(-1),
        camera=CameraData(view=d["view"], proj=d["proj"], viewport=(W, H)),
        background=np.array(d["background"], np.float32),
        degree=d["shDegree"],
        pixel_grads=pg,
        image=np.array(d["image"]).reshape(-1, 3),
        grads=grads,
        fd_error=d["finiteDifferenceError"],
    )


# Where each group sits in the 16-float gradient layout (src/checks/backward.ts:41-47).
GROUPS = [("position", 0, 3), ("scale", 4, 3), ("rotation", 8, 4), ("opacity", 3, 1), ("color", 12, 3)]


def group_errors(gaussian_grads: np.ndarray, sh_grads: np.ndarray, expected: dict) -> dict:
    """Largest disagreement per group relative to the group's largest reference gradient."""
    gg = np.asarray(gaussian_grads, np.float64).reshape(-1, 16)
    out = {}
    for name, off, size in GROUPS:
        ref = np.asarray(expected[name], np.float64).reshape(len(gg), -1)
        out[name] = float(np.abs(gg[:, off:off + size] - ref).max() / max(np.abs(ref).max(), 1e-30))
    ref = np.asarray(expected["sh"], np.float64).reshape(len(gg), -1)
    sg = np.asarray(sh_grads, np.float64).reshape(len(gg), -1)
    out["sh"] = float(np.abs(sg - ref).max() / max(np.abs(ref).max(), 1e-30))
    return out


def elementwise_errors(got, want, floor: float) -> tuple[float, float]:
    """Element-wise relative errors |got - want| / |want| over the values whose
    magnitude is above `floor` times the largest: (largest, median). This is the
    plain "relative" form, reported beside the group-max form above, which leaves
    the small gradients of a group unconstrained."""
    g = np.asarray(got, np.float64).reshape(-1)
    w = np.asarray(want, np.float64).reshape(-1)
    big = np.abs(w) > floor * np.abs(w).max()
    if not big.any():
        return 0.0, 0.0
    rel = np.abs(g[big] - w[big]) / np.abs(w[big])
    return float(rel.max()), float(np.median(rel))


def loss_fixture():
    d = json.loads((GOLDEN / "loss.json").read_text())
    w, h = d["size"]
    render = np.zeros((w * h, 4), np.float32)
    render[:, :3] = np.array(d["render"]).reshape(-1, 3)
    target = np.full((w * h, 4), 255, np.uint8)
    target[:, :3] = np.array(d["target"]).reshape(-1, 3)
    return dict(width=w, height=h, render=render, target=target, loss=d["loss"],
                gradient=np.array(d["gradient"]).reshape(-1, 3), fd_error=d["finiteDifferenceError"])


def stable_sort_reference(keys: np.ndarray) -> np.ndarray:
    """The permutation of a stable sort by key (src/checks/depthSort.ts:94)."""
    return np.argsort(keys, kind="stable").astype(np.uint32)


def sort_keys(size: int) -> np.ndarray:
    """src/checks/depthSort.ts:84-89: half full-range keys, half in 0..15."""
    random = mulberry32(size)
    out = np.zeros(size, np.uint32)
    for i in range(size):
        out[i] = math.floor(random() * 2**32) if i % 2 == 0 else math.floor(random() * 16)
    return out


def pack(gaussians) -> np.ndarray:
    return packGaussians(gaussians)


def neighbor_check_points():
    """src/checks/dataset.ts:28-41: 3,001 points in [-2, 2)³ from mulberry32(31),
    point 1000 an exact copy of point 7, then one colour per point from the same
    generator."""
    random = mulberry32(31)
    count = 3001
    positions = np.array([random() * 4 - 2 for _ in range(count * 3)], np.float64).astype(np.float32)
    positions[3 * 1000:3 * 1001] = positions[3 * 7:3 * 8]
    colors = np.array([math.floor(random() * 256) for _ in range(count * 3)], np.uint8)
    return positions, colors


def neighbor_distance2_f64(positions: np.ndarray) -> np.ndarray:
    """src/checks/dataset.ts:60-80: the CPU brute force in float64."""
    p = positions.reshape(-1, 3).astype(np.float64)
    out = np.zeros(p.shape[0])
    for start in range(0, p.shape[0], 512):
        d = p[start:start + 512, None, :] - p[None, :, :]
        d2 = (d * d).sum(-1)
        rows = np.arange(d2.shape[0])
        d2[rows, start + rows] = np.inf
        out[start:start + 512] = np.sort(np.partition(d2, 2, axis=1)[:, :3], axis=1).sum(1) / 3
    return out


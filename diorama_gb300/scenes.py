"""Seeded synthetic scenes of the benchmark workloads.

The reference trains on the Tanks and Temples "train" photos, which are not
available here; these seeded scenes stand in for them with the shapes, sizes and
value distributions of the workloads. Everything is drawn with
numpy.random.default_rng(seed) in float64 and cast to float32, so every machine
gets the same bits.

- random_gaussians: N Gaussians with means U[-r, r]^3, log-scales N(-3.5, 0.5),
  quaternions N(0, I4) normalized, opacity logits N(0, 1), SH DC N(0, 0.5) and
  the 15 higher coefficients N(0, 0.05) (raw training parameters).
- sphere_camera: a pinhole camera on a radius-4 sphere looking at the origin.
- surface_scene: Gaussians clustered on random planes and boxes, with a ring of
  cameras at radius 3-5 around them, for the full training workload.
"""

from __future__ import annotations

import math

import numpy as np

from .gaussians import FLOATS_PER_GAUSSIAN, SH_REST_FLOATS
from .mat4 import lookAt, perspective
from .renderer import CameraData

SH_C0 = 0.28209479177387814


def random_gaussians(count: int, seed: int, half_extent: float = 1.0):
    """Raw parameters (16 floats each) and SH rest (45 each) of the random scenes' distribution."""
    rng = np.random.default_rng(seed)
    raw = np.zeros((count, FLOATS_PER_GAUSSIAN), np.float64)
    raw[:, 0:3] = rng.uniform(-half_extent, half_extent, (count, 3))
    raw[:, 4:7] = rng.normal(-3.5, 0.5, (count, 3))
    q = rng.normal(0.0, 1.0, (count, 4))
    raw[:, 8:12] = q / np.linalg.norm(q, axis=1, keepdims=True)
    raw[:, 3] = rng.normal(0.0, 1.0, count)
    raw[:, 12:15] = rng.normal(0.0, 0.5, (count, 3))
    sh = rng.normal(0.0, 0.05, (count, SH_REST_FLOATS))
    return raw.astype(np.float32), sh.astype(np.float32)


def activate64(raw: np.ndarray) -> np.ndarray:
    """Activated layout in float64 (position, sigmoid opacity, exp scale, quaternion, 0.5 + SH_C0 dc)."""
    p = np.asarray(raw, np.float64).reshape(-1, FLOATS_PER_GAUSSIAN)
    out = np.zeros_like(p)
    out[:, 0:3] = p[:, 0:3]
    out[:, 3] = 1 / (1 + np.exp(-p[:, 3]))
    out[:, 4:7] = np.exp(p[:, 4:7])
    out[:, 8:12] = p[:, 8:12]
    out[:, 12:15] = 0.5 + SH_C0 * p[:, 12:15]
    return out


def sphere_camera(seed: int, width: int = 256, height: int = 256, fov_deg: float = 60.0, radius: float = 4.0):
    """A seeded direction on a radius-4 sphere, looking at the origin."""
    rng = np.random.default_rng(seed + 1000)
    d = rng.normal(size=3)
    d = d / np.linalg.norm(d)
    eye = [float(v) for v in radius * d]
    up = [0.0, 1.0, 0.0] if abs(d[1]) < 0.95 else [0.0, 0.0, 1.0]
    view = lookAt(eye, [0.0, 0.0, 0.0], up)
    proj = perspective(math.radians(fov_deg), width / height, 0.01, 100.0)
    return CameraData(view=view, proj=proj, viewport=(width, height))


def random_scene_16k(seed: int = 0):
    """16,384 random Gaussians in [-1, 1]^3 seen at 256x256, fov 60 deg (black background, SH degree 3)."""
    raw, sh = random_gaussians(16384, seed)
    return raw, sh, sphere_camera(seed)


def random_scene_1m(seed: int = 0):
    """1.1M random Gaussians of the same distribution over [-3, 3]^3, seen at 1960x1090."""
    raw, sh = random_gaussians(1_100_000, seed, half_extent=3.0)
    return raw, sh, sphere_camera(seed, 1960, 1090)


def surface_scene(count: int, seed: int, noise: float = 0.0, shape_seed: int = 7):
    """Gaussians on 40 seeded planes and boxes (raw params, SH rest). The shapes
    come from shape_seed, so ground truth and initial points share surfaces."""
    shape_rng = np.random.default_rng(shape_seed)
    pts_rng = np.random.default_rng(seed)
    # Draw the shapes from their own stream, then the points from the scene's.
    pts, which = _surface_points_shared(shape_rng, pts_rng, count)
    pts = pts + pts_rng.normal(0.0, noise, pts.shape) if noise > 0 else pts
    raw = np.zeros((count, FLOATS_PER_GAUSSIAN), np.float64)
    raw[:, 0:3] = pts
    raw[:, 4:7] = pts_rng.normal(-4.2, 0.4, (count, 3))
    q = pts_rng.normal(size=(count, 4))
    raw[:, 8:12] = q / np.linalg.norm(q, axis=1, keepdims=True)
    raw[:, 3] = pts_rng.normal(1.0, 1.0, count)
    palette = np.random.default_rng(shape_seed + 1).normal(0.0, 0.8, (40, 3))
    raw[:, 12:15] = palette[which] + pts_rng.normal(0.0, 0.15, (count, 3))
    sh = pts_rng.normal(0.0, 0.05, (count, SH_REST_FLOATS))
    return raw.astype(np.float32), sh.astype(np.float32)


def _surface_points_shared(shape_rng, pts_rng, count: int, shapes: int = 40):
    kinds = shape_rng.integers(0, 2, shapes)
    centers = shape_rng.uniform(-1.2, 1.2, (shapes, 3))
    sizes = shape_rng.uniform(0.15, 0.6, (shapes, 3))
    q = shape_rng.normal(size=(shapes, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    rot = np.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
        2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y),
    ], axis=1).reshape(-1, 3, 3)
    which = pts_rng.integers(0, shapes, count)
    local = pts_rng.uniform(-1, 1, (count, 3)) * sizes[which]
    box = kinds[which] == 1
    face = pts_rng.integers(0, 3, count)
    sign = np.where(pts_rng.uniform(size=count) < 0.5, -1.0, 1.0)
    rows = np.arange(count)
    local[rows[box], face[box]] = sign[box] * sizes[which[box], face[box]]
    local[~box, 2] = 0.0
    return np.einsum("nij,nj->ni", rot[which], local) + centers[which], which


def ring_cameras(count: int = 300, seed: int = 3, width: int = 980, height: int = 545, fov_deg: float = 55.0):
    """The 300-photo scene's cameras: a jittered ellipse ring of radius 3-5 around the origin.
    Every 8th (i % 8 == 7) is held out: 263 training views and 37 held-out ones."""
    rng = np.random.default_rng(seed)
    cams = []
    for i in range(count):
        angle = 2 * math.pi * i / count + rng.normal(0, 0.01)
        a, b = 5.0, 3.0
        r = a * b / math.sqrt((b * math.cos(angle)) ** 2 + (a * math.sin(angle)) ** 2)
        r *= 1 + rng.normal(0, 0.03)
        eye = [r * math.cos(angle), rng.uniform(0.3, 1.5), r * math.sin(angle)]
        target = [float(v) for v in rng.normal(0, 0.1, 3)]
        view = lookAt(eye, target, [0.0, 1.0, 0.0])
        proj = perspective(math.radians(fov_deg), width / height, 0.01, 100.0)
        cams.append(CameraData(view=view, proj=proj, viewport=(width, height)))
    train = [c for i, c in enumerate(cams) if i % 8 != 7]
    held = [c for i, c in enumerate(cams) if i % 8 == 7]
    return train, held


def clustered_cloud(count: int, seed: int) -> np.ndarray:
    """A structure-from-motion-like point cloud (count × 3 floats, flat): dense
    clusters of varied size (80%), a thin plane (15%), far outliers (the rest)
    and some exact duplicates."""
    rng = np.random.default_rng(seed)
    parts = []
    clusters = max(1, count // 2000)
    centres = rng.uniform(-5, 5, (clusters, 3))
    sizes = rng.uniform(0.01, 0.5, clusters)
    n_cluster = int(count * 0.8)
    which = rng.integers(0, clusters, n_cluster)
    parts.append(centres[which] + rng.normal(0, 1, (n_cluster, 3)) * sizes[which, None])
    n_plane = int(count * 0.15)
    plane = rng.uniform(-4, 4, (n_plane, 3))
    plane[:, 1] = -1.5
    parts.append(plane)
    parts.append(rng.normal(0, 60, (count - n_cluster - n_plane, 3)))
    points = np.concatenate(parts).astype(np.float32)
    dup = rng.integers(0, count, count // 200)
    points[rng.integers(0, count, dup.size)] = points[dup]
    return points.reshape(-1)

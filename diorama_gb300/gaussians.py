"""CPU-side layouts of the GPU structs (src/gaussians.ts): 16-float Gaussians,
12-float splats and 45 spherical-harmonic floats per Gaussian."""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

FLOATS_PER_GAUSSIAN = 16  # struct Gaussian: 64 bytes
FLOATS_PER_SPLAT = 12  # struct Splat2D: 48 bytes
# Spherical-harmonic coefficients 1 to 15 per Gaussian, rgb each, coefficient-major.
SH_REST_FLOATS = 45


@dataclass
class Gaussian:
    position: tuple
    scale: tuple
    rotation: tuple  # (w, x, y, z)
    color: tuple
    opacity: float


@dataclass
class Splat2D:
    mean: tuple
    depth: float
    radius: float
    conic: tuple
    color: tuple = field(default=(0.0, 0.0, 0.0, 0.0))  # rgb + opacity


def packGaussians(gaussians) -> np.ndarray:
    data = np.zeros(len(gaussians) * FLOATS_PER_GAUSSIAN, np.float32)
    for i, g in enumerate(gaussians):
        # Float 7 pads scale before the vec4 rotation; float 15 pads the struct.
        data[i * 16 : i * 16 + 16] = [*g.position, g.opacity, *g.scale, 0, *g.rotation, *g.color, 0]
    return data


def packSplats(splats) -> np.ndarray:
    data = np.zeros(len(splats) * FLOATS_PER_SPLAT, np.float32)
    for i, s in enumerate(splats):
        data[i * 12 : i * 12 + 12] = [*s.mean, s.depth, s.radius, *s.conic, 0, *s.color]
    return data


def unpackSplats(data: np.ndarray) -> list[Splat2D]:
    f = np.asarray(data, np.float32).reshape(-1, FLOATS_PER_SPLAT)
    return [Splat2D(mean=(r[0], r[1]), depth=r[2], radius=r[3], conic=(r[4], r[5], r[6]), color=tuple(r[8:12])) for r in f]

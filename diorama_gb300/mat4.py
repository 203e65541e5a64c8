"""4x4 matrices as 16 numbers in column-major order (src/mat4.ts), computed in
double precision on the host like the TypeScript."""

from __future__ import annotations

import math

IDENTITY = [1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0]


def multiply(a, b):
    out = [0.0] * 16
    for col in range(4):
        for row in range(4):
            out[col * 4 + row] = sum(a[k * 4 + row] * b[col * 4 + k] for k in range(4))
    return out


def transform(m, p):
    x, y, z = p
    return [m[r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] for r in range(4)]


def perspective(fov_y, aspect, near, far):
    """WebGPU's 0..1 clip depth (src/mat4.ts:39-48)."""
    f = 1 / math.tan(fov_y / 2)
    depth = 1 / (near - far)
    return [f / aspect, 0, 0, 0, 0, f, 0, 0, 0, 0, far * depth, -1, 0, 0, near * far * depth, 0]


def subtract(a, b):
    return [a[0] - b[0], a[1] - b[1], a[2] - b[2]]


def dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def normalize(v):
    length = math.hypot(v[0], v[1], v[2])
    return [v[0] / length, v[1] / length, v[2] / length]


def lookAt(eye, target, up):
    """A camera at `eye` looking at `target`, down its own -z (src/mat4.ts:51-61)."""
    z = normalize(subtract(eye, target))
    x = normalize(cross(up, z))
    y = cross(z, x)
    return [x[0], y[0], z[0], 0, x[1], y[1], z[1], 0, x[2], y[2], z[2], 0, -dot(x, eye), -dot(y, eye), -dot(z, eye), 1]

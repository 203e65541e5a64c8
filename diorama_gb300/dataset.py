"""Training's starting Gaussians from a point cloud (src/loadDataset.ts:93-149).

meanNeighborDistance2 and initialGaussians keep the reference's signatures
(host arrays in, host arrays out); meanNeighborDistance2Buffers works on device
buffers already holding the points as xyz + padding, as the reference's
`points` buffer does.
"""

from __future__ import annotations

import numpy as np

from . import _lib
from .gaussians import FLOATS_PER_GAUSSIAN, SH_REST_FLOATS
from .gpu import Buffer, Device


def meanNeighborDistance2(device: Device, positions: np.ndarray) -> np.ndarray:
    """For each point (positions: count × 3 floats), the mean squared distance to
    its 3 nearest other points (src/loadDataset.ts:124-149)."""
    positions = np.ascontiguousarray(positions, np.float32).reshape(-1)
    if positions.size % 3:
        raise ValueError("positions must hold 3 floats per point")
    count = positions.size // 3
    out = np.zeros(count, np.float32)
    _lib.call("dg_mean_neighbor_distance2", device.handle, positions.ctypes.data, count, out.ctypes.data)
    return out


def meanNeighborDistance2Buffers(device: Device, points: Buffer, count: int, distance2: Buffer) -> None:
    """meanNeighborDistance2 on device buffers: points holds count × 4 floats
    (xyz + padding), distance2 receives count floats."""
    _lib.call("dg_mean_neighbor_distance2_buffers", device.handle, points.handle, count, distance2.handle)


def initialGaussians(device: Device, positions: np.ndarray, colors: np.ndarray) -> dict:
    """One raw Gaussian per point: its position and colour, opacity 0.1, no
    rotation, and a round size from its 3 nearest neighbours
    (src/loadDataset.ts:99-121). Returns {"params": count × 16, "sh": count × 45}."""
    positions = np.ascontiguousarray(positions, np.float32).reshape(-1)
    colors = np.ascontiguousarray(colors, np.uint8).reshape(-1)
    if positions.size % 3 or colors.size != positions.size:
        raise ValueError("positions and colors must hold 3 values per point")
    count = positions.size // 3
    params = np.zeros(count * FLOATS_PER_GAUSSIAN, np.float32)
    sh = np.zeros(count * SH_REST_FLOATS, np.float32)
    _lib.call("dg_initial_gaussians", device.handle, positions.ctypes.data, colors.ctypes.data, count,
              params.ctypes.data, sh.ctypes.data)
    return {"params": params, "sh": sh}

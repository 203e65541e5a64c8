"""A photo set for training (src/loadDataset.ts, src/colmap.ts, src/sceneCameras.ts):
the COLMAP reconstruction, the train/test split and the scene's extent, the
renderer's camera for each photo, and the starting Gaussians from the
structure-from-motion points.

meanNeighborDistance2 and initialGaussians keep the reference's signatures
(host arrays in, host arrays out); meanNeighborDistance2Buffers works on device
buffers already holding the points as xyz + padding, as the reference's
`points` buffer does. Photos are passed in decoded (rgba8 arrays): decoding
JPEGs is the browser's job in the reference and is not part of this package.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _lib
from .gaussians import FLOATS_PER_GAUSSIAN, SH_REST_FLOATS
from .gpu import Buffer, Device
from .mat4 import dot, perspective
from .renderer import CameraData

# src/loadDataset.ts:10-11: like the reference's --eval, every 8th photo by name is held out.
TEST_EVERY = 8


@dataclass
class TrainingCamera:
    """src/sceneCameras.ts:6-19"""

    name: str
    width: float
    height: float
    position: tuple
    right: tuple  # the camera's axes in world space, OpenCV-style
    down: tuple
    forward: tuple
    fx: float
    fy: float


@dataclass
class Reconstruction:
    cameras: list  # TrainingCamera, sorted by photo name
    positions: np.ndarray  # count × 3 float32
    colors: np.ndarray  # count × 3 uint8


@dataclass
class Dataset:
    name: str
    train: list
    test: list
    positions: np.ndarray
    colors: np.ndarray
    extent: float  # 1.1 × the farthest training camera from their mean


def _pointer(data: bytes):
    arr = np.frombuffer(data, np.uint8)
    return (arr.ctypes.data if arr.size else None), arr.size, arr


def parseColmap(camerasBin: bytes, imagesBin: bytes, pointsBin: bytes) -> Reconstruction:
    """src/colmap.ts:18-31"""
    (cp, cn, ca), (ip, inn, ia), (pp, pn, pa) = _pointer(camerasBin), _pointer(imagesBin), _pointer(pointsBin)
    handle = ctypes.c_void_p()
    _lib.call("dg_parse_colmap", cp, cn, ip, inn, pp, pn, ctypes.byref(handle))
    try:
        cameras = []
        for k in range(int(_lib.fn("dg_colmap_camera_count")(handle))):
            c = _lib.TrainingCameraC()
            _lib.call("dg_colmap_camera", handle, k, ctypes.byref(c))
            cameras.append(TrainingCamera(c.name.decode("utf-8", "replace"), c.width, c.height, tuple(c.position),
                                          tuple(c.right), tuple(c.down), tuple(c.forward), c.fx, c.fy))
        n = int(_lib.fn("dg_colmap_point_count")(handle))
        positions = np.zeros((n, 3), np.float32)
        colors = np.zeros((n, 3), np.uint8)
        _lib.call("dg_colmap_points", handle, positions.ctypes.data, colors.ctypes.data)
    finally:
        _lib.call("dg_colmap_destroy", handle)
    del ca, ia, pa
    return Reconstruction(cameras, positions, colors)


def splitDataset(name: str, reconstruction: Reconstruction) -> Dataset:
    """src/loadDataset.ts:38-48: every 8th photo by name held out; the extent is
    1.1 × the farthest training camera from the training cameras' mean."""
    cams = reconstruction.cameras
    train = [c for i, c in enumerate(cams) if i % TEST_EVERY != 0]
    test = [c for i, c in enumerate(cams) if i % TEST_EVERY == 0]
    centers = [c.position for c in train]
    mean = [sum(c[k] for c in centers) / len(centers) for k in range(3)] if centers else [0.0] * 3
    farthest = max((math.hypot(c[0] - mean[0], c[1] - mean[1], c[2] - mean[2]) for c in centers),
                   default=-math.inf)
    return Dataset(name, train, test, reconstruction.positions, reconstruction.colors, 1.1 * farthest)


def loadDataset(directory) -> Dataset:
    """src/loadDataset.ts:31-49, from <directory>/sparse/0/{cameras,images,points3D}.bin."""
    base = Path(directory) / "sparse" / "0"
    files = []
    for name in ("cameras.bin", "images.bin", "points3D.bin"):
        path = base / name
        if not path.exists():
            raise FileNotFoundError(f"Couldn't load {path}.")
        files.append(path.read_bytes())
    return splitDataset(Path(directory).name, parseColmap(*files))


def verticalFov(camera: TrainingCamera) -> float:
    """src/sceneCameras.ts:53-55"""
    return 2 * math.atan(camera.height / (2 * camera.fy))


def cameraView(camera: TrainingCamera) -> list:
    """src/sceneCameras.ts:58-68: x right, y up, looking down -z."""
    right, position = camera.right, camera.position
    up = [-v for v in camera.down]
    back = [-v for v in camera.forward]
    return [right[0], up[0], back[0], 0, right[1], up[1], back[1], 0, right[2], up[2], back[2], 0,
            -dot(right, position), -dot(up, position), -dot(back, position), 1]


def trainingCameraData(camera: TrainingCamera, viewport) -> CameraData:
    """src/loadDataset.ts:78-84: the renderer's camera for a photo, rendered at viewport."""
    return CameraData(cameraView(camera), perspective(verticalFov(camera), viewport[0] / viewport[1], 0.01, 1000),
                      (viewport[0], viewport[1]))


def loadViews(device: Device, cameras: list, photos: list) -> list:
    """src/loadDataset.ts:57-76 with the photos already decoded: one rgba8 array
    (height × width × 4) per camera, each uploaded and paired with its camera at
    the photo's own size."""
    from .training import TrainingView

    views = []
    for camera, photo in zip(cameras, photos):
        rgba = np.ascontiguousarray(photo, np.uint8)
        h, w = rgba.shape[0], rgba.shape[1]
        tex = device.createTexture(w, h)
        tex.write(rgba.reshape(-1))
        views.append(TrainingView(camera.name, trainingCameraData(camera, (w, h)), tex))
    return views


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

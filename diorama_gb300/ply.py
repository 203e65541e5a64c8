"""parseGaussianPly (src/plyLoader.ts:21-104) and writeGaussianPly
(src/plyWriter.ts:14-43) over the C ABI. Both run on the host; no GPU is needed."""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from .gaussians import FLOATS_PER_GAUSSIAN, SH_REST_FLOATS

SH_C0 = 0.28209479177387814


@dataclass
class GaussianScene:
    count: int
    gaussians: np.ndarray  # count × 16, packed like packGaussians, colour from the degree-0 SH
    shRest: np.ndarray  # count × 45, zero past the file's degree
    shDegree: int


def parseGaussianPly(buffer: bytes) -> GaussianScene:
    data = np.frombuffer(buffer, np.uint8)
    count, degree = ctypes.c_uint32(), ctypes.c_uint32()
    ptr = data.ctypes.data if data.size else None
    _lib.call("dg_parse_gaussian_ply", ptr, data.size, ctypes.byref(count), ctypes.byref(degree), None, None)
    gaussians = np.zeros(count.value * FLOATS_PER_GAUSSIAN, np.float32)
    sh = np.zeros(count.value * SH_REST_FLOATS, np.float32)
    if count.value:
        _lib.call("dg_parse_gaussian_ply", ptr, data.size, ctypes.byref(count), ctypes.byref(degree),
                  gaussians.ctypes.data, sh.ctypes.data)
    return GaussianScene(count.value, gaussians, sh, degree.value)


def writeGaussianPly(raw) -> bytes:
    params = np.ascontiguousarray(raw.params, np.float32).reshape(-1)
    sh = np.ascontiguousarray(raw.sh, np.float32).reshape(-1)
    count = params.size // FLOATS_PER_GAUSSIAN
    if sh.size != count * SH_REST_FLOATS:
        raise ValueError(f"Expected {count * SH_REST_FLOATS} spherical-harmonic floats, got {sh.size}.")
    size = ctypes.c_uint64()
    _lib.call("dg_write_gaussian_ply", params.ctypes.data, sh.ctypes.data, count, None, 0, ctypes.byref(size))
    out = np.empty(size.value, np.uint8)
    _lib.call("dg_write_gaussian_ply", params.ctypes.data, sh.ctypes.data, count, out.ctypes.data, size.value,
              ctypes.byref(size))
    return out.tobytes()

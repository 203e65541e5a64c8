"""The oracle's restatement of the COLMAP sparse-model reader, FOR TESTS ONLY.

Test infrastructure: only tests/ may import it, as the checker. It restates
src/colmap.ts:18-129 (parseColmap) with Python's struct module, in float64, and
writes the same binary format (cameras.bin, images.bin, points3D.bin) so tests
can build reconstructions with known contents.
"""

from __future__ import annotations

import struct

import numpy as np


def rotation_matrix(q):
    """src/colmap.ts:121-128"""
    w, x, y, z = q
    return [[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
            [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
            [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]]


def parse_colmap(cameras_bin: bytes, images_bin: bytes, points_bin: bytes) -> dict:
    """src/colmap.ts:18-31, 71-119. Raises ValueError with the reference's messages."""
    intrinsics = {}
    at = 0

    def take(fmt, data):
        nonlocal at
        values = struct.unpack_from("<" + fmt, data, at)
        at += struct.calcsize("<" + fmt)
        return values

    (count,) = take("Q", cameras_bin)
    for _ in range(count):
        cid, model, width, height = take("iiQQ", cameras_bin)
        if model == 0:
            (f,) = take("d", cameras_bin)
            at += 16
            intrinsics[cid] = (width, height, f, f)
        elif model == 1:
            fx, fy = take("dd", cameras_bin)
            at += 16
            intrinsics[cid] = (width, height, fx, fy)
        else:
            raise ValueError(f"Camera {cid} uses COLMAP model {model}; only undistorted pinhole cameras are supported.")
    at = 0
    cameras = []
    (count,) = take("Q", images_bin)
    for _ in range(count):
        take("i", images_bin)
        q = take("dddd", images_bin)
        t = take("ddd", images_bin)
        (cid,) = take("i", images_bin)
        end = images_bin.index(b"\0", at)
        name = images_bin[at:end].decode()
        at = end + 1
        (points2d,) = take("Q", images_bin)
        at += points2d * 24
        if cid not in intrinsics:
            raise ValueError(f"Photo {name} uses camera {cid}, which isn't in cameras.bin.")
        width, height, fx, fy = intrinsics[cid]
        r = rotation_matrix(q)
        position = tuple(-(r[0][c] * t[0] + r[1][c] * t[1] + r[2][c] * t[2]) for c in range(3))
        cameras.append(dict(name=name, width=float(width), height=float(height), position=position,
                            right=tuple(r[0]), down=tuple(r[1]), forward=tuple(r[2]), fx=fx, fy=fy))
    cameras.sort(key=lambda c: c["name"])
    at = 0
    (count,) = take("Q", points_bin)
    positions = np.zeros((count, 3), np.float32)
    colors = np.zeros((count, 3), np.uint8)
    for i in range(count):
        take("Q", points_bin)
        positions[i] = take("ddd", points_bin)
        colors[i] = take("BBB", points_bin)
        take("d", points_bin)
        (track,) = take("Q", points_bin)
        at += track * 8
    return {"cameras": cameras, "positions": positions, "colors": colors}


def write_cameras(cameras) -> bytes:
    """cameras: (id, model, width, height, params) with 3 (model 0) or 4 (model 1) params."""
    out = struct.pack("<Q", len(cameras))
    for cid, model, width, height, params in cameras:
        out += struct.pack("<iiQQ", cid, model, width, height) + struct.pack(f"<{len(params)}d", *params)
    return out


def write_images(images) -> bytes:
    """images: (id, q (w, x, y, z), t, camera id, name, 2D point count)."""
    out = struct.pack("<Q", len(images))
    for iid, q, t, cid, name, points2d in images:
        out += struct.pack("<i4d3di", iid, *q, *t, cid) + name.encode() + b"\0"
        out += struct.pack("<Q", points2d) + b"\x11" * (24 * points2d)
    return out


def write_points(positions, colors, tracks) -> bytes:
    out = struct.pack("<Q", len(positions))
    for i, (p, c, track) in enumerate(zip(positions, colors, tracks)):
        out += struct.pack("<Q3d3Bd", i + 1, *map(float, p), *map(int, c), 0.5) + struct.pack("<Q", track)
        out += b"\x22" * (8 * track)
    return out

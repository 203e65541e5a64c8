"""The oracle's restatement of the 3DGS .ply reader and writer, FOR TESTS ONLY.

Test infrastructure: only tests/ may import it, as the checker. It restates, with
numpy, src/plyLoader.ts:21-104 (parseGaussianPly) and src/plyWriter.ts:8-43
(writeGaussianPly); the float64 arithmetic there is float64 here, rounded to
float32 where the reference stores into a Float32Array.
"""

from __future__ import annotations

import re

import numpy as np

SH_C0 = 0.28209479177387814
SH_REST_FLOATS = 45

# src/plyWriter.ts:8-12
PROPERTIES = (["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"]
              + [f"f_rest_{k}" for k in range(SH_REST_FLOATS)]
              + ["opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"])


def write_gaussian_ply(params: np.ndarray, sh: np.ndarray) -> bytes:
    """src/plyWriter.ts:14-43"""
    p = np.asarray(params, np.float32).reshape(-1, 16)
    s = np.asarray(sh, np.float32).reshape(-1, SH_REST_FLOATS)
    n = p.shape[0]
    header = "\n".join(["ply", "format binary_little_endian 1.0", f"element vertex {n}",
                        *[f"property float {name}" for name in PROPERTIES], "end_header", ""])
    body = np.zeros((n, len(PROPERTIES)), np.float32)
    body[:, 0:3] = p[:, 0:3]
    body[:, 6:9] = p[:, 12:15]
    per = SH_REST_FLOATS // 3
    for channel in range(3):
        for c in range(per):
            body[:, 9 + channel * per + c] = s[:, c * 3 + channel]
    body[:, 9 + SH_REST_FLOATS] = p[:, 3]
    body[:, 10 + SH_REST_FLOATS:13 + SH_REST_FLOATS] = p[:, 4:7]
    body[:, 13 + SH_REST_FLOATS:17 + SH_REST_FLOATS] = p[:, 8:12]
    return header.encode() + body.astype("<f4").tobytes()


def parse_gaussian_ply(buffer: bytes) -> dict:
    """src/plyLoader.ts:21-104. Raises ValueError with the reference's messages."""
    marker = b"end_header\n"
    at = buffer.find(marker, 0, 64 * 1024)
    if at < 0:
        raise ValueError("No .ply header found.")
    end = at + len(marker)
    header = buffer[:end].decode("utf-8", "replace")
    if not header.startswith("ply\n"):
        raise ValueError("Not a .ply file.")
    if not re.search(r"^format binary_little_endian 1\.0$", header, re.M):
        raise ValueError("Only binary little-endian .ply files are supported.")
    elements, properties, count = [], [], 0
    for line in header.split("\n"):
        words = line.strip().split()
        if not words:
            continue
        if words[0] == "element":
            elements.append(words[1])
            if words[1] == "vertex":
                count = int(words[2])
        elif words[0] == "property" and elements and elements[-1] == "vertex":
            if words[1] != "float":
                raise ValueError(f"Property {words[2]} is {words[1]}; only float properties are supported.")
            properties.append(words[2])
    if not elements or elements[0] != "vertex":
        raise ValueError("Expected the .ply to start with its vertex element.")

    def column(name):
        if name not in properties:
            raise ValueError(f'The .ply has no "{name}" property. Is it a 3D Gaussian Splatting file?')
        return properties.index(name)

    position = [column(n) for n in ("x", "y", "z")]
    dc = [column(f"f_dc_{k}") for k in range(3)]
    opacity = column("opacity")
    scale = [column(f"scale_{k}") for k in range(3)]
    rotation = [column(f"rot_{k}") for k in range(4)]
    rest_count = sum(1 for n in properties if n.startswith("f_rest_"))
    per_channel = rest_count / 3
    degree = round((per_channel + 1) ** 0.5) - 1
    if (degree + 1) ** 2 - 1 != per_channel or degree > 3:
        raise ValueError(f"Unexpected number of spherical-harmonic coefficients ({rest_count}).")
    per_channel = int(per_channel)
    rest = [column(f"f_rest_{k}") for k in range(rest_count)]
    stride = len(properties)
    if end + count * stride * 4 > len(buffer):
        raise ValueError("The .ply file is shorter than its header says.")
    data = np.frombuffer(buffer, "<f4", count * stride, end).reshape(count, stride).astype(np.float64)
    g = np.zeros((count, 16), np.float64)
    g[:, 0:3] = data[:, position]
    g[:, 4:7] = np.exp(data[:, scale])
    g[:, 12:15] = 0.5 + SH_C0 * data[:, dc]
    g[:, 3] = 1 / (1 + np.exp(-data[:, opacity]))
    g[:, 8:12] = data[:, rotation]
    sh = np.zeros((count, SH_REST_FLOATS), np.float64)
    for c in range(per_channel):
        for channel in range(3):
            sh[:, c * 3 + channel] = data[:, rest[channel * per_channel + c]]
    return {"count": count, "gaussians": g.astype(np.float32).reshape(-1),
            "shRest": sh.astype(np.float32).reshape(-1), "shDegree": degree}

"""The .ply reader and writer (src/plyLoader.ts, src/plyWriter.ts) through the C
ABI, against the oracle's restatement and the reference's round-trip check
(src/checks/training.ts:122-136). Host code only: no GPU needed."""

from __future__ import annotations

import numpy as np
import pytest

from diorama_gb300 import DioramaError, RawGaussians, activate
from diorama_gb300.ply import parseGaussianPly, writeGaussianPly
from oracle import ply as oracle_ply


def random_raw(n: int, seed: int) -> RawGaussians:
    rng = np.random.default_rng(seed)
    params = rng.normal(0, 1, (n, 16)).astype(np.float32)
    params[:, 4:7] = rng.uniform(-5, 0, (n, 3))
    params[:, [7, 15]] = 0
    return RawGaussians(params.reshape(-1), rng.normal(0, 0.3, n * 45).astype(np.float32))


def ulps(a, b):
    return np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))


def test_round_trip_matches_the_reference_check():
    raw = random_raw(500, 1)
    scene = parseGaussianPly(writeGaussianPly(raw))
    assert scene.count == 500 and scene.shDegree == 3
    # src/checks/training.ts:129-133
    assert np.abs(scene.gaussians - activate(raw.params)).max() < 1e-6
    assert np.array_equal(scene.shRest, raw.sh)


def test_writer_bytes_match_the_oracle():
    raw = random_raw(300, 2)
    assert writeGaussianPly(raw) == oracle_ply.write_gaussian_ply(raw.params, raw.sh)
    assert writeGaussianPly(RawGaussians(np.zeros(0, np.float32), np.zeros(0, np.float32))) == \
        oracle_ply.write_gaussian_ply(np.zeros(0), np.zeros(0))


def test_reader_matches_the_oracle():
    raw = random_raw(2000, 3)
    data = oracle_ply.write_gaussian_ply(raw.params, raw.sh)
    got, want = parseGaussianPly(data), oracle_ply.parse_gaussian_ply(data)
    assert got.count == want["count"] and got.shDegree == want["shDegree"]
    assert np.array_equal(got.shRest, want["shRest"])
    # float64 exp rounded to float32 on both sides: the two exps may differ in the
    # last double bit, which can move a float by one ulp.
    assert ulps(got.gaussians, want["gaussians"]).max() <= 1


def _ply(properties, rows, extra_header="", fmt="binary_little_endian 1.0", types=None, tail=b""):
    types = types or ["float"] * len(properties)
    header = ["ply", f"format {fmt}", f"element vertex {len(rows)}"]
    header += [f"property {t} {p}" for t, p in zip(types, properties)]
    if extra_header:
        header.append(extra_header)
    header += ["end_header", ""]
    return "\n".join(header).encode() + np.asarray(rows, "<f4").tobytes() + tail


BASE = ["x", "y", "z", "f_dc_0", "f_dc_1", "f_dc_2", "opacity", "scale_0", "scale_1", "scale_2",
        "rot_0", "rot_1", "rot_2", "rot_3"]


@pytest.mark.parametrize("degree", [0, 1, 2, 3])
def test_lower_degrees_and_shuffled_columns(degree):
    rest = [f"f_rest_{k}" for k in range(3 * ((degree + 1) ** 2 - 1))]
    props = list(reversed(BASE + rest)) + ["extra"]
    rows = np.random.default_rng(degree).normal(0, 1, (7, len(props))).astype(np.float32)
    data = _ply(props, rows)
    got, want = parseGaussianPly(data), oracle_ply.parse_gaussian_ply(data)
    assert got.shDegree == degree == want["shDegree"]
    assert np.array_equal(got.shRest, want["shRest"])
    assert ulps(got.gaussians, want["gaussians"]).max() <= 1
    assert not got.shRest.reshape(7, 45)[:, 3 * ((degree + 1) ** 2 - 1):].any()


def test_unaligned_header_and_trailing_elements():
    # A header whose length is not a multiple of 4, and a face element after the
    # vertices (its list property is not read).
    data = _ply(BASE + ["a"], np.ones((3, 15), np.float32), extra_header="comment x",
                tail=b"\x03\x00\x00\x00")
    data = data.replace(b"end_header\n", b"element face 1\nproperty list uchar int vertex_indices\nend_header\n")
    assert parseGaussianPly(data).count == 3 == oracle_ply.parse_gaussian_ply(data)["count"]


@pytest.mark.parametrize("data,message", [
    (b"ply\nformat binary_little_endian 1.0\n", "No .ply header found."),
    (b"plx\nend_header\n", "Not a .ply file."),
    (b"ply\nformat ascii 1.0\nend_header\n", "Only binary little-endian .ply files are supported."),
    (_ply(BASE, np.zeros((1, 14)), types=["double"] + ["float"] * 13),
     "Property x is double; only float properties are supported."),
    (_ply(BASE[1:], np.zeros((1, 13))), 'The .ply has no "x" property. Is it a 3D Gaussian Splatting file?'),
    (_ply(BASE + ["f_rest_0", "f_rest_1"], np.zeros((1, 16))),
     "Unexpected number of spherical-harmonic coefficients (2)."),
    (_ply(BASE, np.zeros((2, 14)))[:-4], "The .ply file is shorter than its header says."),
    (b"ply\nformat binary_little_endian 1.0\nelement face 0\nend_header\n",
     "Expected the .ply to start with its vertex element."),
])
def test_errors_carry_the_reference_messages(data, message):
    with pytest.raises(ValueError, match=message.replace(".", r"\.").replace("(", r"\(").replace(")", r"\)")):
        oracle_ply.parse_gaussian_ply(data)
    with pytest.raises(DioramaError) as info:
        parseGaussianPly(data)
    assert message in str(info.value)

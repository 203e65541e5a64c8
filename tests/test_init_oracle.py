"""The oracle's nearest-neighbour distances and starting Gaussians against the
reference's own check (src/checks/dataset.ts:28-80): 3,001 random points with
one duplicate, against a float64 brute force, with its tolerances."""

from __future__ import annotations

import math

import numpy as np

import oracle
from diorama_gb300 import activate
from helpers import neighbor_check_points, neighbor_distance2_f64


def test_neighbor_distances_match_the_reference_check():
    positions, _ = neighbor_check_points()
    got = oracle.mean_neighbor_distance2(positions)
    want = neighbor_distance2_f64(positions)
    # src/checks/dataset.ts:38
    assert np.all(np.abs(got - want) <= 1e-5 * want + 1e-9)
    # The duplicated pair are each other's nearest neighbour at distance 0.
    assert got[7] < want[7] * 2 and got[1000] == got[7]


def test_starting_gaussians_match_the_reference_check():
    positions, colors = neighbor_check_points()
    d2 = oracle.mean_neighbor_distance2(positions)
    params = oracle.initial_gaussians(positions, colors, d2)
    act = activate(params).reshape(-1, 16)
    cpu = neighbor_distance2_f64(positions)
    p = positions.reshape(-1, 3)
    c = colors.reshape(-1, 3)
    scale = np.sqrt(np.maximum(cpu, 1e-7))
    # src/checks/dataset.ts:45-56
    assert np.all(np.abs(act[:, 0:3] - p) <= 1e-6)
    assert np.all(np.abs(act[:, 4:7] - scale[:, None]) <= 1e-4 * scale[:, None])
    assert np.all(np.abs(act[:, 12:15] - c / 255) <= 1e-5)
    assert np.all(np.abs(act[:, 3] - 0.1) <= 1e-6)
    assert np.array_equal(act[:, 8:12], np.tile([1, 0, 0, 0], (p.shape[0], 1)).astype(np.float32))
    raw = params.reshape(-1, 16)
    assert raw[0, 3] == np.float32(math.log(0.1 / 0.9))


def test_missing_neighbours_count_as_3_4e38():
    # nearestNeighbors.wgsl:19,43: with two missing neighbours the sum overflows
    # to infinity; with one it is (a + b + 3.4e38) / 3 in float32.
    for n in (1, 2):
        assert np.all(np.isinf(oracle.mean_neighbor_distance2(np.arange(n * 3, dtype=np.float32))))
    three = oracle.mean_neighbor_distance2(np.array([0, 0, 0, 1, 0, 0, 3, 0, 0], np.float32))
    f = np.float32
    assert three[0] == (f(1) + f(9) + f(3.4e38)) / f(3)
    four = oracle.mean_neighbor_distance2(np.array([0, 0, 0, 1, 0, 0, 2, 0, 0, 3, 0, 0], np.float32))
    assert np.array_equal(four, np.array([14 / 3, 6 / 3, 6 / 3, 14 / 3], np.float32))

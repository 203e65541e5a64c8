"""Nearest-neighbour distances and starting Gaussians on the GPU
(src/loadDataset.ts:93-149, src/shaders/nearestNeighbors.wgsl) against the
oracle's brute force: the grid search must find the very same values."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from diorama_gb300.dataset import initialGaussians, meanNeighborDistance2, meanNeighborDistance2Buffers
from helpers import clustered_cloud, neighbor_check_points, neighbor_distance2_f64

pytestmark = pytest.mark.gpu


def test_reference_check_points_bit_exact(device):
    positions, _ = neighbor_check_points()
    got = meanNeighborDistance2(device, positions)
    assert np.array_equal(got, oracle.mean_neighbor_distance2(positions))
    want = neighbor_distance2_f64(positions)
    assert np.all(np.abs(got - want) <= 1e-5 * want + 1e-9)  # src/checks/dataset.ts:38


@pytest.mark.parametrize("count,seed", [(20_000, 1), (60_001, 2)])
def test_clustered_cloud_with_outliers_bit_exact(device, count, seed):
    positions = clustered_cloud(count, seed)
    got = meanNeighborDistance2(device, positions)
    assert np.array_equal(got, oracle.mean_neighbor_distance2(positions))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 17])
def test_small_counts(device, n):
    positions = np.random.default_rng(n).uniform(-1, 1, n * 3).astype(np.float32)
    got = meanNeighborDistance2(device, positions)
    assert np.array_equal(got, oracle.mean_neighbor_distance2(positions))


def test_degenerate_clouds(device):
    # All points the same; a line; a plane; points with NaN coordinates, which
    # are nobody's neighbours and get infinity themselves.
    rng = np.random.default_rng(5)
    same = np.tile(np.float32([0.25, -3.0, 7.5]), 1000)
    line = np.zeros((5000, 3), np.float32)
    line[:, 0] = rng.uniform(-1, 1, 5000)
    plane = rng.uniform(-1, 1, (5000, 3)).astype(np.float32)
    plane[:, 2] = 2.0
    nan = rng.uniform(-1, 1, (3000, 3)).astype(np.float32)
    nan[[5, 77, 2999], 1] = np.nan
    for cloud in (same, line.reshape(-1), plane.reshape(-1), nan.reshape(-1)):
        got = meanNeighborDistance2(device, cloud)
        assert np.array_equal(got, oracle.mean_neighbor_distance2(cloud))
    assert np.all(meanNeighborDistance2(device, same) == 0)
    assert np.all(np.isinf(meanNeighborDistance2(device, nan.reshape(-1))[[5, 77, 2999]]))


def test_empty(device):
    assert meanNeighborDistance2(device, np.zeros(0, np.float32)).size == 0


def test_device_buffers(device):
    positions = clustered_cloud(10_000, 9)
    points = np.zeros((10_000, 4), np.float32)
    points[:, :3] = positions.reshape(-1, 3)
    pbuf = device.createBuffer(points.nbytes)
    pbuf.write(points)
    out = device.createBuffer(10_000 * 4)
    meanNeighborDistance2Buffers(device, pbuf, 10_000, out)
    assert np.array_equal(out.read(np.float32), oracle.mean_neighbor_distance2(positions))
    pbuf.destroy()
    out.destroy()


def test_large_cloud_sampled(device):
    # 1.1M points: every point's result is checked for being finite and
    # positive, and 400 sampled points against the brute force over all points.
    positions = clustered_cloud(1_100_000, 3)
    got = meanNeighborDistance2(device, positions)
    which = np.random.default_rng(4).choice(1_100_000, 400, replace=False).astype(np.uint32)
    assert np.array_equal(got[which], oracle.mean_neighbor_distance2_of(positions, which))
    assert np.all(np.isfinite(got))


def test_initial_gaussians_bit_exact(device):
    positions, colors = neighbor_check_points()
    raw = initialGaussians(device, positions, colors)
    d2 = oracle.mean_neighbor_distance2(positions)
    want = oracle.initial_gaussians(positions, colors, d2).reshape(-1, 16)
    got = raw["params"].reshape(-1, 16)
    exact = [k for k in range(16) if k not in (4, 5, 6)]
    assert np.array_equal(got[:, exact], want[:, exact])
    # The log-scale is a float64 log rounded to float32 on both sides; the two
    # logs may differ in their last double bit, which can move the float by 1 ulp.
    ulps = np.abs(got[:, 4:7].view(np.int32) - want[:, 4:7].view(np.int32))
    assert ulps.max() <= 1
    assert not raw["sh"].any() and raw["sh"].size == 3001 * 45

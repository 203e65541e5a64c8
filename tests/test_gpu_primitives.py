"""PrefixSum and RadixSort on the GPU against the reference's checks
(src/checks/depthSort.ts:46-104): bit-exact against sequential and stable CPU
sorts, including partial blocks, ties, device-side counts and large sizes."""

from __future__ import annotations

import math

import numpy as np
import pytest

from diorama_gb300 import PrefixSum, RadixSort
from diorama_gb300.random import mulberry32
from helpers import sort_keys, stable_sort_reference

pytestmark = pytest.mark.gpu


def exclusive(values: np.ndarray) -> np.ndarray:
    out = np.zeros_like(values)
    np.cumsum(values[:-1], out=out[1:])
    return out


def test_prefix_sum_300k(device):
    random = mulberry32(3)
    values = np.array([math.floor(random() * 10) for _ in range(300_000)], np.uint32)
    buf = device.upload(values)
    scan = PrefixSum(device, buf, values.size)
    scan.encode()
    assert np.array_equal(buf.read(np.uint32), exclusive(values))
    assert int(scan.total.read(np.uint32)[0]) == int(values.sum())
    scan.destroy()
    buf.destroy()


@pytest.mark.parametrize("size", [0, 1, 4095, 4096, 4097, 12_000_001])
def test_prefix_sum_sizes(device, size):
    rng = np.random.default_rng(size)
    values = rng.integers(0, 1000, max(size, 1)).astype(np.uint32)
    buf = device.upload(values)
    scan = PrefixSum(device, buf, size)
    scan.encode()
    out = buf.read(np.uint32)
    assert np.array_equal(out[:size], exclusive(values[:size]))
    assert int(scan.total.read(np.uint32)[0]) == int(values[:size].sum(dtype=np.uint64) & 0xFFFFFFFF)
    scan.destroy()
    buf.destroy()


def test_prefix_sum_device_count(device):
    values = np.arange(1, 10_001, dtype=np.uint32)
    buf = device.upload(values)
    count = device.upload(np.array([6000], np.uint32))
    scan = PrefixSum(device, buf, values.size, count)
    scan.encode()
    out = buf.read(np.uint32)
    assert np.array_equal(out[:6000], exclusive(values[:6000]))
    assert np.array_equal(out[6000:], values[6000:])  # past the count: untouched
    assert int(scan.total.read(np.uint32)[0]) == int(values[:6000].sum())
    scan.destroy()
    buf.destroy()
    count.destroy()


# Two-level scans (from 2^21 values): tile sums added up by each re-scanning CTA
# (up to 4096 tiles) or scanned in between (past that), with device counts of
# zero, a partial last tile and the full capacity.
@pytest.mark.parametrize("capacity,n", [(3_000_000, 0), (3_000_000, 2_500_001), (3_000_000, 3_000_000),
                                        (20_000_001, 17_000_000), (20_000_001, 20_000_001)])
def test_prefix_sum_two_level_device_count(device, capacity, n):
    rng = np.random.default_rng(capacity + n)
    values = rng.integers(0, 1000, capacity).astype(np.uint32)
    buf = device.upload(values)
    count = device.upload(np.array([n], np.uint32))
    scan = PrefixSum(device, buf, capacity, count)
    scan.encode()
    out = buf.read(np.uint32)
    assert np.array_equal(out[:n], exclusive(values[:n]))
    assert np.array_equal(out[n:], values[n:])  # past the count: untouched
    assert int(scan.total.read(np.uint32)[0]) == int(values[:n].sum(dtype=np.uint64) & 0xFFFFFFFF)
    assert device.check() == 0
    scan.destroy()
    buf.destroy()
    count.destroy()


@pytest.mark.parametrize("size", [1, 1000, 1024, 3840, 3841, 100_003])
def test_radix_sort_32(device, size):
    keys = sort_keys(size)
    sort = RadixSort(device, size)
    sort.keys.write(keys)
    sort.values.write(np.arange(size, dtype=np.uint32))
    sort.encode()
    order = stable_sort_reference(keys)
    assert np.array_equal(sort.values.read(np.uint32), order)
    assert np.array_equal(sort.keys.read(np.uint32), keys[order])
    sort.destroy()


@pytest.mark.parametrize("size,high_bits", [(3841, 16), (100_003, 16), (2_000_000, 32), (250_000, 8)])
def test_radix_sort_64(device, size, high_bits):
    rng = np.random.default_rng(size)
    low = rng.integers(0, 2**32, size, dtype=np.uint64)
    high = rng.integers(0, 2 ** min(high_bits, 12), size, dtype=np.uint64)  # many equal tiles
    low[::3] = rng.integers(0, 4, low[::3].size)  # and many equal depths
    keys = (high << np.uint64(32)) | low
    sort = RadixSort(device, size, highBits=high_bits)
    sort.keys.write(keys)
    sort.values.write(np.arange(size, dtype=np.uint32))
    sort.encode()
    order = stable_sort_reference(keys)
    assert np.array_equal(sort.values.read(np.uint32), order)
    assert np.array_equal(sort.keys.read(np.uint64), keys[order])
    sort.destroy()


def test_radix_sort_device_count(device):
    size, used = 50_000, 31_337
    keys = sort_keys(size)
    count = device.upload(np.array([used], np.uint32))
    sort = RadixSort(device, size, count=count)
    sort.keys.write(keys)
    sort.values.write(np.arange(size, dtype=np.uint32))
    sort.encode()
    order = stable_sort_reference(keys[:used])
    assert np.array_equal(sort.values.read(np.uint32)[:used], order)
    assert np.array_equal(sort.keys.read(np.uint32)[used:], keys[used:])
    sort.destroy()
    count.destroy()


@pytest.mark.parametrize("pattern", ["equal", "descending", "top_byte_only"])
def test_radix_sort_32_patterns(device, pattern):
    """Stability and digit edge cases: every key equal (the identity order), keys
    in descending order, and keys that differ only in their top byte (three
    passes see a single digit)."""
    size = 50_001
    if pattern == "equal":
        keys = np.full(size, 0xDEADBEEF, np.uint32)
    elif pattern == "descending":
        keys = np.arange(size, 0, -1, dtype=np.uint32) * np.uint32(977)
    else:
        keys = (np.random.default_rng(5).integers(0, 256, size, dtype=np.uint32) << np.uint32(24)) | np.uint32(0x123456)
    sort = RadixSort(device, size)
    sort.keys.write(keys)
    sort.values.write(np.arange(size, dtype=np.uint32))
    sort.encode()
    order = stable_sort_reference(keys)
    assert np.array_equal(sort.values.read(np.uint32), order)
    assert np.array_equal(sort.keys.read(np.uint32), keys[order])
    sort.destroy()


def test_radix_sort_device_count_zero(device):
    """A device-side count of 0 sorts nothing: keys and values stay as written."""
    size = 10_000
    keys = sort_keys(size)
    count = device.upload(np.array([0], np.uint32))
    sort = RadixSort(device, size, count=count)
    sort.keys.write(keys)
    sort.values.write(np.arange(size, dtype=np.uint32))
    sort.encode()
    assert np.array_equal(sort.keys.read(np.uint32), keys)
    assert np.array_equal(sort.values.read(np.uint32), np.arange(size, dtype=np.uint32))
    sort.destroy()
    count.destroy()


def test_no_bounded_wait_gave_up(device):
    assert device.check() == 0

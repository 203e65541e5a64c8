"""The allocation-free scan entry point, dg_prefix_sum_no_alloc.

Some callers cannot allocate device memory (a fixed memory budget, no implicit
synchronization allowed, or a host that owns every allocation). This entry point
serves them: it keeps its scratch in an array inside the library. Here it is
called through the C ABI with device memory the test owns (dg_buffer_create) on
the legacy default stream. Its output must equal the sequential exclusive scan
(numpy's cumsum) and the existing PrefixSum's (dg_prefix_sum_*) exactly, as every
integer result in these tests must: two calls in a row, an empty scan, the
largest scan it accepts, and a large call followed by a small one (leftover
look-back words of the large call must not be read). Its give-up word is
reported by dg_prefix_sum_no_alloc_check. This file is named to be collected
last.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from diorama_gb300 import DioramaError, PrefixSum, _lib

pytestmark = pytest.mark.gpu

MAX_VALUES = 1 << 24
DEFAULT_STREAM = None  # the legacy default stream of the current device


def exclusive_scan(values: np.ndarray) -> tuple[np.ndarray, int]:
    """The sequential scan, in u32 arithmetic (wrapping like the GPU's)."""
    inclusive = np.cumsum(values, dtype=np.uint64)
    out = np.zeros(values.size, np.uint64)
    out[1:] = inclusive[:-1]
    total = int(inclusive[-1]) if values.size else 0
    return (out & 0xFFFFFFFF).astype(np.uint32), total & 0xFFFFFFFF


def existing_scan(device, values: np.ndarray):
    buf = device.upload(values)
    scan = PrefixSum(device, buf, values.size)
    scan.encode()
    out = buf.read(np.uint32)[: values.size].copy()
    total = int(scan.total.read(np.uint32)[0])
    scan.destroy()
    buf.destroy()
    return out, total


def no_alloc_scan(device, values: np.ndarray):
    """Scans `values` with the no-alloc entry point in memory the test owns."""
    data = device.createBuffer(max(16, values.size * 4))
    if values.size:
        data.write(values)
    total = device.createBuffer(16)
    total.write(np.array([0xDEADBEEF], np.uint32))
    device.synchronize()  # the context's stream has written the inputs
    status = _lib.fn("dg_prefix_sum_no_alloc")(DEFAULT_STREAM, data.device_pointer, values.size,
                                                total.device_pointer)
    assert status == _lib.DG_OK, _lib.fn("dg_last_error")()
    bits = ctypes.c_uint32(0xFFFF)
    status = _lib.fn("dg_prefix_sum_no_alloc_check")(DEFAULT_STREAM, ctypes.byref(bits))  # waits for the scan
    assert status == _lib.DG_OK and bits.value == 0, _lib.fn("dg_last_error")()
    out = data.read(np.uint32)[: values.size].copy()
    got_total = int(total.read(np.uint32)[0])
    data.destroy()
    total.destroy()
    return out, got_total


def check(device, values: np.ndarray) -> None:
    got, got_total = no_alloc_scan(device, values)
    want, want_total = exclusive_scan(values)
    assert np.array_equal(got, want)
    assert got_total == want_total
    if values.size:
        prefix_sum, prefix_total = existing_scan(device, values)
        assert np.array_equal(got, prefix_sum)
        assert got_total == prefix_total


def test_no_alloc_scan_matches_prefix_sum_twice(device):
    rng = np.random.default_rng(11)
    for size in (300_001, 4_096 * 37 + 5):  # two calls in a row, different sizes and contents
        check(device, rng.integers(0, 1 << 16, size, dtype=np.uint32))


def test_no_alloc_scan_empty_largest_then_small(device):
    rng = np.random.default_rng(12)
    check(device, np.zeros(0, np.uint32))
    # Every one of the array's 4,096 look-back tiles, with sums that wrap past 2^32.
    check(device, rng.integers(0, 1 << 12, MAX_VALUES, dtype=np.uint32))
    check(device, rng.integers(0, 1 << 30, 9_000, dtype=np.uint32))
    check(device, rng.integers(0, 5, 1, dtype=np.uint32))


def test_no_alloc_scan_reports_a_give_up(device):
    # A look-back that gives up sets the give-up word; the check reports it once.
    lib = _lib.load()
    assert lib.dg_prefix_sum_no_alloc_inject_error(DEFAULT_STREAM, 1) == _lib.DG_OK
    bits = ctypes.c_uint32(0)
    assert lib.dg_prefix_sum_no_alloc_check(DEFAULT_STREAM, ctypes.byref(bits)) == _lib.DG_ERROR_DEVICE_WAIT
    assert bits.value == 1
    assert b"gave up" in lib.dg_last_error()
    assert lib.dg_prefix_sum_no_alloc_check(DEFAULT_STREAM, ctypes.byref(bits)) == _lib.DG_OK
    assert bits.value == 0
    # A scan after the report is correct and reports nothing.
    check(device, np.arange(5_000, dtype=np.uint32))


def test_no_alloc_scan_rejects_sizes_past_its_maximum(device):
    lib = _lib.load()
    dummy = device.createBuffer(16)
    status = lib.dg_prefix_sum_no_alloc(None, dummy.device_pointer, MAX_VALUES + 1, dummy.device_pointer)
    assert status == _lib.DG_ERROR_INVALID_ARGUMENT
    assert b"at most 16777216" in lib.dg_last_error()
    assert lib.dg_prefix_sum_no_alloc(None, None, 4, dummy.device_pointer) == _lib.DG_ERROR_INVALID_ARGUMENT
    dummy.destroy()
    with pytest.raises(DioramaError):
        _lib.call("dg_prefix_sum_encode", None)

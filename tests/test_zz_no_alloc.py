"""The allocation-free scan entry point, dg_prefix_sum_no_alloc.

Some callers cannot allocate device memory (a fixed memory budget, no implicit
synchronization allowed, or a host that owns every allocation). This entry point
serves them: it keeps its scratch in an array inside the library. Here it is
called through the C ABI with memory and a stream the test owns, twice in a row
with different inputs, and its output must equal the existing PrefixSum's
(dg_prefix_sum_*) exactly, as every integer result in these tests must. This
file is named to be collected last.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from diorama_gb300 import DioramaError, PrefixSum, _lib

pytestmark = pytest.mark.gpu

MAX_VALUES = 1 << 24


def no_alloc():
    fn = _lib.load().dg_prefix_sum_no_alloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
    fn.restype = ctypes.c_int32
    return fn


def existing_scan(device, values: np.ndarray):
    buf = device.upload(values)
    scan = PrefixSum(device, buf, values.size)
    scan.encode()
    out = buf.read(np.uint32)[: values.size].copy()
    total = int(scan.total.read(np.uint32)[0])
    scan.destroy()
    buf.destroy()
    return out, total


def test_no_alloc_scan_matches_prefix_sum_twice(device):
    torch = pytest.importorskip("torch")
    fn = no_alloc()
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(11)
    for size in (300_001, 4_096 * 37 + 5):  # two calls in a row, different sizes and contents
        values = rng.integers(0, 1 << 16, size, dtype=np.uint32)
        data = torch.from_numpy(values.view(np.int32)).cuda()
        total = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        status = fn(ctypes.c_void_p(stream.cuda_stream), data.data_ptr(), size, total.data_ptr())
        assert status == _lib.DG_OK, _lib.load().dg_last_error()
        stream.synchronize()
        got = data.cpu().numpy().view(np.uint32)
        want, want_total = existing_scan(device, values)
        assert np.array_equal(got, want)
        assert int(total.cpu().numpy().view(np.uint32)[0]) == want_total


def test_no_alloc_scan_rejects_sizes_past_its_maximum(device):
    fn = no_alloc()
    dummy = device.createBuffer(16)
    status = fn(None, dummy.device_pointer, MAX_VALUES + 1, dummy.device_pointer)
    assert status == _lib.DG_ERROR_INVALID_ARGUMENT
    assert b"at most 16777216" in _lib.load().dg_last_error()
    dummy.destroy()
    with pytest.raises(DioramaError):
        _lib.call("dg_prefix_sum_encode", None)

"""PrefixSum (src/prefixSum.ts) and RadixSort (src/radixSort.ts) over the C ABI."""

from __future__ import annotations

import ctypes
from ctypes import c_void_p

from . import _lib
from .gpu import Buffer, Device, borrowed


class PrefixSum:
    """Exclusive u32 prefix sum of `data`, in place. `count`, if given, holds in
    element 0 how many values (at most `capacity`); otherwise all are scanned.
    After encode(), `total` element 0 holds the sum. One kernel launch."""

    def __init__(self, device: Device, data: Buffer, capacity: int, count: Buffer | None = None):
        self.device = device
        handle = c_void_p()
        _lib.call("dg_prefix_sum_create", device.handle, data.handle, capacity, count.handle if count else None,
                  ctypes.byref(handle))
        self.handle = handle
        self.total = borrowed(device, _lib.fn("dg_prefix_sum_total")(handle))

    def encode(self, _pass=None) -> None:
        _lib.call("dg_prefix_sum_encode", self.handle)

    def destroy(self) -> None:
        if self.handle:
            _lib.call("dg_prefix_sum_destroy", self.handle)
            self.handle = None


class RadixSort:
    """Stable radix sort of u32 keys, or of 64-bit keys stored as (low, high) u32
    pairs looking at `highBits` bits of the high word, each with a u32 value.
    Sorted in place in `keys` / `values`; `count` may hold the key count."""

    def __init__(self, device: Device, capacity: int, highBits: int = 0, count: Buffer | None = None):
        self.device = device
        handle = c_void_p()
        _lib.call("dg_radix_sort_create", device.handle, capacity, highBits, count.handle if count else None,
                  ctypes.byref(handle))
        self.handle = handle
        self.capacity = capacity
        self.keys = borrowed(device, _lib.fn("dg_radix_sort_keys")(handle))
        self.values = borrowed(device, _lib.fn("dg_radix_sort_values")(handle))

    def encode(self, _pass=None) -> None:
        _lib.call("dg_radix_sort_encode", self.handle)

    def destroy(self) -> None:
        if self.handle:
            _lib.call("dg_radix_sort_destroy", self.handle)
            self.handle = None

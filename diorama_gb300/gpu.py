"""The device layer: GPUDevice, its queue, command encoders, buffers and rgba8
textures (src/gpu.ts, src/readback.ts), on one CUDA device and one in-order stream.

WebGPU records commands into an encoder and runs them at queue.submit(). Here
every encode call enqueues on the device's stream at once; the stream runs
them in call order, which is the order submit() would. submit() is therefore
a no-op kept for the reference's call shape, and readbacks block until the
work before them is done, like awaiting mapAsync.
"""

from __future__ import annotations

import ctypes
from ctypes import c_uint32, c_uint64, c_void_p

import numpy as np

from . import _lib


class Buffer:
    """A GPUBuffer. Buffers this handle owns are freed by destroy(); buffers an
    object hands out (its getters) belong to that object."""

    def __init__(self, device: "Device", handle, owned: bool):
        self.device = device
        self.handle = handle
        self.owned = owned

    @property
    def size(self) -> int:
        return int(_lib.fn("dg_buffer_size")(self.handle))

    @property
    def device_pointer(self) -> int:
        return int(_lib.fn("dg_buffer_device_pointer")(self.handle) or 0)

    def read(self, dtype=np.uint8, offset: int = 0, size: int | None = None) -> np.ndarray:
        size = self.size - offset if size is None else size
        out = np.empty(size, np.uint8)
        _lib.call("dg_buffer_read", self.handle, offset, out.ctypes.data, size)
        return out.view(dtype)

    def write(self, data, offset: int = 0) -> None:
        arr = np.ascontiguousarray(data)
        _lib.call("dg_buffer_write", self.handle, offset, arr.ctypes.data, arr.nbytes)

    def writePinned(self, pinned: "PinnedArray", offset: int = 0, nbytes: int | None = None) -> None:
        """Enqueue an upload from pinned memory; keep it unchanged until the copy has run."""
        nbytes = pinned.array.nbytes if nbytes is None else nbytes
        _lib.call("dg_buffer_write_pinned", self.handle, offset, pinned.pointer, nbytes)

    def destroy(self) -> None:
        if self.owned and self.handle:
            _lib.call("dg_buffer_destroy", self.handle)
        self.handle = None

    def __eq__(self, other) -> bool:
        return isinstance(other, Buffer) and self.handle_value == other.handle_value

    def __hash__(self) -> int:
        return hash(self.handle_value)

    @property
    def handle_value(self) -> int:
        return int(self.handle.value if isinstance(self.handle, c_void_p) else (self.handle or 0))


def borrowed(device: "Device", handle) -> Buffer | None:
    """Wraps a buffer an object owns (None for a NULL handle)."""
    if not handle:
        return None
    return Buffer(device, c_void_p(handle), owned=False)


class PinnedArray:
    """A numpy array in pinned (page-locked) host memory."""

    def __init__(self, shape, dtype=np.uint8):
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        ptr = c_void_p()
        _lib.call("dg_host_alloc", max(nbytes, 1), ctypes.byref(ptr))
        self.pointer = ptr.value
        raw = (ctypes.c_uint8 * max(nbytes, 1)).from_address(self.pointer)
        self.array = np.frombuffer(raw, np.uint8, nbytes).view(dtype).reshape(shape)

    def free(self) -> None:
        if self.pointer:
            self.array = None
            _lib.call("dg_host_free", c_void_p(self.pointer))
            self.pointer = None


class Event:
    """A CUDA event recorded on the device's stream."""

    def __init__(self, device: "Device"):
        handle = c_void_p()
        _lib.call("dg_event_create", device.handle, ctypes.byref(handle))
        self.handle = handle

    def record(self) -> None:
        _lib.call("dg_event_record", self.handle)

    def elapsed_ms(self, end: "Event") -> float:
        ms = ctypes.c_float()
        _lib.call("dg_event_elapsed", self.handle, end.handle, ctypes.byref(ms))
        return ms.value

    def destroy(self) -> None:
        if self.handle:
            _lib.call("dg_event_destroy", self.handle)
            self.handle = None


class Texture:
    """An rgba8unorm texture: a device byte buffer of width*height*4."""

    def __init__(self, device: "Device", width: int, height: int):
        self.device = device
        self.width = width
        self.height = height
        self.buffer = device.createBuffer(width * height * 4)

    def createView(self) -> "Texture":
        return self

    def read(self) -> np.ndarray:
        return self.buffer.read(np.uint8).reshape(self.height, self.width, 4)

    def write(self, rgba: np.ndarray) -> None:
        self.buffer.write(np.ascontiguousarray(rgba, np.uint8))

    def destroy(self) -> None:
        self.buffer.destroy()


class Queue:
    def __init__(self, device: "Device"):
        self.device = device

    def writeBuffer(self, buffer: Buffer, offset: int, data) -> None:
        buffer.write(data, offset)

    def writeTexture(self, texture: Texture, data) -> None:
        texture.write(data)

    def submit(self, _commands=None) -> None:
        """Work was enqueued when it was encoded; nothing to do."""

    def onSubmittedWorkDone(self) -> None:
        self.device.synchronize()


class CommandEncoder:
    def __init__(self, device: "Device"):
        self.device = device

    def clearBuffer(self, buffer: Buffer, offset: int = 0, size: int | None = None) -> None:
        size = buffer.size - offset if size is None else size
        _lib.call("dg_buffer_clear", buffer.handle, offset, size)

    def copyBufferToBuffer(self, src: Buffer, src_offset: int, dst: Buffer, dst_offset: int, size: int) -> None:
        _lib.call("dg_buffer_copy", src.handle, src_offset, dst.handle, dst_offset, size)

    def beginComputePass(self, *_args, **_kwargs) -> "CommandEncoder":
        return self

    def end(self) -> None:
        pass

    def finish(self) -> None:
        return None


class Device:
    """GPUDevice + queue on CUDA device `index` (initGpu, src/gpu.ts:8-46)."""

    def __init__(self, index: int = 0):
        self.index = index
        handle = c_void_p()
        _lib.call("dg_context_create", index, ctypes.byref(handle))
        self.handle = handle
        self.queue = Queue(self)

    def createBuffer(self, size: int) -> Buffer:
        handle = c_void_p()
        _lib.call("dg_buffer_create", self.handle, int(size), ctypes.byref(handle))
        return Buffer(self, handle, owned=True)

    def createTexture(self, width: int, height: int) -> Texture:
        return Texture(self, width, height)

    def createCommandEncoder(self, *_args, **_kwargs) -> CommandEncoder:
        return CommandEncoder(self)

    def upload(self, data) -> Buffer:
        arr = np.ascontiguousarray(data)
        buf = self.createBuffer(max(arr.nbytes, 4))
        if arr.nbytes:
            buf.write(arr)
        return buf

    def synchronize(self) -> None:
        _lib.call("dg_context_synchronize", self.handle)

    def check(self) -> int:
        """Raises if a bounded GPU wait gave up since the last check."""
        bits = c_uint32()
        _lib.call("dg_context_check", self.handle, ctypes.byref(bits))
        return bits.value

    @property
    def launch_count(self) -> int:
        out = c_uint64()
        _lib.call("dg_context_launch_count", self.handle, ctypes.byref(out))
        return out.value

    def profile(self, enabled: bool) -> None:
        """Starts or stops a profiler's collection (for profilers started with it off)."""
        _lib.call("dg_context_profile", self.handle, int(enabled))

    def setKernelTiming(self, enabled: bool) -> None:
        _lib.call("dg_context_set_kernel_timing", self.handle, int(enabled))

    def kernelTimingReport(self) -> dict:
        """{kernel name: (launches, total ms)} since the last report; synchronizes."""
        buf = ctypes.create_string_buffer(1 << 16)
        _lib.call("dg_context_kernel_timing_report", self.handle, buf, len(buf))
        out = {}
        for line in buf.value.decode().splitlines():
            name, launches, ms = line.split()
            out[name] = (int(launches), float(ms))
        return out

    def event(self) -> Event:
        return Event(self)

    def destroy(self) -> None:
        if self.handle:
            _lib.call("dg_context_destroy", self.handle)
            self.handle = None


def initGpu(index: int = 0) -> Device:
    return Device(index)


def readBuffer(device: Device, buffer: Buffer, dtype=np.uint8) -> np.ndarray:
    """src/readback.ts: the buffer's contents once the work before it is done."""
    return buffer.read(dtype)

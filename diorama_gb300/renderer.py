"""GaussianRenderer (src/gaussianRenderer.ts) and TileRasterizer
(src/tileRasterizer.ts) over the C ABI. Method names and argument meanings are
the reference's; `encoder` arguments are accepted for the same call shape (work
is enqueued on the device's stream as it is encoded)."""

from __future__ import annotations

import ctypes
from ctypes import c_double, c_uint32, c_void_p
from dataclasses import dataclass

import numpy as np

from . import _lib
from .gaussians import FLOATS_PER_GAUSSIAN, SH_REST_FLOATS
from .gpu import Buffer, Device, Texture, borrowed


@dataclass
class CameraData:
    """src/gaussianRenderer.ts:11-15: column-major view and proj, viewport in pixels."""

    view: list
    proj: list
    viewport: tuple

    def to_c(self) -> _lib.Camera:
        cam = _lib.Camera()
        cam.view[:] = [float(v) for v in self.view]
        cam.proj[:] = [float(v) for v in self.proj]
        cam.viewport[:] = [float(self.viewport[0]), float(self.viewport[1])]
        return cam


@dataclass
class SphericalHarmonics:
    rest: np.ndarray
    degree: int


def _target_handle(target):
    if target is None:
        return None
    if isinstance(target, Texture):
        return target.buffer.handle
    return target.handle


class TileRasterizer:
    """Tiles, sorts and blends `count` 2D splats from `splats`, reading the
    viewport from `camera` (a buffer holding the 144-byte Camera uniform)."""

    def __init__(self, device: Device, camera: Buffer, splats: Buffer, count: int, initialPairCapacity: int | None = None,
                 *, _handle=None):
        self.device = device
        if _handle is None:
            handle = c_void_p()
            _lib.call("dg_tile_rasterizer_create", device.handle, camera.handle, splats.handle, count,
                      initialPairCapacity or 0, ctypes.byref(handle))
            self.handle, self.owned = handle, True
        else:
            self.handle, self.owned = c_void_p(_handle), False

    @property
    def lastPairCount(self) -> int:
        return int(_lib.fn("dg_tile_rasterizer_last_pair_count")(self.handle))

    @property
    def pairCapacity(self) -> int:
        return int(_lib.fn("dg_tile_rasterizer_pair_capacity")(self.handle))

    @property
    def debugBuffers(self) -> dict:
        return {
            "pairSplats": borrowed(self.device, _lib.fn("dg_tile_rasterizer_pair_splats")(self.handle)),
            "ranges": borrowed(self.device, _lib.fn("dg_tile_rasterizer_ranges")(self.handle)),
            "pairKeys": borrowed(self.device, _lib.fn("dg_tile_rasterizer_pair_keys")(self.handle)),
            "tileOffsets": borrowed(self.device, _lib.fn("dg_tile_rasterizer_tile_offsets")(self.handle)),
            "pairTotal": borrowed(self.device, _lib.fn("dg_tile_rasterizer_pair_total")(self.handle)),
        }

    @property
    def pixelColor(self) -> Buffer | None:
        return borrowed(self.device, _lib.fn("dg_tile_rasterizer_pixel_color")(self.handle))

    @property
    def pixelLast(self) -> Buffer | None:
        return borrowed(self.device, _lib.fn("dg_tile_rasterizer_pixel_last")(self.handle))

    def encode(self, encoder, target, viewport, background) -> None:
        _lib.call("dg_tile_rasterizer_encode", self.handle, _target_handle(target), _lib.floats(viewport),
                  _lib.floats(background))

    def encodeBackward(self, encoder, viewport, pixelGrads: Buffer, splatGrads: Buffer) -> None:
        _lib.call("dg_tile_rasterizer_encode_backward", self.handle, _lib.floats(viewport), pixelGrads.handle,
                  splatGrads.handle)

    def afterSubmit(self, wait: bool = True) -> None:
        """Reads back the last frame's pair count and grows the pair buffers if it
        did not fit. Blocks until that frame is done unless wait is False."""
        _lib.call("dg_tile_rasterizer_after_submit", self.handle, int(wait))

    def destroy(self) -> None:
        if self.owned and self.handle:
            _lib.call("dg_tile_rasterizer_destroy", self.handle)
        self.handle = None


class GaussianRenderer:
    """Projects 3D Gaussians to 2D splats, then tiles, sorts and blends them; the
    backward pass turns dL/d(pixel colour) into gradients of every parameter."""

    def __init__(self, device: Device, options: dict | None = None, *, initialPairCapacity: int | None = None,
                 _handle=None):
        self.device = device
        options = options or {}
        capacity = initialPairCapacity or options.get("initialPairCapacity") or 0
        if _handle is None:
            handle = c_void_p()
            _lib.call("dg_renderer_create", device.handle, capacity, ctypes.byref(handle))
            self.handle, self.owned = handle, True
        else:
            self.handle, self.owned = c_void_p(_handle), False

    def setGaussians(self, data, sh: SphericalHarmonics | dict | None = None) -> None:
        arr = np.ascontiguousarray(data, np.float32).reshape(-1)
        count = arr.size // FLOATS_PER_GAUSSIAN
        rest, degree = None, 0
        if sh is not None:
            rest = sh.rest if isinstance(sh, SphericalHarmonics) else sh["rest"]
            degree = sh.degree if isinstance(sh, SphericalHarmonics) else sh["degree"]
            rest = np.ascontiguousarray(rest, np.float32).reshape(-1)
        _lib.call("dg_renderer_set_gaussians", self.handle, arr.ctypes.data if count else None, count,
                  rest.ctypes.data if rest is not None else None, rest.size if rest is not None else 0, degree)

    def adoptGaussians(self, count: int, gaussians: Buffer, sh: Buffer, degree: int) -> None:
        _lib.call("dg_renderer_adopt_gaussians", self.handle, count, gaussians.handle, sh.handle, degree)
        gaussians.owned = False  # the renderer owns them now
        sh.owned = False

    def setShDegree(self, degree: int) -> None:
        _lib.call("dg_renderer_set_sh_degree", self.handle, degree)

    @property
    def count(self) -> int:
        return int(_lib.fn("dg_renderer_count")(self.handle))

    def _buffer(self, name: str) -> Buffer | None:
        return borrowed(self.device, _lib.fn(name)(self.handle))

    @property
    def splatBuffer(self) -> Buffer | None:
        return self._buffer("dg_renderer_splat_buffer")

    @property
    def gaussianBuffer(self) -> Buffer | None:
        return self._buffer("dg_renderer_gaussian_buffer")

    @property
    def shBuffer(self) -> Buffer | None:
        return self._buffer("dg_renderer_sh_buffer")

    @property
    def pixelBuffer(self) -> Buffer | None:
        return self._buffer("dg_renderer_pixel_buffer")

    @property
    def pixelLastBuffer(self) -> Buffer | None:
        return self._buffer("dg_renderer_pixel_last_buffer")

    @property
    def gradients(self) -> dict | None:
        g = self._buffer("dg_renderer_gradient_gaussians")
        if g is None:
            return None
        return {"gaussians": g, "sh": self._buffer("dg_renderer_gradient_sh"),
                "splats": self._buffer("dg_renderer_gradient_splats")}

    @property
    def tiles(self) -> TileRasterizer | None:
        h = _lib.fn("dg_renderer_tiles")(self.handle)
        return TileRasterizer(self.device, None, None, 0, _handle=h) if h else None

    @property
    def drawTiles(self) -> TileRasterizer | None:
        h = _lib.fn("dg_renderer_draw_tiles")(self.handle)
        return TileRasterizer(self.device, None, None, 0, _handle=h) if h else None

    def encode(self, encoder, target, camera: CameraData, background) -> None:
        cam = camera.to_c()
        _lib.call("dg_renderer_encode", self.handle, _target_handle(target), ctypes.byref(cam),
                  _lib.floats(background))

    def encodeDraw(self, encoder, target, splats: Buffer, count: int, viewport, background) -> None:
        _lib.call("dg_renderer_encode_draw", self.handle, _target_handle(target), splats.handle, count,
                  _lib.floats(viewport), _lib.floats(background))

    def encodeBackward(self, encoder, pixelGrads: Buffer) -> None:
        _lib.call("dg_renderer_encode_backward", self.handle, pixelGrads.handle)

    def afterSubmit(self, wait: bool = True) -> None:
        _lib.call("dg_renderer_after_submit", self.handle, int(wait))

    # Batched views: no reference counterpart (the reference renders held-out
    # views one at a time); images are bit-identical to encode()'s.
    def renderViews(self, cameras: list[CameraData], background, targets: Buffer | None = None,
                    pixelColors: Buffer | None = None) -> None:
        """Renders every camera's view (all one size) into targets (rgba8 images
        back to back) and pixelColors (vec4 images), each optional."""
        arr = _cameras_c(cameras)
        _lib.call("dg_renderer_render_views", self.handle, arr, len(cameras), _lib.floats(background),
                  targets.handle if targets is not None else None,
                  pixelColors.handle if pixelColors is not None else None)

    def setViewBatching(self, batch: int = 0, coopMin: int = 0, graph: bool = True) -> None:
        _lib.call("dg_renderer_set_view_batching", self.handle, batch, coopMin, int(graph))

    @property
    def viewBatching(self) -> dict:
        batch, coop = c_uint32(), c_uint32()
        _lib.call("dg_renderer_view_batching", self.handle, ctypes.byref(batch), ctypes.byref(coop))
        return {"batch": batch.value, "coopMin": coop.value}

    def setViewTile(self, width: int = 16, height: int = 16) -> None:
        """The blend tiles of batched views: 16 or 32 pixels each way. Images do
        not change with them (each pixel blends its own 16x16 tile's list)."""
        _lib.call("dg_renderer_set_view_tile", self.handle, width, height)

    @property
    def viewTile(self) -> tuple[int, int]:
        width, height = c_uint32(), c_uint32()
        _lib.call("dg_renderer_view_tile", self.handle, ctypes.byref(width), ctypes.byref(height))
        return width.value, height.value

    def tuneViews(self, cameras: list[CameraData], background, targets: Buffer | None = None) -> dict:
        """Times the (views per batch, cooperative threshold) candidates with 16x16
        blend tiles on these views, then the 32x16, 16x32 and 32x32 blend tiles at
        the fastest, and keeps the fastest; returns it and every candidate's
        seconds (in that order)."""
        arr = _cameras_c(cameras)
        batch, coop, tried = c_uint32(), c_uint32(), c_uint32()
        seconds = (c_double * 32)()
        _lib.call("dg_renderer_tune_views", self.handle, arr, len(cameras), _lib.floats(background),
                  targets.handle if targets is not None else None, ctypes.byref(batch), ctypes.byref(coop),
                  seconds, ctypes.byref(tried))
        return {"batch": batch.value, "coopMin": coop.value, "tile": self.viewTile,
                "seconds": list(seconds[: tried.value])}

    @property
    def viewsPixelLast(self) -> Buffer | None:
        return self._buffer("dg_renderer_views_pixel_last")

    def destroy(self) -> None:
        if self.owned and self.handle:
            _lib.call("dg_renderer_destroy", self.handle)
        self.handle = None


def _cameras_c(cameras: list[CameraData]):
    arr = (_lib.Camera * len(cameras))()
    for k, cam in enumerate(cameras):
        arr[k] = cam.to_c()
    return arr


def shRestFloats(count: int) -> int:
    return count * SH_REST_FLOATS

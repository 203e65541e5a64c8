"""Batched views on the GPU (no reference counterpart: the reference renders
held-out views one at a time, src/trainer.ts:371-386).

Held-out views of the planes-and-boxes scene rendered together must give, view
by view, the same pixel colours, last indices and rgba8 images as
GaussianRenderer.encode, bit for bit: in one batch, in several, with and
without graph replay, in blend tiles of 32x16, 16x32 and 32x32 pixels (pixel
colours and images; the last indices then count positions in the blend tile's
list), and with whatever the autotuner picks."""

from __future__ import annotations

import numpy as np
import pytest

from diorama_gb300 import GaussianRenderer, activate, scenes

pytestmark = pytest.mark.gpu

BG = (0.1, 0.2, 0.3)


def _render_singly(device, size):
    raw, sh = scenes.surface_scene(200_000, 22, noise=0.01)
    _train, held = scenes.ring_cameras(**size)
    r = GaussianRenderer(device)
    r.setGaussians(activate(raw), {"rest": sh.reshape(-1), "degree": 3})
    cams = held[:6]
    W, H = cams[0].viewport
    colors, lasts, images = [], [], []
    tex = device.createTexture(W, H)
    for cam in cams:
        for _ in range(2):  # the first frame may grow the pair buffers
            r.encode(None, tex, cam, BG)
            r.afterSubmit()
        colors.append(r.pixelBuffer.read(np.float32)[: W * H * 4].copy())
        lasts.append(r.pixelLastBuffer.read(np.uint32)[: W * H].copy())
        images.append(tex.buffer.read(np.uint8)[: W * H * 4].copy())
    tex.destroy()
    return r, cams, colors, lasts, images


@pytest.fixture(scope="module")
def scene(device):
    # 980 x 545: 62 x 35 tiles a view, keys view << 16 | tile.
    s = _render_singly(device, {})
    yield s
    s[0].destroy()


@pytest.fixture(scope="module")
def small_scene(device):
    # 200 x 150: 13 x 10 tiles a view, keys view << 8 | tile.
    s = _render_singly(device, {"width": 200, "height": 150})
    yield s
    s[0].destroy()


def _check(device, r, cams, colors, lasts, images, batch, same_lists=True):
    W, H = cams[0].viewport
    n = len(cams)
    targets = device.createBuffer(n * W * H * 4)
    pixel_colors = device.createBuffer(n * W * H * 16)
    r.renderViews(cams, BG, targets, pixel_colors)
    got_color = pixel_colors.read(np.float32).reshape(n, -1)
    got_image = targets.read(np.uint8).reshape(n, -1)
    for k in range(n):
        assert np.array_equal(got_color[k].view(np.uint32), colors[k].view(np.uint32)), (batch, k)
        assert np.array_equal(got_image[k], images[k]), (batch, k)
    # pixel_last of the last batch: its views are the last `size` ones.
    size = n - (batch * ((n - 1) // batch) if batch else 0)
    last = r.viewsPixelLast.read(np.uint32)[: size * W * H].reshape(size, -1)
    for j in range(size):
        want = lasts[n - size + j]
        if same_lists:
            assert np.array_equal(last[j], want), (batch, j)
        else:  # positions in a longer list: a pixel blended something exactly where it did in 16x16 tiles
            assert np.array_equal(last[j] > 0, want > 0) and np.all(last[j] >= want), (batch, j)
    targets.destroy()
    pixel_colors.destroy()


@pytest.mark.parametrize("batch,graph", [(0, True), (0, False), (4, True), (1, True)])
def test_views_match_single_view_renders(device, scene, batch, graph):
    r, cams, colors, lasts, images = scene
    r.setViewBatching(batch, 0, graph)
    _check(device, r, cams, colors, lasts, images, batch)
    _check(device, r, cams, colors, lasts, images, batch)  # replays the captured batch
    assert device.check() == 0


@pytest.mark.parametrize("batch", [0, 4])
def test_small_views_match_single_view_renders(device, small_scene, batch):
    r, cams, colors, lasts, images = small_scene
    r.setViewBatching(batch, 0, True)
    _check(device, r, cams, colors, lasts, images, batch)
    assert device.check() == 0


def test_300_views_in_one_batch(device):
    """More views than one byte numbers: the (view, depth) sort takes two passes
    over the view's bits and the pair keys carry views up to 299 above the local
    tile; every image still equals its own render."""
    raw, sh = scenes.surface_scene(50_000, 22, noise=0.01)
    train, held = scenes.ring_cameras(width=200, height=150)
    cams = train + held
    assert len(cams) == 300
    r = GaussianRenderer(device)
    r.setGaussians(activate(raw), {"rest": sh.reshape(-1), "degree": 3})
    W, H = cams[0].viewport
    tex = device.createTexture(W, H)
    singles = []
    for cam in cams:
        for _ in range(2):  # the first frame may grow the pair buffers
            r.encode(None, tex, cam, BG)
            r.afterSubmit()
        singles.append(r.pixelBuffer.read(np.float32)[: W * H * 4].copy())
    tex.destroy()
    r.setViewBatching(0, 0, True)
    pixel_colors = device.createBuffer(len(cams) * W * H * 16)
    for _ in range(2):  # the second call replays the captured batch
        r.renderViews(cams, BG, None, pixel_colors)
        got = pixel_colors.read(np.float32).reshape(len(cams), -1)
        for k in range(len(cams)):
            assert np.array_equal(got[k].view(np.uint32), singles[k].view(np.uint32)), k
    pixel_colors.destroy()
    assert device.check() == 0
    r.destroy()


@pytest.mark.parametrize("tile", [(32, 16), (16, 32), (32, 32)])
@pytest.mark.parametrize("batch,coop", [(0, 0), (4, 128)])
def test_blend_tiles_match_single_view_renders(device, scene, small_scene, tile, batch, coop):
    """Blend tiles of several 16x16 tiles: fewer pairs, longer lists, each block
    keeping its own 16x16 tile's entries; the images must not change. The small
    views (13 x 10 tiles) end in half-empty blend tiles; coop 128 sends many
    tiles through the cooperative blend."""
    for r, cams, colors, lasts, images in (scene, small_scene):
        r.setViewTile(*tile)
        assert r.viewTile == tile
        r.setViewBatching(batch, coop, True)
        _check(device, r, cams, colors, lasts, images, batch, same_lists=False)
        _check(device, r, cams, colors, lasts, images, batch, same_lists=False)  # graph replay
        r.setViewTile(16, 16)
    assert device.check() == 0


def test_view_tile_rejects_other_sizes(device, scene):
    from diorama_gb300 import DioramaError
    r = scene[0]
    for bad in ((8, 8), (64, 16), (16, 0)):
        with pytest.raises(DioramaError):
            r.setViewTile(*bad)
    assert r.viewTile == (16, 16)


def test_autotuned_views_match(device, scene):
    r, cams, colors, lasts, images = scene
    tuned = r.tuneViews(cams, BG)
    assert tuned["batch"] in {1, 4, len(cams)} and tuned["coopMin"] in {128, 512, 1024, 2048}
    assert tuned["tile"] in {(16, 16), (32, 16), (16, 32), (32, 32)}
    # 3 batch sizes x 4 thresholds in 16x16 blend tiles, then 3 larger blend tiles.
    assert len(tuned["seconds"]) == 15 and min(tuned["seconds"]) > 0
    assert r.viewBatching == {"batch": tuned["batch"], "coopMin": tuned["coopMin"]}
    assert r.viewTile == tuned["tile"]
    _check(device, r, cams, colors, lasts, images, tuned["batch"], same_lists=tuned["tile"] == (16, 16))
    r.setViewTile(16, 16)

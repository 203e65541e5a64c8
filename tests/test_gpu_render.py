"""The renderer's forward pass on the GPU against the reference's checks
(src/checks/gaussians3d.ts, flatSplats.ts, depthSort.ts:106-146, tiles.ts) and
against the oracle: splats, tile lists and pixels bit for bit."""

from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from diorama_gb300 import (CameraData, DioramaError, Gaussian, GaussianRenderer, Splat2D, packGaussians, packSplats,
                           unpackSplats)
from diorama_gb300.mat4 import IDENTITY, perspective
from diorama_gb300.random import mulberry32
from helpers import TILES_CAMERA, TILES_VIEWPORT, assert_splats_match, cam_array, random_scene

pytestmark = pytest.mark.gpu

TOLERANCE = 2.5 / 255
BACKGROUND = (0.1, 0.2, 0.3)
SIZE = 64
CAMERA64 = CameraData(view=IDENTITY, proj=perspective(math.pi / 2, 1, 0.1, 100), viewport=(SIZE, SIZE))


def render_pixels(device, renderer, camera, background):
    w, h = camera.viewport
    tex = device.createTexture(w, h)
    renderer.encode(device.createCommandEncoder(), tex, camera, background)
    pixels = tex.read()
    tex.destroy()
    return pixels


def oracle_frame(renderer, camera, background):
    """The oracle's tile stage and blend from the GPU's own splats."""
    splats = renderer.splatBuffer.read(np.float32)
    cam = cam_array(camera)
    _, total, keys, values, ranges = oracle.tile_stage(cam, splats)
    color, last, rgba = oracle.rasterize(cam, np.asarray(background, np.float32), splats, values, ranges)
    return dict(splats=splats, total=total, keys=keys, values=values, ranges=ranges, color=color, last=last, rgba=rgba)


def white(position, scale, rotation):
    return Gaussian(position=position, scale=scale, rotation=rotation, color=(1, 1, 1), opacity=0.9)


def test_projection_matches_oracle_and_hand_values(device):
    turn = (math.cos(math.pi / 8), 0, 0, math.sin(math.pi / 8))
    cases = [
        white((0, 0, -4), (0.5, 0.5, 0.5), (1, 0, 0, 0)),
        white((0, 0, -4), (1, 0.25, 0.25), turn),
        white((0, 0, 2), (0.5, 0.5, 0.5), (1, 0, 0, 0)),
        white((1.2, 0.7, -5), (0.3, 0.15, 0.6), (0.8, 0.3, -0.4, 0.2)),
        white((40, 0, -4), (0.2, 0.2, 0.2), (1, 0, 0, 0)),
    ]
    r = GaussianRenderer(device)
    data = packGaussians(cases)
    r.setGaussians(data)
    render_pixels(device, r, CAMERA64, (0, 0, 0))
    gpu = r.splatBuffer.read(np.float32).reshape(-1, 12)
    cpu = oracle.preprocess(cam_array(CAMERA64), data, None, 0).reshape(-1, 12)
    assert_splats_match(gpu, cpu)  # bit for bit, but the cutoff in slot 7
    s = unpackSplats(gpu)
    assert np.allclose(s[0].mean, (32, 32), rtol=1e-4) and s[0].radius == 13
    assert np.allclose(s[0].conic, (1 / 16.3, 0, 1 / 16.3), rtol=1e-4, atol=1e-7)
    assert s[1].radius == 25 and np.allclose(s[1].conic, (34.3 / 276.49, 30 / 276.49, 34.3 / 276.49), rtol=1e-4)
    assert s[2].radius == 0 and s[4].radius == 0
    r.destroy()


def test_draw_order(device):
    # src/checks/depthSort.ts:106-146: listed near-first; the near red one must end on top.
    round_ = lambda p, s, c: Gaussian(position=p, scale=(s, s, s), rotation=(1, 0, 0, 0), color=c, opacity=0.8)  # noqa
    gs = [round_((0, 0, -3), 0.3, (1, 0, 0)), round_((0, 0, 2), 0.3, (0, 1, 0)), round_((0, 0, -5), 0.5, (0, 0, 1))]
    r = GaussianRenderer(device)
    r.setGaussians(packGaussians(gs))
    pixels = render_pixels(device, r, CAMERA64, (0, 0, 0))
    ref = oracle_frame(r, CAMERA64, (0, 0, 0))
    assert np.array_equal(pixels.reshape(-1), ref["rgba"])
    red, _, blue = pixels[32, 32, :3]
    assert red > blue
    r.destroy()


def test_flat_splats_hand_values(device):
    # src/checks/flatSplats.ts:16-30
    splats = [Splat2D((20.5, 12.5), 2, 12, (1 / 16, 0, 1 / 16), (1, 1, 1, 0.8)),
              Splat2D((26.5, 12.5), 1, 12, (1 / 16, 0, 1 / 16), (1, 0, 0, 0.5))]
    probes = [((20, 12), (0.832, 0.67, 0.67)), ((26, 12), (0.63, 0.13, 0.13)), ((20, 20), (0.128, 0.106, 0.106)),
              ((39, 12), (0, 0, 0)), ((20, 51), (0, 0, 0))]
    buf = device.upload(packSplats(splats))
    r = GaussianRenderer(device)
    tex = device.createTexture(SIZE, SIZE)
    r.encodeDraw(None, tex, buf, len(splats), (SIZE, SIZE), (0, 0, 0))
    pixels = tex.read().astype(np.float64) / 255
    for (x, y), expected in probes:
        assert np.abs(pixels[y, x, :3] - expected).max() <= TOLERANCE, (x, y, pixels[y, x])
    r.destroy()
    tex.destroy()
    buf.destroy()


def check_frame_against_oracle(device, r, camera, background):
    pixels = render_pixels(device, r, camera, background)
    ref = oracle_frame(r, camera, background)
    tiles = r.tiles
    debug = tiles.debugBuffers
    pairs = int(debug["pairTotal"].read(np.uint32)[0])
    assert pairs == ref["total"]
    assert pairs <= tiles.pairCapacity
    assert np.array_equal(debug["pairKeys"].read(np.uint64)[:pairs], ref["keys"])
    assert np.array_equal(debug["pairSplats"].read(np.uint32)[:pairs], ref["values"])
    n_tiles = ref["ranges"].size
    assert np.array_equal(debug["ranges"].read(np.uint32)[:n_tiles], ref["ranges"])
    color = r.pixelBuffer.read(np.float32)[: ref["color"].size]
    assert np.array_equal(color.view(np.uint32), ref["color"].view(np.uint32))
    assert np.array_equal(r.pixelLastBuffer.read(np.uint32)[: ref["last"].size], ref["last"])
    assert np.array_equal(pixels.reshape(-1), ref["rgba"])
    return pixels, ref


def test_tile_lists_image_and_growth(device):
    # src/checks/tiles.ts:28-107: 300 splats at 120x90, pair capacity 256 forced to grow.
    r = GaussianRenderer(device, {"initialPairCapacity": 256})
    r.setGaussians(packGaussians(random_scene(300)))
    render_pixels(device, r, TILES_CAMERA, BACKGROUND)
    r.afterSubmit()
    pixels, ref = check_frame_against_oracle(device, r, TILES_CAMERA, BACKGROUND)
    r.afterSubmit()
    tiles = r.tiles
    assert tiles.pairCapacity > 256 and tiles.pairCapacity >= tiles.lastPairCount == ref["total"]
    r.destroy()


def test_opaque_scene(device):
    # src/checks/tiles.ts:111-126: 5,000 large, nearly opaque Gaussians; most pixels stop early.
    r = GaussianRenderer(device)
    r.setGaussians(packGaussians(random_scene(5000, scale=(0.1, 0.6), opacity=(0.9, 0.99))))
    render_pixels(device, r, TILES_CAMERA, BACKGROUND)
    r.afterSubmit()
    _, ref = check_frame_against_oracle(device, r, TILES_CAMERA, BACKGROUND)
    transmittance = ref["color"].reshape(-1, 4)[:, 3]
    assert (transmittance < 0.01).sum() > 0.5 * transmittance.size
    r.destroy()


def test_tile_early_exit(device):
    # src/checks/tiles.ts:132-165: 224 pixels finish in the first batch; 32 blend through three.
    random = mulberry32(13)
    splats = []
    for column in range(14):
        for _ in range(4):
            splats.append(Splat2D((column + 0.5, 8), 1 + len(splats) * 0.001, 24, (1 / 0.25**2, 0, 1 / 100**2),
                                  (random(), random(), random(), 0.99)))
    for k in range(600):
        splats.append(Splat2D((random() * 16, random() * 16), 5 + k * 0.001, 60, (1 / 20**2, 0, 1 / 20**2),
                              (random(), random(), random(), 0.01)))
    buf = device.upload(packSplats(splats))
    r = GaussianRenderer(device, {"initialPairCapacity": 1024})
    tex = device.createTexture(16, 16)
    r.encodeDraw(None, tex, buf, len(splats), (16, 16), BACKGROUND)
    cam = oracle.camera_array(IDENTITY, IDENTITY, (16, 16))
    _, total, keys, values, ranges = oracle.tile_stage(cam, packSplats(splats))
    color, last, rgba = oracle.rasterize(cam, np.asarray(BACKGROUND, np.float32), packSplats(splats), values, ranges)
    assert np.array_equal(tex.read().reshape(-1), rgba)
    gpu_last = r.drawTiles.pixelLast.read(np.uint32)[:256].reshape(16, 16)
    assert (gpu_last[:, :14] <= 56).all() and (gpu_last[:, 14:] > 256).all()
    r.destroy()
    tex.destroy()
    buf.destroy()


def test_sh_colour_matches_oracle(device):
    # src/checks/realScene.ts:89-146: view-dependent colour of degrees 1..3.
    rng = np.random.default_rng(5)
    gs = random_scene(200)
    data = packGaussians(gs)
    sh = rng.normal(0, 0.2, 200 * 45).astype(np.float32)
    r = GaussianRenderer(device)
    for degree in (1, 2, 3):
        r.setGaussians(data, {"rest": sh, "degree": degree})
        render_pixels(device, r, TILES_CAMERA, BACKGROUND)
        gpu = r.splatBuffer.read(np.float32)
        cpu = oracle.preprocess(cam_array(TILES_CAMERA), data, sh, degree)
        assert_splats_match(gpu, cpu)
    r.destroy()


def test_empty_scene_clears_to_background(device):
    r = GaussianRenderer(device)
    pixels = render_pixels(device, r, CAMERA64, (0.1, 0.2, 0.3))
    assert (pixels[..., 0] == 26).all() and (pixels[..., 1] == 51).all() and (pixels[..., 2] == 76).all()
    assert (pixels[..., 3] == 255).all()
    r.destroy()


def test_misuse_raises(device):
    r = GaussianRenderer(device)
    data = packGaussians(random_scene(4))
    with pytest.raises(DioramaError, match="spherical-harmonic"):
        r.setGaussians(data, {"rest": np.zeros(10, np.float32), "degree": 1})
    r.setGaussians(data)
    with pytest.raises(DioramaError, match="more tiles"):
        r.encode(None, None, CameraData(IDENTITY, IDENTITY, (4200, 4200)), (0, 0, 0))
    grads = device.createBuffer(64 * 64 * 16)
    with pytest.raises(DioramaError, match="Encode a frame"):
        r.encodeBackward(None, grads)
    grads.destroy()
    r.destroy()

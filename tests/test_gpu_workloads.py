"""The two random-scene workloads on the GPU.

16,384 Gaussians at 256x256 (SH degree 3): one forward + loss + backward
against the reference's float64 PyTorch oracle (golden vectors in
tests/golden/random_16k.npz; image within 1e-5 max-abs, gradients within 1e-4 of
each group's largest) and bit for bit against the oracle's forward.

1.1M Gaussians over [-3, 3]^3 at 1960x1090 (~12M keys): splats, the
scan of tile counts, the sorted (tile, depth) keys, the permutation and the
per-tile ranges bit for bit against the oracle."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from diorama_gb300 import GaussianRenderer, TileRasterizer, TrainingLoss, scenes
from helpers import GOLDEN, assert_splats_match, cam_array, group_errors

pytestmark = pytest.mark.gpu


def test_random_16k_forward_loss_backward(device):
    g = np.load(GOLDEN / "random_16k.npz")
    raw, sh, camera = scenes.random_scene_16k(0)
    act = scenes.activate64(raw).astype(np.float32)
    W, H = camera.viewport
    r = GaussianRenderer(device)
    r.setGaussians(act.reshape(-1), {"rest": sh.reshape(-1), "degree": 3})
    tex = device.createTexture(W, H)
    r.encode(None, tex, camera, (0, 0, 0))
    r.afterSubmit()
    color = r.pixelBuffer.read(np.float32)[: W * H * 4]
    assert np.abs(color.reshape(-1, 4)[:, :3] - g["image"]).max() <= 1e-5

    cam = cam_array(camera)
    frame = oracle.render(cam, np.zeros(3, np.float32), act, sh, 3)
    assert_splats_match(r.splatBuffer.read(np.float32), frame["splats"])
    assert np.array_equal(color.view(np.uint32), frame["pixel_color"].view(np.uint32))
    assert np.array_equal(r.pixelLastBuffer.read(np.uint32)[: W * H], frame["pixel_last"])

    photo = device.createTexture(W, H)
    photo.write(g["target_rgba8"])
    loss = TrainingLoss(device, W, H)
    loss.encode(None, r.pixelBuffer, photo)
    assert abs(loss.read() - float(g["loss"])) <= 1e-6
    r.encodeBackward(None, loss.pixelGrads)
    grads = r.gradients
    expected = {k: g["grad_" + k] for k in ("position", "scale", "rotation", "opacity", "color", "sh")}
    errors = group_errors(grads["gaussians"].read(np.float32), grads["sh"].read(np.float32), expected)
    assert max(errors.values()) <= 1e-4, errors
    for b in (tex, photo):
        b.destroy()
    loss.destroy()
    r.destroy()


def test_random_1m_sort_scan_ranges_bit_exact(device):
    raw, sh, camera = scenes.random_scene_1m(0)
    act = scenes.activate64(raw).astype(np.float32)
    r = GaussianRenderer(device)
    r.setGaussians(act.reshape(-1), {"rest": sh.reshape(-1), "degree": 3})
    r.encode(None, None, camera, (0, 0, 0))
    r.afterSubmit()  # grow the pair buffers to fit, then render again
    r.encode(None, None, camera, (0, 0, 0))
    r.afterSubmit()
    tiles = r.tiles
    debug = tiles.debugBuffers
    cam = cam_array(camera)
    splats = r.splatBuffer.read(np.float32)
    assert_splats_match(splats, oracle.preprocess(cam, act, sh, 3))
    offsets, total, keys, values, ranges = oracle.tile_stage(cam, splats)
    assert total > 5_000_000
    # The renderer's depth-first tile sort: same pairs, order and ranges.
    assert int(debug["pairTotal"].read(np.uint32)[0]) == total == tiles.lastPairCount
    assert np.array_equal(debug["pairKeys"].read(np.uint64)[:total], keys)
    assert np.array_equal(debug["pairSplats"].read(np.uint32)[:total], values)
    assert np.array_equal(debug["ranges"].read(np.uint32)[: ranges.size], ranges)

    # The reference-structured TileRasterizer on the same splats: the scan of tile
    # counts, the 64-bit (tile, depth) keys sorted in 6 passes, the permutation and
    # the ranges.
    camera_buf = device.upload(cam)  # the 144-byte Camera uniform
    tr = TileRasterizer(device, camera_buf, r.splatBuffer, splats.size // 12, tiles.pairCapacity)
    tr.encode(None, None, camera.viewport, (0, 0, 0))
    tr.afterSubmit()
    d2 = tr.debugBuffers
    assert int(d2["pairTotal"].read(np.uint32)[0]) == total == tr.lastPairCount
    assert np.array_equal(d2["tileOffsets"].read(np.uint32)[: offsets.size], offsets)
    assert np.array_equal(d2["pairKeys"].read(np.uint64)[:total], keys)
    assert np.array_equal(d2["pairSplats"].read(np.uint32)[:total], values)
    assert np.array_equal(d2["ranges"].read(np.uint32)[: ranges.size], ranges)
    assert np.array_equal(tr.pixelColor.read(np.float32), r.pixelBuffer.read(np.float32))
    assert device.check() == 0
    tr.destroy()
    camera_buf.destroy()
    r.destroy()

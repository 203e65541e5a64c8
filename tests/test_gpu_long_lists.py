"""Long tile lists on the GPU: the planes-and-boxes scene grown to 1.1M Gaussians
at 980x545 (4.2M pairs; the longest tile lists hold over 30,000 entries).

The forward pass blends tiles with more than 1024 entries cooperatively (a CTA
per 8x4 block) and every other tile one warp per block; both must give the
oracle's pixel colours and last indices bit for bit. The backward pass walks
each list in 512-entry chunks that start from the forward pass's saved pixel
states; its splat gradients must agree with the oracle's back-to-front walk over
the whole list (src/shaders/rasterizeBackward.wgsl) within 1e-4 of each
gradient's largest magnitude."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from diorama_gb300 import GaussianRenderer, scenes
from helpers import cam_array

pytestmark = pytest.mark.gpu

COOP_MIN, CHUNK = 1024, 512
GRAD_NAMES = ("mean x", "mean y", "conic a", "conic b", "conic c", "opacity", "red", "green", "blue")


def test_long_lists_forward_exact_backward_close(device):
    raw, sh = scenes.surface_scene(1_100_000, 22, noise=0.01)
    act = scenes.activate64(raw).astype(np.float32)
    camera = scenes.ring_cameras()[0][0]
    W, H = camera.viewport
    r = GaussianRenderer(device)
    r.setGaussians(act.reshape(-1), {"rest": sh.reshape(-1), "degree": 3})
    for _ in range(2):  # the first frame grows the pair buffers
        r.encode(None, None, camera, (0, 0, 0))
        r.afterSubmit()
    cam = cam_array(camera)
    frame = oracle.render(cam, np.zeros(3, np.float32), act, sh, 3)
    ranges = frame["ranges"].reshape(-1, 2).astype(np.int64)
    lengths = ranges[:, 1] - ranges[:, 0]
    assert lengths.max() > 16 * COOP_MIN and (lengths > COOP_MIN).sum() > 50
    assert np.array_equal(r.tiles.debugBuffers["ranges"].read(np.uint32)[: frame["ranges"].size], frame["ranges"])
    color = r.pixelBuffer.read(np.float32)[: W * H * 4]
    assert np.array_equal(color.view(np.uint32), frame["pixel_color"].view(np.uint32))
    assert np.array_equal(r.pixelLastBuffer.read(np.uint32)[: W * H], frame["pixel_last"])

    rng = np.random.default_rng(5)
    pixel_grads = np.zeros((W * H, 4), np.float32)
    pixel_grads[:, :3] = rng.normal(0.0, 1e-3, (W * H, 3))
    grads_buf = device.upload(pixel_grads)
    r.encodeBackward(None, grads_buf)
    n = act.shape[0]
    got = r.gradients["splats"].read(np.float32)[: n * 9].reshape(n, 9).astype(np.float64)
    want = oracle.rasterize_backward(cam, np.zeros(3, np.float32), frame["splats"], frame, pixel_grads)
    want = want.reshape(n, 9).astype(np.float64)
    errors = {name: float(np.abs(got[:, k] - want[:, k]).max() / np.abs(want[:, k]).max())
              for k, name in enumerate(GRAD_NAMES)}
    assert max(errors.values()) <= 1e-4, errors
    assert device.check() == 0
    grads_buf.destroy()
    r.destroy()

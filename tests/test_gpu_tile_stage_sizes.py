"""The renderer's depth-first tile stage (depth sort of the splats, the scan of
their tile counts gathered in depth order, pair emission, tile sort, ranges) at
scene sizes on both sides of the sort's 3,840-key and the scan's 4,096-value
tiles, up to a scene larger than the test scenes elsewhere, on scenes where
every third Gaussian repeats the position of the one before it, so equal depths
must stay in index order. The pairs (tile keys and splats, in order), their total
and the per-tile ranges are compared bit for bit with the oracle's tile stage on
the same splats."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from diorama_gb300 import GaussianRenderer, scenes
from helpers import cam_array

pytestmark = pytest.mark.gpu

COUNTS = [1, 1000, 3840, 3841, 4096, 4097, 155_649, 1_600_000]


@pytest.mark.parametrize("count", COUNTS)
def test_depth_first_tile_stage_sizes(device, count):
    raw, sh = scenes.random_gaussians(count, seed=count % 997, half_extent=3.0)
    ties = raw[2::3].shape[0]
    raw[2::3, :3] = raw[1::3, :3][:ties]
    act = scenes.activate64(raw).astype(np.float32)
    camera = scenes.sphere_camera(1, 320, 240)
    r = GaussianRenderer(device)
    r.setGaussians(act.reshape(-1), {"rest": sh.reshape(-1), "degree": 3})
    r.encode(None, None, camera, (0, 0, 0))
    r.afterSubmit()  # grow the pair buffers to fit, then render again
    r.encode(None, None, camera, (0, 0, 0))
    r.afterSubmit()
    debug = r.tiles.debugBuffers
    splats = r.splatBuffer.read(np.float32)[: count * 12]
    offsets, total, keys, values, ranges = oracle.tile_stage(cam_array(camera), splats)
    if count >= 1000:
        assert total > 0
    assert int(debug["pairTotal"].read(np.uint32)[0]) == total == r.tiles.lastPairCount
    assert np.array_equal(debug["pairKeys"].read(np.uint64)[:total], keys)
    assert np.array_equal(debug["pairSplats"].read(np.uint32)[:total], values)
    assert np.array_equal(debug["ranges"].read(np.uint32)[: ranges.size], ranges)
    assert device.check() == 0
    r.destroy()

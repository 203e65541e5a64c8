"""Training checkpoints (no reference counterpart): a resumed trainer holds
exactly the saved state and continues as the original does; the file opens as
a scene with the reference's .ply reader."""

from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

from diorama_gb300 import DEFAULT_SETTINGS, DioramaError, RawGaussians, Trainer, activate
from diorama_gb300.ply import parseGaussianPly, writeGaussianPly
from oracle import ply as oracle_ply
from test_gpu_training import ring_views, scrambled_start, truth_scene

pytestmark = pytest.mark.gpu


def test_resume_continues_the_run(device, tmp_path):
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)
    settings = replace(DEFAULT_SETTINGS, extent=3.85, densifyFrom=20, densifyInterval=25, densifyUntil=80,
                       shDegreeInterval=20)
    a = Trainer(device, RawGaussians(params, np.zeros(60 * 45, np.float32)), views, settings)
    for _ in range(61):
        a.step()
    a.optimize()  # mid-step: the maintenance of step 62 is still due
    path = tmp_path / "run.ply"
    a.saveCheckpoint(path)
    b = Trainer.resume(device, path, views, settings)

    assert (b.count, b.iteration, b.shDegree) == (a.count, a.iteration, a.shDegree) == (a.count, 62, 3)
    ra, rb = a.exportRaw(), b.exportRaw()
    assert np.array_equal(ra.params, rb.params) and np.array_equal(ra.sh, rb.sh)
    for name in ("moments", "stats"):
        assert np.array_equal(a.buffers[name].read(np.float32), b.buffers[name].read(np.float32)), name
    assert [vars(d) for d in a.densifications] == [vars(d) for d in b.densifications]
    assert len(a.densifications) == 2

    # The reference's reader opens the checkpoint as a scene.
    data = path.read_bytes()
    scene, ref = parseGaussianPly(data), oracle_ply.parse_gaussian_ply(data)
    assert scene.count == ref["count"] == a.count and scene.shDegree == 3
    assert np.abs(scene.gaussians - activate(ra.params)).max() < 1e-6

    # Both go on the same way (to the rounding of the backward's atomics).
    a.maintain()
    b.maintain()
    for _ in range(5):
        assert a.nextView() == b.nextView()
        a.step()
        b.step()
    ra, rb = a.exportRaw(), b.exportRaw()
    assert a.count == b.count
    assert np.allclose(ra.params, rb.params, rtol=1e-4, atol=1e-5)
    assert abs(a.lastLoss() - b.lastLoss()) < 1e-4
    a.destroy()
    b.destroy()

    with pytest.raises(DioramaError, match="different number of views"):
        Trainer.resume(device, path, views[:4], settings)
    plain = tmp_path / "plain.ply"
    plain.write_bytes(writeGaussianPly(ra))
    with pytest.raises(DioramaError, match="not a training checkpoint"):
        Trainer.resume(device, plain, views, settings)
    for v in views:
        v.image.destroy()

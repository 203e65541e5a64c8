"""The CUDA gradient chain (GaussianRenderer.encode -> TrainingLoss.encode ->
encodeBackward, through the C ABI) against central finite differences in
float64 (tests/golden/fd_20.npz; see tests/test_fd.py for the fixture and the two
error forms): 20 Gaussians, SH degree 3, all 59 trainable values per Gaussian."""

from __future__ import annotations

import numpy as np
import pytest

from diorama_gb300 import CameraData, GaussianRenderer, TrainingLoss
from test_fd import assert_close_to_fd, fd_errors, fd_fixture

pytestmark = pytest.mark.gpu


def test_cuda_gradient_chain_matches_finite_differences(device):
    d = fd_fixture()
    W, H = (int(v) for v in d["viewport"])
    camera = CameraData(view=[float(v) for v in d["view"]], proj=[float(v) for v in d["proj"]], viewport=(W, H))
    r = GaussianRenderer(device)
    r.setGaussians(d["gaussians"].reshape(-1), {"rest": d["sh"].reshape(-1), "degree": 3})
    photo = device.createTexture(W, H)
    photo.write(d["target_rgba8"])
    loss = TrainingLoss(device, W, H)
    r.encode(None, None, camera, d["background"].astype(np.float32))
    loss.encode(None, r.pixelBuffer, photo)
    r.encodeBackward(None, loss.pixelGrads)
    assert abs(loss.read() - float(d["loss"])) <= 1e-6
    gg = r.gradients["gaussians"].read(np.float32)
    sg = r.gradients["sh"].read(np.float32)
    errors = fd_errors(gg, sg, d)
    assert_close_to_fd(errors)
    loss.destroy()
    r.destroy()
    photo.destroy()

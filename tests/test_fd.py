"""The float32 gradient chain against central finite differences in float64
(tests/golden/fd_20.npz, made by tests/golden/make_golden.py from the tile-chunked
restatement of reference/backward_reference.py's renderer and of
reference/loss_reference.py's loss; the reference checks its autograd the same
way, reference/backward_reference.py:190-207): 20 Gaussians, SH degree 3, all 59
trainable values per Gaussian, through render -> L1 + D-SSIM loss -> both
backward passes. Here the oracle's chain on the CPU; tests/test_gpu_fd.py runs the
CUDA chain against the same differences.

Two error forms per group: the largest error relative to the group's largest
gradient (the reference's own form, src/checks/backward.ts:38), and the
element-wise relative error over the gradients above 1e-3 of the group's largest.
"""

from __future__ import annotations

import numpy as np

import oracle
from helpers import GOLDEN, elementwise_errors

# Group: (slots in the 16-float Gaussian gradient, name in the fixture).
FD_GROUPS = [("position", slice(0, 3)), ("scale", slice(4, 7)), ("rotation", slice(8, 12)), ("opacity", slice(3, 4)),
             ("color", slice(12, 15))]


def fd_fixture() -> dict:
    d = np.load(GOLDEN / "fd_20.npz")
    return {k: d[k] for k in d.files}


def fd_errors(gaussian_grads, sh_grads, d) -> dict:
    """{group: (largest error / group's largest, element-wise largest, element-wise median)}."""
    gg = np.asarray(gaussian_grads, np.float64).reshape(-1, 16)
    out = {}
    for name, cols in FD_GROUPS:
        want = d[f"fd_{name}"].reshape(gg.shape[0], -1)
        got = gg[:, cols]
        worst, median = elementwise_errors(got, want, 1e-3)
        out[name] = (float(np.abs(got - want).max() / np.abs(want).max()), worst, median)
    want = d["fd_sh"].reshape(gg.shape[0], -1)
    got = np.asarray(sh_grads, np.float64).reshape(gg.shape[0], -1)
    worst, median = elementwise_errors(got, want, 1e-3)
    out["sh"] = (float(np.abs(got - want).max() / np.abs(want).max()), worst, median)
    return out


def assert_close_to_fd(errors: dict) -> None:
    for name, (group, worst, median) in errors.items():
        assert group <= 1e-4 and worst <= 1e-3 and median <= 1e-5, (name, errors)


def test_fd_fixture_is_self_consistent():
    d = fd_fixture()
    for name in ("position", "scale", "rotation", "opacity", "color", "sh"):
        fd, ag = d[f"fd_{name}"], d[f"autograd_{name}"]
        assert np.abs(fd - ag).max() <= 1e-6 * np.abs(ag).max(), name
    assert d["gaussians"].shape == (20, 16) and d["sh"].shape == (20, 45)


def test_oracle_gradient_chain_matches_finite_differences():
    d = fd_fixture()
    W, H = (int(v) for v in d["viewport"])
    cam = oracle.camera_array(d["view"], d["proj"], (W, H))
    bg = d["background"].astype(np.float32)
    frame = oracle.render(cam, bg, d["gaussians"], d["sh"], 3)
    value, pixel_grads, _ = oracle.loss(frame["pixel_color"], d["target_rgba8"], W, H)
    assert abs(value - float(d["loss"])) <= 1e-6
    splat_grads = oracle.rasterize_backward(cam, bg, frame["splats"], frame, pixel_grads)
    gg, sg = oracle.preprocess_backward(cam, d["gaussians"], d["sh"], 3, frame["splats"], splat_grads)
    assert_close_to_fd(fd_errors(gg, sg, d))

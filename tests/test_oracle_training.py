"""The oracle's training loop on the CPU (oracle/training.py): its mulberry32
against the C restatement (src/random.ts:3-12), the view order's rounds, and a
short run of the reference's training check scene (src/checks/training.ts:
217-302) whose loss falls and whose schedule (SH degree, densifications, Adam's
step counter) follows src/trainer.ts:192-252."""

from __future__ import annotations

import ctypes
import math

import numpy as np

import oracle
from oracle import training as ot
from diorama_gb300 import packGaussians
from diorama_gb300.mat4 import lookAt, perspective
from test_gpu_training import scrambled_start, truth_scene


def test_mulberry32_matches_c():
    lib = oracle.lib()
    lib.or_mulberry32_next.restype = ctypes.c_double
    lib.or_mulberry32_next.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    for seed in (0, 1, 17, 0xFFFFFFFF):
        state = ctypes.c_uint32(seed)
        py = ot.mulberry32(seed)
        for _ in range(1000):
            assert py() == lib.or_mulberry32_next(ctypes.byref(state))


def check_views():
    truth, random = truth_scene()
    views = []
    packed = packGaussians(truth)
    for k in range(8):
        angle = k / 8 * 2 * math.pi
        eye = [3.5 * math.sin(angle), 1.2, 3.5 * math.cos(angle)]
        cam = oracle.camera_array(lookAt(eye, [0, 0, 0], [0, 1, 0]), perspective(math.pi / 3.5, 1, 0.1, 100), (96, 96))
        views.append((cam, oracle.render(cam, np.zeros(3, np.float32), packed, None, 0)["rgba8"]))
    return truth, random, views


def test_view_order_rounds():
    _truth, random, views = check_views()
    t = ot.Trainer(scrambled_start(*truth_scene()), np.zeros(60 * 45, np.float32), views, ot.Settings())
    taken = [t.next_view() for _ in range(24)]
    for r in range(3):  # every view once per round
        assert sorted(taken[8 * r:8 * r + 8]) == list(range(8))
    assert taken[:8] != taken[8:16]


def test_oracle_loop_schedule_and_progress():
    truth, random, views = check_views()
    params = scrambled_start(truth, random)
    settings = ot.Settings(extent=3.85, shDegreeInterval=30, densifyFrom=20, densifyInterval=25, densifyUntil=80,
                           opacityResetInterval=60)
    t = ot.Trainer(params, np.zeros(60 * 45, np.float32), views, settings)
    losses = []
    for _ in range(100):
        t.step()
        losses.append(t.last_loss)
    assert [d[0] for d in t.densifications] == [25, 50, 75]
    assert t.adamSteps == 97 and t.shDegree == 3 and t.iteration == 100
    assert t.count == t.densifications[-1][2] and t.count > 60
    assert np.mean(losses[15:25]) < 0.95 * np.mean(losses[:10])  # learning before the first split
    # The reset after step 60 caps every opacity at 0.01: the next render is far darker.
    assert losses[60] > 1.3 * np.mean(losses[50:60])
    assert np.isfinite(t.params).all() and np.isfinite(t.sh).all()

"""Host-side logic that needs no GPU: camera math, the seeded generator, the
activation and layouts, settings, and the scenes the benchmark uses."""

from __future__ import annotations

import math

import numpy as np

import oracle
from diorama_gb300 import DEFAULT_SETTINGS, Gaussian, Splat2D, activate, packGaussians, packSplats, unpackSplats
from diorama_gb300 import scenes
from diorama_gb300.mat4 import lookAt, multiply, perspective, transform
from diorama_gb300.random import mulberry32


def test_camera_math():
    # src/checks/flatSplats.ts:68-85
    near, far = 0.1, 100
    vp = multiply(perspective(math.pi / 2, 1, near, far), lookAt([0, 0, 5], [0, 0, 0], [0, 1, 0]))

    def ndc(p):
        x, y, z, w = transform(vp, p)
        return x / w, y / w, z / w

    cx, cy, _ = ndc([0, 0, 0])
    assert abs(cx) < 1e-9 and abs(cy) < 1e-9
    assert ndc([1, 0, 0])[0] > 0 and ndc([0, 1, 0])[1] > 0
    assert abs(ndc([0, 0, 5 - near])[2]) < 1e-6
    assert abs(ndc([0, 0, 5 - far])[2] - 1) < 1e-6


def test_mulberry32_matches_the_c_restatement():
    r = mulberry32(17)
    state = np.array([17], np.uint32)
    import ctypes

    lib = oracle.lib()
    lib.or_mulberry32_next.restype = ctypes.c_double
    lib.or_mulberry32_next.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    s = ctypes.c_uint32(17)
    for _ in range(1000):
        assert r() == lib.or_mulberry32_next(ctypes.byref(s))
    assert state[0] == 17


def test_mulberry32_known_values():
    # The first values of mulberry32(1), the view-shuffle generator of src/trainer.ts:121.
    r = mulberry32(1)
    first = [r() for _ in range(3)]
    assert all(0 <= v < 1 for v in first)
    assert len(set(first)) == 3


def test_activate_matches_oracle():
    raw, _ = scenes.random_gaussians(1000, 3)
    host = activate(raw)
    ref = oracle.activate(raw.reshape(-1))
    mask = np.ones(16, bool)
    mask[[7, 15]] = False
    assert np.allclose(host.reshape(-1, 16)[:, mask], ref.reshape(-1, 16)[:, mask], rtol=2e-7, atol=1e-7)


def test_layout_round_trip():
    g = Gaussian((1, 2, 3), (0.1, 0.2, 0.3), (1, 0, 0, 0), (0.5, 0.6, 0.7), 0.8)
    packed = packGaussians([g])
    assert list(packed) == [1, 2, 3, 0.8000000119, 0.1, 0.2, 0.3, 0, 1, 0, 0, 0, 0.5, 0.6, 0.7, 0] or np.allclose(
        packed, [1, 2, 3, 0.8, 0.1, 0.2, 0.3, 0, 1, 0, 0, 0, 0.5, 0.6, 0.7, 0])
    s = Splat2D((1, 2), 3, 4, (5, 6, 7), (0.1, 0.2, 0.3, 0.4))
    back = unpackSplats(packSplats([s]))[0]
    assert back.radius == 4 and np.allclose(back.conic, (5, 6, 7)) and np.allclose(back.color, s.color)


def test_default_settings_are_the_reference_defaults():
    # src/trainer.ts:65-82
    s = DEFAULT_SETTINGS
    assert s.positionLr == (0.00016, 0.0000016) and s.opacityLr == 0.025 and s.shLr == 0.0025 / 20
    assert (s.densifyFrom, s.densifyUntil, s.densifyInterval, s.opacityResetInterval) == (500, 15000, 100, 3000)


def test_config_scenes_are_seeded():
    a, sa = scenes.random_gaussians(100, 0)
    b, sb = scenes.random_gaussians(100, 0)
    assert np.array_equal(a, b) and np.array_equal(sa, sb)
    q = a[:, 8:12]
    assert np.allclose(np.linalg.norm(q, axis=1), 1, atol=1e-6)
    train, held = scenes.ring_cameras()
    assert len(train) == 263 and len(held) == 37
    assert train[0].viewport == (980, 545)

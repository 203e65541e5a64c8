"""The COLMAP reader and the dataset split (src/colmap.ts, src/loadDataset.ts:31-49,
src/sceneCameras.ts) through the C ABI, against the oracle's restatement, on
reconstructions written with known poses. Host code only: no GPU needed."""

from __future__ import annotations

import math

import numpy as np
import pytest

from diorama_gb300 import DioramaError, cameraView, loadDataset, parseColmap, splitDataset, trainingCameraData
from diorama_gb300.mat4 import transform
from oracle import colmap as oc


def scene(n_images=17, n_points=500, seed=0):
    rng = np.random.default_rng(seed)
    cameras = [(1, 0, 1960, 1090, [1100.0, 980.0, 545.0]), (7, 1, 1200, 800, [900.0, 905.5, 600.0, 400.0])]
    images, centers = [], {}
    for k in range(n_images):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        center = rng.uniform(-4, 4, 3)
        r = np.array(oc.rotation_matrix(q))
        t = -r @ center
        name = f"IMG_{(k * 7919) % 1000:04d}.JPG"
        images.append((k + 1, tuple(q), tuple(t), 1 if k % 3 else 7, name, int(rng.integers(0, 40))))
        centers[name] = center
    positions = rng.normal(0, 2, (n_points, 3))
    colors = rng.integers(0, 256, (n_points, 3))
    tracks = rng.integers(0, 12, n_points)
    files = oc.write_cameras(cameras), oc.write_images(images), oc.write_points(positions, colors, tracks)
    return files, centers, positions, colors


def test_parse_matches_the_oracle():
    files, centers, positions, colors = scene()
    got, want = parseColmap(*files), oc.parse_colmap(*files)
    assert [c.name for c in got.cameras] == [c["name"] for c in want["cameras"]] == sorted(centers)
    for g, w in zip(got.cameras, want["cameras"]):
        for key in ("width", "height", "position", "right", "down", "forward", "fx", "fy"):
            assert getattr(g, key) == w[key], key
        # The camera sits where it was put (to float64 rounding).
        assert np.allclose(g.position, centers[g.name], rtol=0, atol=1e-12)
    assert np.array_equal(got.positions, want["positions"])
    assert np.array_equal(got.positions, positions.astype(np.float32))
    assert np.array_equal(got.colors, want["colors"]) and np.array_equal(got.colors, colors.astype(np.uint8))


def test_split_extent_and_cameras(tmp_path):
    files, centers, _, _ = scene(n_images=17)
    base = tmp_path / "garden" / "sparse" / "0"
    base.mkdir(parents=True)
    for name, data in zip(("cameras.bin", "images.bin", "points3D.bin"), files):
        (base / name).write_bytes(data)
    ds = loadDataset(tmp_path / "garden")
    names = sorted(centers)
    assert ds.name == "garden"
    assert [c.name for c in ds.test] == [names[i] for i in (0, 8, 16)]
    assert [c.name for c in ds.train] == [n for i, n in enumerate(names) if i % 8]
    train_centers = np.array([centers[c.name] for c in ds.train])
    mean = train_centers.mean(0)
    assert math.isclose(ds.extent, 1.1 * np.linalg.norm(train_centers - mean, axis=1).max(), rel_tol=1e-12)
    # The renderer's camera puts the photo's centre at the origin, looking down -z.
    cam = ds.train[0]
    data = trainingCameraData(cam, (980, 545))
    assert np.allclose(transform(data.view, cam.position)[:3], 0, atol=1e-9)
    ahead = [cam.position[k] + cam.forward[k] for k in range(3)]
    assert np.allclose(transform(data.view, ahead)[:3], [0, 0, -1], atol=1e-9)
    assert math.isclose(data.proj[5], 1 / math.tan(math.atan(cam.height / (2 * cam.fy))), rel_tol=1e-12)
    assert cameraView(cam) == data.view


def test_errors():
    files, _, _, _ = scene(n_images=3, n_points=5)
    bad_model = oc.write_cameras([(4, 2, 100, 100, [1.0, 2.0, 3.0, 4.0])])
    with pytest.raises(DioramaError, match="Camera 4 uses COLMAP model 2; only undistorted pinhole"):
        parseColmap(bad_model, files[1], files[2])
    with pytest.raises(ValueError, match="Camera 4 uses COLMAP model 2"):
        oc.parse_colmap(bad_model, files[1], files[2])
    only_seven = oc.write_cameras([(7, 1, 1200, 800, [900.0, 905.5, 600.0, 400.0])])
    with pytest.raises(DioramaError, match=r"Photo IMG_\d+\.JPG uses camera 1, which isn't in cameras.bin"):
        parseColmap(only_seven, files[1], files[2])
    for k in range(3):
        cut = list(files)
        cut[k] = cut[k][:-3]
        with pytest.raises(DioramaError, match="is shorter than its contents say"):
            parseColmap(*cut)
    empty = parseColmap(oc.write_cameras([]), oc.write_images([]), oc.write_points([], [], []))
    assert empty.cameras == [] and empty.positions.shape == (0, 3)

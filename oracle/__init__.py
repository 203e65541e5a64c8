"""The oracle: a CPU restatement of the reference's 3DGS training path, FOR TESTS ONLY.

This package is test infrastructure. Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg may import it, and only as the checker (or as the
timed CPU baseline). The diorama_gb300 library never imports it and has no CPU
fallback.

oracle.c restates, in single precision and in a fixed order of float
operations, the WGSL entry points of the reference (src/shaders/*.wgsl) and
the host arithmetic of src/trainer.ts; each C function cites the WGSL it
follows. This module wraps it with numpy arrays. The restatement is pinned
against the reference's own float64 PyTorch oracles through the fixtures in
tests/golden (reference/backward_reference.py, reference/loss_reference.py).
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build

FLOATS_PER_GAUSSIAN = 16
FLOATS_PER_SPLAT = 12
SH_REST_FLOATS = 45
MOMENT_SLOTS = 61

_lib = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_u32 = ctypes.c_uint32


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(str(path))
        sig = {
            "or_num_threads": (ctypes.c_int, []),
            "dg_exp_ref": (ctypes.c_float, [ctypes.c_float]),
            "or_preprocess": (None, [_f32p, _f32p, _f32p, _u32, _u32, _f32p]),
            "or_count_tiles": (None, [_f32p, _f32p, _u32, _u32p]),
            "or_exclusive_scan": (_u32, [_u32p, _u32]),
            "or_duplicate": (None, [_f32p, _f32p, _u32p, _u32, _u32, _u64p, _u32p]),
            "or_radix_sort": (None, [_u64p, _u32p, _u32, _u32]),
            "or_find_ranges": (None, [_u64p, _u32, _u32p]),
            "or_rasterize": (None, [_f32p, _f32p, _f32p, _u32p, _u32p, _f32p, _u32p, ctypes.c_void_p]),
            "or_rasterize_backward": (None, [_f32p, _f32p, _f32p, _u32, _u32p, _u32p, _u32, _f32p, _u32p, _f32p, _f32p]),
            "or_preprocess_backward": (None, [_f32p, _f32p, _f32p, _u32, _u32, _f32p, _f32p, _f32p, _f32p]),
            "or_loss": (ctypes.c_double, [_f32p, _u8p, ctypes.c_int, ctypes.c_int, _f32p, _f32p]),
            "or_ssim": (ctypes.c_double, [_f32p, _f32p, ctypes.c_int, ctypes.c_int]),
            "or_psnr": (ctypes.c_double, [_f32p, _f32p, ctypes.c_size_t]),
            "or_activate": (None, [_f32p, _u32, _f32p]),
            "or_adam_step": (None, [_f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _u32]),
            "or_reset_opacity": (None, [_f32p, _f32p, _f32p, _u32]),
            "or_accumulate_stats": (None, [_f32p, _f32p, ctypes.c_float, ctypes.c_float, _f32p, _u32]),
            "or_densify_count": (None, [_f32p, _f32p, _u32, _f32p, _u32p, _u32p]),
            "or_densify_scatter": (None, [_f32p, _f32p, _f32p, _f32p, _u32p, _u32, _f32p, _u32, _f32p, _f32p, _f32p]),
            "or_pcg": (_u32, [_u32]),
            "or_mean_neighbor_distance2": (None, [_f32p, _u32, _f32p]),
            "or_mean_neighbor_distance2_of": (None, [_f32p, _u32, _u32p, _u32, _f32p]),
            "or_initial_gaussians": (None, [_f32p, _u8p, _f32p, _u32, _f32p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def num_threads() -> int:
    return lib().or_num_threads()


def camera_array(view, proj, viewport) -> np.ndarray:
    """The 36-float Camera layout: view (column-major), proj, viewport, pad."""
    cam = np.zeros(36, np.float32)
    cam[:16] = np.asarray(view, np.float64).astype(np.float32)
    cam[16:32] = np.asarray(proj, np.float64).astype(np.float32)
    cam[32:34] = viewport
    return cam


def tile_grid(viewport) -> tuple[int, int]:
    return (int(viewport[0]) + 15) // 16, (int(viewport[1]) + 15) // 16


def preprocess(cam, gaussians, sh, degree) -> np.ndarray:
    g = np.ascontiguousarray(gaussians, np.float32).reshape(-1)
    n = g.size // FLOATS_PER_GAUSSIAN
    s = np.ascontiguousarray(sh if sh is not None else np.zeros(n * SH_REST_FLOATS), np.float32).reshape(-1)
    out = np.zeros(n * FLOATS_PER_SPLAT, np.float32)
    lib().or_preprocess(cam, g, s, n, degree, out)
    return out


def tile_stage(cam, splats, capacity=None):
    """count_tiles, scan, duplicate, sort and find_ranges on the CPU. Returns
    (offsets, total, keys, values, ranges) with keys/values cut to the pairs kept."""
    splats = np.ascontiguousarray(splats, np.float32).reshape(-1)
    n = splats.size // FLOATS_PER_SPLAT
    offsets = np.zeros(max(n, 1), np.uint32)
    lib().or_count_tiles(cam, splats, n, offsets)
    total = int(lib().or_exclusive_scan(offsets, n))
    cap = total if capacity is None else capacity
    keys = np.zeros(max(cap, 1), np.uint64)
    values = np.zeros(max(cap, 1), np.uint32)
    lib().or_duplicate(cam, splats, offsets, n, cap, keys, values)
    pairs = min(total, cap)
    lib().or_radix_sort(keys, values, pairs, 16)
    tx, ty = tile_grid(cam[32:34])
    ranges = np.zeros(tx * ty * 2, np.uint32)
    lib().or_find_ranges(keys, pairs, ranges)
    return offsets[:n], total, keys[:pairs], values[:pairs], ranges


def rasterize(cam, bg, splats, pair_splats, ranges):
    w, h = int(cam[32]), int(cam[33])
    color = np.zeros(w * h * 4, np.float32)
    last = np.zeros(w * h, np.uint32)
    rgba = np.zeros(w * h * 4, np.uint8)
    pv = np.ascontiguousarray(pair_splats, np.uint32)
    if pv.size == 0:
        pv = np.zeros(1, np.uint32)
    lib().or_rasterize(cam, np.asarray(bg, np.float32), np.ascontiguousarray(splats, np.float32).reshape(-1), pv,
                       np.ascontiguousarray(ranges, np.uint32), color, last, rgba.ctypes.data)
    return color, last, rgba


def render(cam, bg, gaussians, sh, degree):
    """The forward frame: returns a dict of every intermediate."""
    splats = preprocess(cam, gaussians, sh, degree)
    offsets, total, keys, values, ranges = tile_stage(cam, splats)
    color, last, rgba = rasterize(cam, bg, splats, values, ranges)
    return dict(splats=splats, offsets=offsets, total=total, keys=keys, values=values, ranges=ranges,
                pixel_color=color, pixel_last=last, rgba8=rgba)


def rasterize_backward(cam, bg, splats, frame, pixel_grads):
    n = splats.size // FLOATS_PER_SPLAT
    out = np.zeros(max(n, 1) * 9, np.float32)
    values = frame["values"] if frame["values"].size else np.zeros(1, np.uint32)
    lib().or_rasterize_backward(cam, np.asarray(bg, np.float32), splats, n, values, frame["ranges"],
                                frame["values"].size, frame["pixel_color"], frame["pixel_last"],
                                np.ascontiguousarray(pixel_grads, np.float32).reshape(-1), out)
    return out[: n * 9]


def preprocess_backward(cam, gaussians, sh, degree, splats, splat_grads):
    g = np.ascontiguousarray(gaussians, np.float32).reshape(-1)
    n = g.size // FLOATS_PER_GAUSSIAN
    s = np.ascontiguousarray(sh, np.float32).reshape(-1)
    gg = np.zeros(n * FLOATS_PER_GAUSSIAN, np.float32)
    sg = np.zeros(n * SH_REST_FLOATS, np.float32)
    lib().or_preprocess_backward(cam, g, s, n, degree, splats, np.ascontiguousarray(splat_grads, np.float32), gg, sg)
    return gg, sg


def loss(rendered_vec4, target_rgba8, width, height):
    grads = np.zeros(width * height * 4, np.float32)
    per_pixel = np.zeros(width * height, np.float32)
    value = lib().or_loss(np.ascontiguousarray(rendered_vec4, np.float32).reshape(-1),
                          np.ascontiguousarray(target_rgba8, np.uint8).reshape(-1), width, height, grads, per_pixel)
    return value, grads, per_pixel


def ssim(a_vec4, b_vec4, width, height) -> float:
    return lib().or_ssim(np.ascontiguousarray(a_vec4, np.float32).reshape(-1),
                         np.ascontiguousarray(b_vec4, np.float32).reshape(-1), width, height)


def psnr(a_vec4, b_vec4) -> float:
    a = np.ascontiguousarray(a_vec4, np.float32).reshape(-1)
    return lib().or_psnr(a, np.ascontiguousarray(b_vec4, np.float32).reshape(-1), a.size // 4)


def activate(params) -> np.ndarray:
    p = np.ascontiguousarray(params, np.float32).reshape(-1)
    out = np.zeros_like(p)
    lib().or_activate(p, p.size // FLOATS_PER_GAUSSIAN, out)
    return out


def adam_step(adam_params, params, sh, moments, ggrad, sgrad, gaussians):
    """In place on params, sh, moments and gaussians (all float32 C arrays)."""
    n = params.size // FLOATS_PER_GAUSSIAN
    lib().or_adam_step(np.asarray(adam_params, np.float32), params, sh, moments,
                       np.ascontiguousarray(ggrad, np.float32), np.ascontiguousarray(sgrad, np.float32), gaussians, n)


def reset_opacity(params, moments, gaussians):
    lib().or_reset_opacity(params, moments, gaussians, params.size // FLOATS_PER_GAUSSIAN)


def accumulate_stats(splats, splat_grads, viewport, stats):
    lib().or_accumulate_stats(splats, np.ascontiguousarray(splat_grads, np.float32), float(viewport[0]),
                              float(viewport[1]), stats, stats.size // 4)


def densify(params, stats, sh, moments, dp, seed):
    """count_outputs + scan + scatter. Returns (new_params, new_sh, new_moments, tally[4])."""
    n = params.size // FLOATS_PER_GAUSSIAN
    dpa = np.asarray(dp, np.float32)
    outputs = np.zeros(n, np.uint32)
    tally = np.zeros(4, np.uint32)
    lib().or_densify_count(params, stats, n, dpa, outputs, tally)
    total = int(lib().or_exclusive_scan(outputs, n))
    new_params = np.zeros(total * FLOATS_PER_GAUSSIAN, np.float32)
    new_sh = np.zeros(total * SH_REST_FLOATS, np.float32)
    new_moments = np.zeros(total * MOMENT_SLOTS * 2, np.float32)
    lib().or_densify_scatter(params, stats, sh, moments, outputs, n, dpa, seed, new_params, new_sh, new_moments)
    return new_params, new_sh, new_moments, tally


def mean_neighbor_distance2(positions) -> np.ndarray:
    """Brute-force mean squared distance to the 3 nearest other points
    (positions: n × 3 floats)."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    points = np.zeros((pos.shape[0], 4), np.float32)
    points[:, :3] = pos
    out = np.zeros(pos.shape[0], np.float32)
    lib().or_mean_neighbor_distance2(points.reshape(-1), pos.shape[0], out)
    return out


def mean_neighbor_distance2_of(positions, which) -> np.ndarray:
    """mean_neighbor_distance2 for the listed points only, over all points."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    points = np.zeros((pos.shape[0], 4), np.float32)
    points[:, :3] = pos
    which = np.ascontiguousarray(which, np.uint32)
    out = np.zeros(which.size, np.float32)
    lib().or_mean_neighbor_distance2_of(points.reshape(-1), pos.shape[0], which, which.size, out)
    return out


def initial_gaussians(positions, colors, distance2) -> np.ndarray:
    """The starting raw Gaussians (n × 16 floats) from points, colours and
    neighbour distances."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
    n = pos.size // 3
    params = np.zeros(n * FLOATS_PER_GAUSSIAN, np.float32)
    lib().or_initial_gaussians(pos, np.ascontiguousarray(colors, np.uint8).reshape(-1),
                               np.ascontiguousarray(distance2, np.float32), n, params)
    return params


def exp_ref(x: float) -> float:
    return lib().dg_exp_ref(x)

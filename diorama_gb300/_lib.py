"""ctypes binding of libdiorama_gb300.so (include/diorama_gb300.h).

Every entry point returns a status; `call` turns a nonzero one into a
DioramaError carrying dg_last_error(). There is no fallback: if the library
cannot be loaded, importing the classes that need it raises.
"""

from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int32, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIBRARY = Path(__file__).resolve().parent / "_build" / "libdiorama_gb300.so"

DG_OK = 0
DG_ERROR_INVALID_ARGUMENT = 1
DG_ERROR_CUDA = 2
DG_ERROR_OUT_OF_MEMORY = 3
DG_ERROR_DEVICE_WAIT = 4
DG_ERROR_STATE = 5


class DioramaError(RuntimeError):
    """An error status from the library, with its message."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class Camera(ctypes.Structure):
    _fields_ = [("view", c_float * 16), ("proj", c_float * 16), ("viewport", c_float * 2)]


class TrainingSettingsC(ctypes.Structure):
    _fields_ = [
        ("extent", c_double),
        ("position_lr_steps", c_double),
        ("position_lr", c_double * 2),
        ("opacity_lr", c_double),
        ("scale_lr", c_double),
        ("rotation_lr", c_double),
        ("color_lr", c_double),
        ("sh_lr", c_double),
        ("sh_degree_interval", c_uint32),
        ("densify_from", c_uint32),
        ("densify_until", c_uint32),
        ("densify_interval", c_uint32),
        ("densify_grad_threshold", c_double),
        ("percent_dense", c_double),
        ("min_opacity", c_double),
        ("opacity_reset_interval", c_uint32),
        ("background", c_float * 3),
    ]


class TrainingCameraC(ctypes.Structure):
    _fields_ = [("name", c_char_p), ("width", c_double), ("height", c_double), ("position", c_double * 3),
                ("right", c_double * 3), ("down", c_double * 3), ("forward", c_double * 3), ("fx", c_double),
                ("fy", c_double)]


class TrainingViewC(ctypes.Structure):
    _fields_ = [("camera", Camera), ("image", c_void_p)]


class DensificationC(ctypes.Structure):
    _fields_ = [(name, c_uint32) for name in ("step", "before", "after", "kept", "cloned", "split", "removed")]


_P = c_void_p  # opaque handles
_fp = POINTER(c_float)

# name: (restype, argtypes); restype None means it returns dg_status.
SIGNATURES = {
    "dg_last_error": (c_char_p, []),
    "dg_abi_version": (c_int32, []),
    "dg_context_create": (None, [c_int32, POINTER(_P)]),
    "dg_context_destroy": (None, [_P]),
    "dg_context_synchronize": (None, [_P]),
    "dg_context_check": (None, [_P, POINTER(c_uint32)]),
    "dg_context_launch_count": (None, [_P, POINTER(c_uint64)]),
    "dg_context_set_kernel_timing": (None, [_P, c_int32]),
    "dg_context_profile": (None, [_P, c_int32]),
    "dg_context_kernel_timing_report": (None, [_P, ctypes.c_char_p, c_uint64]),
    "dg_event_create": (None, [_P, POINTER(_P)]),
    "dg_event_record": (None, [_P]),
    "dg_event_elapsed": (None, [_P, _P, POINTER(c_float)]),
    "dg_event_destroy": (None, [_P]),
    "dg_host_alloc": (None, [c_uint64, POINTER(c_void_p)]),
    "dg_host_free": (None, [c_void_p]),
    "dg_buffer_write_pinned": (None, [_P, c_uint64, c_void_p, c_uint64]),
    "dg_trainer_loss_value": (None, [_P, POINTER(c_double)]),
    "dg_trainer_next_view": (None, [_P, POINTER(c_uint32)]),
    "dg_buffer_create": (None, [_P, c_uint64, POINTER(_P)]),
    "dg_buffer_wrap": (None, [_P, c_void_p, c_uint64, POINTER(_P)]),
    "dg_buffer_destroy": (None, [_P]),
    "dg_buffer_size": (c_uint64, [_P]),
    "dg_buffer_device_pointer": (c_void_p, [_P]),
    "dg_buffer_write": (None, [_P, c_uint64, c_void_p, c_uint64]),
    "dg_buffer_read": (None, [_P, c_uint64, c_void_p, c_uint64]),
    "dg_buffer_clear": (None, [_P, c_uint64, c_uint64]),
    "dg_buffer_copy": (None, [_P, c_uint64, _P, c_uint64, c_uint64]),
    "dg_prefix_sum_create": (None, [_P, _P, c_uint32, _P, POINTER(_P)]),
    "dg_prefix_sum_encode": (None, [_P]),
    "dg_prefix_sum_total": (_P, [_P]),
    "dg_prefix_sum_destroy": (None, [_P]),
    "dg_prefix_sum_no_alloc": (None, [c_void_p, c_void_p, c_uint32, c_void_p]),
    "dg_prefix_sum_no_alloc_check": (None, [c_void_p, POINTER(c_uint32)]),
    "dg_prefix_sum_no_alloc_inject_error": (None, [c_void_p, c_uint32]),
    "dg_radix_sort_create": (None, [_P, c_uint32, c_uint32, _P, POINTER(_P)]),
    "dg_radix_sort_keys": (_P, [_P]),
    "dg_radix_sort_values": (_P, [_P]),
    "dg_radix_sort_capacity": (c_uint32, [_P]),
    "dg_radix_sort_encode": (None, [_P]),
    "dg_radix_sort_destroy": (None, [_P]),
    "dg_tile_rasterizer_create": (None, [_P, _P, _P, c_uint32, c_uint32, POINTER(_P)]),
    "dg_tile_rasterizer_encode": (None, [_P, _P, _fp, _fp]),
    "dg_tile_rasterizer_encode_backward": (None, [_P, _fp, _P, _P]),
    "dg_tile_rasterizer_after_submit": (None, [_P, c_int32]),
    "dg_tile_rasterizer_last_pair_count": (c_uint32, [_P]),
    "dg_tile_rasterizer_pair_capacity": (c_uint32, [_P]),
    "dg_tile_rasterizer_pair_splats": (_P, [_P]),
    "dg_tile_rasterizer_ranges": (_P, [_P]),
    "dg_tile_rasterizer_pair_keys": (_P, [_P]),
    "dg_tile_rasterizer_pixel_color": (_P, [_P]),
    "dg_tile_rasterizer_pixel_last": (_P, [_P]),
    "dg_tile_rasterizer_tile_offsets": (_P, [_P]),
    "dg_tile_rasterizer_pair_total": (_P, [_P]),
    "dg_tile_rasterizer_destroy": (None, [_P]),
    "dg_renderer_create": (None, [_P, c_uint32, POINTER(_P)]),
    "dg_renderer_set_gaussians": (None, [_P, c_void_p, c_uint32, c_void_p, c_uint64, c_uint32]),
    "dg_renderer_adopt_gaussians": (None, [_P, c_uint32, _P, _P, c_uint32]),
    "dg_renderer_set_sh_degree": (None, [_P, c_uint32]),
    "dg_renderer_encode": (None, [_P, _P, POINTER(Camera), _fp]),
    "dg_renderer_encode_draw": (None, [_P, _P, _P, c_uint32, _fp, _fp]),
    "dg_renderer_encode_backward": (None, [_P, _P]),
    "dg_renderer_after_submit": (None, [_P, c_int32]),
    "dg_renderer_count": (c_uint32, [_P]),
    "dg_renderer_splat_buffer": (_P, [_P]),
    "dg_renderer_gaussian_buffer": (_P, [_P]),
    "dg_renderer_sh_buffer": (_P, [_P]),
    "dg_renderer_pixel_buffer": (_P, [_P]),
    "dg_renderer_pixel_last_buffer": (_P, [_P]),
    "dg_renderer_gradient_gaussians": (_P, [_P]),
    "dg_renderer_gradient_sh": (_P, [_P]),
    "dg_renderer_gradient_splats": (_P, [_P]),
    "dg_renderer_tiles": (_P, [_P]),
    "dg_renderer_draw_tiles": (_P, [_P]),
    "dg_renderer_destroy": (None, [_P]),
    "dg_renderer_render_views": (None, [_P, POINTER(Camera), c_uint32, _fp, _P, _P]),
    "dg_renderer_set_view_batching": (None, [_P, c_uint32, c_uint32, c_int32]),
    "dg_renderer_view_batching": (None, [_P, POINTER(c_uint32), POINTER(c_uint32)]),
    "dg_renderer_set_view_tile": (None, [_P, c_uint32, c_uint32]),
    "dg_renderer_view_tile": (None, [_P, POINTER(c_uint32), POINTER(c_uint32)]),
    "dg_renderer_tune_views": (None, [_P, POINTER(Camera), c_uint32, _fp, _P, POINTER(c_uint32), POINTER(c_uint32),
                                      POINTER(c_double), POINTER(c_uint32)]),
    "dg_renderer_views_pixel_last": (c_void_p, [_P]),
    "dg_training_loss_create": (None, [_P, c_uint32, c_uint32, POINTER(_P)]),
    "dg_training_loss_encode": (None, [_P, _P, _P]),
    "dg_training_loss_pixel_grads": (_P, [_P]),
    "dg_training_loss_pixel_loss": (_P, [_P]),
    "dg_training_loss_read": (None, [_P, POINTER(c_double)]),
    "dg_training_loss_destroy": (None, [_P]),
    "dg_training_settings_default": (c_void_p, [POINTER(TrainingSettingsC), c_double]),
    "dg_trainer_create": (None, [_P, c_void_p, c_void_p, c_uint32, POINTER(TrainingViewC), c_uint32,
                                 POINTER(TrainingSettingsC), POINTER(_P)]),
    "dg_trainer_step": (None, [_P]),
    "dg_trainer_optimize": (None, [_P]),
    "dg_trainer_maintain": (None, [_P]),
    "dg_trainer_densify": (None, [_P, c_int32]),
    "dg_trainer_reset_opacity": (None, [_P]),
    "dg_trainer_export_raw": (None, [_P, c_void_p, c_void_p]),
    "dg_trainer_last_loss": (None, [_P, POINTER(c_double)]),
    "dg_trainer_evaluate": (None, [_P, POINTER(TrainingViewC), c_uint32, c_int32, POINTER(c_double),
                                   POINTER(c_double)]),
    "dg_trainer_iteration": (c_uint32, [_P]),
    "dg_trainer_set_iteration": (None, [_P, c_uint32]),
    "dg_trainer_sh_degree": (c_uint32, [_P]),
    "dg_trainer_adam_steps": (c_uint32, [_P]),
    "dg_trainer_count": (c_uint32, [_P]),
    "dg_trainer_renderer": (_P, [_P]),
    "dg_trainer_params": (_P, [_P]),
    "dg_trainer_moments": (_P, [_P]),
    "dg_trainer_stats": (_P, [_P]),
    "dg_trainer_densification_count": (c_uint32, [_P]),
    "dg_trainer_densification": (None, [_P, c_uint32, POINTER(DensificationC)]),
    "dg_trainer_set_graph": (None, [_P, c_int32]),
    "dg_trainer_set_keep_gradients": (None, [_P, c_int32]),
    "dg_trainer_request_loss": (None, [_P]),
    "dg_trainer_set_host_photos": (None, [_P, c_void_p, c_uint32]),
    "dg_trainer_take_loss": (None, [_P, c_int32, POINTER(c_double), POINTER(c_int32)]),
    "dg_trainer_save_checkpoint": (None, [_P, c_char_p]),
    "dg_trainer_resume": (None, [_P, c_char_p, c_void_p, c_uint32, c_void_p, POINTER(_P)]),
    "dg_parse_gaussian_ply": (None, [c_void_p, c_uint64, POINTER(c_uint32), POINTER(c_uint32), c_void_p, c_void_p]),
    "dg_write_gaussian_ply": (None, [c_void_p, c_void_p, c_uint32, c_void_p, c_uint64, POINTER(c_uint64)]),
    "dg_parse_colmap": (None, [c_void_p, c_uint64, c_void_p, c_uint64, c_void_p, c_uint64, POINTER(_P)]),
    "dg_colmap_camera_count": (c_uint32, [_P]),
    "dg_colmap_camera": (None, [_P, c_uint32, POINTER(TrainingCameraC)]),
    "dg_colmap_point_count": (c_uint64, [_P]),
    "dg_colmap_points": (None, [_P, c_void_p, c_void_p]),
    "dg_colmap_destroy": (None, [_P]),
    "dg_mean_neighbor_distance2": (None, [_P, c_void_p, c_uint32, c_void_p]),
    "dg_mean_neighbor_distance2_buffers": (None, [_P, _P, c_uint32, _P]),
    "dg_initial_gaussians": (None, [_P, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p]),
    "dg_trainer_destroy": (None, [_P]),
    "dg_densify_mlp_create": (None, [_P, c_uint32, POINTER(c_void_p)]),
    "dg_densify_mlp_train": (None, [_P, c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_float, c_float, c_int32,
                                    c_uint32, POINTER(c_double)]),
    "dg_densify_mlp_predict": (None, [_P, _P, c_uint32, _P]),
    "dg_densify_mlp_gradient": (None, [_P, c_void_p, c_void_p, c_uint32, c_void_p]),
    "dg_densify_mlp_get_weights": (None, [_P, c_void_p]),
    "dg_densify_mlp_set_weights": (None, [_P, c_void_p]),
    "dg_densify_mlp_destroy": (None, [_P]),
    "dg_trainer_set_densify_log": (None, [_P, c_int32, c_uint32]),
    "dg_trainer_take_densify_samples": (None, [_P, c_void_p, c_void_p, c_uint32, POINTER(c_uint32),
                                               POINTER(c_uint32)]),
    "dg_trainer_set_densify_mlp": (None, [_P, _P, c_float]),
    "dg_trainer_densify_mlp_stats": (None, [_P, POINTER(c_uint64), POINTER(c_uint64), POINTER(c_uint64)]),
}

_lib = None


def load(path: Path | str | None = None):
    """Loads the library (building it first if it is missing and nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    target = Path(path) if path else LIBRARY
    if not target.exists():
        from . import build as _build

        _build.build()
    lib = ctypes.CDLL(str(target))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = c_int32 if res is None else res
    _lib = lib
    return lib


def call(name: str, *args) -> None:
    """Calls a status-returning entry point and raises DioramaError on failure."""
    lib = load()
    status = getattr(lib, name)(*args)
    if status != DG_OK:
        raise DioramaError(status, lib.dg_last_error().decode("utf-8", "replace"))


def fn(name: str):
    return getattr(load(), name)


def out_handle() -> c_void_p:
    return c_void_p()


def floats(values) -> ctypes.Array:
    values = list(values)
    return (c_float * len(values))(*values)

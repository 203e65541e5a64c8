"""TrainingLoss (src/trainingLoss.ts) and Trainer (src/trainer.ts) over the C ABI."""

from __future__ import annotations

import ctypes
import math
from ctypes import c_double, c_void_p
from dataclasses import dataclass, field, fields, replace

import numpy as np

from . import _lib
from .gaussians import FLOATS_PER_GAUSSIAN, SH_REST_FLOATS
from .gpu import Buffer, Device, Texture, borrowed
from .renderer import CameraData, GaussianRenderer

SH_C0 = 0.28209479177387814
MOMENT_SLOTS = FLOATS_PER_GAUSSIAN + SH_REST_FLOATS


class TrainingLoss:
    """0.8 x L1 + 0.2 x (1 - SSIM) between a render and a photo, and its gradient."""

    def __init__(self, device: Device, width: int, height: int):
        self.device = device
        self.width = width
        self.height = height
        handle = c_void_p()
        _lib.call("dg_training_loss_create", device.handle, width, height, ctypes.byref(handle))
        self.handle = handle
        self.pixelGrads = borrowed(device, _lib.fn("dg_training_loss_pixel_grads")(handle))
        self.pixelLoss = borrowed(device, _lib.fn("dg_training_loss_pixel_loss")(handle))

    def encode(self, encoder, rendered: Buffer, target) -> None:
        t = target.buffer if isinstance(target, Texture) else target
        _lib.call("dg_training_loss_encode", self.handle, rendered.handle, t.handle)

    def read(self) -> float:
        out = c_double()
        _lib.call("dg_training_loss_read", self.handle, ctypes.byref(out))
        return out.value

    def destroy(self) -> None:
        if self.handle:
            _lib.call("dg_training_loss_destroy", self.handle)
            self.handle = None


@dataclass
class TrainingSettings:
    """src/trainer.ts:37-63; the defaults are DEFAULT_SETTINGS (src/trainer.ts:65-82)."""

    extent: float = 1.0
    positionLrSteps: float = 30_000
    positionLr: tuple = (0.00016, 0.0000016)
    opacityLr: float = 0.025
    scaleLr: float = 0.005
    rotationLr: float = 0.001
    colorLr: float = 0.0025
    shLr: float = 0.0025 / 20
    shDegreeInterval: int = 1000
    densifyFrom: int = 500
    densifyUntil: int = 15_000
    densifyInterval: int = 100
    densifyGradThreshold: float = 0.0002
    percentDense: float = 0.01
    minOpacity: float = 0.005
    opacityResetInterval: int = 3000
    background: tuple = (0.0, 0.0, 0.0)

    def to_c(self) -> _lib.TrainingSettingsC:
        s = _lib.TrainingSettingsC()
        s.extent = self.extent
        s.position_lr_steps = self.positionLrSteps
        s.position_lr[:] = list(self.positionLr)
        s.opacity_lr = self.opacityLr
        s.scale_lr = self.scaleLr
        s.rotation_lr = self.rotationLr
        s.color_lr = self.colorLr
        s.sh_lr = self.shLr
        s.sh_degree_interval = self.shDegreeInterval
        s.densify_from = self.densifyFrom
        s.densify_until = self.densifyUntil
        s.densify_interval = self.densifyInterval
        s.densify_grad_threshold = self.densifyGradThreshold
        s.percent_dense = self.percentDense
        s.min_opacity = self.minOpacity
        s.opacity_reset_interval = self.opacityResetInterval
        s.background[:] = list(self.background)
        return s


DEFAULT_SETTINGS = TrainingSettings()


@dataclass
class TrainingView:
    name: str
    camera: CameraData
    image: Texture


@dataclass
class RawGaussians:
    params: np.ndarray
    sh: np.ndarray


@dataclass
class Densification:
    step: int
    before: int
    after: int
    kept: int
    cloned: int
    split: int
    removed: int


def activate(params) -> np.ndarray:
    """Raw parameters to the renderer's activated layout (src/trainer.ts:449-461), on the host."""
    p = np.asarray(params, np.float64).reshape(-1, FLOATS_PER_GAUSSIAN)
    out = np.zeros_like(p)
    out[:, 0:3] = p[:, 0:3]
    out[:, 4:7] = np.exp(p[:, 4:7])
    out[:, 12:15] = 0.5 + SH_C0 * p[:, 12:15]
    out[:, 3] = 1 / (1 + np.exp(-p[:, 3]))
    out[:, 8:12] = p[:, 8:12]
    return out.astype(np.float32).reshape(-1)


def moments_to_reference(planes, count: int) -> np.ndarray:
    """The trainer's moment buffer (two planes: count x 16 parameter slots, then
    count x 45 SH slots, each an (m, v) pair) in the reference's layout: 61 slots
    per Gaussian, parameters first (src/trainer.ts:17), as count * 122 floats."""
    p = np.asarray(planes, np.float32).reshape(-1)[: count * MOMENT_SLOTS * 2]
    params = p[: count * FLOATS_PER_GAUSSIAN * 2].reshape(count, FLOATS_PER_GAUSSIAN * 2)
    sh = p[count * FLOATS_PER_GAUSSIAN * 2:].reshape(count, SH_REST_FLOATS * 2)
    return np.ascontiguousarray(np.concatenate([params, sh], axis=1)).reshape(-1)


def moments_from_reference(reference, count: int) -> np.ndarray:
    """The inverse of moments_to_reference."""
    r = np.asarray(reference, np.float32).reshape(count, MOMENT_SLOTS * 2)
    return np.concatenate([r[:, : FLOATS_PER_GAUSSIAN * 2].reshape(-1), r[:, FLOATS_PER_GAUSSIAN * 2:].reshape(-1)])


def _views_c(views) -> ctypes.Array:
    arr = (_lib.TrainingViewC * len(views))()
    for k, v in enumerate(views):
        arr[k].camera = v.camera.to_c()
        image = v.image.buffer if isinstance(v.image, Texture) else v.image
        arr[k].image = image.handle.value if isinstance(image.handle, c_void_p) else image.handle
    return arr


MLP_FEATURES = 12
MLP_PARAMS = 5122


class DensifyMLP:
    """The learned densification proposal's model: MLP 12 -> 64 -> 64 -> 2, GELU,
    BF16 weights, FP32 accumulation, trained and run by hand-written tensor-core
    kernels. No reference counterpart."""

    def __init__(self, device: Device, seed: int = 0):
        self.device = device
        handle = c_void_p()
        _lib.call("dg_densify_mlp_create", device.handle, seed, ctypes.byref(handle))
        self.handle = handle

    def train(self, features: np.ndarray, labels: np.ndarray, epochs: int = 5, batch: int = 1024,
              lr: float = 1e-3, weightDecay: float = 0.01, seed: int = 0, balanceClasses: bool = False) -> list[float]:
        """AdamW over shuffled minibatches (balanceClasses: both labels weigh the
        same in the loss); returns each epoch's mean cross-entropy."""
        f = np.ascontiguousarray(features, np.float32).reshape(-1, MLP_FEATURES)
        y = np.ascontiguousarray(labels, np.uint8).reshape(-1)
        assert f.shape[0] == y.size
        losses = (c_double * epochs)()
        _lib.call("dg_densify_mlp_train", self.handle, f.ctypes.data, y.ctypes.data, y.size, epochs, batch, lr,
                  weightDecay, int(balanceClasses), seed, losses)
        return list(losses)

    def gradient(self, features: np.ndarray, labels: np.ndarray) -> np.ndarray:
        """The gradient of the mean cross-entropy over these samples at the current
        weights (MLP_PARAMS floats, the layout of weights()); nothing is updated."""
        f = np.ascontiguousarray(features, np.float32).reshape(-1, MLP_FEATURES)
        y = np.ascontiguousarray(labels, np.uint8).reshape(-1)
        assert f.shape[0] == y.size
        out = np.zeros(MLP_PARAMS, np.float32)
        _lib.call("dg_densify_mlp_gradient", self.handle, f.ctypes.data, y.ctypes.data, y.size, out.ctypes.data)
        return out

    def predict(self, features: Buffer, count: int, survive: Buffer) -> None:
        """survive[i] = P(candidate i's children survive), both device buffers."""
        _lib.call("dg_densify_mlp_predict", self.handle, features.handle, count, survive.handle)

    def predictHost(self, features: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(features, np.float32).reshape(-1, MLP_FEATURES)
        fb = self.device.upload(f)
        out = self.device.createBuffer(max(4, f.shape[0] * 4))
        self.predict(fb, f.shape[0], out)
        p = out.read(np.float32)[: f.shape[0]].copy()
        fb.destroy()
        out.destroy()
        return p

    def weights(self) -> np.ndarray:
        """MLP_PARAMS FP32 weights (W1 [12,64], b1, W2 [64,64], b2, W3 [64,2], b3)
        followed by the 24 normalization values (mean, 1/deviation)."""
        out = np.zeros(MLP_PARAMS + 2 * MLP_FEATURES, np.float32)
        _lib.call("dg_densify_mlp_get_weights", self.handle, out.ctypes.data)
        return out

    def setWeights(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, np.float32).reshape(-1)
        assert w.size == MLP_PARAMS + 2 * MLP_FEATURES
        _lib.call("dg_densify_mlp_set_weights", self.handle, w.ctypes.data)

    def destroy(self) -> None:
        if self.handle:
            _lib.call("dg_densify_mlp_destroy", self.handle)
            self.handle = None


class Trainer:
    """Trains Gaussians to match a set of photos, following the reference's loop."""

    def __init__(self, device: Device, raw: RawGaussians | None, views, settings: TrainingSettings,
                 _resume_from: str | None = None):
        self.device = device
        self.views = list(views)
        self.settings = settings
        self._views_c = _views_c(self.views)
        cs = settings.to_c()
        handle = c_void_p()
        if _resume_from is not None:
            _lib.call("dg_trainer_resume", device.handle, str(_resume_from).encode(), self._views_c, len(self.views),
                      ctypes.byref(cs), ctypes.byref(handle))
        else:
            params = np.ascontiguousarray(raw.params, np.float32).reshape(-1)
            sh = np.ascontiguousarray(raw.sh, np.float32).reshape(-1)
            count = params.size // FLOATS_PER_GAUSSIAN
            if sh.size != count * SH_REST_FLOATS:
                raise ValueError(f"Expected {count * SH_REST_FLOATS} spherical-harmonic floats, got {sh.size}.")
            _lib.call("dg_trainer_create", device.handle, params.ctypes.data, sh.ctypes.data, count, self._views_c,
                      len(self.views), ctypes.byref(cs), ctypes.byref(handle))
        self.handle = handle
        self.renderer = GaussianRenderer(device, _handle=_lib.fn("dg_trainer_renderer")(handle))

    @property
    def iteration(self) -> int:
        return int(_lib.fn("dg_trainer_iteration")(self.handle))

    @iteration.setter
    def iteration(self, value: int) -> None:
        _lib.call("dg_trainer_set_iteration", self.handle, value)

    @property
    def shDegree(self) -> int:
        return int(_lib.fn("dg_trainer_sh_degree")(self.handle))

    @property
    def adamSteps(self) -> int:
        """The steps that ran Adam (private in the reference; for checks)."""
        return int(_lib.fn("dg_trainer_adam_steps")(self.handle))

    @property
    def count(self) -> int:
        return int(_lib.fn("dg_trainer_count")(self.handle))

    @property
    def buffers(self) -> dict:
        b = lambda name: borrowed(self.device, _lib.fn(name)(self.handle))  # noqa: E731
        return {"params": b("dg_trainer_params"), "moments": b("dg_trainer_moments"), "stats": b("dg_trainer_stats")}

    def readMoments(self) -> np.ndarray:
        """Adam's moments in the reference's layout (count x 61 (m, v) pairs)."""
        return moments_to_reference(self.buffers["moments"].read(np.float32), self.count)

    def writeMoments(self, reference) -> None:
        """Sets Adam's moments from the reference's layout (count x 61 (m, v) pairs)."""
        self.buffers["moments"].write(moments_from_reference(reference, self.count))

    @property
    def densifications(self) -> list[Densification]:
        out = []
        for k in range(int(_lib.fn("dg_trainer_densification_count")(self.handle))):
            d = _lib.DensificationC()
            _lib.call("dg_trainer_densification", self.handle, k, ctypes.byref(d))
            out.append(Densification(d.step, d.before, d.after, d.kept, d.cloned, d.split, d.removed))
        return out

    def step(self) -> None:
        _lib.call("dg_trainer_step", self.handle)

    def optimize(self) -> None:
        _lib.call("dg_trainer_optimize", self.handle)

    def maintain(self) -> None:
        _lib.call("dg_trainer_maintain", self.handle)

    def densify(self, pruneLarge: bool) -> None:
        _lib.call("dg_trainer_densify", self.handle, int(pruneLarge))

    def resetOpacity(self) -> None:
        _lib.call("dg_trainer_reset_opacity", self.handle)

    @classmethod
    def resume(cls, device: Device, path, views, settings: TrainingSettings) -> "Trainer":
        """A trainer in the state saveCheckpoint recorded (no reference counterpart),
        over the same views in the same order."""
        return cls(device, None, views, settings, _resume_from=str(path))

    def saveCheckpoint(self, path) -> None:
        """Writes a .ply that 3DGS viewers open as the current scene and that
        Trainer.resume continues training from (no reference counterpart)."""
        _lib.call("dg_trainer_save_checkpoint", self.handle, str(path).encode())

    def exportRaw(self) -> RawGaussians:
        n = self.count
        params = np.empty(n * FLOATS_PER_GAUSSIAN, np.float32)
        sh = np.empty(n * SH_REST_FLOATS, np.float32)
        _lib.call("dg_trainer_export_raw", self.handle, params.ctypes.data, sh.ctypes.data)
        return RawGaussians(params, sh)

    def lastLoss(self) -> float:
        out = c_double()
        _lib.call("dg_trainer_last_loss", self.handle, ctypes.byref(out))
        return out.value

    def lossValue(self) -> float:
        """The last step's loss, summed on the GPU (8 bytes read back)."""
        out = c_double()
        _lib.call("dg_trainer_loss_value", self.handle, ctypes.byref(out))
        return out.value

    def setHostPhotos(self, photos) -> None:
        """Read each step's photo from pinned host memory (one PinnedArray per view,
        kept alive and unchanged by the caller), uploading the next step's while the
        current one runs; None goes back to the views' images."""
        if photos is None:
            self._host_photos = None
            _lib.call("dg_trainer_set_host_photos", self.handle, None, 0)
            return
        arr = (ctypes.c_void_p * len(photos))(*[p.pointer for p in photos])
        self._host_photos = (list(photos), arr)
        _lib.call("dg_trainer_set_host_photos", self.handle, arr, len(photos))

    def requestLoss(self) -> None:
        """Start reading the last step's loss without waiting for it (see takeLoss)."""
        _lib.call("dg_trainer_request_loss", self.handle)

    def takeLoss(self, wait: bool = True) -> float | None:
        """The oldest requested loss; None if wait is False and it has not arrived."""
        out, ready = c_double(), ctypes.c_int32()
        _lib.call("dg_trainer_take_loss", self.handle, int(wait), ctypes.byref(out), ctypes.byref(ready))
        return out.value if ready.value else None

    def nextView(self) -> int:
        """Index of the view the next optimize() renders."""
        out = ctypes.c_uint32()
        _lib.call("dg_trainer_next_view", self.handle, ctypes.byref(out))
        return out.value

    def evaluate(self, views, withSsim: bool = True) -> dict:
        arr = _views_c(views)
        psnr, ssim = c_double(), c_double()
        _lib.call("dg_trainer_evaluate", self.handle, arr, len(views), int(withSsim), ctypes.byref(psnr),
                  ctypes.byref(ssim))
        return {"psnr": psnr.value, "ssim": ssim.value}

    def setGraph(self, enabled: bool) -> None:
        """Replay each optimize() step as one captured CUDA graph."""
        _lib.call("dg_trainer_set_graph", self.handle, int(enabled))

    def setKeepGradients(self, enabled: bool) -> None:
        """Also store each step's Gaussian gradients in renderer.gradients (Adam
        consumes them in registers otherwise); the parameters are the same."""
        _lib.call("dg_trainer_set_keep_gradients", self.handle, int(enabled))

    # Learned densification (no reference counterpart; the reference densifies by
    # its gradient threshold alone, which stays the fallback).
    def setDensifyLog(self, enabled: bool, horizon: int = 1000) -> None:
        """Log every clone/split candidate's features; each is labelled `horizon`
        steps later by whether any of its new children is still alive."""
        _lib.call("dg_trainer_set_densify_log", self.handle, int(enabled), horizon)

    def takeDensifySamples(self) -> tuple[np.ndarray, np.ndarray, int]:
        """The labelled samples so far (moved out of the log): features [n, 12],
        labels [n] (0/1), and how many still wait for their horizon."""
        n, pending = ctypes.c_uint32(), ctypes.c_uint32()
        _lib.call("dg_trainer_take_densify_samples", self.handle, None, None, 0, ctypes.byref(n),
                  ctypes.byref(pending))
        features = np.zeros((n.value, MLP_FEATURES), np.float32)
        labels = np.zeros(n.value, np.uint8)
        if n.value:
            _lib.call("dg_trainer_take_densify_samples", self.handle, features.ctypes.data, labels.ctypes.data,
                      n.value, ctypes.byref(n), ctypes.byref(pending))
        return features[: n.value], labels[: n.value], pending.value

    def setDensifyMLP(self, mlp: "DensifyMLP | None", minConfidence: float = 0.6) -> None:
        """Let the model decide the plain rule's clone/split candidates where it is
        confident (max(p, 1 - p) >= minConfidence); None restores the plain rule."""
        _lib.call("dg_trainer_set_densify_mlp", self.handle, mlp.handle if mlp is not None else None, minConfidence)
        self._mlp = mlp

    @property
    def densifyMLPStats(self) -> dict:
        scored, confident, vetoed = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _lib.call("dg_trainer_densify_mlp_stats", self.handle, ctypes.byref(scored), ctypes.byref(confident),
                  ctypes.byref(vetoed))
        return {"scored": scored.value, "confident": confident.value, "vetoed": vetoed.value}

    def destroy(self) -> None:
        if self.handle:
            _lib.call("dg_trainer_destroy", self.handle)
            self.handle = None

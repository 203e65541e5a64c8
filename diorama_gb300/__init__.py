"""diorama_gb300: a GB300-native 3D Gaussian Splatting renderer and trainer.

The classes mirror the reference's TypeScript surface for the training path
(GaussianRenderer, TileRasterizer, RadixSort, PrefixSum, TrainingLoss, Trainer)
on top of the C ABI in include/diorama_gb300.h, whose kernels are hand-written
CUDA for sm_103a. There is no CPU fallback: if libdiorama_gb300.so cannot be
loaded or no CUDA device is present, creating a Device raises.
"""

from ._lib import DioramaError
from .gaussians import (FLOATS_PER_GAUSSIAN, FLOATS_PER_SPLAT, SH_REST_FLOATS, Gaussian, Splat2D, packGaussians,
                        packSplats, unpackSplats)
from .dataset import (Dataset, Reconstruction, TrainingCamera, cameraView, initialGaussians, loadDataset, loadViews,
                      meanNeighborDistance2, meanNeighborDistance2Buffers, parseColmap, splitDataset,
                      trainingCameraData, verticalFov)
from .gpu import Buffer, Device, Texture, initGpu, readBuffer
from .ply import GaussianScene, parseGaussianPly, writeGaussianPly
from .primitives import PrefixSum, RadixSort
from .renderer import CameraData, GaussianRenderer, SphericalHarmonics, TileRasterizer
from .training import (DEFAULT_SETTINGS, MOMENT_SLOTS, Densification, DensifyMLP, RawGaussians, Trainer,
                       TrainingLoss, TrainingSettings, TrainingView, activate)

__all__ = [
    "DioramaError", "FLOATS_PER_GAUSSIAN", "FLOATS_PER_SPLAT", "SH_REST_FLOATS", "MOMENT_SLOTS", "Gaussian",
    "Splat2D", "packGaussians", "packSplats", "unpackSplats", "Buffer", "Device", "Texture", "initGpu", "readBuffer",
    "PrefixSum", "RadixSort", "CameraData", "GaussianRenderer", "SphericalHarmonics", "TileRasterizer",
    "DEFAULT_SETTINGS", "Densification", "DensifyMLP", "RawGaussians", "Trainer", "TrainingLoss", "TrainingSettings",
    "TrainingView", "activate", "GaussianScene", "parseGaussianPly", "writeGaussianPly", "initialGaussians",
    "meanNeighborDistance2", "meanNeighborDistance2Buffers", "Dataset", "Reconstruction", "TrainingCamera",
    "cameraView", "loadDataset", "loadViews", "parseColmap", "splitDataset", "trainingCameraData", "verticalFov",
]

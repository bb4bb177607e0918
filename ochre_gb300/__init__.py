"""GB300-native (sm_103a) implementation of ochre's path-rasterization hot path.

Mirrors glowcoil/ochre 0.2.0's public API (``Rasterizer::fill`` /
``finish(&mut impl TileBuilder)``) over a C ABI (include/ochre_gpu.h) backed by
hand-written CUDA kernels.  There is no CPU fallback: entry points raise if the
CUDA library or a device is missing.
"""
from ._lib import OchreError
from .batch import (CLOSE, CONIC, CUBIC, FILL_RAW, FILL_STROKE, IDENTITY, LINE, MOVE, QUADRATIC, Batch,
                    BatchBuilder, concat, subset)
from .rasterizer import (TILE_SIZE, DeviceBatch, DiffGraph, GpuContext, Graph, Mat2x2, PathCmd, Rasterizer, TileBuilder,
                         Transform, Vec2, default_context, encode_path, validate_batch)

__all__ = [
    "MOVE", "LINE", "QUADRATIC", "CUBIC", "CONIC", "CLOSE", "FILL_RAW", "FILL_STROKE", "IDENTITY", "Batch",
    "BatchBuilder", "OchreError",
    "concat", "subset", "TILE_SIZE", "DeviceBatch", "DiffGraph", "GpuContext", "Graph", "Mat2x2", "PathCmd", "Rasterizer",
    "TileBuilder", "Transform", "Vec2", "default_context", "encode_path", "validate_batch",
]

"""ctypes binding of libochre_gpu.so (include/ochre_gpu.h).

The library is built in-tree (``ochre_gb300/_build``) by ``ochre_gb300.build``.
There is no CPU fallback: if the library or a CUDA device is missing, every
entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

OK, E_INVALID, E_CAPACITY, E_CUDA, E_TIMEOUT, E_NOMEM, E_LIMIT = range(7)
CTX_WANT_COV = 1
CTX_PROFILE = 2
CTX_CHAIN_ONLY = 4

EXPORTS = [
    "ochre_gpu_create", "ochre_gpu_destroy", "ochre_gpu_set_flags", "ochre_gpu_rasterize_device",
    "ochre_gpu_rasterize", "ochre_gpu_last_stats", "ochre_gpu_last_timings", "ochre_gpu_status_string",
    "ochre_rasterizer_new", "ochre_rasterizer_move_to", "ochre_rasterizer_line_to",
    "ochre_rasterizer_command", "ochre_rasterizer_fill", "ochre_rasterizer_stroke", "ochre_rasterizer_finish",
    "ochre_rasterizer_free",
    "ochre_gpu_rasterize_noalloc", "ochre_gpu_set_tunable", "ochre_gpu_get_tunable",
    "ochre_gpu_render_coverage", "ochre_gpu_l2_loss", "ochre_gpu_fill_backward", "ochre_gpu_composite",
    "ochre_graph_create", "ochre_graph_launch", "ochre_graph_last_stats", "ochre_graph_info", "ochre_graph_destroy",
    "ochre_graph_create_diff",
    "ochre_validate_batch",
]


class OchreError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status) if _lib is not None else f"status {status}"
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


class Batch(ctypes.Structure):
    _fields_ = [
        ("verbs", ctypes.c_void_p), ("n_cmds", ctypes.c_uint64),
        ("pts", ctypes.c_void_p), ("n_floats", ctypes.c_uint64),
        ("fill_cmd_off", ctypes.c_void_p), ("fill_xf", ctypes.c_void_p),
        ("fill_flags", ctypes.c_void_p), ("n_fills", ctypes.c_uint32),
        ("raster_fill_off", ctypes.c_void_p), ("n_rasters", ctypes.c_uint32),
        ("fill_width", ctypes.c_void_p),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("n_tiles", ctypes.c_uint32), ("n_spans", ctypes.c_uint32),
        ("tile_xy", ctypes.c_void_p), ("tile_alpha", ctypes.c_void_p), ("tile_cov", ctypes.c_void_p),
        ("span_xy", ctypes.c_void_p), ("span_width", ctypes.c_void_p), ("span_tile", ctypes.c_void_p),
        ("raster_tile_off", ctypes.c_void_p), ("raster_span_off", ctypes.c_void_p),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("n_lines", ctypes.c_uint64), ("n_entries", ctypes.c_uint64), ("n_tiles", ctypes.c_uint64),
        ("n_spans", ctypes.c_uint64), ("key_bits", ctypes.c_uint32), ("sort_passes", ctypes.c_uint32),
        ("n_launches", ctypes.c_uint32), ("pad", ctypes.c_uint32), ("n_bins", ctypes.c_uint64),
        ("fused", ctypes.c_uint32), ("n_incs", ctypes.c_uint32),
    ]


class OutputBuffers(ctypes.Structure):
    """ochre_output_buffers: caller-provided device outputs of
    ochre_gpu_rasterize_noalloc."""
    _fields_ = [
        ("tile_xy", ctypes.c_void_p), ("tile_alpha", ctypes.c_void_p), ("tile_capacity", ctypes.c_uint32),
        ("span_xy", ctypes.c_void_p), ("span_width", ctypes.c_void_p), ("span_tile", ctypes.c_void_p),
        ("span_capacity", ctypes.c_uint32), ("raster_tile_off", ctypes.c_void_p),
        ("raster_span_off", ctypes.c_void_p), ("n_tiles", ctypes.c_uint32), ("n_spans", ctypes.c_uint32),
    ]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("ms", ctypes.c_float)]


TILE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int16, ctypes.c_int16, ctypes.POINTER(ctypes.c_uint8))
SPAN_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int16, ctypes.c_int16, ctypes.c_uint16)

_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) libochre_gpu.so and declare its ABI."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build() if build_if_missing else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(f"libochre_gpu.so is missing at {path}; run ochre_gb300.build.build()")
        L = ctypes.CDLL(path)
        vp, u32, u8 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint8
        L.ochre_gpu_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, u32]
        L.ochre_gpu_destroy.argtypes = [vp]
        L.ochre_gpu_destroy.restype = None
        L.ochre_gpu_set_flags.argtypes = [vp, u32]
        L.ochre_gpu_rasterize_device.argtypes = [vp, ctypes.POINTER(Batch), ctypes.POINTER(Result), vp]
        L.ochre_gpu_rasterize.argtypes = [vp, ctypes.POINTER(Batch), ctypes.POINTER(Result)]
        L.ochre_validate_batch.argtypes = [ctypes.POINTER(Batch)]
        L.ochre_gpu_last_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.ochre_gpu_last_timings.argtypes = [vp, ctypes.POINTER(KernelTime), u32, ctypes.POINTER(u32)]
        L.ochre_gpu_status_string.argtypes = [ctypes.c_int]
        L.ochre_gpu_status_string.restype = ctypes.c_char_p
        L.ochre_rasterizer_new.argtypes = [vp, ctypes.POINTER(vp)]
        L.ochre_rasterizer_move_to.argtypes = [vp, ctypes.c_float, ctypes.c_float]
        L.ochre_rasterizer_line_to.argtypes = [vp, ctypes.c_float, ctypes.c_float]
        L.ochre_rasterizer_command.argtypes = [vp, u8, ctypes.POINTER(ctypes.c_float)]
        L.ochre_rasterizer_fill.argtypes = [vp, ctypes.POINTER(u8), ctypes.c_size_t, ctypes.POINTER(ctypes.c_float),
                                            ctypes.c_size_t, ctypes.POINTER(ctypes.c_float)]
        L.ochre_rasterizer_stroke.argtypes = [vp, ctypes.POINTER(u8), ctypes.c_size_t, ctypes.POINTER(ctypes.c_float),
                                              ctypes.c_size_t, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]
        L.ochre_rasterizer_finish.argtypes = [vp, TILE_FN, SPAN_FN, vp]
        L.ochre_rasterizer_free.argtypes = [vp]
        L.ochre_rasterizer_free.restype = None
        L.ochre_gpu_rasterize_noalloc.argtypes = [ctypes.POINTER(Batch), ctypes.POINTER(OutputBuffers), vp]
        L.ochre_gpu_set_tunable.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
        L.ochre_gpu_render_coverage.argtypes = [vp, ctypes.POINTER(Batch), u32, u32, vp, vp]
        L.ochre_gpu_l2_loss.argtypes = [vp, vp, vp, ctypes.c_uint64, vp, vp, vp]
        L.ochre_gpu_fill_backward.argtypes = [vp, ctypes.POINTER(Batch), u32, u32, vp, vp, vp, vp]
        L.ochre_gpu_get_tunable.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        L.ochre_gpu_composite.argtypes = [vp, ctypes.POINTER(Result), u32, vp, u32, u32, vp, vp]
        L.ochre_graph_create.argtypes = [vp, ctypes.POINTER(Batch), ctypes.c_float, ctypes.POINTER(vp)]
        L.ochre_graph_create_diff.argtypes = [vp, ctypes.POINTER(Batch), u32, u32, vp, vp, vp, vp, vp, vp,
                                              ctypes.c_float, ctypes.POINTER(vp)]
        L.ochre_graph_launch.argtypes = [vp, ctypes.POINTER(Result), vp]
        L.ochre_graph_last_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.ochre_graph_info.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(u32)]
        L.ochre_graph_destroy.argtypes = [vp]
        L.ochre_graph_destroy.restype = None
        _lib = L
        return L


_cudart = None


def memcpy_d2h(dst: int, src: int, nbytes: int) -> None:
    """Synchronous device-to-host copy through the CUDA runtime the library
    itself links (test and inspection helper)."""
    global _cudart
    if _cudart is None:
        load()
        for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
            try:
                _cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if _cudart is None:
            raise RuntimeError("libcudart not found")
        _cudart.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        _cudart.cudaDeviceSynchronize.argtypes = []
    _cudart.cudaDeviceSynchronize()
    err = _cudart.cudaMemcpy(dst, src, nbytes, 2)  # cudaMemcpyDeviceToHost
    if err != 0:
        raise RuntimeError(f"cudaMemcpy failed with error {err}")


def status_string(status: int) -> str:
    L = load()
    return L.ochre_gpu_status_string(int(status)).decode()


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise OchreError(status, what)

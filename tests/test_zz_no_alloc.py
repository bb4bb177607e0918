"""ochre_gpu_rasterize_noalloc: rasterization for callers that may not
allocate GPU memory while running (for example hosts that reserve all device
memory at start-up, because cudaMalloc/cudaFree synchronise the device and
can stall a frame).  Its intermediates live in one static device array of
OCHRE_NOALLOC_SCRATCH_BYTES and its results go to caller buffers.

The test calls it through the C ABI twice in a row on different inputs and
checks each result against ochre_gpu_rasterize_device with the parity bar of
the other GPU tests (structure bit-exact, alpha within 1 LSB).  This file is
named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from compare import compare
from golden.make_golden import load
from ochre_gb300 import DeviceBatch, _lib

pytestmark = pytest.mark.gpu


def _run_noalloc(db, n_rasters, tile_capacity, span_capacity=None):
    import torch
    span_capacity = tile_capacity if span_capacity is None else span_capacity
    dev = torch.device("cuda", 0)
    bufs = {
        "tile_xy": torch.empty(2 * max(1, tile_capacity), dtype=torch.int16, device=dev),
        "tile_alpha": torch.empty(64 * max(1, tile_capacity), dtype=torch.uint8, device=dev),
        "span_xy": torch.empty(2 * max(1, span_capacity), dtype=torch.int16, device=dev),
        "span_w": torch.empty(max(1, span_capacity), dtype=torch.int16, device=dev),
        "span_tile": torch.empty(max(1, span_capacity), dtype=torch.int32, device=dev),
        "rto": torch.empty(n_rasters + 1, dtype=torch.int32, device=dev),
        "rso": torch.empty(n_rasters + 1, dtype=torch.int32, device=dev),
    }
    o = _lib.OutputBuffers()
    o.tile_xy, o.tile_alpha, o.tile_capacity = bufs["tile_xy"].data_ptr(), bufs["tile_alpha"].data_ptr(), tile_capacity
    o.span_xy, o.span_width, o.span_tile = bufs["span_xy"].data_ptr(), bufs["span_w"].data_ptr(), bufs["span_tile"].data_ptr()
    o.span_capacity = span_capacity
    o.raster_tile_off, o.raster_span_off = bufs["rto"].data_ptr(), bufs["rso"].data_ptr()
    torch.cuda.synchronize()
    st = _lib.load().ochre_gpu_rasterize_noalloc(ctypes.byref(db.c), ctypes.byref(o), None)
    torch.cuda.synchronize()
    if st != _lib.OK:
        return st, None
    T, N = o.n_tiles, o.n_spans
    got = {
        "tile_xy": bufs["tile_xy"][: 2 * T].cpu().numpy().reshape(T, 2),
        "tile_alpha": bufs["tile_alpha"][: 64 * T].cpu().numpy().reshape(T, 64),
        "span_xy": bufs["span_xy"][: 2 * N].cpu().numpy().reshape(N, 2),
        "span_w": bufs["span_w"][:N].cpu().numpy().view(np.uint16),
        "span_tile": bufs["span_tile"][:N].cpu().numpy().view(np.uint32),
        "raster_tile_off": bufs["rto"].cpu().numpy().view(np.uint32).astype(np.uint64),
        "raster_span_off": bufs["rso"].cpu().numpy().view(np.uint32).astype(np.uint64),
    }
    return st, got


def test_noalloc_matches_rasterize_device_twice(gpu_ctx):
    for name in ("glyph_run_48", "edge_cases", "cubic_boxes_2"):
        b, _ = load(name)
        db = DeviceBatch(b)
        want = gpu_ctx.device_result_to_numpy(gpu_ctx.rasterize_device(db), b.n_rasters)
        cap = len(want["tile_xy"]) + 16
        for call in range(2):  # two calls in a row share the static scratch
            st, got = _run_noalloc(db, b.n_rasters, cap)
            assert st == _lib.OK, (name, call, _lib.status_string(st))
            compare(got, want, b.n_rasters)


def test_noalloc_rejects_too_small_outputs(gpu_ctx):
    b, exp = load("glyph_run_48")
    db = DeviceBatch(b)
    st, _ = _run_noalloc(db, b.n_rasters, tile_capacity=4)
    assert st == _lib.E_CAPACITY
    # and works again right after
    st, got = _run_noalloc(db, b.n_rasters, len(exp["tile_xy"]))
    assert st == _lib.OK
    compare(got, exp, b.n_rasters)

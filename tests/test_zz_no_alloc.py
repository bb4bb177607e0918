"""ochre_gpu_rasterize_noalloc: rasterization for callers that may not
allocate GPU memory while running (for example hosts that reserve all device
memory at start-up, because cudaMalloc/cudaFree synchronise the device and
can stall a frame).  Its intermediates live in one static device array of
OCHRE_NOALLOC_SCRATCH_BYTES and its results go to caller buffers.

The tests call it through the C ABI, twice in a row on each input, and check
every result against ochre_gpu_rasterize_device and against the oracle's
golden fixture with the parity bar of the other GPU tests (structure
bit-exact, alpha within 1 LSB).  They also check the two ways it can run out
of room: a caller buffer that is too small and a batch whose intermediates do
not fit the array; each returns OCHRE_E_CAPACITY and the next call, on
another stream, is correct.  This file is named so that pytest collects it
last.
"""
import ctypes

import numpy as np
import pytest

from compare import compare
from golden.make_golden import load
from ochre_gb300 import DeviceBatch, _lib, workloads

pytestmark = pytest.mark.gpu


def _run_noalloc(db, n_rasters, tile_capacity, span_capacity=None, stream=None):
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
    handle = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
    st = _lib.load().ochre_gpu_rasterize_noalloc(ctypes.byref(db.c), ctypes.byref(o), handle)
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


def test_noalloc_matches_rasterize_device_and_oracle_twice(gpu_ctx):
    for name in ("glyph_run_48", "edge_cases", "cubic_boxes_2"):
        b, exp = load(name)
        db = DeviceBatch(b)
        want = gpu_ctx.device_result_to_numpy(gpu_ctx.rasterize_device(db), b.n_rasters)
        compare(want, exp, b.n_rasters)
        cap = len(want["tile_xy"]) + 16
        for call in range(2):  # two calls in a row share the static scratch
            st, got = _run_noalloc(db, b.n_rasters, cap)
            assert st == _lib.OK, (name, call, _lib.status_string(st))
            compare(got, want, b.n_rasters)
            compare(got, exp, b.n_rasters)


def test_noalloc_rejects_too_small_outputs(gpu_ctx):
    b, exp = load("glyph_run_48")
    db = DeviceBatch(b)
    st, _ = _run_noalloc(db, b.n_rasters, tile_capacity=4)
    assert st == _lib.E_CAPACITY
    # and works again right after
    st, got = _run_noalloc(db, b.n_rasters, len(exp["tile_xy"]))
    assert st == _lib.OK
    compare(got, exp, b.n_rasters)


def test_noalloc_span_capacity_below_tiles_on_the_chain(gpu_ctx):
    # cubic boxes do not fit the fused kernel: the general chain runs, and its
    # span compaction needs room for one span per tile
    import torch
    b, exp = load("cubic_boxes_2")
    db = DeviceBatch(b)
    n_tiles = len(exp["tile_xy"])
    st, _ = _run_noalloc(db, b.n_rasters, n_tiles, span_capacity=max(1, n_tiles // 4))
    assert st == _lib.E_CAPACITY, _lib.status_string(st)
    side = torch.cuda.Stream()
    st, got = _run_noalloc(db, b.n_rasters, n_tiles, stream=side)
    assert st == _lib.OK, _lib.status_string(st)
    compare(got, exp, b.n_rasters)


def test_noalloc_batch_larger_than_the_scratch(gpu_ctx):
    # 400 paths of the uneven mix need far more than the array for their
    # sort entries (tens of millions of bytes): the call fails partway through
    # the chain, after some of its kernels were queued
    import torch
    big = workloads.uneven_mix(n_paths=400, seed=11)
    dbig = DeviceBatch(big)
    want_big = gpu_ctx.device_result_to_numpy(gpu_ctx.rasterize_device(dbig), big.n_rasters)
    st, _ = _run_noalloc(dbig, big.n_rasters, len(want_big["tile_xy"]) + 16)
    assert st == _lib.E_CAPACITY, _lib.status_string(st)
    # the next call, on another stream, is correct
    b, exp = load("cubic_boxes_2")
    db = DeviceBatch(b)
    want = gpu_ctx.device_result_to_numpy(gpu_ctx.rasterize_device(db), b.n_rasters)
    side = torch.cuda.Stream()
    for _ in range(2):
        st, got = _run_noalloc(db, b.n_rasters, len(want["tile_xy"]) + 16, stream=side)
        assert st == _lib.OK, _lib.status_string(st)
        compare(got, want, b.n_rasters)
        compare(got, exp, b.n_rasters)

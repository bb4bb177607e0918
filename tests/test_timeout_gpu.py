"""Bounded device waits that run out (OCHRE_E_TIMEOUT), without a fault.

Every look-back wait of the chain polls a bounded number of times; the first
wait that gives up flags ERR_TIMEOUT and every other wait of the run gives up
as soon as it sees the flag.  The test makes one run's waits impossible to
finish on the host side: the test hook `test_skip_first_raster` starts the
fused kernel's raster tickets at 1, so raster 0 never publishes its output
counts and every successor's output look-back waits on it; `test_spin_log2`
lowers the poll limit to 2^4 for that run.  The call must return
OCHRE_E_TIMEOUT quickly, and the same context must then reproduce the golden
fixture.  Nothing here faults or hangs the GPU: the waits end by their limit.
"""
import ctypes
import time

import pytest

from compare import compare
from golden.make_golden import load
from ochre_gb300 import DeviceBatch, GpuContext, _lib

pytestmark = pytest.mark.gpu


def _set(ctx, name, value):
    _lib.check(_lib.load().ochre_gpu_set_tunable(ctx.handle, name.encode(), int(value)), name)


def test_unfinishable_lookback_times_out_and_context_recovers():
    b, exp = load("glyph_run_48")
    ctx = GpuContext(0)
    try:
        db = DeviceBatch(b)
        first = ctx.device_result_to_numpy(ctx.rasterize_device(db), b.n_rasters)
        compare(first, exp, b.n_rasters)
        assert ctx.stats()["fused"], "the fixture must run on the fused kernel"

        _set(ctx, "test_spin_log2", 4)
        _set(ctx, "test_skip_first_raster", 1)
        r = _lib.Result()
        t0 = time.perf_counter()
        st = _lib.load().ochre_gpu_rasterize_device(ctx.handle, ctypes.byref(db.c), ctypes.byref(r), None)
        dt = time.perf_counter() - t0
        assert st == _lib.E_TIMEOUT, _lib.status_string(st)
        # 47 waiting rasters of at most 16 polls each, and the abort: well
        # under a second (the default limit alone would be about a second)
        assert dt < 0.5, dt

        # the hooks applied to that run only; the context still works
        for _ in range(2):
            got = ctx.device_result_to_numpy(ctx.rasterize_device(db), b.n_rasters)
            compare(got, exp, b.n_rasters)
        got = ctx.rasterize(b)
        compare(got, exp, b.n_rasters)
    finally:
        ctx.close()


def test_test_hooks_are_checked():
    # argument checks only (no launch)
    ctx = GpuContext(0)
    try:
        L = _lib.load()
        assert L.ochre_gpu_set_tunable(ctx.handle, b"test_spin_log2", 41) == _lib.E_INVALID
        assert L.ochre_gpu_set_tunable(ctx.handle, b"test_skip_first_raster", 2) == _lib.E_INVALID
    finally:
        ctx.close()

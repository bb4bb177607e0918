"""Bounded device waits that run out (OCHRE_E_TIMEOUT), without a fault.

Every look-back wait of the chain polls a bounded number of times; the first
wait that gives up flags ERR_TIMEOUT and every other wait of the run gives up
as soon as it sees the flag.  The test makes one run's waits impossible to
finish on the host side: the test hook `test_skip_first_ticket` starts the
tickets of the fused path's command scan at 1, so that scan's first tile
never publishes and every later tile's look-back waits on it;
`test_spin_log2` lowers the poll limit to 2^4 for that run.  The call must
return OCHRE_E_TIMEOUT quickly, and the same context must then reproduce the
oracle's output.  Nothing here faults or hangs the GPU: the waits end by
their limit, and the kernels after them return at once.
"""
import ctypes
import time

import pytest

import oracle
from compare import compare
from ochre_gb300 import DeviceBatch, GpuContext, _lib, workloads

pytestmark = pytest.mark.gpu


def _set(ctx, name, value):
    _lib.check(_lib.load().ochre_gpu_set_tunable(ctx.handle, name.encode(), int(value)), name)


def test_unfinishable_lookback_times_out_and_context_recovers():
    # 5,000 rasters, 140,000 commands: 69 tiles of the command scan
    b = workloads.glyph_run(n_paths=5000, seed=41)
    exp = oracle.run(b, threads=16)
    ctx = GpuContext(0)
    try:
        db = DeviceBatch(b)
        first = ctx.device_result_to_numpy(ctx.rasterize_device(db), b.n_rasters)
        compare(first, exp, b.n_rasters)
        assert ctx.stats()["fused"], "the fixture must run on the fused kernel"

        _set(ctx, "test_spin_log2", 4)
        _set(ctx, "test_skip_first_ticket", 1)
        r = _lib.Result()
        t0 = time.perf_counter()
        st = _lib.load().ochre_gpu_rasterize_device(ctx.handle, ctypes.byref(db.c), ctypes.byref(r), None)
        dt = time.perf_counter() - t0
        assert st == _lib.E_TIMEOUT, _lib.status_string(st)
        # the first waiting tile gives up after 16 polls and the others see
        # the abort within 8: well under a second (the default limit alone
        # would be about a second)
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
        assert L.ochre_gpu_set_tunable(ctx.handle, b"test_skip_first_ticket", 2) == _lib.E_INVALID
    finally:
        ctx.close()

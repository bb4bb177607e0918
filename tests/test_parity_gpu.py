"""GPU parity: the CUDA path (through the C ABI) against the oracle.

Tile/span structure must be bit-exact and alpha within 1 LSB (compare.py).
"""
import numpy as np
import pytest

import oracle
from compare import compare
from golden.make_golden import NAMES, load
from ochre_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", NAMES)
def test_golden_host_path(any_ctx, name):
    b, exp = load(name)
    any_ctx.set_want_cov(True)
    try:
        got = any_ctx.rasterize(b)
    finally:
        any_ctx.set_want_cov(False)
    st = compare(got, exp, b.n_rasters)
    # pre-quantisation coverage vs the oracle's f32 coverage (summation order
    # only): 1e-3 absolute, relative to |S| where |S| > 1 (at the i16 limits a
    # cell's right edge lies 65,536 px from the line and |S| reaches ~2^17)
    assert st["cov_max_rel_vs_oracle_f32"] < 1e-3, st


@pytest.mark.parametrize("name", NAMES)
def test_golden_device_path(any_ctx, name):
    from ochre_gb300 import DeviceBatch
    b, exp = load(name)
    db = DeviceBatch(b)
    r = any_ctx.rasterize_device(db)
    got = any_ctx.device_result_to_numpy(r, b.n_rasters)
    compare(got, exp, b.n_rasters)


@pytest.mark.parametrize("gen,kw", [
    (W.cubic_boxes, dict(n_paths=60)),
    (W.glyph_run, dict(n_paths=3000)),
    (W.uneven_mix, dict(n_paths=150)),
    (W.diff_union, dict()),
    (W.diff_scenes, dict(n_scenes=6)),
])
def test_workload_parity(any_ctx, gen, kw):
    b = gen(**kw)
    ref = oracle.run(b, threads=8)
    got = any_ctx.rasterize(b)
    st = compare(got, ref, b.n_rasters)
    assert st["diff_fraction"] < 0.01, st


def test_line_and_entry_counts_match_oracle(gpu_ctx_chain):
    b = W.cubic_boxes(n_paths=5)
    ref = oracle.run(b, capture_lines=True)
    gpu_ctx_chain.rasterize(b)
    s = gpu_ctx_chain.stats()
    assert s["n_lines"] == len(ref["lines"])
    assert s["n_tiles"] == len(ref["tile_xy"])


def test_readme_through_rasterizer_api():
    from ochre_gb300 import PathCmd, Rasterizer, TileBuilder, Transform, Vec2

    class Collect(TileBuilder):
        def __init__(self):
            self.events = []

        def tile(self, x, y, data):
            self.events.append(("tile", x, y, bytes(data)))

        def span(self, x, y, width):
            self.events.append(("span", x, y, width))

    r = Rasterizer()
    r.fill([
        PathCmd.Move(Vec2(400.0, 300.0)),
        PathCmd.Quadratic(Vec2(500.0, 200.0), Vec2(400.0, 100.0)),
        PathCmd.Cubic(Vec2(350.0, 150.0), Vec2(100.0, 250.0), Vec2(400.0, 300.0)),
        PathCmd.Close(),
    ], Transform.id())
    c = Collect()
    r.finish(c)
    ref = oracle.run(W.readme_path())
    tiles = [e for e in c.events if e[0] == "tile"]
    assert [(e[1], e[2]) for e in tiles] == [tuple(t) for t in ref["tile_xy"].tolist()]
    a = np.array([np.frombuffer(e[3], np.uint8) for e in tiles]).astype(int)
    assert np.abs(a - ref["tile_alpha"].astype(int)).max() <= 1
    # callback order: each span right after the tile it follows
    order, ti = [], -1
    for e in c.events:
        if e[0] == "tile":
            ti += 1
        else:
            order.append((ti, e[1], e[2], e[3]))
    assert order == [(int(t), int(x), int(y), int(w)) for t, (x, y), w in
                     zip(ref["span_tile"], ref["span_xy"].tolist(), ref["span_w"])]


def test_raw_commands_and_multiple_fills():
    from ochre_gb300 import PathCmd, Rasterizer, TileBuilder, Transform, Vec2, Mat2x2
    from ochre_gb300.batch import BatchBuilder, CUBIC, LINE, MOVE, QUADRATIC, CLOSE

    class Collect(TileBuilder):
        def __init__(self):
            self.tiles, self.spans = [], []

        def tile(self, x, y, data):
            self.tiles.append((x, y, bytes(data)))

        def span(self, x, y, w):
            self.spans.append((x, y, w))

    xf = Transform.new(Mat2x2.new(1.5, 0.25, -0.3, 1.2), Vec2(40.0, 30.0))
    r = Rasterizer()
    r.move_to(Vec2(3.5, 3.5))
    r.line_to(Vec2(70.25, 9.75))
    r.command(PathCmd.Quadratic(Vec2(90.0, 40.0), Vec2(40.0, 60.0)))
    r.fill([PathCmd.Line(Vec2(10.0, 10.0)), PathCmd.Cubic(Vec2(30.0, -20.0), Vec2(60.0, 40.0), Vec2(0.0, 30.0)),
            PathCmd.Close()], xf)
    c = Collect()
    r.finish(c)
    bb = BatchBuilder()
    bb.fill([MOVE, LINE, QUADRATIC], [3.5, 3.5, 70.25, 9.75, 90.0, 40.0, 40.0, 60.0], raw=True)
    bb.fill([LINE, CUBIC, CLOSE], [10.0, 10.0, 30.0, -20.0, 60.0, 40.0, 0.0, 30.0], xf.as_array())
    ref = oracle.run(bb.build())
    assert [(t[0], t[1]) for t in c.tiles] == [tuple(t) for t in ref["tile_xy"].tolist()]
    assert c.spans == [(int(x), int(y), int(w)) for (x, y), w in zip(ref["span_xy"].tolist(), ref["span_w"])]


def test_empty_batch_and_empty_rasterizer(any_ctx):
    from ochre_gb300.batch import BatchBuilder
    b = BatchBuilder().begin_raster().begin_raster().build()
    got = any_ctx.rasterize(b)
    assert got["tile_xy"].tolist() == [[0, 0], [0, 0]]
    assert not got["tile_alpha"].any()
    assert got["raster_tile_off"].tolist() == [0, 1, 2]


def test_invalid_inputs_are_reported(any_ctx):
    from ochre_gb300 import _lib
    b = W.readme_path()
    bad = b.pts.copy()
    bad[3] = np.inf
    b2 = type(b)(b.verbs, bad, b.fill_cmd_off, b.fill_xf, None, None, 1)
    with pytest.raises(_lib.OchreError) as e:
        any_ctx.rasterize(b2)
    assert e.value.status == _lib.E_INVALID
    # the context stays usable
    got = any_ctx.rasterize(b)
    compare(got, oracle.run(b), 1)


@pytest.mark.parametrize("case", ["long_line", "steep_quad"])
def test_iteration_caps_are_reported(any_ctx, case):
    """Finite inputs on which the reference would walk millions of pixel
    cells (a line across 4 million pixel columns: the walk steps on the f32
    geometry while `as i16` saturates the cells) or flatten one curve into
    millions of lines: the call returns OCHRE_E_LIMIT (2^20 cells per line,
    2^20 lines per curve) instead, and the context stays usable.  The oracle
    has no caps, like the reference, and is not run on them."""
    from ochre_gb300 import _lib
    from ochre_gb300.batch import CLOSE, IDENTITY, LINE, MOVE, QUADRATIC, BatchBuilder
    verbs, pts = {"long_line": ([MOVE, LINE, LINE, CLOSE], [-2.0e6, 0.5, 2.0e6, 0.5, 0.0, 40.0]),
                  "steep_quad": ([MOVE, QUADRATIC, CLOSE], [0.0, 0.0, 3.0e12, 0.0, 0.0, 1.0])}[case]
    bb = BatchBuilder()
    bb.begin_raster()
    bb.fill(verbs, pts, IDENTITY)
    with pytest.raises(_lib.OchreError) as e:
        any_ctx.rasterize(bb.build())
    assert e.value.status == _lib.E_LIMIT
    b = W.readme_path()
    compare(any_ctx.rasterize(b), oracle.run(b), 1)


def test_verbs_beyond_the_points_are_reported(any_ctx):
    """Verbs that consume more floats than the point array holds: flagged by
    the kernels that would read them (host and device entries alike)."""
    from ochre_gb300 import DeviceBatch, _lib
    b = W.glyph_run(n_paths=50, seed=3)
    short = type(b)(b.verbs, b.pts[:-5].copy(), b.fill_cmd_off, b.fill_xf, None, None, b.n_rasters)
    with pytest.raises(_lib.OchreError) as e:
        any_ctx.rasterize(short)
    assert e.value.status == _lib.E_INVALID
    with pytest.raises(_lib.OchreError) as e:
        any_ctx.rasterize_device(DeviceBatch(short))
    assert e.value.status == _lib.E_INVALID
    compare(any_ctx.rasterize(b), oracle.run(b), b.n_rasters)


def test_repeatable(any_ctx):
    """Two runs: identical structure; alpha may differ by the f32 summation
    order of shared-memory atomics (<= 1 LSB, the parity bound)."""
    b = W.glyph_run(n_paths=2000, seed=11)
    r1 = any_ctx.rasterize(b)
    r2 = any_ctx.rasterize(b)
    for k in r1:
        if k == "tile_alpha":
            assert np.abs(r1[k].astype(int) - r2[k].astype(int)).max() <= 1
        else:
            assert np.array_equal(r1[k], r2[k]), k


def test_fused_path_taken_for_glyphs_and_chain_for_big_paths(gpu_ctx):
    gpu_ctx.rasterize(W.glyph_run(n_paths=500))
    assert gpu_ctx.stats()["fused"] == 1
    gpu_ctx.rasterize(W.cubic_boxes(n_paths=3))
    assert gpu_ctx.stats()["fused"] == 0


def test_device_entry_remembers_a_batch_beyond_the_fused_limits():
    """A device batch that did not fit the fused kernel runs on the chain
    again without a fused attempt while its arrays and counts stay the same;
    a batch that fits (or the same arrays with other counts) is tried on the
    fused kernel again.  Results match the oracle every time."""
    import dataclasses

    from ochre_gb300 import DeviceBatch, GpuContext
    b = W.glyph_run(n_paths=400, seed=5)
    big = b.fill_xf.copy()
    big[7, :4] *= np.float32(12.0)   # one glyph ~12x larger: past the fused grid
    b_big = dataclasses.replace(b, fill_xf=big)
    ref, ref_big = oracle.run(b, threads=8), oracle.run(b_big, threads=8)
    ctx = GpuContext(0)
    try:
        db = DeviceBatch(b_big)
        for _ in range(2):
            compare(ctx.device_result_to_numpy(ctx.rasterize_device(db), b.n_rasters), ref_big, b.n_rasters)
            assert ctx.stats()["fused"] == 0
        # the same arrays, the glyph back to its size: still the chain (the
        # context keys on arrays and counts, not values), still exact
        db.fill_xf.copy_(db.fill_xf.new_tensor(b.fill_xf.reshape(-1)))
        compare(ctx.device_result_to_numpy(ctx.rasterize_device(db), b.n_rasters), ref, b.n_rasters)
        assert ctx.stats()["fused"] == 0
        # another batch fits and clears the note; the first is tried again
        db2 = DeviceBatch(b)
        compare(ctx.device_result_to_numpy(ctx.rasterize_device(db2), b.n_rasters), ref, b.n_rasters)
        assert ctx.stats()["fused"] == 1
        compare(ctx.device_result_to_numpy(ctx.rasterize_device(db), b.n_rasters), ref, b.n_rasters)
        assert ctx.stats()["fused"] == 1
    finally:
        ctx.close()


def test_full_size_glyph_run_matches_oracle(gpu_ctx):
    """The bench workload at full size (100,000 paths), fused path."""
    b = W.glyph_run(n_paths=100_000)
    ref = oracle.run(b, threads=16)
    got = gpu_ctx.rasterize(b)
    assert gpu_ctx.stats()["fused"] == 1
    st = compare(got, ref, b.n_rasters)
    assert st["diff_fraction"] < 1e-3, st


@pytest.mark.parametrize("name,gen,kw,bound", [
    ("cubic_boxes", W.cubic_boxes, dict(n_paths=20), 2e-3),
    ("glyph_run", W.glyph_run, dict(n_paths=2000), 2e-3),
    ("uneven_mix", W.uneven_mix, dict(n_paths=40), None),
    ("diff_union", W.diff_union, dict(n_paths=128), 2e-3),
    ("diff_scenes", W.diff_scenes, dict(n_scenes=2, max_paths=64), 2e-3),
])
def test_coverage_error_vs_fp64(any_ctx, name, gen, kw, bound):
    """Pre-quantisation f32 coverage against the FP64 analytic area of the same
    lines.  The uneven mix has no absolute bound: its long lines (up to ~8000
    px) drift in the reference's serial f32 walk, which the GPU reproduces,
    so its error is bounded by the f32 restatement's own error instead."""
    b = gen(**kw)
    any_ctx.set_want_cov(True)
    try:
        got = any_ctx.rasterize(b)
    finally:
        any_ctx.set_want_cov(False)
    e = oracle.tile_cov_error_vs_fp64(b, got["tile_xy"], got["tile_cov"], got["raster_tile_off"])
    print(name, e)
    if bound is None:
        ref = oracle.run(b, want_cov=True)
        e_ref = oracle.tile_cov_error_vs_fp64(b, ref["tile_xy"], ref["tile_cov"], ref["raster_tile_off"])
        bound = e_ref["max_abs"] + 1e-3
    assert e["max_abs"] < bound, (e, bound)


def test_host_path_large_batches_match_oracle(gpu_ctx):
    """Large batches through the host-buffer entry: points copied on a side
    stream while the first stages run, outputs written into mapped host
    memory (zero-copy) once a call has sized it, coverage included; then a
    mix that falls back to the general chain, with strokes."""
    b = W.glyph_run(n_paths=40_000, seed=17)
    ref = oracle.run(b, threads=16, want_cov=True)
    gpu_ctx.set_want_cov(True)
    try:
        got = gpu_ctx.rasterize(b)
    finally:
        gpu_ctx.set_want_cov(False)
    st = compare(got, ref, b.n_rasters)
    assert st["cov_max_abs_vs_oracle_f32"] < 1e-3
    # a second call of the same size goes through the mapped outputs
    gpu_ctx.set_want_cov(True)
    try:
        got = gpu_ctx.rasterize(b)
    finally:
        gpu_ctx.set_want_cov(False)
    compare(got, ref, b.n_rasters)
    # points in pinned host memory: read by the kernels in place
    import dataclasses

    import torch
    pinned = dataclasses.replace(b, pts=torch.from_numpy(b.pts.copy()).pin_memory().numpy())
    compare(gpu_ctx.rasterize(pinned), ref, b.n_rasters)
    # and a mix that needs the general chain, with strokes
    from ochre_gb300.batch import concat
    m = concat([W.glyph_run(n_paths=30_000, seed=18), W.uneven_mix(n_paths=20), W.stroke_run(n_paths=3000)])
    ref_m = oracle.run(m, threads=16)
    compare(gpu_ctx.rasterize(m), ref_m, m.n_rasters)
    m_pinned = dataclasses.replace(m, pts=torch.from_numpy(m.pts.copy()).pin_memory().numpy())
    compare(gpu_ctx.rasterize(m_pinned), ref_m, m.n_rasters)


@pytest.mark.parametrize("shape", __import__("ochre_gb300.autotune", fromlist=["fused_candidates"]).fused_candidates(),
                         ids=lambda p: __import__("ochre_gb300.autotune", fromlist=["shape_name"]).shape_name(p))
def test_every_fused_shape_matches_oracle(shape):
    """Every launch shape the autotuner may pick gives the same results."""
    from ochre_gb300 import GpuContext, autotune
    b = W.glyph_run(n_paths=3000, seed=23)
    ref = oracle.run(b, threads=16, want_cov=True)
    ctx = GpuContext(0, want_cov=True)
    autotune.apply(ctx, shape)
    got = ctx.rasterize(b)
    st = ctx.stats()
    assert st["fused"] == 1, st
    cst = compare(got, ref, b.n_rasters)
    assert cst["cov_max_abs_vs_oracle_f32"] < 1e-3, cst
    ctx.close()


@pytest.fixture(scope="session")
def dense_scenes():
    # the full dense-scenes configuration (4,096 scenes of 512^2, about a
    # million fills) takes most of a minute to generate: once per session
    return W.diff_scenes()


@pytest.mark.parametrize("name", ["cubic_boxes", "uneven_mix", "stroke_run", "diff_scenes"])
def test_full_size_configuration_matches_oracle(gpu_ctx, request, name):
    """Full-size seeded configurations against the oracle: every tile
    position, per-raster tile and span offset, span position, width and tile
    index exact; every alpha byte within 1 LSB.  The cubic boxes (1,000
    paths) are the plain-method configuration compared against the CPU
    rasterizer; the uneven mix (20,000 paths, 70 M tiles) carries the
    batched-vs-plain metric; the dense scenes (4,096 rasters) the
    differentiable one."""
    import os

    from ochre_gb300 import DeviceBatch
    b = request.getfixturevalue("dense_scenes") if name == "diff_scenes" else getattr(W, name)()
    db = DeviceBatch(b)
    got = gpu_ctx.device_result_to_numpy(gpu_ctx.rasterize_device(db), b.n_rasters)
    del db
    ref = oracle.run(b, threads=os.cpu_count() or 1)
    st = compare(got, ref, b.n_rasters)
    print(name, st)
    assert st["diff_fraction"] < 1e-3, st


@pytest.mark.parametrize("name,tiles,spans", [
    ("readme_path", 100, 23),
    ("cubic_boxes", 873_599, 170_315),
    ("glyph_run", 2_116_864, 253_952),
    ("uneven_mix", 70_365_373, 17_974_124),
    ("diff_union", 8_635, 992),
    ("stroke_run", 5_825_432, 81_363),
    ("diff_scenes", 12_319_083, 784_530),
])
def test_configuration_counts_match_oracle(gpu_ctx, request, name, tiles, spans):
    """Full-size seeded configurations: the GPU's tile and span counts equal
    the oracle's (pinned in tests/test_oracle.py)."""
    from ochre_gb300 import DeviceBatch
    b = request.getfixturevalue("dense_scenes") if name == "diff_scenes" else getattr(W, name)()
    gpu_ctx.rasterize_device(DeviceBatch(b))
    st = gpu_ctx.stats()
    assert (st["n_tiles"], st["n_spans"]) == (tiles, spans)


class _Dev:
    """A device array of a result, seen by torch (no copy)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def test_stored_increments_above_2_30(gpu_ctx_chain):
    # 36,000 copies of one thin diagonal band (two lines of about 16,000
    # pixel cells each): 1.15e9 stored increments, more than the 2^30 the
    # chain's other counts allow.  Every copy must equal the oracle's
    # rasterization of the band, tile for tile.
    import torch
    from ochre_gb300 import DeviceBatch
    from ochre_gb300.batch import Batch, CLOSE, LINE, MOVE
    R = 36_000
    verbs = np.array([MOVE, LINE, LINE, LINE, CLOSE], np.uint8)
    pts = np.array([0.3, 0.7, 7999.6, 7990.2, 7999.6, 7993.1, 0.3, 3.6], np.float32)
    xf = np.array([1, 0, 0, 1, 0, 0], np.float32)
    one = Batch(verbs, pts, np.array([0, 5], np.uint32), xf[None], None, None, 1)
    big = Batch(np.tile(verbs, R), np.tile(pts, R), (np.arange(R + 1) * 5).astype(np.uint32),
                np.tile(xf, (R, 1)), None, None, R)
    exp = oracle.run(one)
    T1, N1 = len(exp["tile_xy"]), len(exp["span_xy"])
    db = DeviceBatch(big)
    r = gpu_ctx_chain.rasterize_device(db)
    st = gpu_ctx_chain.stats()
    assert st["n_incs"] > (1 << 30), st
    assert (r.n_tiles, r.n_spans) == (R * T1, R * N1)
    rto = torch.as_tensor(_Dev(r.raster_tile_off, (R + 1,), "<u4"), device="cuda").long()
    rso = torch.as_tensor(_Dev(r.raster_span_off, (R + 1,), "<u4"), device="cuda").long()
    steps = torch.arange(R + 1, device="cuda", dtype=torch.int64)
    assert torch.equal(rto, steps * T1) and torch.equal(rso, steps * N1)
    xy = torch.as_tensor(_Dev(r.tile_xy, (R, T1, 2), "<i2"), device="cuda")
    al = torch.as_tensor(_Dev(r.tile_alpha, (R, T1, 64), "|u1"), device="cuda")
    for a in range(0, R, 4096):   # every copy against the first, a slab at a time
        assert torch.equal(xy[a:a + 4096], xy[:1].expand(min(4096, R - a), -1, -1)), a
        assert torch.equal(al[a:a + 4096], al[:1].expand(min(4096, R - a), -1, -1)), a
    if N1:
        sxy = torch.as_tensor(_Dev(r.span_xy, (R, N1, 2), "<i2"), device="cuda")
        assert torch.equal(sxy, sxy[:1].expand(R, -1, -1))
    first = {"tile_xy": xy[0].cpu().numpy(), "tile_alpha": al[0].cpu().numpy(),
             "span_xy": np.zeros((N1, 2), np.int16) if not N1 else
             torch.as_tensor(_Dev(r.span_xy, (N1, 2), "<i2"), device="cuda").cpu().numpy(),
             "span_w": np.zeros(0, np.uint16) if not N1 else
             torch.as_tensor(_Dev(r.span_width, (N1,), "<u2"), device="cuda").cpu().numpy(),
             "span_tile": np.zeros(0, np.uint32) if not N1 else
             torch.as_tensor(_Dev(r.span_tile, (N1,), "<u4"), device="cuda").cpu().numpy(),
             "raster_tile_off": np.array([0, T1], np.uint64), "raster_span_off": np.array([0, N1], np.uint64)}
    compare(first, exp, 1)


@pytest.mark.parametrize("long_cells,refill", [(0, 8), (16, 1), (16, 8), (16, 32), (64, 8), (192, 8)])
def test_long_line_walkers_match_oracle(gpu_ctx_chain, long_cells, refill):
    # Lines of more than long_cells cells are walked by the persistent
    # refilling walkers beside the one-thread-per-line kernels (0: none are);
    # a low threshold sends most of a batch's lines there.  The result must
    # not depend on the split, and must equal the oracle's.
    from ochre_gb300 import autotune, batch as B
    b = B.concat([W.uneven_mix(n_paths=120, seed=21), W.cubic_boxes(n_paths=40, seed=22)])
    ref = oracle.run(b, threads=8)
    old = {k: autotune.get(gpu_ctx_chain, k) for k in ("chain_long_cells", "chain_walk_refill")}
    try:
        autotune.apply(gpu_ctx_chain, {"chain_long_cells": long_cells, "chain_walk_refill": refill})
        for _ in range(2):
            got = gpu_ctx_chain.rasterize(b)
            compare(got, ref, b.n_rasters)
        assert gpu_ctx_chain.stats()["n_incs"] > 0
    finally:
        autotune.apply(gpu_ctx_chain, old)


def _band_copies(n):
    from ochre_gb300.batch import Batch, CLOSE, LINE, MOVE
    verbs = np.array([MOVE, LINE, LINE, LINE, CLOSE], np.uint8)
    pts = np.array([0.3, 0.7, 7999.6, 7990.2, 7999.6, 7993.1, 0.3, 3.6], np.float32)
    xf = np.array([1, 0, 0, 1, 0, 0], np.float32)
    return Batch(np.tile(verbs, n), np.tile(pts, n), (np.arange(n + 1) * 5).astype(np.uint32),
                 np.tile(xf, (n, 1)), None, None, n)


def _result_tensors(r, n_rasters):
    import torch
    T, N = r.n_tiles, r.n_spans
    out = {"rto": torch.as_tensor(_Dev(r.raster_tile_off, (n_rasters + 1,), "<u4"), device="cuda").clone(),
           "rso": torch.as_tensor(_Dev(r.raster_span_off, (n_rasters + 1,), "<u4"), device="cuda").clone()}
    if T:
        out["xy"] = torch.as_tensor(_Dev(r.tile_xy, (T, 2), "<i2"), device="cuda").clone()
        out["alpha"] = torch.as_tensor(_Dev(r.tile_alpha, (T, 64), "|u1"), device="cuda").clone()
    if N:
        out["sxy"] = torch.as_tensor(_Dev(r.span_xy, (N, 2), "<i2"), device="cuda").clone()
        out["sw"] = torch.as_tensor(_Dev(r.span_width, (N,), "<u2"), device="cuda").clone()
    return out


@pytest.mark.parametrize("case", ["mixed_32bit_keys", "bands_64bit_keys"])
def test_sort_digit_widths_agree(gpu_ctx_chain, case):
    # The chain's radix sort with 8- and 11-bit digits (the autotuner picks
    # one per GPU) gives the same result, with 32-bit keys and with 64-bit
    # keys (2,400 rasters of 1,000 x 1,000-tile boxes: a key space above 2^32).
    import torch
    from ochre_gb300 import DeviceBatch, autotune, batch as B
    b = (B.concat([W.uneven_mix(n_paths=150, seed=23), W.cubic_boxes(n_paths=40, seed=24)])
         if case == "mixed_32bit_keys" else _band_copies(2400))
    db = DeviceBatch(b)
    old = autotune.get(gpu_ctx_chain, "sort_digit_bits")
    res = {}
    try:
        for bits in (8, 11):
            autotune.apply(gpu_ctx_chain, {"sort_digit_bits": bits})
            r = gpu_ctx_chain.rasterize_device(db)
            st = gpu_ctx_chain.stats()
            assert (st["key_bits"] > 32) == (case == "bands_64bit_keys"), st
            assert 0 < st["sort_passes"] <= -(-st["key_bits"] // bits), st
            res[bits] = _result_tensors(r, b.n_rasters)
        assert res[8].keys() == res[11].keys()
        for k in res[8]:
            assert torch.equal(res[8][k], res[11][k]), k
        if case == "mixed_32bit_keys":
            autotune.apply(gpu_ctx_chain, {"sort_digit_bits": 11})
            compare(gpu_ctx_chain.rasterize(b), oracle.run(b, threads=8), b.n_rasters)
    finally:
        autotune.apply(gpu_ctx_chain, {"sort_digit_bits": old})

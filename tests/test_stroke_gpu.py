"""Stroked fills on the GPU (Rasterizer::stroke, rasterizer.rs:169-171):
the device stroke stage plus the fill path against the oracle's stroke +
fill, tile/span structure exact and alpha within 1 LSB."""
import numpy as np
import pytest

import oracle
from compare import compare
from ochre_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_stroke_cases(any_ctx):
    import stroke_cases
    b, names = stroke_cases.stroke_batch()
    ref = oracle.run(b)
    got = any_ctx.rasterize(b)
    compare(got, ref, b.n_rasters)


def test_stroke_cases_device_path(any_ctx):
    import stroke_cases
    from ochre_gb300 import DeviceBatch
    b, _ = stroke_cases.stroke_batch()
    ref = oracle.run(b)
    r = any_ctx.rasterize_device(DeviceBatch(b))
    compare(any_ctx.device_result_to_numpy(r, b.n_rasters), ref, b.n_rasters)


def test_stroke_workload(any_ctx):
    b = W.stroke_run(n_paths=3000)
    ref = oracle.run(b, threads=8)
    got = any_ctx.rasterize(b)
    st = compare(got, ref, b.n_rasters)
    assert st["diff_fraction"] < 0.01, st


def test_stroke_mixed_with_fills(gpu_ctx):
    """Stroked and filled paths in one batch (and in one rasterizer)."""
    from ochre_gb300.batch import concat
    import stroke_cases
    s, _ = stroke_cases.stroke_batch()
    b = concat([W.glyph_run(n_paths=50), s, W.stroke_run(n_paths=40), W.cubic_boxes(n_paths=5)])
    ref = oracle.run(b)
    got = gpu_ctx.rasterize(b)
    compare(got, ref, b.n_rasters)


def test_stroke_through_rasterizer_api():
    from ochre_gb300 import PathCmd, Rasterizer, TileBuilder, Transform, Vec2
    from ochre_gb300.batch import BatchBuilder

    class Collect(TileBuilder):
        def __init__(self):
            self.tiles, self.spans = [], []

        def tile(self, x, y, data):
            self.tiles.append((x, y, bytes(data)))

        def span(self, x, y, w):
            self.spans.append((x, y, w))

    path = [PathCmd.Move(Vec2(10.0, 10.0)), PathCmd.Cubic(Vec2(40.0, -5.0), Vec2(60.0, 80.0), Vec2(90.0, 30.0)),
            PathCmd.Line(Vec2(30.0, 60.0))]
    xf = Transform.rotate(0.3).then(Transform.translate(20.0, 15.0))
    r = Rasterizer()
    r.stroke(path, 5.0, xf)
    r.fill([PathCmd.Move(Vec2(0.0, 0.0)), PathCmd.Line(Vec2(20.0, 0.0)), PathCmd.Line(Vec2(0.0, 20.0))],
           Transform.id())
    out = Collect()
    r.finish(out)
    from ochre_gb300.rasterizer import encode_path
    bb = BatchBuilder().begin_raster()
    v, p = encode_path(path)
    bb.fill(v, p, xf.as_array(), stroke_width=5.0)
    v2, p2 = encode_path([PathCmd.Move(Vec2(0.0, 0.0)), PathCmd.Line(Vec2(20.0, 0.0)), PathCmd.Line(Vec2(0.0, 20.0))])
    bb.fill(v2, p2)
    ref = oracle.run(bb.build())
    assert [(x, y) for x, y, _ in out.tiles] == [tuple(t) for t in ref["tile_xy"].tolist()]
    a = np.frombuffer(b"".join(d for _, _, d in out.tiles), np.uint8).reshape(-1, 64).astype(int)
    assert np.abs(a - ref["tile_alpha"].astype(int)).max() <= 1
    assert out.spans == [tuple(int(q) for q in s) + (int(w),) for s, w in zip(ref["span_xy"].tolist(), ref["span_w"])]


def test_fill_backward_rejects_strokes():
    import torch
    from ochre_gb300 import DeviceBatch, GpuContext, OchreError
    b = W.stroke_run(n_paths=4)
    ctx = GpuContext(0)
    db = DeviceBatch(b, 0)
    cov = ctx.render_coverage(db, 256, 256)
    with pytest.raises(OchreError):
        ctx.fill_backward(db, 256, 256, torch.zeros_like(cov))
    ctx.close()

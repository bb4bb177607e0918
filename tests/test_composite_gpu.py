"""Headless compositing (the reference example's GL draw, restated): the
device kernel against the oracle's painter's-order restatement, bit-exact
RGBA8 output."""
import numpy as np
import pytest

import oracle
from ochre_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _run(batch, colors, w, h, canvas=None, ctx_kw=None):
    """GPU rasterization + GPU compositing; returns the image and the
    rasterization result (numpy)."""
    import torch
    from ochre_gb300 import DeviceBatch, GpuContext
    ctx = GpuContext(0, **(ctx_kw or {}))
    r = ctx.rasterize_device(DeviceBatch(batch, 0))
    res = ctx.device_result_to_numpy(r, batch.n_rasters)
    cv = torch.full((h, w, 4), 255, dtype=torch.uint8, device="cuda:0") if canvas is None else \
        torch.as_tensor(canvas, device="cuda:0").contiguous()
    col = torch.as_tensor(np.ascontiguousarray(colors, np.uint8), device="cuda:0")
    ctx.composite(r, batch.n_rasters, col, cv)
    torch.cuda.synchronize()
    out = cv.cpu().numpy()
    ctx.close()
    return out, res


def _check(batch, colors, w, h, canvas=None):
    """The rasterization against the oracle (structure exact, alpha within
    1 LSB), and the compositing bit-exact against the oracle's compositing of
    the same rasterization (so a 1-LSB alpha difference cannot show up as a
    compositing difference)."""
    from compare import compare
    got, res = _run(batch, colors, w, h, canvas)
    compare(res, oracle.run(batch, threads=8), batch.n_rasters)
    ref = oracle.composite(res, batch.n_rasters, colors, w, h, canvas)
    assert got.shape == ref.shape
    assert np.array_equal(got, ref), int((got != ref).any(axis=2).sum())
    return got


@pytest.mark.parametrize("name,gen,kw,w,h", [
    ("glyphs", W.glyph_run, dict(n_paths=400), 4096, 4096),
    ("scenes", W.diff_scenes, dict(n_scenes=3, max_paths=40), 300, 260),
    ("strokes", W.stroke_run, dict(n_paths=300), 2048, 2048),
    ("uneven_clipped", W.uneven_mix, dict(n_paths=30), 1000, 777),
])
def test_composite_matches_oracle(name, gen, kw, w, h):
    b = gen(**kw)
    rng = np.random.default_rng(1)
    colors = rng.integers(0, 256, size=(b.n_rasters, 4), dtype=np.uint8)
    _check(b, colors, w, h)


def test_composite_overlaps_in_raster_order():
    """Many translucent rasters over the same pixels: the order is the
    raster order, and the canvas content is read, not assumed."""
    from ochre_gb300.batch import BatchBuilder
    bb = BatchBuilder()
    for k in range(12):
        bb.begin_raster().fill([0, 1, 1, 1, 5], [4.0 + k, 3.0, 60.5, 5.0 + k, 50.0, 61.0, 3.0, 40.0 - k])
    b = bb.build()
    colors = np.array([[(37 * k) % 256, (91 * k) % 256, (53 * k + 7) % 256, 40 + 15 * k] for k in range(12)], np.uint8)
    canvas = np.random.default_rng(2).integers(0, 256, size=(70, 70, 4), dtype=np.uint8)
    _check(b, colors, 70, 70, canvas)

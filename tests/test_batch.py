"""CPU tests of the host-side input layout and the seeded workloads."""
import numpy as np
import pytest

from ochre_gb300 import batch as B
from ochre_gb300 import workloads as W


def test_builder_and_validate():
    bb = B.BatchBuilder()
    bb.begin_raster().fill([B.MOVE, B.LINE, B.CLOSE], [0, 0, 5, 5])
    bb.begin_raster()
    bb.begin_raster().fill([B.MOVE], [1, 1], raw=True).fill([B.CUBIC], [1, 2, 3, 4, 5, 6])
    b = bb.build()
    assert b.n_rasters == 3 and b.n_fills == 3
    assert b.raster_fill_off.tolist() == [0, 1, 1, 3]
    assert b.fill_cmd_off.tolist() == [0, 3, 4, 5]
    assert b.fill_flags.tolist() == [0, 1, 0]
    assert b.input_bytes() == 5 + 4 * len(b.pts) + 24 * 3


def test_compulsory_bytes_of_the_glyph_run():
    """The roofline numerator of the headline: 1 B per verb, 8 B per point
    (Move and Line one point, a quadratic two), 24 B per transform in; 68 B
    per tile (64 alpha + two i16) and 6 B per span out.  The tile and span
    counts are the oracle's for this workload."""
    import bench
    b = W.glyph_run()
    counts = np.bincount(b.verbs, minlength=6)
    points = counts[B.MOVE] + counts[B.LINE] + 2 * counts[B.QUADRATIC] + 3 * counts[B.CUBIC]
    assert counts[B.CUBIC] == 0 and counts[B.CONIC] == 0
    inp = b.n_cmds + 8 * int(points) + 24 * b.n_fills
    assert inp == b.input_bytes() == 45_194_436
    out = bench.output_bytes(2_116_864, 253_952, b.n_rasters)
    assert out == 68 * 2_116_864 + 6 * 253_952
    assert inp + out == 190_664_900


def test_validate_rejects_bad_input():
    b = W.readme_path()
    bad = B.Batch(b.verbs.copy(), b.pts[:-1].copy(), b.fill_cmd_off, b.fill_xf, None, None, 1)
    with pytest.raises(ValueError):
        bad.validate()
    v = b.verbs.copy()
    v[0] = 9
    with pytest.raises(ValueError):
        B.Batch(v, b.pts, b.fill_cmd_off, b.fill_xf, None, None, 1).validate()


def test_concat_and_subset_roundtrip():
    a = W.glyph_run(n_paths=5)
    c = W.cubic_boxes(n_paths=2)
    ab = B.concat([a, c])
    assert ab.n_rasters == 7
    s = B.subset(ab, [5, 6])
    assert np.array_equal(s.verbs, c.verbs) and np.array_equal(s.pts, c.pts)


@pytest.mark.parametrize("gen,kw,n", [
    (W.cubic_boxes, dict(n_paths=10), 10),
    (W.glyph_run, dict(n_paths=50), 50),
    (W.uneven_mix, dict(n_paths=20), 20),
    (W.diff_union, dict(n_paths=8), 1),
    (W.diff_scenes, dict(n_scenes=2, max_paths=20), 2),
])
def test_workloads_are_seeded_and_valid(gen, kw, n):
    b1, b2 = gen(**kw), gen(**kw)
    b1.validate()
    assert b1.n_rasters == n
    assert np.array_equal(b1.verbs, b2.verbs) and np.array_equal(b1.pts, b2.pts)
    assert np.isfinite(b1.pts).all() and np.isfinite(b1.fill_xf).all()


def test_glyph_run_shape():
    b = W.glyph_run(n_paths=400)
    per = np.diff(b.fill_cmd_off.astype(np.int64))
    quads = np.array([np.sum(b.verbs[b.fill_cmd_off[i]:b.fill_cmd_off[i + 1]] == B.QUADRATIC) for i in range(400)])
    moves = np.array([np.sum(b.verbs[b.fill_cmd_off[i]:b.fill_cmd_off[i + 1]] == B.MOVE) for i in range(400)])
    assert quads.min() >= 8 and quads.max() <= 40
    assert moves.min() >= 1 and moves.max() <= 3
    assert (per == quads + 2 * moves).all()


def test_uneven_mix_in_canvas():
    b = W.uneven_mix(n_paths=200)
    assert b.pts.min() >= 0.0 and b.pts.max() < 8192.0
